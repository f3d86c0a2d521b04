"""Golden fixtures' netlist side (test infrastructure): the package's SPICE
reader (kronspice_gb300/netlist.py) plus the reader of the reference's golden
CSV tables (internal/golden/golden.go Read / LoadTable)."""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))

from kronspice_gb300.netlist import parse, value  # noqa: E402,F401


def read_golden(text):
    """Golden CSV (internal/golden/golden.go Read / LoadTable) as a dict."""
    rows = [ln.strip() for ln in text.splitlines() if ln.strip() and not ln.strip().startswith("#")]
    head = rows[0].lower()
    if head == "name,value":
        vals = {}
        for r in rows[1:]:
            k, v = r.split(",", 1)
            vals[k.strip().lower()] = float(v)
        return {"kind": "values", "values": vals}
    names = [c.strip().lower() for c in rows[0].split(",")]
    cols = {n: [] for n in names[1:]}
    xs = []
    for r in rows[1:]:
        parts = [float(p) for p in r.split(",")]
        xs.append(parts[0])
        for n, v in zip(names[1:], parts[1:]):
            cols[n].append(v)
    return {"kind": "table", "x": names[0], "xs": xs, "names": names[1:], "columns": cols}
