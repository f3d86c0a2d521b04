"""Regenerate tests/golden/reference_cases.json from the reference checkout.

Reads the reference's golden netlists (testdata/netlists/*.cir) and their golden
results -- the independent references in testdata/golden/*.csv and the
ngspice-39 twins in testdata/golden/ngspice/*.csv -- and writes them, parsed,
into one JSON fixture, so the tests need no reference checkout at run time.
Dense ngspice transient tables are thinned to at most 800 rows.

Run where a checkout of the reference exists:
    python tests/golden/make_reference_fixtures.py REF_ROOT
"""
import json
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import spice_subset  # noqa: E402

REF = None  # the reference checkout, the script's one argument
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_cases.json")


def thin(tab, limit=800):
    if tab["kind"] != "table" or len(tab["xs"]) <= limit:
        return tab
    step = -(-len(tab["xs"]) // limit)
    idx = list(range(0, len(tab["xs"]), step))
    if idx[-1] != len(tab["xs"]) - 1:
        idx.append(len(tab["xs"]) - 1)
    out = dict(tab)
    out["xs"] = [tab["xs"][i] for i in idx]
    out["columns"] = {k: [v[i] for i in idx] for k, v in tab["columns"].items()}
    out["thinned"] = step
    return out


def main():
    global REF
    if len(sys.argv) != 2:
        sys.exit("usage: make_reference_fixtures.py REF_ROOT  (the reference checkout)")
    REF = sys.argv[1]
    nl_dir = os.path.join(REF, "testdata", "netlists")
    cases = []
    for fn in sorted(os.listdir(nl_dir)):
        if not fn.endswith(".cir"):
            continue
        name = fn[:-4]
        with open(os.path.join(nl_dir, fn)) as f:
            ckt, why = spice_subset.parse(f.read())
        case = {"name": name, "circuit": ckt, "skip": why, "golden": {}}
        for src, path in (("independent", os.path.join(REF, "testdata", "golden", name + ".csv")),
                          ("ngspice", os.path.join(REF, "testdata", "golden", "ngspice", name + ".csv"))):
            if os.path.exists(path):
                with open(path) as f:
                    case["golden"][src] = thin(spice_subset.read_golden(f.read()))
        cases.append(case)
    with open(OUT, "w") as f:
        json.dump({"source": "fdamador/kronspice testdata (netlists, golden, golden/ngspice)",
                   "cases": cases}, f, separators=(",", ":"))
    print("wrote", OUT, len(cases), "cases")


if __name__ == "__main__":
    main()
