"""Minimal SPICE netlist reader for the golden fixtures (test infrastructure).

Reads the subset of SPICE the reference's golden netlists use for the element
kinds of the engine (R, C, L, V, I, D, Q, M; .model, .op, .dc, .tran) into a
plain dict: the same information circuit.FromDeck (circuit/builder.go:307)
extracts from a parsed deck.  Netlists with other elements or with .subckt /
.param return None from parse() with the reason, and the golden tests skip them.
"""
import re

_SUFFIX = [("meg", 1e6), ("mil", 25.4e-6), ("t", 1e12), ("g", 1e9), ("k", 1e3),
           ("m", 1e-3), ("u", 1e-6), ("n", 1e-9), ("p", 1e-12), ("f", 1e-15)]
_NUM = re.compile(r"^([+-]?(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?)(.*)$")


def value(tok):
    """SPICE number with engineering suffix ('1k', '20u', '1meg', '50f')."""
    m = _NUM.match(tok.strip())
    if not m:
        raise ValueError("bad number %r" % tok)
    v = float(m.group(1))
    rest = m.group(2).lower()
    for s, mul in _SUFFIX:
        if rest.startswith(s):
            return v * mul
    return v


def _tokens(line):
    line = line.replace("(", " ( ").replace(")", " ) ").replace(",", " ")
    line = re.sub(r"\s*=\s*", "=", line)
    return line.split()


def _params(toks):
    out = {}
    for t in toks:
        if t in ("(", ")"):
            continue
        if "=" in t:
            k, v = t.split("=", 1)
            out[k.lower()] = value(v)
    return out


def _source(toks):
    """Value spec of a V/I line after the nodes: DC, AC and a waveform."""
    src = {"dc": 0.0, "has_dc": False, "wave": None, "args": [], "ac": [0.0, 0.0]}
    i = 0
    while i < len(toks):
        t = toks[i].lower()
        if t == "dc":
            src["dc"], src["has_dc"] = value(toks[i + 1]), True
            i += 2
        elif t == "ac":
            mag = value(toks[i + 1]) if i + 1 < len(toks) else 1.0
            ph = 0.0
            i += 2
            if i < len(toks):
                try:
                    ph = value(toks[i])
                    i += 1
                except ValueError:
                    pass
            src["ac"] = [mag, ph]
        elif t in ("pulse", "sin", "exp", "pwl"):
            args = []
            i += 1
            if i < len(toks) and toks[i] == "(":
                i += 1
                while i < len(toks) and toks[i] != ")":
                    args.append(value(toks[i]))
                    i += 1
                i += 1
            else:
                while i < len(toks):
                    try:
                        args.append(value(toks[i]))
                    except ValueError:
                        break
                    i += 1
            src["wave"], src["args"] = t, args
        else:
            src["dc"] = value(toks[i])
            src["has_dc"] = True
            i += 1
    return src


def parse(text):
    """Return (circuit dict, None) or (None, reason)."""
    try:
        return _parse(text)
    except (ValueError, IndexError) as e:
        return None, "unsupported netlist: %s" % e


def _parse(text):
    raw = text.splitlines()
    lines = []
    for k, ln in enumerate(raw):
        if k == 0:
            continue  # title
        s = ln.strip()
        if not s or s.startswith("*"):
            continue
        if s.startswith("+") and lines:
            lines[-1] += " " + s[1:]
        else:
            lines.append(s)
    ckt = {"title": raw[0].strip() if raw else "", "elements": [], "models": {}, "analyses": []}
    for ln in lines:
        if ";" in ln:
            ln = ln.split(";", 1)[0]
        toks = _tokens(ln)
        if not toks:
            continue
        head = toks[0].lower()
        if head.startswith("."):
            if head == ".end":
                break
            if head == ".model":
                name = toks[1].lower()
                typ = toks[2].lower()
                ckt["models"][name] = {"type": typ, "params": _params(toks[3:])}
            elif head == ".op":
                ckt["analyses"].append({"kind": "op"})
            elif head == ".dc":
                ckt["analyses"].append({"kind": "dc", "source": toks[1].lower(), "start": value(toks[2]),
                                        "stop": value(toks[3]), "step": value(toks[4])})
            elif head == ".tran":
                nums, uic = [], False
                for t in toks[1:]:
                    if t.lower() == "uic":
                        uic = True
                    else:
                        nums.append(value(t))
                nums += [0.0] * (4 - len(nums))
                ckt["analyses"].append({"kind": "tran", "step": nums[0], "stop": nums[1], "start": nums[2],
                                        "max_step": nums[3], "uic": uic})
            elif head == ".ac":
                ckt["analyses"].append({"kind": "ac", "variation": toks[1].lower(), "points": int(value(toks[2])),
                                        "fstart": value(toks[3]), "fstop": value(toks[4])})
            else:
                return None, "unsupported control line " + head
            continue
        kind = head[0]
        name = toks[0]
        if kind == "r":
            ckt["elements"].append({"name": name, "kind": "R", "nodes": toks[1:3], "value": value(toks[3])})
        elif kind in "cl":
            e = {"name": name, "kind": kind.upper(), "nodes": toks[1:3], "value": value(toks[3])}
            p = _params(toks[4:])
            if "ic" in p:
                e["ic"] = p["ic"]
            ckt["elements"].append(e)
        elif kind in "vi":
            e = {"name": name, "kind": kind.upper(), "nodes": toks[1:3]}
            e.update(_source(toks[3:]))
            ckt["elements"].append(e)
        elif kind == "d":
            e = {"name": name, "kind": "D", "nodes": toks[1:3], "model": toks[3].lower(), "area": 0.0}
            if len(toks) > 4 and "=" not in toks[4]:
                e["area"] = value(toks[4])
            ckt["elements"].append(e)
        elif kind == "q":
            rest = toks[1:]
            # c b e [s] model [area]: the model is the first token naming a .model
            nodes, model, area = [], None, 0.0
            for t in rest:
                if model is None and t.lower() in _pending_models(lines):
                    model = t.lower()
                elif model is None:
                    nodes.append(t)
                elif "=" not in t:
                    area = value(t)
            ckt["elements"].append({"name": name, "kind": "Q", "nodes": nodes, "model": model, "area": area})
        elif kind == "m":
            ckt["elements"].append({"name": name, "kind": "M", "nodes": toks[1:5], "model": toks[5].lower(),
                                    "params": _params(toks[6:])})
        else:
            return None, "unsupported element " + name
    return ckt, None


def _pending_models(lines):
    out = set()
    for ln in lines:
        t = _tokens(ln)
        if len(t) > 1 and t[0].lower() == ".model":
            out.add(t[1].lower())
    return out


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
