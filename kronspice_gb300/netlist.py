"""SPICE netlist reader: the netlist-to-circuit path of the engine
(netlist/parser.go and circuit.FromDeck, circuit/builder.go:307).

Reads the SPICE subset the reference's netlists use for the engine's element
kinds (R, C, L, V, I, D, Q, M, E, F, G, H, K, S, W; a C or L with Q=pwl /
FLUX=pwl / SCALE= is the nonlinear or time-varying element; .model, .op, .dc,
.tran, .ac, .param with {expression} / 'expression' values, .subckt with params
and nesting, expanded into a flat circuit).  parse(text) gives the plain dict
form (circuit.from_dict builds it; None and the reason for a netlist outside the
subset); read(text) gives the Circuit and its analysis lines, or raises
NetlistError.  Expressions are evaluated by a walker over their syntax tree
(numbers, parameters, + - * / ^, and sqrt exp log ln sin cos abs pow min max),
never by executing text.
"""
import ast
import math
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


# ---------------------------------------------------------------- expressions
_FUNCS = {"sqrt": math.sqrt, "exp": math.exp, "log": math.log, "ln": math.log, "sin": math.sin, "cos": math.cos,
          "abs": abs, "pow": math.pow, "min": min, "max": max}


def _py_expr(text):
    """A SPICE expression as Python source: numbers with engineering suffixes
    converted, identifiers lower-cased, '^' as power."""
    out, i = [], 0
    while i < len(text):
        c = text[i]
        if c.isdigit() or (c == "." and i + 1 < len(text) and text[i + 1].isdigit()):
            j = i
            while j < len(text) and (text[j].isdigit() or text[j] == "."):
                j += 1
            if j < len(text) and text[j] in "eE" and j + 1 < len(text) and (text[j + 1].isdigit() or text[j + 1] in "+-"):
                j += 2
                while j < len(text) and text[j].isdigit():
                    j += 1
            k = j
            while k < len(text) and text[k].isalpha():
                k += 1
            out.append(repr(value(text[i:k])))
            i = k
        elif c.isalpha() or c == "_":
            j = i
            while j < len(text) and (text[j].isalnum() or text[j] == "_"):
                j += 1
            out.append(text[i:j].lower())
            i = j
        elif c == "^":
            out.append("**")
            i += 1
        else:
            out.append(c)
            i += 1
    return "".join(out)


def evaluate(text, scope, _active=None):
    """Value of a SPICE expression over the parameters in scope (names
    lower-case, values numbers or unevaluated expressions)."""
    active = set() if _active is None else _active
    try:
        tree = ast.parse(_py_expr(text).strip(), mode="eval")
    except SyntaxError:
        raise ValueError("bad expression %r" % text)

    def ev(n):
        if isinstance(n, ast.Expression):
            return ev(n.body)
        if isinstance(n, ast.Constant) and isinstance(n.value, (int, float)):
            return float(n.value)
        if isinstance(n, ast.Name):
            if n.id not in scope:
                raise ValueError("unknown parameter %r" % n.id)
            v = scope[n.id]
            if isinstance(v, float):
                return v
            if n.id in active:  # a parameter defined through itself
                raise ValueError("parameter %r depends on itself" % n.id)
            active.add(n.id)
            try:
                return evaluate(v, scope, active)
            finally:
                active.discard(n.id)
        if isinstance(n, ast.BinOp):
            a, b = ev(n.left), ev(n.right)
            ops = {ast.Add: lambda: a + b, ast.Sub: lambda: a - b, ast.Mult: lambda: a * b,
                   ast.Div: lambda: a / b, ast.Pow: lambda: a ** b}
            if type(n.op) not in ops:
                raise ValueError("operator in %r" % text)
            return ops[type(n.op)]()
        if isinstance(n, ast.UnaryOp) and isinstance(n.op, (ast.USub, ast.UAdd)):
            v = ev(n.operand)
            return -v if isinstance(n.op, ast.USub) else v
        if isinstance(n, ast.Call) and isinstance(n.func, ast.Name) and n.func.id in _FUNCS:
            return float(_FUNCS[n.func.id](*[ev(a) for a in n.args]))
        raise ValueError("unsupported expression %r" % text)
    return ev(tree)


_GROUP = re.compile(r"\{[^{}]*\}|'[^']*'")


def _protect(line):
    """Replace {...} and '...' expressions by placeholders before tokenising."""
    exprs = []

    def sub(m):
        exprs.append(m.group(0)[1:-1])
        return "@%d@" % (len(exprs) - 1)
    return _GROUP.sub(sub, line), exprs


def _assignments(toks):
    out = []
    for t in toks:
        if "=" in t:
            k, v = t.split("=", 1)
            out.append((k.lower(), v))
    return out


def _expand(lines):
    """Flatten .param / .subckt: element lines with their nodes renamed and
    every {expression} evaluated; other lines as they are."""
    glob, subckts, top = {}, {}, []
    cur = None
    for ln in lines:
        pl, exprs = _protect(ln)
        toks = _tokens(pl)
        if not toks:
            continue
        head = toks[0].lower()
        if head == ".subckt":
            pnames = [t for t in toks[2:] if "=" in t]
            nodes = [t for t in toks[2:] if "=" not in t and t.lower() != "params:"]
            cur = {"nodes": nodes, "params": [(k, _unprotect(v, exprs)) for k, v in _assignments(pnames)], "body": []}
            subckts[toks[1].lower()] = cur
            continue
        if head == ".ends":
            cur = None
            continue
        if head == ".param":
            for k, v in _assignments(toks[1:]):
                glob[k] = _unprotect(v, exprs)
            continue
        (cur["body"] if cur is not None else top).append(ln)
    out = []

    def emit(body, nodemap, prefix, scope):
        for ln in body:
            pl, exprs = _protect(ln)
            toks = _tokens(pl)
            head = toks[0].lower()
            if head.startswith("."):
                out.append(ln)
                continue
            if head[0] == "x":
                args = [t for t in toks[1:] if "=" not in t]
                sub = subckts.get(args[-1].lower())
                if sub is None:
                    raise ValueError("unknown subcircuit %r" % args[-1])
                actual = [nodemap.get(a, a if a == "0" else prefix + a) for a in args[:-1]]
                inner = dict(scope)
                over = {k: _num(_unprotect(v, exprs), scope) for k, v in _assignments(toks[1:])}
                for k, v in sub["params"]:
                    inner[k] = over[k] if k in over else _num(v, inner)
                m = dict(zip(sub["nodes"], actual))
                emit(sub["body"], m, prefix + toks[0] + ".", inner)
                continue
            # an element: rename nodes, evaluate expressions
            n_nodes = {"r": 2, "c": 2, "l": 2, "v": 2, "i": 2, "d": 2, "q": 4, "m": 4}.get(head[0], 2)
            new = [toks[0] + ("." + prefix[:-1] if prefix else "")]  # kind letter first: R1.XA.X1
            for k, t in enumerate(toks[1:]):
                if k < n_nodes and t not in ("(", ")") and "=" not in t and not t.startswith("@"):
                    new.append(nodemap.get(t, t if t == "0" else prefix + t))
                else:
                    new.append(_evaltok(t, exprs, scope))
            out.append(" ".join(new))

    scope0 = {k: v for k, v in glob.items()}
    emit(top, {}, "", scope0)
    return out


def _unprotect(v, exprs):
    m = re.fullmatch(r"@(\d+)@", v)
    return exprs[int(m.group(1))] if m else v


def _num(v, scope):
    m = _NUM.match(v.strip())
    if m and re.fullmatch(r"[a-zA-Z]*", m.group(2)):  # a plain number, with or without a suffix
        return value(v)
    return evaluate(v, scope)


def _evaltok(t, exprs, scope):
    if "@" not in t:
        return t
    if "=" in t:
        k, v = t.split("=", 1)
        return "%s=%r" % (k, _num(_unprotect(v, exprs), scope))
    return repr(_num(_unprotect(t, exprs), scope))


def parse(text):
    """Return (circuit dict, None) or (None, reason)."""
    try:
        return _parse(text)
    except (ValueError, IndexError, ZeroDivisionError) as e:
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
    lines = [ln.split(";", 1)[0] if ";" in ln else ln for ln in lines]
    lines = _expand(lines)
    ckt = {"title": raw[0].strip() if raw else "", "elements": [], "models": {}, "analyses": []}
    for ln in lines:
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
            # value | Q=pwl(v1 q1 ...) | FLUX=pwl(i1 l1 ...), [SCALE=wave(...)] [IC=x]
            # (netlist/parser.go:703-800)
            e = {"name": name, "kind": kind.upper(), "nodes": toks[1:3], "value": 0.0}
            rest, i, p, curve, scale = toks[3:], 0, {}, None, None
            while i < len(rest):
                t = rest[i]
                if "=" in t and i + 1 < len(rest) and rest[i + 1] == "(":
                    key, fn = t.lower().split("=", 1)
                    j, args = i + 2, []
                    while j < len(rest) and rest[j] != ")":
                        args.append(value(rest[j]))
                        j += 1
                    if key in ("q", "flux") and fn == "pwl":
                        curve = args
                    elif key == "scale" and fn in ("pulse", "sin", "exp", "pwl"):
                        scale = (fn, args)
                    else:
                        return None, "unsupported %s=%s on %s" % (key, fn, name)
                    i = j + 1
                elif "=" in t:
                    k, v = t.split("=", 1)
                    p[k.lower()] = value(v)
                    i += 1
                else:
                    e["value"] = value(t)
                    i += 1
            if set(p) - {"ic"}:
                return None, "unsupported parameter on " + name
            if "ic" in p:
                e["ic"] = p["ic"]
            if curve is not None or scale is not None:
                e["kind"] = kind.upper() + "N"
                e["curve"] = curve or []
                e["scale"] = scale[0] if scale else None
                e["scale_args"] = scale[1] if scale else []
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
        elif kind in "eg":  # E/G n+ n- nc+ nc- gain
            ckt["elements"].append({"name": name, "kind": kind.upper(), "nodes": toks[1:3], "ctrl_nodes": toks[3:5],
                                    "value": value(toks[5])})
        elif kind in "fh":  # F/H n+ n- vcontrol gain
            ckt["elements"].append({"name": name, "kind": kind.upper(), "nodes": toks[1:3], "ctrl_source": toks[3],
                                    "value": value(toks[4])})
        elif kind == "k":  # K L1 L2 k
            ckt["elements"].append({"name": name, "kind": "K", "couples": toks[1:3], "value": value(toks[3])})
        elif kind in "sw":  # S n+ n- nc+ nc- model [ON|OFF]; W n+ n- vname model [ON|OFF] (netlist/parser.go:480-501)
            t = toks[1:]
            init = None
            if t and t[-1].lower() in ("on", "off"):
                init = t[-1].lower()
                t = t[:-1]
            if len(t) != (5 if kind == "s" else 4):
                return None, "bad switch line " + name
            e = {"name": name, "kind": kind.upper(), "nodes": t[0:2], "model": t[-1].lower(),
                 "ic": 1.0 if init == "on" else 0.0, "has_ic": init is not None}
            if kind == "s":
                e["ctrl_nodes"] = t[2:4]
            else:
                e["ctrl_source"] = t[2]
            ckt["elements"].append(e)
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


class NetlistError(ValueError):
    """A netlist outside the subset this reader takes, or a malformed one."""


def read(text):
    """circuit.FromDeck (circuit/builder.go:307): the Circuit of a netlist and its
    analysis lines (dicts: kind "op", "dc", "tran" or "ac" with their fields)."""
    from .circuit import from_dict
    try:
        d, why = parse(text)
    except (ValueError, IndexError, KeyError) as e:
        raise NetlistError("netlist: %s" % e)
    if d is None:
        raise NetlistError("netlist: %s" % why)
    return from_dict(d), list(d["analyses"])
