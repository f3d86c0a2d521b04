"""Circuit model and builder: the host-side mirror of kronspice's circuit package.

``Builder`` follows circuit.Builder (circuit/builder.go:17-295): nodes by
case-insensitive name, "0" and "gnd" are ground, elements in insertion order
(which fixes the MNA unknown layout, device/device.go:36-100), models by name.

``Circuit.pack()`` turns a circuit into the C-ABI form of include/kronspice_gpu.h:
a topology (element kinds, node indices, flags) and one value vector.  It applies
the model-card defaults, aliases and area scaling that NewDiode
(device/diode.go:85-128), NewBJT (device/bjt.go:143-241) and NewMOSFET
(device/mosfet.go:129-214) apply, so the engine receives final parameters.
Circuits whose topology keys are equal can share one plan in a batch.
"""
import math

import numpy as np

KIND = {"R": 1, "C": 2, "L": 3, "V": 4, "I": 5, "D": 6, "Q": 7, "M": 8, "E": 9, "F": 10, "G": 11, "H": 12,
        "K": 13, "S": 14, "W": 15, "CN": 16, "LN": 17}
WAVE = {None: 0, "pulse": 1, "sin": 2, "exp": 3, "pwl": 4}

F_HAS_DC, F_HAS_IC, F_HAS_BV, F_PTYPE = 1, 2, 4, 8
F_INT_A, F_INT_C, F_INT_B, F_INT_E, F_INT_D, F_INT_S, F_LATERAL = 16, 32, 64, 128, 256, 512, 1024

# ks_element of include/kronspice_gpu.h (48 bytes)
ELEMENT_DTYPE = np.dtype({
    "names": ["kind", "node", "flags", "level", "wave", "nargs", "param", "given"],
    "formats": ["<i4", ("<i4", 4), "<i4", "<i4", "<i4", "<i4", "<i4", "<u8"],
    "offsets": [0, 4, 20, 24, 28, 32, 36, 40],
    "itemsize": 48,
})

D_KEYS = ["is", "n", "rs", "cjo", "vj", "m", "tt", "bv", "ibv", "fc"]
Q_KEYS = ["is", "bf", "nf", "vaf", "ikf", "ise", "ne", "br", "nr", "var", "ikr", "isc", "nc",
          "rb", "irb", "rbm", "re", "rc", "cje", "vje", "mje", "tf", "xtf", "vtf", "itf", "cjc",
          "vjc", "mjc", "xcjc", "tr", "cjs", "vjs", "mjs", "fc", "iss", "ns", "subs"]
M_KEYS = ["vto", "kp", "gamma", "phi", "lambda", "rd", "rs", "cbd", "cbs", "is", "pb", "cgso",
          "cgdo", "cgbo", "rsh", "cj", "mj", "cjsw", "mjsw", "js", "tox", "nsub", "nss", "nfs",
          "tpg", "xj", "ld", "uo", "ucrit", "uexp", "utra", "vmax", "neff", "fc", "delta",
          "theta", "eta", "kappa", "wd", "l", "w", "ad", "as", "pd", "ps", "nrd", "nrs", "m"]
M_INSTANCE = ["l", "w", "ad", "as", "pd", "ps", "nrd", "nrs", "m"]
M_GET = {"vto": ["vto", "vt0"], "uo": ["uo", "u0"]}
Q_GET = {"vaf": ["vaf", "va"], "ikf": ["ikf", "ik"], "var": ["var", "vb"], "vje": ["vje", "pe"],
         "mje": ["mje", "me"], "vjc": ["vjc", "pc"], "mjc": ["mjc", "mc"], "cjs": ["cjs", "ccs"],
         "vjs": ["vjs", "ps"], "mjs": ["mjs", "ms"]}
NP = {"R": 2, "C": 2, "L": 2, "D": len(D_KEYS), "Q": len(Q_KEYS), "M": len(M_KEYS)}


class CircuitError(ValueError):
    """A malformed builder call (the engine's structural checks are ks_validate)."""


class Element:
    __slots__ = ("name", "kind", "nodes", "value", "ic", "has_ic", "dc", "has_dc", "wave", "args",
                 "ac", "model", "area", "params", "ctrl", "couples", "curve")

    def __init__(self, name, kind, nodes, **kw):
        self.name, self.kind, self.nodes = name, kind, list(nodes)
        self.value = kw.get("value", 0.0)
        self.ic, self.has_ic = kw.get("ic", 0.0), kw.get("has_ic", False)
        self.dc, self.has_dc = kw.get("dc", 0.0), kw.get("has_dc", False)
        self.wave, self.args = kw.get("wave"), list(kw.get("args", []))
        self.ac = list(kw.get("ac", [0.0, 0.0]))
        self.model, self.area = kw.get("model"), kw.get("area", 0.0)
        self.params = dict(kw.get("params") or {})
        self.ctrl = kw.get("ctrl")            # F, H, W: the controlling voltage source's name
        self.couples = kw.get("couples")      # K: the two inductors' names
        self.curve = [float(v) for v in kw.get("curve") or []]  # CN, LN: Q=pwl / FLUX=pwl knots x0, y0, ...


class Builder:
    """Programmatic circuit construction (circuit.Builder)."""

    def __init__(self, title=""):
        self.title = title
        self.index = {"0": 0, "gnd": 0}
        self.names = ["0"]
        self.elems = []
        self.models = {}

    def node(self, name):
        key = str(name).strip().lower()
        if key not in self.index:
            self.index[key] = len(self.names)
            self.names.append(key)
        return self.index[key]

    def _add(self, e):
        for n in e.nodes:
            self.node(n)
        self.elems.append(e)
        return self

    def resistor(self, name, a, b, ohms):
        return self._add(Element(name, "R", [a, b], value=float(ohms)))

    def capacitor(self, name, a, b, farads, ic=None, curve=None, scale=None, scale_args=()):
        """A capacitor; with a charge curve (Q=pwl, farads 0) or a SCALE waveform
        it is circuit.NonlinearCapacitor, q = s(t) Q(v)."""
        kind = "CN" if curve or scale else "C"
        return self._add(Element(name, kind, [a, b], value=float(farads), ic=ic or 0.0, has_ic=ic is not None,
                                 curve=curve, wave=scale, args=scale_args))

    def inductor(self, name, a, b, henries, ic=None, curve=None, scale=None, scale_args=()):
        """An inductor; with a flux curve (FLUX=pwl, henries 0) or a SCALE waveform
        it is circuit.NonlinearInductor, flux linkage s(t) L(i)."""
        kind = "LN" if curve or scale else "L"
        return self._add(Element(name, kind, [a, b], value=float(henries), ic=ic or 0.0, has_ic=ic is not None,
                                 curve=curve, wave=scale, args=scale_args))

    def voltage_source(self, name, plus, minus, volts, wave=None, args=(), has_dc=True, ac=(0.0, 0.0)):
        return self._add(Element(name, "V", [plus, minus], dc=float(volts), has_dc=has_dc, wave=wave,
                                 args=args, ac=ac))

    def current_source(self, name, plus, minus, amps, wave=None, args=(), has_dc=True, ac=(0.0, 0.0)):
        return self._add(Element(name, "I", [plus, minus], dc=float(amps), has_dc=has_dc, wave=wave,
                                 args=args, ac=ac))

    def voltage_wave(self, name, plus, minus, wave, args):
        return self.voltage_source(name, plus, minus, 0.0, wave=wave, args=args, has_dc=False)

    def current_wave(self, name, plus, minus, wave, args):
        return self.current_source(name, plus, minus, 0.0, wave=wave, args=args, has_dc=False)

    def vcvs(self, name, plus, minus, ctrl_plus, ctrl_minus, gain):
        """E: V(n+) - V(n-) = gain (V(nc+) - V(nc-)) (device/controlled.go:15-23)."""
        return self._add(Element(name, "E", [plus, minus, ctrl_plus, ctrl_minus], value=float(gain)))

    def vccs(self, name, plus, minus, ctrl_plus, ctrl_minus, gain):
        """G: i(n+ -> n-) = gain (V(nc+) - V(nc-))."""
        return self._add(Element(name, "G", [plus, minus, ctrl_plus, ctrl_minus], value=float(gain)))

    def cccs(self, name, plus, minus, source, gain):
        """F: i(n+ -> n-) = gain I(source), I positive into the source's n+ terminal."""
        return self._add(Element(name, "F", [plus, minus], value=float(gain), ctrl=source))

    def ccvs(self, name, plus, minus, source, gain):
        """H: V(n+) - V(n-) = gain I(source)."""
        return self._add(Element(name, "H", [plus, minus], value=float(gain), ctrl=source))

    def mutual(self, name, inductor1, inductor2, k):
        """K: mutual inductance k sqrt(L1 L2) between two inductors (device/mutual.go:15-29)."""
        return self._add(Element(name, "K", [], value=float(k), couples=[inductor1, inductor2]))

    def vswitch(self, name, a, b, ctrl_plus, ctrl_minus, model, on=None):
        """Voltage-controlled switch (SPICE S, circuit/switch.go:81-86) with a model
        of type "sw"; on: the initial state (None: OFF, as when no IC is given)."""
        return self._add(Element(name, "S", [a, b, ctrl_plus, ctrl_minus], model=model.lower(),
                                 ic=1.0 if on else 0.0, has_ic=on is not None))

    def iswitch(self, name, a, b, source, model, on=None):
        """Current-controlled switch (SPICE W, circuit/switch.go:88-94) with a model
        of type "csw", set by the current of voltage source `source`."""
        return self._add(Element(name, "W", [a, b], model=model.lower(), ctrl=source,
                                 ic=1.0 if on else 0.0, has_ic=on is not None))

    def model(self, name, typ, params):
        self.models[name.lower()] = (typ.lower(), {k.lower(): float(v) for k, v in params.items()})
        return self

    def diode(self, name, anode, cathode, model, area=0.0):
        return self._add(Element(name, "D", [anode, cathode], model=model.lower(), area=area))

    def bjt(self, name, collector, base, emitter, model, substrate=None, area=0.0):
        nodes = [collector, emitter, base] + ([substrate] if substrate is not None else [])
        return self._add(Element(name, "Q", nodes, model=model.lower(), area=area))

    def mosfet(self, name, drain, gate, source, bulk, model, params=None):
        p = {k.lower(): float(v) for k, v in (params or {}).items()}
        return self._add(Element(name, "M", [drain, source, gate, bulk], model=model.lower(), params=p))

    def build(self):
        return Circuit(self.title, list(self.names), list(self.elems), dict(self.models))


class Circuit:
    def __init__(self, title, node_names, elements, models):
        self.title, self.node_names, self.elements, self.models = title, node_names, elements, models
        self._idx = {n: i for i, n in enumerate(node_names)}
        self._idx["gnd"] = 0

    @property
    def n_nodes(self):
        return len(self.node_names)

    def node_index(self, name):
        return self._idx.get(str(name).lower(), -1)

    def element_index(self, name):
        for i, e in enumerate(self.elements):
            if e.name.lower() == name.lower():
                return i
        return -1

    def pack(self):
        """Return (elements ndarray[ELEMENT_DTYPE], values float64 ndarray, key)."""
        el = np.zeros(len(self.elements), dtype=ELEMENT_DTYPE)
        vals = []
        for k, e in enumerate(self.elements):
            r = el[k]
            r["kind"] = KIND[e.kind]
            nodes = [self.node_index(n) for n in e.nodes]
            if any(n < 0 for n in nodes):
                raise CircuitError("%s: unknown node" % e.name)
            if e.kind in ("F", "H", "W"):  # node[2]: the controlling source, by element index
                j = self.element_index(e.ctrl)
                if j < 0:
                    raise CircuitError("%s: controlling source %s not found" % (e.name, e.ctrl))
                nodes = nodes[:2] + [j]
            elif e.kind == "K":  # node[0..1]: the coupled inductors, by element index
                nodes = [self.element_index(x) for x in e.couples]
                if any(n < 0 for n in nodes):
                    raise CircuitError("%s: inductor not found" % e.name)
            nn = nodes + [0] * (4 - len(nodes))
            r["node"] = nn
            r["param"] = len(vals)
            flags = 0
            if e.kind in ("E", "F", "G", "H", "K"):
                vals += [e.value]
            elif e.kind in ("S", "W"):
                vals += self._switch(e)
            elif e.kind in ("CN", "LN"):
                if e.has_ic:
                    flags |= F_HAS_IC
                r["wave"] = WAVE[e.wave]
                r["nargs"] = len(e.args)
                r["level"] = len(e.curve)
                vals += [e.value, e.ic] + [float(a) for a in e.args] + e.curve
            elif e.kind in ("R", "C", "L"):
                if e.kind != "R" and e.has_ic:
                    flags |= F_HAS_IC
                vals += [e.value, e.ic]
            elif e.kind in ("V", "I"):
                if e.has_dc:
                    flags |= F_HAS_DC
                r["wave"] = WAVE[e.wave]
                r["nargs"] = len(e.args)
                vals += [e.dc, e.ac[0], e.ac[1]] + [float(a) for a in e.args]
            elif e.kind == "D":
                p, hbv = self._diode(e)
                if hbv:
                    flags |= F_HAS_BV
                if p[2] > 0:
                    flags |= F_INT_A
                vals += p
            elif e.kind == "Q":
                p, pnp = self._bjt(e)
                if pnp:
                    flags |= F_PTYPE
                if p[Q_KEYS.index("rc")] > 0:
                    flags |= F_INT_C
                if p[Q_KEYS.index("rb")] > 0:
                    flags |= F_INT_B
                if p[Q_KEYS.index("re")] > 0:
                    flags |= F_INT_E
                if p[Q_KEYS.index("subs")] < 0:
                    flags |= F_LATERAL
                vals += p
            elif e.kind == "M":
                p, given, level, pmos, intd, ints = self._mos(e)
                if pmos:
                    flags |= F_PTYPE
                if intd:
                    flags |= F_INT_D
                if ints:
                    flags |= F_INT_S
                r["level"] = level
                r["given"] = given
                vals += p
            r["flags"] = flags
        key = (self.n_nodes, el.tobytes())
        return el, np.asarray(vals, dtype=np.float64), key

    def _model(self, e, want):
        if e.model not in self.models:
            raise CircuitError("%s uses undefined model %r" % (e.name, e.model))
        typ, params = self.models[e.model]
        if typ not in want:
            raise CircuitError("%s needs a %s model, %r is type %s" % (e.name, "/".join(want), e.model, typ))
        return typ, params

    def _switch(self, e):
        """[VT or IT, VH or IH, RON, ROFF, initial state]: circuit.SwitchParams
        (circuit/switch.go:36-50) with the ngspice defaults RON = 1, ROFF = 1e12."""
        typ, mp = self._model(e, ("sw",) if e.kind == "S" else ("csw",))
        vt, vh = (mp.get("vt", 0.0), mp.get("vh", 0.0)) if typ == "sw" else (mp.get("it", 0.0), mp.get("ih", 0.0))
        return [vt, vh, mp.get("ron", 1.0), mp.get("roff", 1e12), e.ic if e.has_ic else 0.0]

    def _diode(self, e):
        _, mp = self._model(e, ("d",))
        p = dict(zip(D_KEYS, [1e-14, 1.0, 0.0, 0.0, 1.0, 0.5, 0.0, 0.0, 1e-3, 0.5]))
        for k in ("is", "n", "rs", "cjo", "vj", "m", "tt", "ibv", "fc"):
            if k in mp:
                p[k] = mp[k]
        if "cj0" in mp:
            p["cjo"] = mp["cj0"]
        has_bv = "bv" in mp
        if has_bv:
            p["bv"] = mp["bv"]
        area = e.area or 1.0
        p["is"] *= area
        p["cjo"] *= area
        p["ibv"] *= area
        if p["rs"] > 0:
            p["rs"] /= area
        return [p[k] for k in D_KEYS], has_bv

    def _bjt(self, e):
        typ, mp = self._model(e, ("npn", "pnp"))
        p = {k: 0.0 for k in Q_KEYS}
        p.update({"is": 1e-16, "bf": 100.0, "nf": 1.0, "ne": 1.5, "br": 1.0, "nr": 1.0, "nc": 2.0,
                  "vje": 0.75, "mje": 0.33, "vjc": 0.75, "mjc": 0.33, "xcjc": 1.0, "vjs": 0.75,
                  "fc": 0.5, "ns": 1.0})
        pnp = typ == "pnp"
        for k in Q_KEYS:  # get(dst, keys...) of device/bjt.go:148-155: first key present wins
            if k == "rbm":
                continue
            for kk in Q_GET.get(k, [k]):
                if kk in mp:
                    p[k] = mp[kk]
                    break
        p["rbm"] = p["rb"]
        if "rbm" in mp:
            p["rbm"] = mp["rbm"]
        if p["subs"] == 0:
            p["subs"] = -1.0 if pnp else 1.0
        if p["rbm"] > p["rb"]:
            p["rbm"] = p["rb"]
        area = e.area or 1.0
        for k in ("is", "ise", "isc", "ikf", "ikr", "irb", "itf", "cje", "cjc", "cjs", "iss"):
            p[k] *= area
        for k in ("rb", "rbm", "re", "rc"):
            p[k] /= area
        return [p[k] for k in Q_KEYS], pnp

    def _mos(self, e):
        typ, mp = self._model(e, ("nmos", "pmos"))
        level = int(mp.get("level", 1))
        if level not in (1, 2, 3):
            raise CircuitError("%s: LEVEL must be 1, 2 or 3" % e.model)
        p = {k: 0.0 for k in M_KEYS}
        p.update({"kp": 2e-5, "phi": 0.6, "is": 1e-14, "pb": 0.8, "mj": 0.5, "mjsw": 0.5, "uo": 600.0,
                  "fc": 0.5, "ucrit": 1e4, "neff": 1.0, "delta": 0.0, "tpg": 1.0, "l": 100e-6,
                  "w": 100e-6, "m": 1.0})
        given = 0
        if level >= 2:
            p["mjsw"] = 0.33
            p["tox"] = 1e-7
            given |= 1 << M_KEYS.index("tox")
        for k in M_KEYS:  # set(dst, keys...) of device/mosfet.go:150-158
            if k in M_INSTANCE:
                continue
            for kk in M_GET.get(k, [k]):
                if kk in mp:
                    p[k] = mp[kk]
                    given |= 1 << M_KEYS.index(k)
                    break
        if level == 3 and "kappa" not in mp:
            p["kappa"] = 0.2
        for k in M_INSTANCE:
            if k in e.params:
                p[k] = e.params[k]
        rd, rs = p["rd"], p["rs"]
        if not (given >> M_KEYS.index("rd")) & 1 and p["rsh"] > 0:
            rd = p["rsh"] * p["nrd"]
        if not (given >> M_KEYS.index("rs")) & 1 and p["rsh"] > 0:
            rs = p["rsh"] * p["nrs"]
        return [p[k] for k in M_KEYS], given, level, typ == "pmos", rd > 0, rs > 0


def from_dict(d):
    """Build a Circuit from the dict form of tests/golden/spice_subset.py."""
    b = Builder(d.get("title", ""))
    for name, m in d["models"].items():
        b.model(name, m["type"], {k: v for k, v in m["params"].items()})
    for e in d["elements"]:
        k = e["kind"]
        if k == "R":
            b.resistor(e["name"], *e["nodes"], e["value"])
        elif k in ("C", "CN"):
            b.capacitor(e["name"], *e["nodes"], e["value"], e.get("ic"), curve=e.get("curve"),
                        scale=e.get("scale"), scale_args=e.get("scale_args", ()))
        elif k in ("L", "LN"):
            b.inductor(e["name"], *e["nodes"], e["value"], e.get("ic"), curve=e.get("curve"),
                       scale=e.get("scale"), scale_args=e.get("scale_args", ()))
        elif k in ("V", "I"):
            f = b.voltage_source if k == "V" else b.current_source
            f(e["name"], *e["nodes"], e["dc"], wave=e["wave"], args=e["args"], has_dc=e["has_dc"],
              ac=e.get("ac", (0.0, 0.0)))
        elif k == "D":
            b.diode(e["name"], *e["nodes"], e["model"], e.get("area", 0.0))
        elif k == "Q":
            n = e["nodes"]
            b.bjt(e["name"], n[0], n[1], n[2], e["model"], substrate=n[3] if len(n) > 3 else None,
                  area=e.get("area", 0.0))
        elif k == "M":
            n = e["nodes"]
            b.mosfet(e["name"], n[0], n[1], n[2], n[3], e["model"], e.get("params"))
        elif k in ("E", "G"):
            f = b.vcvs if k == "E" else b.vccs
            f(e["name"], *e["nodes"], *e["ctrl_nodes"], e["value"])
        elif k in ("F", "H"):
            f = b.cccs if k == "F" else b.ccvs
            f(e["name"], *e["nodes"], e["ctrl_source"], e["value"])
        elif k == "K":
            b.mutual(e["name"], e["couples"][0], e["couples"][1], e["value"])
        elif k in ("S", "W"):
            on = (e["ic"] == 1) if e.get("has_ic") else None
            if k == "S":
                b.vswitch(e["name"], *e["nodes"], *e["ctrl_nodes"], e["model"], on=on)
            else:
                b.iswitch(e["name"], *e["nodes"], e["ctrl_source"], e["model"], on=on)
    return b.build()


def isfinite_all(vals):
    return all(math.isfinite(v) for v in vals)
