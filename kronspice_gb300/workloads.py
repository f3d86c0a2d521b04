"""Seeded synthetic batches with the shapes of the engine's benchmark workloads.

Each generator returns (elements, n_nodes, values[n_circ][n_values]) ready for
Plan/Batch: one template circuit is built with the Builder and packed, then the
per-circuit values are written column-wise with numpy, so 10^5 circuits cost
milliseconds.  Random numbers come from numpy's counter-based Philox generator
keyed by (workload id, seed), so every run and every host gets the same inputs.
"""
import numpy as np

from .circuit import Builder, D_KEYS, Q_KEYS, M_KEYS


def rng(workload_id, seed=0):
    return np.random.Generator(np.random.Philox(key=[int(workload_id), int(seed)]))


def log_uniform(g, lo, hi, n):
    return np.exp(g.uniform(np.log(lo), np.log(hi), n))


def _offsets(circuit):
    el, vals, _ = circuit.pack()
    names = [e.name for e in circuit.elements]
    return el, vals, {nm: int(el[i]["param"]) for i, nm in enumerate(names)}


# ------------------------------------------------------------------ BJT CE operating point
def bjt_ce_template():
    """Single-stage common-emitter amplifier: Vcc, bias divider R1/R2, RC, RE, one NPN.
    No RB/RC/RE model resistances, so the system has 5 unknowns (vcc, b, c, e, I(Vcc))."""
    b = Builder("bjt common emitter")
    b.voltage_source("VCC", "vcc", "0", 12.0)
    b.resistor("R1", "vcc", "b", 47e3)
    b.resistor("R2", "b", "0", 10e3)
    b.resistor("RC", "vcc", "c", 3.3e3)
    b.resistor("RE", "e", "0", 1e3)
    b.model("qn", "npn", {"is": 1e-15, "bf": 100})
    b.bjt("Q1", "c", "b", "e", "qn")
    return b.build()


def bjt_ce_batch(n_circ, seed=0):
    """IS log-U[1e-16, 1e-14] A, BF U[50, 300], R1 R2 RC RE log-U[100, 1e6] ohm, Vcc U[5, 15] V."""
    c = bjt_ce_template()
    el, v0, off = _offsets(c)
    g = rng(2, seed)
    vals = np.tile(v0, (n_circ, 1))
    vals[:, off["Q1"] + Q_KEYS.index("is")] = log_uniform(g, 1e-16, 1e-14, n_circ)
    vals[:, off["Q1"] + Q_KEYS.index("bf")] = g.uniform(50, 300, n_circ)
    for r in ("R1", "R2", "RC", "RE"):
        vals[:, off[r]] = log_uniform(g, 1e2, 1e6, n_circ)
    vals[:, off["VCC"]] = g.uniform(5, 15, n_circ)
    return el, c.n_nodes, vals


def bjt_ce_features(vals, el):
    """The 7-D parameter vector of each circuit (log scales), the learned start's input."""
    off = {int(e["kind"]): None for e in el}
    p_q = int(el[5]["param"])
    cols = [np.log(vals[:, p_q + Q_KEYS.index("is")]), vals[:, p_q + Q_KEYS.index("bf")] / 100.0]
    for k in range(1, 5):
        cols.append(np.log(vals[:, int(el[k]["param"])]))
    cols.append(vals[:, int(el[0]["param"])] / 10.0)
    del off
    return np.stack(cols, axis=1)


# ------------------------------------------------------------------ BJT CE small-signal sweep
BJT_CE_AC_MODEL = {"is": 2e-15, "bf": 150.0, "vaf": 80.0, "ikf": 0.05, "rb": 120.0, "rbm": 40.0, "re": 0.8,
                   "rc": 6.0, "cje": 1.2e-11, "vje": 0.75, "mje": 0.35, "tf": 3e-10, "xtf": 3.0, "vtf": 4.0,
                   "itf": 0.04, "cjc": 5e-12, "vjc": 0.6, "mjc": 0.4, "xcjc": 0.6, "tr": 1e-08, "cjs": 3e-12,
                   "vjs": 0.7, "mjs": 0.3}


def bjt_ce_ac_template():
    """Common-emitter amplifier with input coupling and emitter bypass capacitors and a
    Gummel-Poon transistor with base, emitter and collector resistances and junction,
    transit-time and substrate charges (the shape of the reference's bjt_ce_ac netlist):
    10 unknowns (vcc, in, b, c, e, three internal transistor nodes, two source branches)."""
    b = Builder("bjt common emitter, small signal")
    b.voltage_source("VCC", "vcc", "0", 12.0)
    b.voltage_source("VIN", "in", "0", 0.0, ac=(1.0, 0.0))
    b.capacitor("CIN", "in", "b", 10e-6)
    b.resistor("R1", "vcc", "b", 47e3)
    b.resistor("R2", "b", "0", 10e3)
    b.resistor("RC", "vcc", "c", 3.3e3)
    b.resistor("RE", "e", "0", 1e3)
    b.capacitor("CE", "e", "0", 100e-6)
    b.model("qac", "npn", dict(BJT_CE_AC_MODEL))
    b.bjt("Q1", "c", "b", "e", "qac")
    return b.build()


def bjt_ce_ac_batch(n_circ, seed=0):
    """Bias divider R1 log-U[20k, 100k], R2 log-U[5k, 20k], RC log-U[1k, 10k], RE log-U[300, 3k] ohm,
    Vcc U[5, 15] V, IS log-U[1e-16, 1e-14] A, BF U[50, 300], CJE / CJC / TF x log-U[0.5, 2]."""
    c = bjt_ce_ac_template()
    el, v0, off = _offsets(c)
    g = rng(6, seed)
    vals = np.tile(v0, (n_circ, 1))
    q = off["Q1"]
    vals[:, q + Q_KEYS.index("is")] = log_uniform(g, 1e-16, 1e-14, n_circ)
    vals[:, q + Q_KEYS.index("bf")] = g.uniform(50, 300, n_circ)
    for k in ("cje", "cjc", "tf"):
        vals[:, q + Q_KEYS.index(k)] *= log_uniform(g, 0.5, 2.0, n_circ)
    for r, lo, hi in (("R1", 20e3, 100e3), ("R2", 5e3, 20e3), ("RC", 1e3, 10e3), ("RE", 300, 3e3)):
        vals[:, off[r]] = log_uniform(g, lo, hi, n_circ)
    vals[:, off["VCC"]] = g.uniform(5, 15, n_circ)
    return el, c.n_nodes, vals


# ------------------------------------------------------------------ RC ladder transient
def rc_ladder_template(sections=10):
    """V1 PULSE(0 1 0 1n 1n 1u) driving `sections` series-R shunt-C sections."""
    b = Builder("rc ladder")
    b.voltage_wave("V1", "n0", "0", "pulse", [0, 1, 0, 1e-9, 1e-9, 1e-6])
    for k in range(1, sections + 1):
        b.resistor("R%d" % k, "n%d" % (k - 1), "n%d" % k, 1e3)
        b.capacitor("C%d" % k, "n%d" % k, "0", 1e-9)
    return b.build()


def rc_ladder_batch(n_circ, seed=0, sections=10):
    """R log-U[100, 1e5] ohm, C log-U[1 pF, 1 uF] per section."""
    c = rc_ladder_template(sections)
    el, v0, off = _offsets(c)
    g = rng(1, seed)
    vals = np.tile(v0, (n_circ, 1))
    for k in range(1, sections + 1):
        vals[:, off["R%d" % k]] = log_uniform(g, 1e2, 1e5, n_circ)
        vals[:, off["C%d" % k]] = log_uniform(g, 1e-12, 1e-6, n_circ)
    return el, c.n_nodes, vals


# ------------------------------------------------------------------ two-stage CMOS op-amp operating point
OPAMP_DEVICES = ["M1", "M2", "M3", "M4", "M5", "M6", "M7", "M8"]
OPAMP_NMOS = ["M1", "M2", "M5", "M7", "M8"]


def cmos_opamp_template():
    """Two-stage Miller op-amp in unity-gain feedback (level-1 MOSFETs): NMOS input
    pair M1/M2 with PMOS mirror load M3/M4 and tail M5, PMOS common-source second
    stage M6 with NMOS current-source load M7, bias mirror M8 fed by RB, Miller
    capacitor CC and load CL.  The output drives the inverting input, the gate of
    M1 (the input on the mirror's diode side: raising it lowers v(out) through the
    mirror and the inverting second stage), and VCM the non-inverting gate of M2.
    The loop is negative feedback, so the operating point is unique: v(out)
    follows VCM.  (Fed back to M2's gate, the loop would be positive and every
    variant would have three operating points, two of them at the rails.)"""
    b = Builder("two-stage cmos op-amp")
    b.voltage_source("VDD", "vdd", "0", 5.0)
    b.voltage_source("VCM", "inp", "0", 2.5)
    b.resistor("RB", "vdd", "nb", 100e3)
    b.model("nch", "nmos", {"level": 1, "vto": 0.6, "kp": 100e-6, "lambda": 0.04, "gamma": 0.4, "phi": 0.7})
    b.model("pch", "pmos", {"level": 1, "vto": -0.6, "kp": 40e-6, "lambda": 0.05, "gamma": 0.45, "phi": 0.7})
    L = 1e-6
    b.mosfet("M1", "n1", "out", "tail", "0", "nch", {"l": L, "w": 10 * L})
    b.mosfet("M2", "n2", "inp", "tail", "0", "nch", {"l": L, "w": 10 * L})
    b.mosfet("M3", "n1", "n1", "vdd", "vdd", "pch", {"l": L, "w": 20 * L})
    b.mosfet("M4", "n2", "n1", "vdd", "vdd", "pch", {"l": L, "w": 20 * L})
    b.mosfet("M5", "tail", "nb", "0", "0", "nch", {"l": L, "w": 20 * L})
    b.mosfet("M6", "out", "n2", "vdd", "vdd", "pch", {"l": L, "w": 80 * L})
    b.mosfet("M7", "out", "nb", "0", "0", "nch", {"l": L, "w": 40 * L})
    b.mosfet("M8", "nb", "nb", "0", "0", "nch", {"l": L, "w": 10 * L})
    b.capacitor("CC", "n2", "out", 2e-12)
    b.capacitor("CL", "out", "0", 10e-12)
    return b.build()


OPAMP_FEATURES = (["w/l %s" % m for m in OPAMP_DEVICES] +
                  ["vto n", "vto p", "kp n", "kp p", "lambda n", "lambda p", "gamma n", "gamma p", "phi n", "phi p",
                   "rb", "cc", "cl", "vdd", "vcm", "l"])


def cmos_opamp_batch(n_circ, seed=0):
    """24-D parameter vector per variant: W/L of the 8 devices log-U[1, 100]; VTO
    U[0.4, 0.8] V (PMOS negative); KP log-U[20, 200] uA/V^2; LAMBDA U[0.01, 0.1];
    GAMMA U[0.3, 0.6]; PHI U[0.6, 0.8]; RB log-U[10 k, 1 M]; CC log-U[0.1, 10] pF;
    CL log-U[1, 100] pF; VDD U[3, 5] V; VCM U[0.4, 0.6] VDD; L log-U[0.5, 5] um."""
    c = cmos_opamp_template()
    el, v0, off = _offsets(c)
    g = rng(4, seed)
    vals = np.tile(v0, (n_circ, 1))
    k = M_KEYS.index
    L = log_uniform(g, 0.5e-6, 5e-6, n_circ)
    wl = {m: log_uniform(g, 1.0, 100.0, n_circ) for m in OPAMP_DEVICES}
    vto = {"n": g.uniform(0.4, 0.8, n_circ), "p": -g.uniform(0.4, 0.8, n_circ)}
    kp = {"n": log_uniform(g, 20e-6, 200e-6, n_circ), "p": log_uniform(g, 20e-6, 200e-6, n_circ)}
    lam = {"n": g.uniform(0.01, 0.1, n_circ), "p": g.uniform(0.01, 0.1, n_circ)}
    gam = {"n": g.uniform(0.3, 0.6, n_circ), "p": g.uniform(0.3, 0.6, n_circ)}
    phi = {"n": g.uniform(0.6, 0.8, n_circ), "p": g.uniform(0.6, 0.8, n_circ)}
    for m in OPAMP_DEVICES:
        t = "n" if m in OPAMP_NMOS else "p"
        p = off[m]
        vals[:, p + k("l")] = L
        vals[:, p + k("w")] = wl[m] * L
        vals[:, p + k("vto")] = vto[t]
        vals[:, p + k("kp")] = kp[t]
        vals[:, p + k("lambda")] = lam[t]
        vals[:, p + k("gamma")] = gam[t]
        vals[:, p + k("phi")] = phi[t]
    vals[:, off["RB"]] = log_uniform(g, 1e4, 1e6, n_circ)
    vals[:, off["CC"]] = log_uniform(g, 0.1e-12, 10e-12, n_circ)
    vals[:, off["CL"]] = log_uniform(g, 1e-12, 100e-12, n_circ)
    vdd = g.uniform(3.0, 5.0, n_circ)
    vals[:, off["VDD"]] = vdd
    vals[:, off["VCM"]] = vdd * g.uniform(0.4, 0.6, n_circ)
    return el, c.n_nodes, vals


def cmos_opamp_feature_columns(el):
    """Value columns of the 24-D parameter vector (and which are log-scaled)."""
    c = cmos_opamp_template()
    names = [e.name for e in c.elements]
    off = {nm: int(el[i]["param"]) for i, nm in enumerate(names)}
    k = M_KEYS.index
    cols, logs = [], []
    for m in OPAMP_DEVICES:   # W/L enters through W (L is its own feature)
        cols.append(off[m] + k("w")); logs.append(True)
    for key in ("vto", "kp", "lambda", "gamma", "phi"):
        cols.append(off["M1"] + k(key)); logs.append(key == "kp")
        cols.append(off["M3"] + k(key)); logs.append(key == "kp")
    cols += [off["RB"], off["CC"], off["CL"], off["VDD"], off["VCM"], off["M1"] + k("l")]
    logs += [True, True, True, False, False, True]
    return cols, logs, off["VDD"]


# ------------------------------------------------------------------ random netlists
def random_netlist(g, k, nodes=(10, 400)):
    """One connected netlist: U{10..400} nodes, mean degree U[2, 6], a random
    spanning tree of resistors and inductors (edges at ground resistive, so the
    source and the inductors close no loop at DC) plus extra R / C / diode
    edges, 10 % of all elements diodes (IS 1e-14, N U[1, 2]), one SIN source
    (1 V, 1 kHz - 1 MHz) at node n1.  R log-U[1, 1e6] ohm, C log-U[1 pF, 1 uF],
    L log-U[1 nH, 1 mH]."""
    N = int(g.integers(nodes[0], nodes[1] + 1))
    deg = g.uniform(2.0, 6.0)
    E = max(N, int(round(deg * (N + 1) / 2)))
    b = Builder("random %d" % k)
    name = lambda v: "0" if v == 0 else "n%d" % v
    b.voltage_wave("V1", "n1", "0", "sin", [0.0, 1.0, float(np.exp(g.uniform(np.log(1e3), np.log(1e6))))])
    b.model("dm", "d", {"is": 1e-14, "n": 1.0})
    order = g.permutation(np.arange(1, N + 1))
    seen = [0]
    edges = set()
    counts = {"r": 0, "c": 0, "l": 0, "d": 0}
    def add(kind, u, v):
        i = sum(counts.values())
        counts[kind] += 1
        if kind == "r":
            b.resistor("R%d" % i, name(u), name(v), float(np.exp(g.uniform(np.log(1.0), np.log(1e6)))))
        elif kind == "c":
            b.capacitor("C%d" % i, name(u), name(v), float(np.exp(g.uniform(np.log(1e-12), np.log(1e-6)))))
        elif kind == "l":
            b.inductor("L%d" % i, name(u), name(v), float(np.exp(g.uniform(np.log(1e-9), np.log(1e-3)))))
        else:
            n = float(g.uniform(1.0, 2.0))
            b.model("dm%d" % i, "d", {"is": 1e-14, "n": n})
            b.diode("D%d" % i, name(u), name(v), "dm%d" % i)
        edges.add((min(u, v), max(u, v)))
    for v in order:
        u = int(seen[g.integers(0, len(seen))])
        kind = "r" if (u == 0 or g.random() < 0.8) else "l"
        add(kind, int(v), u)
        seen.append(int(v))
    extra = E - N
    tries = 0
    while extra > 0 and tries < 20 * E:
        tries += 1
        u, v = (int(a) for a in g.integers(0, N + 1, 2))
        if u == v or (min(u, v), max(u, v)) in edges:
            continue
        r = g.random()
        kind = "d" if r < 0.18 else ("r" if r < 0.58 else "c")
        add(kind, u, v)
        extra -= 1
    return b.build()


def random_netlists(n_circ, seed=0, nodes=(10, 400)):
    """n_circ seeded random netlists of uneven size (the multi-topology workload)."""
    g = rng(3, seed)
    return [random_netlist(g, k, nodes) for k in range(n_circ)]


# ------------------------------------------------------------------ power grid (Kron tearing)
def power_grid_template(N=256, P=4, loads=1024, seed=0):
    """An N x N resistive-capacitive power-grid mesh torn into P x P square pieces.

    Grid node g{r}_{c}; resistor RH{r}_{c} to the right neighbour and RV{r}_{c} to
    the one below (nominal 0.1 ohm), capacitor CG{r}_{c} to ground (10 pF).  One
    supply pad per piece at its centre: source VP{k} (1 V) at node pad{k}, joined
    to the grid through RPAD{k} (0.05 ohm).  `loads` current loads at seeded grid
    nodes (the same for every variant): a PULSE current sink IL{k} from the node
    to ground with a clamp diode DL{k} across it (IS 1e-14, N 2: a forward-biased
    junction drawing microamps at 1 V).  Returns (circuit, torn element names):
    the resistors that cross a piece boundary."""
    b = Builder("power grid %dx%d" % (N, N))
    g = lambda r, c: "g%d_%d" % (r, c)
    s = N // P
    torn = []
    for r in range(N):
        for c in range(N):
            if c + 1 < N:
                b.resistor("RH%d_%d" % (r, c), g(r, c), g(r, c + 1), 0.1)
                if (c + 1) % s == 0:
                    torn.append("RH%d_%d" % (r, c))
            if r + 1 < N:
                b.resistor("RV%d_%d" % (r, c), g(r, c), g(r + 1, c), 0.1)
                if (r + 1) % s == 0:
                    torn.append("RV%d_%d" % (r, c))
            b.capacitor("CG%d_%d" % (r, c), g(r, c), "0", 10e-12)
    for pr in range(P):
        for pc in range(P):
            k = pr * P + pc
            b.voltage_source("VP%d" % k, "pad%d" % k, "0", 1.0)
            b.resistor("RPAD%d" % k, "pad%d" % k, g(pr * s + s // 2, pc * s + s // 2), 0.05)
    rg = rng(5, seed)
    where = rg.choice(N * N, size=loads, replace=False)
    for k, w in enumerate(sorted(int(v) for v in where)):
        node = g(w // N, w % N)
        b.current_wave("IL%d" % k, node, "0", "pulse", [0.0, 5e-3, 0.0, 0.5e-9, 0.5e-9, 5e-9, 20e-9])
        b.model("dl%d" % k, "d", {"is": 1e-14, "n": 2.0})
        b.diode("DL%d" % k, node, "0", "dl%d" % k)
    return b.build(), torn


def power_grid_batch(n_var, seed=0, N=256, P=4, loads=1024):
    """Seeded variants of power_grid_template: every grid resistor log-U[0.01, 1]
    ohm, every grid capacitor log-U[1, 100] pF, each load's peak current log-U[1,
    10] mA, delay U[0, 20] ns, width U[2, 10] ns, period U[15, 30] ns, and its
    clamp diode's emission coefficient U[1.8, 2.2].
    Returns (elements, n_nodes, values[n_var][n_values], torn element indices, circuit)."""
    c, torn = power_grid_template(N, P, loads, seed)
    el, v0, off = _offsets(c)
    names = [e.name for e in c.elements]
    idx = {nm: i for i, nm in enumerate(names)}
    kinds = np.array([nm[:2] for nm in names])
    gen = rng(5, 1000 + seed)
    vals = np.tile(v0, (n_var, 1))
    params = np.array([int(e["param"]) for e in el])
    rgrid = params[(kinds == "RH") | (kinds == "RV")]
    vals[:, rgrid] = log_uniform(gen, 0.01, 1.0, n_var * len(rgrid)).reshape(n_var, -1)
    cgrid = params[kinds == "CG"]
    vals[:, cgrid] = log_uniform(gen, 1e-12, 100e-12, n_var * len(cgrid)).reshape(n_var, -1)
    il = params[kinds == "IL"] + 3  # KS_SRC_P_ARGS: v1, v2, td, tr, tf, pw, per
    vals[:, il + 1] = log_uniform(gen, 1e-3, 10e-3, n_var * len(il)).reshape(n_var, -1)
    vals[:, il + 2] = gen.uniform(0, 20e-9, (n_var, len(il)))
    vals[:, il + 5] = gen.uniform(2e-9, 10e-9, (n_var, len(il)))
    vals[:, il + 6] = gen.uniform(15e-9, 30e-9, (n_var, len(il)))
    dl = params[kinds == "DL"] + D_KEYS.index("n")
    vals[:, dl] = gen.uniform(1.8, 2.2, (n_var, len(dl)))
    torn_idx = np.array(sorted(idx[t] for t in torn), dtype=np.int32)
    return el, c.n_nodes, vals, torn_idx, c
