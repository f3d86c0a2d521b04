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
