"""GPU parity of the switches (device/switch.go): S and W, abrupt with hysteresis
and smooth, on every kernel family against the oracle.

Batches of the reference's golden switch netlists with seeded thresholds,
hysteresis, resistances and initial states: operating points (each circuit from
its initial state), adaptive transients (the step cut at each threshold crossing
and the backward-Euler restart after it, analysis/tran.go:186-217), fixed-step
transients, the smooth switch's operating point and small-signal response, and a
multi-topology batch.  The golden cases themselves run in the golden
parametrizations of test_gpu_op, test_gpu_tran and test_gpu_results.
"""
import json
import os

import numpy as np
import pytest

from kronspice_gb300 import analysis, build
from kronspice_gb300 import circuit as kc
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "reference_cases.json")) as f:
    CASES = {c["name"]: c for c in json.load(f)["cases"]}
RELTOL = 1e-6
SW_P = dict(vt=0, vh=1, ron=2, roff=3, on=4)


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


def ospec(sp):
    return orc.TranSpec(sp.step, sp.stop, sp.start, sp.max_step, int(sp.uic), 1 if sp.method == "be" else 2,
                        int(sp.fixed_step), sp.max_steps, sp.chgtol, sp.trtol, sp.min_step)


def variants(name, n, seed, scale=1.3, kinds="RC", init=True):
    """n copies of a golden circuit: R and C values and the switches' thresholds,
    hysteresis and resistances scaled by log-uniform factors in [1/scale, scale],
    and (init) each switch's initial state drawn ON or OFF."""
    ckt = kc.from_dict(CASES[name]["circuit"])
    el, v0, _ = ckt.pack()
    g = np.random.default_rng(seed)
    vals = np.tile(v0, (n, 1))
    f = lambda: np.exp(g.uniform(np.log(1 / scale), np.log(scale), n))
    for k, e in enumerate(ckt.elements):
        col = int(el[k]["param"])
        if e.kind in kinds:
            vals[:, col] *= f()
        elif e.kind in "SW":
            for p in ("vt", "vh", "ron", "roff"):
                vals[:, col + SW_P[p]] *= f()
            if init:
                vals[:, col + SW_P["on"]] = g.integers(0, 2, n)
    return ckt, el, vals


def check_op_batch(ckt, el, vals, kernel, stride):
    b = analysis.Batch(analysis.Plan(el, ckt.n_nodes, vals.shape[1]), vals)
    x, st, it = b.op(analysis.Options(reltol=RELTOL, kernel=kernel))
    assert b.last_kernel.startswith(kernel[:4])
    pk = orc.Packed(el, ckt.n_nodes, vals[0])
    for c in range(0, len(vals), stride):
        pk.values[:] = vals[c]
        ost, ox, _, _, msg = orc.op(pk, orc.options(reltol=RELTOL))
        assert st[c] == ost, (c, msg)
        if ost == 0:
            assert np.allclose(x[c], ox, rtol=1e-9, atol=1e-12), c
    return st


@pytest.mark.parametrize("kernel", ["specialized", "generic"])
def test_switch_dc_batch(kernel):
    """switch_dc with the swept source at seeded points of its range and random
    initial states: inside a hysteresis band the state stays the initial one."""
    ckt, el, vals = variants("switch_dc", 2048, 1, kinds="R")
    vals[:, int(el[ckt.element_index("V1")]["param"])] = np.random.default_rng(2).uniform(0, 3, 2048)
    st = check_op_batch(ckt, el, vals, kernel, 31)
    assert np.all(st == 0)


def smooth_batch(n, seed):
    b = kc.Builder("smooth")
    b.voltage_source("V1", "ctl", "0", 1.0, ac=(1.0, 0.0))
    b.resistor("RC", "ctl", "0", 1e3)
    b.voltage_source("V2", "dd", "0", 5.0)
    b.resistor("R1", "dd", "out", 1e3)
    b.voltage_source("VS", "out", "m", 0.0)
    b.model("sm", "sw", {"vt": 1.0, "vh": -0.5, "ron": 10.0, "roff": 1e5})
    b.model("cs", "csw", {"it": 2e-3, "ih": -1e-3, "ron": 100.0, "roff": 1e6})
    b.vswitch("S1", "m", "0", "ctl", "0", "sm")
    b.iswitch("W1", "dd", "out", "VS", "cs")
    ckt = b.build()
    el, v0, _ = ckt.pack()
    vals = np.tile(v0, (n, 1))
    vals[:, int(el[ckt.element_index("V1")]["param"])] = np.random.default_rng(seed).uniform(0.3, 1.8, n)
    return ckt, el, vals


@pytest.mark.parametrize("kernel", ["specialized", "generic"])
def test_smooth_switch_batch(kernel):
    """Smooth S and W switches (negative hysteresis) through their band."""
    ckt, el, vals = smooth_batch(1024, 3)
    st = check_op_batch(ckt, el, vals, kernel, 17)
    assert np.all(st == 0)


def test_smooth_switch_ac_batch():
    """The small-signal model of the smooth switches: conductance and
    transconductance from the operating point's last load."""
    ckt, el, vals = smooth_batch(256, 4)
    freqs = np.logspace(0, 6, 13)
    b = analysis.Batch(analysis.Plan(el, ckt.n_nodes, vals.shape[1]), vals)
    x, st, it = b.ac(freqs, analysis.Options())
    assert np.all(st == 0)
    pk = orc.Packed(el, ckt.n_nodes, vals[0])
    for c in range(0, 256, 11):
        pk.values[:] = vals[c]
        ost, ox, msg = orc.ac(pk, freqs)
        assert ost == 0, msg
        g = x[c][..., 0] + 1j * x[c][..., 1] if x.ndim == 4 else x[c]
        assert np.allclose(g, ox, rtol=1e-8, atol=1e-14), c


def compare_adaptive(ckt, el, vals, sp, sample, cap):
    b = analysis.Batch(analysis.Plan(el, ckt.n_nodes, vals.shape[1]), vals)
    wave, tim, npts, st, steps, it = b.tran(sp, analysis.Options(), capacity=cap)
    assert np.all(st == 0), st
    same = 0
    for c in sample:
        pk = orc.Packed(el, ckt.n_nodes, vals[c])
        ost, ot, ox, _, osteps, _, msg = orc.tran(pk, ospec(sp), capacity=cap)
        assert ost == 0, msg
        k = int(npts[c])
        assert abs(steps[c] - osteps) <= max(2, 0.01 * osteps), (c, steps[c], osteps)
        if k == len(ot) and np.allclose(tim[c, :k], ot, rtol=1e-9, atol=1e-15):
            same += 1
            assert np.allclose(wave[c, :k], ox, rtol=1e-6, atol=1e-9), c
        else:  # a grid that parted: the waveform on the oracle's points
            for i in range(ox.shape[1]):
                y = np.interp(ot, tim[c, :k], wave[c, :k, i])
                assert np.all(np.abs(y - ox[:, i]) <= 2e-2 * (np.abs(ox[:, i]).max() + 1e-9)), (c, i)
    assert same >= 0.9 * len(sample), (same, len(sample))
    return wave, tim, npts


def test_switch_rc_tran_adaptive_batch():
    """switch_rc_tran: the PULSE drives S1 and, through VS, W1; each crossing cuts
    the step to just past it and restarts with backward Euler."""
    ckt, el, vals = variants("switch_rc_tran", 128, 5, scale=1.2, init=False)
    tr = [a for a in CASES["switch_rc_tran"]["circuit"]["analyses"] if a["kind"] == "tran"][-1]
    sp = analysis.TranSpec(step=tr["step"], stop=tr["stop"])
    compare_adaptive(ckt, el, vals, sp, range(0, 128, 9), 20000)


def test_relaxation_oscillator_batch():
    """switch_relax_tran from UIC: a switch that feeds its own control; every
    cycle's two crossings located by the step limiter."""
    ckt, el, vals = variants("switch_relax_tran", 128, 6, scale=1.15, init=False)
    sp = analysis.TranSpec(step=10e-6, stop=30e-3, uic=True)
    wave, tim, npts = compare_adaptive(ckt, el, vals, sp, range(0, 128, 13), 20000)
    # the period of every circuit against the closed form of its own values
    ic = ckt.node_index("c") - 1
    p = {e.name: int(el[k]["param"]) for k, e in enumerate(ckt.elements)}
    for c in range(128):
        k = int(npts[c])
        t, v = tim[c, :k], wave[c, :k, ic]
        r, cap = vals[c, p["R1"]], vals[c, p["C1"]]
        vt, vh, ron = vals[c, p["S1"]], vals[c, p["S1"] + 1], vals[c, p["S1"] + 2]
        hi, lo = vt + vh, vt - vh
        vinf = 5 * ron / (ron + r)
        period = r * cap * np.log((5 - lo) / (5 - hi)) + (r * ron / (r + ron)) * cap * np.log((hi - vinf) / (lo - vinf))
        # upward crossings of VT, interpolated between the accepted points
        rise = [t[j - 1] + (vt - v[j - 1]) / (v[j] - v[j - 1]) * (t[j] - t[j - 1])
                for j in range(1, k) if v[j - 1] < vt <= v[j]]
        got = np.diff(rise)
        assert len(got) >= 3 and np.all(np.abs(got - period) <= 3e-3 * period), (c, got, period)


@pytest.mark.parametrize("kernel", ["specialized", "generic"])
def test_switch_fixed_step_batch(kernel):
    """Fixed-step grid: the state held through each step and changed at its end."""
    ckt, el, vals = variants("switch_rc_tran", 1024, 7, scale=1.2, init=True)
    sp = analysis.TranSpec(step=20e-6, stop=6e-3, fixed_step=True)
    b = analysis.Batch(analysis.Plan(el, ckt.n_nodes, vals.shape[1]), vals)
    wave, _, npts, st, steps, it = b.tran(sp, analysis.Options(reltol=RELTOL, kernel=kernel))
    assert np.all(st == 0)
    sample = np.arange(0, 1024, 41)
    so, xo, so_steps, io = orc.batch_tran(orc.Packed(el, ckt.n_nodes, vals[sample]), len(sample), ospec(sp),
                                          orc.options(reltol=RELTOL))
    assert np.all(so == 0)
    assert np.allclose(wave[:, sample, :], xo, rtol=1e-7, atol=1e-10)


def test_multi_topology_batch_with_switches():
    """switch_dc, switch_rc_tran and controlled_op of different sizes in one batch."""
    circuits = [kc.from_dict(CASES[n]["circuit"]) for n in ("switch_dc", "switch_rc_tran", "controlled_op")] * 16
    mb = analysis.MultiBatch(circuits)
    xs, st, it = mb.op(analysis.Options(reltol=RELTOL))
    assert np.all(st == 0)
    for c, x in zip(circuits[:3], xs[:3]):
        ost, ox, _, _, msg = orc.op(orc.Packed.of(c), orc.options(reltol=RELTOL))
        assert ost == 0, msg
        _, isv = orc.unknowns(orc.Packed.of(c))
        tol = np.where(isv, 1e-6, 1e-12) + 2e-6 * np.abs(ox)
        assert np.all(np.abs(x - ox) <= tol)
    sp = analysis.TranSpec(step=20e-6, stop=4e-3, fixed_step=True)
    waves, st, steps, it = mb.tran(sp, analysis.Options(reltol=RELTOL))
    assert np.all(st == 0)
    ospec_ = orc.TranSpec(20e-6, 4e-3, 0.0, 0.0, 0, 2, 1, 0, 0.0, 0.0, 0.0)
    r = orc.tran(orc.Packed.of(circuits[1]), ospec_, orc.options(reltol=RELTOL))
    assert r[0] == 0
    assert np.allclose(waves[1], r[2], rtol=1e-6, atol=1e-9)


def test_hysteresis_loop_as_a_chained_sweep():
    """A batch of switches with seeded thresholds and hysteresis swept up and back
    down (ks_dc_sweep): inside the band each point keeps the state the previous
    point left, so the way down differs from the way up, as in the oracle's
    chained analysis.DC."""
    b = kc.Builder("loop")
    b.voltage_source("V1", "ctl", "0", 0.0)
    b.voltage_source("V2", "dd", "0", 5.0)
    b.resistor("R1", "dd", "out", 1e3)
    b.model("sw", "sw", {"vt": 1.0, "vh": 0.2, "ron": 1.0, "roff": 1e6})
    b.vswitch("S1", "out", "0", "ctl", "0", "sw")
    b.resistor("RC", "ctl", "s", 1e3).voltage_source("VS", "s", "0", 0.0)
    b.model("cs", "csw", {"it": 1e-3, "ih": 2e-4, "ron": 5.0, "roff": 1e6})
    b.resistor("R2", "dd", "o2", 1e3).iswitch("W1", "o2", "0", "VS", "cs")
    ckt = b.build()
    el, v0, _ = ckt.pack()
    g = np.random.default_rng(9)
    n = 512
    vals = np.tile(v0, (n, 1))
    for name in ("S1", "W1"):
        col = int(el[ckt.element_index(name)]["param"])
        vals[:, col] *= g.uniform(0.7, 1.3, n)
        vals[:, col + 1] *= g.uniform(0.5, 1.5, n)
    pts = np.concatenate([np.linspace(0, 2, 41), np.linspace(2, 0, 41)[1:]])
    src = ckt.element_index("V1")
    bt = analysis.Batch(analysis.Plan(el, ckt.n_nodes, vals.shape[1]), vals)
    x, st, npts, it = bt.dc_sweep(src, pts, analysis.Options(precision="fp64"))
    assert np.all(st == 0) and np.all(npts == len(pts))
    out = ckt.node_index("out") - 1
    up, down = x[:, :41, out], x[:, 40:, out][:, ::-1]
    assert np.any(np.abs(up - down) > 1.0)  # the loop is open inside the band
    pk = orc.Packed(el, ckt.n_nodes, vals[0])
    for c in range(0, n, 29):
        pk.values[:] = vals[c]
        ost, ox, _, msg = orc.dc(pk, src, pts)
        assert ost == 0, msg
        assert np.allclose(x[c], ox, rtol=1e-9, atol=1e-12), c

