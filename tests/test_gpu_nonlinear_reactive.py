"""GPU parity of the nonlinear and time-varying capacitors and inductors
(device/nonlinear_reactive.go): q = s(t) Q(v) and flux s(t) L(i) with
piecewise-linear Q and L (Q=pwl, FLUX=pwl) and a SCALE waveform, against the
oracle.

Batches of the reference's golden netlists with seeded resistances, curve
heights and scale depths: adaptive transients (the charge/flux LTE control, the
landing of each crossed knot on a time point, the scale waveform's corners),
fixed-step transients on the per-topology and generic kernels, the small-signal
model at a curved element's operating point, and a multi-topology batch.  The
golden cases themselves run in the golden parametrizations of test_gpu_tran and
test_gpu_results (waveforms, element powers and the ledger with the power that
leaves through the scale's port).
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
SEEDS = {"nlcap_tran": 1, "nlind_tran": 2, "varcap_tank_tran": 3, "varind_tran": 4}


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


def ospec(sp):
    return orc.TranSpec(sp.step, sp.stop, sp.start, sp.max_step, int(sp.uic), 1 if sp.method == "be" else 2,
                        int(sp.fixed_step), sp.max_steps, sp.chgtol, sp.trtol, sp.min_step)


def variants(name, n, seed, scale=1.2):
    """n copies of a golden netlist: resistances, the curve heights (every y of
    a curve by one factor: still through the origin and rising) and the scale
    waveform's swing (a SIN amplitude, a PWL's excursion from its first value)
    by log-uniform factors in [1/scale, scale]."""
    ckt = kc.from_dict(CASES[name]["circuit"])
    el, v0, _ = ckt.pack()
    g = np.random.default_rng(seed)
    vals = np.tile(v0, (n, 1))
    f = lambda: np.exp(g.uniform(np.log(1 / scale), np.log(scale), n))
    for k, e in enumerate(ckt.elements):
        col = int(el[k]["param"])
        if e.kind == "R":
            vals[:, col] *= f()
        elif e.kind in ("CN", "LN"):
            na, nc = int(el[k]["nargs"]), int(el[k]["level"])
            if nc:
                vals[:, col + 2 + na + 1:col + 2 + na + nc:2] *= f()[:, None]
            else:
                vals[:, col] *= f()
            a = col + 2
            if e.wave == "sin":
                vals[:, a + 1] *= f()
            elif e.wave == "pwl":
                fs = f()
                for j in range(3, na, 2):
                    vals[:, a + j] = vals[:, a + 1] + (vals[:, a + j] - vals[:, a + 1]) * fs
    return ckt, el, vals


def compare_adaptive(ckt, el, vals, sp, sample, cap):
    b = analysis.Batch(analysis.Plan(el, ckt.n_nodes, vals.shape[1]), vals)
    wave, tim, npts, st, steps, it = b.tran(sp, analysis.Options(), capacity=cap)
    assert np.all(st == 0), st
    same = 0
    for c in sample:
        ost, ot, ox, _, osteps, _, msg = orc.tran(orc.Packed(el, ckt.n_nodes, vals[c]), ospec(sp), capacity=cap)
        assert ost == 0, msg
        k = int(npts[c])
        assert abs(steps[c] - osteps) <= max(2, 0.01 * osteps), (c, steps[c], osteps)
        if k == len(ot) and np.allclose(tim[c, :k], ot, rtol=1e-9, atol=1e-15):
            same += 1
            assert np.allclose(wave[c, :k], ox, rtol=1e-6, atol=1e-9), c
        else:  # a grid that parted: the waveform on the oracle's points
            for i in range(ox.shape[1]):
                y = np.interp(ot, tim[c, :k], wave[c, :k, i])
                assert np.all(np.abs(y - ox[:, i]) <= 2e-2 * (np.abs(ox[:, i]).max() + 1e-12)), (c, i)
    assert same >= 0.9 * len(sample), (same, len(sample))


@pytest.mark.parametrize("name", ["nlcap_tran", "nlind_tran", "varcap_tank_tran", "varind_tran"])
def test_adaptive_batch(name):
    ckt, el, vals = variants(name, 64, SEEDS[name])
    tr = [a for a in CASES[name]["circuit"]["analyses"] if a["kind"] == "tran"][-1]
    sp = analysis.TranSpec(step=tr["step"], stop=tr["stop"], start=tr["start"], max_step=tr["max_step"], uic=tr["uic"])
    compare_adaptive(ckt, el, vals, sp, range(0, 64, 7), 20000)


@pytest.mark.parametrize("kernel", ["specialized", "generic"])
@pytest.mark.parametrize("name", ["nlcap_tran", "nlind_tran", "varind_tran"])
def test_fixed_step_batch(name, kernel):
    ckt, el, vals = variants(name, 512, 11)
    sp = analysis.TranSpec(step=1e-6, stop=1e-3, fixed_step=True)
    b = analysis.Batch(analysis.Plan(el, ckt.n_nodes, vals.shape[1]), vals)
    wave, _, npts, st, steps, it = b.tran(sp, analysis.Options(reltol=RELTOL, kernel=kernel))
    assert b.last_kernel.startswith(kernel[:4])
    assert np.all(st == 0)
    sample = np.arange(0, 512, 37)
    so, xo, so_steps, io = orc.batch_tran(orc.Packed(el, ckt.n_nodes, vals[sample]), len(sample), ospec(sp),
                                          orc.options(reltol=RELTOL))
    assert np.all(so == 0)
    scale = np.abs(xo).max(axis=(0, 1)) + 1e-12
    assert np.all(np.abs(wave[:, sample, :] - xo) <= 1e-7 * np.abs(xo) + 1e-7 * scale)


def biased_curves(n, seed):
    """A curved capacitor and a curved inductor at a DC bias with an AC drive
    (biases that put each on any of its segments)."""
    b = kc.Builder("bias")
    b.voltage_source("V1", "in", "0", 1.0, ac=(1.0, 0.0))
    b.resistor("R1", "in", "a", 500.0)
    b.capacitor("CN", "a", "0", 0.0, curve=[-4, -2.5e-6, -1, -1e-6, 0, 0, 1, 1e-6, 4, 2.5e-6])
    b.resistor("R2", "a", "b", 20.0)
    b.inductor("LN", "b", "0", 0.0, curve=[-10, -1.2e-3, -0.1, -0.6e-3, 0, 0, 0.1, 0.6e-3, 10, 1.2e-3])
    ckt = b.build()
    el, v0, _ = ckt.pack()
    vals = np.tile(v0, (n, 1))
    vals[:, int(el[ckt.element_index("V1")]["param"])] = np.random.default_rng(seed).uniform(-60, 60, n)
    return ckt, el, vals


def test_small_signal_at_the_operating_point():
    """LoadAC: s f'(x) of the segment the operating point lies on."""
    ckt, el, vals = biased_curves(256, 5)
    freqs = np.logspace(2, 7, 11)
    b = analysis.Batch(analysis.Plan(el, ckt.n_nodes, vals.shape[1]), vals)
    x, st, it = b.ac(freqs, analysis.Options())
    assert np.all(st == 0)
    pk = orc.Packed(el, ckt.n_nodes, vals[0])
    for c in range(0, 256, 13):
        pk.values[:] = vals[c]
        ost, ox, msg = orc.ac(pk, freqs)
        assert ost == 0, msg
        g = x[c][..., 0] + 1j * x[c][..., 1] if x.ndim == 4 else x[c]
        assert np.allclose(g, ox, rtol=1e-9, atol=1e-15), c


def test_multi_topology_batch():
    circuits = [kc.from_dict(CASES[n]["circuit"]) for n in ("nlcap_tran", "varind_tran", "rc_lowpass_ac")] * 8
    mb = analysis.MultiBatch(circuits)
    sp = analysis.TranSpec(step=2e-6, stop=1e-3, fixed_step=True)
    waves, st, steps, it = mb.tran(sp, analysis.Options(reltol=RELTOL))
    assert np.all(st == 0)
    ospec_ = orc.TranSpec(2e-6, 1e-3, 0.0, 0.0, 0, 2, 1, 0, 0.0, 0.0, 0.0)
    for k in (0, 1):
        r = orc.tran(orc.Packed.of(circuits[k]), ospec_, orc.options(reltol=RELTOL))
        assert r[0] == 0
        assert np.allclose(waves[k], r[2], rtol=1e-6, atol=1e-9)
