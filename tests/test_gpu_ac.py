"""GPU parity of the batched AC sweep (ks_ac) against the golden vectors and the oracle.

The reference's AC golden netlists (checkGolden, analysis/op_test.go:214-236)
run through the engine and must match the independent reference and the
ngspice-39 twin with CompareAC's tolerances (1e-6 relative on |V|, 1e-4 degrees
on the phase, internal/golden/golden.go:290-340).  Seeded batches of the
common-emitter amplifier and of the CMOS op-amp must match the FP64 oracle's
phasors to 1e-7 of each unknown's largest magnitude over the sweep.  Both take
the small-signal model at the polished operating point, exact to round-off, so
the remaining difference is the rounding of the admittance entries: the GPU sums
an entry's capacitances and multiplies by omega once, the oracle (like the
reference) adds omega*C per device, and where a 10 uF coupling capacitor and a
1 pF junction share a diagonal entry (3e5 S against 0.04 S at 5 GHz) the last
bits of the junction's admittance differ by ~1e-9 relative between the two;
the solution inherits that through the cancellation across the coupling
capacitor (observed: 3e-9 of the input current's magnitude).
"""
import json
import os

import numpy as np
import pytest

from kronspice_gb300 import analysis, build, workloads
from kronspice_gb300 import circuit as kc
from oracle import oracle as orc

import golden_compare as gc

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

with open(os.path.join(ROOT, "tests", "golden", "reference_cases.json")) as f:
    AC_CASES = [c for c in json.load(f)["cases"]
                if not c["skip"] and c["circuit"]["analyses"][0]["kind"] == "ac"]


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


def test_ac_cases_present():
    assert len(AC_CASES) >= 6  # five AC netlists plus the .param RC low-pass


@pytest.mark.parametrize("case", AC_CASES, ids=[c["name"] for c in AC_CASES])
@pytest.mark.parametrize("src", ["independent", "ngspice"])
def test_golden_ac(case, src):
    if src not in case["golden"]:
        pytest.skip("no %s vector" % src)
    ckt = kc.from_dict(case["circuit"])
    a = case["circuit"]["analyses"][0]
    freqs = analysis.ACSpec(a["variation"], a["points"], a["fstart"], a["fstop"]).frequencies()
    # the circuit replicated across a batch: every copy runs the same kernels
    el, vals, _ = ckt.pack()
    plan = analysis.Plan(el, ckt.n_nodes, len(vals))
    b = analysis.Batch(plan, np.tile(vals, (37, 1)))
    x, st, _ = b.ac(freqs, analysis.Options())
    assert np.all(st == 0), st
    assert np.array_equal(x, np.broadcast_to(x[:1], x.shape))

    def get(node):
        i = ckt.node_index(node)
        return None if i < 0 else (np.zeros(len(freqs), complex) if i == 0 else x[0, :, i - 1])
    msgs = gc.compare_ac(list(freqs), get, case["golden"][src])
    assert not msgs, "\n".join(msgs)


def _compare_oracle(el, nn, vals, freqs, opt_gpu, rel=1e-7):
    plan = analysis.Plan(el, nn, vals.shape[1])
    b = analysis.Batch(plan, vals)
    xg, sg, _ = b.ac(freqs, opt_gpu)
    oc = orc.options(reltol=opt_gpu.reltol)
    bad = []
    for c in range(vals.shape[0]):
        so, xo, msg = orc.ac(orc.Packed(el, nn, vals[c]), freqs, oc)
        if so != sg[c]:
            bad.append((c, "status", so, sg[c], msg))
            continue
        if so:
            continue
        # per unknown over the sweep, with a floor of 1e-5 of the circuit's largest
        # magnitude for unknowns that are zero up to round-off (a supply node)
        scale = np.maximum(np.abs(xo).max(axis=0), 1e-5 * np.abs(xo).max())
        err = np.abs(xg[c] - xo)
        if np.any(err > rel * scale):
            k = np.unravel_index(np.argmax(err / scale), err.shape)
            bad.append((c, "phasor", k, xg[c][k], xo[k]))
    return sg, bad


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_bjt_ce_ac_batch_matches_oracle(precision):
    el, nn, vals = workloads.bjt_ce_ac_batch(256, seed=3)
    freqs = analysis.ACSpec("dec", 10, 10, 1e10).frequencies()
    sg, bad = _compare_oracle(el, nn, vals, freqs, analysis.Options(reltol=1e-6, precision=precision))
    assert np.all(sg == 0)
    assert not bad, bad[:5]


def test_opamp_ac_batch_matches_oracle():
    el, nn, vals = workloads.cmos_opamp_batch(128, seed=9)
    c = workloads.cmos_opamp_template()
    vcm = int(el[[e.name for e in c.elements].index("VCM")]["param"])
    vals[:, vcm + 1] = 1.0  # AC magnitude of the common-mode input
    freqs = analysis.ACSpec("dec", 5, 1, 1e9).frequencies()
    sg, bad = _compare_oracle(el, nn, vals, freqs, analysis.Options(reltol=1e-6))
    assert (sg == 0).mean() > 0.9
    assert not bad, bad[:5]


def test_lin_sweep_from_dc_and_single_point():
    """A linear sweep starting at 0 Hz (the DC small-signal gain) and a one-point sweep."""
    el, nn, vals = workloads.bjt_ce_ac_batch(64, seed=4)
    for spec in (analysis.ACSpec("lin", 11, 0.0, 1e6), analysis.ACSpec("lin", 1, 1e3, 1e3)):
        freqs = spec.frequencies()
        sg, bad = _compare_oracle(el, nn, vals, freqs, analysis.Options(reltol=1e-6))
        assert np.all(sg == 0)
        assert not bad, bad[:5]


def test_failed_operating_point_gives_status_and_zero_phasors():
    """Circuits whose operating point does not converge within the iteration
    bound keep the OP status and get zero phasors; with the default bound the
    same batch solves."""
    el, nn, vals = workloads.bjt_ce_ac_batch(8, seed=5)
    opt = analysis.Options(reltol=1e-6, max_iter_total=2, no_gmin_stepping=True, no_source_stepping=True,
                           no_pseudo_transient=True)
    plan = analysis.Plan(el, nn, vals.shape[1])
    b = analysis.Batch(plan, vals)
    freqs = np.array([1e3, 1e6])
    x, st, _ = b.ac(freqs, opt)
    assert np.all(st == 3)  # KS_STATUS_NO_CONVERGENCE
    assert np.all(x == 0)
    x2, st2, _ = b.ac(freqs, analysis.Options(reltol=1e-6))
    assert np.all(st2 == 0)
    assert np.all(np.abs(x2[:, :, 1]) > 0.5)  # v(in) is the 1 V source


def test_ac_batch_api():
    """ac_batch groups circuits by topology and returns output.ACResult-shaped phasors."""
    spec = analysis.ACSpec("dec", 3, 100, 1e8)
    freqs = spec.frequencies()
    circuits = [workloads.bjt_ce_ac_template() for _ in range(3)]
    res, errs = analysis.ac_batch(circuits, spec)
    assert all(e is None for e in errs)
    c = circuits[0]
    assert res[0].node_voltages.shape == (c.n_nodes, len(freqs))
    assert np.all(res[0].node_voltages[0] == 0)
    pk = orc.Packed.of(c)
    so, xo, _ = orc.ac(pk, freqs, orc.options())
    assert so == 0
    assert np.all(np.abs(res[1].x - xo) <= 1e-7 * np.maximum(np.abs(xo).max(axis=0), 1e-5 * np.abs(xo).max()))


def test_sweep_about_given_operating_points():
    """ks_ac_at: the sweep alone about operating points the caller holds on the
    device; a circuit marked failed is skipped with zero phasors, the others match
    the full analysis to the accuracy of the unpolished operating point."""
    import torch
    el, nn, vals = workloads.bjt_ce_ac_batch(32, seed=7)
    plan = analysis.Plan(el, nn, vals.shape[1])
    b = analysis.Batch(plan, vals)
    freqs = analysis.ACSpec("dec", 2, 10, 1e9).frequencies()
    full, st_full, _ = b.ac(freqs, analysis.Options(reltol=1e-6))
    assert np.all(st_full == 0)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)  # a real stream: torch's writes and the library's kernels in one order
    s = stream.cuda_stream
    with torch.cuda.stream(stream):
        x_op = torch.empty((32, plan.n), dtype=torch.float64, device=dev)
        ints = torch.zeros((3, 32), dtype=torch.int32, device=dev)
        b.op_async(analysis.Options(reltol=1e-9), None, x_op.data_ptr(), ints[0].data_ptr(), ints[1].data_ptr(), s)
        ints[0, 5] = 3  # circuit 5: operating point failed
        f_dev = torch.from_numpy(freqs).to(dev)
        xac = torch.full((32, len(freqs), plan.n, 2), 7.0, dtype=torch.float64, device=dev)
        b.ac_at_async(None, x_op.data_ptr(), ints[0].data_ptr(), f_dev.data_ptr(), len(freqs), xac.data_ptr(),
                      ints[2].data_ptr(), s)
    torch.cuda.synchronize()
    st = ints[2].cpu().numpy()
    x = xac.cpu().numpy()
    x = x[..., 0] + 1j * x[..., 1]
    assert st[5] == 3 and np.all(np.delete(st, 5) == 0)
    assert np.all(x[5] == 0)
    keep = np.arange(32) != 5
    scale = np.maximum(np.abs(full[keep]).max(axis=1, keepdims=True), 1e-5 * np.abs(full).max())
    assert np.all(np.abs(x[keep] - full[keep]) <= 1e-5 * scale)
