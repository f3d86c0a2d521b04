"""CPU-only checks of the engine's C ABI: the library loads, exports every symbol
include/kronspice_gpu.h declares, and its host symbolic pass (unknown layout,
validation) agrees with the oracle and the reference's Validate semantics.
No compute call is made (no GPU here)."""
import json
import os
import re

import numpy as np
import pytest

from kronspice_gb300 import _lib, analysis, build
from kronspice_gb300 import circuit as kc
from oracle import oracle as orc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def header_symbols():
    with open(os.path.join(ROOT, "include", "kronspice_gpu.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ks_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(lib):
    syms = header_symbols()
    assert len(syms) >= 12
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    assert set(syms) == set(_lib.EXPORTS) | (set(syms) - set(_lib.EXPORTS)) and set(_lib.EXPORTS) <= set(syms)


def test_version(lib):
    assert b"sm_103a" in lib.ks_version()


with open(os.path.join(ROOT, "tests", "golden", "reference_cases.json")) as f:
    CASES = [c for c in json.load(f)["cases"] if not c["skip"]]


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_unknown_layout_matches_oracle(lib, case):
    ckt = kc.from_dict(case["circuit"])
    el, vals, _ = ckt.pack()
    n = np.zeros(1, dtype=np.int32)
    isv = np.zeros(1024, dtype=np.int32)
    topo = _lib.KsTopology(ckt.n_nodes, len(el), len(vals), 0, el.ctypes.data)
    import ctypes
    assert lib.ks_unknowns(ctypes.byref(topo), n.ctypes.data, isv.ctypes.data) == 0
    no, isvo = orc.unknowns(orc.Packed.of(ckt))
    assert n[0] == no
    assert np.array_equal(isv[:no].astype(bool), isvo)
    assert analysis.validate(ckt) is None


def _rv(extra):
    b = kc.Builder("v")
    b.voltage_source("V1", "a", "0", 1.0)
    extra(b)
    return b.build()


def test_validate_floating_node(lib):
    # TestFloatingNodeRejected, analysis/op_test.go:100-111
    b = kc.Builder("f")
    b.resistor("R1", "a", "0", 1.0)
    b.current_source("I1", "b", "0", 1.0)
    err = analysis.validate(b.build())
    assert isinstance(err, analysis.ErrFloatingNode)
    # a capacitor is a path only for a transient without operating point (ValidateTransient)
    b = kc.Builder("c")
    b.voltage_source("V1", "a", "0", 1.0)
    b.resistor("R1", "a", "b", 1.0)
    b.capacitor("C1", "b", "c", 1e-9)
    b.resistor("R2", "c", "d", 1.0)
    c = b.build()
    assert isinstance(analysis.validate(c), analysis.ErrFloatingNode)
    assert analysis.validate(c, transient=True) is None


def test_validate_bad_values(lib):
    c = _rv(lambda b: b.resistor("R1", "a", "0", 0.0))
    assert isinstance(analysis.validate(c), analysis.ErrValidation)
    c = _rv(lambda b: b.capacitor("C1", "a", "0", -1e-9))
    assert isinstance(analysis.validate(c), analysis.ErrValidation)
    c = _rv(lambda b: b.resistor("R1", "a", "a", 1.0))
    assert "itself" in str(analysis.validate(c))
    c = _rv(lambda b: b.resistor("R1", "a", "0", float("nan")))
    assert isinstance(analysis.validate(c), analysis.ErrValidation)
    # negative resistance is allowed (device/passive.go:21-31)
    c = _rv(lambda b: b.resistor("R1", "a", "0", -5.0))
    assert analysis.validate(c) is None


def test_validate_waveforms(lib):
    b = kc.Builder("w")
    b.voltage_wave("V1", "a", "0", "pulse", [0, 1, -1e-9])
    b.resistor("R1", "a", "0", 1.0)
    assert "PULSE" in str(analysis.validate(b.build()))
    b = kc.Builder("w")
    b.voltage_wave("V1", "a", "0", "pwl", [0, 0, 2e-9, 1, 1e-9, 0])
    b.resistor("R1", "a", "0", 1.0)
    assert "PWL" in str(analysis.validate(b.build()))


def test_workload_batches_are_seeded():
    from kronspice_gb300 import workloads as w
    el, nn, v1 = w.bjt_ce_batch(64, 3)
    _, _, v2 = w.bjt_ce_batch(64, 3)
    _, _, v3 = w.bjt_ce_batch(64, 4)
    assert np.array_equal(v1, v2) and not np.array_equal(v1, v3)
    assert v1.shape == (64, len(w.bjt_ce_template().pack()[1]))


def test_per_topology_source_on_cpu():
    """The per-topology source is host work (no GPU): one constant element per
    element of the plan, registers up to 6 unknowns, shared memory above."""
    from kronspice_gb300 import analysis, workloads
    el, nn, vals = workloads.bjt_ce_batch(2, seed=1)
    plan = analysis.Plan(el, nn, vals.shape[1])
    src = plan.kernel_source("op")
    assert src.count("const KElem e{") == len(el)
    assert "RegSys<KS_N>" in src and "ks_spec_op" in src and "ks_spec_tran" not in src
    el2, nn2, vals2 = workloads.rc_ladder_batch(2, seed=1, sections=10)
    plan2 = analysis.Plan(el2, nn2, vals2.shape[1])
    src2 = plan2.kernel_source("tran")
    assert "SmemSys<KS_T, KS_N>" in src2 and "ks_spec_tran" in src2 and "#define KS_N 12" in src2


def test_per_topology_source_compiles_with_nvrtc():
    """The generated source with the device headers as the library embeds them
    compiles under NVRTC for sm_103a (no GPU needed)."""
    nvrtc = pytest.importorskip("cuda.bindings.nvrtc")
    from kronspice_gb300 import analysis, build, workloads
    el, nn, vals = workloads.rc_ladder_batch(2, seed=1, sections=3)
    src = analysis.Plan(el, nn, vals.shape[1]).kernel_source("op")
    names = [n.encode() for n, _ in build.JIT_HEADERS]
    heads = [open(os.path.join(build.CSRC, rel), "rb").read() for _, rel in build.JIT_HEADERS]
    err, prog = nvrtc.nvrtcCreateProgram(src.encode(), b"ks_spec.cu", len(names), heads, names)
    opts = [b"--gpu-architecture=sm_103a", b"-std=c++17", b"-DKS_JIT=1"]
    (rc,) = nvrtc.nvrtcCompileProgram(prog, len(opts), opts)
    _, ls = nvrtc.nvrtcGetProgramLogSize(prog)
    log = b" " * ls
    nvrtc.nvrtcGetProgramLog(prog, log)
    assert rc == nvrtc.nvrtcResult.NVRTC_SUCCESS, log.decode()[:2000]
    _, size = nvrtc.nvrtcGetCUBINSize(prog)
    assert size > 0


def test_ac_frequencies_match_golden_sweeps():
    """ACSpec.Frequencies (analysis/ac.go:33-72) reproduces the golden AC tables' frequency columns."""
    import json
    from kronspice_gb300.analysis import ACSpec
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_cases.json")) as f:
        cases = [c for c in json.load(f)["cases"] if not c["skip"] and c["circuit"]["analyses"][0]["kind"] == "ac"]
    assert cases
    for c in cases:
        a = c["circuit"]["analyses"][0]
        got = ACSpec(a["variation"], a["points"], a["fstart"], a["fstop"]).frequencies()
        for src, want in c["golden"].items():
            assert len(got) == len(want["xs"]), (c["name"], src)
            assert np.all(np.abs(got - np.array(want["xs"])) <= 1e-9 * np.array(want["xs"])), (c["name"], src)


@pytest.mark.parametrize("spec", [("dec", 0, 1.0, 10.0), ("dec", 10, 10.0, 1.0), ("lin", 5, -1.0, 1.0),
                                  ("dec", 10, 0.0, 1e3), ("log", 10, 1.0, 1e3), ("lin", 2, 1.0, float("inf")),
                                  ("dec", 100000, 1.0, 1e30)])
def test_ac_spec_rejects_bad_sweeps(spec):
    from kronspice_gb300.analysis import ACSpec, ErrBadACSpec
    with pytest.raises(ErrBadACSpec):
        ACSpec(*spec).frequencies()


def test_ac_lin_single_point():
    from kronspice_gb300.analysis import ACSpec
    assert list(ACSpec("lin", 1, 5.0, 5.0).frequencies()) == [5.0]
    assert list(ACSpec("lin", 3, 0.0, 2.0).frequencies()) == [0.0, 1.0, 2.0]


def test_torn_refusals_match_reference():
    """TestJacobianErrors (kron/jacobian_test.go:284-308): the torn engine refuses
    a voltage source, an element to ground and an element torn twice with the
    reference's messages, before touching the GPU."""
    from kronspice_gb300 import workloads
    el, nn, vals, torn, c = workloads.power_grid_batch(1, N=16, P=2, loads=16)
    names = [e.name for e in c.elements]
    for bad, want in (([names.index("VP0")], "branch-current unknown"), ([names.index("CG0_0")], "connects to ground"),
                      ([int(torn[0]), int(torn[0])], "torn twice"), ([len(names)], "no element")):
        with pytest.raises(RuntimeError) as e:
            analysis.TornBatch(el, nn, vals, bad)
        assert want in str(e.value), str(e.value)


def test_validation_of_controlled_and_mutual():
    """validateControl / validateMutual (circuit/circuit.go:807-881) on the host."""
    b = kc.Builder("bad")
    b.voltage_source("V1", "a", "0", 1).resistor("R1", "a", "0", 1e3)
    b.vcvs("E1", "e", "0", "a", "a", 2.0).resistor("RE", "e", "0", 1e3)
    assert analysis.validate(b.build()) is not None
    b = kc.Builder("bad2")
    b.voltage_source("V1", "a", "0", 1).inductor("L1", "a", "b", 1e-3).resistor("R1", "b", "0", 1)
    b.inductor("L2", "c", "0", 1e-3).resistor("R2", "c", "0", 1).mutual("K1", "L1", "L2", 1.5)
    assert analysis.validate(b.build()) is not None


def test_untuned_plan_reports_no_choice(lib):
    """ks_plan_tuned on a plan no autotune call has run for: KS_EINVAL, None in Python."""
    from kronspice_gb300 import workloads
    el, nn, vals = workloads.bjt_ce_batch(4, seed=0)
    plan = analysis.Plan(el, nn, vals.shape[1])
    assert plan.tuned(4) is None and plan.tuned(1 << 20) is None
