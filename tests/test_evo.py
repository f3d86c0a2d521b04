"""The batched population evaluator's host logic (kronspice_gb300/evo.py)
without a GPU: the penalty classes of evo/fitness.go:644-681, the measurement
helpers of analysis/measure.go and output/waveforms.go, and candidates that fail
validation (penalized before any analysis runs)."""
import math

import numpy as np
import pytest

from kronspice_gb300 import analysis, evo
from kronspice_gb300 import circuit as kc


def test_penalty_classes():
    cases = [(analysis.ErrInterrupted("x"), evo.PENALTY_TIMEOUT, "timeout"),
             (analysis.ErrLedgerResidual("x"), evo.PENALTY_LEDGER, "ledger"),
             (evo.ErrNoMeasurement("x"), evo.PENALTY_NO_MEASUREMENT, "no-measurement"),
             (analysis.ErrNoConvergence("x"), evo.PENALTY_NO_CONVERGENCE, "no-convergence"),
             (analysis.ErrTimestepTooSmall("x"), evo.PENALTY_NO_CONVERGENCE, "no-convergence"),
             (analysis.ErrTooManySteps("x"), evo.PENALTY_NO_CONVERGENCE, "no-convergence"),
             (analysis.ErrSingularMatrix("x"), evo.PENALTY_SINGULAR, "singular"),
             (analysis.ErrNonFinite("x"), evo.PENALTY_SINGULAR, "singular"),
             (analysis.ErrFloatingNode("x"), evo.PENALTY_INVALID, "invalid"),
             (analysis.ErrValidation("x"), evo.PENALTY_INVALID, "invalid"),
             (analysis.KronspiceError("x"), evo.PENALTY_OTHER, "error")]
    for err, fit, cls in cases:
        assert evo.penalty(err) == (fit, cls), err
    # the classes are ordered: "almost works" below "broken"
    assert evo.PENALTY_NO_MEASUREMENT < evo.PENALTY_NO_CONVERGENCE < evo.PENALTY_SINGULAR < evo.PENALTY_INVALID


def test_measurements():
    f = np.array([10.0, 100.0, 1000.0])
    h = np.array([1.0, 0.5, 0.1], dtype=complex)
    # log-frequency, dB interpolation half way between 100 Hz and 1 kHz
    want = 10 ** ((20 * math.log10(0.5) + 20 * math.log10(0.1)) / 2 / 20)
    assert abs(evo.gain_at(f, h, math.sqrt(1e5)) - want) <= 1e-12
    assert evo.gain_at(f, h, 100.0) == pytest.approx(0.5, rel=1e-14)
    with pytest.raises(evo.ErrNoMeasurement):
        evo.gain_at(f, h, 5.0)
    t = np.array([0.0, 1.0, 2.0])
    y = np.array([0.0, 2.0, 0.0])
    assert evo.interp(t, y, 0.5) == 1.0 and evo.interp(t, y, 1.0) == 2.0 and evo.interp(t, y, 9.0) == 0.0
    assert evo.rel_err(1.1, 1.0, 1e-3) == pytest.approx(0.1)
    assert evo.rel_err(1e-4, 0.0, 1e-3) == pytest.approx(0.1)


def test_invalid_candidates_are_penalized_without_analysis():
    """A negative capacitance and a floating node (no DC path, no transient
    objective) are penalized "invalid" by the host validation alone."""
    b = kc.Builder("bad")
    b.voltage_source("V1", "in", "0", 1.0).resistor("R1", "in", "out", 1e3).capacitor("C1", "out", "0", -1e-9)
    neg = b.build()
    b = kc.Builder("float")
    b.voltage_source("V1", "in", "0", 1.0).resistor("R1", "in", "0", 1e3).capacitor("C1", "a", "b", 1e-9)
    floating = b.build()
    out = evo.evaluate([neg, floating], [evo.op_voltage("out", 0.5)], values=[[1.0], [2.0]])
    for ind in out:
        assert ind.failure == "invalid" and ind.fitness == evo.PENALTY_INVALID and ind.terms is None, ind
    assert out[1].values == [2.0]


class FakeGroup:
    """A topology group whose batched analyses are given arrays (no GPU)."""

    def __init__(self, circuit, op, ac):
        m = len(op[1])
        self.idx, self.circuits, self.row = list(range(m)), [circuit] * m, {i: i for i in range(m)}
        self.cache = {"op": op}
        self._ac = ac

    def op(self):
        return self.cache["op"]

    def ac(self, spec):
        self.cache[("ac", spec.variation, spec.points, spec.fstart, spec.fstop)] = self._ac
        return self._ac


def synthetic(m, seed):
    b = kc.Builder("lp")
    b.voltage_source("V1", "in", "0", 2.0, ac=(1.0, 0.0))
    b.resistor("R1", "in", "out", 1e3).capacitor("C1", "out", "0", 1e-8).resistor("RL", "out", "0", 1e4)
    ckt = b.build()
    g = np.random.default_rng(seed)
    n, ne = 3, 4
    x = g.normal(size=(m, n))
    st = np.zeros(m, np.int32)
    elem = g.normal(size=(m, ne, analysis.RES_COLS))
    led = np.abs(g.normal(size=(m, analysis.LEDGER_COLS)))
    spec = analysis.ACSpec("dec", 5, 10.0, 1e5)
    freqs = spec.frequencies()
    xa = g.normal(size=(m, len(freqs), n)) + 1j * g.normal(size=(m, len(freqs), n))
    sta = np.zeros(m, np.int32)
    st[1] = sta[1] = 1                 # singular
    sta[2] = 3                         # the AC's operating point did not converge
    xa[3, 4, 0] = 0                    # V(in) = 0 at one frequency: no transfer
    return ckt, (x, st, elem, led), (freqs, xa, sta), spec


def test_batch_forms_match_the_per_candidate_objectives():
    """Each built-in objective's vectorized form gives, candidate for candidate,
    the value or the failure class its per-candidate form gives."""
    ckt, op, ac, spec = synthetic(40, 1)
    g = FakeGroup(ckt, op, ac)
    objectives = [evo.gain_at_objective("out", "in", spec, 1e3, -3.0), evo.gain_at_objective("out", "0", spec, 55.0, 6.0),
                  evo.op_voltage("out", 1.0), evo.supply_power("V1"), evo.model_supplied_limit(0.1),
                  evo.op_voltage("nowhere", 1.0)]
    for ob in objectives:
        v, fails = ob.batch(evo.GroupView(g))
        for c in range(40):
            try:
                want, want_err = ob.eval(evo.Eval(ckt, [], g, c)), None
            except analysis.KronspiceError as e:
                want, want_err = None, e
            if want_err is None and fails[c] is None:
                assert v[c] == pytest.approx(want, rel=1e-12, abs=1e-300), (ob.name, c)
            else:
                assert want_err is not None and fails[c] is not None, (ob.name, c, want_err, fails[c])
                assert evo.penalty(want_err) == evo.penalty(fails[c]), (ob.name, c)


def test_group_scoring_first_failure_and_model_supplied():
    """_score_group: a candidate stops at its first failing objective (its class
    that objective's), the others get the weighted sum of their terms, and the
    model-supplied power counts the operating point only where an objective of
    the candidate read it."""
    ckt, op, ac, spec = synthetic(8, 2)
    g = FakeGroup(ckt, op, ac)
    objectives = [evo.gain_at_objective("out", "in", spec, 1e3, -3.0), evo.op_voltage("out", 1.0)]
    objectives[1].weight = 2.0
    out = [evo.Individual(values=[]) for _ in range(8)]

    def fail(ind, err):
        ind.fitness, ind.failure = evo.penalty(err)
        ind.error = str(err)
        ind.terms = None
    evo._score_group(g, objectives, out, fail)
    assert out[1].failure == "singular" and out[2].failure == "no-convergence" and out[3].failure == "no-measurement"
    assert out[1].error.startswith("gain out at 1000 Hz:")
    for c in (0, 4, 5, 6, 7):
        t = out[c].terms
        assert out[c].failure == "" and out[c].fitness == pytest.approx(t[0] + 2.0 * t[1])
        assert out[c].model_supplied == pytest.approx(op[3][c, analysis.LEDGER["model_supplied"]])
    # failed at the AC objective before the operating-point one ran: no model-supplied power
    assert out[2].model_supplied == 0.0 and out[3].model_supplied == 0.0


class OracleBatch:
    """analysis.Batch restated over the oracle, circuit by circuit (no GPU): the
    evaluator's whole host pipeline runs against it."""
    calls = []

    def __init__(self, plan, vals):
        from oracle import oracle as orc
        self.orc, self.plan, self.vals = orc, plan, np.asarray(vals)

    def _pk(self, r):
        return self.orc.Packed(self.plan.elements, self.plan.n_nodes, self.vals[r])

    def op_results(self, opt=None):
        OracleBatch.calls.append("op")
        B, n, ne = len(self.vals), self.plan.n, len(self.plan.elements)
        x, st, it = np.zeros((B, n)), np.zeros(B, np.int32), np.zeros(B, np.int32)
        elem, led = np.zeros((B, ne, analysis.RES_COLS)), np.zeros((B, analysis.LEDGER_COLS))
        for r in range(B):
            st[r], x[r], elem[r], led[r], it[r], _ = self.orc.op_results(self._pk(r))
        return x, st, it, elem, led

    def ac(self, freqs, opt=None):
        OracleBatch.calls.append("ac")
        B, n = len(self.vals), self.plan.n
        x, st, it = np.zeros((B, len(freqs), n), complex), np.zeros(B, np.int32), np.zeros(B, np.int32)
        for r in range(B):
            st[r], x[r], _ = self.orc.ac(self._pk(r), freqs)
        return x, st, it

    def tran_results(self, spec, opt=None, capacity=0):
        OracleBatch.calls.append(("tran", capacity))
        sp = spec.c()
        osp = self.orc.TranSpec(sp.step, sp.stop, sp.start, sp.max_step, sp.uic, sp.method, 0, sp.max_steps,
                                sp.chgtol, sp.trtol, sp.min_step)
        B, n, ne = len(self.vals), self.plan.n, len(self.plan.elements)
        wave, tim = np.zeros((B, capacity, n)), np.zeros((B, capacity))
        led = np.zeros((B, capacity, analysis.TPOINT_COLS))
        elem = np.zeros((B, capacity, ne, 2))
        npts, st = np.zeros(B, np.int32), np.zeros(B, np.int32)
        for r in range(B):
            out = self.orc.tran_results(self._pk(r), osp)
            k = min(len(out[1]), capacity)
            st[r], npts[r] = out[0], k
            tim[r, :k], wave[r, :k], elem[r, :k], led[r, :k] = out[1][:k], out[2][:k], out[3][:k], out[4][:k]
        return wave, tim, elem, led, None, npts, st, None, None


def test_evaluate_against_the_oracle_pipeline(monkeypatch):
    """evaluate() end to end on the CPU with the oracle standing in for the
    batched engine: three topologies and invalid candidates in one generation,
    each analysis run once per group, transient objectives on a recording
    capacity that has to grow, and per-candidate results equal to scoring each
    circuit alone."""
    monkeypatch.setattr(evo.analysis, "Batch", OracleBatch)
    OracleBatch.calls = []
    g = np.random.default_rng(6)
    pop = []
    for r, c in zip(g.uniform(500, 2e3, 6), g.uniform(1e-8, 1e-7, 6)):
        b = kc.Builder("rc")
        b.voltage_source("V1", "in", "0", 0.0, wave="pulse", args=[0, 5, 0, 1e-6, 1e-6, 5e-5, 1e-4], ac=(1.0, 0.0))
        b.resistor("R1", "in", "out", r).capacitor("C1", "out", "0", c)
        pop.append(b.build())
    b = kc.Builder("rl")
    b.voltage_source("V1", "in", "0", 0.0, wave="pulse", args=[0, 5, 0, 1e-6, 1e-6, 5e-5, 1e-4], ac=(1.0, 0.0))
    b.resistor("R1", "in", "out", 1e3).inductor("L1", "out", "0", 1e-2)
    pop.append(b.build())
    b = kc.Builder("loop")
    b.voltage_source("V1", "in", "0", 1.0).voltage_source("V2", "in", "0", 2.0).resistor("R1", "in", "out", 1e3)
    b.resistor("R2", "out", "0", 1e3)
    pop.append(b.build())
    b = kc.Builder("rc")
    b.voltage_source("V1", "in", "0", 0.0).resistor("R1", "in", "out", 1e3).capacitor("C1", "out", "0", -1e-8)
    pop.append(b.build())  # invalid: a negative capacitance
    spec = analysis.TranSpec(step=1e-6, stop=4e-4)
    acs = analysis.ACSpec("dec", 5, 10.0, 1e5)
    objectives = [evo.gain_at_objective("out", "in", acs, 1e3, -3.0), evo.tran_average("out", spec, 2e-4, 4e-4, 2.5),
                  evo.supply_power("V1")]
    out = evo.evaluate(pop, objectives, capacity=64)
    # one AC and one transient per topology that reached them, the capacity grown from 64
    assert OracleBatch.calls.count("ac") == 3
    trans = [c for c in OracleBatch.calls if isinstance(c, tuple)]
    assert trans[0] == ("tran", 64) and trans[-1][1] > 64
    assert [ind.failure for ind in out[7:]] == ["singular", "invalid"]
    assert all(ind.failure == "" for ind in out[:7])
    for ckt, ind in zip(pop[:7], out[:7]):
        alone = evo.evaluate([ckt], objectives, capacity=100000)[0]
        assert ind.terms == pytest.approx(alone.terms, rel=1e-12) and ind.fitness == pytest.approx(alone.fitness)


def test_port_objectives_against_the_thevenin_values(monkeypatch):
    """PortVoc / PortIsc over OpenShort (analysis/port.go:30-69): a divider's
    open-circuit voltage V R2 / (R1 + R2) and short-circuit current V / R1 (out of
    plus through the probe), the short run as one more batch of the group; a
    port on one node is an unknown-node error."""
    monkeypatch.setattr(evo.analysis, "Batch", OracleBatch)
    g = np.random.default_rng(8)
    r1, r2 = g.uniform(500, 5e3, 5), g.uniform(500, 5e3, 5)
    pop = []
    for a, b_ in zip(r1, r2):
        b = kc.Builder("div")
        b.voltage_source("V1", "in", "0", 5.0).resistor("R1", "in", "out", a).resistor("R2", "out", "0", b_)
        pop.append(b.build())
    out = evo.evaluate(pop, [evo.port_voc("out", "0", 2.5), evo.port_isc("out", "gnd", 5e-3)])
    for ind, a, b_ in zip(out, r1, r2):
        assert ind.failure == "", ind
        assert ind.terms[0] == pytest.approx(evo.rel_err(5 * b_ / (a + b_), 2.5, 1e-6), rel=1e-9)
        assert ind.terms[1] == pytest.approx(evo.rel_err(5 / a, 5e-3, 1e-12), rel=1e-9)
    bad = evo.evaluate(pop[:1], [evo.port_voc("out", "out", 1.0)])[0]
    assert bad.failure == "error" and "same node" in bad.error


def test_cutoff_and_shortfalls():
    """Cutoff3dB on an RC low-pass's exact response: the upper edge at
    1 / (2 pi R C) to the sweep's interpolation, no lower edge; the shortfall
    objectives and OPEfficiency on the oracle-backed pipeline."""
    f = np.logspace(1, 7, 121)
    fc = 1 / (2 * np.pi * 1e3 * 1e-8)
    h = 1 / (1 + 1j * f / fc)
    lo, hi = evo.cutoff_3db(f, h)
    assert lo == 0.0 and hi == pytest.approx(fc, rel=2e-3)
    with pytest.raises(evo.ErrNoMeasurement):
        evo.cutoff_3db(f[:1], h[:1])


def test_ac_and_efficiency_objectives(monkeypatch):
    monkeypatch.setattr(evo.analysis, "Batch", OracleBatch)
    b = kc.Builder("lp")
    b.voltage_source("V1", "in", "0", 2.0, ac=(1.0, 0.0))
    b.resistor("R1", "in", "out", 1e3).capacitor("C1", "out", "0", 1e-8).resistor("RL", "out", "0", 1e4)
    ckt = b.build()
    spec = analysis.ACSpec("dec", 20, 10.0, 1e7)
    fc = 1 / (2 * np.pi * (1e3 * 1e4 / 1.1e4) * 1e-8)  # the Thevenin resistance R1 || RL with C1
    obs = [evo.cutoff("out", "in", spec, fc, True), evo.gain_shortfall("out", "in", spec, 10.0, 0.0),
           evo.bandwidth_shortfall("out", "in", spec, 10 * fc), evo.op_efficiency("RL")]
    ind = evo.evaluate([ckt], obs)[0]
    assert ind.failure == "", ind
    assert ind.terms[0] <= 5e-3                                   # the edge found to the sweep's resolution
    assert ind.terms[1] == pytest.approx(-20 * np.log10(1e4 / 1.1e4) / 20, rel=1e-4)  # the divider's loss
    assert ind.terms[2] == pytest.approx(1.0, abs=5e-3)           # one decade short
    assert ind.terms[3] == pytest.approx(1 - 1e4 / 1.1e4, rel=1e-9)  # RL's share of the input power
    low = evo.evaluate([ckt], [evo.cutoff("out", "in", spec, 100.0, False)])[0]
    assert low.failure == "no-measurement"                        # a low-pass has no lower edge


def test_mask_bias_parts_and_transient_efficiency(monkeypatch):
    """FilterMask, ActiveBias, PartCount and TranEfficiency on the oracle-backed
    pipeline: a low-pass inside and outside a mask, a BJT stage biased active
    and one driven into saturation, part counts of topology genomes, and a
    resistive load's share of a transient's delivered energy."""
    monkeypatch.setattr(evo.analysis, "Batch", OracleBatch)
    b = kc.Builder("lp")
    b.voltage_source("V1", "in", "0", 2.0, ac=(1.0, 0.0))
    b.resistor("R1", "in", "out", 1e3).capacitor("C1", "out", "0", 1e-8).resistor("RL", "out", "0", 1e4)
    lp = b.build()
    spec = analysis.ACSpec("dec", 20, 10.0, 1e7)
    ok = evo.filter_mask("out", "in", spec, [evo.Band(10.0, 1e3, -3.0, 0.0), evo.Band(1e6, 1e7, -np.inf, -20.0)])
    tight = evo.filter_mask("out", "in", spec, [evo.Band(10.0, 1e5, -0.1, 0.0)])
    r = evo.evaluate([lp, lp], [ok, tight, evo.part_count()], parts=[3, 5])
    assert r[0].terms[0] == 0.0 and r[0].terms[1] > evo.MASK_VIOLATION_FLOOR and r[1].terms[2] == 5.0
    assert evo.evaluate([lp], [evo.part_count()])[0].failure == "no-measurement"

    def stage(rb):
        b = kc.Builder("ce")
        b.voltage_source("VCC", "vcc", "0", 10.0)
        b.resistor("RB", "vcc", "b", rb).resistor("RC", "vcc", "c", 1e3)
        b.model("qn", "npn", {"is": 1e-15, "bf": 100})
        b.bjt("Q1", "c", "b", "0", "qn")
        return b.build()
    bias = evo.evaluate([stage(1e6), stage(1e4)], [evo.active_bias(1.0, 1e-4, 1e-1)])
    assert bias[0].terms[0] == 0.0          # IC about 1 mA, VCE about 9 V: forward active
    assert bias[1].terms[0] > 0.5           # a base current of 1 mA saturates it
    b = kc.Builder("rc")
    b.voltage_source("V1", "in", "0", 0.0, wave="pulse", args=[0, 5, 0, 1e-6, 1e-6, 5e-5, 1e-4])
    b.resistor("R1", "in", "out", 1e3).resistor("RL", "out", "0", 3e3)
    spec_t = analysis.TranSpec(step=1e-6, stop=4e-4)
    eff = evo.evaluate([b.build()], [evo.tran_efficiency(spec_t, 1e-4, 4e-4, "RL")])[0]
    assert eff.terms[0] == pytest.approx(1 - 3e3 / 4e3, rel=1e-6)  # the load's share of a resistive divider



def test_same_structure_different_names_are_not_grouped(monkeypatch):
    """Two candidates whose topologies match index for index but whose nodes are
    named differently are scored apart: each reads its own names."""
    monkeypatch.setattr(evo.analysis, "Batch", OracleBatch)
    a = kc.Builder("a")
    a.voltage_source("V1", "in", "0", 2.0).resistor("R1", "in", "out", 1e3).resistor("R2", "out", "0", 1e3)
    b = kc.Builder("b")
    b.voltage_source("V1", "x", "0", 2.0).resistor("R1", "x", "y", 1e3).resistor("R2", "y", "0", 1e3)
    ca, cb = a.build(), b.build()
    assert ca.pack()[2] == cb.pack()[2]  # the same topology key
    out = evo.evaluate([ca, cb], [evo.op_voltage("out", 1.0)])
    assert out[0].failure == "" and out[0].terms[0] == pytest.approx(0.0, abs=1e-12)
    assert out[1].failure == "no-measurement"
