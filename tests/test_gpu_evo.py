"""The batched population evaluator on the GPU (kronspice_gb300/evo.py): a
generation scored through the engine's batched analyses gets, candidate for
candidate, the terms, fitness, failure class and model-supplied power that the
reference's worker pool computes one circuit at a time (evo/engine.go:518-612),
here computed per candidate from the oracle's analyses with the same objective
code."""
import numpy as np
import pytest

from kronspice_gb300 import analysis, build, evo
from kronspice_gb300 import circuit as kc
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


class OracleEval:
    """Eval over the oracle's single-circuit analyses (the worker pool's view)."""

    def __init__(self, ckt):
        self.circuit, self.model_supplied = ckt, 0.0
        self.pk = orc.Packed.of(ckt)

    def op(self):
        st, x, elem, led, _, msg = orc.op_results(self.pk)
        err = analysis.status_error(st)
        if err:
            raise err
        r = evo.OPResult(self.circuit, x, elem, led)
        self.model_supplied = max(self.model_supplied, r.model_supplied)
        return r

    def ac(self, spec):
        freqs = spec.frequencies()
        st, x, msg = orc.ac(self.pk, freqs)
        err = analysis.status_error(st)
        if err:
            raise err
        return evo.ACResult(self.circuit, freqs, x)

    def tran(self, spec):
        sp = orc.TranSpec(spec.step, spec.stop, spec.start, spec.max_step, int(spec.uic),
                          1 if spec.method == "be" else 2, 0, 200000, 0.0, 0.0, 0.0)
        out = orc.tran_results(self.pk, sp, capacity=200000)
        err = analysis.status_error(out[0])
        if err:
            raise err
        r = evo.Waveforms(self.circuit, np.asarray(out[1]), out[2], out[4])
        self.model_supplied = max(self.model_supplied, r.model_supplied)
        return r


def oracle_score(ckt, objectives):
    e = OracleEval(ckt)
    terms, total = [], 0.0
    for ob in objectives:
        try:
            v = ob.eval(e)
        except analysis.KronspiceError as err:
            return evo.penalty(err)[1], None, evo.penalty(err)[0], e.model_supplied
        terms.append(v)
        total += ob.weight * v
    return "", terms, total, e.model_supplied


def lowpass(r, c, rl, vneg=None):
    b = kc.Builder("lp")
    b.voltage_source("V1", "in", "0", 2.0, ac=(1.0, 0.0))
    b.resistor("R1", "in", "out", r).capacitor("C1", "out", "0", c).resistor("RL", "out", "0", rl)
    if vneg is not None:  # an active load: a negative resistance supplies power
        b.resistor("RN", "out", "0", vneg)
    return b.build()


def test_population_matches_the_worker_pool():
    """Three topologies in one generation (plain low-pass, one with a negative
    resistance, a voltage-source loop that is singular), and invalid candidates."""
    g = np.random.default_rng(3)
    pop = [lowpass(r, c, rl) for r, c, rl in zip(g.uniform(500, 5e3, 300), g.uniform(1e-9, 1e-7, 300),
                                                 g.uniform(2e3, 2e4, 300))]
    pop += [lowpass(1e3, 1e-8, 1e4, vneg=v) for v in g.uniform(-4e4, -2e4, 20)]
    b = kc.Builder("loop")
    b.voltage_source("V1", "in", "0", 1.0).voltage_source("V2", "in", "0", 2.0)
    b.resistor("R1", "in", "out", 1e3).resistor("R2", "out", "0", 1e3)
    pop += [b.build()] * 3
    pop += [lowpass(1e3, -1e-9, 1e4)] * 2
    spec = analysis.ACSpec("dec", 10, 10.0, 1e6)
    objectives = [evo.gain_at_objective("out", "in", spec, 1e3, -3.0), evo.op_voltage("out", 1.0),
                  evo.supply_power("V1"), evo.model_supplied_limit(0.0)]
    out = evo.evaluate(pop, objectives, values=[[k] for k in range(len(pop))])
    classes = {}
    for k, (ckt, ind) in enumerate(zip(pop, out)):
        fail, terms, fit, ms = oracle_score(ckt, objectives) if ind.failure != "invalid" else ("invalid", None, evo.PENALTY_INVALID, 0.0)
        assert ind.failure == fail, (k, ind, fail)
        assert ind.values == [k]
        classes[fail] = classes.get(fail, 0) + 1
        if fail:
            assert ind.fitness == fit and ind.terms is None
            continue
        assert np.allclose(ind.terms, terms, rtol=1e-7, atol=1e-12), (k, ind.terms, terms)
        assert ind.fitness == pytest.approx(fit, rel=1e-7, abs=1e-12)
        assert ind.model_supplied == pytest.approx(ms, rel=1e-7, abs=1e-15)
    assert classes == {"": 320, "singular": 3, "invalid": 2}, classes
    assert max(ind.model_supplied for ind in out[300:320]) > 0


def test_transient_objectives_match_the_worker_pool():
    """An RC charging network scored on its mean output and ripple from adaptive
    transients (the step control and breakpoints of the reference)."""
    g = np.random.default_rng(4)
    pop = []
    for r, c in zip(g.uniform(500, 2e3, 64), g.uniform(1e-8, 1e-7, 64)):
        b = kc.Builder("rc")
        b.voltage_source("V1", "in", "0", 0.0, wave="pulse", args=[0, 5, 0, 1e-6, 1e-6, 5e-5, 1e-4])
        b.resistor("R1", "in", "out", r).capacitor("C1", "out", "0", c)
        pop.append(b.build())
    spec = analysis.TranSpec(step=1e-6, stop=4e-4)
    objectives = [evo.tran_average("out", spec, 2e-4, 4e-4, 2.5), evo.tran_ripple("out", spec, 2e-4, 4e-4, 1.0)]
    out = evo.evaluate(pop, objectives)
    for k, (ckt, ind) in enumerate(zip(pop, out)):
        fail, terms, fit, ms = oracle_score(ckt, objectives)
        assert ind.failure == fail == "", (k, ind)
        assert np.allclose(ind.terms, terms, rtol=1e-6, atol=1e-9), (k, ind.terms, terms)


def test_value_genomes_score_as_circuits():
    """evaluate_values on the value vectors of one topology scores each candidate
    exactly as evaluate does on the built circuits (invalid rows included)."""
    g = np.random.default_rng(5)
    pop = [lowpass(r, c, rl) for r, c, rl in zip(g.uniform(500, 5e3, 400), g.uniform(1e-9, 1e-7, 400),
                                                 g.uniform(2e3, 2e4, 400))]
    pop[7] = lowpass(1e3, -1e-9, 1e4)  # invalid: a negative capacitance
    spec = analysis.ACSpec("dec", 10, 10.0, 1e6)
    objectives = [evo.gain_at_objective("out", "in", spec, 1e3, -3.0), evo.op_voltage("out", 1.0),
                  evo.supply_power("V1")]
    a = evo.evaluate(pop, objectives)
    vals = np.stack([c.pack()[1] for c in pop])
    b = evo.evaluate_values(pop[0], vals, objectives)
    for x, y in zip(a, b):
        assert x.failure == y.failure and x.fitness == y.fitness and x.terms == y.terms
    assert b[7].failure == "invalid"

