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
