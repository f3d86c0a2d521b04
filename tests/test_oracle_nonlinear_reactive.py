"""Nonlinear and time-varying capacitors and inductors (device/nonlinear_reactive.go)
in the oracle and on the host, without a GPU.

The host's validateStateLaw (circuit/circuit.go:890-986): a curve must rise
strictly, pass through the origin and come without a value, a linear law needs
a positive value, and the scale must be a valid waveform that stays above zero.
Then the oracle's restatement against what the reference's device promises: a
crossed knot of the curve lands on an accepted time point (stateLaw.knotStep,
:171-219), and the transient's energy bookkeeping (stored energy
s (x f(x) - F(x)) and the scale's port power s' F(x)) closes the ledger at every
point.  The golden netlists nlcap_tran, nlind_tran, varcap_tank_tran and
varind_tran are pinned in test_oracle_golden.
"""
import numpy as np
import pytest

from kronspice_gb300 import analysis
from kronspice_gb300 import circuit as kc
from oracle import oracle as orc

CURVE = [-4, -2.5e-6, -1, -1e-6, 0, 0, 1, 1e-6, 4, 2.5e-6]


def cap_circuit(value=0.0, curve=CURVE, scale=None, scale_args=(), amp=3.0):
    b = kc.Builder("cn")
    b.voltage_source("V1", "in", "0", 0.0, wave="sin", args=[0, amp, 2e3])
    b.resistor("R1", "in", "a", 500.0)
    b.capacitor("CN", "a", "0", value, curve=curve, scale=scale, scale_args=scale_args)
    return b.build()


def test_state_law_validation():
    assert analysis.validate(cap_circuit(scale="sin", scale_args=[1, 0.3, 5e3])) is None
    assert analysis.validate(cap_circuit(value=1e-6, curve=None, scale="sin", scale_args=[1, 0.3, 5e3])) is None
    bad = {
        "both a value and a curve": cap_circuit(value=1e-6),
        "strictly increase": cap_circuit(curve=[-1, -1e-6, 0, 0, 0.5, 2e-6, 0.4, 3e-6]),
        "through the origin": cap_circuit(curve=[-1, -1e-6, 1, 2e-6]),
        "must be > 0": cap_circuit(value=-1e-6, curve=None, scale="sin", scale_args=[1, 0.3, 5e3]),
        "scale must stay > 0": cap_circuit(scale="sin", scale_args=[1, 1.5, 5e3]),
        "PWL times must strictly increase": cap_circuit(scale="pwl", scale_args=[0, 1, 1e-3, 2, 1e-3, 3]),
    }
    for want, c in bad.items():
        err = analysis.validate(c)
        assert err is not None and want in str(err), (want, err)


def test_knot_crossings_land_on_time_points():
    """Every knot of the charge curve that the voltage crosses during the
    transient is the voltage of some accepted time point (to a thousandth of the
    neighbouring segment's width, knotStep's tolerance)."""
    c = cap_circuit(amp=20.0)
    spec = orc.TranSpec(5e-6, 2e-3, 0.0, 0.0, 0, 0, 0, 0, 0, 0, 0)
    st, t, x, cur, steps, iters, msg = orc.tran(orc.Packed.of(c), spec)
    assert st == 0, msg
    v = x[:, c.node_index("a") - 1]
    for knot, width in ((-1.0, 1.0), (1.0, 1.0)):
        crossed = np.any((v[:-1] - knot) * (v[1:] - knot) < 0)
        on = np.any(np.abs(v - knot) <= 1e-3 * width)
        assert on or not crossed, (knot, crossed, on)
        assert on, knot  # the 20 V drive through 500 Ohm crosses both inner knots


@pytest.mark.parametrize("scale", [None, ("sin", [1, 0.3, 5e3])])
def test_ledger_closes_with_the_scale_port(scale):
    """At every accepted point the ledger's residual is round-off, with the
    power s'(t) F(v) booked through the scale's port; over the run, the
    integrated inflow less outflow and dissipation equals the change of the
    stored energy s (v Q(v) - F(v)) to the integration's accuracy."""
    c = cap_circuit(scale=scale[0] if scale else None, scale_args=scale[1] if scale else ())
    spec = orc.TranSpec(5e-6, 2e-3, 0.0, 0.0, 0, 0, 0, 0, 0, 0, 0)
    out = orc.tran_results(orc.Packed.of(c), spec)
    st, t, x, elem, led, summ = out[:6]
    assert st == 0, out[-1]
    TP, TS = orc.TPOINT, orc.TSUM
    scale_ = np.abs(led[:, :TP["residual"]]).sum(axis=1).max()
    assert np.abs(led[:, TP["residual"]]).max() <= 1e-9 * scale_
    assert summ[TS["max_relative_residual"]] <= 1e-9
    moved = summ[TS["energy_in"]] + summ[TS["energy_dissipated"]]
    assert abs(summ[TS["integration_mismatch"]]) <= 2e-3 * moved, summ
    # the stored energy at the last point: s(t) (v Q(v) - F(v)), F the integral of
    # the piecewise-linear Q from 0 (exact over its knots)
    k = len(t) - 1
    v = x[k, c.node_index("a") - 1]
    xs, ys = np.array(CURVE[0::2]), np.array(CURVE[1::2])
    q = np.interp(v, xs, ys)
    grid = np.sort(np.concatenate([[0.0, v], xs[(xs > min(0.0, v)) & (xs < max(0.0, v))]]))
    qg = np.interp(grid, xs, ys)
    F = float(np.sum(0.5 * (qg[1:] + qg[:-1]) * np.diff(grid))) * (1 if v >= 0 else -1)
    sv = 1 + 0.3 * np.sin(2 * np.pi * 5e3 * t[k]) if scale else 1.0
    w = led[k, TP["stored_energy"]]
    assert abs(w - sv * (v * q - F)) <= 1e-9 * abs(w) + 1e-18, (w, sv * (v * q - F))
