"""Batched scoring of a population for evolutionary circuit search.

The reference scores a generation on a worker pool, one candidate per
goroutine (evaluator.one, evo/engine.go:511-612): validate the decoded circuit,
then run each objective, whose measurements go through a per-candidate cache of
analyses (Eval.OP / AC / Tran, evo/fitness.go:37-205); the first error becomes a
penalty class (Penalty, evo/fitness.go:644-681), otherwise the fitness is the
weighted sum of the objectives' errors.

Here a generation is scored together.  The candidates are validated on the host
and grouped by topology; the first time any objective asks a candidate for an
analysis, that analysis runs once for every candidate of the group through the
engine's batched entry points (ks_op_results, ks_ac, ks_tran_results); each
candidate's objectives then read its slice of the batched result.  Objectives
keep the reference's per-candidate form (an Eval with op(), ac(spec), tran(spec)
that raise the analysis error of that candidate), so a candidate's terms,
fitness and failure class are what the worker pool computes.
"""
from dataclasses import dataclass, replace
import math

import numpy as np

from . import analysis

# Failure classes and their penalty fitness, evo/fitness.go:644-654: a failed
# candidate scores worse than any successful one with total error below 1e5.
PENALTY_NO_MEASUREMENT = 1e6
PENALTY_NO_CONVERGENCE = 2e6
PENALTY_SINGULAR = 3e6
PENALTY_INVALID = 4e6
PENALTY_LEDGER = 5e6
PENALTY_TIMEOUT = 6e6
PENALTY_OTHER = 1e7


class ErrNoMeasurement(analysis.KronspiceError):
    """analysis.ErrNoMeasurement: an objective could not take its measurement."""


class ErrUnknownNode(analysis.KronspiceError):
    """analysis.ErrUnknownNode: a port names a node the circuit does not have."""


def penalty(err):
    """Penalty (evo/fitness.go:659-681): (fitness, class) of an evaluation error."""
    if isinstance(err, analysis.ErrInterrupted):
        return PENALTY_TIMEOUT, "timeout"
    if isinstance(err, analysis.ErrLedgerResidual):
        return PENALTY_LEDGER, "ledger"
    if isinstance(err, ErrNoMeasurement):
        return PENALTY_NO_MEASUREMENT, "no-measurement"
    if isinstance(err, (analysis.ErrNoConvergence, analysis.ErrTimestepTooSmall, analysis.ErrTooManySteps)):
        return PENALTY_NO_CONVERGENCE, "no-convergence"
    if isinstance(err, (analysis.ErrSingularMatrix, analysis.ErrNonFinite)):
        return PENALTY_SINGULAR, "singular"
    if isinstance(err, analysis.ErrValidation):
        return PENALTY_INVALID, "invalid"
    return PENALTY_OTHER, "error"


# ---------------------------------------------------------------- results of one candidate
def _node_value(ckt, x, node):
    i = ckt.node_index(node)
    if i < 0:
        return None
    return 0.0 if i == 0 else x[..., i - 1]


@dataclass
class OPResult:
    """The candidate's output.Result: node voltages, element results, ledger."""
    circuit: object
    x: np.ndarray
    elements: np.ndarray  # [n_elem][RES_COLS]
    ledger: np.ndarray    # [LEDGER_COLS]

    def voltage(self, node):
        v = _node_value(self.circuit, self.x, node)
        return None if v is None else float(v)

    def element(self, name):
        k = self.circuit.element_index(name)
        if k < 0:
            return None
        r = self.elements[k]
        return {c: float(r[j]) for c, j in analysis.RES.items()}

    @property
    def model_supplied(self):
        return float(self.ledger[analysis.LEDGER["model_supplied"]])


@dataclass
class ACResult:
    """The candidate's output.ACResult: frequencies and complex node voltages."""
    circuit: object
    freq: np.ndarray
    x: np.ndarray  # [n_freq][n] complex

    def node_voltage(self, node):
        i = self.circuit.node_index(node)
        if i < 0:
            return None
        return np.zeros(len(self.freq), complex) if i == 0 else self.x[:, i - 1]


@dataclass
class Waveforms:
    """The candidate's output.Waveforms: accepted times, node voltages, per-point
    ledger and element series."""
    circuit: object
    time: np.ndarray
    x: np.ndarray       # [n_points][n]
    ledger: np.ndarray  # [n_points][TPOINT_COLS]
    elements: np.ndarray = None  # [n_points][n_elem][2]: current, absorbed power

    def power(self, name):
        """Waveforms.P of the named element (absorbed power per point), or None."""
        k = self.circuit.element_index(name)
        return None if k < 0 or self.elements is None else self.elements[:, k, 1]

    def node_voltage(self, node):
        i = self.circuit.node_index(node)
        if i < 0:
            return None
        return np.zeros(len(self.time)) if i == 0 else self.x[:, i - 1]

    @property
    def model_supplied(self):
        col = self.ledger[:, analysis.TPOINT["model_supplied"]]
        return float(col.max()) if len(col) else 0.0


# ---------------------------------------------------------------- measurements (analysis/measure.go)
def rel_err(got, want, floor):
    """relErr, evo/fitness.go:209-211."""
    return abs(got - want) / max(abs(want), floor)


def transfer(r, out, ref):
    """analysis.Transfer (analysis/measure.go:20-40): V(out)/V(ref) per frequency."""
    vo = r.node_voltage(out)
    if vo is None:
        raise ErrNoMeasurement("analysis: no measurement")
    if ref in ("0", "gnd", ""):
        return vo
    vr = r.node_voltage(ref)
    if vr is None or np.any(vr == 0):
        raise ErrNoMeasurement("analysis: no measurement")
    return vo / vr


def db(h):
    return 20 * math.log10(abs(h))


def gain_at(freq, h, f):
    """analysis.GainAt (analysis/measure.go:44-56): |H| at f, linear in log-frequency and dB."""
    if len(freq) == 0 or f < freq[0] or f > freq[-1] or f <= 0:
        raise ErrNoMeasurement("analysis: no measurement")
    for k in range(1, len(freq)):
        if f <= freq[k]:
            d0, d1 = db(h[k - 1]), db(h[k])
            x = (math.log(f) - math.log(freq[k - 1])) / (math.log(freq[k]) - math.log(freq[k - 1]))
            return math.pow(10, (d0 + x * (d1 - d0)) / 20)
    return abs(h[0])


def cutoff_3db(freq, h):
    """analysis.Cutoff3dB (analysis/measure.go:58-95): the frequencies where |H|
    falls 3.0103 dB below its peak on each side of it (0 / inf when it does not),
    interpolated in log-frequency and dB."""
    if len(freq) < 2 or len(h) != len(freq):
        raise ErrNoMeasurement("analysis: no measurement")
    mag = np.abs(h)
    kp = int(np.argmax(mag))  # the first maximum, as the strict > scan keeps it
    peak = float(mag[kp])
    if peak == 0:
        raise ErrNoMeasurement("analysis: no measurement")
    thr = db(peak) - 10 * math.log10(2)

    def cross(k0, k1):
        d0, d1 = db(h[k0]), db(h[k1])
        x = (thr - d0) / (d1 - d0)
        l0, l1 = math.log(freq[k0]), math.log(freq[k1])
        return math.exp(l0 + x * (l1 - l0))
    lo, hi = 0.0, math.inf
    for k in range(kp, 0, -1):
        if db(h[k - 1]) < thr:
            lo = cross(k, k - 1)
            break
    for k in range(kp, len(h) - 1):
        if db(h[k + 1]) < thr:
            hi = cross(k, k + 1)
            break
    return lo, hi


def interp(t, y, tq):
    """output.Interp (output/waveforms.go:87-104)."""
    n = len(t)
    if n == 0:
        return math.nan
    if tq <= t[0]:
        return float(y[0])
    if tq >= t[n - 1]:
        return float(y[n - 1])
    k = int(np.searchsorted(t, tq))
    if t[k] == tq:
        return float(y[k])
    return float(y[k - 1] + (y[k] - y[k - 1]) * (tq - t[k - 1]) / (t[k] - t[k - 1]))


# ---------------------------------------------------------------- the batched cache
class _Group:
    """The candidates of one topology and the analyses run for all of them."""

    def __init__(self, idx, circuits, packed, options, capacity):
        self.idx = idx
        self.circuits = [circuits[i] for i in idx]
        self.el = packed[idx[0]][0]
        self.vals = np.stack([packed[i][1] for i in idx])
        self.plan = analysis.Plan(self.el, self.circuits[0].n_nodes, self.vals.shape[1])
        self.options = options
        self.capacity = capacity
        self.row = {i: r for r, i in enumerate(idx)}
        self._batch = None
        self.cache = {}

    def batch(self):
        if self._batch is None:
            self._batch = analysis.Batch(self.plan, self.vals)
        return self._batch

    def op(self):
        if "op" not in self.cache:
            x, st, it, elem, led = self.batch().op_results(self.options)
            self.cache["op"] = (x, st, elem, led)
        return self.cache["op"]

    def ac(self, spec):
        key = ("ac", spec.variation, spec.points, spec.fstart, spec.fstop)
        if key not in self.cache:
            freqs = spec.frequencies()
            x, st, it = self.batch().ac(freqs, self.options)
            self.cache[key] = (freqs, x, st)
        return self.cache[key]

    def port(self, plus, minus):
        """analysis.OpenShort (analysis/port.go:30-69) for every candidate: Voc from
        the group's operating points, Isc from the operating points of the same
        circuits with a 0 V probe source appended from plus to minus (its
        current, into its + terminal, is what the circuit drives out of plus).
        (voc [m], isc [m], failures [m])."""
        key = ("port", plus.lower(), minus.lower())
        if key in self.cache:
            return self.cache[key]
        ckt = self.circuits[0]
        ip, im = ckt.node_index(plus), ckt.node_index(minus)
        m = len(self.idx)
        if ip < 0 or im < 0 or ip == im:
            err = ErrUnknownNode("analysis: unknown node: %s or %s" % (plus, minus) if ip != im or ip < 0
                                 else "analysis: unknown node: %s and %s are the same node" % (plus, minus))
            self.cache[key] = (np.zeros(m), np.zeros(m), [err] * m)
            return self.cache[key]
        x, st, _, _ = self.op()
        vp = np.zeros(m) if ip == 0 else x[:, ip - 1]
        vm = np.zeros(m) if im == 0 else x[:, im - 1]
        fails = [None if s == 0 else type(analysis.status_error(s))("open circuit: %s" % analysis.status_error(s))
                 for s in st]
        # the short: one more element, a V source with its DC value 0 (value block dc, ac magnitude, ac phase)
        from .circuit import ELEMENT_DTYPE, KIND, F_HAS_DC
        el = np.zeros(len(self.el) + 1, dtype=ELEMENT_DTYPE)
        el[:-1] = self.el
        el[-1]["kind"], el[-1]["node"], el[-1]["flags"] = KIND["V"], [ip, im, 0, 0], F_HAS_DC
        el[-1]["param"] = self.vals.shape[1]
        vals = np.hstack([self.vals, np.zeros((m, 3))])
        plan = analysis.Plan(el, ckt.n_nodes, vals.shape[1])
        xs, sts, _, elem, _ = analysis.Batch(plan, vals).op_results(self.options)
        isc = elem[:, len(self.el), analysis.RES["current"]]
        for c in range(m):
            if fails[c] is None and sts[c] != 0:
                e = analysis.status_error(sts[c])
                fails[c] = type(e)("short circuit: %s" % e)
        self.cache[key] = (vp - vm, isc, fails)
        return self.cache[key]

    def tran(self, spec):
        key = ("tran",) + tuple(sorted(vars(spec).items()))
        if key not in self.cache:
            # the adaptive transient with evo's step limit (evo/fitness.go:177); the
            # recording capacity grows until every candidate's points fit
            sp = replace(spec, fixed_step=False, max_steps=spec.max_steps or 200000)
            cap = self.capacity
            while True:
                wave, tim, elem, led, summ, npts, st, steps, it = self.batch().tran_results(sp, self.options,
                                                                                         capacity=cap)
                if int(npts.max()) < cap or cap >= sp.max_steps + 2:
                    break
                cap = min(cap * 4, sp.max_steps + 2)
            self.cache[key] = (wave, tim, led, npts, st, elem)
        return self.cache[key]


class Eval:
    """The per-candidate context handed to objectives (evo/fitness.go:37-63): its
    circuit and gene values, and its analyses, each the candidate's slice of the
    group's batched run (the first request runs it for the whole group)."""

    def __init__(self, circuit, values, group, row, parts=-1):
        self.circuit, self.values = circuit, values
        self._g, self._r = group, row
        self.parts = parts  # evolved parts of a topology genome, -1 for a value genome
        self.model_supplied = 0.0
        self._memo = {}

    def _fail(self, st):
        err = analysis.status_error(st)
        if err is not None:
            raise err

    def op(self):
        """Eval.OP (evo/fitness.go:96-108)."""
        x, st, elem, led = self._g.op()
        self._fail(st[self._r])
        r = OPResult(self.circuit, x[self._r], elem[self._r], led[self._r])
        self.model_supplied = max(self.model_supplied, r.model_supplied)
        return r

    def ac(self, spec):
        """Eval.AC (evo/fitness.go:111-131)."""
        freqs, x, st = self._g.ac(spec)
        self._fail(st[self._r])
        return ACResult(self.circuit, freqs, x[self._r])

    def tran(self, spec):
        """Eval.Tran (evo/fitness.go:171-189)."""
        wave, tim, led, npts, st, elem = self._g.tran(spec)
        self._fail(st[self._r])
        k = int(npts[self._r])
        r = Waveforms(self.circuit, tim[self._r, :k], wave[self._r, :k], led[self._r, :k],
                      None if elem is None else elem[self._r, :k])
        self.model_supplied = max(self.model_supplied, r.model_supplied)
        return r

    def port(self, plus, minus):
        """Eval.Port (evo/fitness.go:191-205): (Voc, Isc) between plus and minus."""
        voc, isc, fails = self._g.port(plus, minus)
        if fails[self._r] is not None:
            raise fails[self._r]
        return float(voc[self._r]), float(isc[self._r])

    def memo(self, key, f):
        """Eval.Memo (evo/fitness.go:69-79): f once per candidate and key."""
        if key not in self._memo:
            try:
                self._memo[key] = (f(), None)
            except analysis.KronspiceError as e:
                self._memo[key] = (None, e)
        v, err = self._memo[key]
        if err is not None:
            raise err
        return v


# ---------------------------------------------------------------- objectives
@dataclass
class Objective:
    """evo.Objective (evo/fitness.go:20-35): eval(Eval) returns a non-negative error.
    batch (optional): the same measurement for every candidate of a topology group
    at once, batch(GroupView) -> (errors [m], failures [m]: None or the exception
    eval would raise); the evaluator uses it in place of eval when present."""
    name: str
    weight: float
    eval: object
    constraint: bool = False
    batch: object = None


class GroupView:
    """The batched analyses of one topology group, for the batch form of objectives."""

    def __init__(self, group):
        self.g = group
        self.circuit = group.circuits[0]
        self.m = len(group.idx)
        self.used_op = False  # the objective read the operating point

    def _status(self, st):
        return [analysis.status_error(s) for s in st]

    def op(self):
        """(x [m][n], elem [m][n_elem][RES_COLS], ledger [m][LEDGER_COLS], failures [m])."""
        self.used_op = True
        x, st, elem, led = self.g.op()
        return x, elem, led, self._status(st)

    def ac(self, spec):
        """(freqs, x [m][n_freq][n] complex, failures [m])."""
        freqs, x, st = self.g.ac(spec)
        return freqs, x, self._status(st)

    def node(self, name):
        return self.circuit.node_index(name)


def _no_measurement():
    return ErrNoMeasurement("analysis: no measurement")


def op_voltage(node, target):
    """OPVoltage (evo/fitness.go:528-540)."""
    def ev(e):
        v = e.op().voltage(node)
        if v is None:
            raise ErrNoMeasurement("analysis: no measurement")
        return rel_err(v, target, 1e-3)

    def batch(gv):
        x, _, _, fails = gv.op()
        i = gv.node(node)
        if i < 0:
            return np.zeros(gv.m), [f or _no_measurement() for f in fails]
        v = np.zeros(gv.m) if i == 0 else x[:, i - 1]
        return np.abs(v - target) / max(abs(target), 1e-3), fails
    return Objective("v(%s)" % node, 1.0, ev, batch=batch)


def supply_power(*sources):
    """SupplyPower (evo/fitness.go:312-329)."""
    def ev(e):
        r = e.op()
        p = 0.0
        for s in sources:
            el = r.element(s)
            if el is None:
                raise ErrNoMeasurement("analysis: no measurement: no element %r" % s)
            p -= el["power"]
        return max(0.0, p)

    def batch(gv):
        x, elem, _, fails = gv.op()
        ks = [gv.circuit.element_index(s) for s in sources]
        if any(k < 0 for k in ks):
            return np.zeros(gv.m), [f or _no_measurement() for f in fails]
        p = np.zeros(gv.m)
        for k in ks:
            p -= elem[:, k, analysis.RES["power"]]
        return np.maximum(0.0, p), fails
    return Objective("supply power", 1.0, ev, batch=batch)


def port_voc(plus, minus, target):
    """PortVoc (evo/fitness.go:608-617): the open-circuit voltage between plus and minus."""
    def ev(e):
        return rel_err(e.port(plus, minus)[0], target, 1e-6)
    return Objective("Voc %s,%s" % (plus, minus), 1.0, ev)


def port_isc(plus, minus, target):
    """PortIsc (evo/fitness.go:619-628): the short-circuit current out of plus."""
    def ev(e):
        return rel_err(e.port(plus, minus)[1], target, 1e-12)
    return Objective("Isc %s,%s" % (plus, minus), 1.0, ev)


def model_supplied_limit(pmax):
    """ModelSuppliedLimit (evo/fitness.go:630-641)."""
    def ev(e):
        return max(0.0, e.op().model_supplied - pmax) / max(pmax, 1e-12)

    def batch(gv):
        _, _, led, fails = gv.op()
        return np.maximum(0.0, led[:, analysis.LEDGER["model_supplied"]] - pmax) / max(pmax, 1e-12), fails
    return Objective("model-supplied power", 1.0, ev, batch=batch)


def gain_at_objective(node, ref, spec, f, target_db):
    """GainAt (evo/fitness.go:241-259)."""
    def ev(e):
        h = transfer(e.ac(spec), node, ref)
        g = gain_at(e.ac(spec).freq, h, f)
        if g <= 0:
            raise ErrNoMeasurement("analysis: no measurement")
        return abs(20 * math.log10(g) - target_db) / 20

    def batch(gv):
        freqs, x, fails = gv.ac(spec)
        io, ir = gv.node(node), gv.node(ref)
        bad = io < 0 or (ref not in ("0", "gnd", "") and ir < 0) or len(freqs) == 0 or not (
            freqs[0] <= f <= freqs[-1]) or f <= 0
        if bad:
            return np.zeros(gv.m), [fl or _no_measurement() for fl in fails]
        vo = np.zeros(x.shape[:2], complex) if io == 0 else x[:, :, io - 1]
        if ref in ("0", "gnd", ""):
            h = vo
            zero = np.zeros(gv.m, bool)
        else:
            vr = np.zeros(x.shape[:2], complex) if ir == 0 else x[:, :, ir - 1]
            zero = np.any(vr == 0, axis=1)
            with np.errstate(divide="ignore", invalid="ignore"):
                h = vo / np.where(vr == 0, 1.0, vr)
        k = int(np.searchsorted(freqs, f))  # the first frequency >= f (GainAt's segment end)
        with np.errstate(divide="ignore", invalid="ignore"):
            if k == 0:
                g = np.abs(h[:, 0])
            else:
                d0, d1 = 20 * np.log10(np.abs(h[:, k - 1])), 20 * np.log10(np.abs(h[:, k]))
                t = (math.log(f) - math.log(freqs[k - 1])) / (math.log(freqs[k]) - math.log(freqs[k - 1]))
                g = np.power(10.0, (d0 + t * (d1 - d0)) / 20)
            err = np.abs(20 * np.log10(g) - target_db) / 20
        out = []
        for c in range(gv.m):
            if fails[c] is not None:
                out.append(fails[c])
            elif zero[c] or not (g[c] > 0) or not np.isfinite(err[c]):
                out.append(_no_measurement())
            else:
                out.append(None)
        return np.where(np.isfinite(err), err, 0.0), out
    return Objective("gain %s at %g Hz" % (node, f), 1.0, ev, batch=batch)


def cutoff(node, ref, spec, target, high):
    """Cutoff (evo/fitness.go:213-238): the upper (high) or lower -3 dB edge of
    V(node)/V(ref) against target [Hz]."""
    def ev(e):
        r = e.ac(spec)
        lo, hi = cutoff_3db(r.freq, transfer(r, node, ref))
        f = hi if high else lo
        if f == 0 or math.isinf(f):
            raise ErrNoMeasurement("analysis: no measurement")
        return rel_err(f, target, 0)
    return Objective("cutoff " + node, 1.0, ev)


def gain_shortfall(node, ref, spec, f, ceiling_db):
    """GainShortfall (evo/fitness.go:261-281): max(0, ceiling - gain at f) / 20."""
    def ev(e):
        r = e.ac(spec)
        g = gain_at(r.freq, transfer(r, node, ref), f)
        if g <= 0:
            raise ErrNoMeasurement("analysis: no measurement")
        return max(0.0, ceiling_db - 20 * math.log10(g)) / 20
    return Objective("gain short %s at %g Hz" % (node, f), 1.0, ev)


def bandwidth_shortfall(node, ref, spec, ceiling_hz):
    """BandwidthShortfall (evo/fitness.go:283-309): decades the upper -3 dB edge
    (the sweep's stop when the response has not fallen) lies below the ceiling."""
    def ev(e):
        r = e.ac(spec)
        _, hi = cutoff_3db(r.freq, transfer(r, node, ref))
        hi = min(hi, float(r.freq[-1]))
        if not hi > 0:
            raise ErrNoMeasurement("analysis: no measurement")
        return max(0.0, math.log10(ceiling_hz / hi))
    return Objective("bandwidth short " + node, 1.0, ev)


def op_efficiency(*loads):
    """OPEfficiency (evo/fitness.go:331-346, em/efficiency.go:29-43): 1 - the
    loads' absorbed power over the net inflow of the operating point's ledger."""
    def ev(e):
        r = e.op()
        net = r.ledger[analysis.LEDGER["inflow"]] - r.ledger[analysis.LEDGER["outflow"]]
        if net <= 0:
            raise ErrNoMeasurement("analysis: no measurement: em: no net inflow")
        p = 0.0
        for n in loads:
            el = r.element(n)
            if el is None:
                raise ErrNoMeasurement("analysis: no measurement: em: OPEfficiency: no element %r" % n)
            p += el["power"]
        return 1 - p / net
    return Objective("1 - efficiency", 1.0, ev)


@dataclass
class Band:
    """evo.Band (evo/fitness.go:364-370): between lo and hi [Hz] the gain must
    lie within [min_db, max_db] (-inf / inf for an open side)."""
    lo: float
    hi: float
    min_db: float
    max_db: float


MASK_VIOLATION_FLOOR = 0.1  # evo.MaskViolationFloor, evo/fitness.go:376


def filter_mask(node, ref, spec, bands):
    """FilterMask (evo/fitness.go:378-449): 0 inside the mask everywhere, else the
    floor + the fraction of checked points outside + their mean excess in dB/20."""
    def ev(e):
        r = e.ac(spec)
        h = transfer(r, node, ref)
        fr = r.freq
        n = bad = 0
        excess = 0.0

        def check(f, b):
            nonlocal n, bad, excess
            lo, hi = fr[0], fr[-1]  # a band edge a rounding error outside the sweep
            if lo * (1 - 1e-9) < f < lo:
                f = lo
            elif hi < f < hi * (1 + 1e-9):
                f = hi
            g = gain_at(fr, h, f)
            d_b = 20 * math.log10(g) if g > 0 else -math.inf
            n += 1
            d = 0.0
            if d_b > b.max_db:
                d = d_b - b.max_db
            elif d_b < b.min_db:
                d = min(b.min_db - d_b, 200.0)  # a dead output counts 200 dB
            if d > 0:
                bad += 1
                excess += d
        for b in bands:
            check(b.lo, b)
            for f in fr:
                if b.lo < f < b.hi:
                    check(f, b)
            check(b.hi, b)
        return 0.0 if bad == 0 else MASK_VIOLATION_FLOOR + bad / n + excess / 20 / n
    return Objective("mask " + node, 1.0, ev)


def active_bias(vmin, imin, imax):
    """ActiveBias (evo/fitness.go:451-516): how near the best-biased transistor is
    to its forward-active region at the operating point (0 inside, at most 1; 1
    without a transistor)."""
    def ev(e):
        r = e.op()
        c = e.circuit
        best = 1.0
        for k, el in enumerate(c.elements):
            if el.kind not in ("Q", "M"):
                continue
            res = r.elements[k]
            typ = c.models.get(el.model, ("",))[0]
            sign = -1.0 if typ in ("pnp", "pmos") else 1.0
            v, i = sign * res[analysis.RES["voltage"]], sign * res[analysis.RES["current"]]
            d = max(0.0, (vmin - v) / vmin)
            if i <= 0:
                d += 1
            elif i < imin:
                d += math.log10(imin / i) / 3
            elif i > imax:
                d += math.log10(i / imax) / 3
            if el.kind == "Q":  # nodes: collector, emitter, base
                vc, ve, vb = (r.voltage(nm) for nm in el.nodes[:3])
                vbe, vbc = sign * (vb - ve), sign * (vb - vc)
                d += (max(0.0, 0.4 - vbe) + max(0.0, vbe - 1.0)) / 0.5
                d += max(0.0, vbc - 0.4) / 0.4
            best = min(best, d)
        return min(best, 1.0)
    return Objective("active bias", 1.0, ev)


def part_count():
    """PartCount (evo/fitness.go:518-526): the evolved parts of a topology genome."""
    def ev(e):
        if e.parts < 0:
            raise ErrNoMeasurement("analysis: no measurement: parts objective needs a topology genome")
        return float(e.parts)
    return Objective("parts", 1.0, ev)


def _integrate(t, y, t_from, t_to):
    """em.integrate (em/efficiency.go:83-94): trapezoids over the points, interpolated at the ends."""
    s_ = 0.0
    for k in range(1, len(t)):
        t0, t1 = t[k - 1], t[k]
        if t1 <= t_from or t0 >= t_to:
            continue
        a, b = max(t0, t_from), min(t1, t_to)
        s_ += 0.5 * (interp(t, y, a) + interp(t, y, b)) * (b - a)
    return s_


def tran_efficiency(spec, t_from, t_to, *loads):
    """TranEfficiency (evo/fitness.go:347-362, em/efficiency.go:52-80): 1 - the
    loads' absorbed energy over the net energy the exterior delivered in [from, to]."""
    def ev(e):
        wf = e.tran(spec)
        if not t_to > t_from:
            raise ErrNoMeasurement("analysis: no measurement: em: TranEfficiency: empty window")
        load = np.zeros(len(wf.time))
        for n in loads:
            p = wf.power(n)
            if p is None:
                raise ErrNoMeasurement("analysis: no measurement: em: TranEfficiency: no element %r" % n)
            load = load + p
        e_load = _integrate(wf.time, load, t_from, t_to)
        e_in = (_integrate(wf.time, wf.ledger[:, analysis.TPOINT["inflow"]], t_from, t_to)
                - _integrate(wf.time, wf.ledger[:, analysis.TPOINT["outflow"]], t_from, t_to))
        if e_in <= 0:
            raise ErrNoMeasurement("analysis: no measurement: em: no net inflow")
        return 1 - e_load / e_in
    return Objective("1 - efficiency", 1.0, ev)


def tran_average(node, spec, t_from, t_to, target):
    """TranAverage (evo/fitness.go:553-583): the mean of V(node) over [from, to]."""
    def ev(e):
        wf = e.tran(spec)
        y = wf.node_voltage(node)
        if y is None:
            raise ErrNoMeasurement("analysis: no measurement")
        t = wf.time
        area = span = 0.0
        for k in range(1, len(t)):
            t0, t1 = t[k - 1], t[k]
            if t1 <= t_from or t0 >= t_to:
                continue
            a, b = max(t0, t_from), min(t1, t_to)
            area += 0.5 * (interp(t, y, a) + interp(t, y, b)) * (b - a)
            span += b - a
        if span <= 0:
            raise ErrNoMeasurement("analysis: no measurement")
        return rel_err(area / span, target, 1e-3)
    return Objective("mean v(%s)" % node, 1.0, ev)


def tran_ripple(node, spec, t_from, t_to, vmax):
    """TranRipple (evo/fitness.go:584-606): a constraint on V(node)'s peak to peak."""
    def ev(e):
        wf = e.tran(spec)
        y = wf.node_voltage(node)
        if y is None:
            raise ErrNoMeasurement("analysis: no measurement")
        w = y[(wf.time >= t_from) & (wf.time <= t_to)]
        if len(w) < 2 or vmax <= 0:
            raise ErrNoMeasurement("analysis: no measurement")
        return max(0.0, float(w.max() - w.min()) - vmax) / vmax
    return Objective("ripple v(%s)" % node, 1.0, ev)


# ---------------------------------------------------------------- the population
@dataclass
class Individual:
    """evo.Individual (evo/engine.go:185-203) without the genome and Pareto fields."""
    values: list
    fitness: float = 0.0
    terms: list = None
    failure: str = ""
    error: str = ""
    model_supplied: float = 0.0


def evaluate(circuits, objectives, options=None, values=None, capacity=20000, parts=None):
    """Score a population (evaluator.evaluate + one, evo/engine.go:518-612): one
    Individual per circuit, in order.  `values` are the candidates' gene values
    (reported back); `capacity` is the transient recording capacity a group
    starts from; `parts` the evolved part counts of topology genomes (None: value
    genomes, Eval.Parts = -1)."""
    opt = options or analysis.Options()
    n = len(circuits)
    out = [Individual(values=list(values[i]) if values is not None else []) for i in range(n)]

    def fail(ind, err):
        ind.fitness, ind.failure = penalty(err)
        ind.error = str(err)
        ind.terms = None

    # Validate (:564-574): a floating node is tolerated when the transient is defined
    ok, keys, packed = [], {}, {}
    for i, c in enumerate(circuits):
        try:
            el, vals, key = c.pack()
            err = analysis.validate_packed(el, c.n_nodes, vals)
            if isinstance(err, analysis.ErrFloatingNode) and analysis.validate_packed(el, c.n_nodes, vals, True) is None:
                err = None
            packed[i] = (el, vals)
            # the names too: a group's objectives read node and element names once for all its rows
            key = (key, tuple(c.node_names), tuple(e.name.lower() for e in c.elements))
        except analysis.KronspiceError as e:
            err = e
        except (ValueError, KeyError) as e:  # the circuit does not pack: a bad value or model
            err = analysis.ErrValidation("circuit: %s" % e)
        if err is not None:
            fail(out[i], err)
            continue
        ok.append(i)
        keys.setdefault(key, []).append(i)
    groups = {}
    for key, idx in keys.items():
        # small groups run the generic kernels: no per-topology compilation
        g_opt = opt if len(idx) >= 256 or opt.kernel != "auto" else replace(opt, kernel="generic")
        g = _Group(idx, circuits, packed, g_opt, capacity)
        for i in idx:
            groups[i] = g
    seen = []
    for i in ok:
        if groups[i] not in seen:
            seen.append(groups[i])
    for g in seen:
        _score_group(g, objectives, out, fail, parts)
    return out


def _score_group(g, objectives, out, fail, parts=None):
    """The objectives of one topology group in order (:591-607), each in its batch
    form when it has one (else candidate by candidate); a candidate stops at its
    first failing objective."""
    m = len(g.idx)
    terms = np.zeros((m, len(objectives)))
    first_fail = [None] * m
    evals = [None] * m
    ran_op = np.zeros(m, bool)  # an objective read the candidate's operating point (Eval.OP)
    for k, ob in enumerate(objectives):
        live = [c for c in range(m) if first_fail[c] is None]
        if not live:
            break
        if ob.batch is not None:
            gv = GroupView(g)
            v, fails = ob.batch(gv)
            if gv.used_op:
                ran_op[live] = True
            for c in live:
                err = fails[c]
                if err is None and (math.isnan(v[c]) or math.isinf(v[c]) or v[c] < 0):
                    err = ErrNoMeasurement("analysis: no measurement: objective %r returned %r" % (ob.name, v[c]))
                if err is not None:
                    first_fail[c] = type(err)("%s: %s" % (ob.name, err))
                else:
                    terms[c, k] = v[c]
            continue
        for c in live:
            if evals[c] is None:
                i = g.idx[c]
                evals[c] = Eval(g.circuits[c], out[i].values, g, c, -1 if parts is None else parts[i])
            try:
                v = ob.eval(evals[c])
                if v is None or math.isnan(v) or math.isinf(v) or v < 0:
                    raise ErrNoMeasurement("analysis: no measurement: objective %r returned %r" % (ob.name, v))
            except analysis.KronspiceError as err:
                first_fail[c] = type(err)("%s: %s" % (ob.name, err))
                continue
            terms[c, k] = v
    # model-supplied power: the largest over the operating points and transients the
    # candidate's own objectives ran (Eval.noteSupplied, evo/fitness.go:90-94)
    ms = np.zeros(m)
    if "op" in g.cache:
        st, led = g.cache["op"][1], g.cache["op"][3]
        ms = np.where(ran_op & (st == 0), led[:, analysis.LEDGER["model_supplied"]], 0.0)
    for c in range(m):
        if evals[c] is not None:
            ms[c] = max(ms[c], evals[c].model_supplied)
    w = np.array([ob.weight for ob in objectives])
    for c in range(m):
        ind = out[g.idx[c]]
        ind.model_supplied = float(ms[c])
        if first_fail[c] is not None:
            fail(ind, first_fail[c])
            continue
        ind.terms = [float(t) for t in terms[c]]
        ind.fitness = float(np.dot(w, terms[c]))


def evaluate_values(circuit, values, objectives, options=None, genes=None, capacity=20000):
    """Score candidates of one topology given as value vectors (the value genome,
    Eval.Parts = -1): row i of `values` is candidate i's value vector in the
    layout circuit.pack() gives, so no circuit is built or packed per candidate.
    Each row is validated as circuit.Validate would the decoded circuit; then the
    candidates are scored as evaluate scores one topology group."""
    opt = options or analysis.Options()
    el, v0, _ = circuit.pack()
    vals = np.ascontiguousarray(values, dtype=np.float64)
    if vals.ndim != 2 or vals.shape[1] != len(v0):
        raise ValueError("evaluate_values: values must be [n_candidates][%d]" % len(v0))
    n = vals.shape[0]
    out = [Individual(values=list(genes[i]) if genes is not None else []) for i in range(n)]

    def fail(ind, err):
        ind.fitness, ind.failure = penalty(err)
        ind.error = str(err)
        ind.terms = None

    ok, packed = [], {}
    for i in range(n):
        err = analysis.validate_packed(el, circuit.n_nodes, vals[i])
        if isinstance(err, analysis.ErrFloatingNode) and analysis.validate_packed(el, circuit.n_nodes, vals[i], True) is None:
            err = None
        if err is not None:
            fail(out[i], err)
            continue
        ok.append(i)
        packed[i] = (el, vals[i])
    if ok:
        g_opt = opt if len(ok) >= 256 or opt.kernel != "auto" else replace(opt, kernel="generic")
        _score_group(_Group(ok, [circuit] * n, packed, g_opt, capacity), objectives, out, fail)
    return out
