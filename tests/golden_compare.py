"""Golden-vector comparators with the reference's tolerances (test infrastructure).

Restates internal/golden/golden.go: Compare (:84-107), CompareTable (:188-214),
CompareTableAtSim (:226-260, bracketDistance :272-287), CompareSweep (:341-372)
and output.Interp (output/waveforms.go:87-104).
"""
import bisect
import math

ABS_V, ABS_I, REL = 1e-6, 1e-12, 1e-3   # internal/golden/golden.go:22-27
TRAN_FULL_SCALE = 2e-3                  # internal/golden/golden.go:184


def interp(t, y, tq):
    n = len(t)
    if n == 0:
        return math.nan
    if tq <= t[0]:
        return y[0]
    if tq >= t[n - 1]:
        return y[n - 1]
    k = bisect.bisect_left(t, tq)
    if t[k] == tq:
        return y[k]
    t0, t1 = t[k - 1], t[k]
    return y[k - 1] + (y[k] - y[k - 1]) * (tq - t0) / (t1 - t0)


def compare_values(got, want):
    msgs = []
    for k in sorted(want):
        w = want[k]
        if k not in got:
            msgs.append("%s: missing (want %g)" % (k, w))
            continue
        ab = ABS_I if k.startswith("i(") else ABS_V
        tol = max(ab, REL * abs(w))
        if abs(got[k] - w) > tol:
            msgs.append("%s: got %.9g, want %.9g (tolerance %.3g)" % (k, got[k], w, tol))
    return msgs


def compare_table(sim_t, get, want):
    msgs = []
    for name in want["names"]:
        y = get(name)
        if y is None:
            msgs.append("%s: not in simulation" % name)
            continue
        ref = want["columns"][name]
        full = max(abs(v) for v in ref)
        tol = max(TRAN_FULL_SCALE * full, ABS_V)
        worst, at = 0.0, 0.0
        for k, tq in enumerate(want["xs"]):
            d = abs(interp(sim_t, y, tq) - ref[k])
            if d > worst:
                worst, at = d, tq
        if worst > tol:
            msgs.append("%s: max error %.3g at t = %.4g s (tolerance %.3g)" % (name, worst, at, tol))
    return msgs


def _bracket(ts, ref, t, v):
    i = bisect.bisect_left(ts, t)
    if i == 0 or i >= len(ts):
        return math.inf
    lo, hi = min(ref[i - 1], ref[i]), max(ref[i - 1], ref[i])
    if v < lo:
        return lo - v
    if v > hi:
        return v - hi
    return 0.0


def compare_table_at_sim(sim_t, get, want):
    msgs = []
    t0, t1 = want["xs"][0], want["xs"][-1]
    for name in want["names"]:
        y = get(name)
        if y is None:
            msgs.append("%s: not in simulation" % name)
            continue
        ref = want["columns"][name]
        full = max(abs(v) for v in ref)
        tol = max(TRAN_FULL_SCALE * full, ABS_V)
        worst, at = 0.0, 0.0
        for k, ts in enumerate(sim_t):
            if ts < t0 or ts > t1:
                continue
            d = abs(y[k] - interp(want["xs"], ref, ts))
            if d > tol:
                d = min(d, _bracket(want["xs"], ref, ts, y[k]))
            if d > worst:
                worst, at = d, ts
        if worst > tol:
            msgs.append("%s: max error %.3g at t = %.6g s (tolerance %.3g)" % (name, worst, at, tol))
    return msgs


def compare_sweep(sweep, get, want):
    if len(sweep) != len(want["xs"]):
        return ["sweep has %d points, want %d" % (len(sweep), len(want["xs"]))]
    msgs = []
    for name in want["names"]:
        y = get(name)
        if y is None:
            msgs.append("%s: not in simulation" % name)
            continue
        ab = ABS_I if name.startswith("i(") else ABS_V
        for k, ref in enumerate(want["columns"][name]):
            if abs(sweep[k] - want["xs"][k]) > 1e-9 * max(1, abs(want["xs"][k])):
                return msgs + ["sweep point %d is %g, want %g" % (k, sweep[k], want["xs"][k])]
            tol = max(ab, REL * abs(ref))
            if abs(y[k] - ref) > tol:
                msgs.append("%s at %g: got %.9g, want %.9g (tolerance %.3g)" % (name, sweep[k], y[k], ref, tol))
                break
    return msgs


def sweep_values(start, stop, step):
    """DCSweep.values, analysis/dc.go:36-50."""
    n = (stop - start) / step
    count = int(math.floor(n + 1e-9)) + 1
    return [start + k * step for k in range(count)]


def ac_frequencies(variation, points, fstart, fstop):
    """ACSpec.Frequencies, analysis/ac.go:33-72."""
    import math
    if points < 1 or fstop < fstart or fstart < 0:
        raise ValueError("bad AC spec")
    if variation == "lin":
        if points == 1:
            return [fstart]
        step = (fstop - fstart) / (points - 1)
        return [fstart + k * step for k in range(points)]
    base = 10.0 if variation == "dec" else 2.0
    ratio = math.pow(base, 1.0 / points)
    n = int(math.floor(math.log(fstop / fstart) / math.log(ratio) + 1e-9)) + 1
    return [fstart * math.pow(ratio, k) for k in range(n)]


AC_REL, AC_PHASE_DEG = 1e-6, 1e-4  # internal/golden/golden.go:290-295


def compare_ac(freq, get, want):
    """CompareAC, internal/golden/golden.go:297-340: vm() to 1e-6 relative, vp() to 1e-4 degrees."""
    import cmath
    import math
    msgs = []
    xs = want["xs"]
    if len(freq) != len(xs):
        return ["frequency count %d, want %d" % (len(freq), len(xs))]
    for k in range(len(freq)):
        if abs(freq[k] - xs[k]) > 1e-9 * xs[k]:
            return ["frequency %d is %g, want %g" % (k, freq[k], xs[k])]
    for name in want["names"]:
        if len(name) < 4 or name[:3] not in ("vm(", "vp("):
            msgs.append("%s: unsupported AC column" % name)
            continue
        v = get(name[3:-1])
        if v is None:
            msgs.append("%s: node not in simulation" % name)
            continue
        for k, ref in enumerate(want["columns"][name]):
            if name[:3] == "vm(":
                got = abs(v[k])
                if abs(got - ref) > AC_REL * max(abs(ref), 1e-12):
                    msgs.append("%s at %g Hz: got %.10g, want %.10g" % (name, freq[k], got, ref))
                    break
            else:
                got = cmath.phase(v[k]) * 180 / math.pi
                d = math.fmod(abs(got - ref), 360)
                if d > 180:
                    d = 360 - d
                if d > AC_PHASE_DEG:
                    msgs.append("%s at %g Hz: got %.8g, want %.8g" % (name, freq[k], got, ref))
                    break
    return msgs
