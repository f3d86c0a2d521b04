// ks_devices.cuh — device models of the GB300 engine, evaluated in FP64.
//
// One thread evaluates one circuit; every thread of a warp runs the same
// element program (same topology), so the kind switch is warp-uniform and the
// per-circuit operands are coalesced columns of the SoA arrays.  The model
// equations are those of the reference's devices, cited per function.
// Stamps go into a per-thread dense matrix in shared memory (stride TPB).
#pragma once
#ifndef __CUDACC_RTC__
#include <cuda_runtime.h>
#include <stdint.h>
#endif
#include "ks_engine.h"
#include "../../include/kronspice_gpu.h"

namespace ksg {

#define KS_INF __longlong_as_double(0x7ff0000000000000LL)
// Element callbacks are inlined at every call: with a per-topology program each
// call sees its element as constants and the per-thread system stays in registers.
#define KS_INLINE_LAMBDA __attribute__((always_inline))

constexpr double kQ = 1.602176634e-19;     // device/diode.go:15
constexpr double kK = 1.380649e-23;        // device/diode.go:16
constexpr double kTNom = 300.15;           // device/diode.go:18
constexpr double kE = 2.718281828459045235360287;
constexpr double kSqrt2 = 1.41421356237309504880168872;
constexpr double kPi = 3.14159265358979323846264338;
constexpr double kEpsOx = 3.9 * 8.854214871e-12;   // device/mosfet.go:117
constexpr double kEpsSi = 11.7 * 8.854214871e-12;  // device/mosfet.go:118
constexpr double kNiSi = 1.45e16;                  // device/mosfet.go:119

enum { ModeOP = 0, ModeTranOP = 1, ModeUICInit = 2, ModeTran = 3 };
enum { BE = 1, TRAP = 2 };

// One circuit's column of a SoA array: element k at p[k * B].
struct Col {
  double* p;
  int64_t B;
  __device__ __forceinline__ double& operator[](int k) const { return p[(int64_t)k * B]; }
};

// Stamping into a thread's system S (shared-memory or register storage, see
// ks_solve.cuh): S provides a(i, j), rhs(i), xo(i) (the linearization point X of
// the current load) and xn(i) (the new iterate).  Ground (-1) is dropped.
// Systems shared by the lanes of a warp (kAtomic) take the adds atomically.
template <class S>
__device__ __forceinline__ void sadd(S& s, int i, int j, double v) {
  if (i < 0 || j < 0) return;
  if constexpr (S::kAtomic) s.add(i, j, v);
  else s.a(i, j) += v;
}
template <class S>
__device__ __forceinline__ void srhs(S& s, int i, double v) {
  if (i < 0) return;
  if constexpr (S::kAtomic) s.add_rhs(i, v);
  else s.rhs(i) += v;
}
template <class S>
__device__ __forceinline__ double xo_(S& s, int i) { return i >= 0 ? s.xo(i) : 0.0; }
template <class S>
__device__ __forceinline__ double xn_(S& s, int i) { return i >= 0 ? s.xn(i) : 0.0; }

struct LoadParams {  // device/device.go:127-148
  int mode, method;
  double time, h;
  double rh;  // 1/h, set with h: the companion models multiply instead of dividing per element
  bool initJct;
  double gmin;
  bool srcStepping;
  double srcFact;
};

struct TruncParams { double time, h; int method; double reltol, abstol, vntol, chgtol, trtol; };

// ---------------------------------------------------------------- history / LTE
__device__ inline void hist_push(const Col& S, int h, double t, double q) {  // device/lte.go:23-31
  S[h + H_T2] = S[h + H_T1]; S[h + H_T1] = S[h + H_T0]; S[h + H_T0] = t;
  S[h + H_Q2] = S[h + H_Q1]; S[h + H_Q1] = S[h + H_Q0]; S[h + H_Q0] = q;
  if (S[h + H_N] < 3) S[h + H_N] += 1;
}
__device__ inline void hist_reset(const Col& S, int h) { S[h + H_N] = 0; }

// lteStep, device/lte.go:50-85.
__device__ inline double lte_step(const Col& S, int h, double qn, double in, double inPrev, double absTol,
                                  const TruncParams& tc) {
  int k = tc.method;
  if (k < 1 || k > 2 || S[h + H_N] < k + 1) return KS_INF;
  double ts[4] = {tc.time, S[h + H_T0], S[h + H_T1], S[h + H_T2]};
  double dd[4] = {qn, S[h + H_Q0], S[h + H_Q1], S[h + H_Q2]};
  for (int order = 1; order <= k + 1; order++) {
    for (int i = 0; i + order <= k + 1; i++) {
      double den = ts[i] - ts[i + order];
      if (den == 0) return KS_INF;
      dd[i] = (dd[i] - dd[i + 1]) / den;
    }
  }
  double fact = k == 2 ? 6.0 : 2.0, c = k == 2 ? 1.0 / 12 : 0.5;
  double hh = tc.h;
  double errI = c * (k == 2 ? hh * hh : hh) * fabs(dd[0] * fact);
  if (errI == 0 || isnan(errI)) return KS_INF;
  double qmax = fmax(fabs(qn), fabs(S[h + H_Q0]));
  double allowed = tc.trtol * fmax(tc.reltol * fmax(fabs(in), fabs(inPrev)) + absTol, tc.reltol * fmax(qmax, tc.chgtol) / hh);
  return k == 2 ? hh * sqrt(allowed / errI) : hh * (allowed / errI);
}

// pnjlim, device/diode.go:214-226 (rvt = 1/vt).
__device__ __forceinline__ double pnjlim(double vnew, double vold, double vt, double rvt, double vcrit, bool* lim) {
  if (vnew > vcrit && fabs(vnew - vold) > 2 * vt) {
    *lim = true;
    if (vold > 0) {
      double arg = 1 + (vnew - vold) * rvt;
      return arg > 0 ? vold + vt * log(arg) : vcrit;
    }
    return vt * log(vnew * rvt);
  }
  *lim = false;
  return vnew;
}

// ---------------------------------------------------------------- waveforms
// resolveWave, device/waveform.go:25-66: into the derived block a[0..6].
__device__ inline void wave_resolve(int kind, const Col& V, int args, int nargs, const Col& D, int d,
                                    double step, double stop) {
  if (step <= 0) step = 1e-9;
  if (stop <= 0) stop = 1e-6;
  auto arg = [&](int i, double def) { return i < nargs ? V[args + i] : def; };
  double a[7] = {0, 0, 0, 0, 0, 0, 0};
  if (kind == KS_WAVE_PULSE) {
    a[0] = arg(0, 0); a[1] = arg(1, 0); a[2] = arg(2, 0); a[3] = arg(3, step); a[4] = arg(4, step);
    a[5] = arg(5, stop); a[6] = arg(6, stop);
    if (a[3] == 0) a[3] = step;
    if (a[4] == 0) a[4] = step;
  } else if (kind == KS_WAVE_SIN) {
    a[0] = arg(0, 0); a[1] = arg(1, 0); a[2] = arg(2, 1 / stop); a[3] = arg(3, 0); a[4] = arg(4, 0); a[5] = arg(5, 0);
  } else if (kind == KS_WAVE_EXP) {
    double td1 = arg(2, 0);
    a[0] = arg(0, 0); a[1] = arg(1, 0); a[2] = td1; a[3] = arg(3, step); a[4] = arg(4, td1 + step); a[5] = arg(5, step);
    if (a[3] == 0) a[3] = step;
    if (a[5] == 0) a[5] = step;
  }
  for (int i = 0; i < 7; i++) D[d + i] = a[i];
}

// wave.value, device/waveform.go:69-126.
__device__ inline double wave_value(int kind, const Col& D, int d, const Col& V, int args, int nargs, double t) {
  if (kind == KS_WAVE_PULSE) {
    double v1 = D[d], v2 = D[d + 1], td = D[d + 2], tr = D[d + 3], tf = D[d + 4], pw = D[d + 5], per = D[d + 6];
    if (t < td) return v1;
    double tt = t - td;
    if (per > 0) tt = fmod(tt, per);
    if (tt < tr) return v1 + (v2 - v1) * tt / tr;
    if (tt < tr + pw) return v2;
    if (tt < tr + pw + tf) return v2 + (v1 - v2) * (tt - tr - pw) / tf;
    return v1;
  }
  if (kind == KS_WAVE_SIN) {
    double vo = D[d], va = D[d + 1], f = D[d + 2], td = D[d + 3], theta = D[d + 4], ph = D[d + 5] * kPi / 180;
    if (t < td) return vo + va * sin(ph);
    double tt = t - td;
    return vo + va * exp(-tt * theta) * sin(2 * kPi * f * tt + ph);
  }
  if (kind == KS_WAVE_EXP) {
    double v1 = D[d], v2 = D[d + 1], td1 = D[d + 2], tau1 = D[d + 3], td2 = D[d + 4], tau2 = D[d + 5];
    if (t < td1) return v1;
    if (t < td2) return v1 + (v2 - v1) * (1 - exp(-(t - td1) / tau1));
    return v1 + (v2 - v1) * (1 - exp(-(t - td1) / tau1)) + (v1 - v2) * (1 - exp(-(t - td2) / tau2));
  }
  if (kind == KS_WAVE_PWL) {
    int n = nargs / 2;
    if (t <= V[args]) return V[args + 1];
    if (t >= V[args + 2 * (n - 1)]) return V[args + 2 * n - 1];
    int k = 1;
    while (k < n && !(V[args + 2 * k] > t)) k++;
    double t0 = V[args + 2 * (k - 1)], v0 = V[args + 2 * (k - 1) + 1], t1 = V[args + 2 * k], v1 = V[args + 2 * k + 1];
    if (t1 == t0) return v1;
    return v0 + (v1 - v0) * (t - t0) / (t1 - t0);
  }
  return 0;
}

// wave.slope, device/waveform.go:131-186.
__device__ inline double wave_slope(int kind, const Col& D, int d, const Col& V, int args, int nargs, double t) {
  if (kind == KS_WAVE_PULSE) {
    double v1 = D[d], v2 = D[d + 1], td = D[d + 2], tr = D[d + 3], tf = D[d + 4], pw = D[d + 5], per = D[d + 6];
    if (t <= td) return 0;
    double tt = t - td;
    if (per > 0) {
      tt = fmod(tt, per);
      if (tt == 0) tt = per;  // the end of the previous period
    }
    if (tt <= tr) return (v2 - v1) / tr;
    if (tt <= tr + pw) return 0;
    if (tt <= tr + pw + tf) return (v1 - v2) / tf;
    return 0;
  }
  if (kind == KS_WAVE_SIN) {
    double va = D[d + 1], f = D[d + 2], td = D[d + 3], theta = D[d + 4], ph = D[d + 5] * kPi / 180;
    if (t <= td) return 0;
    double tt = t - td, om = 2 * kPi * f;
    return va * exp(-tt * theta) * (om * cos(om * tt + ph) - theta * sin(om * tt + ph));
  }
  if (kind == KS_WAVE_EXP) {
    double v1 = D[d], v2 = D[d + 1], td1 = D[d + 2], tau1 = D[d + 3], td2 = D[d + 4], tau2 = D[d + 5];
    if (t <= td1) return 0;
    double r = (v2 - v1) / tau1 * exp(-(t - td1) / tau1);
    if (t > td2) r += (v1 - v2) / tau2 * exp(-(t - td2) / tau2);
    return r;
  }
  if (kind == KS_WAVE_PWL) {
    int n = nargs / 2;
    if (t <= V[args] || t > V[args + 2 * (n - 1)]) return 0;
    int k = 1;  // segment k-1 -> k ends at or after t
    while (k < n && !(V[args + 2 * k] >= t)) k++;
    double t0 = V[args + 2 * (k - 1)], v0 = V[args + 2 * (k - 1) + 1], t1 = V[args + 2 * k], v1 = V[args + 2 * k + 1];
    if (t1 == t0) return 0;
    return (v1 - v0) / (t1 - t0);
  }
  return 0;
}

// wave.nextBreakpoint, device/waveform.go:190-239.
__device__ inline double wave_next_breakpoint(int kind, const Col& D, int d, const Col& V, int args, int nargs, double t) {
  const double rel = 1e-12;
  double lim = t + rel * fmax(fabs(t), 1e-15);
  if (kind == KS_WAVE_PULSE) {
    double td = D[d + 2], tr = D[d + 3], tf = D[d + 4], pw = D[d + 5], per = D[d + 6];
    double edges[4] = {0, tr, tr + pw, tr + pw + tf};
    if (per <= 0) {
      for (int i = 0; i < 4; i++) if (td + edges[i] > lim) return td + edges[i];
      return KS_INF;
    }
    double k = floor((t - td) / per);
    if (k < 0) k = 0;
    for (double kk = k; kk <= k + 1; kk++) {
      double base = td + kk * per;
      for (int i = 0; i < 4; i++) if (base + edges[i] > lim) return base + edges[i];
    }
    return td + (k + 2) * per;
  }
  if (kind == KS_WAVE_SIN) { if (D[d + 3] > lim) return D[d + 3]; }
  else if (kind == KS_WAVE_EXP) {
    if (D[d + 2] > lim) return D[d + 2];
    if (D[d + 4] > lim) return D[d + 4];
  } else if (kind == KS_WAVE_PWL) {
    for (int k = 0; k < nargs / 2; k++) if (V[args + 2 * k] > lim) return V[args + 2 * k];
  }
  return KS_INF;
}

// sourceValue.at, device/source.go:43-66 (SV_OVR/SV_OVRON: the .DC override).
__device__ inline double source_at(const KElem& e, const Col& V, const Col& D, const Col& S, const LoadParams& lp) {
  double v;
  if (S[SV_OVRON] != 0 && lp.mode == ModeOP) v = S[SV_OVR];
  else if (e.wave == KS_WAVE_NONE) v = V[e.param + KS_SRC_P_DC];
  else if (lp.mode == ModeOP && (e.flags & KS_F_HAS_DC)) v = V[e.param + KS_SRC_P_DC];
  else v = wave_value(e.wave, D, e.derived, V, e.param + KS_SRC_P_ARGS, e.nargs, lp.mode == ModeTran ? lp.time : 0.0);
  if (lp.srcStepping && lp.mode != ModeTran) v *= lp.srcFact;
  return v;
}

// ---------------------------------------------------------------- diode
// current, device/diode.go:148-162 (dd: derived block of the diode).
__device__ inline void diode_iv(const Col& V, const Col& Dv, int p, int dd, bool hasBV, double v, double* id, double* g) {
  double IS = V[p + KS_D_P_IS], vte = Dv[dd + DD_VTE], rvte = Dv[dd + DD_RVTE];
  if (v >= -3 * vte) {
    double e = exp(fmin(v * rvte, 700.0));
    *id = IS * (e - 1); *g = IS * e * rvte; return;
  }
  double xbv = Dv[dd + DD_XBV];
  if (!hasBV || v >= -xbv) {
    double a = 3 * vte / (v * kE); a = a * a * a;
    *id = -IS * (1 + a); *g = IS * 3 * a / v; return;
  }
  double e = exp(fmin(-(xbv + v) * rvte, 700.0));
  *id = -IS * e; *g = IS * e * rvte;
}

// charge, device/diode.go:191-211.
__device__ inline void diode_charge(const Col& V, int p, double v, double id, double g, double* q, double* c) {
  double TT = V[p + KS_D_P_TT], CJO = V[p + KS_D_P_CJO], VJ = V[p + KS_D_P_VJ], M = V[p + KS_D_P_M], FC = V[p + KS_D_P_FC];
  *q = TT * id; *c = TT * g;
  if (CJO == 0) return;
  double fcv = FC * VJ;
  if (v < fcv) {
    double arg = 1 - v / VJ, sarg = pow(arg, -M);
    *q += CJO * VJ * (1 - arg * sarg) / (1 - M);
    *c += CJO * sarg;
    return;
  }
  double f1 = VJ * (1 - pow(1 - FC, 1 - M)) / (1 - M), f2 = pow(1 - FC, 1 + M), f3 = 1 - FC * (1 + M);
  *q += CJO * f1 + CJO / f2 * (f3 * (v - fcv) + M / (2 * VJ) * (v * v - fcv * fcv));
  *c += CJO / f2 * (f3 + M * v / VJ);
}

// Load, device/diode.go:229-275.
template <class SY>
__device__ __forceinline__ void diode_load(const KElem& e, const Col& V, const Col& Dv, const Col& S, SY& sys,
                                  const LoadParams& lp) {
  int p = e.param, dd = e.derived;
  int a = e.u[0], k = e.u[1], ai = e.u[2];
  bool hasBV = e.flags & KS_F_HAS_BV;
  double vte = Dv[dd + DD_VTE], vcrit = Dv[dd + DD_VCRIT], xbv = Dv[dd + DD_XBV];
  double vraw = xo_(sys, ai) - xo_(sys, k);
  double vd;
  bool lim;
  if (lp.initJct) { vd = vcrit; lim = true; }
  else {
    double vacc = S[SD_VDACC];
    const double rvte = Dv[dd + DD_RVTE];
    vd = pnjlim(vraw, vacc, vte, rvte, vcrit, &lim);
    if (hasBV && vraw < fmin(0.0, -xbv + 10 * vte)) {
      bool l2;
      double vt = pnjlim(-(vraw + xbv), -(vacc + xbv), vte, rvte, vcrit, &l2);
      vd = -(vt + xbv); lim = l2;
    }
  }
  S[SD_VDACC] = vd;
  double id, g0;
  diode_iv(V, Dv, p, dd, hasBV, vd, &id, &g0);
  double cd = id + lp.gmin * vd, gd = g0 + lp.gmin;
  double iq = 0, geq = 0;
  bool tran = false;
  if (lp.mode == ModeTran && (V[p + KS_D_P_CJO] > 0 || V[p + KS_D_P_TT] > 0)) {
    double q, c;
    diode_charge(V, p, vd, id, g0, &q, &c);
    tran = true;
    if (lp.method == TRAP) { iq = 2 * (q - S[SD_QPREV]) * lp.rh - S[SD_IQPREV]; geq = 2 * c * lp.rh; }
    else { iq = (q - S[SD_QPREV]) * lp.rh; geq = c * lp.rh; }
  }
  S[SD_VD] = vd; S[SD_CD] = cd; S[SD_GD] = gd; S[SD_IQ] = iq; S[SD_GEQ] = geq;
  S[SD_LIM] = lim ? 1.0 : 0.0; S[SD_TRAN] = tran ? 1.0 : 0.0;
  double gg = gd + geq, ieq = cd + iq - gg * vd;
  sadd(sys, ai, ai, gg); sadd(sys, k, k, gg); sadd(sys, ai, k, -gg); sadd(sys, k, ai, -gg);
  srhs(sys, ai, -ieq); srhs(sys, k, ieq);
  double grs = Dv[dd + DD_GRS];
  if (grs > 0) { sadd(sys, a, a, grs); sadd(sys, ai, ai, grs); sadd(sys, a, ai, -grs); sadd(sys, ai, a, -grs); }
}

// ConvTest, device/diode.go:282-289.
template <class SY>
__device__ __forceinline__ bool diode_conv(const KElem& e, const Col& V, const Col& Dv, const Col& S, SY& sys,
                                  double reltol, double abstol, double gmin) {
  double v = xn_(sys, e.u[2]) - xn_(sys, e.u[1]);
  double cdhat = S[SD_CD] + S[SD_GD] * (v - S[SD_VD]);
  double id, g;
  diode_iv(V, Dv, e.param, e.derived, e.flags & KS_F_HAS_BV, v, &id, &g);
  double cdn = id + gmin * v;
  return fabs(cdhat - cdn) <= reltol * fmax(fabs(cdhat), fabs(cdn)) + abstol;
}

// Accept, device/diode.go:304-322.
template <class SY>
__device__ __forceinline__ void diode_accept(const KElem& e, const Col& V, const Col& Dv, const Col& S, SY& sys,
                                    double t, int mode) {
  double v = xn_(sys, e.u[2]) - xn_(sys, e.u[1]);
  S[SD_VDACC] = v;
  double id, g, q, c;
  diode_iv(V, Dv, e.param, e.derived, e.flags & KS_F_HAS_BV, v, &id, &g);
  diode_charge(V, e.param, v, id, g, &q, &c);
  if (mode == ModeTran) S[SD_IQPREV] = S[SD_TRAN] != 0 ? S[SD_IQ] + S[SD_GEQ] * (v - S[SD_VD]) : 0.0;
  else { S[SD_IQPREV] = 0; hist_reset(S, SD_HIST); }
  S[SD_QPREV] = q;
  hist_push(S, SD_HIST, t, q);
}

// ---------------------------------------------------------------- BJT
// junction, device/bjt.go:272-283 (rnvt = 1/nvt).
__device__ __forceinline__ void junction(double is, double v, double nvt, double rnvt, double* i, double* g) {
  if (is == 0) { *i = 0; *g = 0; return; }
  if (v >= -3 * nvt) {
    double e = exp(fmin(v * rnvt, 700.0));
    *i = is * (e - 1); *g = is * e * rnvt; return;
  }
  double a = 3 * nvt / (v * kE); a = a * a * a;
  *i = -is * (1 + a); *g = is * 3 * a / v;
}

struct BjtDC { double cbe, gbe, cbc, gbc, it, itBE, itBC, ibe, gpi, ibc, gmu, qb, dqbdve, dqbdvc, gx; };

// evalDC, device/bjt.go:294-354, with the divisions by per-circuit constants
// taken from their reciprocals and the three divisions by qb as one.
__device__ __forceinline__ BjtDC bjt_eval_dc(const Col& V, const Col& Dv, int p, int dd, double vbe, double vbc,
                                             double gmin) {
  BjtDC d;
  double vt = Dv[dd + DQ_VT];
  junction(V[p + KS_Q_P_IS], vbe, V[p + KS_Q_P_NF] * vt, Dv[dd + DQ_RNF], &d.cbe, &d.gbe);
  double cben, gben;
  junction(V[p + KS_Q_P_ISE], vbe, V[p + KS_Q_P_NE] * vt, Dv[dd + DQ_RNE], &cben, &gben);
  cben += gmin * vbe; gben += gmin;
  junction(V[p + KS_Q_P_IS], vbc, V[p + KS_Q_P_NR] * vt, Dv[dd + DQ_RNR], &d.cbc, &d.gbc);
  double cbcn, gbcn;
  junction(V[p + KS_Q_P_ISC], vbc, V[p + KS_Q_P_NC] * vt, Dv[dd + DQ_RNC], &cbcn, &gbcn);
  cbcn += gmin * vbc; gbcn += gmin;
  double ivaf = Dv[dd + DQ_IVAF], ivar = Dv[dd + DQ_IVAR], oik = Dv[dd + DQ_OIK], oikr = Dv[dd + DQ_OIKR];
  double q1 = 1 / (1 - ivaf * vbc - ivar * vbe);
  if (oik == 0 && oikr == 0) {
    d.qb = q1; d.dqbdve = q1 * d.qb * ivar; d.dqbdvc = q1 * d.qb * ivaf;
  } else {
    double q2 = oik * d.cbe + oikr * d.cbc;
    double arg = fmax(0.0, 1 + 4 * q2);
    double sq = arg != 0 ? sqrt(arg) : 1.0;
    double rsq = 1 / sq;
    d.qb = q1 * (1 + sq) / 2;
    d.dqbdve = q1 * (d.qb * ivar + oik * d.gbe * rsq);
    d.dqbdvc = q1 * (d.qb * ivaf + oikr * d.gbc * rsq);
  }
  double rqb = 1 / d.qb;
  d.it = (d.cbe - d.cbc) * rqb;
  d.itBE = (d.gbe - d.it * d.dqbdve) * rqb;
  d.itBC = (-d.gbc - d.it * d.dqbdvc) * rqb;
  double rBF = Dv[dd + DQ_RBF], rBR = Dv[dd + DQ_RBR];
  d.ibe = d.cbe * rBF + cben; d.gpi = d.gbe * rBF + gben;
  d.ibc = d.cbc * rBR + cbcn; d.gmu = d.gbc * rBR + gbcn;
  double rbpr = Dv[dd + DQ_RBPR], rbpi = Dv[dd + DQ_RBPI];
  double gx = rbpr + rbpi * rqb;
  double IRB = V[p + KS_Q_P_IRB];
  if (IRB > 0 && rbpi != 0) {
    double cb = d.ibe + d.ibc;
    double a1 = fmax(cb / IRB, 1e-9);
    double z = (-1 + sqrt(1 + 14.59025 * a1)) / 2.4317 / sqrt(a1);
    double tz = tan(z);
    gx = rbpr + 3 * rbpi * (tz - z) / z / tz / tz;
  }
  d.gx = gx != 0 ? 1 / gx : 0;
  return d;
}

// depletion, device/bjt.go:358-370.
__device__ inline void depletion(double v, double cz, double vj, double m, double fc, double f1, double f2, double f3,
                                 double* q, double* c) {
  if (cz == 0) { *q = 0; *c = 0; return; }
  double fcv = fc * vj;
  if (v < fcv) {
    double arg = 1 - v / vj, sarg = exp(-m * log(arg));
    *q = vj * cz * (1 - arg * sarg) / (1 - m); *c = cz * sarg; return;
  }
  double czf2 = cz / f2;
  *q = cz * f1 + czf2 * (f3 * (v - fcv) + (m / (vj + vj)) * (v * v - fcv * fcv));
  *c = czf2 * (f3 + m * v / vj);
}

struct BjtCh { double q[4], c[4], dqbeDvbc; };

// charges, device/bjt.go:373-412.
__device__ inline BjtCh bjt_charges(const Col& V, const Col& Dv, int p, int dd, double vbe, double vbc, double vbx,
                                    double vcs, const BjtDC& d) {
  BjtCh ch;
  ch.dqbeDvbc = 0;
  double cbe = d.cbe, gbe = d.gbe;
  double TF = V[p + KS_Q_P_TF], XTF = V[p + KS_Q_P_XTF], ITF = V[p + KS_Q_P_ITF], ovtf = Dv[dd + DQ_OVTF];
  if (TF != 0 && vbe > 0) {
    double argtf = 0, arg2 = 0, arg3 = 0;
    if (XTF != 0) {
      argtf = XTF;
      if (ovtf != 0) argtf *= exp(vbc * ovtf);
      arg2 = argtf;
      if (ITF != 0) {
        double t = cbe / (cbe + ITF);
        argtf *= t * t;
        arg2 = argtf * (3 - t - t);
      }
      arg3 = cbe * argtf * ovtf;
    }
    double rqb = 1 / d.qb;
    cbe = cbe * (1 + argtf) * rqb;
    gbe = (gbe * (1 + arg2) - cbe * d.dqbdve) * rqb;
    ch.dqbeDvbc = TF * (arg3 - cbe * d.dqbdvc) * rqb;
  }
  double qd, cd;
  double FC = V[p + KS_Q_P_FC];
  depletion(vbe, V[p + KS_Q_P_CJE], V[p + KS_Q_P_VJE], V[p + KS_Q_P_MJE], FC, Dv[dd + DQ_F1E], Dv[dd + DQ_F2E],
            Dv[dd + DQ_F3E], &qd, &cd);
  ch.q[0] = TF * cbe + qd; ch.c[0] = TF * gbe + cd;
  double CJC = V[p + KS_Q_P_CJC], czbc = CJC * V[p + KS_Q_P_XCJC];
  double VJC = V[p + KS_Q_P_VJC], MJC = V[p + KS_Q_P_MJC];
  depletion(vbc, czbc, VJC, MJC, FC, Dv[dd + DQ_F1C], Dv[dd + DQ_F2C], Dv[dd + DQ_F3C], &qd, &cd);
  double TR = V[p + KS_Q_P_TR];
  ch.q[1] = TR * d.cbc + qd; ch.c[1] = TR * d.gbc + cd;
  depletion(vbx, CJC - czbc, VJC, MJC, FC, Dv[dd + DQ_F1C], Dv[dd + DQ_F2C], Dv[dd + DQ_F3C], &ch.q[2], &ch.c[2]);
  ch.q[3] = 0; ch.c[3] = 0;
  double CJS = V[p + KS_Q_P_CJS];
  if (CJS != 0) {
    double VJS = V[p + KS_Q_P_VJS], MJS = V[p + KS_Q_P_MJS];
    if (vcs < 0) {
      double arg = 1 - vcs / VJS, sarg = exp(-MJS * log(arg));
      ch.q[3] = VJS * CJS * (1 - arg * sarg) / (1 - MJS); ch.c[3] = CJS * sarg;
    } else {
      ch.q[3] = vcs * CJS * (1 + MJS * vcs / (2 * VJS)); ch.c[3] = CJS * (1 + MJS * vcs / VJS);
    }
  }
  return ch;
}

template <bool NEW, class SY>
__device__ inline void bjt_voltages(const KElem& e, SY& s, double* vbe, double* vbc, double* vbx,
                                    double* vcs) {  // device/bjt.go:415-419 (NEW: at the new iterate, else at X)
  auto X = [&](int i) { return NEW ? xn_(s, i) : xo_(s, i); };
  double t = (e.flags & KS_F_PTYPE) ? -1.0 : 1.0;
  double vb = X(e.u[2]), vbp = X(e.u[5]), vcp = X(e.u[4]), vep = X(e.u[6]);
  *vbe = t * (vbp - vep); *vbc = t * (vbp - vcp); *vbx = t * (vb - vcp);
  *vcs = t * (X(e.u[7]) - X(e.u[8]));
}

template <class SY>
__device__ __forceinline__ void bjt_branch(SY& s, double typ, int a, int b, double i0, double g1, int p1,
                                           int n1, double v10, double g2, int p2, int n2, double v20) {  // :463-480
  if (g1 != 0) { sadd(s, a, p1, g1); sadd(s, a, n1, -g1); sadd(s, b, p1, -g1); sadd(s, b, n1, g1); }
  if (g2 != 0) { sadd(s, a, p2, g2); sadd(s, a, n2, -g2); sadd(s, b, p2, -g2); sadd(s, b, n2, g2); }
  double ieq = typ * (i0 - g1 * v10 - g2 * v20);
  srhs(s, a, -ieq); srhs(s, b, ieq);
}

template <class SY>
__device__ __forceinline__ void stamp_g(SY& s, int a, int b, double g) {  // device/bjt.go:482-490
  if (g == 0) return;
  sadd(s, a, a, g); sadd(s, b, b, g); sadd(s, a, b, -g); sadd(s, b, a, -g);
}

// Load + stamp, device/bjt.go:422-515.
template <class SY>
__device__ __forceinline__ void bjt_load(const KElem& e, const Col& V, const Col& Dv, const Col& S, SY& sys,
                                const LoadParams& lp) {
  int p = e.param, dd = e.derived;
  double vt = Dv[dd + DQ_VT], vcrit = Dv[dd + DQ_VCRIT];
  double vbe, vbc, vbx, vcs;
  bjt_voltages<false>(e, sys, &vbe, &vbc, &vbx, &vcs);
  bool lim;
  if (lp.initJct) { vbe = vcrit; vbc = 0; lim = true; vbx = 0; vcs = 0; }
  else {
    bool l1, l2;
    const double rvt = Dv[dd + DQ_RVT];
    vbe = pnjlim(vbe, S[SQ_VBEACC], vt, rvt, vcrit, &l1);
    vbc = pnjlim(vbc, S[SQ_VBCACC], vt, rvt, vcrit, &l2);
    lim = l1 || l2;
  }
  S[SQ_VBEACC] = vbe; S[SQ_VBCACC] = vbc;
  S[SQ_VBE] = vbe; S[SQ_VBC] = vbc; S[SQ_VBX] = vbx; S[SQ_VCS] = vcs;
  BjtDC d = bjt_eval_dc(V, Dv, p, dd, vbe, vbc, lp.gmin);
  double isub, gsub;
  junction(V[p + KS_Q_P_ISS], vcs, V[p + KS_Q_P_NS] * vt, Dv[dd + DQ_RNS], &isub, &gsub);
  isub += lp.gmin * vcs; gsub += lp.gmin;
  S[SQ_CBE] = d.cbe; S[SQ_GBE] = d.gbe; S[SQ_CBC] = d.cbc; S[SQ_GBC] = d.gbc; S[SQ_IT] = d.it;
  S[SQ_ITBE] = d.itBE; S[SQ_ITBC] = d.itBC; S[SQ_IBE] = d.ibe; S[SQ_GPI] = d.gpi; S[SQ_IBC] = d.ibc;
  S[SQ_GMU] = d.gmu; S[SQ_QB] = d.qb; S[SQ_DQBDVE] = d.dqbdve; S[SQ_DQBDVC] = d.dqbdvc; S[SQ_GX] = d.gx;
  S[SQ_ISUB] = isub; S[SQ_GSUB] = gsub; S[SQ_LIM] = lim ? 1.0 : 0.0;
  bool hasCharge = V[p + KS_Q_P_CJE] > 0 || V[p + KS_Q_P_CJC] > 0 || V[p + KS_Q_P_CJS] > 0 ||
                   V[p + KS_Q_P_TF] > 0 || V[p + KS_Q_P_TR] > 0;
  bool tran = lp.mode == ModeTran && hasCharge;
  double ag = 0, iq[4] = {0, 0, 0, 0};
  BjtCh ch;
  if (tran) {
    ch = bjt_charges(V, Dv, p, dd, vbe, vbc, vbx, vcs, d);
    ag = lp.method == TRAP ? 2 * lp.rh : lp.rh;
    for (int k = 0; k < 4; k++) {
      iq[k] = ag * (ch.q[k] - S[SQ_QPREV0 + k]);
      if (lp.method == TRAP) iq[k] -= S[SQ_IQPREV0 + k];
      S[SQ_C0 + k] = ch.c[k];
    }
    S[SQ_DQBEDVBC] = ch.dqbeDvbc;
  }
  S[SQ_TRAN] = tran ? 1.0 : 0.0; S[SQ_AG] = ag;
  for (int k = 0; k < 4; k++) S[SQ_IQ0 + k] = iq[k];
  double typ = (e.flags & KS_F_PTYPE) ? -1.0 : 1.0;
  int b = e.u[2], cp = e.u[4], bp = e.u[5], ep = e.u[6], sa = e.u[7], sb = e.u[8];
  bjt_branch(sys, typ, cp, ep, d.it, d.itBE, bp, ep, vbe, d.itBC, bp, cp, vbc);
  bjt_branch(sys, typ, bp, ep, d.ibe, d.gpi, bp, ep, vbe, 0, 0, 0, 0);
  bjt_branch(sys, typ, bp, cp, d.ibc, d.gmu, bp, cp, vbc, 0, 0, 0, 0);
  bjt_branch(sys, typ, sa, sb, isub, gsub, sa, sb, vcs, 0, 0, 0, 0);
  if (tran) {
    bjt_branch(sys, typ, bp, ep, iq[0], ag * ch.c[0], bp, ep, vbe, ag * ch.dqbeDvbc, bp, cp, vbc);
    bjt_branch(sys, typ, bp, cp, iq[1], ag * ch.c[1], bp, cp, vbc, 0, 0, 0, 0);
    bjt_branch(sys, typ, b, cp, iq[2], ag * ch.c[2], b, cp, vbx, 0, 0, 0, 0);
    bjt_branch(sys, typ, sa, sb, iq[3], ag * ch.c[3], sa, sb, vcs, 0, 0, 0, 0);
  }
  if (bp != b) stamp_g(sys, b, bp, d.gx);
  if (cp != e.u[0]) stamp_g(sys, e.u[0], cp, Dv[dd + DQ_GCPR]);
  if (ep != e.u[1]) stamp_g(sys, e.u[1], ep, Dv[dd + DQ_GEPR]);
}

// ConvTest, device/bjt.go:522-532.
template <class SY>
__device__ __forceinline__ bool bjt_conv(const KElem& e, const Col& V, const Col& Dv, const Col& S, SY& sys,
                                double reltol, double abstol, double gmin) {
  double vbe, vbc, vbx, vcs;
  bjt_voltages<true>(e, sys, &vbe, &vbc, &vbx, &vcs);
  double dbe = vbe - S[SQ_VBE], dbc = vbc - S[SQ_VBC];
  double ichat = S[SQ_IT] - S[SQ_IBC] + S[SQ_ITBE] * dbe + (S[SQ_ITBC] - S[SQ_GMU]) * dbc;
  double ibhat = S[SQ_IBE] + S[SQ_IBC] + S[SQ_GPI] * dbe + S[SQ_GMU] * dbc;
  BjtDC n = bjt_eval_dc(V, Dv, e.param, e.derived, vbe, vbc, gmin);
  double ic = n.it - n.ibc, ib = n.ibe + n.ibc;
  return fabs(ichat - ic) <= reltol * fmax(fabs(ichat), fabs(ic)) + abstol &&
         fabs(ibhat - ib) <= reltol * fmax(fabs(ibhat), fabs(ib)) + abstol;
}

// Accept, device/bjt.go:579-601.
template <class SY>
__device__ __forceinline__ void bjt_accept(const KElem& e, const Col& V, const Col& Dv, const Col& S, SY& sys,
                                  double t, int mode, double gmin) {
  double vbe, vbc, vbx, vcs;
  bjt_voltages<true>(e, sys, &vbe, &vbc, &vbx, &vcs);
  S[SQ_VBEACC] = vbe; S[SQ_VBCACC] = vbc;
  BjtDC d = bjt_eval_dc(V, Dv, e.param, e.derived, vbe, vbc, gmin);
  BjtCh ch = bjt_charges(V, Dv, e.param, e.derived, vbe, vbc, vbx, vcs, d);
  double dv[4] = {vbe - S[SQ_VBE], vbc - S[SQ_VBC], vbx - S[SQ_VBX], vcs - S[SQ_VCS]};
  bool tran = S[SQ_TRAN] != 0;
  for (int k = 0; k < 4; k++) {
    if (mode == ModeTran && tran) {
      double i = S[SQ_IQ0 + k] + S[SQ_AG] * S[SQ_C0 + k] * dv[k];
      if (k == 0) i += S[SQ_AG] * S[SQ_DQBEDVBC] * dv[1];
      S[SQ_IQPREV0 + k] = i;
    } else S[SQ_IQPREV0 + k] = 0;
    if (mode != ModeTran) hist_reset(S, SQ_HIST + k * H_SIZE);
    S[SQ_QPREV0 + k] = ch.q[k];
    hist_push(S, SQ_HIST + k * H_SIZE, t, ch.q[k]);
  }
}

// ---------------------------------------------------------------- switch
// device/switch.go:28-332: S (u[3], u[4] the control nodes) and W (u[3] the
// controlling source's branch).  Abrupt: RON or ROFF with hysteresis about VT,
// the state referred to the last accepted solution and held through a transient
// step; smooth (VH < 0): ln R a cubic in the control between VT -+ |VH|.
// The control at the new iterate xn (NEW) or at the load's linearization point xo.
template <bool NEW = true, class SY>
__device__ __forceinline__ double sw_control(const KElem& e, SY& sys) {  // :132-137
  auto X = [&](int i) { return NEW ? xn_(sys, i) : xo_(sys, i); };
  return e.kind == KS_ELEM_W ? X(e.u[3]) : X(e.u[3]) - X(e.u[4]);
}

__device__ __forceinline__ bool sw_next(const Col& V, const Col& Dv, const KElem& e, double c, bool prev) {  // :140-148
  const double vt = V[e.param + KS_SW_P_VT], vh = Dv[e.derived + DW_VH];
  if (c > vt + vh) return true;
  if (c < vt - vh) return false;
  return prev;
}

// smoothG, :151-162: the smooth switch's conductance and dg/dc at control c.
__device__ __forceinline__ void sw_smooth_g(const Col& V, const Col& Dv, const KElem& e, double c, double* g, double* dg) {
  const double vt = V[e.param + KS_SW_P_VT], vh = Dv[e.derived + DW_VH];
  const double x = (c - vt) / vh;
  if (x >= 1) { *g = 1 / V[e.param + KS_SW_P_RON]; *dg = 0; return; }
  if (x <= -1) { *g = 1 / V[e.param + KS_SW_P_ROFF]; *dg = 0; return; }
  const double lratio = Dv[e.derived + DW_LRATIO];
  *g = exp(-(Dv[e.derived + DW_LMEAN] + lratio * (3 * x - x * x * x) / 4));
  *dg = -*g * lratio * 3 * (1 - x * x) / (4 * vh);
}

// Load, :174-226.
template <class SY>
__device__ __forceinline__ void sw_load(const KElem& e, const Col& V, const Col& Dv, const Col& S, SY& sys,
                                        const LoadParams& lp) {
  const int a = e.u[0], b = e.u[1];
  double g;
  if (Dv[e.derived + DW_SMOOTH] != 0) {
    double c = sw_control<false>(e, sys), v = xo_(sys, a) - xo_(sys, b);
    if (lp.initJct) {
      const double vt = V[e.param + KS_SW_P_VT], vh = Dv[e.derived + DW_VH];
      c = Dv[e.derived + DW_INIT] != 0 ? vt + vh : vt - vh;
      v = 0;
    }
    double dg;
    sw_smooth_g(V, Dv, e, c, &g, &dg);
    const double k = dg * v;
    S[SW_G] = g; S[SW_K] = k; S[SW_C0] = c;
    sadd(sys, a, a, g); sadd(sys, b, b, g); sadd(sys, a, b, -g); sadd(sys, b, a, -g);
    if (k != 0) {
      if (e.kind == KS_ELEM_W) { sadd(sys, a, e.u[3], k); sadd(sys, b, e.u[3], -k); }
      else { sadd(sys, a, e.u[3], k); sadd(sys, a, e.u[4], -k); sadd(sys, b, e.u[3], -k); sadd(sys, b, e.u[4], k); }
      const double j0 = -k * c;
      srhs(sys, a, -j0); srhs(sys, b, j0);
    }
    return;
  }
  const bool frozen = lp.mode == ModeTran;
  const bool acc = S[SW_ACC] != 0;
  const bool on = (lp.initJct || frozen) ? acc : sw_next(V, Dv, e, sw_control<false>(e, sys), acc);
  g = on ? 1 / V[e.param + KS_SW_P_RON] : 1 / V[e.param + KS_SW_P_ROFF];
  S[SW_FROZEN] = frozen; S[SW_ON] = on; S[SW_G] = g; S[SW_K] = 0;
  sadd(sys, a, a, g); sadd(sys, b, b, g); sadd(sys, a, b, -g); sadd(sys, b, a, -g);
}

// ConvTest, :231-243.
template <class SY>
__device__ __forceinline__ bool sw_conv(const KElem& e, const Col& V, const Col& Dv, const Col& S, SY& sys,
                                        double reltol, double abstol) {
  const double c = sw_control(e, sys);
  if (Dv[e.derived + DW_SMOOTH] == 0)
    return S[SW_FROZEN] != 0 || sw_next(V, Dv, e, c, S[SW_ACC] != 0) == (S[SW_ON] != 0);
  const double v = xn_(sys, e.u[0]) - xn_(sys, e.u[1]);
  double g, dg;
  sw_smooth_g(V, Dv, e, c, &g, &dg);
  const double ihat = S[SW_G] * v + S[SW_K] * (c - S[SW_C0]), i = g * v;
  return fabs(ihat - i) <= reltol * fmax(fabs(i), fabs(ihat)) + abstol;
}

// Accept, :253-261.
template <class SY>
__device__ __forceinline__ void sw_accept(const KElem& e, const Col& V, const Col& Dv, const Col& S, SY& sys) {
  const double c = sw_control(e, sys);
  S[SW_CACC] = c; S[SW_ACCEPTED] = 1;
  if (Dv[e.derived + DW_SMOOTH] == 0) {
    const bool acc = S[SW_ACC] != 0, on = sw_next(V, Dv, e, c, acc);
    S[SW_FLIP] = on != acc;
    S[SW_ACC] = on; S[SW_ON] = on;
  }
}

// LimitStep, :268-285: cut a transient step in which an abrupt switch changed
// state to just past the crossing, unless it lies in the step's last hundredth.
template <class SY>
__device__ __forceinline__ double sw_limit_step(const KElem& e, const Col& V, const Col& Dv, const Col& S, SY& sys,
                                                double h) {
  if (Dv[e.derived + DW_SMOOTH] != 0 || S[SW_ACCEPTED] == 0) return KS_INF;
  const double c = sw_control(e, sys), cacc = S[SW_CACC];
  const bool acc = S[SW_ACC] != 0;
  if (sw_next(V, Dv, e, c, acc) == acc || c == cacc) return KS_INF;
  const double vt = V[e.param + KS_SW_P_VT], vh = Dv[e.derived + DW_VH];
  const double th = acc ? vt - vh : vt + vh;
  const double frac = (th - cacc) / (c - cacc);
  if (!(frac > 0) || frac >= 0.99) return KS_INF;
  return h * fmin(frac + 0.005, 1.0);
}

// ---------------------------------------------------------------- nonlinear / time-varying C and L
// stateLaw, device/nonlinear_reactive.go:15-249: y(x, t) = s(t) f(x), f the
// element's piecewise-linear curve (knots x0, y0, x1, y1, ... after the SCALE
// arguments in its value block) or value * x.
struct NlLaw {
  const Col& V;
  const Col& D;
  int c0, n, d;      // first curve value, knots, derived block
  double lin;
  int wave, args, nargs;
  __device__ __forceinline__ NlLaw(const KElem& e, const Col& V_, const Col& D_)
      : V(V_), D(D_), c0(e.param + KS_NL_P_ARGS + e.nargs), n(e.level / 2), d(e.derived),
        lin(V_[e.param + KS_NL_P_VALUE]), wave(e.wave), args(e.param + KS_NL_P_ARGS), nargs(e.nargs) {}
  __device__ __forceinline__ double xs(int k) const { return V[c0 + 2 * k]; }
  __device__ __forceinline__ double ys(int k) const { return V[c0 + 2 * k + 1]; }
  // the first knot >= x (sort.SearchFloat64s)
  __device__ __forceinline__ int lower(double x) const {
    int lo = 0, hi = n;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (xs(mid) < x) lo = mid + 1; else hi = mid;
    }
    return lo;
  }
  __device__ __forceinline__ int segment(double x) const {  // :93-104
    const int k = lower(x);
    return k <= 0 ? 1 : k >= n ? n - 1 : k;
  }
  __device__ __forceinline__ void f(double x, double* y, double* dy) const {  // :107-115
    if (n == 0) { *y = lin * x; *dy = lin; return; }
    const int k = segment(x);
    const double g = (ys(k) - ys(k - 1)) / (xs(k) - xs(k - 1));
    *y = ys(k - 1) + g * (x - xs(k - 1));
    *dy = g;
  }
  __device__ __forceinline__ double cum(double x) const {  // :118-123
    const int k = segment(x);
    const double g = (ys(k) - ys(k - 1)) / (xs(k) - xs(k - 1));
    const double dx = x - xs(k - 1);
    return D[d + DN_PRE + k - 1] + ys(k - 1) * dx + 0.5 * g * dx * dx;
  }
  __device__ __forceinline__ double coenergy(double x) const {  // :126-131
    return n == 0 ? 0.5 * lin * x * x : cum(x) - D[d + DN_G0];
  }
  __device__ __forceinline__ double energy(double x) const {  // :134-137
    double y, dy;
    f(x, &y, &dy);
    return x * y - coenergy(x);
  }
  __device__ __forceinline__ double s(double t) const {
    return wave == KS_WAVE_NONE ? 1.0 : wave_value(wave, D, d + DN_A0, V, args, nargs, t);
  }
  __device__ __forceinline__ double sdot(double t) const {
    return wave == KS_WAVE_NONE ? 0.0 : wave_slope(wave, D, d + DN_A0, V, args, nargs, t);
  }
  __device__ __forceinline__ double limit(double x, double prev, bool* lim) const {  // :150-159
    *lim = false;
    const double ms = D[d + DN_MAXSTEP];
    if (ms == 0 || fabs(x - prev) <= ms) return x;
    const double lo = xs(0), hi = xs(n - 1);
    if ((x <= lo && prev <= lo) || (x >= hi && prev >= hi)) return x;
    *lim = true;
    return prev + copysign(ms, x - prev);
  }
  __device__ __forceinline__ double knot_step(double x0, double x1, double h) const {  // :171-206
    if (n == 0 || x0 == x1) return KS_INF;
    int k = lower(x0);
    double xk;
    if (x1 > x0) {
      while (k < n && xs(k) <= x0) k++;
      if (k == n || xs(k) >= x1) return KS_INF;
      xk = xs(k);
    } else {
      if (--k < 0 || xs(k) <= x1) return KS_INF;
      xk = xs(k);
    }
    double w = KS_INF;
    if (k > 0) w = xs(k) - xs(k - 1);
    if (k < n - 1) w = fmin(w, xs(k + 1) - xs(k));
    if (fabs(xk - x0) <= 1e-3 * w) return KS_INF;
    const double fr = (xk - x0) / (x1 - x0);
    if (fr > 0.9) return KS_INF;
    return fr * h;
  }
};

// The per-circuit constants of the law (newStateLaw, :47-64): the integrals of
// f from the first knot, and the Newton step limit.
__device__ inline void nl_setup(const KElem& e, const Col& V, const Col& D, double step, double stop) {
  const int d = e.derived;
  if (e.wave != KS_WAVE_NONE) wave_resolve(e.wave, V, e.param + KS_NL_P_ARGS, e.nargs, D, d + DN_A0, step, stop);
  const int c0 = e.param + KS_NL_P_ARGS + e.nargs, n = e.level / 2;
  D[d + DN_G0] = 0; D[d + DN_MAXSTEP] = 0;
  if (n < 2) return;
  D[d + DN_PRE] = 0;
  for (int k = 1; k < n; k++)
    D[d + DN_PRE + k] = D[d + DN_PRE + k - 1] + 0.5 * (V[c0 + 2 * (k - 1) + 1] + V[c0 + 2 * k + 1]) * (V[c0 + 2 * k] - V[c0 + 2 * (k - 1)]);
  const KElem& ee = e;
  NlLaw law(ee, V, D);
  D[d + DN_G0] = law.cum(0);
  D[d + DN_MAXSTEP] = 4 * (V[c0 + 2 * (n - 1)] - V[c0]) / double(n - 1);
}

// NonlinearCapacitor.Load / NonlinearInductor.Load, :318-357 and :531-566.
template <class SY>
__device__ __forceinline__ void nl_load(const KElem& e, const Col& V, const Col& Dv, const Col& S, SY& sys,
                                        const LoadParams& lp) {
  const int p = e.u[0], nn = e.u[1], k = e.u[2];
  const bool ind = e.kind == KS_ELEM_LN;
  S[SN_LIM] = 0; S[SN_T] = lp.time; S[SN_TRAN] = 0;
  if (!ind) { S[SN_G] = 0; S[SN_Y0] = 0; }
  if (ind) { sadd(sys, p, k, 1); sadd(sys, nn, k, -1); }
  if (lp.mode == ModeOP || lp.mode == ModeTranOP) {
    if (ind) { sadd(sys, k, p, 1); sadd(sys, k, nn, -1); }
    return;
  }
  if (lp.mode == ModeUICInit) {
    if (ind) { sadd(sys, k, k, 1); srhs(sys, k, S[SN_IPREV]); }
    else {
      const double g = 1e9, vp = S[SN_VPREV];  // uicConductance
      sadd(sys, p, p, g); sadd(sys, nn, nn, g); sadd(sys, p, nn, -g); sadd(sys, nn, p, -g);
      srhs(sys, p, g * vp); srhs(sys, nn, -g * vp);
    }
    return;
  }
  S[SN_TRAN] = 1;
  NlLaw law(e, V, Dv);
  bool lim;
  const double xraw = ind ? xo_(sys, k) : xo_(sys, p) - xo_(sys, nn);
  const double x = law.limit(xraw, S[SN_XITER], &lim);
  S[SN_XITER] = x; S[SN_LIM] = lim; S[SN_X0] = x;
  const double sn = law.s(lp.time);
  S[SN_SN] = sn; S[SN_SDOT] = law.sdot(lp.time);
  double a, b;
  if (lp.method == TRAP) { a = 2 / lp.h; b = -2 * S[SN_QPREV] / lp.h - (ind ? S[SN_VPREV] : S[SN_IPREV]); }
  else { a = 1 / lp.h; b = -S[SN_QPREV] / lp.h; }
  S[SN_A] = a; S[SN_B] = b;
  double y, dy;
  law.f(x, &y, &dy);
  if (ind) {
    const double lam0 = sn * y, ld = sn * dy;
    S[SN_Y0] = lam0; S[SN_G] = ld;
    // V(n+) - V(n-) - a ld i = a (lam0 - ld i0) + b
    sadd(sys, k, p, 1); sadd(sys, k, nn, -1); sadd(sys, k, k, -a * ld);
    srhs(sys, k, a * (lam0 - ld * x) + b);
  } else {
    const double iq = a * sn * y + b, g = a * sn * dy;
    S[SN_Y0] = iq; S[SN_G] = g;
    sadd(sys, p, p, g); sadd(sys, nn, nn, g); sadd(sys, p, nn, -g); sadd(sys, nn, p, -g);
    const double ieq = iq - g * x;
    srhs(sys, p, -ieq); srhs(sys, nn, ieq);
  }
}

// The element's current at the new iterate (the capacitor's linearized
// companion current, the inductor's branch current).
template <class SY>
__device__ __forceinline__ double nl_current(const KElem& e, const Col& S, SY& sys) {
  if (e.kind == KS_ELEM_LN) return xn_(sys, e.u[2]);
  if (S[SN_TRAN] == 0) return 0.0;
  return S[SN_Y0] + S[SN_G] * (xn_(sys, e.u[0]) - xn_(sys, e.u[1]) - S[SN_X0]);
}

// ConvTest of the curved elements, :458-468 and :672-682 (the inductor's
// absolute tolerance is vntol's 1e-6).
template <class SY>
__device__ __forceinline__ bool nl_conv(const KElem& e, const Col& V, const Col& Dv, const Col& S, SY& sys,
                                        double reltol, double abstol) {
  if (S[SN_TRAN] == 0 || e.level == 0) return true;
  NlLaw law(e, V, Dv);
  const double a = S[SN_A], b = S[SN_B], sn = S[SN_SN];
  double y, dy;
  if (e.kind == KS_ELEM_LN) {
    const double i = xn_(sys, e.u[2]);
    const double vhat = a * (S[SN_Y0] + S[SN_G] * (i - S[SN_X0])) + b;
    law.f(i, &y, &dy);
    const double v = a * sn * y + b;
    return fabs(vhat - v) <= reltol * fmax(fabs(v), fabs(vhat)) + 1e-6;
  }
  const double v = xn_(sys, e.u[0]) - xn_(sys, e.u[1]);
  const double ihat = S[SN_Y0] + S[SN_G] * (v - S[SN_X0]);
  law.f(v, &y, &dy);
  const double i = a * sn * y + b;
  return fabs(ihat - i) <= reltol * fmax(fabs(i), fabs(ihat)) + abstol;
}

// Accept, :379-399 and :585-602.
template <class SY>
__device__ __forceinline__ void nl_accept(const KElem& e, const Col& V, const Col& Dv, const Col& S, SY& sys,
                                          double t, int mode) {
  const bool ind = e.kind == KS_ELEM_LN;
  double v = xn_(sys, e.u[0]) - xn_(sys, e.u[1]);
  double x;
  if (ind) {
    double i = xn_(sys, e.u[2]);
    if (mode == ModeUICInit) { i = S[SN_IPREV]; v = 0; hist_reset(S, SN_HIST); }
    else if (mode == ModeOP || mode == ModeTranOP) { v = 0; hist_reset(S, SN_HIST); }
    S[SN_IPREV] = i; S[SN_VPREV] = v;
    x = i;
  } else {
    if (mode == ModeUICInit) { v = S[SN_VPREV]; S[SN_IPREV] = 0; hist_reset(S, SN_HIST); }
    else if (mode == ModeOP || mode == ModeTranOP) { S[SN_IPREV] = 0; hist_reset(S, SN_HIST); }
    else S[SN_IPREV] = S[SN_Y0] + S[SN_G] * (v - S[SN_X0]);
    S[SN_VPREV] = v;
    x = v;
  }
  S[SN_XITER] = x; S[SN_XACC] = x;
  NlLaw law(e, V, Dv);
  const double sa = law.s(t);
  S[SN_SACC] = sa;
  double y, dy;
  law.f(x, &y, &dy);
  S[SN_QPREV] = sa * y;
  hist_push(S, SN_HIST, t, S[SN_QPREV]);
  if (S[SN_KNOTT] != 0 && t >= S[SN_KNOTT]) S[SN_KNOTT] = 0;  // stateLaw.accepted, :222-226
}

// Truncate, :417-424 and :620-625: the LTE step of the charge (flux) history and
// the landing of a crossed knot on a time point (registered as a breakpoint).
template <class SY>
__device__ __forceinline__ double nl_truncate(const KElem& e, const Col& V, const Col& Dv, const Col& S, SY& sys,
                                              const TruncParams& tc) {
  NlLaw law(e, V, Dv);
  const bool ind = e.kind == KS_ELEM_LN;
  const double v = xn_(sys, e.u[0]) - xn_(sys, e.u[1]);
  const double i = nl_current(e, S, sys);
  const double x = ind ? i : v;
  double y, dy;
  law.f(x, &y, &dy);
  const double h = ind ? lte_step(S, SN_HIST, law.s(tc.time) * y, v, S[SN_VPREV], tc.vntol, tc)
                       : lte_step(S, SN_HIST, law.s(tc.time) * y, i, S[SN_IPREV], tc.abstol, tc);
  const double p = law.knot_step(S[SN_XACC], x, tc.h);
  if (p < KS_INF) S[SN_KNOTT] = tc.time - tc.h + p;
  return fmin(h, p);
}

}  // namespace ksg
