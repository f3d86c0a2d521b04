// ks_solve.cuh — per-thread element program, dense LU and Newton bookkeeping shared by
// the operating-point and transient kernels of the GB300 engine.
#pragma once
#include "ks_devices.cuh"
#include "ks_mos.cuh"

namespace ksg {

enum { SOLVE_OK = 0, SOLVE_SINGULAR = KS_STATUS_SINGULAR, SOLVE_NONFINITE = KS_STATUS_NONFINITE, SOLVE_FP32_FAIL = 99 };

// Per-thread views into the block's shared memory (stride T between entries).
template <int T>
struct ThreadSys {
  double* A;     // n*n   stamped matrix (FP64)
  double* rhs;   // n
  double* x;     // n     new iterate
  double* xold;  // n     linearization point
  double* col;   // n     column maxima
  int* piv;      // n
  float* L32;    // n*n   FP32 factor (mixed precision only)
  int n;
  __device__ __forceinline__ double& a(int i, int j) const { return A[(i * n + j) * T]; }
  __device__ __forceinline__ float& l(int i, int j) const { return L32[(i * n + j) * T]; }
};

// Stamp every element at xold (analysis/op.go:289-322 without the solve).
template <int T>
__device__ inline void load_all(const KElem* el, int n_elem, const Col& Vb, const Col& Db, const Col& Sb,
                                const ThreadSys<T>& s, const LoadParams& lp) {
  int n = s.n;
  for (int i = 0; i < n * n; i++) s.A[i * T] = 0.0;
  for (int i = 0; i < n; i++) s.rhs[i * T] = 0.0;
  SysRef<T> sys{s.A, s.rhs, s.xold, n};
  for (int k = 0; k < n_elem; k++) {
    const KElem& e = el[k];
    Col S{Sb.p + (int64_t)e.state * Sb.B, Sb.B};
    switch (e.kind) {
      case KS_ELEM_R: {  // device/passive.go:72-84
        double g = Db[e.derived + DR_G];
        int a = e.u[0], b = e.u[1];
        sys.add(a, a, g); sys.add(b, b, g); sys.add(a, b, -g); sys.add(b, a, -g);
        break;
      }
      case KS_ELEM_C: {  // device/reactive.go:60-106
        int a = e.u[0], b = e.u[1];
        if (lp.mode == ModeOP || lp.mode == ModeTranOP) { S[SC_TRAN] = 0; S[SC_GEQ] = 0; S[SC_IHIST] = 0; break; }
        if (lp.mode == ModeUICInit) {
          double g = 1e9, vp = S[SC_VPREV];
          sys.add(a, a, g); sys.add(b, b, g); sys.add(a, b, -g); sys.add(b, a, -g);
          sys.addRHS(a, g * vp); sys.addRHS(b, -g * vp);
          S[SC_TRAN] = 0; S[SC_GEQ] = 0; S[SC_IHIST] = 0;
          break;
        }
        double C = Vb[e.param + KS_RCL_P_VALUE], geq, ih;
        if (lp.method == TRAP) { geq = 2 * C / lp.h; ih = -(geq * S[SC_VPREV] + S[SC_IPREV]); }
        else { geq = C / lp.h; ih = -geq * S[SC_VPREV]; }
        S[SC_TRAN] = 1; S[SC_GEQ] = geq; S[SC_IHIST] = ih;
        sys.add(a, a, geq); sys.add(b, b, geq); sys.add(a, b, -geq); sys.add(b, a, -geq);
        sys.addRHS(a, -ih); sys.addRHS(b, ih);
        break;
      }
      case KS_ELEM_L: {  // device/reactive.go:230-259
        int a = e.u[0], b = e.u[1], kk = e.u[2];
        sys.add(a, kk, 1); sys.add(b, kk, -1);
        if (lp.mode == ModeOP || lp.mode == ModeTranOP) { sys.add(kk, a, 1); sys.add(kk, b, -1); break; }
        if (lp.mode == ModeUICInit) { sys.add(kk, kk, 1); sys.addRHS(kk, S[SL_IPREV]); break; }
        double L = Vb[e.param + KS_RCL_P_VALUE];
        double req = L / lp.h, r = -req * S[SL_IPREV];
        if (lp.method == TRAP) { req = 2 * L / lp.h; r = -req * S[SL_IPREV] - S[SL_VPREV]; }
        sys.add(kk, a, 1); sys.add(kk, b, -1); sys.add(kk, kk, -req);
        sys.addRHS(kk, r);
        break;
      }
      case KS_ELEM_V: {  // device/source.go:102-112
        Col D{Db.p, Db.B};
        double v = source_at(e, Vb, D, S, lp);
        S[SV_VALUE] = v;
        int a = e.u[0], b = e.u[1], kk = e.u[2];
        sys.add(a, kk, 1); sys.add(b, kk, -1); sys.add(kk, a, 1); sys.add(kk, b, -1);
        sys.addRHS(kk, v);
        break;
      }
      case KS_ELEM_I: {  // device/source.go:155-160
        double v = source_at(e, Vb, Db, S, lp);
        S[SV_VALUE] = v;
        sys.addRHS(e.u[0], -v); sys.addRHS(e.u[1], v);
        break;
      }
      case KS_ELEM_D: diode_load<T>(e, Vb, Db, S, sys, lp); break;
      case KS_ELEM_Q: bjt_load<T>(e, Vb, Db, S, sys, lp); break;
      case KS_ELEM_M: mos_load<T>(e, Vb, Db, S, sys, lp); break;
    }
  }
}

// Dense LU with partial pivoting in FP64, solver/dense.go:80-177; A is factored in place.
template <int T>
__device__ inline int lu_solve_fp64(const ThreadSys<T>& s, const double* b, double* out) {
  int n = s.n;
  double scale = 0;
  for (int i = 0; i < n * n; i++) {
    double v = s.A[i * T];
    if (!isfinite(v)) return SOLVE_NONFINITE;
    scale = fmax(scale, fabs(v));
  }
  if (scale == 0) return SOLVE_SINGULAR;
  for (int j = 0; j < n; j++) {
    double m = 0;
    for (int i = 0; i < n; i++) m = fmax(m, fabs(s.a(i, j)));
    s.col[j * T] = m;
  }
  for (int k = 0; k < n; k++) {
    int p = k;
    double maxv = fabs(s.a(k, k));
    for (int i = k + 1; i < n; i++) {
      double v = fabs(s.a(i, k));
      if (v > maxv) { maxv = v; p = i; }
    }
    if (maxv <= s.col[k * T] * double(n) * 1e-14) return SOLVE_SINGULAR;
    s.piv[k * T] = p;
    if (p != k)
      for (int j = 0; j < n; j++) { double t = s.a(k, j); s.a(k, j) = s.a(p, j); s.a(p, j) = t; }
    double pivot = s.a(k, k);
    for (int i = k + 1; i < n; i++) {
      double f = s.a(i, k) / pivot;
      s.a(i, k) = f;
      if (f == 0) continue;
      for (int j = k + 1; j < n; j++) s.a(i, j) -= f * s.a(k, j);
    }
  }
  // y = P b in `out`, then forward (unit lower) and back substitution.
  for (int i = 0; i < n; i++) out[i * T] = b[i * T];
  for (int k = 0; k < n; k++) {
    int p = s.piv[k * T];
    if (p != k) { double t = out[k * T]; out[k * T] = out[p * T]; out[p * T] = t; }
  }
  for (int i = 0; i < n; i++) {
    double acc = out[i * T];
    for (int j = 0; j < i; j++) acc -= s.a(i, j) * out[j * T];
    out[i * T] = acc;
  }
  for (int i = n - 1; i >= 0; i--) {
    double acc = out[i * T];
    for (int j = i + 1; j < n; j++) acc -= s.a(i, j) * out[j * T];
    out[i * T] = acc / s.a(i, i);
  }
  for (int i = 0; i < n; i++) if (!isfinite(out[i * T])) return SOLVE_NONFINITE;
  return SOLVE_OK;
}

// FP32 forward/back substitution with the factor in L32: y (FP64 in/out, in place).
template <int T>
__device__ inline void lu32_apply(const ThreadSys<T>& s, double* y) {
  const int n = s.n;
  for (int k = 0; k < n; k++) {
    int p = s.piv[k * T];
    if (p != k) { double t = y[k * T]; y[k * T] = y[p * T]; y[p * T] = t; }
  }
  for (int i = 0; i < n; i++) {
    float acc = (float)y[i * T];
    for (int j = 0; j < i; j++) acc = fmaf(-s.l(i, j), (float)y[j * T], acc);
    y[i * T] = acc;
  }
  for (int i = n - 1; i >= 0; i--) {
    float acc = (float)y[i * T];
    for (int j = i + 1; j < n; j++) acc = fmaf(-s.l(i, j), (float)y[j * T], acc);
    y[i * T] = acc / s.l(i, i);
  }
}

// Mixed precision: FP32 LU with partial pivoting of the FP64 matrix, then
// x = xold + LU32^-1 (rhs - A*xold) and iterative refinement with the FP64
// residual rhs - A*x until the correction is at FP64 round-off (at most 6
// passes).  A and rhs are left intact.  Returns SOLVE_FP32_FAIL when a pivot is
// below the FP32 threshold or refinement does not contract (the caller then
// solves in FP64).
template <int T>
__device__ inline int lu_solve_mixed(const ThreadSys<T>& s) {
  const int n = s.n;
  double scale = 0;
  for (int i = 0; i < n * n; i++) {
    double v = s.A[i * T];
    if (!isfinite(v)) return SOLVE_NONFINITE;
    scale = fmax(scale, fabs(v));
  }
  if (scale == 0) return SOLVE_SINGULAR;
  for (int j = 0; j < n; j++) {
    double m = 0;
    for (int i = 0; i < n; i++) m = fmax(m, fabs(s.a(i, j)));
    s.col[j * T] = m;
  }
  for (int i = 0; i < n * n; i++) s.L32[i * T] = (float)s.A[i * T];
  for (int k = 0; k < n; k++) {
    int p = k;
    float maxv = fabsf(s.l(k, k));
    for (int i = k + 1; i < n; i++) {
      float v = fabsf(s.l(i, k));
      if (v > maxv) { maxv = v; p = i; }
    }
    if ((double)maxv <= s.col[k * T] * double(n) * 1e-6) return SOLVE_FP32_FAIL;
    s.piv[k * T] = p;
    if (p != k)
      for (int j = 0; j < n; j++) { float t = s.l(k, j); s.l(k, j) = s.l(p, j); s.l(p, j) = t; }
    float rp = 1.0f / s.l(k, k);
    for (int i = k + 1; i < n; i++) {
      float f = s.l(i, k) * rp;
      s.l(i, k) = f;
      if (f == 0.0f) continue;
      for (int j = k + 1; j < n; j++) s.l(i, j) = fmaf(-f, s.l(k, j), s.l(i, j));
    }
  }
  // x starts at the linearization point; each pass adds LU32^-1 of the FP64 residual.
  for (int i = 0; i < n; i++) s.x[i * T] = s.xold[i * T];
  double prev = CUDART_INF;
  for (int pass = 0; pass < 6; pass++) {
    for (int i = 0; i < n; i++) {  // residual in col (the column maxima are no longer needed)
      double r = s.rhs[i * T];
      for (int j = 0; j < n; j++) r -= s.a(i, j) * s.x[j * T];
      s.col[i * T] = r;
    }
    lu32_apply<T>(s, s.col);
    double dmax = 0, xmax = 0;
    for (int i = 0; i < n; i++) {
      double v = s.x[i * T] + s.col[i * T];
      if (!isfinite(v)) return SOLVE_NONFINITE;
      s.x[i * T] = v;
      dmax = fmax(dmax, fabs(s.col[i * T]));
      xmax = fmax(xmax, fabs(v));
    }
    if (dmax <= 4e-16 * xmax || dmax == 0) break;
    if (pass > 0 && dmax > 0.5 * prev) {  // refinement stopped contracting
      if (dmax <= 1e-11 * xmax) break;      // at the round-off floor of this system
      return SOLVE_FP32_FAIL;
    }
    prev = dmax;
  }
  return SOLVE_OK;
}

// converged, analysis/newton.go:59-82.
template <int T>
__device__ inline bool converged(const KElem* el, int n_elem, const int8_t* isv, const Col& Vb, const Col& Db,
                                 const Col& Sb, const ThreadSys<T>& s, const KOpts& o, double gmin) {
  for (int k = 0; k < n_elem; k++) {
    const KElem& e = el[k];
    int lim = e.kind == KS_ELEM_D ? SD_LIM : e.kind == KS_ELEM_Q ? SQ_LIM : e.kind == KS_ELEM_M ? SM_LIM : -1;
    if (lim >= 0 && Sb.p[(int64_t)(e.state + lim) * Sb.B] != 0) return false;
  }
  for (int i = 0; i < s.n; i++) {
    double x = s.x[i * T], old = s.xold[i * T];
    double tol = (isv[i] ? o.vntol : o.abstol) + o.reltol * fmax(fabs(x), fabs(old));
    if (fabs(x - old) > tol) return false;
  }
  for (int k = 0; k < n_elem; k++) {
    const KElem& e = el[k];
    Col S{Sb.p + (int64_t)e.state * Sb.B, Sb.B};
    if (e.kind == KS_ELEM_D) { if (!diode_conv<T>(e, Vb, Db, S, s.x, o.reltol, o.abstol, gmin)) return false; }
    else if (e.kind == KS_ELEM_Q) { if (!bjt_conv<T>(e, Vb, Db, S, s.x, o.reltol, o.abstol, gmin)) return false; }
    else if (e.kind == KS_ELEM_M) { if (!mos_conv<T>(e, Vb, Db, S, s.x, o.reltol, o.abstol, gmin)) return false; }
  }
  return true;
}

// Accept every element at x (analysis/op.go:324-328).
template <int T>
__device__ inline void accept_all(const KElem* el, int n_elem, const Col& Vb, const Col& Db, const Col& Sb,
                                  const double* x, double t, int mode, double gmin, bool nonlinOnly) {
  for (int k = 0; k < n_elem; k++) {
    const KElem& e = el[k];
    Col S{Sb.p + (int64_t)e.state * Sb.B, Sb.B};
    switch (e.kind) {
      case KS_ELEM_C: {  // device/reactive.go:144-161
        if (nonlinOnly) break;
        double v = xat(x, e.u[0], T) - xat(x, e.u[1], T);
        if (mode == ModeUICInit) { S[SC_IPREV] = 0; hist_reset(S, SC_HIST); }
        else if (mode == ModeOP || mode == ModeTranOP) { S[SC_VPREV] = v; S[SC_IPREV] = 0; hist_reset(S, SC_HIST); }
        else { double i = S[SC_TRAN] != 0 ? S[SC_GEQ] * v + S[SC_IHIST] : 0.0; S[SC_VPREV] = v; S[SC_IPREV] = i; }
        hist_push(S, SC_HIST, t, Vb[e.param] * S[SC_VPREV]);
        break;
      }
      case KS_ELEM_L: {  // device/reactive.go:312-329
        if (nonlinOnly) break;
        double v = xat(x, e.u[0], T) - xat(x, e.u[1], T), i = x[e.u[2] * T];
        if (mode == ModeUICInit) { S[SL_VPREV] = 0; hist_reset(S, SL_HIST); }
        else if (mode == ModeOP || mode == ModeTranOP) { S[SL_VPREV] = 0; S[SL_IPREV] = i; hist_reset(S, SL_HIST); }
        else { S[SL_VPREV] = v; S[SL_IPREV] = i; }
        hist_push(S, SL_HIST, t, Vb[e.param] * S[SL_IPREV]);
        break;
      }
      case KS_ELEM_D: diode_accept<T>(e, Vb, Db, S, x, t, mode); break;
      case KS_ELEM_Q: bjt_accept<T>(e, Vb, Db, S, x, t, mode, gmin); break;
      case KS_ELEM_M: mos_accept<T>(e, Vb, Db, S, x, t, mode); break;
    }
  }
}

// Fresh device state of one circuit (the zero state of newly built devices, with
// each MOSFET's limiting threshold at VTO, device/mosfet.go:321).
__device__ inline void init_state(const KElem* el, int n_elem, int n_state, const Col& Db, const Col& Sb) {
  for (int k = 0; k < n_state; k++) Sb[k] = 0.0;
  for (int k = 0; k < n_elem; k++)
    if (el[k].kind == KS_ELEM_M) Sb[el[k].state + SM_AVON] = Db[el[k].derived + DM_VTO];
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

}  // namespace ksg
