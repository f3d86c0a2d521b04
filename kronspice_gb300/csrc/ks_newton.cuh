// ks_newton.cuh — per-thread Newton and DC-solve state machine of the GB300 engine,
// shared by the operating-point and transient kernels.
//
// One pass of the kernels' loop is one (*Sim).solve (analysis/op.go:289-322); the
// scalar control code here decides what the next solve is, restating
//   (*Sim).newton / converged   analysis/newton.go:36-82
//   (*Sim).dcSolve + fallbacks   analysis/newton.go:95-311 (gmin stepping, source
//                                stepping, pseudo-transient continuation)
// with every loop bounded by the reference's own limits.
#pragma once
#include "ks_solve.cuh"

namespace ksg {

enum Phase { PH_MAIN = 0, PH_GMIN, PH_SRC_INIT, PH_SRC, PH_PT, PH_PT_FINAL, PH_DONE };

struct OpState {
  int phase, it, maxIter, total, firstErr, status, nsteps, quiet;
  bool initJct, ok, srcStepping, fp64;
  double diagGmin, g, factor, srcFact, done, step, ptG, h;
};

__device__ __forceinline__ bool retryable(int e) {  // analysis/newton.go:86-89
  return e == KS_STATUS_NO_CONVERGENCE || e == KS_STATUS_NONFINITE || e == KS_STATUS_SINGULAR;
}

// Everything one thread needs: its shared-memory system, its SoA columns, the
// element program and the options.
template <int T>
struct Thr {
  ThreadSys<T> s;
  const KElem* el;
  const int8_t* isv;
  int ne, n, n_nodes, n_state;
  bool nonlinEmpty;
  Col V, D, Sb;
  Col save, ptPrev, xacc;  // work columns (n each)
  KOpts o;
};

// Shared-memory layout of a block: element table, is_voltage flags, then the
// per-thread arrays with stride T.  Returns the per-thread views.
template <int T>
__device__ inline void thr_init(Thr<T>& t, const KPlan& plan, const KOpts& o, unsigned char* smem, const double* values,
                                const double* derived, double* state, double* work, int64_t B, int64_t c) {
  const int n = plan.n, ne = plan.n_elem;
  KElem* el = reinterpret_cast<KElem*>(smem);
  for (int i = threadIdx.x; i < ne * (int)(sizeof(KElem) / 4); i += T)
    reinterpret_cast<int32_t*>(el)[i] = reinterpret_cast<const int32_t*>(plan.elem)[i];
  int8_t* isv = reinterpret_cast<int8_t*>(smem + ne * sizeof(KElem));
  for (int i = threadIdx.x; i < n; i += T) isv[i] = plan.is_v[i];
  size_t off = ne * sizeof(KElem) + ((n + 15) / 16) * 16;
  double* base = reinterpret_cast<double*>(smem + off);
  const int tid = threadIdx.x;
  t.s.n = n;
  t.s.A = base + tid;
  t.s.rhs = base + (size_t)n * n * T + tid;
  t.s.x = t.s.rhs + (size_t)n * T;
  t.s.xold = t.s.x + (size_t)n * T;
  t.s.col = t.s.xold + (size_t)n * T;
  t.s.piv = reinterpret_cast<int*>(base + (size_t)(n * n + 4 * n) * T) + tid;
  t.s.L32 = reinterpret_cast<float*>(base + (size_t)(n * n + 4 * n) * T + ((size_t)n * T + 1) / 2) + tid;
  t.el = el; t.isv = isv; t.ne = ne; t.n = n; t.n_nodes = plan.n_nodes; t.n_state = plan.n_state;
  t.nonlinEmpty = plan.n_nonlin == 0;
  t.V = Col{const_cast<double*>(values) + c, B};
  t.D = Col{const_cast<double*>(derived) + c, B};
  t.Sb = Col{state + c, B};
  t.save = Col{work + c, B};
  t.ptPrev = Col{work + (int64_t)n * B + c, B};
  t.xacc = Col{work + (int64_t)2 * n * B + c, B};
  t.o = o;
}

// Point a thread's SoA columns at circuit c (persistent kernels move a thread
// from circuit to circuit).
template <int T>
__device__ inline void thr_bind(Thr<T>& t, const double* values, const double* derived, double* state, double* work,
                                int64_t B, int64_t c) {
  const int n = t.n;
  t.V = Col{const_cast<double*>(values) + c, B};
  t.D = Col{const_cast<double*>(derived) + c, B};
  t.Sb = Col{state + c, B};
  t.save = Col{work + c, B};
  t.ptPrev = Col{work + (int64_t)n * B + c, B};
  t.xacc = Col{work + (int64_t)2 * n * B + c, B};
}

// Bytes of dynamic shared memory thr_init lays out.
inline size_t thr_smem(int n, int ne, int T) {
  size_t off = (size_t)ne * sizeof(KElem) + ((n + 15) / 16) * 16;
  size_t per = (size_t)(n * n + 4 * n) * 8 + (size_t)n * 4 + 8 + (size_t)n * n * 4 + 8;
  return off + per * T;
}

template <int T>
__device__ inline void op_state_reset(OpState& st, const KOpts& o) {
  st.phase = PH_MAIN; st.it = 0; st.maxIter = o.itl1; st.total = 0; st.firstErr = 0; st.status = KS_STATUS_NOT_RUN;
  st.nsteps = 0; st.quiet = 0; st.ok = false; st.srcStepping = false; st.fp64 = !o.mixed; st.initJct = true;
  st.diagGmin = 0; st.g = 0; st.factor = 0; st.srcFact = 0; st.done = 0; st.step = 0; st.ptG = 0; st.h = 0;
}

// One (*Sim).solve: stamp at x (copied to xold), add the gmin-stepping and
// pseudo-transient diagonals, solve.  Returns 0 or the solver error.
template <int T>
__device__ inline int solve_once(Thr<T>& t, OpState& st, LoadParams lp) {
  ThreadSys<T>& s = t.s;
  const int n = t.n;
  for (int i = 0; i < n; i++) s.xold[i * T] = s.x[i * T];
  lp.initJct = st.initJct;
  lp.gmin = t.o.gmin;
  lp.srcStepping = st.srcStepping;
  lp.srcFact = st.srcFact;
  load_all<T>(t.el, t.ne, t.V, t.D, t.Sb, s, lp);
  if (st.ptG > 0) {
    for (int i = 0; i < n; i++) {
      double pv = t.ptPrev[i];
      if (t.isv[i]) { s.a(i, i) += st.ptG; s.rhs[i * T] += st.ptG * pv; }
      else { s.a(i, i) -= st.ptG; s.rhs[i * T] -= st.ptG * pv; }
    }
  }
  if (st.diagGmin > 0) for (int i = 0; i < n; i++) if (t.isv[i]) s.a(i, i) += st.diagGmin;
  int err;
  if (!st.fp64) {
    err = lu_solve_mixed<T>(s);
    if (err == SOLVE_FP32_FAIL) {  // the FP64 path takes over this circuit
      st.fp64 = true;
      err = lu_solve_fp64<T>(s, s.rhs, s.x);
    }
  } else {
    err = lu_solve_fp64<T>(s, s.rhs, s.x);
  }
  st.total++;
  return err;
}

// One Newton iteration: a solve plus the bookkeeping of analysis/newton.go:36-57.
// Returns -1 while the current newton() call goes on, else its result.
template <int T>
__device__ inline int newton_step(Thr<T>& t, OpState& st, const LoadParams& lp) {
  int err = solve_once<T>(t, st, lp);
  int res = -1;
  if (err) res = err;
  else if (t.nonlinEmpty) res = KS_STATUS_OK;
  else if (st.initJct) st.initJct = false;
  else if (converged<T>(t.el, t.ne, t.isv, t.V, t.D, t.Sb, t.s, t.o, t.o.gmin)) res = KS_STATUS_OK;
  if (res < 0) {
    st.it++;
    if (st.it < st.maxIter) return -1;
    res = KS_STATUS_NO_CONVERGENCE;
  }
  st.it = 0;
  return res;
}

// dcSolve start, analysis/newton.go:96-102, with applyNodeSet (:221-243) when x0
// holds a starting point (node voltages; other unknowns start at 0).
template <int T>
__device__ inline void dc_start(Thr<T>& t, OpState& st, const double* x0, int64_t c, int mode) {
  op_state_reset<T>(st, t.o);
  for (int i = 0; i < t.n; i++) t.s.x[i * T] = 0.0;
  if (x0) {
    for (int i = 0; i < t.n_nodes - 1; i++) t.s.x[i * T] = x0[c * t.n + i];
    accept_all<T>(t.el, t.ne, t.V, t.D, t.Sb, t.s.x, 0.0, ModeOP, t.o.gmin, true);
    st.initJct = false;
  }
  (void)mode;
}

// Advance dcSolve with the result of a finished newton() call.  Sets st.phase to
// PH_DONE and st.status when the DC solve is over.
template <int T>
__device__ inline void dc_advance(Thr<T>& t, OpState& st, int res) {
  const KOpts& o = t.o;
  ThreadSys<T>& s = t.s;
  const int n = t.n;
  bool advance = true;
  while (advance) {
    advance = false;
    switch (st.phase) {
      case PH_MAIN:
        if (res == KS_STATUS_OK || t.nonlinEmpty || !retryable(res)) { st.status = res; st.phase = PH_DONE; break; }
        st.firstErr = res;
        st.phase = PH_GMIN;
        if (!o.no_gmin) {  // gminStepping start, :134-142
          for (int i = 0; i < n; i++) { s.x[i * T] = 0.0; t.save[i] = 0.0; }
          st.initJct = true; st.g = 1e-2; st.factor = 10.0; st.ok = false; st.nsteps = 0;
          st.diagGmin = st.g;
        } else { st.nsteps = -1; res = KS_STATUS_NO_CONVERGENCE; advance = true; }
        break;
      case PH_GMIN: {  // :143-175
        bool fail = false;
        if (st.nsteps < 0) fail = true;
        else if (res == KS_STATUS_OK) {
          for (int i = 0; i < n; i++) t.save[i] = s.x[i * T];
          if (st.g == 0) { st.diagGmin = 0; st.status = KS_STATUS_OK; st.phase = PH_DONE; break; }
          st.ok = true;
          st.factor = fmin(st.factor * sqrt(st.factor), 10.0);
          st.g = st.g / st.factor < o.gmin ? 0.0 : st.g / st.factor;
          if (++st.nsteps >= 200) fail = true;
        } else if (!retryable(res) || !st.ok) {
          fail = true;
        } else {
          for (int i = 0; i < n; i++) s.x[i * T] = t.save[i];
          double prev = st.g == 0 ? o.gmin : st.g * st.factor;
          st.factor = sqrt(st.factor);
          if (st.factor < 1.00005) fail = true;
          else { st.g = prev / st.factor; if (++st.nsteps >= 200) fail = true; }
        }
        st.diagGmin = st.g;
        if (fail) {
          st.diagGmin = 0;
          if (!o.no_source) {  // sourceStepping start, :180-192
            st.phase = PH_SRC_INIT;
            for (int i = 0; i < n; i++) { s.x[i * T] = 0.0; t.save[i] = 0.0; }
            st.srcStepping = true; st.done = 0; st.step = 0.1; st.srcFact = 0; st.nsteps = 0;
          } else { st.phase = PH_SRC; st.nsteps = -1; res = KS_STATUS_NO_CONVERGENCE; advance = true; }
        }
        break;
      }
      case PH_SRC_INIT:
        if (res != KS_STATUS_OK) { st.phase = PH_SRC; st.nsteps = -1; advance = true; break; }
        for (int i = 0; i < n; i++) t.save[i] = s.x[i * T];
        st.phase = PH_SRC;
        st.srcFact = fmin(st.done + st.step, 1.0);
        break;
      case PH_SRC: {  // :193-213
        bool fail = false;
        if (st.nsteps < 0) fail = true;
        else if (res == KS_STATUS_OK) {
          if (st.srcFact == 1) { st.srcStepping = false; st.srcFact = 0; st.status = KS_STATUS_OK; st.phase = PH_DONE; break; }
          for (int i = 0; i < n; i++) t.save[i] = s.x[i * T];
          st.done = st.srcFact; st.step = fmin(st.step * 1.5, 0.5);
          if (++st.nsteps >= 1000) fail = true;
        } else if (!retryable(res)) fail = true;
        else {
          for (int i = 0; i < n; i++) s.x[i * T] = t.save[i];
          st.step /= 2;
          if (st.step < 1e-3) fail = true;
          else if (++st.nsteps >= 1000) fail = true;
        }
        if (fail) {
          st.srcStepping = false; st.srcFact = 0;
          if (!o.no_pt) {  // pseudoTransient start, :260-273
            st.phase = PH_PT;
            for (int i = 0; i < n; i++) { s.x[i * T] = 0.0; t.ptPrev[i] = 0.0; }
            st.initJct = true; st.h = 1e-6; st.quiet = 0; st.nsteps = 0; st.ptG = 1 / st.h;
          } else { st.status = st.firstErr; st.phase = PH_DONE; }
        } else st.srcFact = fmin(st.done + st.step, 1.0);
        break;
      }
      case PH_PT: {  // :272-310
        bool fail = false;
        if (res != KS_STATUS_OK) {
          if (!retryable(res)) fail = true;
          else {
            for (int i = 0; i < n; i++) s.x[i * T] = t.ptPrev[i];
            st.h /= 4;
            if (st.h < 1e-15) fail = true;
          }
        } else {
          bool moved = false;
          for (int i = 0; i < n; i++) {
            double xv = s.x[i * T];
            double tol = t.isv[i] ? o.vntol : o.abstol;
            if (fabs(xv - t.ptPrev[i]) > o.reltol * fabs(xv) + tol) { moved = true; break; }
          }
          for (int i = 0; i < n; i++) t.ptPrev[i] = s.x[i * T];
          st.quiet = moved ? 0 : st.quiet + 1;
          if (st.quiet >= 3 && st.h >= 1e6) { st.ptG = 0; st.phase = PH_PT_FINAL; break; }
          st.h = fmin(st.h * 2, 1e12);
        }
        if (!fail && ++st.nsteps >= 2000) fail = true;
        if (fail) { st.ptG = 0; st.status = st.firstErr; st.phase = PH_DONE; }
        else st.ptG = 1 / st.h;
        break;
      }
      case PH_PT_FINAL:
        st.status = res == KS_STATUS_OK ? KS_STATUS_OK : st.firstErr;
        st.phase = PH_DONE;
        break;
      default: break;
    }
  }
}

}  // namespace ksg
