// ks_newton.cuh — per-thread Newton and DC-solve state machine of the GB300 engine,
// shared by the operating-point and transient kernels (generic and per-topology).
//
// One pass of the kernels' loop is one (*Sim).solve (analysis/op.go:289-322); the
// scalar control code here decides what the next solve is, restating
//   (*Sim).newton / converged   analysis/newton.go:36-82
//   (*Sim).dcSolve + fallbacks   analysis/newton.go:95-311 (gmin stepping, source
//                                stepping, pseudo-transient continuation)
// with every loop bounded by the reference's own limits.
#pragma once
#include "ks_start32.cuh"

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

// Everything one thread needs: its system, the element program, its SoA columns
// and the options.
template <class SY, class P>
struct Thr {
  SY s;
  P prog;
  Col V, D, Sb;
  Col save, ptPrev, xacc;  // work columns (n each)
  KOpts o;
  __device__ __forceinline__ int n() const { return s.size(); }
};

// Point a thread's SoA columns at circuit c (persistent kernels move a thread
// from circuit to circuit).
template <class SY, class P>
__device__ __forceinline__ void thr_bind(Thr<SY, P>& t, const double* values, const double* derived, double* state, double* work,
                                int64_t B, int64_t c) {
  if constexpr (P::kWarp) {  // per-circuit layout of the multi-topology kernels
    t.prog.bind(t, c);
    return;
  }
  const int n = t.n();
  t.V = Col{const_cast<double*>(values) + c, B};
  t.D = Col{const_cast<double*>(derived) + c, B};
  t.Sb = Col{state + c, B};
  t.save = Col{work + c, B};
  t.ptPrev = Col{work + (int64_t)n * B + c, B};
  t.xacc = Col{work + (int64_t)2 * n * B + c, B};
}

// Generic kernels: element table and is_voltage flags copied to shared memory,
// then each thread's system in shared memory with stride T.
template <int T>
__device__ inline void smem_layout(Thr<SmemSys<T>, RtProg>& t, const KPlan& plan, unsigned char* smem) {
  const int n = plan.n, ne = plan.n_elem;
  KElem* el = reinterpret_cast<KElem*>(smem);
  for (int i = threadIdx.x; i < ne * (int)(sizeof(KElem) / 4); i += T)
    reinterpret_cast<int32_t*>(el)[i] = reinterpret_cast<const int32_t*>(plan.elem)[i];
  int8_t* isv = reinterpret_cast<int8_t*>(smem + ne * sizeof(KElem));
  for (int i = threadIdx.x; i < n; i += T) isv[i] = plan.is_v[i];
  size_t off = ne * sizeof(KElem) + ((n + 15) / 16) * 16;
  double* base = reinterpret_cast<double*>(smem + off);
  const int tid = threadIdx.x;
  t.s.n_ = n;
  t.s.A_ = base + tid;
  t.s.rhs_ = base + (size_t)n * n * T + tid;
  t.s.x_ = t.s.rhs_ + (size_t)n * T;
  t.s.xold_ = t.s.x_ + (size_t)n * T;
  t.s.col_ = t.s.xold_ + (size_t)n * T;
  t.s.piv_ = reinterpret_cast<int*>(base + (size_t)(n * n + 4 * n) * T) + tid;
  t.s.L_ = reinterpret_cast<float*>(base + (size_t)(n * n + 4 * n) * T + ((size_t)n * T + 1) / 2) + tid;
  t.prog.el = el; t.prog.isv = isv; t.prog.ne = ne; t.prog.n_nodes = plan.n_nodes; t.prog.n_state = plan.n_state;
  t.prog.nonlin_empty = plan.n_nonlin == 0;
}

// Per-topology kernels with a shared-memory system of compile-time size N: the
// same per-thread layout without the element table.
template <int T, int N>
__device__ inline void smem_layout_static(SmemSys<T, N>& s, unsigned char* smem) {
  double* base = reinterpret_cast<double*>(smem);
  const int tid = threadIdx.x;
  s.n_ = N;
  s.A_ = base + tid;
  s.rhs_ = base + N * N * T + tid;
  s.x_ = s.rhs_ + N * T;
  s.xold_ = s.x_ + N * T;
  s.col_ = s.xold_ + N * T;
  s.piv_ = reinterpret_cast<int*>(base + (N * N + 4 * N) * T) + tid;
  s.L_ = reinterpret_cast<float*>(base + (N * N + 4 * N) * T + (N * T + 1) / 2) + tid;
}


__device__ __forceinline__ void op_state_reset(OpState& st, const KOpts& o) {
  st.phase = PH_MAIN; st.it = 0; st.maxIter = o.itl1; st.total = 0; st.firstErr = 0; st.status = KS_STATUS_NOT_RUN;
  st.nsteps = 0; st.quiet = 0; st.ok = false; st.srcStepping = false; st.fp64 = !o.mixed; st.initJct = true;
  st.diagGmin = 0; st.g = 0; st.factor = 0; st.srcFact = 0; st.done = 0; st.step = 0; st.ptG = 0; st.h = 0;
}

// One (*Sim).solve: stamp at x (copied to xold), add the gmin-stepping and
// pseudo-transient diagonals, solve.  Returns 0 or the solver error.
template <class SY, class P>
__device__ __forceinline__ int solve_once(Thr<SY, P>& t, OpState& st, LoadParams lp) {
  SY& s = t.s;
  const int n = t.n();
#pragma unroll
  for (int i = 0; i < n; i++) s.xo(i) = s.xn(i);
  lp.initJct = st.initJct;
  lp.gmin = t.o.gmin;
  lp.srcStepping = st.srcStepping;
  lp.srcFact = st.srcFact;
  // systems with one pivot sequence at DC and one for transient steps
  if constexpr (SY::kModes) s.set_mode(lp.mode == ModeOP || lp.mode == ModeTranOP ? 0 : 1);
  load_all(t.prog, t.V, t.D, t.Sb, s, lp);
  if (st.ptG > 0) {
#pragma unroll
    for (int i = 0; i < n; i++) {
      if (!prog_owns(t.prog, i)) continue;
      double pv = t.ptPrev[i];
      if (t.prog.is_v(i)) { s.a(i, i) += st.ptG; s.rhs(i) += st.ptG * pv; }
      else { s.a(i, i) -= st.ptG; s.rhs(i) -= st.ptG * pv; }
    }
  }
  if (st.diagGmin > 0) {
#pragma unroll
    for (int i = 0; i < n; i++) if (prog_owns(t.prog, i) && t.prog.is_v(i)) s.a(i, i) += st.diagGmin;
  }
  prog_sync(t.prog);
  // a per-topology program factors on its fixed pivot sequence first; a pivot
  // that fails its threshold hands the solve to partial pivoting
  int err = SOLVE_STATIC_FAIL;
  if (!st.fp64) {
    const double rtol = t.prog.nonlin_empty ? 1e-11 : t.o.refine_tol;
    if constexpr (P::kStaticLU) err = t.prog.lu_mixed(s, t.o.passes, rtol);
    if (err == SOLVE_STATIC_FAIL) err = lu_solve_mixed(s, t.o.passes, rtol);
    if (err == SOLVE_FP32_FAIL) {  // the FP64 path takes over this circuit
      st.fp64 = true;
      err = lu_solve_fp64(s);
    }
  } else {
    if constexpr (P::kStaticLU) err = t.prog.lu_fp64(s);
    if (err == SOLVE_STATIC_FAIL) err = lu_solve_fp64(s);
  }
  st.total++;
  return err;
}

// One Newton iteration: a solve plus the bookkeeping of analysis/newton.go:36-57.
// Returns -1 while the current newton() call goes on, else its result.
template <class SY, class P>
__device__ __forceinline__ int newton_step(Thr<SY, P>& t, OpState& st, const LoadParams& lp) {
  int err = solve_once(t, st, lp);
  int res = -1;
  if (err) res = err;
  else if (t.prog.nonlin_empty) res = KS_STATUS_OK;
  else if (st.initJct) st.initJct = false;
  else if (converged(t.prog, t.V, t.D, t.Sb, t.s, t.o, t.o.gmin)) res = KS_STATUS_OK;
  if (res < 0) {
    st.it++;
    if (st.it < st.maxIter) return -1;
    res = KS_STATUS_NO_CONVERGENCE;
  }
  st.it = 0;
  return res;
}

template <class SY, class P>
__device__ __forceinline__ void x_from_col(Thr<SY, P>& t, const Col& c) {
#pragma unroll
  for (int i = 0; i < t.n(); i++) t.s.xn(i) = c[i];
}
template <class SY, class P>
__device__ __forceinline__ void x_to_col(Thr<SY, P>& t, const Col& c) {
#pragma unroll
  for (int i = 0; i < t.n(); i++) c[i] = t.s.xn(i);
}
template <class SY, class P>
__device__ __forceinline__ void x_zero(Thr<SY, P>& t, const Col& also) {
#pragma unroll
  for (int i = 0; i < t.n(); i++) { t.s.xn(i) = 0.0; also[i] = 0.0; }
}

// dcSolve start, analysis/newton.go:96-102, with applyNodeSet (:221-243) when x0
// holds a starting point (node voltages; other unknowns start at 0).  With the
// FP32 start stage on (k32, o.start32 > 0; one thread per circuit), the point the
// stage reaches from x0 (or from InitJct when x0 is null) is the NodeSet instead;
// where the stage fails the start is x0 (or InitJct) as without it.
template <class SY, class P>
__device__ __forceinline__ void dc_start(Thr<SY, P>& t, OpState& st, const double* x0, int64_t c,
                                         const K32* k32 = nullptr, int64_t B = 0) {
  op_state_reset(st, t.o);
  const int n = t.n();
  bool seeded = false;
  if constexpr (!P::kWarp) {
    if (k32 && t.o.start32 > 0) seeded = start32(t, *k32, x0, c, B, t.o.start32);
  }
  if (!seeded) {
#pragma unroll
    for (int i = 0; i < n; i++) t.s.xn(i) = 0.0;
    if (x0) {
#pragma unroll
      for (int i = 0; i < n; i++)
        if (i < t.prog.n_nodes - 1) t.s.xn(i) = x0[c * n + i];
      seeded = true;
    }
  }
  if (seeded) {
    accept_all(t.prog, t.V, t.D, t.Sb, t.s, 0.0, ModeOP, t.o.gmin, true);
    st.initJct = false;
  }
}

// The learned start's own check: largest distance of a node voltage of the
// solution from the start x0.
template <class SY, class P>
__device__ __forceinline__ double start_distance(Thr<SY, P>& t, const double* x0, int64_t c) {
  const int n = t.n();
  long long k = 0;
#pragma unroll
  for (int i = 0; i < n; i++)
    if (i < t.prog.n_nodes - 1) k = key_max(k, mag_key(t.s.xn(i) - x0[c * n + i]));
  return key_mag(k);
}

// Advance dcSolve with the result of a finished newton() call.  Sets st.phase to
// PH_DONE and st.status when the DC solve is over.
template <class SY, class P>
__device__ __forceinline__ void dc_advance(Thr<SY, P>& t, OpState& st, int res) {
  const KOpts& o = t.o;
  const int n = t.n();
  bool advance = true;
  while (advance) {
    advance = false;
    switch (st.phase) {
      case PH_MAIN:
        if (res == KS_STATUS_OK || t.prog.nonlin_empty || !retryable(res)) { st.status = res; st.phase = PH_DONE; break; }
        st.firstErr = res;
        st.phase = PH_GMIN;
        if (!o.no_gmin) {  // gminStepping start, :134-142
          x_zero(t, t.save);
          st.initJct = true; st.g = 1e-2; st.factor = 10.0; st.ok = false; st.nsteps = 0;
          st.diagGmin = st.g;
        } else { st.nsteps = -1; res = KS_STATUS_NO_CONVERGENCE; advance = true; }
        break;
      case PH_GMIN: {  // :143-175
        bool fail = false;
        if (st.nsteps < 0) fail = true;
        else if (res == KS_STATUS_OK) {
          x_to_col(t, t.save);
          if (st.g == 0) { st.diagGmin = 0; st.status = KS_STATUS_OK; st.phase = PH_DONE; break; }
          st.ok = true;
          st.factor = fmin(st.factor * sqrt(st.factor), 10.0);
          st.g = st.g / st.factor < o.gmin ? 0.0 : st.g / st.factor;
          if (++st.nsteps >= 200) fail = true;
        } else if (!retryable(res) || !st.ok) {
          fail = true;
        } else {
          x_from_col(t, t.save);
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
            x_zero(t, t.save);
            st.srcStepping = true; st.done = 0; st.step = 0.1; st.srcFact = 0; st.nsteps = 0;
          } else { st.phase = PH_SRC; st.nsteps = -1; res = KS_STATUS_NO_CONVERGENCE; advance = true; }
        }
        break;
      }
      case PH_SRC_INIT:
        if (res != KS_STATUS_OK) { st.phase = PH_SRC; st.nsteps = -1; advance = true; break; }
        x_to_col(t, t.save);
        st.phase = PH_SRC;
        st.srcFact = fmin(st.done + st.step, 1.0);
        break;
      case PH_SRC: {  // :193-213
        bool fail = false;
        if (st.nsteps < 0) fail = true;
        else if (res == KS_STATUS_OK) {
          if (st.srcFact == 1) { st.srcStepping = false; st.srcFact = 0; st.status = KS_STATUS_OK; st.phase = PH_DONE; break; }
          x_to_col(t, t.save);
          st.done = st.srcFact; st.step = fmin(st.step * 1.5, 0.5);
          if (++st.nsteps >= 1000) fail = true;
        } else if (!retryable(res)) fail = true;
        else {
          x_from_col(t, t.save);
          st.step /= 2;
          if (st.step < 1e-3) fail = true;
          else if (++st.nsteps >= 1000) fail = true;
        }
        if (fail) {
          st.srcStepping = false; st.srcFact = 0;
          if (!o.no_pt) {  // pseudoTransient start, :260-273
            st.phase = PH_PT;
            x_zero(t, t.ptPrev);
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
            x_from_col(t, t.ptPrev);
            st.h /= 4;
            if (st.h < 1e-15) fail = true;
          }
        } else {
          bool moved = false;
#pragma unroll
          for (int i = 0; i < n; i++) {
            double xv = t.s.xn(i);
            double tol = t.prog.is_v(i) ? o.vntol : o.abstol;
            moved |= fabs(xv - t.ptPrev[i]) > o.reltol * fabs(xv) + tol;
          }
          x_to_col(t, t.ptPrev);
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

// polish, analysis/op.go:251-271: up to two more FP64 solves at the accepted
// operating point, so that the small-signal model of an AC sweep is taken at x
// exact to round-off instead of at the Newton tolerance.
template <class SY, class P>
__device__ __forceinline__ int polish(Thr<SY, P>& t, OpState& st, const LoadParams& lp) {
  st.initJct = false; st.ptG = 0; st.diagGmin = 0; st.srcStepping = false; st.srcFact = 0; st.fp64 = true;
  const int n = t.n();
  for (int k = 0; k < 2; k++) {
    int err = solve_once(t, st, lp);
    if (err) return err;
    bool done = true;
#pragma unroll
    for (int i = 0; i < n; i++)
      if (prog_owns(t.prog, i) && fabs(t.s.xn(i) - t.s.xo(i)) > 1e-12 * fmax(1.0, fabs(t.s.xn(i)))) done = false;
    if (prog_all(t.prog, done)) break;
  }
  return KS_STATUS_OK;
}

// Element results and the ledger of circuit c at its accepted operating point
// (ks_results.cuh; the results instantiation of the generic kernels only).
template <class SY, class P>
__device__ inline int op_results(Thr<SY, P>& t, const LoadParams& lp, int64_t c, int64_t B);

// The operating point of one circuit after another, pulled from the queue.
// kRes: with the element results and the energy ledger (ks_op_results).
template <class SY, class P, bool kRes = false>
__device__ __forceinline__ void op_persistent(Thr<SY, P>& t, const double* values, const double* derived, double* state,
                                     double* work, int64_t B, const double* x0, double* out_x, int32_t* out_status,
                                     int32_t* out_iters, uint64_t deadline_ns, unsigned long long* queue,
                                     const K32* k32 = nullptr) {
  const uint64_t t0 = deadline_ns ? prog_clock(t.prog) : 0;
  const KOpts& o = t.o;
  const int maxTotal = o.max_iter_total > 0 ? o.max_iter_total : 3300 * o.itl1 + 16;
  LoadParams lp;
  lp.mode = ModeOP; lp.method = BE; lp.time = 0; lp.h = 0; lp.rh = 0; lp.initJct = false; lp.gmin = o.gmin;
  lp.srcStepping = false; lp.srcFact = 0;
  OpState st;
  bool restarted = false;  // the circuit is being solved again from the standard start
  int64_t c = prog_next(t.prog, queue);
  if (c < B) {
    thr_bind(t, values, derived, state, work, B, c);
    init_state(t.prog, t.D, t.Sb);
    dc_start(t, st, x0, c, k32, B);
  }
  while (c < B) {
    bool done = false;
    if (deadline_ns && prog_clock(t.prog) - t0 > deadline_ns) { st.status = KS_STATUS_INTERRUPTED; done = true; }
    else if (o.cancel && (st.total & 7) == 0 && prog_cancelled(t.prog, o.cancel)) {  // every 8th solve
      st.status = KS_STATUS_INTERRUPTED; done = true;
    } else if (st.total >= maxTotal) { st.status = KS_STATUS_NO_CONVERGENCE; done = true; }
    else {
      int res = newton_step(t, st, lp);
      if (res >= 0) dc_advance(t, st, res);
      done = st.phase == PH_DONE;
    }
    if (!done) continue;
    // a solution far from the learned start: the start led Newton elsewhere (another
    // basin of a circuit with several operating points, or a prediction too poor
    // to trust); solve the circuit again as the reference does, from InitJct
    if (x0 && !restarted && t.o.start_check > 0 && st.status == KS_STATUS_OK &&
        start_distance(t, x0, c) > t.o.start_check) {
      const int spent = st.total;
      restarted = true;
      init_state(t.prog, t.D, t.Sb);
      dc_start(t, st, nullptr, c);
      st.total = spent;
      continue;
    }
    if (st.status == KS_STATUS_OK && o.polish && !t.prog.nonlin_empty) {
      accept_all(t.prog, t.V, t.D, t.Sb, t.s, 0.0, ModeOP, o.gmin, false);
      st.status = polish(t, st, lp);
    }
    // the results read each device's linearization before its Accept (which
    // leaves that linearization as it is, analysis/op.go:348-349)
    if constexpr (kRes) {
      if (st.status == KS_STATUS_OK) st.status = op_results(t, lp, c, B);
    }
    if (st.status == KS_STATUS_OK || st.status == KS_STATUS_LEDGER)
      accept_all(t.prog, t.V, t.D, t.Sb, t.s, 0.0, ModeOP, o.gmin, false);
    if (out_x) {
      const int n = t.n();  // per circuit for the multi-topology kernels
      const int64_t base = t.prog.x_base(c, n);
#pragma unroll
      for (int i = 0; i < n; i++) out_x[base + i] = t.s.xn(i);
    }
    if (out_status) out_status[c] = st.status;
    if (out_iters) out_iters[c] = st.total;
    c = prog_next(t.prog, queue);
    restarted = false;
    if (c < B) {
      thr_bind(t, values, derived, state, work, B, c);
      init_state(t.prog, t.D, t.Sb);
      dc_start(t, st, x0, c, k32, B);
    }
  }
}

// analysis.DC (analysis/dc.go:51-133) of one circuit after another: the swept
// source `src` (its .DC override, device/source.go:43-66) takes pts[0..npts-1]
// in order (for each value of a second, outer source src2 >= 0 in turn), and
// each point is an operating point (dcSolve + Accept at ModeOP)
// warm-started from the previous point's solution and device state, so no
// InitJct once a point has converged (analysis/newton.go:96) and a switch's
// state, a junction's limiting history follow the sweep.  The sweep of a circuit
// stops at its first failing point: out_status[c] is that point's status
// (KS_STATUS_OK when all converged), out_points[c] the points solved, out_x
// [B][npts2][npts][n] their solutions.
template <class SY, class P>
__device__ __forceinline__ void dc_sweep_persistent(Thr<SY, P>& t, const double* values, const double* derived,
                                                    double* state, double* work, int64_t B, int src,
                                                    const double* pts, int npts, int src2, const double* pts2,
                                                    int npts2, double* out_x, int32_t* out_status,
                                                    int32_t* out_points, int32_t* out_iters, uint64_t deadline_ns,
                                                    unsigned long long* queue) {
  const uint64_t t0 = deadline_ns ? prog_clock(t.prog) : 0;
  const KOpts& o = t.o;
  const int maxTotal = o.max_iter_total > 0 ? o.max_iter_total : 3300 * o.itl1 + 16;
  LoadParams lp;
  lp.mode = ModeOP; lp.method = BE; lp.time = 0; lp.h = 0; lp.rh = 0; lp.initJct = false; lp.gmin = o.gmin;
  lp.srcStepping = false; lp.srcFact = 0;
  OpState st;
  for (int64_t c = prog_next(t.prog, queue); c < B; c = prog_next(t.prog, queue)) {
    thr_bind(t, values, derived, state, work, B, c);
    init_state(t.prog, t.D, t.Sb);
    KElem se{}, se2{};
    int k = 0;
    t.prog.each([&](const KElem& e) KS_INLINE_LAMBDA {
      if (k == src) se = e;
      if (k == src2) se2 = e;
      k++;
    });
    const Col S = state_col(t.Sb, se), S2 = state_col(t.Sb, se2);
    bool warm = false;
    int status = KS_STATUS_OK, done = 0, iters = 0;
    const int n = t.n(), total = npts * (src2 >= 0 ? npts2 : 1);
    for (int p = 0; p < total && status == KS_STATUS_OK; p++) {
      // the inner source steps fastest; the outer one (a second sweep) holds each
      // of its values through a whole inner sweep (analysis/dc.go:105-111)
      if (src2 >= 0) { S2[SV_OVR] = pts2[p / npts]; S2[SV_OVRON] = 1; }
      S[SV_OVR] = pts[p % npts]; S[SV_OVRON] = 1;  // SetDCOverride, device/source.go:70-73
      if (warm) { op_state_reset(st, o); st.initJct = false; }
      else dc_start(t, st, nullptr, c);
      while (true) {
        if (deadline_ns && prog_clock(t.prog) - t0 > deadline_ns) { st.status = KS_STATUS_INTERRUPTED; break; }
        if (o.cancel && (st.total & 7) == 0 && prog_cancelled(t.prog, o.cancel)) { st.status = KS_STATUS_INTERRUPTED; break; }
        if (st.total >= maxTotal) { st.status = KS_STATUS_NO_CONVERGENCE; break; }
        const int res = newton_step(t, st, lp);
        if (res >= 0) dc_advance(t, st, res);
        if (st.phase == PH_DONE) break;
      }
      iters += st.total;
      status = st.status;
      if (status != KS_STATUS_OK) break;
      accept_all(t.prog, t.V, t.D, t.Sb, t.s, 0.0, ModeOP, o.gmin, false);
      warm = true;
      done = p + 1;
      if (out_x) {
        const int64_t base = ((int64_t)c * total + p) * n;
#pragma unroll
        for (int i = 0; i < n; i++) out_x[base + i] = t.s.xn(i);
      }
    }
    S[SV_OVRON] = 0;  // ClearDCOverride
    if (src2 >= 0) S2[SV_OVRON] = 0;
    if (out_status) out_status[c] = status;
    if (out_points) out_points[c] = done;
    if (out_iters) out_iters[c] = iters;
  }
}

}  // namespace ksg
