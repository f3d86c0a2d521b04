// ks_kernels.cu — batched operating-point kernels of the GB300 engine.
//
// One thread owns one circuit; a warp runs 32 circuits of the same topology in
// lock-step through the same element program, with every per-circuit operand a
// coalesced SoA column.  The per-thread dense system lives in shared memory.
// The Newton loop and the whole DC fallback chain of analysis/newton.go run on
// the device as a per-thread state machine: each pass of the loop body is one
// (*Sim).solve (stamp + LU), and the scalar control code decides what the next
// solve is.  Every loop is bounded (the reference's own step limits, plus a
// total-iteration guard and an optional wall-clock deadline), so no circuit can
// keep a warp spinning.
#include <cuda_runtime.h>
#include <cstdio>
#include "ks_internal.h"
#include "ks_solve.cuh"

using namespace ksg;

// [rows][cols] -> [cols][rows] (host value vectors to SoA columns).
__global__ void k_transpose(const double* __restrict__ src, double* __restrict__ dst, int64_t rows, int64_t cols) {
  __shared__ double tile[32][33];
  int64_t r0 = (int64_t)blockIdx.y * 32, c0 = (int64_t)blockIdx.x * 32;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    int64_t r = r0 + i, c = c0 + threadIdx.x;
    if (r < rows && c < cols) tile[i][threadIdx.x] = src[r * cols + c];
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    int64_t c = c0 + i, r = r0 + threadIdx.x;
    if (r < rows && c < cols) dst[c * rows + r] = tile[threadIdx.x][i];
  }
}

int ks_launch_transpose(const double* src, double* dst, int64_t rows, int64_t cols, void* stream) {
  if (rows <= 0 || cols <= 0) return 0;
  dim3 grid((unsigned)((cols + 31) / 32), (unsigned)((rows + 31) / 32)), block(32, 8);
  k_transpose<<<grid, block, 0, (cudaStream_t)stream>>>(src, dst, rows, cols);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// breakdownVoltage, device/diode.go:166-187.
__device__ double breakdown_voltage(double is, double bv, double ibv, double vt) {
  if (ibv < is * bv / vt) return bv;
  auto g = [&](double x) { return is * (exp(fmin((bv - x) / vt, 700.0)) - 1 + x / vt) - ibv; };
  double lo = fmin(0.0, bv - vt * log1p(ibv / is)) - 10 * vt, hi = bv;
  for (int i = 0; i < 200 && g(lo) <= 0; i++) lo -= 10 * vt;
  for (int i = 0; i < 200; i++) {
    double mid = 0.5 * (lo + hi);
    if (mid == lo || mid == hi) break;
    if (g(mid) > 0) lo = mid; else hi = mid;
  }
  return 0.5 * (lo + hi);
}

// Per-circuit constants (NewDiode, NewBJT, NewMOSFET/derive, resolveWave with the
// analysis's print step and stop time).
__global__ void k_setup(KPlan plan, const double* __restrict__ values, double* derived, int64_t B,
                        double step, double stop) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= B) return;
  Col V{const_cast<double*>(values) + c, B}, D{derived + c, B};
  for (int k = 0; k < plan.n_elem; k++) {
    KElem e = plan.elem[k];
    int p = e.param, d = e.derived;
    switch (e.kind) {
      case KS_ELEM_R: D[d + DR_G] = 1 / V[p]; break;
      case KS_ELEM_V: case KS_ELEM_I:
        wave_resolve(e.wave, V, p + KS_SRC_P_ARGS, e.nargs, D, d, step, stop);
        break;
      case KS_ELEM_D: {
        double vt0 = kK * kTNom / kQ, vte = V[p + KS_D_P_N] * vt0, IS = V[p + KS_D_P_IS];
        D[d + DD_VTE] = vte;
        D[d + DD_VCRIT] = vte * log(vte / (kSqrt2 * IS));
        D[d + DD_XBV] = (e.flags & KS_F_HAS_BV) ? breakdown_voltage(IS, V[p + KS_D_P_BV], V[p + KS_D_P_IBV], vt0) : 0.0;
        double RS = V[p + KS_D_P_RS];
        D[d + DD_GRS] = RS > 0 ? 1 / RS : 0.0;
        break;
      }
      case KS_ELEM_Q: {
        double vt = kK * kTNom / kQ;
        D[d + DQ_VT] = vt;
        D[d + DQ_VCRIT] = vt * log(vt / (kSqrt2 * V[p + KS_Q_P_IS]));
        D[d + DQ_RBPR] = V[p + KS_Q_P_RBM];
        D[d + DQ_RBPI] = V[p + KS_Q_P_RB] - V[p + KS_Q_P_RBM];
        D[d + DQ_GCPR] = V[p + KS_Q_P_RC] > 0 ? 1 / V[p + KS_Q_P_RC] : 0.0;
        D[d + DQ_GEPR] = V[p + KS_Q_P_RE] > 0 ? 1 / V[p + KS_Q_P_RE] : 0.0;
        D[d + DQ_OVTF] = V[p + KS_Q_P_VTF] > 0 ? 1 / (1.44 * V[p + KS_Q_P_VTF]) : 0.0;
        double fc = V[p + KS_Q_P_FC];
        double vje = V[p + KS_Q_P_VJE], mje = V[p + KS_Q_P_MJE], vjc = V[p + KS_Q_P_VJC], mjc = V[p + KS_Q_P_MJC];
        D[d + DQ_F1E] = vje * (1 - pow(1 - fc, 1 - mje)) / (1 - mje);
        D[d + DQ_F2E] = pow(1 - fc, 1 + mje);
        D[d + DQ_F3E] = 1 - fc * (1 + mje);
        D[d + DQ_F1C] = vjc * (1 - pow(1 - fc, 1 - mjc)) / (1 - mjc);
        D[d + DQ_F2C] = pow(1 - fc, 1 + mjc);
        D[d + DQ_F3C] = 1 - fc * (1 + mjc);
        break;
      }
      case KS_ELEM_M: mos_derive(e, V, D); break;
      default: break;
    }
  }
}

int ks_launch_setup(const KsDeviceBatch& b, double step, double stop, void* stream) {
  int tpb = 128;
  unsigned grid = (unsigned)((b.B + tpb - 1) / tpb);
  k_setup<<<grid, tpb, 0, (cudaStream_t)stream>>>(b.plan, b.values, b.derived, b.B, step, stop);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// ---------------------------------------------------------------- operating point
namespace {

enum Phase { PH_MAIN = 0, PH_GMIN, PH_SRC_INIT, PH_SRC, PH_PT, PH_PT_FINAL, PH_DONE };

struct OpState {  // the per-circuit control state of dcSolve and its fallbacks
  int phase, it, maxIter, total, firstErr, status, nsteps;
  bool initJct, ok, srcStepping, fp64;
  double diagGmin, g, factor, srcFact, done, step, ptG, h;
  int quiet;
};

__device__ __forceinline__ bool retryable(int e) {
  return e == KS_STATUS_NO_CONVERGENCE || e == KS_STATUS_NONFINITE || e == KS_STATUS_SINGULAR;
}

}  // namespace

// Shared memory per block: element table, then per-thread arrays (stride T).
template <int T>
__global__ void __launch_bounds__(T) k_op(KPlan plan, KOpts o, const double* __restrict__ values,
                                          const double* __restrict__ derived, double* state, double* work,
                                          int64_t B, const double* __restrict__ x0, double* out_x,
                                          int32_t* out_status, int32_t* out_iters, uint64_t deadline_ns) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int n = plan.n, ne = plan.n_elem;
  KElem* el = reinterpret_cast<KElem*>(smem);
  for (int i = threadIdx.x; i < ne * (int)(sizeof(KElem) / 4); i += T)
    reinterpret_cast<int32_t*>(el)[i] = reinterpret_cast<const int32_t*>(plan.elem)[i];
  int8_t* isv = reinterpret_cast<int8_t*>(smem + ne * sizeof(KElem));
  for (int i = threadIdx.x; i < n; i += T) isv[i] = plan.is_v[i];
  size_t off = ne * sizeof(KElem) + ((n + 15) / 16) * 16;
  double* base = reinterpret_cast<double*>(smem + off);
  const int tid = threadIdx.x;
  ThreadSys<T> s;
  s.n = n;
  s.A = base + tid;
  s.rhs = base + (size_t)n * n * T + tid;
  s.x = s.rhs + (size_t)n * T;
  s.xold = s.x + (size_t)n * T;
  s.col = s.xold + (size_t)n * T;
  s.piv = reinterpret_cast<int*>(base + (size_t)(n * n + 4 * n) * T) + tid;
  s.L32 = reinterpret_cast<float*>(base + (size_t)(n * n + 4 * n) * T + ((size_t)n * T + 1) / 2) + tid;
  __syncthreads();

  int64_t c = (int64_t)blockIdx.x * T + tid;
  if (c >= B) return;
  Col V{const_cast<double*>(values) + c, B}, D{const_cast<double*>(derived) + c, B}, Sb{state + c, B};
  Col save{work + c, B}, ptPrev{work + (int64_t)n * B + c, B};
  const uint64_t t0 = deadline_ns ? globaltimer_ns() : 0;
  const bool nonlinEmpty = plan.n_nonlin == 0;
  const int maxTotal = o.max_iter_total > 0 ? o.max_iter_total : 3300 * o.itl1 + 16;
  init_state(el, ne, plan.n_state, D, Sb);

  OpState st;
  st.phase = PH_MAIN; st.it = 0; st.maxIter = o.itl1; st.total = 0; st.firstErr = 0; st.status = KS_STATUS_NOT_RUN;
  st.nsteps = 0; st.ok = false; st.srcStepping = false; st.fp64 = !o.mixed;
  st.diagGmin = 0; st.g = 0; st.factor = 0; st.srcFact = 0; st.done = 0; st.step = 0; st.ptG = 0; st.h = 0; st.quiet = 0;
  // dcSolve start, analysis/newton.go:96-102 (applyNodeSet when a start is given).
  st.initJct = true;
  for (int i = 0; i < n; i++) s.x[i * T] = 0.0;
  if (x0) {
    for (int i = 0; i < plan.n_nodes - 1; i++) s.x[i * T] = x0[c * n + i];
    accept_all<T>(el, ne, V, D, Sb, s.x, 0.0, ModeOP, o.gmin, true);
    st.initJct = false;
  }

  while (st.phase != PH_DONE) {
    if (deadline_ns && globaltimer_ns() - t0 > deadline_ns) { st.status = KS_STATUS_INTERRUPTED; break; }
    if (st.total >= maxTotal) { st.status = KS_STATUS_NO_CONVERGENCE; break; }
    // ---- one (*Sim).solve, analysis/op.go:289-322
    for (int i = 0; i < n; i++) s.xold[i * T] = s.x[i * T];
    LoadParams lp;
    lp.mode = ModeOP; lp.method = BE; lp.time = 0; lp.h = 0; lp.initJct = st.initJct; lp.gmin = o.gmin;
    lp.srcStepping = st.srcStepping; lp.srcFact = st.srcFact;
    load_all<T>(el, ne, V, D, Sb, s, lp);
    if (st.ptG > 0) {
      for (int i = 0; i < n; i++) {
        double pv = ptPrev[i];
        if (isv[i]) { s.a(i, i) += st.ptG; s.rhs[i * T] += st.ptG * pv; }
        else { s.a(i, i) -= st.ptG; s.rhs[i * T] -= st.ptG * pv; }
      }
    }
    if (st.diagGmin > 0) for (int i = 0; i < n; i++) if (isv[i]) s.a(i, i) += st.diagGmin;
    int err;
    if (!st.fp64) {
      err = lu_solve_mixed<T>(s);
      if (err == SOLVE_FP32_FAIL) {  // the FP64 path takes over this circuit
        st.fp64 = true;
        err = lu_solve_fp64<T>(s, s.rhs, s.x);  // rhs holds the FP64 residual
        if (err == SOLVE_OK) for (int i = 0; i < n; i++) s.x[i * T] += s.xold[i * T];
      }
    } else {
      err = lu_solve_fp64<T>(s, s.rhs, s.x);
    }
    st.total++;
    // ---- newton bookkeeping, analysis/newton.go:36-57
    int res = -1;  // -1: keep iterating this newton call
    if (err) res = err;
    else if (nonlinEmpty) res = KS_STATUS_OK;
    else if (st.initJct) st.initJct = false;
    else if (converged<T>(el, ne, isv, V, D, Sb, s, o, o.gmin)) res = KS_STATUS_OK;
    if (res < 0) {
      st.it++;
      if (st.it >= st.maxIter) res = KS_STATUS_NO_CONVERGENCE;
      else continue;
    }
    st.it = 0;
    // ---- dcSolve and fallbacks, analysis/newton.go:95-311
    bool advance = true;
    while (advance) {
      advance = false;
      switch (st.phase) {
        case PH_MAIN:
          if (res == KS_STATUS_OK || nonlinEmpty || !retryable(res)) { st.status = res; st.phase = PH_DONE; break; }
          st.firstErr = res;
          res = -1;
          // fall into the first enabled fallback
          if (!o.no_gmin) {  // gminStepping start, :134-142
            st.phase = PH_GMIN;
            for (int i = 0; i < n; i++) s.x[i * T] = 0.0, save[i] = 0.0;
            st.initJct = true; st.g = 1e-2; st.factor = 10.0; st.ok = false; st.nsteps = 0;
            st.diagGmin = st.g;
          } else { st.phase = PH_GMIN; res = KS_STATUS_NO_CONVERGENCE; st.nsteps = -1; advance = true; }
          break;
        case PH_GMIN: {
          bool fail = false;
          if (st.nsteps < 0) fail = true;  // disabled
          else if (res == KS_STATUS_OK) {
            for (int i = 0; i < n; i++) save[i] = s.x[i * T];
            if (st.g == 0) { st.diagGmin = 0; st.status = KS_STATUS_OK; st.phase = PH_DONE; break; }
            st.ok = true;
            st.factor = fmin(st.factor * sqrt(st.factor), 10.0);
            st.g = st.g / st.factor < o.gmin ? 0.0 : st.g / st.factor;
            if (++st.nsteps >= 200) fail = true;
          } else if (!retryable(res) || !st.ok) {
            fail = true;
          } else {
            for (int i = 0; i < n; i++) s.x[i * T] = save[i];
            double prev = st.g == 0 ? o.gmin : st.g * st.factor;
            st.factor = sqrt(st.factor);
            if (st.factor < 1.00005) fail = true;
            else { st.g = prev / st.factor; if (++st.nsteps >= 200) fail = true; }
          }
          if (fail) {
            st.diagGmin = 0;
            if (!o.no_source) {  // sourceStepping start, :180-192
              st.phase = PH_SRC_INIT;
              for (int i = 0; i < n; i++) s.x[i * T] = 0.0, save[i] = 0.0;
              st.srcStepping = true; st.done = 0; st.step = 0.1; st.srcFact = 0; st.nsteps = 0;
            } else { st.phase = PH_SRC; st.nsteps = -1; res = KS_STATUS_NO_CONVERGENCE; advance = true; }
          } else st.diagGmin = st.g;
          break;
        }
        case PH_SRC_INIT:
          if (res != KS_STATUS_OK) { st.phase = PH_SRC; st.nsteps = -1; advance = true; break; }
          for (int i = 0; i < n; i++) save[i] = s.x[i * T];
          st.phase = PH_SRC;
          st.srcFact = fmin(st.done + st.step, 1.0);
          break;
        case PH_SRC: {
          bool fail = false;
          if (st.nsteps < 0) fail = true;
          else if (res == KS_STATUS_OK) {
            if (st.srcFact == 1) { st.srcStepping = false; st.srcFact = 0; st.status = KS_STATUS_OK; st.phase = PH_DONE; break; }
            for (int i = 0; i < n; i++) save[i] = s.x[i * T];
            st.done = st.srcFact; st.step = fmin(st.step * 1.5, 0.5);
            if (++st.nsteps >= 1000) fail = true;
          } else if (!retryable(res)) fail = true;
          else {
            for (int i = 0; i < n; i++) s.x[i * T] = save[i];
            st.step /= 2;
            if (st.step < 1e-3) fail = true;
            else if (++st.nsteps >= 1000) fail = true;
          }
          if (fail) {
            st.srcStepping = false; st.srcFact = 0;
            if (!o.no_pt) {  // pseudoTransient start, :260-273
              st.phase = PH_PT;
              for (int i = 0; i < n; i++) s.x[i * T] = 0.0, ptPrev[i] = 0.0;
              st.initJct = true; st.h = 1e-6; st.quiet = 0; st.nsteps = 0; st.ptG = 1 / st.h;
            } else { st.status = st.firstErr; st.phase = PH_DONE; }
          } else st.srcFact = fmin(st.done + st.step, 1.0);
          break;
        }
        case PH_PT: {
          bool fail = false;
          if (res != KS_STATUS_OK) {
            if (!retryable(res)) fail = true;
            else {
              for (int i = 0; i < n; i++) s.x[i * T] = ptPrev[i];
              st.h /= 4;
              if (st.h < 1e-15) fail = true;
            }
          } else {
            bool moved = false;
            for (int i = 0; i < n; i++) {
              double xv = s.x[i * T];
              double tol = isv[i] ? o.vntol : o.abstol;
              if (fabs(xv - ptPrev[i]) > o.reltol * fabs(xv) + tol) { moved = true; break; }
            }
            for (int i = 0; i < n; i++) ptPrev[i] = s.x[i * T];
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
  if (st.status == KS_STATUS_OK) accept_all<T>(el, ne, V, D, Sb, s.x, 0.0, ModeOP, o.gmin, false);
  if (out_x) for (int i = 0; i < n; i++) out_x[c * n + i] = s.x[i * T];
  if (out_status) out_status[c] = st.status;
  if (out_iters) out_iters[c] = st.total;
}

static size_t op_smem(int n, int ne, int T, bool mixed) {
  size_t off = (size_t)ne * sizeof(KElem) + ((n + 15) / 16) * 16;
  size_t per = (size_t)(n * n + 4 * n) * 8 + (size_t)n * 4 + 8;
  if (mixed) per += (size_t)n * n * 4 + 8;
  return off + per * T;
}

int ks_launch_op(const KsDeviceBatch& b, const KOpts& o, const double* x0, double* out_x, int32_t* out_status,
                 int32_t* out_iters, double deadline_s, void* stream) {
  int n = b.plan.n, ne = b.plan.n_elem;
  if (n > KS_MAX_DENSE) return -2;
  uint64_t dl = deadline_s > 0 ? (uint64_t)(deadline_s * 1e9) : 0;
  int maxSmem = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&maxSmem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  bool mixed = o.mixed != 0;
  int T = 64;
  size_t sm = op_smem(n, ne, 64, true);
  if (sm > (size_t)maxSmem) { T = 32; sm = op_smem(n, ne, 32, true); }
  if (sm > (size_t)maxSmem) return -2;
  (void)mixed;
  unsigned grid = (unsigned)((b.B + T - 1) / T);
  cudaStream_t st = (cudaStream_t)stream;
  if (T == 64) {
    cudaFuncSetAttribute(k_op<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_op<64><<<grid, 64, sm, st>>>(b.plan, o, b.values, b.derived, b.state, b.work, b.B, x0, out_x, out_status,
                                   out_iters, dl);
  } else {
    cudaFuncSetAttribute(k_op<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_op<32><<<grid, 32, sm, st>>>(b.plan, o, b.values, b.derived, b.state, b.work, b.B, x0, out_x, out_status,
                                   out_iters, dl);
  }
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}
