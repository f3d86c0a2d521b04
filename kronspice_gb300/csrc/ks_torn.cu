// ks_torn.cu — transient analyses of large circuits torn into pieces, batched
// over variants of one topology (kron.JacobianTearing as Options.Solver,
// kron/jacobian.go, under analysis.OP / analysis.Tran).
//
// The Newton Jacobian J of every variant is torn as the reference tears it
// (buildPlan, kron/jacobian.go:296-389): the pieces are the connected
// components of J's pattern with the torn elements' node pairs removed; every
// entry joining two pieces is a coupling entry; B is the block diagonal and the
// interconnection (Aitchison) is
//     z = B^-1 b,   (I + M.Q.B^-1.P) w = M.Q.z,   x = B^-1 (b - P.w).
// GB300 layout:
//   * per-variant arrays are [item][variant] (variant fastest), so a warp loads
//     or stamps one element / unknown of 32 variants with coalesced accesses;
//   * each piece is factored as a band matrix (its unknowns in reverse
//     Cuthill-McKee order, rows and columns equilibrated as the reference's
//     denseLU does, partial pivoting in the band as LAPACK's gbtf2): one CTA per
//     (variant, piece), all pieces of all variants in one launch;
//   * the interconnection matrix of each variant is dense, column-major,
//     factored by a blocked right-looking LU (panel, interchange, triangular and
//     trailing-update kernels here: the update is a batched FP64 GEMM over the
//     variants being refactored, 64 x 64 tiles of C per CTA);
//   * factors are kept between Newton iterations and time steps while the
//     refinement against the exact J (componentwise backward error <= 1e-14,
//     accepted at 1e-12, kron/jacobian.go:551-589) converges on them; when it
//     does not, every variant is refactored at its current J and the solve is
//     repeated (the reference's stale-factor retry, :404-411).  With reuse off
//     the factors are remade at every solve.
//   * a variant whose torn solve is still not accepted is solved untorn, as the
//     reference falls back to a plain LU of the whole J (:412-434): a second
//     instance of the same topology without torn elements (one band piece per
//     connected component, no interconnection), built at the first fallback,
//     takes that variant's J and right-hand side.
// Device loads, limiting, convergence tests and Accept are the engine's
// per-element device code (ks_solve.cuh), one thread per (element, variant).
#include <cuda_pipeline.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "ks_internal.h"
#include "ks_newton.cuh"

using namespace ksg;
using ksh::set_error;

namespace {

// J (and the right-hand side) of variant v as the device loads see it: stamps
// go atomically into the slot of (i, j) in J's row-sorted pattern.
struct TornSys {
  static constexpr bool kStatic = false;
  static constexpr bool kAtomic = true;
  static constexpr bool kModes = false;
  static constexpr int kUnroll = 1;
  const int32_t *rp, *ci;
  double *J, *rhs;
  const double *xn_p, *xo_p;
  int64_t V;
  int v;
  __device__ __forceinline__ int slot(int i, int j) const {
    int lo = rp[i], hi = rp[i + 1] - 1;
    while (lo < hi) {
      int mid = (lo + hi) >> 1;
      if (ci[mid] < j) lo = mid + 1; else hi = mid;
    }
    return lo;
  }
  __device__ __forceinline__ void add(int i, int j, double val) { atomicAdd(&J[(int64_t)slot(i, j) * V + v], val); }
  __device__ __forceinline__ void add_rhs(int i, double val) { atomicAdd(&rhs[(int64_t)i * V + v], val); }
  __device__ __forceinline__ double xn(int i) const { return xn_p[(int64_t)i * V + v]; }
  __device__ __forceinline__ double xo(int i) const { return xo_p[(int64_t)i * V + v]; }
};

struct PieceD {  // one piece, device view
  int n, kl, ku, ldab;
  int64_t band_off;  // doubles, per variant
  int idx_off;       // into pidx (band order -> global unknown)
  int port_off, nports;
  int cc_off, ncc;
  int64_t wc_off;    // doubles, per variant: [ncc][nports]
  int64_t y_off;     // doubles, per variant: multi-RHS scratch [n][nports]
  int pslot_off, npslot;
};

__device__ __forceinline__ unsigned long long dkey(double x) {  // monotone key of a non-negative double
  return (unsigned long long)__double_as_longlong(x);
}

}  // namespace

// ------------------------------------------------------------------ element kernels
__global__ void k_tl_init_state(KPlan plan, const double* derived, double* state, int64_t V) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)plan.n_state * V) return;
  state[t] = 0.0;
}

__global__ void k_tl_init_mos(KPlan plan, const double* derived, double* state, int64_t V) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)plan.n_elem * V) return;
  const int e = (int)(t / V), v = (int)(t % V);
  const KElem el = plan.elem[e];
  if (el.kind == KS_ELEM_M) state[(int64_t)(el.state + SM_AVON) * V + v] = derived[(int64_t)(el.derived + DM_VTO) * V + v];
  if (el.kind == KS_ELEM_S || el.kind == KS_ELEM_W) {  // the ON / OFF initial state, device/switch.go:105-106
    const double on = derived[(int64_t)(el.derived + DW_INIT) * V + v];
    state[(int64_t)(el.state + SW_ON) * V + v] = on;
    state[(int64_t)(el.state + SW_ACC) * V + v] = on;
  }
}

// One Load per (element, variant) into J and rhs at the linearization point xo.
__global__ void k_tl_load(KPlan plan, const double* values, const double* derived, double* state, int64_t V,
                          const int32_t* rp, const int32_t* ci, double* J, double* rhs, const double* x,
                          const double* xo, LoadParams lp, const uint8_t* mask) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)plan.n_elem * V) return;
  const int e = (int)(t / V), v = (int)(t % V);
  if (!mask[v]) return;
  const KElem el = plan.elem[e];
  Col Vb{const_cast<double*>(values) + v, V}, Db{const_cast<double*>(derived) + v, V}, Sb{state + v, V};
  TornSys s{rp, ci, J, rhs, x, xo, V, v};
  elem_load(el, Vb, Db, Sb, s, lp);
}

// converged (analysis/newton.go:59-82): flags[v] |= 1 when an unknown moved, 2
// when a device was limited or failed its ConvTest.
__global__ void k_tl_conv_x(int n, int64_t V, const int8_t* isv, const double* x, const double* xo, KOpts o,
                            const uint8_t* mask, int32_t* flags) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * V) return;
  const int i = (int)(t / V), v = (int)(t % V);
  if (!mask[v]) return;
  const double a = x[t], b = xo[t];
  const double tol = (isv[i] ? o.vntol : o.abstol) + o.reltol * fmax(fabs(a), fabs(b));
  if (fabs(a - b) > tol) atomicOr(&flags[v], 1);
}

__global__ void k_tl_conv_elem(KPlan plan, const double* values, const double* derived, double* state, int64_t V,
                               const int32_t* nonlin, int n_nonlin, const double* x, const double* xo, KOpts o,
                               const uint8_t* mask, int32_t* flags) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n_nonlin * V) return;
  const int k = (int)(t / V), v = (int)(t % V);
  if (!mask[v]) return;
  const KElem el = plan.elem[nonlin[k]];
  Col Vb{const_cast<double*>(values) + v, V}, Db{const_cast<double*>(derived) + v, V}, Sb{state + v, V};
  TornSys s{nullptr, nullptr, nullptr, nullptr, x, xo, V, v};
  if (!elem_converged(el, Vb, Db, Sb, s, o, o.gmin)) atomicOr(&flags[v], 2);
}

__global__ void k_tl_accept(KPlan plan, const double* values, const double* derived, double* state, int64_t V,
                            const double* x, double time, int mode, double gmin, const uint8_t* mask) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)plan.n_elem * V) return;
  const int e = (int)(t / V), v = (int)(t % V);
  if (!mask[v]) return;
  const KElem el = plan.elem[e];
  Col Vb{const_cast<double*>(values) + v, V}, Db{const_cast<double*>(derived) + v, V}, Sb{state + v, V};
  TornSys s{nullptr, nullptr, nullptr, nullptr, x, x, V, v};
  elem_accept(el, Vb, Db, Sb, s, time, mode, gmin, false);
}

// ------------------------------------------------------------------ vectors
__global__ void k_tl_copy_masked(int64_t n, int64_t V, const double* src, double* dst, const uint8_t* mask) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * V || !mask[t % V]) return;
  dst[t] = src[t];
}

__global__ void k_tl_axpy_masked(int64_t n, int64_t V, const double* dx, double* x, const uint8_t* mask) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * V || !mask[t % V]) return;
  x[t] += dx[t];
}

// r = b - J x and the componentwise backward error max_i |r_i| / (|b_i| + sum_j |J_ij x_j|)
// per variant (kron/jacobian.go:551-570), as a monotone key.
__global__ void k_tl_resid(int n, int64_t V, const int32_t* rp, const int32_t* ci, const double* J, const double* b,
                           const double* x, double* r, unsigned long long* berr, const uint8_t* mask) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * V) return;
  const int i = (int)(t / V), v = (int)(t % V);
  if (!mask[v]) return;
  double ri = b[t], den = fabs(ri);
  for (int s = rp[i]; s < rp[i + 1]; s++) {
    const double p = J[(int64_t)s * V + v] * x[(int64_t)ci[s] * V + v];
    ri -= p;
    den += fabs(p);
  }
  r[t] = ri;
  double e;
  if (den > 0) e = fabs(ri) / den;
  else e = ri != 0 ? INFINITY : 0.0;
  if (isnan(e)) e = INFINITY;
  atomicMax(&berr[v], dkey(e));
}

// ------------------------------------------------------------------ refactor
// Row and column equilibration of each piece (denseLU.factor, kron/jacobian.go:626-648):
// rs_i = 1 / max |J_ij| over row i's entries inside its piece, cs_j likewise after rs.
__global__ void k_tl_equil_rows(int n, int64_t V, const int32_t* rp, const uint8_t* slot_in, const double* J,
                                double* rs, int32_t* bad, const uint8_t* mask) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * V) return;
  const int i = (int)(t / V), v = (int)(t % V);
  if (!mask[v]) return;
  double m = 0;
  for (int s = rp[i]; s < rp[i + 1]; s++)
    if (slot_in[s]) m = fmax(m, fabs(J[(int64_t)s * V + v]));
  if (m == 0) { atomicOr(&bad[v], 1); rs[t] = 0; return; }
  rs[t] = 1 / m;
}

__global__ void k_tl_equil_cols(int n, int64_t V, const int32_t* cp, const int32_t* cslot, const int32_t* crow,
                                const double* J, const double* rs, double* cs, int32_t* bad, const uint8_t* mask) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * V) return;
  const int j = (int)(t / V), v = (int)(t % V);
  if (!mask[v]) return;
  double m = 0;
  for (int k = cp[j]; k < cp[j + 1]; k++)
    m = fmax(m, fabs(J[(int64_t)cslot[k] * V + v]) * rs[(int64_t)crow[k] * V + v]);
  if (m == 0) { atomicOr(&bad[v], 1); cs[t] = 0; return; }
  cs[t] = 1 / m;
}

// The equilibrated block of each piece in LAPACK band storage: A(i, j) at
// AB[kl + ku + i - j + j * ldab], kl extra rows on top for the fill of pivoting.
__global__ void k_tl_band_fill(const PieceD* pcs, int P, int64_t V, int64_t band_stride, double* band,
                               const int32_t* pslot, const int32_t* pli, const int32_t* plj, const int32_t* pidx,
                               const double* J, const double* rs, const double* cs, const uint8_t* mask) {
  const int v = blockIdx.x % V, p = blockIdx.x / V;
  if (!mask[v]) return;
  const PieceD pc = pcs[p];
  double* AB = band + (int64_t)v * band_stride + pc.band_off;
  const int64_t sz = (int64_t)pc.ldab * pc.n;
  for (int64_t k = threadIdx.x; k < sz; k += blockDim.x) AB[k] = 0.0;
  __syncthreads();
  const int kv = pc.kl + pc.ku;
  for (int k = threadIdx.x; k < pc.npslot; k += blockDim.x) {
    const int q = pc.pslot_off + k;
    const int li = pli[q], lj = plj[q];
    const int gi = pidx[pc.idx_off + li], gj = pidx[pc.idx_off + lj];
    AB[kv + li - lj + (int64_t)lj * pc.ldab] =
        J[(int64_t)pslot[q] * V + v] * rs[(int64_t)gi * V + v] * cs[(int64_t)gj * V + v];
  }
}

// Band LU with partial pivoting (LAPACK gbtf2) of one piece of one variant.
__global__ void __launch_bounds__(256) k_tl_band_lu(const PieceD* pcs, int64_t V, int64_t band_stride, double* band,
                                                    int64_t piv_stride, int32_t* piv_all, int32_t* bad,
                                                    const uint8_t* mask) {
  const int v = blockIdx.x % V, p = blockIdx.x / V;
  if (!mask[v]) return;
  const PieceD pc = pcs[p];
  double* AB = band + (int64_t)v * band_stride + pc.band_off;
  int32_t* piv = piv_all + (int64_t)v * piv_stride + pc.idx_off;
  const int n = pc.n, kl = pc.kl, ku = pc.ku, ldab = pc.ldab, kv = kl + ku;
  __shared__ int s_p, s_ju;
  __shared__ double s_piv;
  int ju = 0;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int j = 0; j < n; j++) {
    const int km = min(kl, n - 1 - j);
    // pivot: largest |A(j + i, j)|, i = 0..km (first of equals)
    if (wid == 0) {
      double best = -1;
      int bi = 0;
      for (int i = lane; i <= km; i += 32) {
        const double a = fabs(AB[kv + i + (int64_t)j * ldab]);
        if (a > best) { best = a; bi = i; }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (lane == 0) {
        s_p = bi;
        s_piv = AB[kv + bi + (int64_t)j * ldab];
        if (best > 0) ju = max(ju, min(j + ku + bi, n - 1));
        s_ju = ju;
      }
    }
    __syncthreads();
    const int pr = s_p;
    const double pv = s_piv;
    ju = s_ju;
    if (threadIdx.x == 0) piv[j] = j + pr;
    if (pv == 0) {  // exactly singular column: the reference refuses the piece
      if (threadIdx.x == 0) atomicOr(&bad[v], 2);
      __syncthreads();
      continue;
    }
    if (pr != 0)
      for (int c = j + (int)threadIdx.x; c <= ju; c += blockDim.x) {
        double* a = &AB[kv + j - c + (int64_t)c * ldab];
        double* b = &AB[kv + j + pr - c + (int64_t)c * ldab];
        const double tmp = *a; *a = *b; *b = tmp;
      }
    __syncthreads();
    const double rpv = 1 / pv;
    for (int i = 1 + (int)threadIdx.x; i <= km; i += blockDim.x) AB[kv + i + (int64_t)j * ldab] *= rpv;
    __syncthreads();
    // rank-1 update of A(j+1..j+km, j+1..ju)
    const int ncol = ju - j;
    const int work = km * ncol;
    for (int w = threadIdx.x; w < work; w += blockDim.x) {
      const int i = 1 + w % km, c = j + 1 + w / km;
      AB[kv + j + i - c + (int64_t)c * ldab] -= AB[kv + i + (int64_t)j * ldab] * AB[kv + j - c + (int64_t)c * ldab];
    }
    __syncthreads();
  }
}

// Solve of every piece of the selected variants: out = cs . Ab^-1 (rs . (b - P.w)),
// with the subtraction only when w is given (the second solve of the apply).
// One warp per (variant, piece): the band is swept column by column with warp
// barriers only (a column step is a few shared-memory accesses and one
// multiply-add per row a lane owns).  The part of each column a sweep reads (the
// kl multipliers below the diagonal going down, the kl + ku entries above it
// and the diagonal coming back) is staged into shared memory CH columns at a
// time with asynchronous copies, NB - 1 blocks ahead, so the sweep waits on
// barriers, not on memory.
template <typename F, int CH, int NB>
__global__ void __launch_bounds__(32) k_tl_band_solve(const PieceD* pcs, int64_t V, int64_t band_stride,
                                                      const F* band, int64_t piv_stride, const int32_t* piv_all,
                                                      const int32_t* pidx, const double* rs, const double* cs,
                                                      const double* b, const int32_t* row_a, const double* w,
                                                      double* out, const uint8_t* mask, int max_n, int max_colw) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  F* smem = reinterpret_cast<F*>(smem_raw);
  const int v = blockIdx.x % V, p = blockIdx.x / V;
  if (!mask[v]) return;
  const PieceD pc = pcs[p];
  const F* AB = band + (int64_t)v * band_stride + pc.band_off;
  const int32_t* piv = piv_all + (int64_t)v * piv_stride + pc.idx_off;
  const int n = pc.n, kl = pc.kl, ldab = pc.ldab, kv = pc.kl + pc.ku;
  const int t = threadIdx.x;
  F* y = smem;                                      // [max_n], rounded to 2
  F* buf = smem + ((max_n + 1) & ~1);               // [NBUF][CH][max_colw]
  int* spiv = reinterpret_cast<int*>(buf + NB * CH * max_colw);  // [NBUF][CH]
  const int bufsz = CH * max_colw;
  for (int i = t; i < n; i += 32) {
    const int g = pidx[pc.idx_off + i];
    double bi = b[(int64_t)g * V + v];
    if (w) {
      const int a = row_a[g];
      if (a >= 0) bi -= w[(int64_t)a * V + v];
    }
    y[i] = (F)(bi * rs[(int64_t)g * V + v]);
  }
  const int nch = (n + CH - 1) / CH;
  // stage block c: `width` doubles of each column from row offset `first`
  auto stage = [&](int c, int first, int width, bool pivots) {
    if (c < 0 || c >= nch) { __pipeline_commit(); return; }
    const int j0 = c * CH, cols = min(CH, n - j0);
    F* dst = buf + (c % NB) * bufsz;
    const F* src = AB + first + (int64_t)j0 * ldab;
    for (int jj = 0; jj < cols; jj++, dst += max_colw, src += ldab)
      for (int r = t; r < width; r += 32) __pipeline_memcpy_async(dst + r, src + r, sizeof(F));
    __pipeline_commit();
    if (pivots && t < cols) spiv[(c % NB) * CH + t] = piv[j0 + t];
  };
  // L: row interchanges and the unit lower band (staged: rows kv+1 .. kv+kl of each column)
  for (int c = 0; c < NB - 1; c++) stage(c, kv + 1, kl, true);
  for (int c = 0; c < nch; c++) {
    stage(c + NB - 1, kv + 1, kl, true);
    __pipeline_wait_prior(NB - 1);
    __syncwarp();
    const F* B = buf + (c % NB) * bufsz;
    const int* P = spiv + (c % NB) * CH;
    const int j0 = c * CH, cols = min(CH, n - j0);
    for (int jj = 0; jj < cols; jj++) {
      const int j = j0 + jj;
      const int km = min(kl, n - 1 - j);
      const int pj = P[jj];
      if (pj != j) {  // the same for every lane
        if (t == 0) { const F tmp = y[j]; y[j] = y[pj]; y[pj] = tmp; }
        __syncwarp();
      }
      const F yj = y[j];
      if (kl <= 128) {  // up to 4 rows a lane: loads first, then the updates (independent)
        F lv[4], yv[4];
#pragma unroll
        for (int r = 0; r < 4; r++) {
          const int o = t + 32 * r;
          lv[r] = o < km ? B[jj * max_colw + o] : F(0);
          yv[r] = o < km ? y[j + 1 + o] : F(0);
        }
#pragma unroll
        for (int r = 0; r < 4; r++) {
          const int o = t + 32 * r;
          if (o < km) y[j + 1 + o] = yv[r] - lv[r] * yj;
        }
      } else {
        for (int o = t; o < km; o += 32) y[j + 1 + o] -= B[jj * max_colw + o] * yj;
      }
      __syncwarp();
    }
  }
  __pipeline_wait_prior(0);
  __syncwarp();
  // U: rows 0 .. kv of each column (row j - kv + o at o, the diagonal at kv), last block first
  for (int k = 0; k < NB - 1; k++) stage(nch - 1 - k, 0, kv + 1, false);
  for (int c = nch - 1; c >= 0; c--) {
    stage(c - (NB - 1), 0, kv + 1, false);
    __pipeline_wait_prior(NB - 1);
    __syncwarp();
    const F* B = buf + (c % NB) * bufsz;
    const int j0 = c * CH, cols = min(CH, n - j0);
    for (int jj = cols - 1; jj >= 0; jj--) {
      const int j = j0 + jj;
      const F yj = y[j] * B[jj * max_colw + kv];  // the diagonal slot holds 1 / u_jj
      __syncwarp();
      if (t == 0) y[j] = yj;
      if (kv <= 256) {  // up to 8 rows a lane: loads first, then the updates
        F uv[8], yv[8];
#pragma unroll
        for (int r = 0; r < 8; r++) {
          const int o = t + 32 * r, i = j - kv + o;
          const bool on = o < kv && i >= 0;
          uv[r] = on ? B[jj * max_colw + o] : F(0);
          yv[r] = on ? y[i] : F(0);
        }
#pragma unroll
        for (int r = 0; r < 8; r++) {
          const int o = t + 32 * r, i = j - kv + o;
          if (o < kv && i >= 0) y[i] = yv[r] - uv[r] * yj;
        }
      } else {
        for (int o = t; o < kv; o += 32) {
          const int i = j - kv + o;
          if (i >= 0) y[i] -= B[jj * max_colw + o] * yj;
        }
      }
      __syncwarp();
    }
  }
  __pipeline_wait_prior(0);
  __syncwarp();
  for (int i = t; i < n; i += 32) {
    const int g = pidx[pc.idx_off + i];
    out[(int64_t)g * V + v] = (double)y[i] * cs[(int64_t)g * V + v];
  }
}

// Blocked form of the same solve, the rows a block of 32 columns can reach held
// in registers: lane l keeps rows base + 32 k + l (k < NS) of a window that
// slides 32 rows per block, so a column step is one shuffle broadcast of the
// pivot row and one shared-memory load and multiply-add per slot, and the
// sweep's dependency chain runs at register latency.  Each staged column sits
// in a zero-padded row (its entries from 32 going forward, from PB coming back)
// so that window slot k of lane l reads 31 + l - jj + 32 k (jj: the column's
// place in its block of 32): the multiply-adds need no bounds tests, rows the
// column does not reach read zeros.  Rows enter the window from the
// right-hand side (forward) or from the scratch ys (backward) and leave it
// final; the band's columns stream through shared memory in chunks of SC, NBUF
// deep.  NSL >= 1 + kl / 32 and NSU >= 1 + (kl + ku) / 32.
template <typename F, int NSL, int NSU, int SC, int NBUF>
__global__ void __launch_bounds__(32) k_tl_band_solve_rw(const PieceD* pcs, int64_t V, int64_t band_stride,
                                                         const F* band, int64_t piv_stride, const int32_t* piv_all,
                                                         const int32_t* pidx, const double* rs, const double* cs,
                                                         const double* b, const int32_t* row_a, const double* w,
                                                         double* out, F* ys_all, const uint8_t* mask, int max_colw) {
  static_assert(32 % SC == 0, "chunks tile the 32-column blocks");
  constexpr int WF = 32 * NSL + 32, WB = 32 * NSU + 32;  // padded row widths, forward and backward
  extern __shared__ __align__(16) unsigned char smem_raw[];
  F* buf = reinterpret_cast<F*>(smem_raw);                                 // [NBUF][SC][WF or WB]
  F* dg = buf + NBUF * SC * WB;                                            // [NBUF][SC] 1 / u_jj
  int* spiv = reinterpret_cast<int*>(dg + NBUF * SC);                      // [NBUF][SC]
  const int v = blockIdx.x % V, p = blockIdx.x / V;
  if (!mask[v]) return;
  const PieceD pc = pcs[p];
  const F* AB = band + (int64_t)v * band_stride + pc.band_off;
  const int32_t* piv = piv_all + (int64_t)v * piv_stride + pc.idx_off;
  F* ys = ys_all + (int64_t)v * piv_stride + pc.idx_off;
  const int n = pc.n, kl = pc.kl, ldab = pc.ldab, kv = pc.kl + pc.ku;
  const int lane = threadIdx.x;
  const int nch = (n + SC - 1) / SC;
  const int PB = 32 * NSU - kv - 1;  // backward: U(j - kv + o, j) at PB + o
  auto zero_buf = [&](int width) {
    for (int q = lane; q < NBUF * SC * width; q += 32) buf[q] = F(0);
    __syncwarp();
  };
  // stage chunk c: `width` entries from row offset `first` of each of its
  // columns to its rows (c % NBUF, j % SC), at 32 going forward and at PB back
  // (the rest of every row stays zero)
  auto stage = [&](int c, int first, int width, int W, bool fwd) {
    if (c < 0 || c >= nch) { __pipeline_commit(); return; }
    const int j0 = c * SC, cols = min(SC, n - j0);
    for (int jj = 0; jj < cols; jj++) {
      const int j = j0 + jj;
      F* dst = buf + ((c % NBUF) * SC + jj) * W + (fwd ? 32 : PB);
      const F* src = AB + first + (int64_t)j * ldab;
      for (int r = lane; r < width; r += 32) __pipeline_memcpy_async(dst + r, src + r, sizeof(F));
    }
    __pipeline_commit();
    if (fwd && lane < cols) spiv[(c % NBUF) * SC + lane] = piv[j0 + lane];
  };
  auto rhs_row = [&](int i) -> F {  // (b - P.w) of row i, scaled by the row equilibration
    if (i < 0 || i >= n) return F(0);
    const int g = pidx[pc.idx_off + i];
    double bi = b[(int64_t)g * V + v];
    if (w) {
      const int a = row_a[g];
      if (a >= 0) bi -= w[(int64_t)a * V + v];
    }
    return (F)(bi * rs[(int64_t)g * V + v]);
  };
  // ---- forward: row interchanges and the unit lower band
  zero_buf(WF);
  F y[NSL];
#pragma unroll
  for (int k = 0; k < NSL; k++) y[k] = rhs_row(32 * k + lane);
  for (int c = 0; c < NBUF - 1; c++) stage(c, kv + 1, kl, WF, true);
  for (int j0 = 0; j0 < n; j0 += 32) {
#pragma unroll
    for (int jj = 0; jj < 32; jj++) {
      const int j = j0 + jj;
      if (j < n) {
        if (jj % SC == 0) {
          __syncwarp();  // every lane is done with the buffer the next chunk goes to
          stage(j / SC + NBUF - 1, kv + 1, kl, WF, true);
          __pipeline_wait_prior(NBUF - 1);
          __syncwarp();
        }
        const int slot = ((j / SC) % NBUF) * SC + jj % SC;
        const int dp = spiv[slot] - j0;  // pivot row, window coordinates
        if (dp != jj) {                  // interchange rows j and p (warp-uniform, rare)
          const int ks = dp >> 5, ls = dp & 31;
          F at_p = y[0];
#pragma unroll
          for (int k = 1; k < NSL; k++)
            if (k == ks) at_p = y[k];
          const F vp = __shfl_sync(0xffffffffu, at_p, ls);
          const F vj = __shfl_sync(0xffffffffu, y[0], jj);
          if (lane == jj) y[0] = vp;
#pragma unroll
          for (int k = 0; k < NSL; k++)
            if (k == ks && lane == ls) y[k] = vj;
        }
        const F yj = __shfl_sync(0xffffffffu, y[0], jj);
        const F* B = buf + slot * WF + 31 + lane - jj;
#pragma unroll
        for (int k = 0; k < NSL; k++) y[k] -= B[32 * k] * yj;
      }
    }
    // rows j0 .. j0 + 31 are final: out to the scratch, the window slides
    if (j0 + lane < n) ys[j0 + lane] = y[0];
#pragma unroll
    for (int k = 0; k + 1 < NSL; k++) y[k] = y[k + 1];
    y[NSL - 1] = rhs_row(j0 + 32 * NSL + lane);
  }
  __pipeline_wait_prior(0);
  __syncwarp();
  // ---- backward: the upper band (U(j - kv + o, j) at o, 1 / u_jj at kv)
  zero_buf(WB);
  const int nb = (n + 31) / 32;
  F u[NSU];
  {
    const int base = 32 * (nb - 1) + 32 - 32 * NSU;
#pragma unroll
    for (int k = 0; k < NSU; k++) {
      const int i = base + 32 * k + lane;
      u[k] = (i >= 0 && i < n) ? ys[i] : F(0);
    }
  }
  // chunks in descending order; chunk c's diagonal moved out of its rows once it lands
  auto land = [&](int c) {
    const int j0 = c * SC, cols = min(SC, n - j0);
    if (lane < cols) {
      F* row = buf + ((c % NBUF) * SC + lane) * WB + PB;
      dg[(c % NBUF) * SC + lane] = row[kv];
      row[kv] = F(0);
    }
    __syncwarp();
  };
  for (int k = 0; k < NBUF - 1; k++) stage(nch - 1 - k, 0, kv + 1, WB, false);
  for (int j0 = 32 * (nb - 1); j0 >= 0; j0 -= 32) {
#pragma unroll
    for (int jj = 31; jj >= 0; jj--) {
      const int j = j0 + jj;
      if (j < n) {
        if (jj % SC == SC - 1 || j == n - 1) {
          const int c = j / SC;
          __syncwarp();
          stage(c - (NBUF - 1), 0, kv + 1, WB, false);
          __pipeline_wait_prior(NBUF - 1);
          __syncwarp();
          land(c);
        }
        const int slot = ((j / SC) % NBUF) * SC + jj % SC;
        if (lane == jj) u[NSU - 1] *= dg[slot];
        const F yj = __shfl_sync(0xffffffffu, u[NSU - 1], jj);
        const F* B = buf + slot * WB + 31 + lane - jj;
#pragma unroll
        for (int k = 0; k < NSU; k++) u[k] -= B[32 * k] * yj;
      }
    }
    {  // rows j0 .. j0 + 31 are final: out, unscaled by the column equilibration
      const int i = j0 + lane;
      if (i < n) {
        const int g = pidx[pc.idx_off + i];
        out[(int64_t)g * V + v] = (double)u[NSU - 1] * cs[(int64_t)g * V + v];
      }
    }
#pragma unroll
    for (int k = NSU - 1; k > 0; k--) u[k] = u[k - 1];
    const int i = j0 - 32 * NSU + lane;  // the window's new bottom rows
    u[0] = (i >= 0 && i < n) ? ys[i] : F(0);
  }
  __pipeline_wait_prior(0);
  __syncwarp();
}

// After a refactor (the port columns made): each band's U diagonal replaced by
// its reciprocal (the solves multiply by it) and the FP32 copy of the factors
// the applications stream under mixed precision.
__global__ void __launch_bounds__(256) k_tl_band_finish(const PieceD* pcs, int64_t V, int64_t band_stride, double* band,
                                                        float* band32, const uint8_t* mask) {
  const int v = blockIdx.x % V, p = blockIdx.x / V;
  if (!mask[v]) return;
  const PieceD pc = pcs[p];
  double* AB = band + (int64_t)v * band_stride + pc.band_off;
  float* AB32 = band32 + (int64_t)v * band_stride + pc.band_off;
  const int kv = pc.kl + pc.ku;
  for (int j = threadIdx.x; j < pc.n; j += blockDim.x) AB[kv + (int64_t)j * pc.ldab] = 1.0 / AB[kv + (int64_t)j * pc.ldab];
  __syncthreads();
  const int64_t total = (int64_t)pc.ldab * pc.n;
  for (int64_t q = threadIdx.x; q < total; q += blockDim.x) AB32[q] = (float)AB[q];
}

// The same for the interconnection factors (column-major [R][R] per variant).
__global__ void k_tl_ic_finish(int R, int64_t V, double* IC, float* IC32, const uint8_t* mask) {
  const int64_t per = (int64_t)R * R;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= per * V || !mask[t / per]) return;
  const int64_t e = t % per;
  double a = IC[t];
  if (e % R == e / R) { a = 1.0 / a; IC[t] = a; }
  IC32[t] = (float)a;
}

// W_c = (B^-1 e_port) at the piece's coupling-column unknowns, for every port of
// every piece (kron/jacobian.go:460-466), through a multi-RHS band solve in Y.
__global__ void __launch_bounds__(256) k_tl_wc(const PieceD* pcs, int64_t V, int64_t band_stride, const double* band,
                                               int64_t piv_stride, const int32_t* piv_all, const int32_t* pidx,
                                               const int32_t* plocal, const int32_t* ports_g, const int32_t* cc_g,
                                               const double* rs, const double* cs, int64_t y_stride, double* Yall,
                                               int64_t wc_stride, double* Wc_all, const uint8_t* mask) {
  const int v = blockIdx.x % V, p = blockIdx.x / V;
  if (!mask[v]) return;
  const PieceD pc = pcs[p];
  const int m = pc.nports;
  if (m == 0) return;
  const double* AB = band + (int64_t)v * band_stride + pc.band_off;
  const int32_t* piv = piv_all + (int64_t)v * piv_stride + pc.idx_off;
  double* Y = Yall + (int64_t)v * y_stride + pc.y_off;  // [n][m]
  const int n = pc.n, kl = pc.kl, ldab = pc.ldab, kv = pc.kl + pc.ku;
  for (int64_t k = threadIdx.x; k < (int64_t)n * m; k += blockDim.x) Y[k] = 0.0;
  __syncthreads();
  for (int k = threadIdx.x; k < m; k += blockDim.x) {
    const int g = ports_g[pc.port_off + k];
    Y[(int64_t)plocal[g] * m + k] = rs[(int64_t)g * V + v];
  }
  __syncthreads();
  for (int j = 0; j < n; j++) {
    const int km = min(kl, n - 1 - j);
    const int pj = piv[j];
    if (pj != j)
      for (int k = threadIdx.x; k < m; k += blockDim.x) {
        const double t = Y[(int64_t)j * m + k];
        Y[(int64_t)j * m + k] = Y[(int64_t)pj * m + k];
        Y[(int64_t)pj * m + k] = t;
      }
    __syncthreads();
    const int work = km * m;
    for (int w = threadIdx.x; w < work; w += blockDim.x) {
      const int i = 1 + w / m, k = w % m;
      Y[(int64_t)(j + i) * m + k] -= AB[kv + i + (int64_t)j * ldab] * Y[(int64_t)j * m + k];
    }
    __syncthreads();
  }
  for (int j = n - 1; j >= 0; j--) {
    const double rd = 1 / AB[kv + (int64_t)j * ldab];
    for (int k = threadIdx.x; k < m; k += blockDim.x) Y[(int64_t)j * m + k] *= rd;
    __syncthreads();
    const int top = max(0, j - kv);
    const int work = (j - top) * m;
    for (int w = threadIdx.x; w < work; w += blockDim.x) {
      const int i = top + w / m, k = w % m;
      Y[(int64_t)i * m + k] -= AB[kv + i - j + (int64_t)j * ldab] * Y[(int64_t)j * m + k];
    }
    __syncthreads();
  }
  double* Wc = Wc_all + (int64_t)v * wc_stride + pc.wc_off;  // [ncc][m]
  for (int64_t q = threadIdx.x; q < (int64_t)pc.ncc * m; q += blockDim.x) {
    const int c = (int)(q / m), k = (int)(q % m);
    const int g = cc_g[pc.cc_off + c];
    Wc[q] = Y[(int64_t)plocal[g] * m + k] * cs[(int64_t)g * V + v];
  }
}

// I + M.Q.B^-1.P, column-major [R][R] per variant (kron/jacobian.go:468-502):
// row a of the thread, over the coupling entries of its row.
__global__ void k_tl_ic_build(int R, int64_t V, const int32_t* offp, const int32_t* offs, const int32_t* ci,
                              const int32_t* pieceOf, const int32_t* slot_cc, const PieceD* pcs, const int32_t* port_a,
                              const double* J, int64_t wc_stride, const double* Wc_all, double* IC,
                              const uint8_t* mask) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)R * V) return;
  const int a = (int)(t % R), v = (int)(t / R);
  if (!mask[v]) return;
  double* A = IC + (int64_t)v * R * R;
  A[a + (int64_t)a * R] = 1.0;
  for (int q = offp[a]; q < offp[a + 1]; q++) {
    const int s = offs[q];
    const double val = J[(int64_t)s * V + v];
    if (val == 0) continue;
    const int p = pieceOf[ci[s]];
    const PieceD pc = pcs[p];
    const double* Wc = Wc_all + (int64_t)v * wc_stride + pc.wc_off + (int64_t)slot_cc[s] * pc.nports;
    for (int k = 0; k < pc.nports; k++) {
      const double g = Wc[k];
      if (g != 0) A[a + (int64_t)port_a[pc.port_off + k] * R] += val * g;
    }
  }
}

// Blocked LU of the interconnection matrices: panel of columns k0..k0+jb-1,
// partial pivoting over rows k0..R-1 (one CTA per variant).
__global__ void __launch_bounds__(1024) k_tl_ic_panel(int R, int k0, int jb, double* IC, int32_t* ipiv, int32_t* bad,
                                                      const uint8_t* mask) {
  const int v = blockIdx.x;
  if (!mask[v]) return;
  double* A = IC + (int64_t)v * R * R;
  int32_t* piv = ipiv + (int64_t)v * R;
  __shared__ double sv[32];
  __shared__ int si[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int j = k0; j < k0 + jb; j++) {
    double best = -1;
    int bi = j;
    for (int i = j + (int)threadIdx.x; i < R; i += blockDim.x) {
      const double a = fabs(A[i + (int64_t)j * R]);
      if (a > best || (a == best && i < bi)) { best = a; bi = i; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    if (lane == 0) { sv[wid] = best; si[wid] = bi; }
    __syncthreads();
    if (wid == 0) {
      best = lane < nw ? sv[lane] : -1;
      bi = lane < nw ? si[lane] : INT_MAX;
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (lane == 0) { sv[0] = best; si[0] = bi; }
    }
    __syncthreads();
    const int p = si[0];
    const double mx = sv[0];
    __syncthreads();
    if (threadIdx.x == 0) piv[j] = p;
    if (!(mx > 0)) {
      if (threadIdx.x == 0) atomicOr(&bad[v], 4);
      continue;
    }
    if (p != j)
      for (int c = k0 + (int)threadIdx.x; c < k0 + jb; c += blockDim.x) {
        const double t = A[j + (int64_t)c * R];
        A[j + (int64_t)c * R] = A[p + (int64_t)c * R];
        A[p + (int64_t)c * R] = t;
      }
    __syncthreads();
    const double rp = 1 / A[j + (int64_t)j * R];
    for (int i = j + 1 + (int)threadIdx.x; i < R; i += blockDim.x) A[i + (int64_t)j * R] *= rp;
    __syncthreads();
    const int rows = R - j - 1, cols = k0 + jb - j - 1;
    for (int64_t w = threadIdx.x; w < (int64_t)rows * cols; w += blockDim.x) {
      const int i = j + 1 + (int)(w % rows), c = j + 1 + (int)(w / rows);
      A[i + (int64_t)c * R] -= A[i + (int64_t)j * R] * A[j + (int64_t)c * R];
    }
    __syncthreads();
  }
}

// The panel's row interchanges applied to the columns outside it.
__global__ void k_tl_ic_swap(int R, int k0, int jb, double* IC, const int32_t* ipiv, int64_t V, const uint8_t* mask) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)R * V) return;
  const int c = (int)(t % R), v = (int)(t / R);
  if (!mask[v] || (c >= k0 && c < k0 + jb)) return;
  double* A = IC + (int64_t)v * R * R + (int64_t)c * R;
  const int32_t* piv = ipiv + (int64_t)v * R;
  for (int j = k0; j < k0 + jb; j++) {
    const int p = piv[j];
    if (p != j) { const double tmp = A[j]; A[j] = A[p]; A[p] = tmp; }
  }
}

// U12 = L11^-1 A12 for the columns right of the panel.
__global__ void k_tl_ic_trsm(int R, int k0, int jb, double* IC, int64_t V, const uint8_t* mask) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int ncol = R - k0 - jb;
  if (t >= (int64_t)ncol * V) return;
  const int c = k0 + jb + (int)(t % ncol), v = (int)(t / ncol);
  if (!mask[v]) return;
  double* A = IC + (int64_t)v * R * R;
  for (int j = k0; j < k0 + jb; j++) {
    const double u = A[j + (int64_t)c * R];
    if (u == 0) continue;
    for (int i = j + 1; i < k0 + jb; i++) A[i + (int64_t)c * R] -= A[i + (int64_t)j * R] * u;
  }
}

__global__ void k_tl_zero_ic(int64_t per, int64_t V, double* IC, const uint8_t* mask) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= per * V || !mask[t / per]) return;
  IC[t] = 0.0;
}

// Trailing update of the blocked LU, A22 -= A21 U12, for the listed variants
// (blockIdx.z: the variant's place in the list): A21 = A(k0+jb.., k0..k0+jb),
// U12 = A(k0..k0+jb, k0+jb..), column-major with leading dimension R.  A CTA of
// 256 threads owns a 64 x 64 tile of A22: both operand panels (jb <= 64 columns /
// rows) in shared memory, each thread 4 x 4 entries of the tile (rows tr + 16 r,
// columns tc + 16 c: 16 consecutive threads touch 16 consecutive rows of a
// column, so every global access is coalesced and every shared read is a
// broadcast or conflict-free), FP64 multiply-adds over jb.
#define KS_IC_TILE 64
__global__ void __launch_bounds__(256) k_tl_ic_gemm(int R, int k0, int jb, double* IC, const int32_t* list) {
  __shared__ double As[KS_IC_TILE][KS_IC_TILE + 1];  // [k][i]
  __shared__ double Bs[KS_IC_TILE][KS_IC_TILE + 1];  // [k][j]
  double* A = IC + (int64_t)list[blockIdx.z] * R * R;
  const int rest = R - k0 - jb, i0 = blockIdx.x * KS_IC_TILE, j0 = blockIdx.y * KS_IC_TILE;
  const int t = threadIdx.x, tr = t & 15, tc = t >> 4;
  const int off = k0 + jb;
  for (int e = t; e < KS_IC_TILE * KS_IC_TILE; e += 256) {
    const int ii = e & 63, kk = e >> 6;  // consecutive threads: consecutive rows of a column
    As[kk][ii] = (kk < jb && i0 + ii < rest) ? A[(off + i0 + ii) + (int64_t)(k0 + kk) * R] : 0.0;
    Bs[ii][kk] = (ii < jb && j0 + kk < rest) ? A[(k0 + ii) + (int64_t)(off + j0 + kk) * R] : 0.0;
  }
  __syncthreads();
  double acc[4][4];
#pragma unroll
  for (int r = 0; r < 4; r++)
#pragma unroll
    for (int c = 0; c < 4; c++) acc[r][c] = 0.0;
  for (int kk = 0; kk < jb; kk++) {
    double a[4], b[4];
#pragma unroll
    for (int r = 0; r < 4; r++) a[r] = As[kk][tr + 16 * r];
#pragma unroll
    for (int c = 0; c < 4; c++) b[c] = Bs[kk][tc + 16 * c];
#pragma unroll
    for (int r = 0; r < 4; r++)
#pragma unroll
      for (int c = 0; c < 4; c++) acc[r][c] = fma(a[r], b[c], acc[r][c]);
  }
#pragma unroll
  for (int c = 0; c < 4; c++) {
    const int j = j0 + tc + 16 * c;
    if (j >= rest) continue;
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const int i = i0 + tr + 16 * r;
      if (i < rest) A[(off + i) + (int64_t)(off + j) * R] -= acc[r][c];
    }
  }
}

// w = IC^-1 h with the factors (getrs: interchanges, unit lower, upper), one CTA
// per variant, by panels of 32 columns: warp 0 solves a panel's small triangle
// with warp barriers, then every thread updates the rest of the vector by the
// panel as one matrix-vector product (coalesced column reads).
template <typename F>
__global__ void __launch_bounds__(512) k_tl_ic_solve(int R, int64_t V, const F* IC, const int32_t* ipiv,
                                                      const double* h, double* w, const uint8_t* mask) {
  extern __shared__ __align__(16) unsigned char ic_smem[];  // y [R] then the pivots [R]
  F* y = reinterpret_cast<F*>(ic_smem);
  const int v = blockIdx.x;
  if (!mask[v]) return;
  int* sp = reinterpret_cast<int*>(y + R);
  const F* A = IC + (int64_t)v * R * R;
  const int32_t* piv = ipiv + (int64_t)v * R;
  const int t = threadIdx.x, T = blockDim.x, lane = t & 31;
  constexpr int NB = 32;
  for (int i = t; i < R; i += T) { y[i] = (F)h[(int64_t)i * V + v]; sp[i] = piv[i]; }
  __syncthreads();
  if (t == 0)
    for (int j = 0; j < R; j++) {
      const int p = sp[j];
      if (p != j) { const F tmp = y[j]; y[j] = y[p]; y[p] = tmp; }
    }
  __syncthreads();
  for (int k0 = 0; k0 < R; k0 += NB) {
    const int k1 = min(k0 + NB, R);
    if (t < 32) {  // unit lower triangle of the panel: lane l owns row k0 + l (its row loaded first)
      const int i = k0 + lane;
      F yi = i < k1 ? y[i] : F(0), a[NB];
#pragma unroll
      for (int q = 0; q < NB; q++) a[q] = (i < k1 && k0 + q < i) ? A[i + (int64_t)(k0 + q) * R] : F(0);
#pragma unroll
      for (int q = 0; q < NB; q++) {
        const F yj = __shfl_sync(0xffffffffu, yi, q);
        if (k0 + q < k1) yi -= a[q] * yj;
      }
      if (i < k1) y[i] = yi;
    }
    __syncthreads();
    for (int i = k1 + t; i < R; i += T) {  // the rows below: y_i -= L(i, k0:k1) . y(k0:k1)
      F s = 0;
      for (int j = k0; j < k1; j++) s += A[i + (int64_t)j * R] * y[j];
      y[i] -= s;
    }
    __syncthreads();
  }
  for (int k1 = R; k1 > 0; k1 -= NB) {
    const int k0 = max(0, k1 - NB);
    if (t < 32) {  // upper triangle of the panel (the lane's row and diagonal loaded first)
      const int i = k0 + lane;
      F yi = i < k1 ? y[i] : F(0), a[NB];
#pragma unroll
      for (int q = 0; q < NB; q++) a[q] = (i < k1 && k0 + q >= i && k0 + q < k1) ? A[i + (int64_t)(k0 + q) * R] : F(0);
#pragma unroll
      for (int q = NB - 1; q >= 0; q--) {
        if (k0 + q >= k1) continue;
        if (lane == q) yi *= a[q];  // the diagonal holds 1 / u_ii
        const F yj = __shfl_sync(0xffffffffu, yi, q);
        if (lane < q) yi -= a[q] * yj;
      }
      if (i < k1) y[i] = yi;
    }
    __syncthreads();
    for (int i = t; i < k0; i += T) {  // the rows above: y_i -= U(i, k0:k1) . y(k0:k1)
      F s = 0;
      for (int j = k0; j < k1; j++) s += A[i + (int64_t)j * R] * y[j];
      y[i] -= s;
    }
    __syncthreads();
  }
  for (int i = t; i < R; i += T) w[(int64_t)i * V + v] = (double)y[i];
}

// h = M.Q.z: each coupling row's entries times z at their columns.
__global__ void k_tl_h(int R, int64_t V, const int32_t* offp, const int32_t* offs, const int32_t* ci, const double* J,
                       const double* z, double* h, const uint8_t* mask) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)R * V) return;
  const int a = (int)(t / V), v = (int)(t % V);
  if (!mask[v]) return;
  double s = 0;
  for (int q = offp[a]; q < offp[a + 1]; q++) s += J[(int64_t)offs[q] * V + v] * z[(int64_t)ci[offs[q]] * V + v];
  h[t] = s;
}

// Step predictor on fixed steps: x <- the extrapolation of the accepted
// history (x_n in x, x_(n-1) in x1, x_(n-2) in x2) through its last `order` + 1
// points, and the history shifted (x1 <- x_n, x2 <- x_(n-1)).
__global__ void k_tl_predict(int64_t n, int order, double* x, double* x1, double* x2) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const double a = x[i], b = x1[i];
    x[i] = order >= 2 ? 3 * a - 3 * b + x2[i] : order == 1 ? 2 * a - b : a;
    x2[i] = b;
    x1[i] = a;
  }
}

__global__ void k_tl_record(int n_probes, const int32_t* probes, int64_t V, const double* x, double* out) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n_probes * V) return;
  const int q = (int)(t % n_probes), v = (int)(t / n_probes);
  out[t] = x[(int64_t)probes[q] * V + v];
}

// ------------------------------------------------------------------ host
namespace {

unsigned blocks_for(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

struct HostPiece {
  std::vector<int> idx;  // band order -> global unknown
  int kl = 0, ku = 0;
  std::vector<int> ports;  // coupling rows in this piece (global)
  std::vector<int> cc;     // coupling columns in this piece (global)
  std::vector<int> slots;  // in-piece slots
};

// Breadth-first levels from k within the unseen part of a piece: the last level's
// node of least degree and the eccentricity (George and Liu's pseudo-peripheral
// node search, 1979).
std::pair<int, int> far_node(int k, const std::vector<int>& nodes, const std::vector<std::vector<int>>& adj,
                             const std::vector<int>& local, const std::vector<int>& deg, const std::vector<char>& seen) {
  std::vector<int> d(nodes.size(), -1), q{k};
  d[k] = 0;
  for (size_t h = 0; h < q.size(); h++)
    for (int g : adj[nodes[q[h]]]) {
      const int j = local[g];
      if (j >= 0 && !seen[j] && d[j] < 0) { d[j] = d[q[h]] + 1; q.push_back(j); }
    }
  const int ecc = d[q.back()];
  int best = q.back();
  for (int j : q)
    if (d[j] == ecc && (deg[j] < deg[best] || (deg[j] == deg[best] && j < best))) best = j;
  return {best, ecc};
}

// reverse Cuthill-McKee order of a piece (symmetric pattern within the piece),
// each component started at a pseudo-peripheral node, so a grid piece gets
// levels across its diagonal and a band about as wide as one of its sides
std::vector<int> rcm(const std::vector<int>& nodes, const std::vector<std::vector<int>>& adj, const std::vector<int>& local) {
  const int m = (int)nodes.size();
  std::vector<int> deg(m), order;
  order.reserve(m);
  for (int k = 0; k < m; k++) deg[k] = (int)adj[nodes[k]].size();
  std::vector<char> seen(m, 0);
  while ((int)order.size() < m) {
    int start = -1;
    for (int k = 0; k < m; k++)
      if (!seen[k] && (start < 0 || deg[k] < deg[start])) start = k;
    auto f = far_node(start, nodes, adj, local, deg, seen);
    for (int it = 0; it < 8; it++) {
      auto g = far_node(f.first, nodes, adj, local, deg, seen);
      if (g.second <= f.second) break;
      f = g;
    }
    start = f.first;
    seen[start] = 1;
    size_t head = order.size();
    order.push_back(start);
    while (head < order.size()) {
      const int u = order[head++];
      std::vector<int> nb;
      for (int g : adj[nodes[u]]) {
        const int k = local[g];
        if (k >= 0 && !seen[k]) { seen[k] = 1; nb.push_back(k); }
      }
      std::sort(nb.begin(), nb.end(), [&](int a, int b) { return deg[a] < deg[b] || (deg[a] == deg[b] && a < b); });
      order.insert(order.end(), nb.begin(), nb.end());
    }
  }
  std::reverse(order.begin(), order.end());
  std::vector<int> out(m);
  for (int k = 0; k < m; k++) out[k] = nodes[order[k]];
  return out;
}

template <class T>
T* dalloc(size_t n, std::vector<void*>& owned) {
  void* p = nullptr;
  if (n == 0) n = 1;
  if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) return nullptr;
  owned.push_back(p);
  return static_cast<T*>(p);
}

template <class T>
bool upload(T** dst, const std::vector<T>& v, std::vector<void*>& owned) {
  *dst = dalloc<T>(v.size(), owned);
  if (!*dst) return false;
  if (!v.empty() && cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess) return false;
  return true;
}

}  // namespace

struct ks_torn {
  ksh::HostPlan hp;
  int V = 0, n = 0, nnz = 0, R = 0, P = 0, n_nonlin = 0;
  int max_piece = 0, max_band = 0;
  int max_colw = 0;  // widest staged column part of a band solve (max of kl, kl + ku + 1)
  int max_klu = 0;   // largest lower or upper bandwidth of a piece
  std::vector<HostPiece> pieces;
  std::vector<int> rp, ci;
  std::vector<int> h_pieceOf, h_rows;  // piece of each unknown, coupling rows (the plan, host side)
  std::vector<void*> owned;
  cudaStream_t st = nullptr, own = nullptr;  // the stream in use, the one created here
  // device symbolic
  KElem* d_elem = nullptr;
  int8_t* d_isv = nullptr;
  int32_t *d_rp, *d_ci, *d_cp, *d_cslot, *d_crow, *d_pidx, *d_plocal, *d_row_a, *d_offp, *d_offs, *d_pieceOf,
      *d_slot_cc, *d_port_a, *d_ports_g, *d_cc_g, *d_pslot, *d_pli, *d_plj, *d_nonlin;
  uint8_t* d_slot_in;
  PieceD* d_pcs;
  int64_t band_stride = 0, piv_stride = 0, wc_stride = 0, y_stride = 0;
  // device numeric
  double *values, *derived, *state, *x, *xo, *J, *rhs, *r, *dx, *z, *rs, *cs, *band, *Y, *Wc, *IC, *h, *w;
  double* ysweep = nullptr;  // the blocked band solve's rows between its two sweeps [V][piv_stride]
  float *band32 = nullptr, *IC32 = nullptr;  // FP32 copies of the factors (mixed precision applications)
  bool fp32 = false;                          // this call's applications stream the FP32 copies
  int32_t *piv, *icpiv, *bad, *flags, *list;
  unsigned long long* berr;
  uint8_t* mask;  // variants a launch works on
  std::vector<uint8_t> have;  // factors exist, per variant
  // counters
  int64_t solves = 0, refactors = 0, refines = 0, max_passes = 0, failed = 0, launches = 0, fallbacks = 0;
  // the untorn instance of the same topology (the fallback solver), built on first use
  ks_torn* untorn = nullptr;
  bool is_untorn = false, untorn_failed = false;
  // device time per phase (refactor, apply, load, residual): event pairs summed at the end of a call
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> marks;
  double phase_ms[4] = {0, 0, 0, 0};
  cudaEvent_t ev() {
    if (ev_used == ev_pool.size()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      ev_pool.push_back(e);
    }
    return ev_pool[ev_used++];
  }
  void mark_begin(int ph, cudaEvent_t* b) { *b = ev(); cudaEventRecord(*b, st); (void)ph; }
  void mark_end(int ph, cudaEvent_t b) {
    cudaEvent_t e = ev();
    cudaEventRecord(e, st);
    marks.push_back({ph, {b, e}});
  }
  void collect() {  // after a stream synchronisation
    for (auto& m : marks) {
      float ms = 0;
      if (cudaEventElapsedTime(&ms, m.second.first, m.second.second) == cudaSuccess) phase_ms[m.first] += ms;
    }
    marks.clear();
    ev_used = 0;
  }
  KPlan view() const {
    KPlan p;
    p.n = hp.n; p.n_elem = hp.n_elem; p.n_values = hp.n_values; p.n_derived = hp.n_derived;
    p.n_state = hp.n_state; p.n_nodes = hp.n_nodes; p.n_nonlin = hp.n_nonlin; p.n_reactive = hp.n_reactive;
    p.elem = d_elem; p.is_v = d_isv;
    return p;
  }
  ~ks_torn() {
    delete untorn;
    for (auto e : ev_pool) cudaEventDestroy(e);
    for (void* p : owned) cudaFree(p);
    if (own) cudaStreamDestroy(own);
  }
};

namespace {

int ck(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return KS_OK;
  set_error(std::string("ks_torn: ") + what + ": " + cudaGetErrorString(e));
  return KS_ECUDA;
}

// Every stamp position of every element (the pattern of J), as the device loads add them.
void stamp_pattern(const ksh::HostPlan& hp, std::vector<std::vector<int>>& rows) {
  auto add = [&](int i, int j) { if (i >= 0 && j >= 0) rows[i].push_back(j); };
  auto block = [&](const int* u, int k) { for (int a = 0; a < k; a++) for (int b = 0; b < k; b++) add(u[a], u[b]); };
  for (const KElem& e : hp.elem) {
    const int* u = e.u;
    switch (e.kind) {
      case KS_ELEM_R: case KS_ELEM_C: case KS_ELEM_CN: block(u, 2); break;
      case KS_ELEM_V: case KS_ELEM_L: case KS_ELEM_LN:
        add(u[0], u[2]); add(u[1], u[2]); add(u[2], u[0]); add(u[2], u[1]); add(u[2], u[2]); break;
      case KS_ELEM_D: block(u, 3); break;
      case KS_ELEM_Q: block(u, 9); break;
      case KS_ELEM_M: block(u, 6); break;
      case KS_ELEM_E: case KS_ELEM_H:  // device/controlled.go:83-100
        add(u[0], u[2]); add(u[1], u[2]); add(u[2], u[0]); add(u[2], u[1]); add(u[2], u[3]);
        if (e.kind == KS_ELEM_E) add(u[2], u[4]);
        break;
      case KS_ELEM_G: add(u[0], u[3]); add(u[0], u[4]); add(u[1], u[3]); add(u[1], u[4]); break;
      case KS_ELEM_F: add(u[0], u[3]); add(u[1], u[3]); break;
      case KS_ELEM_K: add(u[0], u[1]); add(u[1], u[0]); break;  // device/mutual.go:110-113
      // an abrupt switch's conductance (device/switch.go:204-211); the plan has no
      // values, so a smooth switch's transconductance is not in it (the torn
      // engine itself takes no switches)
      case KS_ELEM_S: case KS_ELEM_W: block(u, 2); break;
      default: break;
    }
  }
  for (int i = 0; i < hp.n; i++) add(i, i);
}

// Staging of a band solve: CH columns a block, NB blocks in shared memory.  FP32
// factors take twice the blocks in the same space, so the sweep runs further
// ahead of its loads; KS_TORN_BAND="CH,NB" picks another of the built shapes.
struct BandCfg { int ch, nb; };
constexpr BandCfg kBandShapes[] = {{4, 4}, {4, 6}, {8, 3}, {8, 4}, {2, 8}, {4, 8}, {8, 6}};
BandCfg band_cfg(bool fp32) {
  BandCfg d = fp32 ? BandCfg{8, 3} : BandCfg{4, 4};  // measured best at 64 variants of the 256 x 256 grid
  if (const char* e = getenv("KS_TORN_BAND")) {
    int c = 0, b = 0;
    if (sscanf(e, "%d,%d", &c, &b) == 2)
      for (const BandCfg& k : kBandShapes)
        if (k.ch == c && k.nb == b) return k;
  }
  return d;
}

// Dynamic shared memory of a band solve with elements of `es` bytes: the
// right-hand side of the largest piece, NB x CH staged columns, their pivots.
size_t band_smem(const ks_torn* T, size_t es, BandCfg c) {
  return es * (((size_t)T->max_piece + 1) & ~(size_t)1) + es * (size_t)c.nb * c.ch * (size_t)T->max_colw +
         sizeof(int) * (size_t)c.nb * c.ch;
}
size_t torn_solve_smem(const ks_torn* T) {
  return std::max(band_smem(T, sizeof(double), band_cfg(false)), band_smem(T, sizeof(float), band_cfg(true)));
}

// The blocked band solve (k_tl_band_solve_rw): register window of NS = (32 +
// the widest lower or upper band) / 32 slots going forward, 2 NS - 1 coming
// back, for bands up to 160 wide; chunks of 8 columns, RW_NBUF deep (the
// shared memory holds only the staged columns).
constexpr int kRwSC = 8, kRwMaxNS = 5;
int rw_nbuf() {
  const char* e = getenv("KS_TORN_RW_NBUF");
  const int nb = e ? atoi(e) : 3;
  return nb == 2 || nb == 4 ? nb : 3;
}
int rw_slots(const ks_torn* T) { return std::max(2, (32 + T->max_klu + 31) / 32); }
size_t rw_smem(const ks_torn* T, size_t es, int nbuf) {
  const int nsu = 2 * rw_slots(T) - 1;  // the backward rows are the wider ones
  return es * (size_t)nbuf * kRwSC * (32 * nsu + 32) + es * nbuf * kRwSC + sizeof(int) * (size_t)nbuf * kRwSC;
}
template <typename F>
using BandSolveRwFn = void (*)(const PieceD*, int64_t, int64_t, const F*, int64_t, const int32_t*, const int32_t*,
                               const double*, const double*, const double*, const int32_t*, const double*, double*, F*,
                               const uint8_t*, int);
template <typename F, int NS>
BandSolveRwFn<F> rw_fn_ns(int nbuf) {
  switch (nbuf) {
    case 2: return k_tl_band_solve_rw<F, NS, 2 * NS - 1, kRwSC, 2>;
    case 4: return k_tl_band_solve_rw<F, NS, 2 * NS - 1, kRwSC, 4>;
    default: return k_tl_band_solve_rw<F, NS, 2 * NS - 1, kRwSC, 3>;
  }
}
template <typename F>
BandSolveRwFn<F> rw_fn(int ns, int nbuf, size_t smem) {
  BandSolveRwFn<F> f = nullptr;
  switch (ns) {
    case 2: f = rw_fn_ns<F, 2>(nbuf); break;
    case 3: f = rw_fn_ns<F, 3>(nbuf); break;
    case 4: f = rw_fn_ns<F, 4>(nbuf); break;
    case 5: f = rw_fn_ns<F, 5>(nbuf); break;
    default: return nullptr;
  }
  if (smem > 48 * 1024) cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  return f;
}

// The kernel instance of a band-solve shape (its shared memory opted in once).
template <typename F>
using BandSolveFn = void (*)(const PieceD*, int64_t, int64_t, const F*, int64_t, const int32_t*, const int32_t*,
                             const double*, const double*, const double*, const int32_t*, const double*, double*,
                             const uint8_t*, int, int);
template <typename F>
BandSolveFn<F> band_solve_fn(BandCfg c, size_t smem) {
  BandSolveFn<F> f = nullptr;
  if (c.ch == 4 && c.nb == 4) f = k_tl_band_solve<F, 4, 4>;
  else if (c.ch == 4 && c.nb == 6) f = k_tl_band_solve<F, 4, 6>;
  else if (c.ch == 8 && c.nb == 3) f = k_tl_band_solve<F, 8, 3>;
  else if (c.ch == 8 && c.nb == 4) f = k_tl_band_solve<F, 8, 4>;
  else if (c.ch == 2 && c.nb == 8) f = k_tl_band_solve<F, 2, 8>;
  else if (c.ch == 4 && c.nb == 8) f = k_tl_band_solve<F, 4, 8>;
  else f = k_tl_band_solve<F, 8, 6>;
  if (smem > 48 * 1024) cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  return f;
}

int build_plan(ks_torn* T, const ks_topology* topo, const int32_t* torn, int n_torn, std::string* err,
               bool to_device = true) {
  const ksh::HostPlan& hp = T->hp;
  const int n = hp.n;
  T->n = n;
  // J's pattern, rows sorted
  std::vector<std::vector<int>> rows(n);
  stamp_pattern(hp, rows);
  T->rp.assign(n + 1, 0);
  T->ci.clear();
  for (int i = 0; i < n; i++) {
    auto& r = rows[i];
    std::sort(r.begin(), r.end());
    r.erase(std::unique(r.begin(), r.end()), r.end());
    T->rp[i] = (int)T->ci.size();
    T->ci.insert(T->ci.end(), r.begin(), r.end());
  }
  T->rp[n] = (int)T->ci.size();
  T->nnz = (int)T->ci.size();
  // the torn node pairs (tearTerminals, kron/jacobian.go:196-232)
  std::vector<std::pair<int, int>> cuts;
  std::vector<char> seen(hp.n_elem, 0);
  for (int k = 0; k < n_torn; k++) {
    const int e = torn[k];
    if (e < 0 || e >= hp.n_elem) { *err = "kron: unsupported: no element " + std::to_string(e); return KS_EINVAL; }
    if (seen[e]) { *err = "kron: unsupported: element " + std::to_string(e) + " is torn twice"; return KS_EINVAL; }
    seen[e] = 1;
    const ks_element& el = hp.src[e];
    if (el.kind == KS_ELEM_V || el.kind == KS_ELEM_L || el.kind == KS_ELEM_E || el.kind == KS_ELEM_F ||
        el.kind == KS_ELEM_H || el.kind == KS_ELEM_K || el.kind == KS_ELEM_W || el.kind == KS_ELEM_LN) {  // tearTerminals, kron/jacobian.go:143-147
      *err = "kron: unsupported: tearing element " + std::to_string(e) +
             ": its coupling runs through a branch-current unknown; tear a neighbouring element";
      return KS_EINVAL;
    }
    const int nn = el.kind == KS_ELEM_Q || el.kind == KS_ELEM_M || el.kind == KS_ELEM_G || el.kind == KS_ELEM_S ? 4 : 2;
    std::vector<int> terms;
    for (int a = 0; a < nn; a++)
      if (el.node[a] != 0 && std::find(terms.begin(), terms.end(), el.node[a]) == terms.end()) terms.push_back(el.node[a]);
    if (terms.size() < 2) {
      *err = "kron: unsupported: tearing element " + std::to_string(e) + ": it connects to ground, so tearing it separates nothing";
      return KS_EINVAL;
    }
    for (size_t x = 0; x < terms.size(); x++)
      for (size_t y = x + 1; y < terms.size(); y++) cuts.push_back({terms[x] - 1, terms[y] - 1});
  }
  std::vector<char> cutmark(T->nnz, 0);
  auto find_slot = [&](int i, int j) {
    auto b = T->ci.begin() + T->rp[i], e = T->ci.begin() + T->rp[i + 1];
    auto it = std::lower_bound(b, e, j);
    return (it != e && *it == j) ? (int)(it - T->ci.begin()) : -1;
  };
  for (auto& c : cuts) {
    int s = find_slot(c.first, c.second);
    if (s >= 0) cutmark[s] = 1;
    s = find_slot(c.second, c.first);
    if (s >= 0) cutmark[s] = 1;
  }
  // pieces: union-find over the pattern without the torn pairs (buildPlan)
  std::vector<int> parent(n);
  for (int i = 0; i < n; i++) parent[i] = i;
  auto findr = [&](int i) { while (parent[i] != i) { parent[i] = parent[parent[i]]; i = parent[i]; } return i; };
  for (int i = 0; i < n; i++)
    for (int s = T->rp[i]; s < T->rp[i + 1]; s++) {
      const int j = T->ci[s];
      if (i == j || cutmark[s]) continue;
      int a = findr(i), b = findr(j);
      if (a != b) { if (a < b) parent[b] = a; else parent[a] = b; }
    }
  std::vector<int> root(n, -1), pieceOf(n);
  std::vector<std::vector<int>> members;
  for (int i = 0; i < n; i++) {
    const int r = findr(i);
    if (root[r] < 0) { root[r] = (int)members.size(); members.emplace_back(); }
    pieceOf[i] = root[r];
    members[root[r]].push_back(i);
  }
  const int P = (int)members.size();
  T->P = P;
  // in-piece adjacency (symmetrised) for the band order
  std::vector<std::vector<int>> adj(n);
  std::vector<uint8_t> slot_in(T->nnz, 0);
  for (int i = 0; i < n; i++)
    for (int s = T->rp[i]; s < T->rp[i + 1]; s++) {
      const int j = T->ci[s];
      if (pieceOf[i] != pieceOf[j]) continue;
      slot_in[s] = 1;
      if (i != j) { adj[i].push_back(j); adj[j].push_back(i); }
    }
  for (auto& a : adj) { std::sort(a.begin(), a.end()); a.erase(std::unique(a.begin(), a.end()), a.end()); }
  T->pieces.assign(P, HostPiece());
  std::vector<int> plocal(n, -1), tmp_local(n, -1);
  for (int p = 0; p < P; p++) {
    auto& m = members[p];
    for (size_t k = 0; k < m.size(); k++) tmp_local[m[k]] = (int)k;
    T->pieces[p].idx = rcm(m, adj, tmp_local);
    for (int g : m) tmp_local[g] = -1;
    for (size_t k = 0; k < T->pieces[p].idx.size(); k++) plocal[T->pieces[p].idx[k]] = (int)k;
  }
  // bands, in-piece slots, coupling rows / columns
  std::vector<int> row_a(n, -1), rows_list;
  std::vector<int> cc_local(n, -1);
  std::vector<int> offp, offs;
  std::vector<std::vector<int>> off_of_row(n);
  for (int i = 0; i < n; i++)
    for (int s = T->rp[i]; s < T->rp[i + 1]; s++) {
      const int j = T->ci[s];
      HostPiece& pi = T->pieces[pieceOf[i]];
      if (slot_in[s]) {
        const int d = plocal[i] - plocal[j];
        if (d > 0) pi.kl = std::max(pi.kl, d); else pi.ku = std::max(pi.ku, -d);
        pi.slots.push_back(s);
        continue;
      }
      if (row_a[i] < 0) { row_a[i] = (int)rows_list.size(); rows_list.push_back(i); pi.ports.push_back(i); }
      off_of_row[i].push_back(s);
      HostPiece& pj = T->pieces[pieceOf[j]];
      if (cc_local[j] < 0) { cc_local[j] = (int)pj.cc.size(); pj.cc.push_back(j); }
    }
  T->R = (int)rows_list.size();
  offp.push_back(0);
  for (int a = 0; a < T->R; a++) {
    for (int s : off_of_row[rows_list[a]]) offs.push_back(s);
    offp.push_back((int)offs.size());
  }
  std::vector<int32_t> slot_cc(T->nnz, -1);
  for (int s : offs) slot_cc[s] = cc_local[T->ci[s]];
  // per-piece device descriptors
  std::vector<PieceD> pcs(P);
  std::vector<int32_t> pidx, port_a, ports_g, cc_g, pslot, pli, plj;
  int64_t band = 0, wc = 0, y = 0;
  for (int p = 0; p < P; p++) {
    HostPiece& h = T->pieces[p];
    PieceD& d = pcs[p];
    d.n = (int)h.idx.size(); d.kl = h.kl; d.ku = h.ku; d.ldab = (2 * h.kl + h.ku + 2) & ~1;  // even: aligned columns
    d.band_off = band; band += (int64_t)d.ldab * d.n;
    d.idx_off = (int)pidx.size();
    pidx.insert(pidx.end(), h.idx.begin(), h.idx.end());
    d.port_off = (int)ports_g.size(); d.nports = (int)h.ports.size();
    for (int g : h.ports) { ports_g.push_back(g); port_a.push_back(row_a[g]); }
    d.cc_off = (int)cc_g.size(); d.ncc = (int)h.cc.size();
    cc_g.insert(cc_g.end(), h.cc.begin(), h.cc.end());
    d.wc_off = wc; wc += (int64_t)d.ncc * d.nports;
    d.y_off = y; y += (int64_t)d.n * d.nports;
    d.pslot_off = (int)pslot.size(); d.npslot = (int)h.slots.size();
    for (int s : h.slots) {
      int i = (int)(std::upper_bound(T->rp.begin(), T->rp.end(), s) - T->rp.begin()) - 1;
      pslot.push_back(s); pli.push_back(plocal[i]); plj.push_back(plocal[T->ci[s]]);
    }
    T->max_piece = std::max(T->max_piece, d.n);
    T->max_colw = std::max(T->max_colw, std::max(d.kl, d.kl + d.ku + 1));
    T->max_band = std::max(T->max_band, d.kl + d.ku);
    T->max_klu = std::max(T->max_klu, std::max(d.kl, d.ku));
    if (d.n > 12000) { *err = "ks_torn: a piece of " + std::to_string(d.n) + " unknowns (the band solve holds at most 12,000)"; return KS_EUNSUPPORTED; }
  }
  T->band_stride = band; T->piv_stride = n; T->wc_stride = wc; T->y_stride = y;
  if (torn_solve_smem(T) > 227 * 1024) {
    *err = "ks_torn: a piece of " + std::to_string(T->max_piece) + " unknowns with a band of " +
           std::to_string(T->max_band) + " does not fit the band solve's shared memory";
    return KS_EUNSUPPORTED;
  }
  if (T->R > 6000) { *err = "ks_torn: " + std::to_string(T->R) + " coupling rows (the interconnection solve holds at most 6,000)"; return KS_EUNSUPPORTED; }
  // CSC of the in-piece slots (column equilibration)
  std::vector<int32_t> cp(n + 1, 0), cslot, crow;
  for (int s = 0; s < T->nnz; s++) if (slot_in[s]) cp[T->ci[s] + 1]++;
  for (int j = 0; j < n; j++) cp[j + 1] += cp[j];
  cslot.assign(cp[n], 0); crow.assign(cp[n], 0);
  std::vector<int> nxt(cp.begin(), cp.end() - 1);
  for (int i = 0; i < n; i++)
    for (int s = T->rp[i]; s < T->rp[i + 1]; s++)
      if (slot_in[s]) { const int q = nxt[T->ci[s]]++; cslot[q] = s; crow[q] = i; }
  std::vector<int32_t> nonlin;
  for (int e = 0; e < hp.n_elem; e++) {
    const int k = hp.elem[e].kind;
    if (k == KS_ELEM_D || k == KS_ELEM_Q || k == KS_ELEM_M || k == KS_ELEM_S || k == KS_ELEM_W ||
        ((k == KS_ELEM_CN || k == KS_ELEM_LN) && hp.elem[e].level > 0))  // the curved laws
      nonlin.push_back(e);
  }
  T->n_nonlin = (int)nonlin.size();
  T->h_pieceOf = pieceOf;
  T->h_rows = rows_list;
  if (!to_device) return KS_OK;
  auto& o = T->owned;
  std::vector<int32_t> rp32(T->rp.begin(), T->rp.end()), ci32(T->ci.begin(), T->ci.end()), pof(pieceOf.begin(), pieceOf.end());
  std::vector<int32_t> pl(plocal.begin(), plocal.end()), ra(row_a.begin(), row_a.end());
  std::vector<int32_t> offp32(offp.begin(), offp.end()), offs32(offs.begin(), offs.end());
  std::vector<KElem> el(hp.elem.begin(), hp.elem.end());
  std::vector<int8_t> isv(hp.is_v.begin(), hp.is_v.end());
  bool ok = upload(&T->d_elem, el, o) && upload(&T->d_isv, isv, o) && upload(&T->d_rp, rp32, o) &&
            upload(&T->d_ci, ci32, o) && upload(&T->d_cp, cp, o) && upload(&T->d_cslot, cslot, o) &&
            upload(&T->d_crow, crow, o) && upload(&T->d_pidx, pidx, o) && upload(&T->d_plocal, pl, o) &&
            upload(&T->d_row_a, ra, o) && upload(&T->d_offp, offp32, o) && upload(&T->d_offs, offs32, o) &&
            upload(&T->d_pieceOf, pof, o) && upload(&T->d_slot_cc, slot_cc, o) && upload(&T->d_port_a, port_a, o) &&
            upload(&T->d_ports_g, ports_g, o) && upload(&T->d_cc_g, cc_g, o) && upload(&T->d_pslot, pslot, o) &&
            upload(&T->d_pli, pli, o) && upload(&T->d_plj, plj, o) && upload(&T->d_nonlin, nonlin, o) &&
            upload(&T->d_slot_in, slot_in, o) && upload(&T->d_pcs, pcs, o);
  if (!ok) { *err = "ks_torn: device allocation for the plan failed"; return KS_ENOMEM; }
  return KS_OK;
}

int alloc_numeric(ks_torn* T) {
  const int64_t V = T->V, n = T->n;
  auto& o = T->owned;
  const ksh::HostPlan& hp = T->hp;
  T->values = dalloc<double>((size_t)hp.n_values * V, o);
  T->derived = dalloc<double>((size_t)(hp.n_derived + 1) * V, o);
  T->state = dalloc<double>((size_t)(hp.n_state + 1) * V, o);
  T->x = dalloc<double>(n * V, o); T->xo = dalloc<double>(n * V, o);
  T->J = dalloc<double>((size_t)T->nnz * V, o); T->rhs = dalloc<double>(n * V, o);
  T->r = dalloc<double>(n * V, o); T->dx = dalloc<double>(n * V, o); T->z = dalloc<double>(n * V, o);
  T->rs = dalloc<double>(n * V, o); T->cs = dalloc<double>(n * V, o);
  T->band = dalloc<double>((size_t)T->band_stride * V, o);
  T->band32 = dalloc<float>((size_t)T->band_stride * V, o);
  T->piv = dalloc<int32_t>((size_t)T->piv_stride * V, o);
  T->ysweep = dalloc<double>((size_t)T->piv_stride * V, o);
  T->Y = dalloc<double>((size_t)T->y_stride * V, o);
  T->Wc = dalloc<double>((size_t)T->wc_stride * V, o);
  T->IC = dalloc<double>((size_t)T->R * T->R * V, o);
  T->IC32 = dalloc<float>((size_t)T->R * T->R * V, o);
  T->icpiv = dalloc<int32_t>((size_t)T->R * V, o);
  T->h = dalloc<double>((size_t)T->R * V, o); T->w = dalloc<double>((size_t)T->R * V, o);
  T->bad = dalloc<int32_t>(V, o); T->flags = dalloc<int32_t>(V, o);
  T->berr = dalloc<unsigned long long>(V, o);
  T->mask = dalloc<uint8_t>(V, o);
  T->list = dalloc<int32_t>(V, o);
  T->have.assign(V, 0);
  for (void* p : {(void*)T->values, (void*)T->derived, (void*)T->state, (void*)T->x, (void*)T->xo, (void*)T->J,
                  (void*)T->rhs, (void*)T->r, (void*)T->dx, (void*)T->z, (void*)T->rs, (void*)T->cs, (void*)T->band,
                  (void*)T->piv, (void*)T->ysweep, (void*)T->Y, (void*)T->Wc, (void*)T->IC, (void*)T->icpiv, (void*)T->h, (void*)T->w,
                  (void*)T->bad, (void*)T->flags, (void*)T->berr, (void*)T->mask,
                  (void*)T->list, (void*)T->band32, (void*)T->IC32})
    if (!p) { set_error("ks_torn: device allocation failed"); return KS_ENOMEM; }
  return KS_OK;
}

int set_mask(ks_torn* T, const std::vector<uint8_t>& m) {
  return ck(cudaMemcpyAsync(T->mask, m.data(), m.size(), cudaMemcpyHostToDevice, T->st), "mask");
}

// Factors of the listed variants at their current J.
int refactor(ks_torn* T, const std::vector<int32_t>& list) {
  const int64_t V = T->V, n = T->n;
  const int R = T->R;
  cudaStream_t s = T->st;
  if (list.empty()) return KS_OK;
  T->refactors++;
  cudaEvent_t e0;
  T->mark_begin(0, &e0);
  std::vector<uint8_t> m(V, 0);
  for (int v : list) m[v] = 1;
  int rc = set_mask(T, m);
  if (rc) return rc;
  if (ck(cudaMemsetAsync(T->bad, 0, sizeof(int32_t) * V, s), "memset")) return KS_ECUDA;
  T->launches++;
  k_tl_equil_rows<<<blocks_for(n * V, 256), 256, 0, s>>>(n, V, T->d_rp, T->d_slot_in, T->J, T->rs, T->bad, T->mask);
  T->launches++;
  k_tl_equil_cols<<<blocks_for(n * V, 256), 256, 0, s>>>(n, V, T->d_cp, T->d_cslot, T->d_crow, T->J, T->rs, T->cs,
                                                         T->bad, T->mask);
  const unsigned grid = (unsigned)(V * T->P);
  T->launches++;
  k_tl_band_fill<<<grid, 256, 0, s>>>(T->d_pcs, T->P, V, T->band_stride, T->band, T->d_pslot, T->d_pli, T->d_plj,
                                      T->d_pidx, T->J, T->rs, T->cs, T->mask);
  T->launches++;
  k_tl_band_lu<<<grid, 256, 0, s>>>(T->d_pcs, V, T->band_stride, T->band, T->piv_stride, T->piv, T->bad, T->mask);
  if (R > 0) {
    T->launches++;
    k_tl_wc<<<grid, 256, 0, s>>>(T->d_pcs, V, T->band_stride, T->band, T->piv_stride, T->piv, T->d_pidx, T->d_plocal,
                                 T->d_ports_g, T->d_cc_g, T->rs, T->cs, T->y_stride, T->Y, T->wc_stride, T->Wc, T->mask);
    const int64_t per = (int64_t)R * R;
    T->launches++;
    k_tl_zero_ic<<<blocks_for(per * V, 256), 256, 0, s>>>(per, V, T->IC, T->mask);
    T->launches++;
    k_tl_ic_build<<<blocks_for((int64_t)R * V, 128), 128, 0, s>>>(R, V, T->d_offp, T->d_offs, T->d_ci, T->d_pieceOf,
                                                                  T->d_slot_cc, T->d_pcs, T->d_port_a, T->J,
                                                                  T->wc_stride, T->Wc, T->IC, T->mask);
    if (ck(cudaMemcpyAsync(T->list, list.data(), sizeof(int32_t) * list.size(), cudaMemcpyHostToDevice, s), "list"))
      return KS_ECUDA;
    const int count = (int)list.size();
    const int nb = KS_IC_TILE;
    for (int k0 = 0; k0 < R; k0 += nb) {
      const int jb = std::min(nb, R - k0);
      T->launches++;
      k_tl_ic_panel<<<(unsigned)V, 1024, 0, s>>>(R, k0, jb, T->IC, T->icpiv, T->bad, T->mask);
      T->launches++;
      k_tl_ic_swap<<<blocks_for((int64_t)R * V, 256), 256, 0, s>>>(R, k0, jb, T->IC, T->icpiv, V, T->mask);
      const int rest = R - k0 - jb;
      if (rest <= 0) continue;
      T->launches++;
      k_tl_ic_trsm<<<blocks_for((int64_t)rest * V, 128), 128, 0, s>>>(R, k0, jb, T->IC, V, T->mask);
      T->launches++;
      const unsigned tiles = (unsigned)((rest + KS_IC_TILE - 1) / KS_IC_TILE);
      k_tl_ic_gemm<<<dim3(tiles, tiles, (unsigned)count), 256, 0, s>>>(R, k0, jb, T->IC, T->list);
    }
    T->launches++;
    k_tl_ic_finish<<<blocks_for((int64_t)R * R * V, 256), 256, 0, s>>>(R, V, T->IC, T->IC32, T->mask);
  }
  T->launches++;  // after the port columns: the bands' reciprocal diagonals and FP32 copies
  k_tl_band_finish<<<grid, 256, 0, s>>>(T->d_pcs, V, T->band_stride, T->band, T->band32, T->mask);
  if (ck(cudaGetLastError(), "refactor launch")) return KS_ECUDA;
  T->mark_end(0, e0);
  for (int v : list) T->have[v] = 1;
  return KS_OK;
}

int apply_(ks_torn* T, const double* b, double* out);
int untorn_solve(ks_torn* T, const std::vector<uint8_t>& want, std::vector<uint8_t>* ok);

// out = M^-1 b with the current factors, for the masked variants.
int apply(ks_torn* T, const double* b, double* out) {
  cudaEvent_t e0;
  T->mark_begin(1, &e0);
  int rc = apply_(T, b, out);
  T->mark_end(1, e0);
  return rc;
}

int apply_(ks_torn* T, const double* b, double* out) {
  const int64_t V = T->V;
  const int R = T->R;
  cudaStream_t s = T->st;
  const unsigned grid = (unsigned)(V * T->P);
  const int bt = 32;  // one warp per (variant, piece)
  // the band solves: FP32 factors under mixed precision, else FP64
  const int ns = rw_slots(T);  // 2 .. kRwMaxNS: the blocked solve has an instance
  const char* rwe = getenv("KS_TORN_RW");  // "0": the column-by-column solve
  const bool rw = ns <= kRwMaxNS && !(rwe && atoi(rwe) == 0);
  auto band_solve = [&](const double* w, double* o) {
    T->launches++;
    if (rw) {  // the blocked solve
      const int nbuf = rw_nbuf();
      if (T->fp32) {
        const size_t sm = rw_smem(T, sizeof(float), nbuf);
        if (auto f = rw_fn<float>(ns, nbuf, sm)) {
          f<<<grid, bt, sm, s>>>(T->d_pcs, V, T->band_stride, T->band32, T->piv_stride, T->piv, T->d_pidx, T->rs,
                                 T->cs, b, T->d_row_a, w, o, reinterpret_cast<float*>(T->ysweep), T->mask,
                                 T->max_colw);
          return;
        }
      } else {
        const size_t sm = rw_smem(T, sizeof(double), nbuf);
        if (auto f = rw_fn<double>(ns, nbuf, sm)) {
          f<<<grid, bt, sm, s>>>(T->d_pcs, V, T->band_stride, T->band, T->piv_stride, T->piv, T->d_pidx, T->rs,
                                 T->cs, b, T->d_row_a, w, o, T->ysweep, T->mask, T->max_colw);
          return;
        }
      }
    }
    if (T->fp32) {
      const BandCfg c = band_cfg(true);
      const size_t sm = band_smem(T, sizeof(float), c);
      band_solve_fn<float>(c, sm)<<<grid, bt, sm, s>>>(T->d_pcs, V, T->band_stride, T->band32, T->piv_stride, T->piv,
                                                        T->d_pidx, T->rs, T->cs, b, T->d_row_a, w, o, T->mask,
                                                        T->max_piece, T->max_colw);
    } else {
      const BandCfg c = band_cfg(false);
      const size_t sm = band_smem(T, sizeof(double), c);
      band_solve_fn<double>(c, sm)<<<grid, bt, sm, s>>>(T->d_pcs, V, T->band_stride, T->band, T->piv_stride, T->piv,
                                                         T->d_pidx, T->rs, T->cs, b, T->d_row_a, w, o, T->mask,
                                                         T->max_piece, T->max_colw);
    }
  };
  if (R == 0) {
    band_solve(nullptr, out);
    return ck(cudaGetLastError(), "apply");
  }
  band_solve(nullptr, T->z);
  T->launches++;
  k_tl_h<<<blocks_for((int64_t)R * V, 256), 256, 0, s>>>(R, V, T->d_offp, T->d_offs, T->d_ci, T->J, T->z, T->h, T->mask);
  T->launches++;
  if (T->fp32)
    k_tl_ic_solve<float><<<(unsigned)V, 512, (sizeof(float) + sizeof(int)) * R, s>>>(R, V, T->IC32, T->icpiv, T->h,
                                                                                     T->w, T->mask);
  else
    k_tl_ic_solve<double><<<(unsigned)V, 512, (sizeof(double) + sizeof(int)) * R, s>>>(R, V, T->IC, T->icpiv, T->h,
                                                                                       T->w, T->mask);
  band_solve(T->w, out);
  return ck(cudaGetLastError(), "apply");
}

// J x = rhs for the variants in `want` (x receives the solution): apply, then
// refinement against J (kron/jacobian.go:508-589).  ok[v] = 1 when accepted.
// With reuse, factors made at an earlier J serve while the refinement
// converges on them; a variant whose solve is not accepted is refactored at its
// current J and solved once more (kron/jacobian.go:404-411).
int torn_solve(ks_torn* T, const std::vector<uint8_t>& want, bool reuse, std::vector<uint8_t>* ok) {
  const int64_t V = T->V, n = T->n;
  cudaStream_t s = T->st;
  std::vector<uint8_t> cur = want;
  ok->assign(V, 0);
  for (int attempt = 0; attempt < 2; attempt++) {
    std::vector<int32_t> need;
    for (int64_t v = 0; v < V; v++)
      if (cur[v] && (!T->have[v] || !reuse || attempt == 1)) need.push_back((int32_t)v);
    int rc = refactor(T, need);
    if (rc) return rc;
    if ((rc = set_mask(T, cur)) || (rc = apply(T, T->rhs, T->x))) return rc;
    std::vector<unsigned long long> be(V);
    std::vector<double> prev(V, INFINITY);
    std::vector<uint8_t> refine = cur;
    int pass = 0;
    for (;; pass++) {
      if ((rc = set_mask(T, refine))) return rc;
      if ((rc = ck(cudaMemsetAsync(T->berr, 0, sizeof(unsigned long long) * V, s), "memset"))) return rc;
      cudaEvent_t e0;
      T->mark_begin(3, &e0);
      T->launches++;
      k_tl_resid<<<blocks_for(n * V, 256), 256, 0, s>>>((int)n, V, T->d_rp, T->d_ci, T->J, T->rhs, T->x, T->r, T->berr,
                                                        T->mask);
      T->mark_end(3, e0);
      if ((rc = ck(cudaMemcpyAsync(be.data(), T->berr, sizeof(unsigned long long) * V, cudaMemcpyDeviceToHost, s), "berr")))
        return rc;
      if ((rc = ck(cudaStreamSynchronize(s), "sync"))) return rc;
      T->collect();
      bool any = false;
      for (int64_t v = 0; v < V; v++) {
        if (!refine[v]) continue;
        double e;
        memcpy(&e, &be[v], sizeof e);
        // stop at 1e-14, after 12 passes, or when a pass no longer halves the
        // error (stale factors too far from J: a refactor follows)
        const bool stalled = pass >= 2 && e > 0.5 * prev[v];
        prev[v] = e;
        if (e <= 1e-14 || pass == 12 || stalled) {
          refine[v] = 0;
          if (e <= 1e-12) (*ok)[v] = 1;
        } else {
          any = true;
        }
      }
      if (!any) break;
      if ((rc = set_mask(T, refine)) || (rc = apply(T, T->r, T->dx))) return rc;
      T->launches++;
      k_tl_axpy_masked<<<blocks_for(n * V, 256), 256, 0, s>>>(n, V, T->dx, T->x, T->mask);
      T->refines++;
    }
    T->max_passes = std::max<int64_t>(T->max_passes, pass);
    T->solves++;
    bool all_ok = true;
    for (int64_t v = 0; v < V; v++)
      if (cur[v] && !(*ok)[v]) all_ok = false;
    if (all_ok) return KS_OK;
    if (!reuse) break;  // fresh factors already
    for (int64_t v = 0; v < V; v++) cur[v] = cur[v] && !(*ok)[v];
  }
  for (int64_t v = 0; v < V; v++)
    if (want[v] && !(*ok)[v]) T->failed++;
  if (T->is_untorn) return KS_OK;
  // not accepted torn, even on fresh factors: the untorn LU (kron/jacobian.go:412-414)
  std::vector<uint8_t> fb(V, 0), okf;
  bool anyf = false;
  for (int64_t v = 0; v < V; v++) { fb[v] = want[v] && !(*ok)[v]; anyf = anyf || fb[v]; }
  if (!anyf) return KS_OK;
  int rc = untorn_solve(T, fb, &okf);
  if (rc) return rc;
  for (int64_t v = 0; v < V; v++) if (okf[v]) (*ok)[v] = 1;
  return KS_OK;
}

// The untorn instance of T's topology: every unknown in the band piece of its
// connected component, no coupling rows (buildPlan of an empty tearing), its own
// factors and vectors for T's variants, on T's stream.  Null when a component is
// too large for a band piece (those variants then keep their failed status).
ks_torn* untorn_of(ks_torn* T) {
  if (T->untorn || T->untorn_failed || T->is_untorn) return T->untorn;
  ks_torn* U = new ks_torn();
  U->hp = T->hp;
  U->V = T->V;
  U->is_untorn = true;
  ks_topology topo{T->hp.n_nodes, T->hp.n_elem, T->hp.n_values, 0, T->hp.src.data()};
  std::string err;
  if (build_plan(U, &topo, nullptr, 0, &err) || alloc_numeric(U)) {
    delete U;
    T->untorn_failed = true;
    return nullptr;
  }

  U->st = T->st;
  U->fp32 = T->fp32;
  T->untorn = U;
  return U;
}

int torn_solve(ks_torn* T, const std::vector<uint8_t>& want, bool reuse, std::vector<uint8_t>* ok);

// J x = rhs untorn for the variants in `want` (kron/jacobian.go:418-434): J and
// the right-hand side go to the untorn instance, which factors afresh and
// refines against the same J; x comes back for those variants.  ok[v] = 1 when
// accepted.
int untorn_solve(ks_torn* T, const std::vector<uint8_t>& want, std::vector<uint8_t>* ok) {
  const int64_t V = T->V, n = T->n;
  ok->assign(V, 0);
  int64_t count = 0;
  for (auto w : want) count += w != 0;
  if (!count) return KS_OK;
  ks_torn* U = untorn_of(T);
  if (!U) return KS_OK;
  cudaStream_t s = T->st;
  U->st = s;
  if (ck(cudaMemcpyAsync(U->J, T->J, sizeof(double) * (size_t)T->nnz * V, cudaMemcpyDeviceToDevice, s), "untorn J") ||
      ck(cudaMemcpyAsync(U->rhs, T->rhs, sizeof(double) * n * V, cudaMemcpyDeviceToDevice, s), "untorn rhs"))
    return KS_ECUDA;
  U->have.assign(V, 0);
  const int64_t l0 = U->launches, s0 = U->solves, f0 = U->refactors, r0 = U->refines;
  std::vector<uint8_t> oku;
  int rc = torn_solve(U, want, false, &oku);
  if (rc) return rc;
  if ((rc = set_mask(U, want))) return rc;
  U->launches++;
  k_tl_copy_masked<<<blocks_for(n * V, 256), 256, 0, s>>>(n, V, U->x, T->x, U->mask);
  if ((rc = ck(cudaGetLastError(), "untorn x"))) return rc;
  for (int64_t v = 0; v < V; v++) (*ok)[v] = want[v] && oku[v];
  T->fallbacks += count;
  T->launches += U->launches - l0 + 2;
  T->solves += U->solves - s0;
  T->refactors += U->refactors - f0;
  T->refines += U->refines - r0;
  T->max_passes = std::max(T->max_passes, U->max_passes);
  return KS_OK;
}

// One Newton solve (newton(), analysis/newton.go:36-57) of every active variant.
// status[v] receives KS_STATUS_NO_CONVERGENCE / SINGULAR on failure.
int newton(ks_torn* T, LoadParams lp, const KOpts& o, int max_iter, int reuse, std::vector<int32_t>& status,
           std::vector<int32_t>& iters) {
  const int64_t V = T->V, n = T->n;
  cudaStream_t s = T->st;
  KPlan plan = T->view();
  std::vector<uint8_t> live(V, 0);
  for (int64_t v = 0; v < V; v++) live[v] = status[v] == KS_STATUS_OK;
  bool initJct = lp.initJct;
  for (int it = 0; it < max_iter; it++) {
    bool any = false;
    for (auto l : live) any = any || l;
    if (!any) return KS_OK;
    int rc = set_mask(T, live);
    if (rc) return rc;
    T->launches++;
    k_tl_copy_masked<<<blocks_for(n * V, 256), 256, 0, s>>>(n, V, T->x, T->xo, T->mask);
    if ((rc = ck(cudaMemsetAsync(T->J, 0, sizeof(double) * (size_t)T->nnz * V, s), "memset")) ||
        (rc = ck(cudaMemsetAsync(T->rhs, 0, sizeof(double) * n * V, s), "memset")))
      return rc;
    lp.initJct = initJct;
    cudaEvent_t e0;
    T->mark_begin(2, &e0);
    T->launches++;
    k_tl_load<<<blocks_for((int64_t)plan.n_elem * V, 256), 256, 0, s>>>(plan, T->values, T->derived, T->state, V, T->d_rp,
                                                                         T->d_ci, T->J, T->rhs, T->x, T->xo, lp, T->mask);
    T->mark_end(2, e0);
    std::vector<uint8_t> ok;
    if (reuse == KS_TORN_UNTORN) rc = untorn_solve(T, live, &ok);  // every system untorn
    else rc = torn_solve(T, live, reuse != 0, &ok);
    if (rc) return rc;
    for (int64_t v = 0; v < V; v++) {
      if (!live[v]) continue;
      iters[v]++;
      if (!ok[v]) { status[v] = KS_STATUS_SINGULAR; live[v] = 0; }
    }
    if (T->n_nonlin == 0) {  // linear: one solve is the answer
      return KS_OK;
    }
    if (initJct) { initJct = false; continue; }
    if ((rc = set_mask(T, live))) return rc;
    if ((rc = ck(cudaMemsetAsync(T->flags, 0, sizeof(int32_t) * V, s), "memset"))) return rc;
    T->launches++;
    k_tl_conv_x<<<blocks_for(n * V, 256), 256, 0, s>>>((int)n, V, T->d_isv, T->x, T->xo, o, T->mask, T->flags);
    T->launches++;
    k_tl_conv_elem<<<blocks_for((int64_t)T->n_nonlin * V, 256), 256, 0, s>>>(
        plan, T->values, T->derived, T->state, V, T->d_nonlin, T->n_nonlin, T->x, T->xo, o, T->mask, T->flags);
    std::vector<int32_t> fl(V);
    if ((rc = ck(cudaMemcpyAsync(fl.data(), T->flags, sizeof(int32_t) * V, cudaMemcpyDeviceToHost, s), "flags")) ||
        (rc = ck(cudaStreamSynchronize(s), "sync")))
      return rc;
    for (int64_t v = 0; v < V; v++)
      if (live[v] && fl[v] == 0) live[v] = 0;  // converged
  }
  for (int64_t v = 0; v < V; v++)
    if (live[v]) status[v] = KS_STATUS_NO_CONVERGENCE;
  return KS_OK;
}

}  // namespace

KOpts ks_kopts_from(const ks_options* o);

extern "C" int ks_torn_create(const ks_topology* topo, int32_t n_variants, const double* values, const int32_t* torn_elems,
                              int32_t n_torn, ks_torn** out) {
  if (!topo || n_variants <= 0 || !values || !out || (n_torn > 0 && !torn_elems)) {
    set_error("ks_torn_create: bad argument");
    return KS_EINVAL;
  }
  ks_torn* T = new ks_torn();
  std::string err;
  int rc = ksh::plan_layout(topo, &T->hp, &err);
  if (rc) { set_error(err); delete T; return rc; }
  for (int k = 0; k < T->hp.n_elem; k++) {
    const KElem& e = T->hp.elem[k];
    if (e.kind != KS_ELEM_S && e.kind != KS_ELEM_W) continue;
    // a smooth switch stamps its transconductance on entries the plan (made
    // without values) does not hold; the abrupt switch stamps its conductance only
    for (int v = 0; v < n_variants; v++)
      if (values[(size_t)v * T->hp.n_values + e.param + KS_SW_P_VH] < 0) {
        set_error("ks_torn_create: smooth switches (negative hysteresis) are not supported by the torn engine");
        delete T;
        return KS_EUNSUPPORTED;
      }
  }
  T->V = n_variants;
  rc = build_plan(T, topo, torn_elems, n_torn, &err);
  if (rc) { set_error(err); delete T; return rc; }
  if ((rc = alloc_numeric(T))) { delete T; return rc; }
  const size_t ic_smem = (sizeof(double) + sizeof(int)) * (size_t)T->R;
  if (ic_smem > 48 * 1024) {
    cudaFuncSetAttribute(k_tl_ic_solve<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ic_smem);
    cudaFuncSetAttribute(k_tl_ic_solve<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ic_smem);
  }
  if (cudaStreamCreateWithFlags(&T->own, cudaStreamNonBlocking) != cudaSuccess) {
    set_error("ks_torn_create: stream creation failed");
    delete T;
    return KS_ECUDA;
  }
  T->st = T->own;
  // values to [n_values][V], then the per-variant constants
  const int64_t V = n_variants;
  double* rows = nullptr;
  if (cudaMalloc(&rows, sizeof(double) * T->hp.n_values * V) != cudaSuccess) { delete T; set_error("ks_torn_create: allocation"); return KS_ENOMEM; }
  cudaMemcpyAsync(rows, values, sizeof(double) * T->hp.n_values * V, cudaMemcpyHostToDevice, T->st);
  ks_launch_transpose(rows, T->values, V, T->hp.n_values, T->st);
  KsDeviceBatch b{};
  b.plan = T->view(); b.B = V; b.values = T->values; b.derived = T->derived; b.state = T->state;
  rc = ks_launch_setup(b, 0.0, 0.0, T->st);
  cudaError_t e = cudaStreamSynchronize(T->st);
  cudaFree(rows);
  if (rc || e != cudaSuccess) { set_error(std::string("ks_torn_create: ") + cudaGetErrorString(e)); delete T; return KS_ECUDA; }
  *out = T;
  return KS_OK;
}

extern "C" int ks_torn_plan(const ks_topology* topo, const int32_t* torn_elems, int32_t n_torn, int32_t* piece_of,
                            int32_t* n_pieces, int32_t* rows, int32_t rows_cap, int32_t* n_rows, int32_t* max_piece,
                            int32_t* max_band) {
  if (!topo || (n_torn > 0 && !torn_elems)) { set_error("ks_torn_plan: bad argument"); return KS_EINVAL; }
  ks_torn T;
  std::string err;
  int rc = ksh::plan_layout(topo, &T.hp, &err);
  if (rc) { set_error(err); return rc; }
  rc = build_plan(&T, topo, torn_elems, n_torn, &err, false);
  if (rc) { set_error(err); return rc; }
  if (piece_of) for (int i = 0; i < T.n; i++) piece_of[i] = T.h_pieceOf[i];
  if (n_pieces) *n_pieces = T.P;
  if (rows) for (int a = 0; a < T.R && a < rows_cap; a++) rows[a] = T.h_rows[a];
  if (n_rows) *n_rows = T.R;
  if (max_piece) *max_piece = T.max_piece;
  if (max_band) *max_band = T.max_band;
  return KS_OK;
}

extern "C" void ks_torn_destroy(ks_torn* T) { delete T; }

extern "C" int ks_torn_set_stream(ks_torn* T, void* stream) {
  if (!T) return KS_EINVAL;
  T->st = stream ? static_cast<cudaStream_t>(stream) : T->own;
  return KS_OK;
}

extern "C" int ks_torn_info(const ks_torn* T, int32_t* n_unknowns, int32_t* n_pieces, int32_t* n_coupling_rows,
                            int32_t* max_piece, int32_t* max_band) {
  if (!T) return KS_EINVAL;
  if (n_unknowns) *n_unknowns = T->n;
  if (n_pieces) *n_pieces = T->P;
  if (n_coupling_rows) *n_coupling_rows = T->R;
  if (max_piece) *max_piece = T->max_piece;
  if (max_band) *max_band = T->max_band;
  return KS_OK;
}

namespace {

void stats_out(const ks_torn* T, int64_t* s) {
  if (!s) return;
  s[0] = T->solves; s[1] = T->refactors; s[2] = T->refines; s[3] = T->max_passes; s[4] = T->failed;
  s[5] = T->P; s[6] = T->R; s[7] = T->max_band; s[8] = T->band_stride; s[9] = T->launches;
  for (int k = 0; k < 4; k++) s[10 + k] = (int64_t)(T->phase_ms[k] * 1000.0);  // microseconds
  s[14] = T->fallbacks;
}

int fresh_state(ks_torn* T, double step, double stop) {
  const int64_t V = T->V;
  KPlan plan = T->view();
  KsDeviceBatch b{};
  b.plan = plan; b.B = V; b.values = T->values; b.derived = T->derived; b.state = T->state;
  if (ks_launch_setup(b, step, stop, T->st)) return ck(cudaGetLastError(), "setup");
  T->launches++;
  k_tl_init_state<<<blocks_for((int64_t)(plan.n_state + 1) * V, 256), 256, 0, T->st>>>(plan, T->derived, T->state, V);
  T->launches++;
  k_tl_init_mos<<<blocks_for((int64_t)plan.n_elem * V, 256), 256, 0, T->st>>>(plan, T->derived, T->state, V);
  if (ck(cudaMemsetAsync(T->x, 0, sizeof(double) * T->n * V, T->st), "memset")) return KS_ECUDA;
  T->solves = T->refactors = T->refines = T->max_passes = T->failed = T->fallbacks = 0;
  T->launches = 3;
  for (double& m : T->phase_ms) m = 0;
  T->marks.clear();
  T->ev_used = 0;
  T->have.assign(T->V, 0);
  return ck(cudaGetLastError(), "init");
}

int accept_all_variants(ks_torn* T, const std::vector<int32_t>& status, double t, int mode, double gmin) {
  std::vector<uint8_t> m(T->V);
  for (int64_t v = 0; v < T->V; v++) m[v] = status[v] == KS_STATUS_OK;
  int rc = set_mask(T, m);
  if (rc) return rc;
  KPlan plan = T->view();
  T->launches++;
  k_tl_accept<<<blocks_for((int64_t)plan.n_elem * T->V, 256), 256, 0, T->st>>>(plan, T->values, T->derived, T->state,
                                                                                T->V, T->x, t, mode, gmin, T->mask);
  return ck(cudaGetLastError(), "accept");
}

int x_out(ks_torn* T, double* out) {  // [V][n] from [n][V]
  if (!out) {
    if (ck(cudaStreamSynchronize(T->st), "sync")) return KS_ECUDA;
    T->collect();
    return KS_OK;
  }
  std::vector<double> h((size_t)T->n * T->V);
  if (ck(cudaMemcpyAsync(h.data(), T->x, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, T->st), "x") ||
      ck(cudaStreamSynchronize(T->st), "sync"))
    return KS_ECUDA;
  T->collect();
  for (int64_t v = 0; v < T->V; v++)
    for (int i = 0; i < T->n; i++) out[(size_t)v * T->n + i] = h[(size_t)i * T->V + v];
  return KS_OK;
}

}  // namespace

extern "C" int ks_torn_op(ks_torn* T, const ks_options* opt, int32_t reuse, double* out_x, int32_t* out_status,
                          int32_t* out_iters, int64_t* stats) {
  if (!T) return KS_EINVAL;
  int rc = fresh_state(T, 0.0, 0.0);
  if (rc) return rc;
  KOpts o = ks_kopts_from(opt);
  T->fp32 = o.mixed != 0;
  if (T->untorn) T->untorn->fp32 = T->fp32;
  LoadParams lp;
  lp.mode = ModeOP; lp.method = BE; lp.time = 0; lp.h = 0; lp.rh = 0; lp.initJct = true; lp.gmin = o.gmin;
  lp.srcStepping = false; lp.srcFact = 0;
  std::vector<int32_t> status(T->V, KS_STATUS_OK), iters(T->V, 0);
  if ((rc = newton(T, lp, o, o.itl1, reuse, status, iters))) return rc;
  if ((rc = accept_all_variants(T, status, 0.0, ModeOP, o.gmin))) return rc;
  if ((rc = x_out(T, out_x))) return rc;
  if (out_status) memcpy(out_status, status.data(), sizeof(int32_t) * T->V);
  if (out_iters) memcpy(out_iters, iters.data(), sizeof(int32_t) * T->V);
  stats_out(T, stats);
  return KS_OK;
}

extern "C" int ks_torn_tran(ks_torn* T, const ks_tran_spec* spec, const ks_options* opt, int32_t reuse,
                            const int32_t* probes, int32_t n_probes, double* out_wave, double* out_x,
                            int32_t* out_status, int32_t* out_steps, int32_t* out_iters, int64_t* stats) {
  if (!T || !spec || spec->step <= 0 || spec->stop <= 0 || (n_probes > 0 && !probes)) return KS_EINVAL;
  if (!spec->fixed_step || spec->uic) {
    set_error("ks_torn_tran: fixed-step transients from the operating point only");
    return KS_EUNSUPPORTED;
  }
  for (int q = 0; q < n_probes; q++)
    if (probes[q] < 0 || probes[q] >= T->n) { set_error("ks_torn_tran: probe out of range"); return KS_EINVAL; }
  const int64_t V = T->V;
  const long npts = std::lround(spec->stop / spec->step) + 1;
  int rc = fresh_state(T, spec->step, spec->stop);
  if (rc) return rc;
  KOpts o = ks_kopts_from(opt);
  T->fp32 = o.mixed != 0;
  if (T->untorn) T->untorn->fp32 = T->fp32;
  std::vector<int32_t> status(V, KS_STATUS_OK), iters(V, 0), steps(V, 0);
  int32_t* d_probes = nullptr;
  double* d_wave = nullptr;
  double* d_xprev = nullptr;  // step predictor: the two accepted points before the last
  if (o.predict && cudaMalloc(&d_xprev, 2 * sizeof(double) * (size_t)T->n * V) != cudaSuccess) {
    set_error("ks_torn_tran: allocation");
    return KS_ENOMEM;
  }
  const size_t wave_elems = (size_t)npts * V * std::max(n_probes, 0);
  if (n_probes > 0) {
    if (cudaMalloc(&d_probes, sizeof(int32_t) * n_probes) != cudaSuccess ||
        cudaMalloc(&d_wave, sizeof(double) * wave_elems) != cudaSuccess) {
      cudaFree(d_probes);
      cudaFree(d_xprev);
      set_error("ks_torn_tran: allocation");
      return KS_ENOMEM;
    }
    cudaMemcpyAsync(d_probes, probes, sizeof(int32_t) * n_probes, cudaMemcpyHostToDevice, T->st);
  }
  auto record = [&](long k) {
    if (n_probes > 0) {
      T->launches++;
      k_tl_record<<<blocks_for((int64_t)n_probes * V, 256), 256, 0, T->st>>>(n_probes, d_probes, V, T->x,
                                                                               d_wave + (size_t)k * V * n_probes);
    }
  };
  // the transient operating point (analysis/tran.go: dcSolve at ModeTranOP, Accept)
  LoadParams lp;
  lp.mode = ModeTranOP; lp.method = BE; lp.time = 0; lp.h = 0; lp.rh = 0; lp.initJct = true; lp.gmin = o.gmin;
  lp.srcStepping = false; lp.srcFact = 0;
  rc = newton(T, lp, o, o.itl1, reuse, status, iters);
  if (!rc) rc = accept_all_variants(T, status, 0.0, ModeTranOP, o.gmin);
  if (!rc) record(0);
  // fixed steps; backward Euler at the first, then the spec's method
  // the companion models change every Jacobian at the first step: fresh factors
  T->have.assign(V, 0);
  int order = BE;
  const int method = spec->method == KS_METHOD_BE ? BE : TRAP;
  for (long k = 1; k < npts && !rc; k++) {
    const double t = (double)k * spec->step, h = spec->step;
    lp.mode = ModeTran; lp.time = t; lp.h = h; lp.rh = 1 / h; lp.method = order; lp.initJct = false;
    if (d_xprev) {  // Newton from the extrapolated history (x_0 .. x_(k-1) accepted)
      const int64_t nv = T->n * V;
      T->launches++;
      k_tl_predict<<<blocks_for(nv, 256), 256, 0, T->st>>>(nv, (int)std::min<long>(k - 1, 2), T->x, d_xprev,
                                                           d_xprev + nv);
    }
    rc = newton(T, lp, o, o.itl4, reuse, status, iters);
    if (rc) break;
    rc = accept_all_variants(T, status, t, ModeTran, o.gmin);
    if (rc) break;
    for (int64_t v = 0; v < V; v++) if (status[v] == KS_STATUS_OK) steps[v]++;
    record(k);
    order = method;
  }
  if (!rc && out_wave && n_probes > 0) {
    std::vector<double> hw(wave_elems);
    if (cudaMemcpyAsync(hw.data(), d_wave, sizeof(double) * wave_elems, cudaMemcpyDeviceToHost, T->st) != cudaSuccess ||
        cudaStreamSynchronize(T->st) != cudaSuccess)
      rc = ck(cudaGetLastError(), "wave");
    else
      memcpy(out_wave, hw.data(), sizeof(double) * wave_elems);
  }
  cudaFree(d_probes);
  cudaFree(d_wave);
  cudaFree(d_xprev);
  if (rc) return rc;
  if ((rc = x_out(T, out_x))) return rc;
  if (out_status) memcpy(out_status, status.data(), sizeof(int32_t) * V);
  if (out_steps) memcpy(out_steps, steps.data(), sizeof(int32_t) * V);
  if (out_iters) memcpy(out_iters, iters.data(), sizeof(int32_t) * V);
  stats_out(T, stats);
  return KS_OK;
}
