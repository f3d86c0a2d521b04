// ks_multi.cu — batches of circuits of different topologies and sizes (up to
// thousands of unknowns each), one warp per circuit.
//
// The batched kernels elsewhere in the engine give each circuit one thread and a
// dense system; that serves thousands of copies of one small topology.  Here every
// circuit has its own element table and its own sparse system, so the unit of
// parallelism is a warp: the 32 lanes run the circuit's Newton / dcSolve /
// transient control code together (the same device templates, with a warp
// program, ks_solve.cuh) and split its element loops and its matrix work:
//   - stamping: lanes take the elements in turn and add into the sparse values
//     atomically (slots found by binary search in the row's sorted columns);
//   - LU: the fixed pivot sequence of the host's symbolic analysis
//     (ks_sparse.cpp), factored row by row in step order, the updates of each
//     L entry shared between lanes; FP64, or FP32 with FP64-residual refinement;
//   - triangular solves: one row after another, each row's dot product split
//     between lanes and summed by shuffles.
// Per-circuit arrays are contiguous (stride 1) in a few large device buffers,
// addressed through a per-circuit offset record.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "ks_internal.h"
#include "ks_tran.cuh"

using namespace ksg;
using ksh::set_error;

struct MultiCirc {     // offsets of one circuit in the shared buffers
  int64_t eoff, noff, voff, doff, soff, rpoff, woff;
  int64_t foff[2];     // factor slots: DC layout, transient layout
  int32_t n, ne, n_nodes, n_state, nonlin_empty, pad;
};

// One pivot sequence and factor pattern (rows in step order) for every circuit:
// layout 0 is chosen at DC, layout 1 with the transient companions.
struct MultiLayout {
  const int32_t* rp;    // [total unknowns + circuits]
  const int32_t* ci;    // [total slots]
  const int32_t* dg;    // [total unknowns]
  const int32_t* prow;
  const int32_t* q;
  const int32_t* pinv;
  const int32_t* qinv;
  double* av;           // A in the factor's pattern (fill slots zero)
  double* fv;           // FP64 factor
  float* f32;           // FP32 factor
};

struct MultiArgs {
  const MultiCirc* circ;
  const KElem* elem;
  const int8_t* isv;
  const double* values;
  double* derived;
  double* state;
  double* work;     // [3 * total unknowns]
  double* rhs;      // [total unknowns] each
  double* x;
  double* xo;
  double* col;
  double* y;
  float* y32;
  double* rpiv;
  float* rpiv32;
  long long* cmax;      // [total unknowns]: magnitude key of each step column's largest A entry
  MultiLayout lay[2];
  int npts;             // fixed-step points per circuit (waveform layout)
  int wcap;             // doubles of shared memory per warp for the accumulator (0: use y)
};

namespace ksg {

__device__ __forceinline__ int lane_id() { return (int)(threadIdx.x & 31); }

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ long long warp_max(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}

// One circuit's sparse system, shared by the lanes of a warp.  The matrix, the
// right-hand side and the column maxima are built by atomics, which complete in
// L2; they are read through volatile pointers (not cached in L1), so no lane
// sees a line its SM cached before the atomics.
struct WarpSys {
  static constexpr bool kStatic = false;
  static constexpr bool kAtomic = true;
  static constexpr bool kModes = true;
  static constexpr int kUnroll = 1;
  int n_, mode;
  const int32_t *rp, *ci, *dg, *prow, *q, *pinv, *qinv;  // the active layout
  volatile double* av;
  double* fv;
  float* f32;
  const int32_t *rp2, *ci2, *dg2, *prow2, *q2, *pinv2, *qinv2;  // the other one
  volatile double* av2;
  double* fv2;
  float* f322;
  volatile double* rhs_;
  double *x_, *xo_, *col_, *y, *rpiv;
  double* w;  // dense accumulator of the row being eliminated [n]: shared memory, or global for large n
  float *y32, *rpiv32;
  volatile long long* cmax;
  template <class T>
  __device__ __forceinline__ static void swp(T& a, T& b) { T t = a; a = b; b = t; }
  // 0: DC pivot sequence, 1: transient (the layouts trade places)
  __device__ __forceinline__ void set_mode(int m) {
    if (m == mode) return;
    mode = m;
    swp(rp, rp2); swp(ci, ci2); swp(dg, dg2); swp(prow, prow2); swp(q, q2); swp(pinv, pinv2); swp(qinv, qinv2);
    swp(av, av2); swp(fv, fv2); swp(f32, f322);
  }
  __device__ __forceinline__ int size() const { return n_; }
  // slot of A(i, j) (A coordinates): binary search of step column qinv[j] in step row pinv[i]
  __device__ __forceinline__ int slot(int i, int j) const {
    const int r = pinv[i], c = qinv[j];
    int lo = rp[r], hi = rp[r + 1] - 1;
    while (lo < hi) {
      int mid = (lo + hi) >> 1;
      if (ci[mid] < c) lo = mid + 1; else hi = mid;
    }
    return lo;
  }
  __device__ __forceinline__ volatile double& a(int i, int j) { return av[slot(i, j)]; }
  __device__ __forceinline__ void add(int i, int j, double v) { atomicAdd(const_cast<double*>(&av[slot(i, j)]), v); }
  __device__ __forceinline__ volatile double& rhs(int i) { return rhs_[i]; }
  __device__ __forceinline__ void add_rhs(int i, double v) { atomicAdd(const_cast<double*>(&rhs_[i]), v); }
  __device__ __forceinline__ double& xn(int i) { return x_[i]; }
  __device__ __forceinline__ double& xo(int i) { return xo_[i]; }
  __device__ __forceinline__ double& col(int i) { return col_[i]; }
  __device__ __forceinline__ void zero() {
    const int nnz = rp[n_];
    for (int p = lane_id(); p < nnz; p += 32) av[p] = 0.0;
    for (int i = lane_id(); i < n_; i += 32) rhs_[i] = 0.0;
  }
};

// The element program of the circuit a warp is working on.
struct WarpProg {
  static constexpr bool kStaticLU = false;
  static constexpr bool kWarp = true;
  const MultiArgs* args;
  const KElem* el;
  const int8_t* isv;
  int ne, n_nodes, n_state;
  bool nonlin_empty;
  int64_t xb, wb;
  template <class F>
  __device__ __forceinline__ void each(F&& f) const {
    for (int k = lane_id(); k < ne; k += 32) f(el[k]);
  }
  __device__ __forceinline__ bool is_v(int i) const { return isv[i] != 0; }
  __device__ __forceinline__ int64_t x_base(int64_t, int) const { return xb; }
  __device__ __forceinline__ int64_t wave_base(int64_t, int64_t, int n, int k) const { return wb + (int64_t)k * n; }
  template <class T>
  __device__ __forceinline__ void bind(T& t, int64_t c) {
    const MultiArgs& a = *args;
    const MultiCirc m = a.circ[c];
    el = a.elem + m.eoff;
    isv = a.isv + m.noff;
    ne = m.ne; n_nodes = m.n_nodes; n_state = m.n_state; nonlin_empty = m.nonlin_empty != 0;
    xb = m.noff;
    wb = m.woff;
    const int n = m.n;
    t.V = Col{const_cast<double*>(a.values) + m.voff, 1};
    t.D = Col{a.derived + m.doff, 1};
    t.Sb = Col{a.state + m.soff, 1};
    t.save = Col{a.work + 3 * m.noff, 1};
    t.ptPrev = Col{a.work + 3 * m.noff + n, 1};
    t.xacc = Col{a.work + 3 * m.noff + 2 * n, 1};
    WarpSys& s = t.s;
    s.n_ = n;
    s.mode = 0;
    const MultiLayout& L0 = a.lay[0];
    s.rp = L0.rp + m.rpoff; s.ci = L0.ci + m.foff[0]; s.dg = L0.dg + m.noff; s.prow = L0.prow + m.noff;
    s.q = L0.q + m.noff; s.pinv = L0.pinv + m.noff; s.qinv = L0.qinv + m.noff;
    s.av = L0.av + m.foff[0]; s.fv = L0.fv + m.foff[0]; s.f32 = L0.f32 + m.foff[0];
    const MultiLayout& L1 = a.lay[1].rp ? a.lay[1] : a.lay[0];  // no transient layout: DC for both
    const int64_t f1 = a.lay[1].rp ? m.foff[1] : m.foff[0];
    s.rp2 = L1.rp + m.rpoff; s.ci2 = L1.ci + f1; s.dg2 = L1.dg + m.noff; s.prow2 = L1.prow + m.noff;
    s.q2 = L1.q + m.noff; s.pinv2 = L1.pinv + m.noff; s.qinv2 = L1.qinv + m.noff;
    s.av2 = L1.av + f1; s.fv2 = L1.fv + f1; s.f322 = L1.f32 + f1;
    s.rhs_ = a.rhs + m.noff;
    s.x_ = a.x + m.noff;
    s.xo_ = a.xo + m.noff;
    s.col_ = a.col + m.noff;
    s.y = a.y + m.noff;
    s.y32 = a.y32 + m.noff;
    s.rpiv = a.rpiv + m.noff;
    s.rpiv32 = a.rpiv32 + m.noff;
    s.cmax = a.cmax + m.noff;
    if (n <= a.wcap) {
      extern __shared__ __align__(16) double ks_multi_smem[];
      s.w = ks_multi_smem + (size_t)(threadIdx.x >> 5) * a.wcap;
    } else {
      s.w = s.y;
    }
    __syncwarp();
  }
};

// Largest |A| of every step column (magnitude keys), for the singular test.
__device__ __forceinline__ void column_keys(WarpSys& s) {
  const int n = s.n_, nnz = s.rp[n], lane = lane_id();
  for (int i = lane; i < n; i += 32) s.cmax[i] = 0;
  __syncwarp();
  for (int p = lane; p < nnz; p += 32) {
    long long k = mag_key(s.av[p]);
    if (k) atomicMax(const_cast<long long*>(&s.cmax[s.ci[p]]), k);
  }
  __syncwarp();
}

// Numeric LU on the fixed pivot sequence, row by row in step order, into F
// (T = double: fv, rpiv; T = float: f32, rpiv32), with the row being
// eliminated expanded into a dense accumulator W [n] (row-by-row elimination:
// the lanes update W at the columns of each U row directly, no search).  A
// pivot at or below colmax * n * 1e-14 (colmax: the largest |A| of its
// column) is singular, the test of solver/sparse.go:240,271.
template <class T>
__device__ __forceinline__ int warp_factor(WarpSys& s, T* F, T* rp_, T* W) {
  const int n = s.n_, lane = lane_id();
  column_keys(s);
  for (int i = 0; i < n; i++) {
    const int r0 = s.rp[i], r1 = s.rp[i + 1], d = s.dg[i];
    for (int p = r0 + lane; p < r1; p += 32) W[s.ci[p]] = (T)s.av[p];  // A row, fill at zero
    __syncwarp();
    for (int p = r0; p < d; p++) {
      const int k = s.ci[p];
      const T f = W[k] * rp_[k];
      const int k1 = s.rp[k + 1];
      for (int qq = s.dg[k] + 1 + lane; qq < k1; qq += 32) W[s.ci[qq]] -= f * F[qq];
      __syncwarp();
      if (lane == 0) W[k] = f;
      __syncwarp();
    }
    for (int p = r0 + lane; p < r1; p += 32) F[p] = W[s.ci[p]];
    const double dv = (double)W[i];
    __syncwarp();
    if (!(fabs(dv) > key_mag(s.cmax[i]) * (double)n * 1e-14) || !isfinite(dv)) return SOLVE_SINGULAR;
    if (lane == 0) rp_[i] = (T)1 / (T)dv;
    __syncwarp();
  }
  return SOLVE_OK;
}

// y = C^-1 v (v given per A row through vin, solution written per A column via xout)
template <class T, class VIN, class XOUT>
__device__ __forceinline__ void warp_lu_solve(WarpSys& s, const T* F, const T* rp_, T* y, VIN&& vin, XOUT&& xout) {
  const int n = s.n_, lane = lane_id();
  for (int i = 0; i < n; i++) {
    const int r0 = s.rp[i], d = s.dg[i];
    T acc = 0;
    for (int p = r0 + lane; p < d; p += 32) acc += F[p] * y[s.ci[p]];
    acc = warp_sum(acc);
    if (lane == 0) y[i] = (T)vin(s.prow[i]) - acc;
    __syncwarp();
  }
  for (int i = n - 1; i >= 0; i--) {
    const int d = s.dg[i], r1 = s.rp[i + 1];
    T acc = 0;
    for (int p = d + 1 + lane; p < r1; p += 32) acc += F[p] * y[s.ci[p]];
    acc = warp_sum(acc);
    if (lane == 0) y[i] = (y[i] - acc) * rp_[i];
    __syncwarp();
  }
  for (int i = lane; i < n; i += 32) xout(s.q[i], y[i]);
  __syncwarp();
}

// FP64 solve of the warp's system (the overload the shared Newton code calls).
__device__ __noinline__ int lu_solve_fp64(WarpSys& s) {
  const int n = s.n_, nnz = s.rp[n], lane = lane_id();
  long long kall = 0;
  for (int p = lane; p < nnz; p += 32) kall = key_max(kall, mag_key(s.av[p]));
  kall = warp_max(kall);
  if (kall >= KS_INF_KEY) return SOLVE_NONFINITE;
  if (kall == 0) return SOLVE_SINGULAR;
  int rc = warp_factor<double>(s, s.fv, s.rpiv, s.w);
  if (rc) return rc;
  warp_lu_solve<double>(s, s.fv, s.rpiv, s.y, [&](int r) { return s.rhs_[r]; },
                        [&](int c, double v) { s.x_[c] = v; });
  long long kx = 0;
  for (int i = lane; i < n; i += 32) kx = key_max(kx, mag_key(s.x_[i]));
  kx = warp_max(kx);
  return kx >= KS_INF_KEY ? SOLVE_NONFINITE : SOLVE_OK;
}

// FP32 factor, FP64 residual over A's pattern, refinement as lu_solve_mixed.
__device__ __noinline__ int lu_solve_mixed(WarpSys& s, int passes, double rtol) {
  const int n = s.n_, nnz = s.rp[n], lane = lane_id();
  long long kall = 0;
  for (int p = lane; p < nnz; p += 32) kall = key_max(kall, mag_key(s.av[p]));
  kall = warp_max(kall);
  if (kall >= KS_INF_KEY) return SOLVE_NONFINITE;
  if (kall == 0) return SOLVE_SINGULAR;
  if (warp_factor<float>(s, s.f32, s.rpiv32, reinterpret_cast<float*>(s.w))) return SOLVE_FP32_FAIL;
  for (int i = lane; i < n; i += 32) s.x_[i] = s.xo_[i];
  __syncwarp();
  double prev = KS_INF;
  for (int pass = 0; pass < passes; pass++) {
    for (int i = lane; i < n; i += 32) {  // FP64 residual of step row i (A row prow[i]) into col
      double r = s.rhs_[s.prow[i]];
      for (int p = s.rp[i]; p < s.rp[i + 1]; p++) r = fma(-s.av[p], s.x_[s.q[s.ci[p]]], r);
      s.col_[s.prow[i]] = r;
    }
    __syncwarp();
    warp_lu_solve<float>(s, s.f32, s.rpiv32, s.y32, [&](int r) { return (float)s.col_[r]; },
                         [&](int c, float v) { s.col_[c] = v; });
    long long kd = 0, kx = 0;
    for (int i = lane; i < n; i += 32) {
      const double v = s.x_[i] + s.col_[i];
      s.x_[i] = v;
      kd = key_max(kd, mag_key(s.col_[i]));
      kx = key_max(kx, mag_key(v));
    }
    kd = warp_max(kd);
    kx = warp_max(kx);
    __syncwarp();
    if (kx >= KS_INF_KEY || kd >= KS_INF_KEY) return SOLVE_NONFINITE;
    const double dmax = key_mag(kd), xmax = key_mag(kx);
    if (dmax <= rtol * xmax || dmax == 0) break;
    if (pass > 0 && dmax > 0.5 * prev) return SOLVE_FP32_FAIL;
    if (pass == passes - 1 && passes > 1) return SOLVE_FP32_FAIL;
    prev = dmax;
  }
  return SOLVE_OK;
}

}  // namespace ksg

// ---------------------------------------------------------------- kernels
__global__ void k_multi_setup(MultiArgs a, int64_t B, double step, double stop) {
  const int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (c >= B) return;
  const MultiCirc m = a.circ[c];
  Col V{const_cast<double*>(a.values) + m.voff, 1}, D{a.derived + m.doff, 1};
  for (int k = lane_id(); k < m.ne; k += 32) setup_elem(a.elem[m.eoff + k], V, D, step, stop);
}

__global__ void __launch_bounds__(128) k_multi_op(MultiArgs a, KOpts o, int64_t B, double* out_x, int32_t* out_status,
                                                  int32_t* out_iters, uint64_t deadline_ns, unsigned long long* queue) {
  Thr<WarpSys, WarpProg> t;
  t.prog.args = &a;
  t.o = o;
  op_persistent(t, nullptr, nullptr, nullptr, nullptr, B, nullptr, out_x, out_status, out_iters, deadline_ns, queue);
}

__global__ void __launch_bounds__(128) k_multi_tran(MultiArgs a, KOpts o, TranSpecK sp, int64_t B, double* out_wave,
                                                    int32_t* out_npts, int32_t* out_status, int32_t* out_steps,
                                                    int32_t* out_iters, uint64_t deadline_ns,
                                                    unsigned long long* queue) {
  Thr<WarpSys, WarpProg> t;
  t.prog.args = &a;
  t.o = o;
  tran_persistent(t, sp, nullptr, nullptr, nullptr, nullptr, B, nullptr, out_wave, out_npts, out_status, out_steps,
                  out_iters, deadline_ns, queue);
}

// ---------------------------------------------------------------- host side
struct ks_multi {
  int64_t B = 0, N = 0;          // circuits, total unknowns
  int64_t F[2] = {0, 0};         // factor slots per layout
  int64_t flops[2] = {0, 0};     // multiply-adds of one factorization of every circuit, per layout
  double lay_h[2] = {0, -1};     // step each layout was chosen for (layout 1 absent while < 0)
  std::vector<ksh::HostPlan> hp;
  std::vector<double> vals;
  std::vector<int64_t> voff;
  std::vector<MultiCirc> circ;
  std::vector<int32_t> n_of;
  MultiArgs a{};
  void* buf = nullptr;           // elements, values and the per-unknown working arrays
  void* lay_buf[2] = {nullptr, nullptr};
  unsigned long long* queue = nullptr;
  cudaStream_t stream = nullptr;
  double setup_step = -1, setup_stop = -1;
};

KOpts ks_kopts_from(const ks_options* o);

namespace {

template <class T>
size_t put(std::vector<unsigned char>& h, size_t& off, const std::vector<T>& v) {
  off = (off + 255) & ~(size_t)255;
  size_t at = off, need = off + v.size() * sizeof(T);
  if (h.size() < need) h.resize(need);
  if (!v.empty()) std::memcpy(h.data() + off, v.data(), v.size() * sizeof(T));
  off += v.size() * sizeof(T);
  return at;
}

size_t carve(size_t& off, size_t bytes) {
  off = (off + 255) & ~(size_t)255;
  size_t r = off;
  off += bytes;
  return r;
}

// Pivot sequences of every circuit (h = 0: DC, else the transient companions of
// step h), uploaded as layout L.
int build_layout(ks_multi* m, int L, double h, std::string* err) {
  const int64_t B = m->B;
  std::vector<ksh::SparseSym> sy(B);
  std::vector<std::string> errs(B);
  std::vector<int> rcs(B, 0);
  unsigned nth = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  std::vector<std::thread> th;
  for (unsigned w = 0; w < nth; w++)
    th.emplace_back([&, w]() {
      for (int64_t c = w; c < B; c += nth) rcs[c] = ksh::sparse_symbolic(m->hp[c], m->vals.data() + m->voff[c], h, &sy[c], &errs[c]);
    });
  for (auto& t : th) t.join();
  for (int64_t c = 0; c < B; c++)
    if (rcs[c]) { *err = "circuit " + std::to_string(c) + ": " + errs[c]; return rcs[c]; }
  std::vector<int32_t> rp, ci, dg, prow, q, pinv, qinv;
  int64_t F = 0, fl = 0;
  for (int64_t c = 0; c < B; c++) {
    const ksh::SparseSym& y = sy[c];
    m->circ[c].foff[L] = F;
    rp.insert(rp.end(), y.rp.begin(), y.rp.end());
    ci.insert(ci.end(), y.ci.begin(), y.ci.end());
    dg.insert(dg.end(), y.dg.begin(), y.dg.end());
    prow.insert(prow.end(), y.prow.begin(), y.prow.end());
    q.insert(q.end(), y.q.begin(), y.q.end());
    pinv.insert(pinv.end(), y.pinv.begin(), y.pinv.end());
    qinv.insert(qinv.end(), y.qinv.begin(), y.qinv.end());
    F += y.rp[y.n];
    fl += y.flops;
  }
  std::vector<unsigned char> host;
  size_t off = 0;
  size_t o_rp = put(host, off, rp), o_ci = put(host, off, ci), o_dg = put(host, off, dg), o_prow = put(host, off, prow),
         o_q = put(host, off, q), o_pinv = put(host, off, pinv), o_qinv = put(host, off, qinv);
  size_t o_av = carve(off, 8 * F), o_fv = carve(off, 8 * F), o_f32 = carve(off, 4 * F);
  if (m->lay_buf[L]) { cudaFree(m->lay_buf[L]); m->lay_buf[L] = nullptr; }
  if (cudaMalloc(&m->lay_buf[L], off) != cudaSuccess) { *err = "device allocation of " + std::to_string(off) + " bytes failed"; return KS_ENOMEM; }
  if (cudaMemcpy(m->lay_buf[L], host.data(), host.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
    *err = "upload failed";
    return KS_ECUDA;
  }
  unsigned char* b = static_cast<unsigned char*>(m->lay_buf[L]);
  MultiLayout& y = m->a.lay[L];
  y.rp = reinterpret_cast<const int32_t*>(b + o_rp);
  y.ci = reinterpret_cast<const int32_t*>(b + o_ci);
  y.dg = reinterpret_cast<const int32_t*>(b + o_dg);
  y.prow = reinterpret_cast<const int32_t*>(b + o_prow);
  y.q = reinterpret_cast<const int32_t*>(b + o_q);
  y.pinv = reinterpret_cast<const int32_t*>(b + o_pinv);
  y.qinv = reinterpret_cast<const int32_t*>(b + o_qinv);
  y.av = reinterpret_cast<double*>(b + o_av);
  y.fv = reinterpret_cast<double*>(b + o_fv);
  y.f32 = reinterpret_cast<float*>(b + o_f32);
  m->F[L] = F;
  m->flops[L] = fl;
  m->lay_h[L] = h;
  // the per-circuit records carry the layouts' slot offsets
  if (cudaMemcpy(const_cast<MultiCirc*>(m->a.circ), m->circ.data(), sizeof(MultiCirc) * B, cudaMemcpyHostToDevice) !=
      cudaSuccess) {
    *err = "upload failed";
    return KS_ECUDA;
  }
  return KS_OK;
}

}  // namespace

extern "C" int ks_multi_create(int32_t n_circ, const ks_topology* topos, const double* values,
                               const int64_t* value_offsets, ks_multi** out) {
  if (n_circ <= 0 || !topos || !values || !value_offsets || !out) { set_error("ks_multi_create: bad argument"); return KS_EINVAL; }
  ks_multi* m = new ks_multi();
  const int64_t B = n_circ;
  m->B = B;
  m->hp.resize(B);
  std::vector<std::string> errs(B);
  std::vector<int> rcs(B, 0);
  for (int64_t c = 0; c < B; c++) {
    rcs[c] = ksh::plan_layout(&topos[c], &m->hp[c], &errs[c]);
    if (rcs[c]) { set_error("ks_multi_create: circuit " + std::to_string(c) + ": " + errs[c]); int rc = rcs[c]; delete m; return rc; }
  }
  m->circ.resize(B);
  std::vector<KElem> elem;
  std::vector<int8_t> isv;
  int64_t E = 0, N = 0, V = 0, D = 0, S = 0, R = 0;
  for (int64_t c = 0; c < B; c++) {
    const ksh::HostPlan& h = m->hp[c];
    MultiCirc mc{};
    mc.eoff = E; mc.noff = N; mc.voff = V; mc.doff = D; mc.soff = S; mc.rpoff = R;
    mc.n = h.n; mc.ne = h.n_elem; mc.n_nodes = h.n_nodes; mc.n_state = h.n_state; mc.nonlin_empty = h.n_nonlin == 0;
    m->circ[c] = mc;
    m->n_of.push_back(h.n);
    elem.insert(elem.end(), h.elem.begin(), h.elem.end());
    isv.insert(isv.end(), h.is_v.begin(), h.is_v.begin() + h.n);
    m->voff.push_back(V);
    m->vals.insert(m->vals.end(), values + value_offsets[c], values + value_offsets[c] + h.n_values);
    E += h.n_elem; N += h.n; V += h.n_values; D += h.n_derived + 1; S += h.n_state + 1; R += h.n + 1;
  }
  m->N = N;
  std::vector<unsigned char> host;
  size_t off = 0;
  size_t o_circ = put(host, off, m->circ), o_elem = put(host, off, elem), o_isv = put(host, off, isv),
         o_vals = put(host, off, m->vals);
  size_t o_der = carve(off, 8 * D), o_state = carve(off, 8 * S), o_work = carve(off, 8 * 3 * N),
         o_rhs = carve(off, 8 * N), o_x = carve(off, 8 * N), o_xo = carve(off, 8 * N), o_col = carve(off, 8 * N),
         o_y = carve(off, 8 * N), o_y32 = carve(off, 4 * N), o_rpiv = carve(off, 8 * N), o_rpiv32 = carve(off, 4 * N),
         o_cmax = carve(off, 8 * N), o_queue = carve(off, 64);
  if (cudaMalloc(&m->buf, off) != cudaSuccess) {
    set_error("ks_multi_create: device allocation of " + std::to_string(off) + " bytes failed");
    delete m;
    return KS_ENOMEM;
  }
  if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMemcpy(m->buf, host.data(), host.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
    ks_multi_destroy(m);
    set_error("ks_multi_create: upload failed");
    return KS_ECUDA;
  }
  unsigned char* b = static_cast<unsigned char*>(m->buf);
  MultiArgs& a = m->a;
  a.circ = reinterpret_cast<const MultiCirc*>(b + o_circ);
  a.elem = reinterpret_cast<const KElem*>(b + o_elem);
  a.isv = reinterpret_cast<const int8_t*>(b + o_isv);
  a.values = reinterpret_cast<const double*>(b + o_vals);
  a.derived = reinterpret_cast<double*>(b + o_der);
  a.state = reinterpret_cast<double*>(b + o_state);
  a.work = reinterpret_cast<double*>(b + o_work);
  a.rhs = reinterpret_cast<double*>(b + o_rhs);
  a.x = reinterpret_cast<double*>(b + o_x);
  a.xo = reinterpret_cast<double*>(b + o_xo);
  a.col = reinterpret_cast<double*>(b + o_col);
  a.y = reinterpret_cast<double*>(b + o_y);
  a.y32 = reinterpret_cast<float*>(b + o_y32);
  a.rpiv = reinterpret_cast<double*>(b + o_rpiv);
  a.rpiv32 = reinterpret_cast<float*>(b + o_rpiv32);
  a.cmax = reinterpret_cast<long long*>(b + o_cmax);
  m->queue = reinterpret_cast<unsigned long long*>(b + o_queue);
  std::string err;
  int rc = build_layout(m, 0, 0.0, &err);
  if (rc) {
    ks_multi_destroy(m);
    set_error("ks_multi_create: " + err);
    return rc;
  }
  *out = m;
  return KS_OK;
}

extern "C" int ks_sparse_analyze(const ks_topology* topo, const double* values, double step, int32_t* n, int64_t* slots, int64_t* lu_flops,
                                 int32_t* prow, int32_t* pcol, int32_t* rowptr, int32_t* cols) {
  if (!topo) return KS_EINVAL;
  ksh::HostPlan hp;
  ksh::SparseSym sy;
  std::string err;
  int rc = ksh::plan_layout(topo, &hp, &err);
  if (!rc) rc = ksh::sparse_symbolic(hp, values, step, &sy, &err);
  if (rc) { set_error(err); return rc; }
  if (n) *n = sy.n;
  if (slots) *slots = sy.rp[sy.n];
  if (lu_flops) *lu_flops = sy.flops;
  if (prow) std::memcpy(prow, sy.prow.data(), sizeof(int32_t) * sy.n);
  if (pcol) std::memcpy(pcol, sy.q.data(), sizeof(int32_t) * sy.n);
  if (rowptr) std::memcpy(rowptr, sy.rp.data(), sizeof(int32_t) * (sy.n + 1));
  if (cols) std::memcpy(cols, sy.ci.data(), sizeof(int32_t) * sy.ci.size());
  return KS_OK;
}

extern "C" int ks_sparse_pattern(const ks_topology* topo, const double* values, int32_t transient, int32_t* n,
                                 uint8_t* pattern) {
  if (!topo) return KS_EINVAL;
  ksh::HostPlan hp;
  std::string err;
  int rc = ksh::plan_layout(topo, &hp, &err);
  if (rc) { set_error(err); return rc; }
  if (n) *n = hp.n;
  if (pattern) ksh::sparse_pattern(hp, values, transient != 0, pattern);
  return KS_OK;
}

extern "C" void ks_multi_destroy(ks_multi* m) {
  if (!m) return;
  cudaFree(m->buf);
  cudaFree(m->lay_buf[0]);
  cudaFree(m->lay_buf[1]);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
}

extern "C" int ks_multi_info(const ks_multi* m, int64_t* total_unknowns, int64_t* factor_slots, int64_t* lu_flops,
                             int32_t* n_per_circuit) {
  if (!m) return KS_EINVAL;
  if (total_unknowns) *total_unknowns = m->N;
  if (factor_slots) *factor_slots = m->F[0];
  if (lu_flops) *lu_flops = m->flops[0];
  if (n_per_circuit) std::memcpy(n_per_circuit, m->n_of.data(), sizeof(int32_t) * m->B);
  return KS_OK;
}

// Shared memory for the warps' accumulators: room for the largest circuit when
// four of them fit in 96 KB per block, else none (the accumulator is then global).
static int multi_wcap(const ks_multi* m) {
  int nmax = *std::max_element(m->n_of.begin(), m->n_of.end());
  return nmax * 8 * 4 <= 96 * 1024 ? nmax : 0;
}

static unsigned multi_grid(const void* kernel, int64_t B, size_t smem) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, 128, smem);
  int64_t need = (B + 3) / 4, cap = (int64_t)sms * (per > 0 ? per : 1);
  return (unsigned)(need < cap ? need : cap);
}

static int multi_setup(ks_multi* m, double step, double stop, cudaStream_t st) {
  if (m->setup_step == step && m->setup_stop == stop) return KS_OK;
  k_multi_setup<<<(unsigned)((m->B * 32 + 127) / 128), 128, 0, st>>>(m->a, m->B, step, stop);
  if (cudaGetLastError() != cudaSuccess) { set_error("ks_multi: setup launch failed"); return KS_ECUDA; }
  m->setup_step = step;
  m->setup_stop = stop;
  return KS_OK;
}

extern "C" int ks_multi_op_async(ks_multi* m, const ks_options* opt, double* out_x_dev, int32_t* out_status_dev,
                                 int32_t* out_iters_dev, void* stream) {
  if (!m) return KS_EINVAL;
  cudaStream_t st = stream ? (cudaStream_t)stream : m->stream;
  int rc = multi_setup(m, 0.0, 0.0, st);
  if (rc) return rc;
  KOpts o = ks_kopts_from(opt);
  uint64_t dl = opt && opt->deadline_s > 0 ? (uint64_t)(opt->deadline_s * 1e9) : 0;
  if (cudaMemsetAsync(m->queue, 0, 8, st) != cudaSuccess) { set_error("ks_multi_op: memset failed"); return KS_ECUDA; }
  MultiArgs a = m->a;
  a.wcap = multi_wcap(m);
  const size_t smem = (size_t)a.wcap * 8 * 4;
  k_multi_op<<<multi_grid((const void*)k_multi_op, m->B, smem), 128, smem, st>>>(a, o, m->B, out_x_dev, out_status_dev,
                                                                                 out_iters_dev, dl, m->queue);
  if (cudaGetLastError() != cudaSuccess) { set_error("ks_multi_op: launch failed"); return KS_ECUDA; }
  return KS_OK;
}

extern "C" int ks_multi_tran_async(ks_multi* m, const ks_tran_spec* spec, const ks_options* opt, double* out_wave_dev,
                                   int32_t* out_npts_dev, int32_t* out_status_dev, int32_t* out_steps_dev,
                                   int32_t* out_iters_dev, void* stream) {
  if (!m || !spec) return KS_EINVAL;
  if (!spec->fixed_step) { set_error("ks_multi_tran: fixed-step transients only"); return KS_EUNSUPPORTED; }
  if (!(spec->step > 0 && spec->stop > 0 && spec->start >= 0 && spec->start < spec->stop)) {
    set_error("analysis: invalid transient specification");
    return KS_EINVAL;
  }
  cudaStream_t st = stream ? (cudaStream_t)stream : m->stream;
  if (m->lay_h[1] != spec->step) {  // pivot sequences for this step's companion models
    std::string err;
    if (cudaStreamSynchronize(st) != cudaSuccess) { set_error("ks_multi_tran: CUDA error"); return KS_ECUDA; }
    int lrc = build_layout(m, 1, spec->step, &err);
    if (lrc) { set_error("ks_multi_tran: " + err); return lrc; }
  }
  int rc = multi_setup(m, spec->step, spec->stop, st);
  if (rc) return rc;
  KOpts o = ks_kopts_from(opt);
  TranSpecK sp;
  sp.step = spec->step; sp.stop = spec->stop; sp.start = spec->start;
  sp.maxStep = spec->step;
  sp.fixed = 1;
  sp.minStep = spec->min_step > 0 ? spec->min_step : 1e-12 * spec->stop;
  sp.chgtol = spec->chgtol > 0 ? spec->chgtol : 1e-14;
  sp.trtol = spec->trtol > 0 ? spec->trtol : 7;
  sp.uic = spec->uic;
  sp.method = spec->method == KS_METHOD_BE ? BE : TRAP;
  sp.maxSteps = spec->max_steps > 0 ? spec->max_steps : 1000000;
  sp.cap = 0;
  sp.npts = (int)llround(spec->stop / spec->step) + 1;
  MultiArgs a = m->a;
  a.npts = sp.npts;
  a.wcap = multi_wcap(m);
  const size_t smem = (size_t)a.wcap * 8 * 4;
  std::vector<MultiCirc> circ = m->circ;  // waveform offsets: npts * (unknowns before the circuit)
  bool changed = false;
  for (auto& c : circ) {
    int64_t w = (int64_t)sp.npts * c.noff;
    if (c.woff != w) { c.woff = w; changed = true; }
  }
  if (changed) {
    if (cudaMemcpyAsync(const_cast<MultiCirc*>(m->a.circ), circ.data(), sizeof(MultiCirc) * m->B,
                        cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
      set_error("ks_multi_tran: offset upload failed");
      return KS_ECUDA;
    }
    m->circ = circ;
  }
  uint64_t dl = opt && opt->deadline_s > 0 ? (uint64_t)(opt->deadline_s * 1e9) : 0;
  if (cudaMemsetAsync(m->queue, 0, 8, st) != cudaSuccess) { set_error("ks_multi_tran: memset failed"); return KS_ECUDA; }
  k_multi_tran<<<multi_grid((const void*)k_multi_tran, m->B, smem), 128, smem, st>>>(
      a, o, sp, m->B, out_wave_dev, out_npts_dev, out_status_dev, out_steps_dev, out_iters_dev, dl, m->queue);
  if (cudaGetLastError() != cudaSuccess) { set_error("ks_multi_tran: launch failed"); return KS_ECUDA; }
  return KS_OK;
}

extern "C" int ks_multi_op(ks_multi* m, const ks_options* opt, double* out_x, int32_t* out_status, int32_t* out_iters) {
  if (!m) return KS_EINVAL;
  cudaStream_t st = m->stream;
  double* dx = nullptr;
  int32_t* di = nullptr;
  if (cudaMalloc(&dx, 8 * m->N) != cudaSuccess || cudaMalloc(&di, 8 * m->B) != cudaSuccess) {
    cudaFree(dx);
    set_error("ks_multi_op: allocation failed");
    return KS_ENOMEM;
  }
  int rc = ks_multi_op_async(m, opt, dx, di, di + m->B, st);
  cudaError_t e = cudaSuccess;
  if (!rc && out_x) e = cudaMemcpyAsync(out_x, dx, 8 * m->N, cudaMemcpyDeviceToHost, st);
  if (!rc && e == cudaSuccess && out_status) e = cudaMemcpyAsync(out_status, di, 4 * m->B, cudaMemcpyDeviceToHost, st);
  if (!rc && e == cudaSuccess && out_iters) e = cudaMemcpyAsync(out_iters, di + m->B, 4 * m->B, cudaMemcpyDeviceToHost, st);
  if (!rc && e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(dx);
  cudaFree(di);
  if (rc) return rc;
  if (e != cudaSuccess) { set_error(std::string("ks_multi_op: ") + cudaGetErrorString(e)); return KS_ECUDA; }
  return KS_OK;
}

extern "C" int ks_multi_tran(ks_multi* m, const ks_tran_spec* spec, const ks_options* opt, double* out_wave,
                             int32_t* out_status, int32_t* out_steps, int32_t* out_iters) {
  if (!m || !spec) return KS_EINVAL;
  if (!spec->fixed_step) { set_error("ks_multi_tran: fixed-step transients only"); return KS_EUNSUPPORTED; }
  cudaStream_t st = m->stream;
  const int64_t npts = (int64_t)llround(spec->stop / spec->step) + 1;
  double* dw = nullptr;
  int32_t* di = nullptr;
  if ((out_wave && cudaMalloc(&dw, 8 * npts * m->N) != cudaSuccess) || cudaMalloc(&di, 16 * m->B) != cudaSuccess) {
    cudaFree(dw);
    set_error("ks_multi_tran: allocation failed");
    return KS_ENOMEM;
  }
  int rc = ks_multi_tran_async(m, spec, opt, dw, di, di + m->B, di + 2 * m->B, di + 3 * m->B, st);
  cudaError_t e = cudaSuccess;
  if (!rc && out_wave) e = cudaMemcpyAsync(out_wave, dw, 8 * npts * m->N, cudaMemcpyDeviceToHost, st);
  if (!rc && e == cudaSuccess && out_status) e = cudaMemcpyAsync(out_status, di + m->B, 4 * m->B, cudaMemcpyDeviceToHost, st);
  if (!rc && e == cudaSuccess && out_steps) e = cudaMemcpyAsync(out_steps, di + 2 * m->B, 4 * m->B, cudaMemcpyDeviceToHost, st);
  if (!rc && e == cudaSuccess && out_iters) e = cudaMemcpyAsync(out_iters, di + 3 * m->B, 4 * m->B, cudaMemcpyDeviceToHost, st);
  if (!rc && e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(dw);
  cudaFree(di);
  if (rc) return rc;
  if (e != cudaSuccess) { set_error(std::string("ks_multi_tran: ") + cudaGetErrorString(e)); return KS_ECUDA; }
  return KS_OK;
}
