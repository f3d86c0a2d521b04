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
#include "ks_results.cuh"

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

// Per-circuit constants (NewDiode, NewBJT, NewMOSFET/derive, resolveWave with the
// analysis's print step and stop time): setup_elem per element.
__global__ void k_setup(KPlan plan, const double* __restrict__ values, double* derived, int64_t B,
                        double step, double stop) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= B) return;
  Col V{const_cast<double*>(values) + c, B}, D{derived + c, B};
  for (int k = 0; k < plan.n_elem; k++) setup_elem(plan.elem[k], V, D, step, stop);
}

// FP32 copies of the value and derived-constant columns (the FP32 start stage's inputs).
__global__ void k_to32(const double* __restrict__ a, float* __restrict__ a32, int64_t na,
                       const double* __restrict__ b, float* __restrict__ b32, int64_t nb) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < na + nb; i += stride) {
    if (i < na) a32[i] = (float)a[i];
    else b32[i - na] = (float)b[i - na];
  }
}

int ks_launch_setup(const KsDeviceBatch& b, double step, double stop, void* stream) {
  int tpb = 128;
  unsigned grid = (unsigned)((b.B + tpb - 1) / tpb);
  k_setup<<<grid, tpb, 0, (cudaStream_t)stream>>>(b.plan, b.values, b.derived, b.B, step, stop);
  if (cudaGetLastError() != cudaSuccess) return -1;
  if (b.values32 && b.derived32) {
    const int64_t na = (int64_t)b.plan.n_values * b.B, nb = (int64_t)b.plan.n_derived * b.B;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t want = (na + nb + 255) / 256, cap = (int64_t)sms * 8;
    k_to32<<<(unsigned)(want < cap ? want : cap), 256, 0, (cudaStream_t)stream>>>(b.values, b.values32, na, b.derived,
                                                                                   b.derived32, nb);
  }
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// ---------------------------------------------------------------- operating point
// analysis.OP for every circuit: dcSolve (Newton, then the fallback chain) at
// ModeOP, then Accept.  Persistent: each thread takes the next circuit from the
// queue counter as soon as its circuit is done, so a warp's lanes stay busy
// while circuits need different numbers of Newton iterations.  R: with the
// element results and the energy ledger (ks_results.cuh).
template <int T, bool R>
__global__ void __launch_bounds__(T) k_op(KPlan plan, KOpts o, const double* __restrict__ values,
                                          const double* __restrict__ derived, double* state, double* work,
                                          int64_t B, const double* __restrict__ x0, double* out_x,
                                          int32_t* out_status, int32_t* out_iters, uint64_t deadline_ns,
                                          unsigned long long* queue, K32 k32) {
  extern __shared__ __align__(16) unsigned char smem[];
  Thr<SmemSys<T>, RtProg> t;
  smem_layout<T>(t, plan, smem);
  t.o = o;
  __syncthreads();
  op_persistent<SmemSys<T>, RtProg, R>(t, values, derived, state, work, B, x0, out_x, out_status, out_iters,
                                       deadline_ns, queue, k32.values ? &k32 : nullptr);
}

// analysis.DC for every circuit: the sweep's points in order, each warm-started
// from the previous one (dc_sweep_persistent, ks_newton.cuh).
template <int T>
__global__ void __launch_bounds__(T) k_dc_sweep(KPlan plan, KOpts o, const double* __restrict__ values,
                                                const double* __restrict__ derived, double* state, double* work,
                                                int64_t B, int src, const double* __restrict__ pts, int npts,
                                                int src2, const double* __restrict__ pts2, int npts2,
                                                double* out_x, int32_t* out_status, int32_t* out_points,
                                                int32_t* out_iters, uint64_t deadline_ns, unsigned long long* queue) {
  extern __shared__ __align__(16) unsigned char smem[];
  Thr<SmemSys<T>, RtProg> t;
  smem_layout<T>(t, plan, smem);
  t.o = o;
  __syncthreads();
  dc_sweep_persistent(t, values, derived, state, work, B, src, pts, npts, src2, pts2, npts2, out_x, out_status,
                      out_points, out_iters, deadline_ns, queue);
}

// Blocks of T threads that keep every SM full (persistent grid), capped by the work.
template <typename K>
static unsigned persistent_grid(K kernel, int T, size_t smem, int64_t B, int cpt = 0) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, T, smem);
  if (per < 1) per = 1;
  if (cpt <= 0) cpt = circuits_per_thread();
  int64_t need = (B + (int64_t)T * cpt - 1) / ((int64_t)T * cpt);
  int64_t g = (int64_t)sms * per;
  return (unsigned)(need < g ? need : g);
}

int ks_launch_op(const KsDeviceBatch& b, const KOpts& o, const double* x0, double* out_x, int32_t* out_status,
                 int32_t* out_iters, double deadline_s, void* stream, const KsSpec* kspec) {
  int n = b.plan.n, ne = b.plan.n_elem;
  if (n > KS_MAX_DENSE) return -2;
  uint64_t dl = deadline_s > 0 ? (uint64_t)(deadline_s * 1e9) : 0;
  const bool res = o.res_scratch != nullptr;  // results: the generic kernels' results instantiation
  if (kspec && !res) {  // per-topology kernel of the plan (ks_jit.cpp)
    if (cudaMemsetAsync(b.queue, 0, sizeof(unsigned long long), (cudaStream_t)stream) != cudaSuccess) return -1;
    KOpts ko = o;
    const double *values = b.values, *derived = b.derived;
    double *state = b.state, *work = b.work;
    int64_t B = b.B;
    unsigned long long* queue = b.queue;
    K32 k32{b.values32, b.derived32, b.state32};
    if (!b.values32 || !b.derived32 || !b.state32) k32 = K32{nullptr, nullptr, nullptr};
    void* args[] = {&ko, &values, &derived, &state, &work, &B, &x0, &out_x, &out_status, &out_iters, &dl, &queue, &k32};
    const int cpt = o.cpt > 0 ? o.cpt : circuits_per_thread();
    int64_t need = (B + (int64_t)kspec->T * cpt - 1) / ((int64_t)kspec->T * cpt);
    unsigned grid = (unsigned)(need < kspec->blocks ? need : kspec->blocks);
    std::string err;
    if (ksj::launch(kspec->fn, grid, kspec->T, kspec->smem, stream, args, &err)) { ksh::set_error(err); return -1; }
    return 0;
  }
  int maxSmem = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&maxSmem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  int T = 64;
  size_t sm = ks_sys_smem(n, ne, 64);
  if (sm > (size_t)maxSmem) { T = 32; sm = ks_sys_smem(n, ne, 32); }
  if (sm > (size_t)maxSmem) return -2;
  cudaStream_t st = (cudaStream_t)stream;
  if (cudaMemsetAsync(b.queue, 0, sizeof(unsigned long long), st) != cudaSuccess) return -1;
  K32 k32{b.values32, b.derived32, b.state32};
  if (!b.values32 || !b.derived32 || !b.state32) k32 = K32{nullptr, nullptr, nullptr};
  auto go = [&](auto kernel, int threads) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    unsigned grid = persistent_grid(kernel, threads, sm, b.B, o.cpt);
    kernel<<<grid, threads, sm, st>>>(b.plan, o, b.values, b.derived, b.state, b.work, b.B, x0, out_x, out_status,
                                      out_iters, dl, b.queue, k32);
  };
  if (T == 64) res ? go(k_op<64, true>, 64) : go(k_op<64, false>, 64);
  else res ? go(k_op<32, true>, 32) : go(k_op<32, false>, 32);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int ks_launch_dc_sweep(const KsDeviceBatch& b, const KOpts& o, int src, const double* pts, int npts, int src2,
                       const double* pts2, int npts2, double* out_x, int32_t* out_status, int32_t* out_points,
                       int32_t* out_iters, double deadline_s, void* stream) {
  const int n = b.plan.n, ne = b.plan.n_elem;
  if (n > KS_MAX_DENSE) return -2;
  const uint64_t dl = deadline_s > 0 ? (uint64_t)(deadline_s * 1e9) : 0;
  int maxSmem = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&maxSmem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  int T = 64;
  size_t sm = ks_sys_smem(n, ne, 64);
  if (sm > (size_t)maxSmem) { T = 32; sm = ks_sys_smem(n, ne, 32); }
  if (sm > (size_t)maxSmem) return -2;
  cudaStream_t st = (cudaStream_t)stream;
  if (cudaMemsetAsync(b.queue, 0, sizeof(unsigned long long), st) != cudaSuccess) return -1;
  auto go = [&](auto kernel, int threads) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    unsigned grid = persistent_grid(kernel, threads, sm, b.B);
    kernel<<<grid, threads, sm, st>>>(b.plan, o, b.values, b.derived, b.state, b.work, b.B, src, pts, npts, src2,
                                      pts2, npts2, out_x, out_status, out_points, out_iters, dl, b.queue);
  };
  if (T == 64) go(k_dc_sweep<64>, 64);
  else go(k_dc_sweep<32>, 32);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}
