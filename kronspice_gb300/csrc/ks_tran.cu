// ks_tran.cu — launch of the generic batched transient kernel of the GB300 engine.
#include <cuda_runtime.h>
#include "ks_internal.h"
#include "ks_results.cuh"

using namespace ksg;

// R: with the element results and the energy ledger of every point (ks_results.cuh).
template <int T, bool R>
__global__ void __launch_bounds__(T) k_tran(KPlan plan, KOpts o, TranSpecK sp, const double* __restrict__ values,
                                            const double* __restrict__ derived, double* state, double* work, int64_t B,
                                            double* out_time, double* out_wave, int32_t* out_npts, int32_t* out_status,
                                            int32_t* out_steps, int32_t* out_iters, uint64_t deadline_ns,
                                            unsigned long long* queue) {
  extern __shared__ __align__(16) unsigned char smem[];
  Thr<SmemSys<T>, RtProg> t;
  smem_layout<T>(t, plan, smem);
  t.o = o;
  __syncthreads();
  tran_persistent<SmemSys<T>, RtProg, R>(t, sp, values, derived, state, work, B, out_time, out_wave, out_npts,
                                         out_status, out_steps, out_iters, deadline_ns, queue);
}

int ks_launch_tran(const KsDeviceBatch& b, const KOpts& o, const ks_tran_spec& spec, int cap, double* out_time,
                   double* out_wave, int32_t* out_npts, int32_t* out_status, int32_t* out_steps, int32_t* out_iters,
                   double deadline_s, void* stream, const KsSpec* kspec) {
  int n = b.plan.n, ne = b.plan.n_elem;
  if (n > KS_MAX_DENSE) return -2;
  TranSpecK sp;
  sp.step = spec.step; sp.stop = spec.stop; sp.start = spec.start;
  sp.maxStep = spec.max_step;
  if (sp.maxStep == 0) sp.maxStep = fmin(spec.step, (spec.stop - spec.start) / 50);  // analysis/tran.go:96-100
  sp.fixed = spec.fixed_step != 0;
  if (sp.fixed) sp.maxStep = spec.step;
  sp.minStep = spec.min_step > 0 ? spec.min_step : 1e-12 * spec.stop;
  sp.chgtol = spec.chgtol > 0 ? spec.chgtol : 1e-14;
  sp.trtol = spec.trtol > 0 ? spec.trtol : 7;
  sp.uic = spec.uic;
  sp.method = spec.method == KS_METHOD_BE ? BE : TRAP;
  sp.maxSteps = spec.max_steps > 0 ? spec.max_steps : 1000000;
  sp.cap = cap;
  sp.npts = (int)llround(spec.stop / spec.step) + 1;
  uint64_t dl = deadline_s > 0 ? (uint64_t)(deadline_s * 1e9) : 0;
  const bool res = o.res_scratch != nullptr;  // results: the generic kernels' results instantiation
  if (kspec && !res) {  // per-topology kernel of the plan (ks_jit.cpp)
    if (cudaMemsetAsync(b.queue, 0, sizeof(unsigned long long), (cudaStream_t)stream) != cudaSuccess) return -1;
    KOpts ko = o;
    const double *values = b.values, *derived = b.derived;
    double *state = b.state, *work = b.work;
    int64_t B = b.B;
    unsigned long long* queue = b.queue;
    void* args[] = {&ko, &sp, &values, &derived, &state, &work, &B, &out_time, &out_wave, &out_npts,
                    &out_status, &out_steps, &out_iters, &dl, &queue};
    int64_t need = (B + (int64_t)kspec->T * circuits_per_thread() - 1) / ((int64_t)kspec->T * circuits_per_thread());
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
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  auto go = [&](auto kernel, int threads) {
    int per = 0;
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, sm);
    int64_t need = (b.B + (int64_t)threads * circuits_per_thread() - 1) / ((int64_t)threads * circuits_per_thread());
    int64_t cap_blocks = (int64_t)sms * (per > 0 ? per : 1);
    unsigned grid = (unsigned)(need < cap_blocks ? need : cap_blocks);
    kernel<<<grid, threads, sm, st>>>(b.plan, o, sp, b.values, b.derived, b.state, b.work, b.B, out_time, out_wave,
                                      out_npts, out_status, out_steps, out_iters, dl, b.queue);
  };
  if (T == 64) res ? go(k_tran<64, true>, 64) : go(k_tran<64, false>, 64);
  else res ? go(k_tran<32, true>, 32) : go(k_tran<32, false>, 32);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}
