// ks_peak.cu — FP64 throughput of the current device, the denominator of the
// FP64 roofline fractions the engine's benchmarks report for its FP64-issue-bound
// kernels (the device's HBM and tensor peaks are measured elsewhere; its FP64
// rate is not).
//
// Every SM runs 16 warps (four per sub-partition), each lane eight independent
// FMA chains, so the FP64 pipe of every sub-partition always has an instruction
// ready; the rate is the FMAs issued over the kernel's event time.
#include <cuda_runtime.h>

#include <string>

#include "ks_internal.h"

namespace {

__global__ void k_fp64_rate(int iters, double b, double c, double* out) {
  double a0 = threadIdx.x * 1e-3, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6,
         a7 = a0 + 7;
  for (int i = 0; i < iters; i++) {
    a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
    a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
  }
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

}  // namespace

extern "C" int ks_fp64_peak(double* flops_per_s, double* fma_per_clk_per_sm) {
  if (!flops_per_s) { ksh::set_error("ks_fp64_peak: null argument"); return KS_EINVAL; }
  int dev = 0, sms = 0, khz = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) { ksh::set_error("ks_fp64_peak: no CUDA device"); return KS_ECUDA; }
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, dev);
  const int threads = 512, iters = 4096;
  double* out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  std::string err;
  float best = 0.0f;
  if (cudaMalloc(&out, sizeof(double) * threads * sms) != cudaSuccess) {
    ksh::set_error("ks_fp64_peak: device allocation failed");
    return KS_ENOMEM;
  }
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) err = "event creation";
  for (int rep = 0; rep < 4 && err.empty(); rep++) {  // the first run warms up; the fastest counts
    cudaEventRecord(e0);
    k_fp64_rate<<<sms, threads>>>(iters, 1.0000001, 1e-9, out);
    cudaEventRecord(e1);
    if (cudaEventSynchronize(e1) != cudaSuccess) { err = "kernel"; break; }
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms > 0 && (best == 0.0f || ms < best)) best = ms;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(out);
  if (!err.empty() || best <= 0.0f) {
    ksh::set_error("ks_fp64_peak: " + (err.empty() ? std::string("no time measured") : err));
    return KS_ECUDA;
  }
  const double fmas = (double)sms * threads * iters * 8;
  *flops_per_s = 2.0 * fmas / (best * 1e-3);
  if (fma_per_clk_per_sm) *fma_per_clk_per_sm = fmas / sms / (best * 1e-3 * khz * 1e3);
  return KS_OK;
}
