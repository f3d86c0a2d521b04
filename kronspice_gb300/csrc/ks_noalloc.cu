// ks_noalloc.cu — batched operating point that allocates no device memory.
//
// ks_op needs a batch (ks_batch_create), which cudaMallocs the per-circuit
// working arrays.  Some callers cannot allocate device memory at the time they
// solve: code running under a memory pool or arena that owns every byte of the
// device and forbids other allocations, code on a path where an allocation may
// synchronise the device or fail under memory pressure, and hosts that budget
// device memory up front.  ks_op_noalloc serves them: the caller passes its
// inputs and outputs in device memory, and every intermediate array (the
// element table, the circuits' values in column layout, derived constants,
// device state, Newton work columns and the work-queue counter) lives in one
// file-scope __device__ array of KS_NOALLOC_SCRATCH_BYTES, which each GPU that
// loads the library holds until the process exits.
//
// The scratch array is shared by every call on a device and keeps the last
// call's contents; each call rewrites everything it reads before reading it
// (values, derived constants, element table, per-circuit state) and clears the
// work-queue counter itself.  Calls whose kernels overlap on the GPU (two
// streams, or two host threads) race on the array: serialise them.
//
// The first call on a device looks up the array's device address
// (cudaGetSymbolAddress) with that device current; make that first call before
// capturing a stream, so the look-up is not part of a capture.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "ks_internal.h"

using ksh::set_error;

// 64 MiB (KS_NOALLOC_SCRATCH_BYTES): 16,384 BJT common-emitter circuits take
// 22 MiB; a two-stage op-amp with eight MOSFETs takes 12 KiB, so about 5,300 fit.
static __device__ __align__(256) unsigned char g_noalloc_scratch[KS_NOALLOC_SCRATCH_BYTES];

namespace {

std::mutex g_mu;
// Device address of g_noalloc_scratch, per device ordinal, looked up once per
// process.  A cudaDeviceReset ends the context this address belongs to: a
// process that resets a device must not call ks_op_noalloc on it again.
void* g_scratch_dev[64];

// Device address of the scratch array on the current device (set-up on the
// device's first call).
int scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) { set_error(std::string("ks_op_noalloc: ") + cudaGetErrorString(e)); return KS_ECUDA; }
  if (dev < 0 || dev >= 64) { set_error("ks_op_noalloc: device ordinal above 63"); return KS_EUNSUPPORTED; }
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_dev[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      set_error(std::string("ks_op_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      return KS_ECUDA;
    }
    g_scratch_dev[dev] = p;
  }
  *out = g_scratch_dev[dev];
  return KS_OK;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

KOpts ks_kopts_from(const ks_options* o);

extern "C" int ks_op_noalloc_scratch_bytes(const ks_topology* topo, int32_t n_circ, size_t* bytes) {
  if (!topo || n_circ <= 0 || !bytes) { set_error("ks_op_noalloc_scratch_bytes: bad argument"); return KS_EINVAL; }
  ksh::HostPlan hp;
  std::string err;
  int rc = ksh::plan_layout(topo, &hp, &err);
  if (rc) { set_error(err); return rc; }
  size_t B = (size_t)n_circ;
  *bytes = align256(sizeof(KElem) * hp.n_elem) + align256((size_t)hp.n + 8) +
           align256(sizeof(double) * hp.n_values * B) + align256(sizeof(double) * (hp.n_derived + 1) * B) +
           align256(sizeof(double) * (hp.n_state + 1) * B) + align256(sizeof(double) * (3 * hp.n + 1) * B) + 256;
  return KS_OK;
}

extern "C" int ks_op_noalloc(const ks_topology* topo, int32_t n_circ, const double* values_dev,
                             const ks_options* opt, double* out_x_dev, int32_t* out_status_dev,
                             int32_t* out_iters_dev, void* stream) {
  if (!topo || n_circ <= 0 || !values_dev || !out_x_dev || !out_status_dev) {
    set_error("ks_op_noalloc: bad argument");
    return KS_EINVAL;
  }
  if (opt && opt->backend == KS_BACKEND_SPECIALIZED) {
    set_error("ks_op_noalloc: runs the generic kernel only (loading the per-topology kernels allocates device memory)");
    return KS_EUNSUPPORTED;
  }
  ksh::HostPlan hp;
  std::string err;
  int rc = ksh::plan_layout(topo, &hp, &err);
  if (rc) { set_error(err); return rc; }
  if (hp.n > KS_MAX_DENSE) {
    set_error("ks_op_noalloc: " + std::to_string(hp.n) + " unknowns; the thread-per-circuit kernels take up to " +
              std::to_string(KS_MAX_DENSE));
    return KS_EUNSUPPORTED;
  }
  size_t need = 0;
  rc = ks_op_noalloc_scratch_bytes(topo, n_circ, &need);
  if (rc) return rc;
  if (need > (size_t)KS_NOALLOC_SCRATCH_BYTES) {
    set_error("ks_op_noalloc: " + std::to_string(n_circ) + " circuits of this topology need " + std::to_string(need) +
              " bytes of scratch; the library's fixed scratch holds " + std::to_string((size_t)KS_NOALLOC_SCRATCH_BYTES) +
              " (split the batch, or use ks_batch_create + ks_op)");
    return KS_EINVAL;
  }
  void* base = nullptr;
  rc = scratch_address(&base);
  if (rc) return rc;

  // carve the scratch: element table, is-voltage flags, values, derived, state, work, queue counter
  const size_t B = (size_t)n_circ;
  unsigned char* p = static_cast<unsigned char*>(base);
  KElem* d_elem = reinterpret_cast<KElem*>(p);
  p += align256(sizeof(KElem) * hp.n_elem);
  int8_t* d_isv = reinterpret_cast<int8_t*>(p);
  p += align256((size_t)hp.n + 8);
  KsDeviceBatch b{};
  b.values = reinterpret_cast<double*>(p);
  p += align256(sizeof(double) * hp.n_values * B);
  b.derived = reinterpret_cast<double*>(p);
  p += align256(sizeof(double) * (hp.n_derived + 1) * B);
  b.state = reinterpret_cast<double*>(p);
  p += align256(sizeof(double) * (hp.n_state + 1) * B);
  b.work = reinterpret_cast<double*>(p);
  p += align256(sizeof(double) * (3 * hp.n + 1) * B);
  b.queue = reinterpret_cast<unsigned long long*>(p);
  b.B = n_circ;
  b.plan.n = hp.n; b.plan.n_elem = hp.n_elem; b.plan.n_values = hp.n_values; b.plan.n_derived = hp.n_derived;
  b.plan.n_state = hp.n_state; b.plan.n_nodes = hp.n_nodes; b.plan.n_nonlin = hp.n_nonlin;
  b.plan.n_reactive = hp.n_reactive; b.plan.elem = d_elem; b.plan.is_v = d_isv;

  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // the element table goes through the stream, so overlapping calls on one stream stay ordered
  cudaError_t e = cudaMemcpyAsync(d_elem, hp.elem.data(), sizeof(KElem) * hp.n_elem, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_isv, hp.is_v.data(), (size_t)hp.n, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // host vectors go out of scope on return
  if (e != cudaSuccess) { set_error(std::string("ks_op_noalloc: ") + cudaGetErrorString(e)); return KS_ECUDA; }
  if (ks_launch_transpose(values_dev, b.values, (int64_t)n_circ, hp.n_values, st) ||
      ks_launch_setup(b, 0.0, 0.0, st)) {
    set_error(std::string("ks_op_noalloc: launch failed: ") + cudaGetErrorString(cudaGetLastError()));
    return KS_ECUDA;
  }
  KOpts o = ks_kopts_from(opt);
  // the generic kernel: the per-topology kernels load code, which allocates device memory
  rc = ks_launch_op(b, o, nullptr, out_x_dev, out_status_dev, out_iters_dev, opt ? opt->deadline_s : 0.0, st,
                    nullptr);
  if (rc == -2) { set_error("ks_op_noalloc: system too large for the dense kernels"); return KS_EUNSUPPORTED; }
  if (rc) { set_error(std::string("ks_op_noalloc: kernel launch failed: ") + cudaGetErrorString(cudaGetLastError())); return KS_ECUDA; }
  return KS_OK;
}
