// ks_api.cu — C ABI of the GB300 engine (include/kronspice_gpu.h): plans, batches,
// operating points.  Plans own device copies of the compiled element program; a
// batch owns the SoA value, derived-constant, state and work arrays of its
// circuits and one CUDA stream.  Host buffers are staged through pinned memory.
#include <cuda_runtime.h>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>
#include <algorithm>
#include <cstdlib>
#include <map>
#include "ks_internal.h"

using ksh::set_error;

struct ks_plan {
  ksh::HostPlan hp;
  KElem* d_elem = nullptr;
  int8_t* d_isv = nullptr;
  std::mutex spec_mu;                  // per-topology kernels, per device
  std::map<std::pair<int, int>, KsSpec> spec;           // (device, kind)
  std::map<std::pair<int, int>, std::string> spec_err;  // compile failure (not retried)
  // the autotuner's choices, per (analysis kind, power-of-two bucket of the batch size)
  struct Tuned { int backend, cpt, kernel; double ms; };
  std::mutex tune_mu;
  std::map<std::pair<int, int>, Tuned> tuned;
  KPlan view() const {
    KPlan p;
    p.n = hp.n; p.n_elem = hp.n_elem; p.n_values = hp.n_values; p.n_derived = hp.n_derived;
    p.n_state = hp.n_state; p.n_nodes = hp.n_nodes; p.n_nonlin = hp.n_nonlin; p.n_reactive = hp.n_reactive;
    p.elem = d_elem; p.is_v = d_isv;
    return p;
  }
};

struct ks_batch {
  ks_plan* plan = nullptr;
  int64_t B = 0;
  KsDeviceBatch dev{};
  double* d_rows = nullptr;  // staging for row-major uploads [B][n_values]
  cudaStream_t stream = nullptr;
  // output staging
  double* d_x = nullptr;
  double* d_x0 = nullptr;
  int32_t* d_status = nullptr;
  int32_t* d_iters = nullptr;
  double* h_pin = nullptr;
  size_t h_pin_bytes = 0;
  double setup_step = -1, setup_stop = -1;  // analysis the derived constants were made for
  int last_kernel = -1;                       // KS_KERNEL_* of the last launch
  // ks_tran's device staging, kept between calls (grow only)
  double* d_wave = nullptr;
  size_t d_wave_elems = 0;
  double* d_time = nullptr;
  size_t d_time_elems = 0;
  int32_t* d_tints = nullptr;
  // ks_ac's device scratch (operating point, G / C / b columns, status, first
  // failing frequency) and output, kept between calls (grow only)
  unsigned char* d_ac = nullptr;
  size_t d_ac_bytes = 0;
  double* d_acout = nullptr;
  size_t d_acout_bytes = 0;
  // cancel word (ks_batch_cancel_word): page-locked, mapped for the device
  int32_t* h_cancel = nullptr;
  int32_t* d_cancel = nullptr;
  // results (ks_op_results, ks_tran_results): the state copy of the round-off
  // load [n_state][B], and the host calls' device output staging (grow only)
  void* d_res_scratch = nullptr;
  size_t d_res_scratch_bytes = 0;
  void* d_res_out = nullptr;
  size_t d_res_out_bytes = 0;
};

// Element results and ledger outputs of one call (device pointers; on: the
// results instantiation of the generic kernels runs).
struct ResOut {
  double* elem = nullptr;
  double* ledger = nullptr;
  double* summary = nullptr;
  bool on = false;
};

// Derived constants for an analysis with print step / stop time (0, 0 outside a transient).
static int batch_setup(ks_batch* b, double step, double stop, cudaStream_t st) {
  if (b->setup_step == step && b->setup_stop == stop) return KS_OK;
  if (ks_launch_setup(b->dev, step, stop, st)) { set_error("setup kernel launch failed"); return KS_ECUDA; }
  b->setup_step = step;
  b->setup_stop = stop;
  return KS_OK;
}

#define CK(call)                                                                            \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess) {                                                                \
      set_error(std::string("CUDA: ") + cudaGetErrorString(e_) + " at " #call);            \
      return KS_ECUDA;                                                                      \
    }                                                                                       \
  } while (0)

static KOpts make_opts(const ks_options* o) {  // analysis/op.go:91-110
  KOpts k{};
  k.reltol = o && o->reltol > 0 ? o->reltol : 1e-3;
  k.abstol = o && o->abstol > 0 ? o->abstol : 1e-12;
  k.vntol = o && o->vntol > 0 ? o->vntol : 1e-6;
  k.gmin = o && o->gmin > 0 ? o->gmin : 1e-12;
  k.itl1 = o && o->itl1 > 0 ? o->itl1 : 100;
  k.itl4 = o && o->itl4 > 0 ? o->itl4 : 10;
  k.no_gmin = o ? o->no_gmin_stepping : 0;
  k.no_source = o ? o->no_source_stepping : 0;
  k.no_pt = o ? o->no_pseudo_transient : 0;
  k.mixed = o ? (o->precision == KS_PREC_MIXED) : 0;
  k.passes = o && o->mixed_passes > 0 ? std::min(o->mixed_passes, 8) : 6;
  // refinement stops three orders under the Newton tolerance (nonlinear circuits;
  // linear ones, whose single solve per point is final, refine to 1e-11)
  k.refine_tol = std::min(1e-9, 1e-3 * k.reltol);
  k.max_iter_total = o ? o->max_iter_total : 0;
  k.start32 = o && o->fp32_start_iters > 0 ? std::min(o->fp32_start_iters, 100000) : 0;
  k.start_check = o && o->start_check > 0 ? o->start_check : 0.0;
  k.predict = o && o->step_predictor > 0 ? 1 : 0;
  return k;
}

// The autotuner's batch-size bucket: floor(log2(B)).
static int size_bucket(int64_t B) {
  int k = 0;
  while (k < 62 && ((int64_t)1 << (k + 1)) <= B) k++;
  return k;
}

// The options as the kernels read them, for the other translation units.
KOpts ks_kopts_from(const ks_options* o) { return make_opts(o); }

extern "C" int ks_plan_create(const ks_topology* topo, ks_plan** out) {
  if (!topo || !out) { set_error("ks_plan_create: null argument"); return KS_EINVAL; }
  ks_plan* p = new ks_plan();
  std::string err;
  int rc = ksh::plan_layout(topo, &p->hp, &err);
  if (rc) { set_error(err); delete p; return rc; }
  if (p->hp.n > KS_MAX_DENSE) {
    set_error("ks_plan_create: " + std::to_string(p->hp.n) + " unknowns; the thread-per-circuit kernels take up to " +
              std::to_string(KS_MAX_DENSE));
    delete p;
    return KS_EUNSUPPORTED;
  }
  *out = p;
  return KS_OK;
}

extern "C" void ks_plan_destroy(ks_plan* p) {
  if (!p) return;
  if (p->d_elem) cudaFree(p->d_elem);
  if (p->d_isv) cudaFree(p->d_isv);
  delete p;
}

extern "C" int ks_plan_info(const ks_plan* p, int32_t* n_unknowns, int32_t* n_values, int32_t* n_state) {
  if (!p) return KS_EINVAL;
  if (n_unknowns) *n_unknowns = p->hp.n;
  if (n_values) *n_values = p->hp.n_values;
  if (n_state) *n_state = p->hp.n_state;
  return KS_OK;
}

static int batch_stage(ks_batch* b, size_t bytes) {
  if (b->h_pin_bytes >= bytes) return KS_OK;
  if (b->h_pin) cudaFreeHost(b->h_pin);
  b->h_pin = nullptr;
  b->h_pin_bytes = 0;
  CK(cudaMallocHost(&b->h_pin, bytes));
  b->h_pin_bytes = bytes;
  return KS_OK;
}

// Device copy of the element program, made with the plan's first batch (a plan
// itself is host-only symbolic work).
static int plan_upload(ks_plan* p) {
  std::lock_guard<std::mutex> lk(p->spec_mu);
  if (p->d_elem) return KS_OK;
  KElem* de = nullptr;
  int8_t* di = nullptr;
  if (cudaMalloc(&de, sizeof(KElem) * p->hp.n_elem) != cudaSuccess || cudaMalloc(&di, p->hp.n + 8) != cudaSuccess) {
    set_error("ks_batch_create: device allocation for the plan failed");
    cudaFree(de);
    return KS_ENOMEM;
  }
  if (cudaMemcpy(de, p->hp.elem.data(), sizeof(KElem) * p->hp.n_elem, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(di, p->hp.is_v.data(), p->hp.n, cudaMemcpyHostToDevice) != cudaSuccess) {
    set_error("ks_batch_create: plan upload failed");
    cudaFree(de);
    cudaFree(di);
    return KS_ECUDA;
  }
  p->d_elem = de;
  p->d_isv = di;
  return KS_OK;
}

extern "C" int ks_batch_create(ks_plan* plan, int32_t n_circ, const double* values, ks_batch** out) {
  if (!plan || n_circ <= 0 || !out) { set_error("ks_batch_create: bad argument"); return KS_EINVAL; }
  int urc = plan_upload(plan);
  if (urc) return urc;
  ks_batch* b = new ks_batch();
  b->plan = plan;
  b->B = n_circ;
  const ksh::HostPlan& hp = plan->hp;
  size_t B = (size_t)n_circ;
  auto fail = [&](int rc) { ks_batch_destroy(b); return rc; };
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(KS_ECUDA);
  if (cudaMalloc(&b->dev.values, sizeof(double) * hp.n_values * B) != cudaSuccess ||
      cudaMalloc(&b->dev.derived, sizeof(double) * (hp.n_derived + 1) * B) != cudaSuccess ||
      cudaMalloc(&b->dev.state, sizeof(double) * (hp.n_state + 1) * B) != cudaSuccess ||
      cudaMalloc(&b->dev.work, sizeof(double) * (3 * hp.n + 1) * B) != cudaSuccess ||
      cudaMalloc(&b->d_rows, sizeof(double) * hp.n_values * B) != cudaSuccess ||
      cudaMalloc(&b->d_x, sizeof(double) * hp.n * B) != cudaSuccess ||
      cudaMalloc(&b->d_x0, sizeof(double) * hp.n * B) != cudaSuccess ||
      cudaMalloc(&b->d_status, sizeof(int32_t) * B) != cudaSuccess ||
      cudaMalloc(&b->d_iters, sizeof(int32_t) * B) != cudaSuccess ||
      cudaMalloc(&b->dev.queue, 64) != cudaSuccess ||
      cudaMalloc(&b->dev.values32, sizeof(float) * hp.n_values * B) != cudaSuccess ||
      cudaMalloc(&b->dev.derived32, sizeof(float) * (hp.n_derived + 1) * B) != cudaSuccess ||
      cudaMalloc(&b->dev.state32, sizeof(float) * (hp.n_state + 1) * B) != cudaSuccess) {
    set_error("ks_batch_create: device allocation failed");
    return fail(KS_ENOMEM);
  }
  b->dev.plan = plan->view();
  b->dev.B = n_circ;
  if (values) {
    int rc = ks_batch_set_values(b, values, 0, nullptr);
    if (rc) return fail(rc);
  }
  *out = b;
  return KS_OK;
}

extern "C" int ks_batch_set_values(ks_batch* b, const double* values, int values_are_device, void* stream) {
  if (!b || !values) return KS_EINVAL;
  cudaStream_t st = stream ? (cudaStream_t)stream : b->stream;
  size_t nv = b->plan->hp.n_values;
  size_t bytes = sizeof(double) * nv * b->B;
  const double* rows = values;
  if (!values_are_device) {
    CK(cudaMemcpyAsync(b->d_rows, values, bytes, cudaMemcpyHostToDevice, st));
    rows = b->d_rows;
  }
  if (ks_launch_transpose(rows, b->dev.values, b->B, (int64_t)nv, st)) { set_error("transpose launch failed"); return KS_ECUDA; }
  b->setup_step = b->setup_stop = -1;
  int rc = batch_setup(b, 0.0, 0.0, st);
  if (rc) return rc;
  if (!stream) CK(cudaStreamSynchronize(st));
  return KS_OK;
}

extern "C" void ks_batch_destroy(ks_batch* b) {
  if (!b) return;
  cudaFree(b->dev.values); cudaFree(b->dev.derived); cudaFree(b->dev.state); cudaFree(b->dev.work);
  cudaFree(b->dev.queue);
  cudaFree(b->dev.values32); cudaFree(b->dev.derived32); cudaFree(b->dev.state32);
  cudaFree(b->d_rows); cudaFree(b->d_x); cudaFree(b->d_x0); cudaFree(b->d_status); cudaFree(b->d_iters);
  if (b->h_pin) cudaFreeHost(b->h_pin);
  cudaFree(b->d_wave);
  cudaFree(b->d_time);
  cudaFree(b->d_tints);
  cudaFree(b->d_ac);
  cudaFree(b->d_acout);
  cudaFree(b->d_res_scratch);
  cudaFree(b->d_res_out);
  if (b->h_cancel) cudaFreeHost(b->h_cancel);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

// Per-topology kernels of a plan for the current device, compiled (or loaded from
// a cache) on first use.
static int plan_spec(ks_plan* p, int kind, const KsSpec** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) { set_error("no CUDA device"); return KS_ECUDA; }
  auto key = std::make_pair(dev, kind);
  std::lock_guard<std::mutex> lk(p->spec_mu);
  auto it = p->spec.find(key);
  if (it != p->spec.end()) { *out = &it->second; return KS_OK; }
  auto ie = p->spec_err.find(key);
  if (ie != p->spec_err.end()) { set_error(ie->second); return KS_EUNSUPPORTED; }
  KsSpec k;
  std::string err;
  if (ksj::get(p->hp, kind, &k, &err)) {
    p->spec_err[key] = "per-topology kernels: " + err;
    set_error(p->spec_err[key]);
    return KS_EUNSUPPORTED;
  }
  *out = &(p->spec[key] = k);
  return KS_OK;
}

static int64_t env_int(const char* name, int64_t dflt) {
  const char* e = getenv(name);
  return e && *e ? atoll(e) : dflt;
}

// Kernel choice (ks_options.backend): the per-topology kernels always under
// KS_BACKEND_SPECIALIZED, never under KS_BACKEND_GENERIC, and under
// KS_BACKEND_AUTO for systems that fit in registers (KS_JIT_REG_MAX unknowns,
// default 6) in batches of at least KS_JIT_MIN_BATCH circuits (default 2048: the
// NVRTC compile, about ten seconds, is paid once per topology and process and
// then comes from the disk cache), unless KS_JIT=0; a failed compile then falls
// back to the generic kernels.  Larger systems stay on the generic kernels under
// AUTO: their per-topology code unrolls every element (megabytes of code for a
// few dozen devices, and as long to compile).
static int pick_kernel(ks_batch* b, const ks_options* opt, int kind, const KsSpec** out) {
  *out = nullptr;
  int backend = opt ? opt->backend : KS_BACKEND_AUTO;
  bool want = backend == KS_BACKEND_SPECIALIZED ||
              (backend != KS_BACKEND_GENERIC && env_int("KS_JIT", 1) != 0 && b->plan->hp.n <= ksj::reg_max() &&
               b->B >= env_int("KS_JIT_MIN_BATCH", 2048));
  if (want) {
    int rc = plan_spec(b->plan, kind, out);
    if (rc && backend == KS_BACKEND_SPECIALIZED) return rc;
    if (rc) *out = nullptr;
  }
  b->last_kernel = *out ? ((*out)->reg ? KS_KERNEL_SPEC_REG : KS_KERNEL_SPEC_SMEM) : KS_KERNEL_GENERIC;
  return KS_OK;
}

extern "C" int ks_plan_specialize(ks_plan* plan, int32_t analysis, int32_t* kernel, double* compile_s) {
  if (!plan || (analysis != KS_ANALYSIS_OP && analysis != KS_ANALYSIS_TRAN)) return KS_EINVAL;
  const KsSpec* k = nullptr;
  int rc = plan_spec(plan, analysis == KS_ANALYSIS_OP ? ksj::KIND_OP : ksj::KIND_TRAN, &k);
  if (rc) return rc;
  if (kernel) *kernel = k->reg ? KS_KERNEL_SPEC_REG : KS_KERNEL_SPEC_SMEM;
  if (compile_s) *compile_s = k->compile_s;
  return KS_OK;
}

extern "C" int ks_plan_kernel_source(const ks_plan* plan, int32_t analysis, char* buf, size_t cap, size_t* len) {
  if (!plan || (analysis != KS_ANALYSIS_OP && analysis != KS_ANALYSIS_TRAN)) return KS_EINVAL;
  std::string s = ksj::source(plan->hp, plan->hp.n <= ksj::reg_max() ? 32 : 64, analysis == KS_ANALYSIS_OP ? ksj::KIND_OP : ksj::KIND_TRAN, nullptr);
  if (len) *len = s.size();
  if (buf && cap) {
    size_t m = std::min(cap - 1, s.size());
    std::memcpy(buf, s.data(), m);
    buf[m] = 0;
  }
  return KS_OK;
}

extern "C" int ks_batch_last_kernel(const ks_batch* b) { return b ? b->last_kernel : -1; }

extern "C" int ks_plan_tuned(const ks_plan* plan, int32_t analysis, int64_t n_circ, int32_t* kernel, int32_t* cpt,
                             double* ms) {
  if (!plan || analysis != KS_ANALYSIS_OP || n_circ <= 0) return KS_EINVAL;
  ks_plan* p = const_cast<ks_plan*>(plan);
  std::lock_guard<std::mutex> g(p->tune_mu);
  auto it = p->tuned.find({ksj::KIND_OP, size_bucket(n_circ)});
  if (it == p->tuned.end()) return KS_EINVAL;
  if (kernel) *kernel = it->second.kernel;
  if (cpt) *cpt = it->second.cpt;
  if (ms) *ms = it->second.ms;
  return KS_OK;
}

extern "C" int ks_batch_cancel_word(ks_batch* b, volatile int32_t** word) {
  if (!b || !word) { set_error("ks_batch_cancel_word: null argument"); return KS_EINVAL; }
  if (!b->h_cancel) {
    int32_t* h = nullptr;
    int32_t* d = nullptr;
    CK(cudaHostAlloc(reinterpret_cast<void**>(&h), 64, cudaHostAllocMapped));
    *h = 0;
    cudaError_t e = cudaHostGetDevicePointer(reinterpret_cast<void**>(&d), h, 0);
    if (e != cudaSuccess) {
      cudaFreeHost(h);
      set_error(std::string("ks_batch_cancel_word: ") + cudaGetErrorString(e));
      return KS_ECUDA;
    }
    b->h_cancel = h;
    b->d_cancel = d;
  }
  *word = b->h_cancel;
  return KS_OK;
}

// Grow-only device buffer.
static int grow_dev(void** p, size_t* have, size_t need, const char* what) {
  if (*have >= need) return KS_OK;
  cudaFree(*p);
  *p = nullptr;
  *have = 0;
  if (cudaMalloc(p, need) != cudaSuccess) { set_error(std::string(what) + ": device allocation failed"); return KS_ENOMEM; }
  *have = need;
  return KS_OK;
}

// The results options of a call: output pointers, the scratch state of the
// round-off load, the ledger tolerance; the results run on the generic kernels.
static int results_opts(ks_batch* b, const ks_options* opt, const ResOut& r, KOpts* o) {
  if (!r.on) return KS_OK;
  const size_t need = sizeof(double) * (b->plan->hp.n_state + 1) * b->B;
  int rc = grow_dev(&b->d_res_scratch, &b->d_res_scratch_bytes, need, "results");
  if (rc) return rc;
  o->res_elem = r.elem; o->res_ledger = r.ledger; o->res_summary = r.summary;
  o->res_scratch = static_cast<double*>(b->d_res_scratch);
  o->ledger_tol = opt && opt->ledger_tol > 0 ? opt->ledger_tol : 1e-9;  // em.DefaultTolerance, em/energy.go:21
  o->energy_check = !(opt && opt->skip_energy_check);
  return KS_OK;
}

// The autotuner's trials for the operating points of batch b: each kernel the
// batch can run (the per-topology kernel when the plan gets one, the generic
// kernel) with 1, 2 and 4 circuits per thread of the persistent grid, run twice
// on the batch's own circuits (outputs into the caller's buffers) and timed by
// CUDA events on the second run; the fastest wins.
static int op_autotune(ks_batch* b, const ks_options* opt, const KOpts& base, const double* x0_dev, double* out_x_dev,
                       int32_t* out_status_dev, int32_t* out_iters_dev, cudaStream_t st, ks_plan::Tuned* best) {
  ks_options oo = opt ? *opt : ks_options{};
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    set_error("ks_op: autotune: event creation failed");
    return KS_ECUDA;
  }
  best->ms = -1;
  int rc = KS_OK;
  for (int be : {KS_BACKEND_SPECIALIZED, KS_BACKEND_GENERIC}) {
    oo.backend = be;
    const KsSpec* ks = nullptr;
    if (pick_kernel(b, &oo, ksj::KIND_OP, &ks) != KS_OK || (be == KS_BACKEND_SPECIALIZED && !ks)) continue;
    for (int cpt : {1, 2, 4}) {
      KOpts o = base;
      o.cpt = cpt;
      float ms = -1;
      for (int rep = 0; rep < 2 && !rc; rep++) {
        cudaEventRecord(e0, st);
        const int lr = ks_launch_op(b->dev, o, x0_dev, out_x_dev, out_status_dev, out_iters_dev,
                                    opt ? opt->deadline_s : 0.0, st, ks);
        cudaEventRecord(e1, st);
        if (lr == -2) { ms = -1; break; }  // too large for this kernel: not a candidate
        if (lr || cudaEventSynchronize(e1) != cudaSuccess) {
          set_error(std::string("ks_op: autotune: ") + cudaGetErrorString(cudaGetLastError()));
          rc = KS_ECUDA;
          break;
        }
        cudaEventElapsedTime(&ms, e0, e1);
      }
      if (rc) break;
      if (ms >= 0 && (best->ms < 0 || ms < best->ms)) {
        best->backend = be; best->cpt = cpt; best->ms = ms;
        best->kernel = ks ? (ks->reg ? KS_KERNEL_SPEC_REG : KS_KERNEL_SPEC_SMEM) : KS_KERNEL_GENERIC;
      }
    }
    if (rc) break;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (!rc && best->ms < 0) { set_error("ks_op: system too large for the dense kernels"); rc = KS_EUNSUPPORTED; }
  return rc;
}

static int op_async(ks_batch* b, const ks_options* opt, const double* x0_dev, double* out_x_dev,
                    int32_t* out_status_dev, int32_t* out_iters_dev, const ResOut& res, void* stream) {
  if (!b) return KS_EINVAL;
  cudaStream_t st = stream ? (cudaStream_t)stream : b->stream;
  KOpts o = make_opts(opt);
  o.cancel = b->d_cancel;
  const KsSpec* ks = nullptr;
  int rc = KS_OK;
  if (res.on) {
    rc = results_opts(b, opt, res, &o);
    if (rc) return rc;
    const size_t ne = b->plan->hp.n_elem;
    if (res.elem) CK(cudaMemsetAsync(res.elem, 0, sizeof(double) * KS_RES_COLS * ne * b->B, st));
    if (res.ledger) CK(cudaMemsetAsync(res.ledger, 0, sizeof(double) * KS_LEDGER_COLS * b->B, st));
    b->last_kernel = KS_KERNEL_GENERIC;
  } else if (opt && opt->autotune > 0) {
    const std::pair<int, int> key{ksj::KIND_OP, size_bucket(b->B)};
    ks_plan::Tuned t{};
    bool have = false;
    {
      std::lock_guard<std::mutex> g(b->plan->tune_mu);
      auto it = b->plan->tuned.find(key);
      if (it != b->plan->tuned.end()) { t = it->second; have = true; }
    }
    if (!have) {
      rc = batch_setup(b, 0.0, 0.0, st);
      if (!rc) rc = op_autotune(b, opt, o, x0_dev, out_x_dev, out_status_dev, out_iters_dev, st, &t);
      if (rc) return rc;
      std::lock_guard<std::mutex> g(b->plan->tune_mu);
      b->plan->tuned[key] = t;
    }
    ks_options oo = *opt;
    oo.backend = t.backend;
    rc = pick_kernel(b, &oo, ksj::KIND_OP, &ks);
    o.cpt = t.cpt;
  } else {
    rc = pick_kernel(b, opt, ksj::KIND_OP, &ks);
  }
  if (rc) return rc;
  rc = batch_setup(b, 0.0, 0.0, st);
  if (rc) return rc;
  rc = ks_launch_op(b->dev, o, x0_dev, out_x_dev, out_status_dev, out_iters_dev, opt ? opt->deadline_s : 0.0, st, ks);
  if (rc == -2) { set_error("ks_op: system too large for the dense kernels"); return KS_EUNSUPPORTED; }
  if (rc && ks) return KS_ECUDA;  // message set by the launcher
  if (rc) { set_error(std::string("op kernel launch failed: ") + cudaGetErrorString(cudaGetLastError())); return KS_ECUDA; }
  return KS_OK;
}

extern "C" int ks_op_async(ks_batch* b, const ks_options* opt, const double* x0_dev, double* out_x_dev,
                           int32_t* out_status_dev, int32_t* out_iters_dev, void* stream) {
  return op_async(b, opt, x0_dev, out_x_dev, out_status_dev, out_iters_dev, ResOut{}, stream);
}

extern "C" int ks_op_results_async(ks_batch* b, const ks_options* opt, const double* x0_dev, double* out_x_dev,
                                   int32_t* out_status_dev, int32_t* out_iters_dev, double* out_elem_dev,
                                   double* out_ledger_dev, void* stream) {
  ResOut r;
  r.elem = out_elem_dev; r.ledger = out_ledger_dev; r.on = true;
  return op_async(b, opt, x0_dev, out_x_dev, out_status_dev, out_iters_dev, r, stream);
}

// ks_op / ks_op_results on host buffers: results staged on the device, copied
// back through the batch's page-locked buffer.
static int op_host(ks_batch* b, const ks_options* opt, const double* x0, double* out_x, int32_t* out_status,
                   int32_t* out_iters, double* out_elem, double* out_ledger, bool results, void* stream) {
  if (!b) return KS_EINVAL;
  cudaStream_t st = stream ? (cudaStream_t)stream : b->stream;
  const ksh::HostPlan& hp = b->plan->hp;
  size_t B = b->B, n = hp.n;
  size_t xbytes = sizeof(double) * n * B;
  size_t ebytes = results && out_elem ? sizeof(double) * KS_RES_COLS * hp.n_elem * B : 0;
  size_t lbytes = results && out_ledger ? sizeof(double) * KS_LEDGER_COLS * B : 0;
  int rc = batch_stage(b, xbytes + 2 * sizeof(int32_t) * B + ebytes + lbytes + 64);
  if (rc) return rc;
  ResOut r;
  if (results) {
    rc = grow_dev(&b->d_res_out, &b->d_res_out_bytes, ebytes + lbytes + 64, "ks_op_results");
    if (rc) return rc;
    r.on = true;
    r.elem = ebytes ? static_cast<double*>(b->d_res_out) : nullptr;
    r.ledger = lbytes ? reinterpret_cast<double*>(static_cast<char*>(b->d_res_out) + ebytes) : nullptr;
  }
  if (x0) {
    std::memcpy(b->h_pin, x0, xbytes);
    CK(cudaMemcpyAsync(b->d_x0, b->h_pin, xbytes, cudaMemcpyHostToDevice, st));
  }
  rc = op_async(b, opt, x0 ? b->d_x0 : nullptr, b->d_x, b->d_status, b->d_iters, r, st);
  if (rc) return rc;
  char* hp_bytes = reinterpret_cast<char*>(b->h_pin);
  const size_t so = xbytes, io = so + sizeof(int32_t) * B, eo = io + sizeof(int32_t) * B, lo = eo + ebytes;
  CK(cudaMemcpyAsync(hp_bytes, b->d_x, xbytes, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(hp_bytes + so, b->d_status, sizeof(int32_t) * B, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(hp_bytes + io, b->d_iters, sizeof(int32_t) * B, cudaMemcpyDeviceToHost, st));
  if (ebytes) CK(cudaMemcpyAsync(hp_bytes + eo, r.elem, ebytes, cudaMemcpyDeviceToHost, st));
  if (lbytes) CK(cudaMemcpyAsync(hp_bytes + lo, r.ledger, lbytes, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (out_x) std::memcpy(out_x, hp_bytes, xbytes);
  if (out_status) std::memcpy(out_status, hp_bytes + so, sizeof(int32_t) * B);
  if (out_iters) std::memcpy(out_iters, hp_bytes + io, sizeof(int32_t) * B);
  if (ebytes) std::memcpy(out_elem, hp_bytes + eo, ebytes);
  if (lbytes) std::memcpy(out_ledger, hp_bytes + lo, lbytes);
  return KS_OK;
}

extern "C" int ks_op(ks_batch* b, const ks_options* opt, const double* x0, double* out_x, int32_t* out_status,
                     int32_t* out_iters, void* stream) {
  return op_host(b, opt, x0, out_x, out_status, out_iters, nullptr, nullptr, false, stream);
}

extern "C" int ks_op_results(ks_batch* b, const ks_options* opt, const double* x0, double* out_x,
                             int32_t* out_status, int32_t* out_iters, double* out_elem, double* out_ledger,
                             void* stream) {
  return op_host(b, opt, x0, out_x, out_status, out_iters, out_elem, out_ledger, true, stream);
}

extern "C" int ks_dc_sweep(ks_batch* b, const ks_options* opt, int32_t src, const double* values, int32_t npts,
                           int32_t src2, const double* values2, int32_t npts2, double* out_x, int32_t* out_status,
                           int32_t* out_points, int32_t* out_iters, void* stream) {
  const bool nested = src2 >= 0;
  if (!b || !values || npts <= 0 || (nested && (!values2 || npts2 <= 0)) ||
      (int64_t)npts * (nested ? npts2 : 1) > 1000000) {  // analysis.MaxDCPoints
    set_error("ks_dc_sweep: bad argument");
    return KS_EINVAL;
  }
  const ksh::HostPlan& hp = b->plan->hp;
  auto source = [&](int e) { return e >= 0 && e < hp.n_elem && (hp.src[e].kind == KS_ELEM_V || hp.src[e].kind == KS_ELEM_I); };
  if (!source(src) || (nested && (!source(src2) || src2 == src))) {
    set_error("analysis: swept source not found");  // analysis.ErrUnknownSource, analysis/dc.go:66-76
    return KS_EINVAL;
  }
  cudaStream_t st = stream ? (cudaStream_t)stream : b->stream;
  const int64_t B = b->B, n = hp.n, total = (int64_t)npts * (nested ? npts2 : 1);
  const size_t xb = sizeof(double) * (size_t)B * total * n, pb = sizeof(double) * (npts + (nested ? npts2 : 0));
  const size_t ib = sizeof(int32_t) * B;
  char* d = nullptr;
  if (cudaMalloc(&d, xb + pb + 3 * ib + 64) != cudaSuccess) { set_error("ks_dc_sweep: device allocation failed"); return KS_ENOMEM; }
  double* d_x = reinterpret_cast<double*>(d);
  double* d_pts = reinterpret_cast<double*>(d + xb);
  double* d_pts2 = nested ? d_pts + npts : nullptr;
  int32_t* d_status = reinterpret_cast<int32_t*>(d + xb + pb);
  int32_t* d_points = d_status + B;
  int32_t* d_iters = d_points + B;
  KOpts o = make_opts(opt);
  o.cancel = b->d_cancel;
  int rc = batch_setup(b, 0.0, 0.0, st);
  if (!rc && cudaMemcpyAsync(d_pts, values, sizeof(double) * npts, cudaMemcpyHostToDevice, st) != cudaSuccess) rc = KS_ECUDA;
  if (!rc && nested && cudaMemcpyAsync(d_pts2, values2, sizeof(double) * npts2, cudaMemcpyHostToDevice, st) != cudaSuccess)
    rc = KS_ECUDA;
  if (!rc) {
    const int lr = ks_launch_dc_sweep(b->dev, o, src, d_pts, npts, nested ? src2 : -1, d_pts2, nested ? npts2 : 0, d_x,
                                      d_status, d_points, d_iters, opt ? opt->deadline_s : 0.0, st);
    if (lr == -2) { set_error("ks_dc_sweep: system too large for the dense kernels"); rc = KS_EUNSUPPORTED; }
    else if (lr) { set_error(std::string("ks_dc_sweep: kernel launch failed: ") + cudaGetErrorString(cudaGetLastError())); rc = KS_ECUDA; }
  }
  if (!rc && cudaStreamSynchronize(st) != cudaSuccess) { set_error("ks_dc_sweep: CUDA error"); rc = KS_ECUDA; }
  if (!rc) {
    if (out_x) cudaMemcpy(out_x, d_x, xb, cudaMemcpyDeviceToHost);
    if (out_status) cudaMemcpy(out_status, d_status, ib, cudaMemcpyDeviceToHost);
    if (out_points) cudaMemcpy(out_points, d_points, ib, cudaMemcpyDeviceToHost);
    if (out_iters) cudaMemcpy(out_iters, d_iters, ib, cudaMemcpyDeviceToHost);
  }
  cudaFree(d);
  return rc;
}

static int grow(void** p, size_t* have, size_t need) {
  if (*have >= need) return KS_OK;
  cudaFree(*p);
  *p = nullptr;
  *have = 0;
  if (cudaMalloc(p, need) != cudaSuccess) { set_error("ks_ac: device allocation failed"); return KS_ENOMEM; }
  *have = need;
  return KS_OK;
}

static size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

// ks_ac's device scratch: x at the operating point, status, first failing
// frequency, then the G / C / b columns.
struct AcScratch { double* x_op; int32_t* status; int32_t* err_at; double* cols; };

static int ac_scratch(ks_batch* b, AcScratch* s) {
  const int64_t B = b->B;
  const int n = b->plan->hp.n;
  const size_t xb = a256(sizeof(double) * n * B), sb = a256(sizeof(int32_t) * B);
  const size_t need = xb + 2 * sb + sizeof(double) * ks_ac_scratch_doubles(n, B);
  int rc = grow(reinterpret_cast<void**>(&b->d_ac), &b->d_ac_bytes, need);
  if (rc) return rc;
  s->x_op = reinterpret_cast<double*>(b->d_ac);
  s->status = reinterpret_cast<int32_t*>(b->d_ac + xb);
  s->err_at = reinterpret_cast<int32_t*>(b->d_ac + xb + sb);
  s->cols = reinterpret_cast<double*>(b->d_ac + xb + 2 * sb);
  return KS_OK;
}

static int ac_sweep(ks_batch* b, const KOpts& o, const double* x_op, int32_t* status, const double* freqs_dev,
                    int32_t n_freq, double* out_x_dev, const AcScratch& s, cudaStream_t st) {
  int rc = batch_setup(b, 0.0, 0.0, st);
  if (rc) return rc;
  rc = ks_launch_ac(b->dev, o.gmin, x_op, freqs_dev, n_freq, s.cols, s.err_at, status, out_x_dev, st);
  if (rc == -2) { set_error("ks_ac: system too large for the AC kernel"); return KS_EUNSUPPORTED; }
  if (rc) { set_error(std::string("ks_ac: kernel launch failed: ") + cudaGetErrorString(cudaGetLastError())); return KS_ECUDA; }
  return KS_OK;
}

extern "C" int ks_ac_async(ks_batch* b, const ks_options* opt, const double* x0_dev, const double* freqs_dev,
                           int32_t n_freq, double* out_x_dev, int32_t* out_status_dev, int32_t* out_iters_dev,
                           void* stream) {
  if (!b || n_freq <= 0 || !freqs_dev || !out_x_dev) { set_error("ks_ac: bad argument"); return KS_EINVAL; }
  cudaStream_t st = stream ? (cudaStream_t)stream : b->stream;
  AcScratch s;
  int rc = ac_scratch(b, &s);
  if (rc) return rc;
  KOpts o = make_opts(opt);
  o.cancel = b->d_cancel;
  o.polish = 1;
  const KsSpec* ks = nullptr;
  rc = pick_kernel(b, opt, ksj::KIND_OP, &ks);
  if (rc) return rc;
  rc = batch_setup(b, 0.0, 0.0, st);
  if (rc) return rc;
  rc = ks_launch_op(b->dev, o, x0_dev, s.x_op, s.status, out_iters_dev, opt ? opt->deadline_s : 0.0, st, ks);
  if (rc == -2) { set_error("ks_ac: system too large for the dense kernels"); return KS_EUNSUPPORTED; }
  if (rc && ks) return KS_ECUDA;
  if (rc) { set_error(std::string("op kernel launch failed: ") + cudaGetErrorString(cudaGetLastError())); return KS_ECUDA; }
  rc = ac_sweep(b, o, s.x_op, s.status, freqs_dev, n_freq, out_x_dev, s, st);
  if (rc) return rc;
  if (out_status_dev) CK(cudaMemcpyAsync(out_status_dev, s.status, sizeof(int32_t) * b->B, cudaMemcpyDeviceToDevice, st));
  return KS_OK;
}

extern "C" int ks_ac_at(ks_batch* b, const ks_options* opt, const double* x_op_dev, const int32_t* status_dev,
                        const double* freqs_dev, int32_t n_freq, double* out_x_dev, int32_t* out_status_dev,
                        void* stream) {
  if (!b || n_freq <= 0 || !x_op_dev || !freqs_dev || !out_x_dev || !out_status_dev) {
    set_error("ks_ac_at: bad argument");
    return KS_EINVAL;
  }
  cudaStream_t st = stream ? (cudaStream_t)stream : b->stream;
  AcScratch s;
  int rc = ac_scratch(b, &s);
  if (rc) return rc;
  if (status_dev) {
    if (status_dev != out_status_dev)
      CK(cudaMemcpyAsync(out_status_dev, status_dev, sizeof(int32_t) * b->B, cudaMemcpyDeviceToDevice, st));
  } else {
    CK(cudaMemsetAsync(out_status_dev, 0, sizeof(int32_t) * b->B, st));
  }
  return ac_sweep(b, make_opts(opt), x_op_dev, out_status_dev, freqs_dev, n_freq, out_x_dev, s, st);
}

extern "C" int ks_ac(ks_batch* b, const ks_options* opt, const double* x0, const double* freqs, int32_t n_freq,
                     double* out_x, int32_t* out_status, int32_t* out_iters, void* stream) {
  if (!b || n_freq <= 0 || !freqs) { set_error("ks_ac: bad argument"); return KS_EINVAL; }
  cudaStream_t st = stream ? (cudaStream_t)stream : b->stream;
  const size_t B = b->B, n = b->plan->hp.n;
  const size_t xbytes = sizeof(double) * n * B, obytes = sizeof(double) * 2 * n * B * (size_t)n_freq;
  const size_t fbytes = sizeof(double) * (size_t)n_freq;
  const size_t fb = a256(fbytes);
  int rc = grow(reinterpret_cast<void**>(&b->d_acout), &b->d_acout_bytes, a256(obytes) + fb);
  if (rc) return rc;
  double* d_freq = reinterpret_cast<double*>(reinterpret_cast<unsigned char*>(b->d_acout) + a256(obytes));
  rc = batch_stage(b, std::max(obytes, std::max(xbytes, fbytes)) + 2 * sizeof(int32_t) * B + 64);
  if (rc) return rc;
  std::memcpy(b->h_pin, freqs, fbytes);
  CK(cudaMemcpyAsync(d_freq, b->h_pin, fbytes, cudaMemcpyHostToDevice, st));
  if (x0) {
    // after the frequencies' copy has left the staging buffer
    CK(cudaStreamSynchronize(st));
    std::memcpy(b->h_pin, x0, xbytes);
    CK(cudaMemcpyAsync(b->d_x0, b->h_pin, xbytes, cudaMemcpyHostToDevice, st));
  }
  rc = ks_ac_async(b, opt, x0 ? b->d_x0 : nullptr, d_freq, n_freq, b->d_acout, b->d_status, b->d_iters, st);
  if (rc) return rc;
  // page-locked output (cudaHostAlloc / cudaHostRegister) takes the phasors
  // directly; pageable output goes through the batch's pinned staging
  cudaPointerAttributes pa{};
  const bool pinned_out = out_x && cudaPointerGetAttributes(&pa, out_x) == cudaSuccess && pa.type == cudaMemoryTypeHost;
  cudaGetLastError();  // a pageable pointer may leave an error behind on older drivers
  char* hp_bytes = reinterpret_cast<char*>(b->h_pin);
  const size_t xoff = pinned_out ? 0 : obytes;
  if (pinned_out) CK(cudaMemcpyAsync(out_x, b->d_acout, obytes, cudaMemcpyDeviceToHost, st));
  else if (out_x) CK(cudaMemcpyAsync(hp_bytes, b->d_acout, obytes, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(hp_bytes + xoff, b->d_status, sizeof(int32_t) * B, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(hp_bytes + xoff + sizeof(int32_t) * B, b->d_iters, sizeof(int32_t) * B, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (out_x && !pinned_out) std::memcpy(out_x, hp_bytes, obytes);
  if (out_status) std::memcpy(out_status, hp_bytes + xoff, sizeof(int32_t) * B);
  if (out_iters) std::memcpy(out_iters, hp_bytes + xoff + sizeof(int32_t) * B, sizeof(int32_t) * B);
  return KS_OK;
}

// TranSpec check of analysis.Tran (analysis/tran.go:71-74): ErrBadTranSpec.
static bool tran_spec_ok(const ks_tran_spec* sp) {
  if (!sp) return false;
  double sum = sp->step + sp->stop + sp->start + sp->max_step;
  return sp->step > 0 && sp->stop > 0 && sp->start >= 0 && sp->start < sp->stop && sp->max_step >= 0 &&
         !std::isnan(sum) && !std::isinf(sp->stop);
}

static int tran_host(ks_batch* b, const ks_tran_spec* spec, const ks_options* opt, int32_t capacity,
                     double* out_time, double* out_wave, int32_t* out_npts, int32_t* out_status, int32_t* out_steps,
                     int32_t* out_iters, const ResOut& res, void* stream);

// Points a transient records per circuit in the output layouts: fixed-step
// n_points, adaptive the capacity.
static size_t tran_slots(const ks_tran_spec* spec, int32_t capacity) {
  return spec->fixed_step ? (size_t)llround(spec->stop / spec->step) + 1 : (size_t)std::max(capacity, 0);
}

static int tran_async(ks_batch* b, const ks_tran_spec* spec, const ks_options* opt, int32_t capacity,
                      double* out_time_dev, double* out_wave_dev, int32_t* out_npts_dev, int32_t* out_status_dev,
                      int32_t* out_steps_dev, int32_t* out_iters_dev, const ResOut& res, void* stream) {
  if (!b) return KS_EINVAL;
  if (!tran_spec_ok(spec)) { set_error("analysis: invalid transient specification"); return KS_EINVAL; }
  if (!spec->fixed_step && capacity <= 0 && (out_time_dev || out_wave_dev || res.elem || res.ledger)) {
    set_error("ks_tran: capacity"); return KS_EINVAL;
  }
  cudaStream_t st = stream ? (cudaStream_t)stream : b->stream;
  KOpts o = make_opts(opt);
  o.cancel = b->d_cancel;
  const KsSpec* ks = nullptr;
  int rc = KS_OK;
  if (res.on) {
    rc = results_opts(b, opt, res, &o);
    if (rc) return rc;
    const size_t slots = tran_slots(spec, capacity) * b->B, ne = b->plan->hp.n_elem;
    if (res.elem) CK(cudaMemsetAsync(res.elem, 0, sizeof(double) * 2 * ne * slots, st));
    if (res.ledger) CK(cudaMemsetAsync(res.ledger, 0, sizeof(double) * KS_TPOINT_COLS * slots, st));
    if (res.summary) CK(cudaMemsetAsync(res.summary, 0, sizeof(double) * KS_TSUM_COLS * b->B, st));
    b->last_kernel = KS_KERNEL_GENERIC;
  } else {
    rc = pick_kernel(b, opt, ksj::KIND_TRAN, &ks);
  }
  if (rc) return rc;
  rc = batch_setup(b, spec->step, spec->stop, st);
  if (rc) return rc;
  rc = ks_launch_tran(b->dev, o, *spec, capacity, out_time_dev, out_wave_dev, out_npts_dev, out_status_dev,
                      out_steps_dev, out_iters_dev, opt ? opt->deadline_s : 0.0, st, ks);
  if (rc == -2) { set_error("ks_tran: system too large for the dense kernels"); return KS_EUNSUPPORTED; }
  if (rc && ks) return KS_ECUDA;  // message set by the launcher
  if (rc) { set_error(std::string("tran kernel launch failed: ") + cudaGetErrorString(cudaGetLastError())); return KS_ECUDA; }
  return KS_OK;
}

extern "C" int ks_tran_async(ks_batch* b, const ks_tran_spec* spec, const ks_options* opt, int32_t capacity,
                             double* out_time_dev, double* out_wave_dev, int32_t* out_npts_dev,
                             int32_t* out_status_dev, int32_t* out_steps_dev, int32_t* out_iters_dev, void* stream) {
  return tran_async(b, spec, opt, capacity, out_time_dev, out_wave_dev, out_npts_dev, out_status_dev, out_steps_dev,
                    out_iters_dev, ResOut{}, stream);
}

extern "C" int ks_tran_results_async(ks_batch* b, const ks_tran_spec* spec, const ks_options* opt, int32_t capacity,
                                     double* out_time_dev, double* out_wave_dev, double* out_elem_dev,
                                     double* out_ledger_dev, double* out_summary_dev, int32_t* out_npts_dev,
                                     int32_t* out_status_dev, int32_t* out_steps_dev, int32_t* out_iters_dev,
                                     void* stream) {
  ResOut r;
  r.elem = out_elem_dev; r.ledger = out_ledger_dev; r.summary = out_summary_dev; r.on = true;
  return tran_async(b, spec, opt, capacity, out_time_dev, out_wave_dev, out_npts_dev, out_status_dev, out_steps_dev,
                    out_iters_dev, r, stream);
}

extern "C" int ks_tran_results(ks_batch* b, const ks_tran_spec* spec, const ks_options* opt, int32_t capacity,
                               double* out_time, double* out_wave, double* out_elem, double* out_ledger,
                               double* out_summary, int32_t* out_npts, int32_t* out_status, int32_t* out_steps,
                               int32_t* out_iters, void* stream) {
  if (!b) return KS_EINVAL;
  if (!tran_spec_ok(spec)) { set_error("analysis: invalid transient specification"); return KS_EINVAL; }
  cudaStream_t st = stream ? (cudaStream_t)stream : b->stream;
  const size_t slots = tran_slots(spec, capacity) * b->B, ne = b->plan->hp.n_elem;
  const size_t eb = out_elem ? sizeof(double) * 2 * ne * slots : 0, lb = out_ledger ? sizeof(double) * KS_TPOINT_COLS * slots : 0;
  const size_t sb = out_summary ? sizeof(double) * KS_TSUM_COLS * b->B : 0;
  int rc = grow_dev(&b->d_res_out, &b->d_res_out_bytes, eb + lb + sb + 64, "ks_tran_results");
  if (rc) return rc;
  char* base = static_cast<char*>(b->d_res_out);
  ResOut r;
  r.on = true;
  r.elem = eb ? reinterpret_cast<double*>(base) : nullptr;
  r.ledger = lb ? reinterpret_cast<double*>(base + eb) : nullptr;
  r.summary = sb ? reinterpret_cast<double*>(base + eb + lb) : nullptr;
  rc = tran_host(b, spec, opt, capacity, out_time, out_wave, out_npts, out_status, out_steps, out_iters, r, st);
  if (rc) return rc;
  cudaError_t e = cudaSuccess;
  if (eb) e = cudaMemcpyAsync(out_elem, r.elem, eb, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && lb) e = cudaMemcpyAsync(out_ledger, r.ledger, lb, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && sb) e = cudaMemcpyAsync(out_summary, r.summary, sb, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) { set_error(std::string("ks_tran_results: ") + cudaGetErrorString(e)); return KS_ECUDA; }
  return KS_OK;
}

extern "C" int ks_tran(ks_batch* b, const ks_tran_spec* spec, const ks_options* opt, int32_t capacity,
                       double* out_time, double* out_wave, int32_t* out_npts, int32_t* out_status, int32_t* out_steps,
                       int32_t* out_iters, void* stream) {
  return tran_host(b, spec, opt, capacity, out_time, out_wave, out_npts, out_status, out_steps, out_iters, ResOut{},
                   stream);
}

// ks_tran / ks_tran_results on host buffers (the results' device outputs are the caller's r).
static int tran_host(ks_batch* b, const ks_tran_spec* spec, const ks_options* opt, int32_t capacity,
                     double* out_time, double* out_wave, int32_t* out_npts, int32_t* out_status, int32_t* out_steps,
                     int32_t* out_iters, const ResOut& res, void* stream) {
  if (!b) return KS_EINVAL;
  if (!tran_spec_ok(spec)) { set_error("analysis: invalid transient specification"); return KS_EINVAL; }
  cudaStream_t st = stream ? (cudaStream_t)stream : b->stream;
  size_t B = b->B, n = b->plan->hp.n;
  size_t npts = spec->fixed_step ? (size_t)llround(spec->stop / spec->step) + 1 : 0;
  size_t wave_elems = spec->fixed_step ? npts * B * n : (size_t)std::max(capacity, 0) * B * n;
  size_t time_elems = spec->fixed_step ? 0 : (size_t)std::max(capacity, 0) * B;
  // device staging kept in the batch between calls
  auto grow = [&](double** p, size_t* have, size_t need) {
    if (need <= *have) return true;
    cudaFree(*p);
    *p = nullptr;
    *have = 0;
    if (cudaMalloc(p, need * sizeof(double)) != cudaSuccess) return false;
    *have = need;
    return true;
  };
  if (out_wave && wave_elems && !grow(&b->d_wave, &b->d_wave_elems, wave_elems)) {
    set_error("ks_tran: device allocation for the waveforms failed"); return KS_ENOMEM;
  }
  if (out_time && time_elems && !grow(&b->d_time, &b->d_time_elems, time_elems)) {
    set_error("ks_tran: device allocation failed"); return KS_ENOMEM;
  }
  if (!b->d_tints && cudaMalloc(&b->d_tints, 4 * B * sizeof(int32_t)) != cudaSuccess) {
    set_error("ks_tran: allocation failed"); return KS_ENOMEM;
  }
  double* d_wave = (out_wave && wave_elems) ? b->d_wave : nullptr;
  double* d_time = (out_time && time_elems) ? b->d_time : nullptr;
  int32_t* d_ints = b->d_tints;
  auto cleanup = [&]() {};
  int rc = tran_async(b, spec, opt, capacity, d_time, d_wave, d_ints, d_ints + B, d_ints + 2 * B, d_ints + 3 * B, res, st);
  if (rc) { cleanup(); return rc; }
  cudaError_t e = cudaSuccess;
  if (out_wave && d_wave) e = cudaMemcpyAsync(out_wave, d_wave, wave_elems * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && out_time && d_time) e = cudaMemcpyAsync(out_time, d_time, time_elems * sizeof(double), cudaMemcpyDeviceToHost, st);
  std::vector<int32_t> ints(4 * B);
  if (e == cudaSuccess) e = cudaMemcpyAsync(ints.data(), d_ints, 4 * B * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cleanup();
  if (e != cudaSuccess) { set_error(std::string("ks_tran: ") + cudaGetErrorString(e)); return KS_ECUDA; }
  if (out_npts) std::memcpy(out_npts, ints.data(), B * sizeof(int32_t));
  if (out_status) std::memcpy(out_status, ints.data() + B, B * sizeof(int32_t));
  if (out_steps) std::memcpy(out_steps, ints.data() + 2 * B, B * sizeof(int32_t));
  if (out_iters) std::memcpy(out_iters, ints.data() + 3 * B, B * sizeof(int32_t));
  return KS_OK;
}

// The batch's SoA values [n_values][B], circuit count and unknown count (for the
// learned-start kernels, which read their features from the values in place).
int ks_batch_values_view(ks_batch* b, const double** vals, int64_t* B, int* n) {
  *vals = b->dev.values;
  *B = b->B;
  *n = b->plan->hp.n;
  return KS_OK;
}
