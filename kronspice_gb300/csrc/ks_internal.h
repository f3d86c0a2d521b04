// ks_internal.h — host-side structures shared by the planner, the API and the launchers.
#pragma once
#include <stdint.h>
#include <string>
#include <vector>
#include "ks_engine.h"
#include "../../include/kronspice_gpu.h"

namespace ksh {

// Result of the symbolic pass over one topology.
struct HostPlan {
  int n_nodes = 0, n = 0, n_elem = 0, n_values = 0, n_derived = 0, n_state = 0;
  int n_nonlin = 0, n_reactive = 0, n_breakpointer = 0;
  std::vector<KElem> elem;
  std::vector<int8_t> is_v;
  std::vector<ks_element> src;  // the topology as given
};

// Unknown layout and per-element offsets (device Setup order).
int plan_layout(const ks_topology* t, HostPlan* hp, std::string* err);
// circuit.Validate / ValidateTransient for one circuit (values of that circuit).
int validate(const ks_topology* t, const double* values, bool transient, std::string* err);

void set_error(const std::string& s);

// Symbolic sparse LU of one circuit (ks_sparse.cpp): fixed pivot sequence
// (step k pivots A row prow[k] on A column q[k]) and the pattern of L + U in
// step coordinates, rows in step order, columns ascending.
struct SparseSym {
  int n = 0;
  std::vector<int> prow, q, pinv, qinv;  // step -> A row / col, A row / col -> step
  std::vector<int> rp, ci, dg;           // row pointers [n+1], column (step) of each slot, slot of each diagonal
  std::vector<uint8_t> in_a;             // slot is structurally in A (else fill)
  int64_t flops = 0;                     // multiply-adds of one numeric factorization
};
// h = 0: pivot rows chosen at DC; h > 0: with the companion models of step h.
int sparse_symbolic(const HostPlan& hp, const double* values, double h, SparseSym* sy, std::string* err);
// The reference's stamp pattern of one circuit (operating point, or transient), n x n bytes.
void sparse_pattern(const HostPlan& hp, const double* values, bool transient, uint8_t* out);

}  // namespace ksh

// Kernel launchers (ks_kernels.cu).
struct KsDeviceBatch {
  KPlan plan;          // device pointers inside
  int64_t B;           // circuits
  double* values;      // [n_values][B]
  double* derived;     // [n_derived][B]
  double* state;       // [n_state][B]
  double* work;        // [3*n][B]: save, ptPrev, xacc
  unsigned long long* queue;  // next-circuit counter of the persistent kernels
  // FP32 copies of values and derived, and the FP32 start stage's state (null:
  // no FP32 stage for this batch)
  float* values32 = nullptr;   // [n_values][B]
  float* derived32 = nullptr;  // [n_derived][B]
  float* state32 = nullptr;    // [n_state][B]
};

int ks_launch_transpose(const double* src_rows, double* dst_cols, int64_t rows, int64_t cols, void* stream);
int ks_launch_setup(const KsDeviceBatch& b, double step, double stop, void* stream);
struct KsSpec;
// Launch shape of the persistent kernels: at least this many circuits per thread
// (KS_CIRCUITS_PER_THREAD, default 1), so that a lane whose circuit converges
// takes the next one from the queue instead of idling while the rest of its warp
// iterates.
int circuits_per_thread();
// spec: the plan's per-topology kernels, or null for the generic kernels.
int ks_launch_tran(const KsDeviceBatch& b, const KOpts& o, const ks_tran_spec& spec, int cap, double* out_time,
                   double* out_wave, int32_t* out_npts, int32_t* out_status, int32_t* out_steps, int32_t* out_iters,
                   double deadline_s, void* stream, const KsSpec* kspec);
int ks_launch_dc_sweep(const KsDeviceBatch& b, const KOpts& o, int src, const double* pts, int npts, int src2,
                       const double* pts2, int npts2, double* out_x, int32_t* out_status, int32_t* out_points,
                       int32_t* out_iters, double deadline_s, void* stream);
int ks_launch_op(const KsDeviceBatch& b, const KOpts& o, const double* x0, double* out_x, int32_t* out_status,
                 int32_t* out_iters, double deadline_s, void* stream, const KsSpec* kspec);
// AC sweep after the operating point x_op [B][n] (ks_ac.cu): G / C / b columns in
// scratch (ks_ac_scratch_doubles), out_x [B][nf][n][2]; status updated with the
// first failing frequency.  -2: the system does not fit the solve kernel.
size_t ks_ac_scratch_doubles(int n, int64_t B);
int ks_launch_ac(const KsDeviceBatch& b, double gmin, const double* x_op, const double* freqs_dev, int32_t nf,
                 double* scratch, int32_t* err_at, int32_t* status, double* out_x, void* stream);

// One per-topology kernel of a plan on one device (ks_jit.cpp).
struct KsSpec {
  void* fn = nullptr;    // cudaKernel_t of ks_spec_op or ks_spec_tran
  int T = 0;             // threads per block
  size_t smem = 0;       // dynamic shared memory per block
  bool reg = false;      // system in registers (else shared memory)
  int device = -1;
  int blocks = 0;        // resident blocks over all SMs
  double compile_s = 0;  // NVRTC time (0 when the cubin came from a cache)
  bool from_disk = false;
  uint64_t key = 0;
};

namespace ksj {
enum { KIND_OP = 0, KIND_TRAN = 1 };
int reg_max();  // largest system the per-topology kernels keep in registers
std::string source(const ksh::HostPlan& hp, int T, int kind, bool* reg);
int get(const ksh::HostPlan& hp, int kind, KsSpec* out, std::string* err);
int launch(void* fn, unsigned grid, int T, size_t smem, void* stream, void** args, std::string* err);
}  // namespace ksj
