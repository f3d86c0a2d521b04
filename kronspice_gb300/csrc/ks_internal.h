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
};

int ks_launch_transpose(const double* src_rows, double* dst_cols, int64_t rows, int64_t cols, void* stream);
int ks_launch_setup(const KsDeviceBatch& b, double step, double stop, void* stream);
int ks_launch_tran(const KsDeviceBatch& b, const KOpts& o, const ks_tran_spec& spec, int cap, double* out_time,
                   double* out_wave, int32_t* out_npts, int32_t* out_status, int32_t* out_steps, int32_t* out_iters,
                   double deadline_s, void* stream);
int ks_launch_op(const KsDeviceBatch& b, const KOpts& o, const double* x0, double* out_x, int32_t* out_status,
                 int32_t* out_iters, double deadline_s, void* stream);
