// ks_solve.cuh — the per-thread linear system, element dispatch and dense LU of the
// GB300 engine, shared by the generic kernels and the per-topology kernels.
//
// A thread's system S lives either in shared memory (SmemSys: one column per
// thread, stride T; runtime or compile-time size) or in registers (RegSys:
// compile-time size, every index a constant after unrolling).  The element
// program P is either the runtime table of a plan (RtProg, interpreted) or a
// generated list of constant elements (per-topology kernels), so the same device
// code becomes straight-line code with constant matrix positions.
#pragma once
#include "ks_devices.cuh"
#include "ks_mos.cuh"

namespace ksg {

// SOLVE_STATIC_FAIL: a pivot of a per-topology program's fixed pivot sequence
// failed its threshold; the caller factors with partial pivoting instead.
enum { SOLVE_OK = 0, SOLVE_SINGULAR = KS_STATUS_SINGULAR, SOLVE_NONFINITE = KS_STATUS_NONFINITE, SOLVE_FP32_FAIL = 99,
       SOLVE_STATIC_FAIL = 98 };

// Shared-memory system with stride T; N = 0: size known at run time.  Rows are
// swapped by run-time index (kStatic = false) whatever N is.
template <int T, int N = 0>
struct SmemSys {
  static constexpr bool kStatic = false;
  static constexpr bool kAtomic = false;
  static constexpr bool kModes = false;
  static constexpr int kUnroll = 1;  // LU loops stay loops (code size)
  static constexpr int kN = N;
  double *A_, *rhs_, *x_, *xold_, *col_;
  int* piv_;
  float* L_;
  int n_;
  __device__ __forceinline__ int size() const { return N > 0 ? N : n_; }
  __device__ __forceinline__ double& a(int i, int j) { return A_[(i * size() + j) * T]; }
  __device__ __forceinline__ double& rhs(int i) { return rhs_[i * T]; }
  __device__ __forceinline__ double& xn(int i) { return x_[i * T]; }
  __device__ __forceinline__ double& xo(int i) { return xold_[i * T]; }
  __device__ __forceinline__ double& col(int i) { return col_[i * T]; }
  __device__ __forceinline__ int& piv(int i) { return piv_[i * T]; }
  __device__ __forceinline__ float& l(int i, int j) { return L_[(i * size() + j) * T]; }
  // FP32 start stage: the matrix in the FP32 factor's storage, the vectors in
  // the low halves of the FP64 rhs / x / x_old / col slots (unused while it runs)
  __device__ __forceinline__ float& a32(int i, int j) { return l(i, j); }
  __device__ __forceinline__ float& r32(int i) { return *reinterpret_cast<float*>(rhs_ + i * T); }
  __device__ __forceinline__ float& x32(int i) { return *reinterpret_cast<float*>(x_ + i * T); }
  __device__ __forceinline__ float& xo32(int i) { return *reinterpret_cast<float*>(xold_ + i * T); }
  __device__ __forceinline__ float& sv32(int i) { return *reinterpret_cast<float*>(col_ + i * T); }
};

// Register system of compile-time size N.
template <int N>
struct RegSys {
  static constexpr bool kStatic = true;
  static constexpr bool kAtomic = false;
  static constexpr bool kModes = false;
  static constexpr int kUnroll = N;  // LU loops fully unrolled (trip counts are at most N): every register index a constant
  static constexpr int kN = N;
  double A_[N * N], rhs_[N], x_[N], xold_[N], col_[N];
  int piv_[N];
  float L_[N * N];
  float r32_[N], x32_[N], xo32_[N], sv32_[N];  // FP32 start stage (the matrix is L_)
  __device__ __forceinline__ static constexpr int size() { return N; }
  __device__ __forceinline__ double& a(int i, int j) { return A_[i * N + j]; }
  __device__ __forceinline__ double& rhs(int i) { return rhs_[i]; }
  __device__ __forceinline__ double& xn(int i) { return x_[i]; }
  __device__ __forceinline__ double& xo(int i) { return xold_[i]; }
  __device__ __forceinline__ double& col(int i) { return col_[i]; }
  __device__ __forceinline__ int& piv(int i) { return piv_[i]; }
  __device__ __forceinline__ float& l(int i, int j) { return L_[i * N + j]; }
  __device__ __forceinline__ float& a32(int i, int j) { return L_[i * N + j]; }
  __device__ __forceinline__ float& r32(int i) { return r32_[i]; }
  __device__ __forceinline__ float& x32(int i) { return x32_[i]; }
  __device__ __forceinline__ float& xo32(int i) { return xo32_[i]; }
  __device__ __forceinline__ float& sv32(int i) { return sv32_[i]; }
};

// breakdownVoltage, device/diode.go:166-187.
__device__ inline double breakdown_voltage(double is, double bv, double ibv, double vt) {
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

// Per-circuit constants of one element (NewDiode, NewBJT, NewMOSFET/derive,
// resolveWave with the analysis's print step and stop time) into its derived block.
__device__ inline void setup_elem(const KElem& e, const Col& V, const Col& D, double step, double stop) {
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
      D[d + DD_RVTE] = 1 / vte;
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
      D[d + DQ_RVT] = 1 / vt;
      D[d + DQ_RNF] = 1 / (V[p + KS_Q_P_NF] * vt);
      D[d + DQ_RNE] = 1 / (V[p + KS_Q_P_NE] * vt);
      D[d + DQ_RNR] = 1 / (V[p + KS_Q_P_NR] * vt);
      D[d + DQ_RNC] = 1 / (V[p + KS_Q_P_NC] * vt);
      D[d + DQ_RNS] = 1 / (V[p + KS_Q_P_NS] * vt);
      double VAF = V[p + KS_Q_P_VAF], VAR = V[p + KS_Q_P_VAR], IKF = V[p + KS_Q_P_IKF], IKR = V[p + KS_Q_P_IKR];
      D[d + DQ_IVAF] = VAF > 0 ? 1 / VAF : 0;
      D[d + DQ_IVAR] = VAR > 0 ? 1 / VAR : 0;
      D[d + DQ_OIK] = IKF > 0 ? 1 / IKF : 0;
      D[d + DQ_OIKR] = IKR > 0 ? 1 / IKR : 0;
      D[d + DQ_RBF] = 1 / V[p + KS_Q_P_BF];
      D[d + DQ_RBR] = 1 / V[p + KS_Q_P_BR];
      break;
    }
    case KS_ELEM_M: mos_derive(e, V, D); break;
    case KS_ELEM_K:  // NewMutual, device/mutual.go:44-49: M = k sqrt(L1 L2)
      D[d + DK_M] = V[p + KS_K_P_COUPLING] * sqrt(V[e.u[2] + KS_RCL_P_VALUE] * V[e.u[3] + KS_RCL_P_VALUE]);
      break;
    case KS_ELEM_CN: case KS_ELEM_LN: nl_setup(e, V, D, step, stop); break;
    case KS_ELEM_S: case KS_ELEM_W: {  // NewSwitch, device/switch.go:92-108
      const double vh = V[p + KS_SW_P_VH], ron = V[p + KS_SW_P_RON], roff = V[p + KS_SW_P_ROFF];
      D[d + DW_VH] = fabs(vh);
      D[d + DW_SMOOTH] = vh < 0;
      D[d + DW_LMEAN] = vh < 0 ? log(sqrt(ron * roff)) : 0.0;
      D[d + DW_LRATIO] = vh < 0 ? log(ron / roff) : 0.0;
      D[d + DW_INIT] = V[p + KS_SW_P_ON] == 1;
      break;
    }
    default: break;
  }
}

// The runtime element program of a plan (element table in shared memory).
struct RtProg {
  const KElem* el;
  const int8_t* isv;
  int ne, n_nodes, n_state;
  bool nonlin_empty;
  template <class F>
  __device__ __forceinline__ void each(F&& f) const { for (int k = 0; k < ne; k++) f(el[k]); }
  __device__ __forceinline__ bool is_v(int i) const { return isv[i] != 0; }
  static constexpr bool kStaticLU = false;  // no fixed pivot sequence: partial pivoting
  static constexpr bool kWarp = false;      // one thread per circuit
  // result layouts of a batch of one topology: x [B][n], fixed-step waveforms [points][B][n]
  __device__ __forceinline__ static int64_t x_base(int64_t c, int n) { return c * n; }
  __device__ __forceinline__ static int64_t wave_base(int64_t c, int64_t B, int n, int k) {
    return ((int64_t)k * B + c) * n;
  }
};

// Programs whose circuit is shared by the 32 lanes of a warp (kWarp; the
// multi-topology kernels) run the scalar control code redundantly on every lane
// and split the element and matrix work between lanes: element loops are
// lane-strided, so their results are combined (prog_any / prog_all / prog_min),
// and read-modify-writes of shared per-circuit data are done by the owning lane
// (prog_owns) with a warp barrier (prog_sync) before others read them.  For one
// thread per circuit these are identities.
template <class P>
__device__ __forceinline__ void prog_sync(const P&) {
  if constexpr (P::kWarp) __syncwarp();
}
template <class P>
__device__ __forceinline__ bool prog_any(const P&, bool v) {
  if constexpr (P::kWarp) return __any_sync(0xffffffffu, v);
  else return v;
}
template <class P>
__device__ __forceinline__ bool prog_all(const P&, bool v) {
  if constexpr (P::kWarp) return __all_sync(0xffffffffu, v);
  else return v;
}
template <class P>
__device__ __forceinline__ double prog_min(const P&, double v) {
  if constexpr (P::kWarp) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  }
  return v;
}
template <class P>
__device__ __forceinline__ bool prog_owns(const P&, int i) {
  if constexpr (P::kWarp) return (i & 31) == (int)(threadIdx.x & 31);
  else return true;
}
// The next circuit from the persistent kernels' queue (one ticket per warp for warp programs).
template <class P>
__device__ __forceinline__ int64_t prog_next(const P&, unsigned long long* queue) {
  if constexpr (P::kWarp) {
    unsigned long long c = 0;
    if ((threadIdx.x & 31) == 0) c = atomicAdd(queue, 1ull);
    return (int64_t)__shfl_sync(0xffffffffu, c, 0);
  } else {
    return (int64_t)atomicAdd(queue, 1ull);
  }
}

__device__ __forceinline__ Col state_col(const Col& Sb, const KElem& e) { return Col{Sb.p + (int64_t)e.state * Sb.B, Sb.B}; }

__device__ __forceinline__ int lim_slot(int kind) {
  return kind == KS_ELEM_D ? SD_LIM : kind == KS_ELEM_Q ? SQ_LIM : kind == KS_ELEM_M ? SM_LIM
       : (kind == KS_ELEM_CN || kind == KS_ELEM_LN) ? SN_LIM : -1;
}

// Stamp one element at the linearization point (the element's Load).
template <class SY>
__device__ __forceinline__ void elem_load(const KElem& e, const Col& Vb, const Col& Db, const Col& Sb, SY& sys,
                                          const LoadParams& lp) {
  Col S = state_col(Sb, e);
  switch (e.kind) {
    case KS_ELEM_R: {  // device/passive.go:72-84
      double g = Db[e.derived + DR_G];
      int a = e.u[0], b = e.u[1];
      sadd(sys, a, a, g); sadd(sys, b, b, g); sadd(sys, a, b, -g); sadd(sys, b, a, -g);
      break;
    }
    case KS_ELEM_C: {  // device/reactive.go:60-106
      int a = e.u[0], b = e.u[1];
      if (lp.mode == ModeOP || lp.mode == ModeTranOP) { S[SC_TRAN] = 0; S[SC_GEQ] = 0; S[SC_IHIST] = 0; break; }
      if (lp.mode == ModeUICInit) {
        double g = 1e9, vp = S[SC_VPREV];
        sadd(sys, a, a, g); sadd(sys, b, b, g); sadd(sys, a, b, -g); sadd(sys, b, a, -g);
        srhs(sys, a, g * vp); srhs(sys, b, -g * vp);
        S[SC_TRAN] = 0; S[SC_GEQ] = 0; S[SC_IHIST] = 0;
        break;
      }
      double C = Vb[e.param + KS_RCL_P_VALUE], geq, ih;
      if (lp.method == TRAP) { geq = 2 * C * lp.rh; ih = -(geq * S[SC_VPREV] + S[SC_IPREV]); }
      else { geq = C * lp.rh; ih = -geq * S[SC_VPREV]; }
      S[SC_TRAN] = 1; S[SC_GEQ] = geq; S[SC_IHIST] = ih;
      sadd(sys, a, a, geq); sadd(sys, b, b, geq); sadd(sys, a, b, -geq); sadd(sys, b, a, -geq);
      srhs(sys, a, -ih); srhs(sys, b, ih);
      break;
    }
    case KS_ELEM_L: {  // device/reactive.go:230-259
      int a = e.u[0], b = e.u[1], kk = e.u[2];
      sadd(sys, a, kk, 1); sadd(sys, b, kk, -1);
      if (lp.mode == ModeOP || lp.mode == ModeTranOP) { sadd(sys, kk, a, 1); sadd(sys, kk, b, -1); break; }
      if (lp.mode == ModeUICInit) { sadd(sys, kk, kk, 1); srhs(sys, kk, S[SL_IPREV]); break; }
      double L = Vb[e.param + KS_RCL_P_VALUE];
      double req = L * lp.rh, r = -req * S[SL_IPREV];
      if (lp.method == TRAP) { req = 2 * L * lp.rh; r = -req * S[SL_IPREV] - S[SL_VPREV]; }
      sadd(sys, kk, a, 1); sadd(sys, kk, b, -1); sadd(sys, kk, kk, -req);
      srhs(sys, kk, r);
      break;
    }
    case KS_ELEM_V: {  // device/source.go:102-112
      double v = source_at(e, Vb, Db, S, lp);
      S[SV_VALUE] = v;
      int a = e.u[0], b = e.u[1], kk = e.u[2];
      sadd(sys, a, kk, 1); sadd(sys, b, kk, -1); sadd(sys, kk, a, 1); sadd(sys, kk, b, -1);
      srhs(sys, kk, v);
      break;
    }
    case KS_ELEM_I: {  // device/source.go:155-160
      double v = source_at(e, Vb, Db, S, lp);
      S[SV_VALUE] = v;
      srhs(sys, e.u[0], -v); srhs(sys, e.u[1], v);
      break;
    }
    case KS_ELEM_D: diode_load(e, Vb, Db, S, sys, lp); break;
    case KS_ELEM_Q: bjt_load(e, Vb, Db, S, sys, lp); break;
    case KS_ELEM_M: mos_load(e, Vb, Db, S, sys, lp); break;
    case KS_ELEM_E: case KS_ELEM_H: {  // device/controlled.go:83-100: the output branch row
      const double g = Vb[e.param + KS_CTL_P_GAIN];
      const int a = e.u[0], b = e.u[1], kk = e.u[2];
      sadd(sys, a, kk, 1); sadd(sys, b, kk, -1); sadd(sys, kk, a, 1); sadd(sys, kk, b, -1);
      if (e.kind == KS_ELEM_E) { sadd(sys, kk, e.u[3], -g); sadd(sys, kk, e.u[4], g); }
      else sadd(sys, kk, e.u[3], -g);
      break;
    }
    case KS_ELEM_G: {  // device/controlled.go:101-106
      const double g = Vb[e.param + KS_CTL_P_GAIN];
      sadd(sys, e.u[0], e.u[3], g); sadd(sys, e.u[0], e.u[4], -g);
      sadd(sys, e.u[1], e.u[3], -g); sadd(sys, e.u[1], e.u[4], g);
      break;
    }
    case KS_ELEM_F: {  // device/controlled.go:107-110
      const double g = Vb[e.param + KS_CTL_P_GAIN];
      sadd(sys, e.u[0], e.u[3], g); sadd(sys, e.u[1], e.u[3], -g);
      break;
    }
    case KS_ELEM_K: {  // device/mutual.go:75-118 (no torsion terms): the coupling of a time step
      if (lp.mode == ModeOP || lp.mode == ModeTranOP || lp.mode == ModeUICInit) break;
      const double f = (lp.method == TRAP ? 2 : 1) * Db[e.derived + DK_M] * lp.rh;
      const int k1 = e.u[0], k2 = e.u[1];
      sadd(sys, k1, k2, -f); sadd(sys, k2, k1, -f);
      srhs(sys, k1, -f * S[SK_I2PREV]); srhs(sys, k2, -f * S[SK_I1PREV]);
      break;
    }
    case KS_ELEM_S: case KS_ELEM_W: sw_load(e, Vb, Db, S, sys, lp); break;
    case KS_ELEM_CN: case KS_ELEM_LN: nl_load(e, Vb, Db, S, sys, lp); break;
  }
}

// Stamp every element (analysis/op.go:289-322 without the solve).
template <class SY, class P>
__device__ __forceinline__ void load_all(const P& prog, const Col& Vb, const Col& Db, const Col& Sb, SY& s,
                                         const LoadParams& lp) {
  const int n = s.size();
  // -0.0 is the identity of addition (x + -0.0 == x for every x), so in a
  // register system the first stamp into an entry folds into a plain move
  const double z = SY::kStatic ? -0.0 : 0.0;
  if constexpr (SY::kAtomic) {
    s.zero();
    prog_sync(prog);
  } else {
#pragma unroll
    for (int i = 0; i < n; i++) {
#pragma unroll
      for (int j = 0; j < n; j++) s.a(i, j) = z;
      s.rhs(i) = z;
    }
  }
  prog.each([&](const KElem& e) KS_INLINE_LAMBDA { elem_load(e, Vb, Db, Sb, s, lp); });
  prog_sync(prog);
}

// Swap rows k and p (static systems compare p against every later row, so every
// register index stays a constant).
template <class SY>
__device__ __forceinline__ void swap_rows(SY& s, int k, int p) {
  const int n = s.size();
  if constexpr (SY::kStatic) {
#pragma unroll (SY::kUnroll)
    for (int i = 0; i < n; i++)
      if (i > k && i == p)
#pragma unroll (SY::kUnroll)
        for (int j = 0; j < n; j++) { double t = s.a(k, j); s.a(k, j) = s.a(i, j); s.a(i, j) = t; }
  } else if (p != k) {
    for (int j = 0; j < n; j++) { double t = s.a(k, j); s.a(k, j) = s.a(p, j); s.a(p, j) = t; }
  }
}
template <class SY>
__device__ __forceinline__ void swap_rows32(SY& s, int k, int p) {
  const int n = s.size();
  if constexpr (SY::kStatic) {
#pragma unroll (SY::kUnroll)
    for (int i = 0; i < n; i++)
      if (i > k && i == p)
#pragma unroll (SY::kUnroll)
        for (int j = 0; j < n; j++) { float t = s.l(k, j); s.l(k, j) = s.l(i, j); s.l(i, j) = t; }
  } else if (p != k) {
    for (int j = 0; j < n; j++) { float t = s.l(k, j); s.l(k, j) = s.l(p, j); s.l(p, j) = t; }
  }
}
// y <- P y with the recorded pivots (y given as an accessor).
template <class SY, class Y>
__device__ __forceinline__ void permute(SY& s, Y&& y) {
  const int n = s.size();
#pragma unroll (SY::kUnroll)
  for (int k = 0; k < n; k++) {
    int p = s.piv(k);
    if constexpr (SY::kStatic) {
#pragma unroll (SY::kUnroll)
      for (int i = 0; i < n; i++)
        if (i > k && i == p) { double t = y(k); y(k) = y(i); y(i) = t; }
    } else if (p != k) {
      double t = y(k); y(k) = y(p); y(p) = t;
    }
  }
}

// Magnitude of a double as an integer key: key(a) < key(b) iff |a| < |b| for
// every non-NaN pair, and keys at or above KS_INF_KEY are infinities and NaNs.
// The LU's scans for the largest entry and for non-finite entries run on these
// keys in the integer pipes; GB300's FP64 pipe is kept for the arithmetic.
#define KS_INF_KEY 0x7ff0000000000000LL
__device__ __forceinline__ long long mag_key(double x) { return __double_as_longlong(x) & 0x7fffffffffffffffLL; }
__device__ __forceinline__ double key_mag(long long k) { return __longlong_as_double(k); }
__device__ __forceinline__ long long key_max(long long a, long long b) { return a > b ? a : b; }
// Biased exponent field of a double / float (0: zero or subnormal; 2047 / 255:
// infinity or NaN), for the pivot thresholds of the fixed pivot sequence.
__device__ __forceinline__ int ks_exp64(double v) { return (int)((__double_as_longlong(v) >> 52) & 0x7ff); }
__device__ __forceinline__ int ks_exp32(float v) { return (__float_as_int(v) >> 23) & 0xff; }

// Largest |a(i,j)| of every column into col(j); returns the key of the largest
// entry of the matrix (>= KS_INF_KEY: a non-finite entry).
template <class SY>
__device__ __forceinline__ long long column_scales(SY& s) {
  const int n = s.size();
  long long kall = 0;
#pragma unroll (SY::kUnroll)
  for (int j = 0; j < n; j++) {
    long long m = 0;
#pragma unroll (SY::kUnroll)
    for (int i = 0; i < n; i++) m = key_max(m, mag_key(s.a(i, j)));
    s.col(j) = key_mag(m);
    kall = key_max(kall, m);
  }
  return kall;
}

// Dense LU with partial pivoting in FP64, solver/dense.go:80-177; A is factored in
// place and x = A^-1 rhs.  Each column divides by its pivot once (a reciprocal,
// kept in col(k) for the back substitution) instead of once per row.
template <class SY>
__device__ __forceinline__ int lu_solve_fp64(SY& s) {
  const int n = s.size();
  long long kall = column_scales(s);
  if (kall >= KS_INF_KEY) return SOLVE_NONFINITE;
  if (kall == 0) return SOLVE_SINGULAR;
#pragma unroll (SY::kUnroll)
  for (int k = 0; k < n; k++) {
    int p = k;
    long long km = mag_key(s.a(k, k));
#pragma unroll (SY::kUnroll)
    for (int i = k + 1; i < n; i++) {
      long long v = mag_key(s.a(i, k));
      if (v > km) { km = v; p = i; }
    }
    if (key_mag(km) <= s.col(k) * double(n) * 1e-14) return SOLVE_SINGULAR;
    s.piv(k) = p;
    swap_rows(s, k, p);
    double rp = 1.0 / s.a(k, k);
    s.col(k) = rp;
#pragma unroll (SY::kUnroll)
    for (int i = k + 1; i < n; i++) {
      double f = s.a(i, k) * rp;
      s.a(i, k) = f;
#pragma unroll (SY::kUnroll)
      for (int j = k + 1; j < n; j++) s.a(i, j) -= f * s.a(k, j);
    }
  }
#pragma unroll (SY::kUnroll)
  for (int i = 0; i < n; i++) s.xn(i) = s.rhs(i);
  permute(s, [&](int i) -> double& { return s.xn(i); });
#pragma unroll (SY::kUnroll)
  for (int i = 0; i < n; i++) {
    double acc = s.xn(i);
#pragma unroll (SY::kUnroll)
    for (int j = 0; j < i; j++) acc -= s.a(i, j) * s.xn(j);
    s.xn(i) = acc;
  }
  long long kx = 0;
#pragma unroll (SY::kUnroll)
  for (int i = n - 1; i >= 0; i--) {
    double acc = s.xn(i);
#pragma unroll (SY::kUnroll)
    for (int j = i + 1; j < n; j++) acc -= s.a(i, j) * s.xn(j);
    s.xn(i) = acc * s.col(i);
    kx = key_max(kx, mag_key(s.xn(i)));
  }
  return kx >= KS_INF_KEY ? SOLVE_NONFINITE : SOLVE_OK;
}

// FP32 forward/back substitution with the factor in L32, in place on col().
template <class SY>
__device__ __forceinline__ void lu32_apply_col(SY& s) {
  const int n = s.size();
  permute(s, [&](int i) -> double& { return s.col(i); });
#pragma unroll (SY::kUnroll)
  for (int i = 0; i < n; i++) {
    float acc = (float)s.col(i);
#pragma unroll (SY::kUnroll)
    for (int j = 0; j < i; j++) acc = fmaf(-s.l(i, j), (float)s.col(j), acc);
    s.col(i) = acc;
  }
#pragma unroll (SY::kUnroll)
  for (int i = n - 1; i >= 0; i--) {
    float acc = (float)s.col(i);
#pragma unroll (SY::kUnroll)
    for (int j = i + 1; j < n; j++) acc = fmaf(-s.l(i, j), (float)s.col(j), acc);
    s.col(i) = acc / s.l(i, i);
  }
}

// Mixed precision: FP32 LU with partial pivoting of the FP64 matrix, then
// x = xold + LU32^-1 (rhs - A*xold) with the residual in FP64, repeated as
// iterative refinement (x += LU32^-1 (rhs - A*x)) until the correction is below
// rtol of the solution, for at most `passes` passes.  The caller's rtol is three
// orders under the Newton tolerance for nonlinear circuits (the Newton test
// cannot tell the solve's error from zero) and 1e-11 for linear ones (one solve
// per time point, errors would accumulate).  A and rhs are left intact.  Returns
// SOLVE_FP32_FAIL when a pivot is below the FP32 threshold or the refinement
// stops contracting or does not reach rtol (the caller then solves in FP64), so
// a system too ill-conditioned for FP32 factors never yields an unrefined step.
// One pass (passes = 1) skips those checks: each Newton step is then the FP32
// solve of the FP64 residual, for well-conditioned systems only.
template <class SY>
__device__ __forceinline__ int lu_solve_mixed(SY& s, int passes, double rtol) {
  const int n = s.size();
  long long kall = column_scales(s);
  if (kall >= KS_INF_KEY) return SOLVE_NONFINITE;
  if (kall == 0) return SOLVE_SINGULAR;
#pragma unroll (SY::kUnroll)
  for (int i = 0; i < n; i++)
#pragma unroll (SY::kUnroll)
    for (int j = 0; j < n; j++) s.l(i, j) = (float)s.a(i, j);
#pragma unroll (SY::kUnroll)
  for (int k = 0; k < n; k++) {
    int p = k;
    float maxv = fabsf(s.l(k, k));
#pragma unroll (SY::kUnroll)
    for (int i = k + 1; i < n; i++) {
      float v = fabsf(s.l(i, k));
      if (v > maxv) { maxv = v; p = i; }
    }
    if ((double)maxv <= s.col(k) * double(n) * 1e-6) return SOLVE_FP32_FAIL;
    s.piv(k) = p;
    swap_rows32(s, k, p);
    float rp = 1.0f / s.l(k, k);
#pragma unroll (SY::kUnroll)
    for (int i = k + 1; i < n; i++) {
      float f = s.l(i, k) * rp;
      s.l(i, k) = f;
#pragma unroll (SY::kUnroll)
      for (int j = k + 1; j < n; j++) s.l(i, j) = fmaf(-f, s.l(k, j), s.l(i, j));
    }
  }
#pragma unroll (SY::kUnroll)
  for (int i = 0; i < n; i++) s.xn(i) = s.xo(i);
  double prev = KS_INF;
  for (int pass = 0; pass < passes; pass++) {
#pragma unroll (SY::kUnroll)
    for (int i = 0; i < n; i++) {  // FP64 residual in col()
      double r = s.rhs(i);
#pragma unroll (SY::kUnroll)
      for (int j = 0; j < n; j++) r -= s.a(i, j) * s.xn(j);
      s.col(i) = r;
    }
    lu32_apply_col(s);
    long long kd = 0, kx = 0;
#pragma unroll (SY::kUnroll)
    for (int i = 0; i < n; i++) {
      double v = s.xn(i) + s.col(i);
      s.xn(i) = v;
      kd = key_max(kd, mag_key(s.col(i)));
      kx = key_max(kx, mag_key(v));
    }
    if (kx >= KS_INF_KEY || kd >= KS_INF_KEY) return SOLVE_NONFINITE;
    double dmax = key_mag(kd), xmax = key_mag(kx);
    if (dmax <= rtol * xmax || dmax == 0) break;
    if (pass > 0 && dmax > 0.5 * prev) return SOLVE_FP32_FAIL;  // refinement stopped contracting
    if (pass == passes - 1 && passes > 1) return SOLVE_FP32_FAIL;  // not refined within the passes
    prev = dmax;
  }
  return SOLVE_OK;
}

// converged, analysis/newton.go:59-82.
template <class SY, class P>
__device__ __forceinline__ bool converged(const P& prog, const Col& Vb, const Col& Db, const Col& Sb, SY& s, const KOpts& o,
                                 double gmin) {
  bool lim = false;
  prog.each([&](const KElem& e) KS_INLINE_LAMBDA {
    int ls = lim_slot(e.kind);
    if (ls >= 0 && Sb[e.state + ls] != 0) lim = true;
  });
  if (prog_any(prog, lim)) return false;
  const int n = s.size();
  bool moved = false;
#pragma unroll
  for (int i = 0; i < n; i++) {
    double x = s.xn(i), old = s.xo(i);
    double tol = (prog.is_v(i) ? o.vntol : o.abstol) + o.reltol * key_mag(key_max(mag_key(x), mag_key(old)));
    moved |= fabs(x - old) > tol;
  }
  if (prog_any(prog, moved)) return false;
  bool ok = true;
  prog.each([&](const KElem& e) KS_INLINE_LAMBDA {
    if (!ok) return;
    Col S = state_col(Sb, e);
    if (e.kind == KS_ELEM_D) ok = diode_conv(e, Vb, Db, S, s, o.reltol, o.abstol, gmin);
    else if (e.kind == KS_ELEM_Q) ok = bjt_conv(e, Vb, Db, S, s, o.reltol, o.abstol, gmin);
    else if (e.kind == KS_ELEM_M) ok = mos_conv(e, Vb, Db, S, s, o.reltol, o.abstol, gmin);
    else if (e.kind == KS_ELEM_S || e.kind == KS_ELEM_W) ok = sw_conv(e, Vb, Db, S, s, o.reltol, o.abstol);
    else if (e.kind == KS_ELEM_CN || e.kind == KS_ELEM_LN) ok = nl_conv(e, Vb, Db, S, s, o.reltol, o.abstol);
  });
  return prog_all(prog, ok);
}

// Accept one element at the new iterate (its Accept).
template <class SY>
__device__ __forceinline__ void elem_accept(const KElem& e, const Col& Vb, const Col& Db, const Col& Sb, SY& s,
                                            double t, int mode, double gmin, bool nonlinOnly) {
  Col S = state_col(Sb, e);
  switch (e.kind) {
    case KS_ELEM_C: {  // device/reactive.go:144-161
      if (nonlinOnly) break;
      double v = xn_(s, e.u[0]) - xn_(s, e.u[1]);
      if (mode == ModeUICInit) { S[SC_IPREV] = 0; hist_reset(S, SC_HIST); }
      else if (mode == ModeOP || mode == ModeTranOP) { S[SC_VPREV] = v; S[SC_IPREV] = 0; hist_reset(S, SC_HIST); }
      else { double i = S[SC_TRAN] != 0 ? S[SC_GEQ] * v + S[SC_IHIST] : 0.0; S[SC_VPREV] = v; S[SC_IPREV] = i; }
      hist_push(S, SC_HIST, t, Vb[e.param] * S[SC_VPREV]);
      break;
    }
    case KS_ELEM_L: {  // device/reactive.go:312-329
      if (nonlinOnly) break;
      double v = xn_(s, e.u[0]) - xn_(s, e.u[1]), i = xn_(s, e.u[2]);
      if (mode == ModeUICInit) { S[SL_VPREV] = 0; hist_reset(S, SL_HIST); }
      else if (mode == ModeOP || mode == ModeTranOP) { S[SL_VPREV] = 0; S[SL_IPREV] = i; hist_reset(S, SL_HIST); }
      else { S[SL_VPREV] = v; S[SL_IPREV] = i; }
      hist_push(S, SL_HIST, t, Vb[e.param] * S[SL_IPREV]);
      break;
    }
    case KS_ELEM_D: diode_accept(e, Vb, Db, S, s, t, mode); break;
    case KS_ELEM_Q: bjt_accept(e, Vb, Db, S, s, t, mode, gmin); break;
    case KS_ELEM_M: mos_accept(e, Vb, Db, S, s, t, mode); break;
    case KS_ELEM_K:  // device/mutual.go:134-137
      if (nonlinOnly) break;
      S[SK_I1PREV] = xn_(s, e.u[0]); S[SK_I2PREV] = xn_(s, e.u[1]);
      break;
    case KS_ELEM_S: case KS_ELEM_W: sw_accept(e, Vb, Db, S, s); break;  // nonlinear: seeded by a NodeSet too
    case KS_ELEM_CN: case KS_ELEM_LN:  // a curved law is nonlinear (seeded by a NodeSet), a linear one is not
      if (nonlinOnly && e.level == 0) break;
      nl_accept(e, Vb, Db, S, s, t, mode);
      break;
  }
}

// One element's part of converged (analysis/newton.go:59-82): not limited at
// its last load, and its ConvTest passes.
template <class SY>
__device__ __forceinline__ bool elem_converged(const KElem& e, const Col& Vb, const Col& Db, const Col& Sb, SY& s,
                                               const KOpts& o, double gmin) {
  if (e.kind == KS_ELEM_S || e.kind == KS_ELEM_W) return sw_conv(e, Vb, Db, state_col(Sb, e), s, o.reltol, o.abstol);
  const int ls = lim_slot(e.kind);
  if (ls < 0) return true;
  Col S = state_col(Sb, e);
  if (S[ls] != 0) return false;
  if (e.kind == KS_ELEM_D) return diode_conv(e, Vb, Db, S, s, o.reltol, o.abstol, gmin);
  if (e.kind == KS_ELEM_Q) return bjt_conv(e, Vb, Db, S, s, o.reltol, o.abstol, gmin);
  if (e.kind == KS_ELEM_CN || e.kind == KS_ELEM_LN) return nl_conv(e, Vb, Db, S, s, o.reltol, o.abstol);
  return mos_conv(e, Vb, Db, S, s, o.reltol, o.abstol, gmin);
}

// Accept every element at the new iterate (analysis/op.go:324-328).
template <class SY, class P>
__device__ __forceinline__ void accept_all(const P& prog, const Col& Vb, const Col& Db, const Col& Sb, SY& s, double t,
                                  int mode, double gmin, bool nonlinOnly) {
  prog.each([&](const KElem& e) KS_INLINE_LAMBDA { elem_accept(e, Vb, Db, Sb, s, t, mode, gmin, nonlinOnly); });
  prog_sync(prog);
}

// Fresh device state of one circuit (the zero state of newly built devices, with
// each MOSFET's limiting threshold at VTO, device/mosfet.go:321, and each
// switch in its initial state).
template <class P>
__device__ inline void init_state(const P& prog, const Col& Db, const Col& Sb) {
  for (int k = 0; k < prog.n_state; k++) Sb[k] = 0.0;
  prog_sync(prog);
  prog.each([&](const KElem& e) KS_INLINE_LAMBDA {
    if (e.kind == KS_ELEM_M) Sb[e.state + SM_AVON] = Db[e.derived + DM_VTO];
    if (e.kind == KS_ELEM_S || e.kind == KS_ELEM_W)  // the ON / OFF initial state, device/switch.go:105-106
      Sb[e.state + SW_ON] = Sb[e.state + SW_ACC] = Db[e.derived + DW_INIT];
  });
  prog_sync(prog);
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// The batch's cancel word, written by the host while the kernel runs: a volatile
// load of the mapped host word (lane 0's reading for warp programs, so a cancel
// ends the circuit on all lanes together).
template <class P>
__device__ __forceinline__ bool prog_cancelled(const P&, const int32_t* w) {
  int v = *reinterpret_cast<const volatile int32_t*>(w);
  if constexpr (P::kWarp) v = __shfl_sync(0xffffffffu, v, 0);
  return v != 0;
}

// The wall clock as every lane of a warp program sees it (lane 0's reading), so a
// deadline ends the circuit on all lanes together.
template <class P>
__device__ __forceinline__ uint64_t prog_clock(const P&) {
  uint64_t t = globaltimer_ns();
  if constexpr (P::kWarp) t = __shfl_sync(0xffffffffu, t, 0);
  return t;
}

}  // namespace ksg
