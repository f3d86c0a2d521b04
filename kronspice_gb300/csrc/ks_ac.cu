// ks_ac.cu — batched AC small-signal sweep (analysis.AC, analysis/ac.go:76-150).
//
// After the operating point (ks_op's kernels, with the polish of
// analysis/op.go:251-271), every device's small-signal model is linear in the
// angular frequency: its LoadAC stamps g + j*omega*c.  So the sweep splits in two
// kernels:
//   k_ac_model  one thread per circuit evaluates the LoadAC stamps of every
//               element at the circuit's operating point once, into a real
//               conductance matrix G, a real capacitance matrix C and the
//               complex source vector b (SoA columns: entry e of circuit c at
//               [e * B + c], so a warp's loads and stores are coalesced);
//   k_ac_solve  one thread per (frequency, circuit) builds Y = G + j*omega*C in
//               shared memory and solves Y x = b with the complex LU of
//               solver/cdense.go (partial pivoting on the entry's magnitude, the
//               column-relative singular test of solver/dense.go:126, non-finite
//               checks on the matrix and the result).  Frequency-major unit order
//               keeps 32 circuits of one frequency in a warp, so the G / C reads
//               stay coalesced; each circuit's G and C are read by every
//               frequency and stay in L2.
// A circuit's first failing frequency (lowest index) decides its status, as the
// reference returns at the first failing frequency.
#include <cuda_runtime.h>
#include <algorithm>
#include <climits>
#include "ks_internal.h"
#include "ks_newton.cuh"

using namespace ksg;

namespace {

// One circuit's operating point x (row-major output of the OP kernels) seen as
// a system whose new iterate and linearization point are both x.
struct XView {
  const double* x;
  __device__ __forceinline__ double xn(int i) const { return x[i]; }
  __device__ __forceinline__ double xo(int i) const { return x[i]; }
};

// One circuit's AC stamp columns.
struct AcCols {
  double *G, *C, *br, *bi;
  int64_t B;
  int n;
  __device__ __forceinline__ void add(int i, int j, double g, double cap) const {
    if (i < 0 || j < 0) return;
    int64_t k = (int64_t)(i * n + j) * B;
    if (g != 0) G[k] += g;
    if (cap != 0) C[k] += cap;
  }
  __device__ __forceinline__ void rhs(int i, double re, double im) const {
    if (i < 0) return;
    br[(int64_t)i * B] += re; bi[(int64_t)i * B] += im;
  }
  // stampY, device/device.go:333-338
  __device__ __forceinline__ void y(int a, int b, double g, double cap) const {
    add(a, a, g, cap); add(b, b, g, cap); add(a, b, -g, -cap); add(b, a, -g, -cap);
  }
  // acBranch, device/bjt.go:713-726: y1 controlled by (p1, n1), y2 by (p2, n2)
  __device__ __forceinline__ void branch(int a, int b, double g1, double c1, int p1, int n1, double g2, double c2,
                                         int p2, int n2) const {
    if (g1 != 0 || c1 != 0) { add(a, p1, g1, c1); add(a, n1, -g1, -c1); add(b, p1, -g1, -c1); add(b, n1, g1, c1); }
    if (g2 != 0 || c2 != 0) { add(a, p2, g2, c2); add(a, n2, -g2, -c2); add(b, p2, -g2, -c2); add(b, n2, g2, c2); }
  }
};

// The AC phasor of a source: cmplx.Rect(acmag, acphase in degrees), device/source.go.
__device__ __forceinline__ void source_ac(const Col& V, int p, double* re, double* im) {
  double s, c;
  sincos(V[p + KS_SRC_P_ACPHASE] * kPi / 180, &s, &c);
  const double m = V[p + KS_SRC_P_ACMAG];
  *re = m * c; *im = m * s;
}

__device__ void diode_ac(const KElem& e, const Col& V, const Col& Dv, const XView& xv, const AcCols& y, double gmin) {
  // device/diode.go:409-421
  const int a = e.u[0], k = e.u[1], ai = e.u[2];
  const double v = xn_(xv, ai) - xn_(xv, k);
  double id, gd, q, cap;
  diode_iv(V, Dv, e.param, e.derived, e.flags & KS_F_HAS_BV, v, &id, &gd);
  diode_charge(V, e.param, v, id, gd, &q, &cap);
  y.y(ai, k, gd + gmin, cap);
  const double grs = Dv[e.derived + DD_GRS];
  if (grs > 0) y.y(a, ai, grs, 0);
}

__device__ void bjt_ac(const KElem& e, const Col& V, const Col& Dv, const XView& xv, const AcCols& y, double gmin) {
  // device/bjt.go:689-711
  const int p = e.param, dd = e.derived;
  double vbe, vbc, vbx, vcs;
  bjt_voltages<true>(e, xv, &vbe, &vbc, &vbx, &vcs);
  BjtDC d = bjt_eval_dc(V, Dv, p, dd, vbe, vbc, gmin);
  BjtCh h = bjt_charges(V, Dv, p, dd, vbe, vbc, vbx, vcs, d);
  double isub, gsub;
  junction(V[p + KS_Q_P_ISS], vcs, V[p + KS_Q_P_NS] * Dv[dd + DQ_VT], Dv[dd + DQ_RNS], &isub, &gsub);
  gsub += gmin;
  const int b = e.u[2], cp = e.u[4], bp = e.u[5], ep = e.u[6], sa = e.u[7], sb = e.u[8];
  y.branch(cp, ep, d.itBE, 0, bp, ep, d.itBC, 0, bp, cp);
  y.branch(bp, ep, d.gpi, h.c[0], bp, ep, 0, h.dqbeDvbc, bp, cp);
  y.branch(bp, cp, d.gmu, h.c[1], bp, cp, 0, 0, 0, 0);
  y.branch(b, cp, 0, h.c[2], b, cp, 0, 0, 0, 0);
  y.branch(sa, sb, gsub, h.c[3], sa, sb, 0, 0, 0, 0);
  if (bp != b) y.y(b, bp, d.gx, 0);
  if (cp != e.u[0]) y.y(e.u[0], cp, Dv[dd + DQ_GCPR], 0);
  if (ep != e.u[1]) y.y(e.u[1], ep, Dv[dd + DQ_GEPR], 0);
}

__device__ void mos_ac(const KElem& e, const Col& V, const Col& D, const XView& xv, const AcCols& y, double gmin) {
  // device/mosfet.go:779-813
  const int d = e.derived, p = e.param;
  double vgs, vds, vbs, vgb;
  mos_voltages<true>(e, xv, &vgs, &vds, &vbs, &vgb);
  const double vgd = vgs - vds, vbd = vbs - vds;
  double o[7];
  mos_channel(e, V, D, vgs, vds, vbs, o);
  double gch[3];
  if (o[0] > 0) { gch[0] = o[2]; gch[1] = o[3]; gch[2] = o[4]; }
  else { gch[0] = -o[2]; gch[1] = o[2] + o[3] + o[4]; gch[2] = -o[4]; }
  const double vt = D[d + DM_VT];
  double ib, gbs, gbd;
  mos_bulk_diode(vbs, D[d + DM_ISS], vt, D[d + DM_RVT], gmin, &ib, &gbs);
  mos_bulk_diode(vbd, D[d + DM_ISD], vt, D[d + DM_RVT], gmin, &ib, &gbd);
  double mc[3], q, cbs, cbd;
  meyer_caps(D, d, vgs, vgd, o[5], o[6], o[0], mc);
  mos_bulk_charge(V, p, D, d, vbs, D[d + DM_CZBS], D[d + DM_CZBSSW], &q, &cbs);
  mos_bulk_charge(V, p, D, d, vbd, D[d + DM_CZBD], D[d + DM_CZBDSW], &q, &cbd);
  const int g = e.u[2], b = e.u[3], dp = e.u[4], sp = e.u[5];
  const int ctrl[3] = {g, dp, b};
  for (int k = 0; k < 3; k++) y.branch(dp, sp, gch[k], 0, ctrl[k], sp, 0, 0, 0, 0);
  y.y(b, sp, gbs, 0);
  y.y(b, dp, gbd, 0);
  y.y(g, sp, 0, mc[0] + D[d + DM_CGSO]);
  y.y(g, dp, 0, mc[1] + D[d + DM_CGDO]);
  y.y(g, b, 0, mc[2] + D[d + DM_CGBO]);
  y.y(b, sp, 0, cbs);
  y.y(b, dp, 0, cbd);
  if (dp != e.u[0]) y.y(e.u[0], dp, D[d + DM_GDPR], 0);
  if (sp != e.u[1]) y.y(e.u[1], sp, D[d + DM_GSPR], 0);
}

}  // namespace

// G, C and b of every circuit at its operating point x [B][n] (a switch: the
// linearization of the last load, in the device state).
__global__ void __launch_bounds__(128) k_ac_model(KPlan plan, const double* __restrict__ values,
                                                  const double* __restrict__ derived,
                                                  const double* __restrict__ state, int64_t B,
                                                  const double* __restrict__ x, double gmin, double* G, double* C,
                                                  double* br, double* bi) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= B) return;
  const int n = plan.n;
  const AcCols y{G + c, C + c, br + c, bi + c, B, n};
  for (int k = 0; k < n * n; k++) { y.G[(int64_t)k * B] = 0; y.C[(int64_t)k * B] = 0; }
  for (int k = 0; k < n; k++) { y.br[(int64_t)k * B] = 0; y.bi[(int64_t)k * B] = 0; }
  const Col V{const_cast<double*>(values) + c, B}, D{const_cast<double*>(derived) + c, B};
  const XView xv{x + c * n};
  for (int k = 0; k < plan.n_elem; k++) {
    const KElem e = plan.elem[k];
    const int a = e.u[0], b = e.u[1];
    switch (e.kind) {
      case KS_ELEM_R: y.y(a, b, D[e.derived + DR_G], 0); break;                 // device/passive.go:116-123
      case KS_ELEM_C: y.y(a, b, 0, V[e.param + KS_RCL_P_VALUE]); break;          // device/reactive.go:355-363
      case KS_ELEM_L: {                                                          // device/reactive.go:377-393
        const int br_ = e.u[2];
        y.add(a, br_, 1, 0); y.add(b, br_, -1, 0); y.add(br_, a, 1, 0); y.add(br_, b, -1, 0);
        y.add(br_, br_, 0, -V[e.param + KS_RCL_P_VALUE]);
        break;
      }
      case KS_ELEM_V: {                                                          // device/source.go:186-194
        const int br_ = e.u[2];
        y.add(a, br_, 1, 0); y.add(b, br_, -1, 0); y.add(br_, a, 1, 0); y.add(br_, b, -1, 0);
        double re, im;
        source_ac(V, e.param, &re, &im);
        y.rhs(br_, re, im);
        break;
      }
      case KS_ELEM_I: {                                                          // device/source.go:208-212
        double re, im;
        source_ac(V, e.param, &re, &im);
        y.rhs(a, -re, -im); y.rhs(b, re, im);
        break;
      }
      case KS_ELEM_D: diode_ac(e, V, D, xv, y, gmin); break;
      case KS_ELEM_Q: bjt_ac(e, V, D, xv, y, gmin); break;
      case KS_ELEM_M: mos_ac(e, V, D, xv, y, gmin); break;
      case KS_ELEM_E: case KS_ELEM_H: {                                          // device/controlled.go:144-148
        const double g = V[e.param + KS_CTL_P_GAIN];
        const int br_ = e.u[2];
        y.add(a, br_, 1, 0); y.add(b, br_, -1, 0); y.add(br_, a, 1, 0); y.add(br_, b, -1, 0);
        y.add(br_, e.u[3], -g, 0);
        if (e.kind == KS_ELEM_E) y.add(br_, e.u[4], g, 0);
        break;
      }
      case KS_ELEM_G: {
        const double g = V[e.param + KS_CTL_P_GAIN];
        y.add(a, e.u[3], g, 0); y.add(a, e.u[4], -g, 0); y.add(b, e.u[3], -g, 0); y.add(b, e.u[4], g, 0);
        break;
      }
      case KS_ELEM_F: {
        const double g = V[e.param + KS_CTL_P_GAIN];
        y.add(a, e.u[3], g, 0); y.add(b, e.u[3], -g, 0);
        break;
      }
      case KS_ELEM_K: {                                                          // device/mutual.go:146-151
        const double m = D[e.derived + DK_M];
        y.add(e.u[0], e.u[1], 0, -m); y.add(e.u[1], e.u[0], 0, -m);
        break;
      }
      case KS_ELEM_CN: case KS_ELEM_LN: {  // device/nonlinear_reactive.go:440-449, :640-651: s f'(x) at the accepted point
        const Col S{const_cast<double*>(state) + c + (int64_t)e.state * B, B};
        NlLaw law(e, V, D);
        double y0, dy;
        law.f(S[SN_XACC], &y0, &dy);
        const double inc = S[SN_SACC] * dy;
        if (e.kind == KS_ELEM_CN) y.y(a, b, 0, inc);
        else {
          const int br_ = e.u[2];
          y.add(a, br_, 1, 0); y.add(b, br_, -1, 0); y.add(br_, a, 1, 0); y.add(br_, b, -1, 0);
          y.add(br_, br_, 0, -inc);
        }
        break;
      }
      case KS_ELEM_S: case KS_ELEM_W: {                                          // device/switch.go:314-329
        const Col S{const_cast<double*>(state) + c + (int64_t)e.state * B, B};
        y.y(a, b, S[SW_G], 0);
        const double k = S[SW_K];
        if (D[e.derived + DW_SMOOTH] != 0 && k != 0) {
          if (e.kind == KS_ELEM_W) { y.add(a, e.u[3], k, 0); y.add(b, e.u[3], -k, 0); }
          else { y.add(a, e.u[3], k, 0); y.add(a, e.u[4], -k, 0); y.add(b, e.u[3], -k, 0); y.add(b, e.u[4], k, 0); }
        }
        break;
      }
      default: break;
    }
  }
}

// One complex solve per (frequency, circuit): Y = G + j*omega*C, CDense
// (solver/cdense.go:77-193) in shared memory, T = blockDim.x threads with
// their matrices interleaved at stride T.  Circuits whose operating point
// failed (status != 0) are skipped.
__global__ void k_ac_solve(int n, int64_t B, int32_t nf, const double* __restrict__ freqs,
                           const double* __restrict__ G, const double* __restrict__ C,
                           const double* __restrict__ br, const double* __restrict__ bi,
                           const int32_t* __restrict__ status, double* out_x, int32_t* err_at) {
  extern __shared__ __align__(16) double sm[];
  const int T = blockDim.x, tid = threadIdx.x;
  const int nn = n * n;
  double* Ar = sm + tid;              // [nn][T]
  double* Ai = Ar + (int64_t)nn * T;  // [nn][T]
  double* xr = Ai + (int64_t)nn * T;  // [n][T]
  double* xi = xr + (int64_t)n * T;
  // squared column maxima [n][T], only compared against a tolerance: float,
  // after the T threads' double arrays
  float* cm = reinterpret_cast<float*>(sm + (int64_t)(2 * nn + 2 * n) * T) + tid;
  const int64_t units = B * (int64_t)nf;
  for (int64_t u = (int64_t)blockIdx.x * T + tid; u < units; u += (int64_t)gridDim.x * T) {
    const int32_t f = (int32_t)(u / B);
    const int64_t c = u - (int64_t)f * B;
    double* o = out_x + ((c * nf + f) * (int64_t)n) * 2;
    if (status[c] != KS_STATUS_OK) {  // no operating point: zero phasors
      for (int i = 0; i < 2 * n; i++) o[i] = 0;
      continue;
    }
    const double w = 2 * kPi * freqs[f];
#define AR(i, j) Ar[(int64_t)((i) * n + (j)) * T]
#define AI(i, j) Ai[(int64_t)((i) * n + (j)) * T]
    bool finite = true;
    double scale = 0;
    for (int k = 0; k < n; k++) cm[(int64_t)k * T] = 0;
    for (int i = 0; i < n; i++) {
      for (int j = 0; j < n; j++) {
        const int64_t e = (int64_t)(i * n + j) * B + c;
        const double re = G[e], im = w * C[e];
        AR(i, j) = re; AI(i, j) = im;
        const double m2 = re * re + im * im;
        finite = finite && isfinite(re) && isfinite(im);
        scale = fmax(scale, m2);
        cm[(int64_t)j * T] = fmaxf(cm[(int64_t)j * T], (float)fmin(m2, 3e38));
      }
      xr[(int64_t)i * T] = br[(int64_t)i * B + c];
      xi[(int64_t)i * T] = bi[(int64_t)i * B + c];
    }
    int code = 0;
    if (!finite) code = KS_STATUS_NONFINITE;
    else if (scale == 0) code = KS_STATUS_SINGULAR;
    // LU with partial pivoting on |entry| (compared squared), row swaps applied to
    // the right-hand side as they happen (the same permutation as solver/cdense.go)
    const double tol = (double)n * 1e-14;
    for (int k = 0; k < n && !code; k++) {
      int p = k;
      double mv = AR(k, k) * AR(k, k) + AI(k, k) * AI(k, k);
      for (int i = k + 1; i < n; i++) {
        const double v = AR(i, k) * AR(i, k) + AI(i, k) * AI(i, k);
        if (v > mv) { mv = v; p = i; }
      }
      if (mv <= (double)cm[(int64_t)k * T] * tol * tol) { code = KS_STATUS_SINGULAR; break; }
      if (p != k) {
        for (int j = 0; j < n; j++) {
          double t = AR(k, j); AR(k, j) = AR(p, j); AR(p, j) = t;
          t = AI(k, j); AI(k, j) = AI(p, j); AI(p, j) = t;
        }
        double t = xr[(int64_t)k * T]; xr[(int64_t)k * T] = xr[(int64_t)p * T]; xr[(int64_t)p * T] = t;
        t = xi[(int64_t)k * T]; xi[(int64_t)k * T] = xi[(int64_t)p * T]; xi[(int64_t)p * T] = t;
      }
      const double pr = AR(k, k), pi = AI(k, k), rm = 1 / mv;
      const double qr = pr * rm, qi = -pi * rm;  // 1 / pivot
      for (int i = k + 1; i < n; i++) {
        const double ar = AR(i, k), ai = AI(i, k);
        const double fr = ar * qr - ai * qi, fi = ar * qi + ai * qr;
        AR(i, k) = fr; AI(i, k) = fi;
        if (fr == 0 && fi == 0) continue;
        for (int j = k + 1; j < n; j++) {
          const double ur = AR(k, j), ui = AI(k, j);
          AR(i, j) -= fr * ur - fi * ui;
          AI(i, j) -= fr * ui + fi * ur;
        }
      }
    }
    if (!code) {
      for (int i = 0; i < n; i++) {  // forward substitution (unit lower)
        double sr = xr[(int64_t)i * T], si = xi[(int64_t)i * T];
        for (int j = 0; j < i; j++) {
          const double lr = AR(i, j), li = AI(i, j), vr = xr[(int64_t)j * T], vi = xi[(int64_t)j * T];
          sr -= lr * vr - li * vi; si -= lr * vi + li * vr;
        }
        xr[(int64_t)i * T] = sr; xi[(int64_t)i * T] = si;
      }
      for (int i = n - 1; i >= 0; i--) {  // back substitution
        double sr = xr[(int64_t)i * T], si = xi[(int64_t)i * T];
        for (int j = i + 1; j < n; j++) {
          const double ur = AR(i, j), ui = AI(i, j), vr = xr[(int64_t)j * T], vi = xi[(int64_t)j * T];
          sr -= ur * vr - ui * vi; si -= ur * vi + ui * vr;
        }
        const double dr = AR(i, i), di = AI(i, i), rm = 1 / (dr * dr + di * di);
        const double vr = (sr * dr + si * di) * rm, vi = (si * dr - sr * di) * rm;
        xr[(int64_t)i * T] = vr; xi[(int64_t)i * T] = vi;
        if (!isfinite(vr) || !isfinite(vi)) code = KS_STATUS_NONFINITE;
      }
    }
#undef AR
#undef AI
    if (code) {  // zero phasors at a failing frequency
      atomicMin(err_at + c, f * 4 + code);
      for (int i = 0; i < 2 * n; i++) o[i] = 0;
      continue;
    }
    for (int i = 0; i < n; i++) { o[2 * i] = xr[(int64_t)i * T]; o[2 * i + 1] = xi[(int64_t)i * T]; }
  }
}

// The status of each circuit from its first failing frequency.
__global__ void k_ac_finish(int64_t B, const int32_t* __restrict__ err_at, int32_t* status) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= B) return;
  const int32_t e = err_at[c];
  if (status[c] == KS_STATUS_OK && e != INT_MAX) status[c] = e & 3;
}

__global__ void k_fill_i32(int32_t* p, int64_t n, int32_t v) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

size_t ks_ac_scratch_doubles(int n, int64_t B) { return (size_t)(2 * n * n + 2 * n) * (size_t)B; }

int ks_launch_ac(const KsDeviceBatch& b, double gmin, const double* x_op, const double* freqs_dev, int32_t nf,
                 double* scratch, int32_t* err_at, int32_t* status, double* out_x, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  const int n = b.plan.n;
  const int64_t B = b.B;
  double* G = scratch;
  double* C = G + (int64_t)n * n * B;
  double* br = C + (int64_t)n * n * B;
  double* bi = br + (int64_t)n * B;
  k_ac_model<<<(unsigned)((B + 127) / 128), 128, 0, st>>>(b.plan, b.values, b.derived, b.state, B, x_op, gmin, G, C,
                                                          br, bi);
  k_fill_i32<<<(unsigned)((B + 255) / 256), 256, 0, st>>>(err_at, B, INT_MAX);
  int dev = 0, sms = 0, maxSmem = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&maxSmem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  // every SM sub-partition needs a warp: as many threads as the shared memory
  // holds (up to 256), not rounded to whole warps
  const size_t perThread = (size_t)(2 * n * n + 2 * n) * sizeof(double) + (size_t)n * sizeof(float);
  int T = (int)std::min<size_t>(256, (size_t)maxSmem / perThread);
  if (T < 1) return -2;
  const size_t smem = perThread * T;
  cudaFuncSetAttribute(k_ac_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_ac_solve, T, smem);
  if (per < 1) per = 1;
  const int64_t units = B * (int64_t)nf;
  const int64_t need = (units + T - 1) / T;
  const int64_t grid = std::min<int64_t>(need, (int64_t)sms * per * 8);
  k_ac_solve<<<(unsigned)grid, T, smem, st>>>(n, B, nf, freqs_dev, G, C, br, bi, status, out_x, err_at);
  k_ac_finish<<<(unsigned)((B + 255) / 256), 256, 0, st>>>(B, err_at, status);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}
