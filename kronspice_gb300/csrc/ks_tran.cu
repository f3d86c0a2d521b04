// ks_tran.cu — batched transient analysis of the GB300 engine.
//
// One thread owns one circuit and runs (*Sim).tran (analysis/tran.go:95-231) as a
// state machine on top of the shared Newton/dcSolve machine: starting point
// (dcSolve at ModeTranOP, or the UIC solve), then time steps with BE/trapezoidal
// companion models, the h/8 retry on Newton failure, LTE step control
// (device/lte.go:50-85) and landing on source breakpoints (device/waveform.go:190),
// or the fixed-step mode of ks_tran_spec.  Circuits advance through time
// independently; every loop is bounded by the reference's limits.
#include <cuda_runtime.h>
#include "ks_internal.h"
#include "ks_newton.cuh"

using namespace ksg;

namespace {

// Truncate of every reactive element at the candidate solution x
// (device/reactive.go:178-181, :346-349; device/diode.go:388-397; BJT and
// MOSFET Truncate in device/bjt.go and device/mosfet.go:734-757).
template <int T>
__device__ double truncate_all(Thr<T>& t, const TruncParams& tc) {
  double prop = CUDART_INF;
  const double* x = t.s.x;
  for (int k = 0; k < t.ne; k++) {
    const KElem& e = t.el[k];
    Col S{t.Sb.p + (int64_t)e.state * t.Sb.B, t.Sb.B};
    switch (e.kind) {
      case KS_ELEM_C: {
        double v = xat(x, e.u[0], T) - xat(x, e.u[1], T);
        double i = S[SC_TRAN] != 0 ? S[SC_GEQ] * v + S[SC_IHIST] : 0.0;
        prop = fmin(prop, lte_step(S, SC_HIST, t.V[e.param] * v, i, S[SC_IPREV], tc.abstol, tc));
        break;
      }
      case KS_ELEM_L: {
        double v = xat(x, e.u[0], T) - xat(x, e.u[1], T);
        prop = fmin(prop, lte_step(S, SL_HIST, t.V[e.param] * x[e.u[2] * T], v, S[SL_VPREV], tc.vntol, tc));
        break;
      }
      case KS_ELEM_D: {
        int p = e.param;
        if (!(t.V[p + KS_D_P_CJO] > 0 || t.V[p + KS_D_P_TT] > 0)) break;
        double v = xat(x, e.u[2], T) - xat(x, e.u[1], T);
        double id, g, q, c;
        diode_iv(t.V, t.D, p, e.derived, e.flags & KS_F_HAS_BV, v, &id, &g);
        diode_charge(t.V, p, v, id, g, &q, &c);
        double ic = S[SD_IQ] + S[SD_GEQ] * (v - S[SD_VD]);
        prop = fmin(prop, lte_step(S, SD_HIST, q, ic, S[SD_IQPREV], tc.abstol, tc));
        break;
      }
      case KS_ELEM_Q: {
        if (S[SQ_TRAN] == 0) break;
        double vbe, vbc, vbx, vcs;
        bjt_voltages<T>(e, t.V, x, &vbe, &vbc, &vbx, &vcs);
        BjtDC d = bjt_eval_dc(t.V, t.D, e.param, e.derived, vbe, vbc, t.o.gmin);
        BjtCh ch = bjt_charges(t.V, t.D, e.param, e.derived, vbe, vbc, vbx, vcs, d);
        double dv[4] = {vbe - S[SQ_VBE], vbc - S[SQ_VBC], vbx - S[SQ_VBX], vcs - S[SQ_VCS]};
        for (int j = 0; j < 4; j++) {
          if (ch.q[j] == 0 && S[SQ_QPREV0 + j] == 0) continue;
          double i = S[SQ_IQ0 + j] + S[SQ_AG] * S[SQ_C0 + j] * dv[j];
          if (j == 0) i += S[SQ_AG] * S[SQ_DQBEDVBC] * dv[1];
          prop = fmin(prop, lte_step(S, SQ_HIST + j * H_SIZE, ch.q[j], i, S[SQ_IQPREV0 + j], tc.abstol, tc));
        }
        break;
      }
      case KS_ELEM_M: {
        if (S[SM_TRAN] == 0) break;
        double vgs, vds, vbs, vgb;
        mos_voltages<T>(e, x, &vgs, &vds, &vbs, &vgb);
        double v[5] = {vgs, vgs - vds, vgb, vbs, vbs - vds};
        for (int j = 0; j < 5; j++) {
          double qk, cap, tmp;
          if (j < 3) { cap = S[SM_CAPG0 + j]; qk = S[SM_QPREV0 + j] + cap * (v[j] - S[SM_VPREV0 + j]); }
          else {
            cap = S[SM_CAPB0 + j - 3];
            if (j == 3) mos_bulk_charge(t.V, e.param, t.D, e.derived, v[j], t.D[e.derived + DM_CZBS], t.D[e.derived + DM_CZBSSW], &qk, &tmp);
            else mos_bulk_charge(t.V, e.param, t.D, e.derived, v[j], t.D[e.derived + DM_CZBD], t.D[e.derived + DM_CZBDSW], &qk, &tmp);
          }
          if (qk == 0 && S[SM_QPREV0 + j] == 0) continue;
          double i = S[SM_IQ0 + j] + S[SM_AG] * cap * (v[j] - S[SM_DV0 + j]);
          prop = fmin(prop, lte_step(S, SM_HIST + j * H_SIZE, qk, i, S[SM_IQPREV0 + j], tc.abstol, tc));
        }
        break;
      }
      default: break;
    }
  }
  return prop;
}

// (*Sim).nextBreakpoint, analysis/tran.go:233-243.
template <int T>
__device__ double next_breakpoint(Thr<T>& t, double tnow) {
  double nb = CUDART_INF;
  for (int k = 0; k < t.ne; k++) {
    const KElem& e = t.el[k];
    if ((e.kind == KS_ELEM_V || e.kind == KS_ELEM_I) && e.wave != KS_WAVE_NONE)
      nb = fmin(nb, wave_next_breakpoint(e.wave, t.D, e.derived, t.V, e.param + KS_SRC_P_ARGS, e.nargs, tnow));
  }
  return nb;
}

// C and L initial conditions for UIC (device/reactive.go:298-303, :466-471).
template <int T>
__device__ void set_initial_conditions(Thr<T>& t) {
  for (int k = 0; k < t.ne; k++) {
    const KElem& e = t.el[k];
    Col S{t.Sb.p + (int64_t)e.state * t.Sb.B, t.Sb.B};
    bool has = e.flags & KS_F_HAS_IC;
    if (e.kind == KS_ELEM_C) { S[SC_VPREV] = has ? t.V[e.param + KS_RCL_P_IC] : 0.0; S[SC_IPREV] = 0; }
    if (e.kind == KS_ELEM_L) { S[SL_VPREV] = 0; S[SL_IPREV] = has ? t.V[e.param + KS_RCL_P_IC] : 0.0; }
  }
}

enum { TR_START = 0, TR_STEP, TR_DONE };

struct TranSpecK {
  double step, stop, start, maxStep, minStep, chgtol, trtol;
  int uic, method, fixed, maxSteps, cap, npts;
};

template <int T>
__device__ inline void record(Thr<T>& t, const TranSpecK& sp, int64_t c, int64_t B, double tnow, int kgrid, int* npts,
                              double* out_time, double* out_wave) {
  const int n = t.n;
  if (sp.fixed) {
    if (out_wave && kgrid < sp.npts)
      for (int i = 0; i < n; i++) out_wave[((int64_t)kgrid * B + c) * n + i] = t.s.x[i * T];
    return;
  }
  if (tnow < sp.start) return;
  if (*npts < sp.cap) {
    if (out_time) out_time[c * sp.cap + *npts] = tnow;
    if (out_wave) for (int i = 0; i < n; i++) out_wave[(c * sp.cap + *npts) * n + i] = t.s.x[i * T];
  }
  (*npts)++;
}

}  // namespace

template <int T>
__global__ void __launch_bounds__(T) k_tran(KPlan plan, KOpts o, TranSpecK sp, const double* __restrict__ values,
                                            const double* __restrict__ derived, double* state, double* work, int64_t B,
                                            double* out_time, double* out_wave, int32_t* out_npts, int32_t* out_status,
                                            int32_t* out_steps, int32_t* out_iters, uint64_t deadline_ns,
                                            unsigned long long* queue) {
  extern __shared__ __align__(16) unsigned char smem[];
  Thr<T> t;
  thr_init<T>(t, plan, o, smem, values, derived, state, work, B, 0);
  __syncthreads();
  const int n = t.n;
  const uint64_t t0 = deadline_ns ? globaltimer_ns() : 0;
  const double eps = 1e-12 * sp.stop;
  const int maxTotal = o.max_iter_total > 0 ? o.max_iter_total : 0x7fffffff;
  TruncParams tc{0, 0, BE, o.reltol, o.abstol, o.vntol, sp.chgtol, sp.trtol};
  OpState st;
  LoadParams lp;
  int phase = TR_DONE, status = KS_STATUS_OK, accepted = 0, npts = 0, kgrid = 1, order = BE;
  bool hitBreak = false, onGrid = false;
  double tnow = 0, h = 0, tn = 0;
  int64_t c = B;

  // Starting point of circuit c: analysis/tran.go:103-126.
  auto start = [&]() {
    thr_bind<T>(t, values, derived, state, work, B, c);
    init_state(t.el, t.ne, t.n_state, t.D, t.Sb);
    lp.method = BE; lp.time = 0; lp.h = 0;
    phase = TR_START; status = KS_STATUS_OK; accepted = 0; npts = 0; kgrid = 1; order = BE;
    tnow = 0; h = 0; tn = 0;
    if (sp.uic) {
      set_initial_conditions<T>(t);
      op_state_reset<T>(st, o);
      for (int i = 0; i < n; i++) t.s.x[i * T] = 0.0;
      lp.mode = ModeUICInit;
    } else {
      dc_start<T>(t, st, nullptr, c, ModeTranOP);
      lp.mode = ModeTranOP;
    }
  };
  // The head of the time loop, analysis/tran.go:145-163.
  auto begin_step = [&]() {
    if (sp.fixed ? (kgrid > sp.npts - 1) : !(tnow < sp.stop - eps)) { phase = TR_DONE; status = KS_STATUS_OK; return; }
    if (accepted >= sp.maxSteps) { phase = TR_DONE; status = KS_STATUS_TOO_MANY_STEPS; return; }
    hitBreak = false; onGrid = false;
    if (sp.fixed) {
      double target = (double)kgrid * sp.step;
      tn = tnow + h;
      if (tn >= target - eps) { tn = target; onGrid = true; }
    } else {
      double nb = next_breakpoint<T>(t, tnow);
      tn = tnow + h;
      if (tn >= nb - eps) { tn = nb; hitBreak = true; }
      if (tn >= sp.stop - eps) { tn = sp.stop; hitBreak = false; }
    }
    h = tn - tnow;
    lp.mode = ModeTran; lp.time = tn; lp.h = h; lp.method = order;
    st.it = 0; st.maxIter = o.itl4;
  };
  auto reject = [&](double hNew) -> bool {  // analysis/tran.go:136-143
    for (int i = 0; i < n; i++) t.s.x[i * T] = t.xacc[i];
    if (hNew < sp.minStep) { phase = TR_DONE; status = KS_STATUS_TIMESTEP_TOO_SMALL; return false; }
    return true;
  };

  c = (int64_t)atomicAdd(queue, 1ull);
  if (c < B) start();
  while (c < B) {
    if (phase != TR_DONE) {
      if (deadline_ns && globaltimer_ns() - t0 > deadline_ns) { status = KS_STATUS_INTERRUPTED; phase = TR_DONE; }
      else if (st.total >= maxTotal) { status = KS_STATUS_NO_CONVERGENCE; phase = TR_DONE; }
    }
    if (phase != TR_DONE) {
      int res = newton_step<T>(t, st, lp);
      if (res < 0) continue;
      if (phase == TR_START) {
        if (!sp.uic) {
          dc_advance<T>(t, st, res);
          if (st.phase != PH_DONE) continue;
          res = st.status;
        }
        if (res != KS_STATUS_OK) { status = res; phase = TR_DONE; }
        else {
          accept_all<T>(t.el, t.ne, t.V, t.D, t.Sb, t.s.x, 0.0, sp.uic ? ModeUICInit : ModeTranOP, o.gmin, false);
          record<T>(t, sp, c, B, 0.0, 0, &npts, out_time, out_wave);
          for (int i = 0; i < n; i++) t.xacc[i] = t.s.x[i * T];
          phase = TR_STEP;
          st.initJct = false;
          h = sp.fixed ? sp.step : fmin(sp.maxStep, fmin(sp.step, sp.stop / 100)) / 10;
          order = BE;
          begin_step();
        }
      } else if (res != KS_STATUS_OK) {  // a time step's newton failed
        if (!retryable(res) || t.nonlinEmpty) { status = res; phase = TR_DONE; }
        else {
          h /= 8;  // analysis/tran.go:168-175
          if (reject(h)) { order = BE; begin_step(); }
        }
      } else {
        double proposal = CUDART_INF;
        bool rejected = false;
        if (!sp.fixed) {  // analysis/tran.go:178-197
          tc.time = tn; tc.h = h; tc.method = order;
          proposal = truncate_all<T>(t, tc);
          if (proposal < 0.9 * h) {
            h = fmax(proposal, h / 8);
            rejected = true;
            if (reject(h)) begin_step();
          }
        }
        if (!rejected) {
          accept_all<T>(t.el, t.ne, t.V, t.D, t.Sb, t.s.x, tn, ModeTran, o.gmin, false);  // :200-208
          if (!sp.fixed || onGrid) record<T>(t, sp, c, B, tn, kgrid, &npts, out_time, out_wave);
          for (int i = 0; i < n; i++) t.xacc[i] = t.s.x[i * T];
          accepted++;
          tnow = tn;
          order = sp.method;
          if (sp.fixed) {
            if (onGrid) kgrid++;
            h = fmax(fmin(2 * h, sp.maxStep), sp.minStep);
          } else {  // :211-225
            double next = fmin(fmin(proposal, 2 * h), sp.maxStep);
            if (hitBreak) {
              order = BE;
              double nb2 = next_breakpoint<T>(t, tnow);
              next = fmin(next, 0.1 * fmin(sp.maxStep, nb2 - tnow));
            }
            h = fmax(next, sp.minStep);
          }
          begin_step();
        }
      }
      if (phase != TR_DONE) continue;
    }
    // circuit c finished: write its results and take the next one
    if (out_status) out_status[c] = status;
    if (out_steps) out_steps[c] = accepted;
    if (out_iters) out_iters[c] = st.total;
    if (out_npts) out_npts[c] = sp.fixed ? kgrid : (npts < sp.cap ? npts : sp.cap);
    c = (int64_t)atomicAdd(queue, 1ull);
    if (c < B) start();
  }
}

int ks_launch_tran(const KsDeviceBatch& b, const KOpts& o, const ks_tran_spec& spec, int cap, double* out_time,
                   double* out_wave, int32_t* out_npts, int32_t* out_status, int32_t* out_steps, int32_t* out_iters,
                   double deadline_s, void* stream) {
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
  int maxSmem = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&maxSmem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  int T = 64;
  size_t sm = thr_smem(n, ne, 64);
  if (sm > (size_t)maxSmem) { T = 32; sm = thr_smem(n, ne, 32); }
  if (sm > (size_t)maxSmem) return -2;
  cudaStream_t st = (cudaStream_t)stream;
  if (cudaMemsetAsync(b.queue, 0, sizeof(unsigned long long), st) != cudaSuccess) return -1;
  int sms = 0, per = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (T == 64) {
    cudaFuncSetAttribute(k_tran<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_tran<64>, 64, sm);
  } else {
    cudaFuncSetAttribute(k_tran<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_tran<32>, 32, sm);
  }
  int64_t need = (b.B + T - 1) / T, cap_blocks = (int64_t)sms * (per > 0 ? per : 1);
  unsigned grid = (unsigned)(need < cap_blocks ? need : cap_blocks);
  if (T == 64)
    k_tran<64><<<grid, 64, sm, st>>>(b.plan, o, sp, b.values, b.derived, b.state, b.work, b.B, out_time, out_wave,
                                     out_npts, out_status, out_steps, out_iters, dl, b.queue);
  else
    k_tran<32><<<grid, 32, sm, st>>>(b.plan, o, sp, b.values, b.derived, b.state, b.work, b.B, out_time, out_wave,
                                     out_npts, out_status, out_steps, out_iters, dl, b.queue);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}
