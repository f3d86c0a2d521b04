// ks_tran.cuh — batched transient analysis of the GB300 engine (shared by the generic
// and the per-topology kernels).
//
// One thread runs (*Sim).tran (analysis/tran.go:95-231) for one circuit after another
// as a state machine on top of the shared Newton/dcSolve machine: starting point
// (dcSolve at ModeTranOP, or the UIC solve), then time steps with BE/trapezoidal
// companion models, the h/8 retry on Newton failure, LTE step control
// (device/lte.go:50-85) and landing on source breakpoints (device/waveform.go:190),
// or the fixed-step mode of ks_tran_spec.  Circuits advance through time
// independently; every loop is bounded by the reference's limits.
#pragma once
#include "ks_newton.cuh"

namespace ksg {

// Truncate of every reactive element at the candidate solution x
// (device/reactive.go:178-181, :346-349; device/diode.go:388-397; BJT and
// MOSFET Truncate in device/bjt.go and device/mosfet.go:734-757).
template <class SY, class P>
__device__ __forceinline__ double truncate_all(Thr<SY, P>& t, const TruncParams& tc) {
  double prop = KS_INF;
  SY& x = t.s;
  t.prog.each([&](const KElem& e) KS_INLINE_LAMBDA {
    Col S = state_col(t.Sb, e);
    switch (e.kind) {
      case KS_ELEM_C: {
        double v = xn_(x, e.u[0]) - xn_(x, e.u[1]);
        double i = S[SC_TRAN] != 0 ? S[SC_GEQ] * v + S[SC_IHIST] : 0.0;
        prop = fmin(prop, lte_step(S, SC_HIST, t.V[e.param] * v, i, S[SC_IPREV], tc.abstol, tc));
        break;
      }
      case KS_ELEM_L: {
        double v = xn_(x, e.u[0]) - xn_(x, e.u[1]);
        prop = fmin(prop, lte_step(S, SL_HIST, t.V[e.param] * xn_(x, e.u[2]), v, S[SL_VPREV], tc.vntol, tc));
        break;
      }
      case KS_ELEM_D: {
        int p = e.param;
        if (!(t.V[p + KS_D_P_CJO] > 0 || t.V[p + KS_D_P_TT] > 0)) break;
        double v = xn_(x, e.u[2]) - xn_(x, e.u[1]);
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
        bjt_voltages<true>(e, x, &vbe, &vbc, &vbx, &vcs);
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
        mos_voltages<true>(e, x, &vgs, &vds, &vbs, &vgb);
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
      case KS_ELEM_S: case KS_ELEM_W:  // the step limiters, analysis/tran.go:186-190
        prop = fmin(prop, sw_limit_step(e, t.V, t.D, S, x, tc.h));
        break;
      case KS_ELEM_CN: case KS_ELEM_LN: prop = fmin(prop, nl_truncate(e, t.V, t.D, S, x, tc)); break;
      default: break;
    }
  });
  return prog_min(t.prog, prop);
}

// Restart of every step limiter, analysis/tran.go:213-217: true when the solution
// just accepted changed a switch's state.
template <class SY, class P>
__device__ __forceinline__ bool switch_restart(Thr<SY, P>& t) {
  bool r = false;
  t.prog.each([&](const KElem& e) KS_INLINE_LAMBDA {
    if ((e.kind == KS_ELEM_S || e.kind == KS_ELEM_W) && state_col(t.Sb, e)[SW_FLIP] != 0) r = true;
  });
  return prog_any(t.prog, r);
}

// (*Sim).nextBreakpoint, analysis/tran.go:233-243.
template <class SY, class P>
__device__ __forceinline__ double next_breakpoint(Thr<SY, P>& t, double tnow) {
  double nb = KS_INF;
  t.prog.each([&](const KElem& e) KS_INLINE_LAMBDA {
    if ((e.kind == KS_ELEM_V || e.kind == KS_ELEM_I) && e.wave != KS_WAVE_NONE)
      nb = fmin(nb, wave_next_breakpoint(e.wave, t.D, e.derived, t.V, e.param + KS_SRC_P_ARGS, e.nargs, tnow));
    if (e.kind == KS_ELEM_CN || e.kind == KS_ELEM_LN) {  // stateLaw.nextBreakpoint, device/nonlinear_reactive.go:228-237
      double b = e.wave != KS_WAVE_NONE
                     ? wave_next_breakpoint(e.wave, t.D, e.derived + DN_A0, t.V, e.param + KS_NL_P_ARGS, e.nargs, tnow)
                     : KS_INF;
      const double kt = state_col(t.Sb, e)[SN_KNOTT];
      if (kt > tnow && kt < b) b = kt;
      nb = fmin(nb, b);
    }
  });
  return prog_min(t.prog, nb);
}

// C and L initial conditions for UIC (device/reactive.go:298-303, :466-471).
template <class SY, class P>
__device__ __forceinline__ void set_initial_conditions(Thr<SY, P>& t) {
  t.prog.each([&](const KElem& e) KS_INLINE_LAMBDA {
    Col S = state_col(t.Sb, e);
    bool has = e.flags & KS_F_HAS_IC;
    if (e.kind == KS_ELEM_C) { S[SC_VPREV] = has ? t.V[e.param + KS_RCL_P_IC] : 0.0; S[SC_IPREV] = 0; }
    if (e.kind == KS_ELEM_L) { S[SL_VPREV] = 0; S[SL_IPREV] = has ? t.V[e.param + KS_RCL_P_IC] : 0.0; }
    // device/nonlinear_reactive.go:402-407, :605-610
    if (e.kind == KS_ELEM_CN) { S[SN_VPREV] = has ? t.V[e.param + KS_NL_P_IC] : 0.0; S[SN_IPREV] = 0; }
    if (e.kind == KS_ELEM_LN) { S[SN_VPREV] = 0; S[SN_IPREV] = has ? t.V[e.param + KS_NL_P_IC] : 0.0; }
  });
  prog_sync(t.prog);
}

enum { TR_START = 0, TR_STEP, TR_DONE };

struct TranSpecK {
  double step, stop, start, maxStep, minStep, chgtol, trtol;
  int uic, method, fixed, maxSteps, cap, npts;
};

template <class SY, class P>
__device__ __forceinline__ void record(Thr<SY, P>& t, const TranSpecK& sp, int64_t c, int64_t B, double tnow, int kgrid, int* npts,
                              double* out_time, double* out_wave) {
  const int n = t.n();
  if (sp.fixed) {
    if (out_wave && kgrid < sp.npts) {
      const int64_t base = t.prog.wave_base(c, B, n, kgrid);
#pragma unroll
      for (int i = 0; i < n; i++) out_wave[base + i] = t.s.xn(i);
    }
    return;
  }
  if (tnow < sp.start) return;
  if (*npts < sp.cap) {
    if (out_time) out_time[c * sp.cap + *npts] = tnow;
    if (out_wave) {
#pragma unroll
      for (int i = 0; i < n; i++) out_wave[(c * sp.cap + *npts) * n + i] = t.s.xn(i);
    }
  }
  (*npts)++;
}


// The transient recorder's running ledger state for one circuit
// (analysis/tran.go:248-386): peak power, worst residual, the trapezoid sums of
// inflow, outflow, dissipation and model-supplied power, stored energy at the
// first and last recorded points.
struct TranLedger {
  double peakScale, worstAbs, tPrev, yPrev[4], e[4], storedStart, storedEnd;
  int recorded;
  bool imposedFirst;
  __device__ __forceinline__ void reset() {
    peakScale = worstAbs = tPrev = storedStart = storedEnd = 0;
    for (int q = 0; q < 4; q++) { yPrev[q] = 0; e[q] = 0; }
    recorded = 0;
    imposedFirst = false;
  }
};

// recorder.record and recorder.finish with the element results (ks_results.cuh;
// the results instantiation of the generic kernels only).
template <class SY, class P>
__device__ inline bool tran_point_results(Thr<SY, P>& t, TranLedger& L, const LoadParams& lp, int64_t c, int64_t B,
                                          double tp, bool imposed, bool stored_point, int64_t row);
template <class SY, class P>
__device__ inline bool tran_finish(Thr<SY, P>& t, const TranLedger& L, int64_t c);

// analysis.Tran of one circuit after another, pulled from the queue.  kRes: with
// the element results and the energy ledger of every point (ks_tran_results).
template <class SY, class P, bool kRes = false>
__device__ __forceinline__ void tran_persistent(Thr<SY, P>& t, const TranSpecK& sp, const double* values, const double* derived,
                                       double* state, double* work, int64_t B, double* out_time, double* out_wave,
                                       int32_t* out_npts, int32_t* out_status, int32_t* out_steps, int32_t* out_iters,
                                       uint64_t deadline_ns, unsigned long long* queue) {
  const KOpts& o = t.o;
  const uint64_t t0 = deadline_ns ? prog_clock(t.prog) : 0;
  const double eps = 1e-12 * sp.stop;
  const int maxTotal = o.max_iter_total > 0 ? o.max_iter_total : 0x7fffffff;
  TruncParams tc{0, 0, BE, o.reltol, o.abstol, o.vntol, sp.chgtol, sp.trtol};
  OpState st;
  LoadParams lp;
  int phase = TR_DONE, status = KS_STATUS_OK, accepted = 0, npts = 0, kgrid = 1, order = BE;
  bool hitBreak = false, onGrid = false;
  double tnow = 0, h = 0, tn = 0;
  // step predictor: the accepted history xacc = x_n, save = x_(n-1), ptPrev =
  // x_(n-2) (the DC fallbacks that use save and ptPrev are over by then), the
  // steps h1 = t_n - t_(n-1) and h2 = t_(n-1) - t_(n-2), and how many of those
  // points lie on the present side of the last breakpoint
  double h1 = 0, h2 = 0;
  int hist = 0;
  int64_t c = B;
  TranLedger L;
  // The results of the point at tp before its Accept; true: out of balance (the
  // transient stops after recording it).  Its rows go where record() puts the
  // point: fixed-step [points][B], adaptive [B][cap] (not stored before `start`
  // or beyond the capacity).
  auto point_results = [&](double tp, int k, bool imposed) -> bool {
    if constexpr (kRes) {
      bool stored = sp.fixed || tp >= sp.start;
      int64_t row = -1;
      if (sp.fixed) { if (k < sp.npts) row = (int64_t)k * B + c; }
      else if (stored && npts < sp.cap) row = c * sp.cap + npts;
      return tran_point_results(t, L, lp, c, B, tp, imposed, stored, row);
    } else {
      return false;
    }
  };

  // Starting point of circuit c: analysis/tran.go:103-126.
  auto start = [&]() {
    thr_bind(t, values, derived, state, work, B, c);
    init_state(t.prog, t.D, t.Sb);
    if constexpr (kRes) L.reset();
    lp.method = BE; lp.time = 0; lp.h = 0; lp.rh = 0;
    phase = TR_START; status = KS_STATUS_OK; accepted = 0; npts = 0; kgrid = 1; order = BE;
    tnow = 0; h = 0; tn = 0; h1 = 0; h2 = 0; hist = 0;
    if (sp.uic) {
      set_initial_conditions(t);
      op_state_reset(st, o);
#pragma unroll
      for (int i = 0; i < t.n(); i++) t.s.xn(i) = 0.0;
      lp.mode = ModeUICInit;
    } else {
      dc_start(t, st, nullptr, c);
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
      double nb = next_breakpoint(t, tnow);
      tn = tnow + h;
      if (tn >= nb - eps) { tn = nb; hitBreak = true; }
      if (tn >= sp.stop - eps) { tn = sp.stop; hitBreak = false; }
    }
    h = tn - tnow;
    if (h != lp.h) lp.rh = 1 / h;  // one division per new step size
    lp.mode = ModeTran; lp.time = tn; lp.h = h; lp.method = order;
    st.it = 0; st.maxIter = o.itl4;
    if (o.predict && hist >= 2) {  // Newton starts from the extrapolated history
      // Lagrange extrapolation through the last three points (two after a corner)
      double w0, w1, w2 = 0;
      if (hist >= 3) {
        w0 = (h + h1) * (h + h1 + h2) / (h1 * (h1 + h2));
        w1 = -h * (h + h1 + h2) / (h1 * h2);
        w2 = h * (h + h1) / (h2 * (h1 + h2));
      } else {
        w0 = 1 + h / h1;
        w1 = -h / h1;
      }
#pragma unroll
      for (int i = 0; i < t.n(); i++)
        t.s.xn(i) = w0 * t.xacc[i] + w1 * t.save[i] + (hist >= 3 ? w2 * t.ptPrev[i] : 0.0);
      prog_sync(t.prog);
    }
  };
  auto reject = [&](double hNew) -> bool {  // analysis/tran.go:136-143
    x_from_col(t, t.xacc);
    if (hNew < sp.minStep) { phase = TR_DONE; status = KS_STATUS_TIMESTEP_TOO_SMALL; return false; }
    return true;
  };

  c = prog_next(t.prog, queue);
  if (c < B) start();
  while (c < B) {
    if (phase != TR_DONE) {
      if (deadline_ns && prog_clock(t.prog) - t0 > deadline_ns) { status = KS_STATUS_INTERRUPTED; phase = TR_DONE; }
      else if (o.cancel && (st.total & 7) == 0 && prog_cancelled(t.prog, o.cancel)) {
        status = KS_STATUS_INTERRUPTED; phase = TR_DONE;
      } else if (st.total >= maxTotal) { status = KS_STATUS_NO_CONVERGENCE; phase = TR_DONE; }
    }
    if (phase != TR_DONE) {
      int res = newton_step(t, st, lp);
      if (res < 0) continue;
      if (phase == TR_START) {
        if (!sp.uic) {
          dc_advance(t, st, res);
          if (st.phase != PH_DONE) continue;
          res = st.status;
        }
        if (res != KS_STATUS_OK) { status = res; phase = TR_DONE; }
        else {
          const bool unbalanced = point_results(0.0, 0, sp.uic != 0);  // the UIC point is imposed: not checked
          accept_all(t.prog, t.V, t.D, t.Sb, t.s, 0.0, sp.uic ? ModeUICInit : ModeTranOP, o.gmin, false);
          record(t, sp, c, B, 0.0, 0, &npts, out_time, out_wave);
          if (unbalanced) { status = KS_STATUS_LEDGER; phase = TR_DONE; }
          else {
            hist = 1;
            x_to_col(t, t.xacc);
            phase = TR_STEP;
            st.initJct = false;
            h = sp.fixed ? sp.step : fmin(sp.maxStep, fmin(sp.step, sp.stop / 100)) / 10;
            order = BE;
            begin_step();
          }
        }
      } else if (res != KS_STATUS_OK) {  // a time step's newton failed
        if (!retryable(res) || t.prog.nonlin_empty) { status = res; phase = TR_DONE; }
        else {
          h /= 8;  // analysis/tran.go:168-175
          if (reject(h)) { order = BE; begin_step(); }
        }
      } else {
        double proposal = KS_INF;
        bool rejected = false;
        if (!sp.fixed) {  // analysis/tran.go:178-197
          tc.time = tn; tc.h = h; tc.method = order;
          proposal = truncate_all(t, tc);
          if (proposal < 0.9 * h) {
            h = fmax(proposal, h / 8);
            rejected = true;
            if (reject(h)) begin_step();
          }
        }
        bool unbalanced = false;
        if (!rejected && (!sp.fixed || onGrid)) unbalanced = point_results(tn, kgrid, false);
        if (!rejected) {
          accept_all(t.prog, t.V, t.D, t.Sb, t.s, tn, ModeTran, o.gmin, false);  // :200-208
          if (!sp.fixed || onGrid) record(t, sp, c, B, tn, kgrid, &npts, out_time, out_wave);
          if (switch_restart(t)) hitBreak = true;  // :213-217: restart like a corner
        }
        if (unbalanced) { status = KS_STATUS_LEDGER; phase = TR_DONE; }
        else if (!rejected) {
          if (o.predict) {  // shift the history before x_n <- the new point
#pragma unroll
            for (int i = 0; i < t.n(); i++) { t.ptPrev[i] = t.save[i]; t.save[i] = t.xacc[i]; }
            prog_sync(t.prog);
            h2 = h1; h1 = h;
            // a point on a source corner starts a new history: no extrapolation across it
            hist = hitBreak ? 1 : hist + 1;
          }
          x_to_col(t, t.xacc);
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
              double nb2 = next_breakpoint(t, tnow);
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
    if constexpr (kRes) {
      if (tran_finish(t, L, c) && status == KS_STATUS_OK) status = KS_STATUS_LEDGER;
    }
    if (out_status) out_status[c] = status;
    if (out_steps) out_steps[c] = accepted;
    if (out_iters) out_iters[c] = st.total;
    if (out_npts) out_npts[c] = sp.fixed ? kgrid : (npts < sp.cap ? npts : sp.cap);
    c = prog_next(t.prog, queue);
    if (c < B) start();
  }
}


}  // namespace ksg
