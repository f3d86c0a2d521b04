// ks_results.cuh — element results and the energy ledger of the GB300 engine.
//
// What the reference returns beside the solution, computed per circuit on the
// device at the accepted solution x:
//   element operating points  device Operating (passive.go:86, reactive.go:109 and
//                             :289, source.go:114 and :163, diode.go:293,
//                             bjt.go:537-576, mosfet.go:635-665), from the
//                             linearization of each device's last load (its state
//                             block), so the reported currents satisfy KCL exactly
//   exterior / model powers   ExteriorPower and ModelSuppliedPower of each device
//   stored energy             StoredEnergy (reactive.go:172, :340; diode.go:329-387
//                             in closed form; bjt.go:630-650 and mosfet.go:710-731
//                             by 16-point Gauss-Legendre quadrature on 8 panels)
//   the ledger                em.Accumulator (em/energy.go:24-80) in the order of
//                             em.BuildLedger (:90-121) for an operating point and
//                             of recorder.record (analysis/tran.go:291-347) for a
//                             transient point
//   round-off estimate        (*Sim).roundoff (analysis/op.go:275-282) of the last
//                             linear system, rebuilt by loading every element once
//                             more at the last linearization point (the solve's
//                             system has been factored in place), on a scratch
//                             copy of the device state.
// Only the generic kernels' results instantiation includes this code.
#pragma once
#include "ks_tran.cuh"

namespace ksg {

struct ElemOp {
  double v, i, p, ps, w, ext, sup;  // Voltage, Current, PowerAbsorbed, StoragePower, StoredEnergy, ExteriorPower, ModelSupplied
  bool thermal;                     // the exterior port is the thermal one (else electrical)
  bool stores;                      // a device.Reactive element
};

// integrate, device/bjt.go:607-627: 16-point Gauss-Legendre on n equal panels
// (Abramowitz & Stegun, Table 25.4).
template <class F>
__device__ inline double gl16(F&& f, double a, double b, int n) {
  const double gx[8] = {0.0950125098376374, 0.2816035507792589, 0.4580167776572274, 0.6178762444026438,
                        0.7554044083550030, 0.8656312023878318, 0.9445750230732326, 0.9894009349916499};
  const double gw[8] = {0.1894506104550685, 0.1826034150449236, 0.1691565193950025, 0.1495959888165767,
                        0.1246289712555339, 0.0951585116824928, 0.0622535239386479, 0.0271524594117541};
  double h = (b - a) / n, s = 0;
  for (int p = 0; p < n; p++) {
    double mid = a + (p + 0.5) * h, half = h / 2;
    for (int k = 0; k < 8; k++) s += gw[k] * (f(mid - half * gx[k]) + f(mid + half * gx[k]));
  }
  return s * h / 2;
}

// Diode StoredEnergy, device/diode.go:329-387: v q(v) - (integral of the depletion
// charge) - TT (integral of the junction current), both integrals in closed form.
__device__ inline double diode_stored(const KElem& e, const Col& V, const Col& Dv, double v) {
  const int p = e.param, dd = e.derived;
  const double IS = V[p + KS_D_P_IS], CJO = V[p + KS_D_P_CJO], VJ = V[p + KS_D_P_VJ], M = V[p + KS_D_P_M];
  const double FC = V[p + KS_D_P_FC], TT = V[p + KS_D_P_TT], vte = Dv[dd + DD_VTE], xbv = Dv[dd + DD_XBV];
  const bool hasBV = e.flags & KS_F_HAS_BV;
  double id, g, q, c;
  diode_iv(V, Dv, p, dd, hasBV, v, &id, &g);
  diode_charge(V, p, v, id, g, &q, &c);
  double idep = 0;  // intDepletion, :340-361
  if (CJO != 0) {
    const double fcv = FC * VJ;
    auto below = [&](double w) { return CJO * VJ / (1 - M) * (w + VJ / (2 - M) * (pow(1 - w / VJ, 2 - M) - 1)); };
    if (v < fcv) idep = below(v);
    else {
      double f1 = VJ * (1 - pow(1 - FC, 1 - M)) / (1 - M), f2 = pow(1 - FC, 1 + M), f3 = 1 - FC * (1 + M);
      double dv = v - fcv;
      idep = below(fcv) + CJO * f1 * dv +
             CJO / f2 * (f3 * dv * dv / 2 + M / (2 * VJ) * ((v * v * v - fcv * fcv * fcv) / 3 - fcv * fcv * dv));
    }
  }
  double icur;  // intCurrent, :363-387
  auto fwd = [&](double w) { return IS * (vte * expm1(fmin(w / vte, 700.0)) - w); };
  const double v1 = -3 * vte;
  if (v >= v1) icur = fwd(v);
  else {
    double a3 = pow(3 * vte / kE, 3.0);
    auto rev = [&](double w) { return -IS * (w - a3 / (2 * w * w)); };
    double v2 = v;
    if (hasBV && v < -xbv) v2 = -xbv;
    icur = fwd(v1) + (rev(v2) - rev(v1));
    if (v2 != v) {
      auto brk = [&](double w) { return IS * vte * exp(fmin(-(xbv + w) / vte, 700.0)); };
      icur = icur + brk(v) - brk(v2);
    }
  }
  return v * q - idep - TT * icur;
}

// One element's operating point at the solution xn of the thread's system (the
// stored energy only when `energy`).
template <class SY>
__device__ inline ElemOp elem_operating(const KElem& e, const Col& V, const Col& Dv, const Col& S, SY& s,
                                        double gmin, bool energy) {
  ElemOp o{0, 0, 0, 0, 0, 0, 0, true, false};
  auto X = [&](int i) { return xn_(s, i); };
  const int p = e.param, dd = e.derived;
  switch (e.kind) {
    case KS_ELEM_R: {  // device/passive.go:86-113
      o.v = X(e.u[0]) - X(e.u[1]);
      o.i = o.v * Dv[dd + DR_G];
      o.p = o.v * o.i;
      if (V[p + KS_RCL_P_VALUE] > 0) o.ext = -o.p;  // Joule heat out through the thermal port
      else o.sup = -o.p;                            // negative resistance: model-supplied
      break;
    }
    case KS_ELEM_C: {  // device/reactive.go:109-130, :172-175
      o.v = X(e.u[0]) - X(e.u[1]);
      o.i = S[SC_TRAN] != 0 ? S[SC_GEQ] * o.v + S[SC_IHIST] : 0.0;
      o.p = o.v * o.i; o.ps = o.v * o.i;
      if (energy) o.w = 0.5 * V[p + KS_RCL_P_VALUE] * o.v * o.v;
      o.stores = true;
      break;
    }
    case KS_ELEM_L: {  // device/reactive.go:289-300, :340-342
      o.v = X(e.u[0]) - X(e.u[1]);
      o.i = X(e.u[2]);
      o.p = o.v * o.i; o.ps = o.v * o.i;
      if (energy) o.w = 0.5 * V[p + KS_RCL_P_VALUE] * o.i * o.i;
      o.stores = true;
      break;
    }
    case KS_ELEM_V:  // device/source.go:114-129
    case KS_ELEM_I: {  // device/source.go:163-177
      o.v = X(e.u[0]) - X(e.u[1]);
      o.i = e.kind == KS_ELEM_V ? X(e.u[2]) : S[SV_VALUE];
      o.p = o.v * o.i;
      o.ext = -o.p;
      o.thermal = false;
      break;
    }
    case KS_ELEM_D: {  // device/diode.go:293-301, :400-405
      const double vj = X(e.u[2]) - X(e.u[1]), d = vj - S[SD_VD];
      const double ir = S[SD_CD] + S[SD_GD] * d, ic = S[SD_IQ] + S[SD_GEQ] * d;
      o.i = ir + ic;
      o.v = X(e.u[0]) - X(e.u[1]);
      o.p = o.v * o.i; o.ps = vj * ic;
      o.ext = -(o.p - o.ps);
      o.stores = true;
      if (energy && (V[p + KS_D_P_CJO] > 0 || V[p + KS_D_P_TT] > 0)) o.w = diode_stored(e, V, Dv, vj);
      break;
    }
    case KS_ELEM_Q: {  // terminalCurrents + Operating, device/bjt.go:537-576; ExteriorPower :675-680
      double vbe, vbc, vbx, vcs;
      bjt_voltages<true>(e, s, &vbe, &vbc, &vbx, &vcs);
      const double t = (e.flags & KS_F_PTYPE) ? -1.0 : 1.0;
      const double dbe = vbe - S[SQ_VBE], dbc = vbc - S[SQ_VBC];
      const double it = t * (S[SQ_IT] + S[SQ_ITBE] * dbe + S[SQ_ITBC] * dbc);
      const double ibe = t * (S[SQ_IBE] + S[SQ_GPI] * dbe);
      const double ibc = t * (S[SQ_IBC] + S[SQ_GMU] * dbc);
      double iqbe = 0, iqbc = 0, iqbx = 0, iqcs = 0;
      if (S[SQ_TRAN] != 0) {
        const double ag = S[SQ_AG];
        iqbe = t * (S[SQ_IQ0] + ag * S[SQ_C0] * dbe + ag * S[SQ_DQBEDVBC] * dbc);
        iqbc = t * (S[SQ_IQ0 + 1] + ag * S[SQ_C0 + 1] * dbc);
        iqbx = t * (S[SQ_IQ0 + 2] + ag * S[SQ_C0 + 2] * (vbx - S[SQ_VBX]));
        iqcs = t * (S[SQ_IQ0 + 3] + ag * S[SQ_C0 + 3] * (vcs - S[SQ_VCS]));
        o.ps = vbe * t * iqbe + vbc * t * iqbc + vbx * t * iqbx + vcs * t * iqcs;
      }
      const double isb = t * (S[SQ_ISUB] + S[SQ_GSUB] * (vcs - S[SQ_VCS])) + iqcs;
      double ic = it - ibc - iqbc - iqbx, ib = ibe + ibc + iqbe + iqbc + iqbx, ie = -it - ibe - iqbe, is;
      if (V[p + KS_Q_P_SUBS] > 0) { is = isb; ic = ic - isb; }
      else { ib = ib + isb; is = -isb; }
      const double vc = X(e.u[0]), ve = X(e.u[1]);
      o.p = vc * ic + X(e.u[2]) * ib + ve * ie + X(e.u[3]) * is;
      o.v = vc - ve; o.i = ic;
      o.ext = -(o.p - o.ps);
      o.stores = true;
      // StoredEnergy, :630-650: co-energy of the four charges
      if (energy && (V[p + KS_Q_P_CJE] > 0 || V[p + KS_Q_P_CJC] > 0 || V[p + KS_Q_P_CJS] > 0 ||
                     V[p + KS_Q_P_TF] > 0 || V[p + KS_Q_P_TR] > 0)) {
        const double v4[4] = {vbe, vbc, vbx, vcs};
        for (int k = 0; k < 4; k++) {
          if (v4[k] == 0) continue;
          auto qk = [&](double u) {
            double w0 = k == 0 ? u : v4[0], w1 = k == 1 ? u : v4[1], w2 = k == 2 ? u : v4[2], w3 = k == 3 ? u : v4[3];
            BjtDC dc = bjt_eval_dc(V, Dv, p, dd, w0, w1, gmin);
            return bjt_charges(V, Dv, p, dd, w0, w1, w2, w3, dc).q[k];
          };
          o.w += v4[k] * qk(v4[k]) - gl16(qk, 0.0, v4[k], 8);
        }
      }
      break;
    }
    case KS_ELEM_M: {  // terminalCurrents + Operating, device/mosfet.go:635-665; ExteriorPower :760-765
      double vgs, vds, vbs, vgb;
      mos_voltages<true>(e, s, &vgs, &vds, &vbs, &vgb);
      const double vbd = vbs - vds, vgd = vgs - vds, t = (e.flags & KS_F_PTYPE) ? -1.0 : 1.0;
      double i0 = S[SM_CDRAIN], g0 = S[SM_GM], g1 = S[SM_GDS], g2 = S[SM_GMBS];
      if (S[SM_MODE] <= 0) { const double gm = g0; i0 = -i0; g0 = -gm; g1 = gm + g1 + g2; g2 = -g2; }
      const double ich = t * (i0 + g0 * (vgs - S[SM_VGS]) + g1 * (vds - S[SM_VDS]) + g2 * (vbs - S[SM_VBS]));
      const double ibs = t * (S[SM_CBS] + S[SM_GBS] * (vbs - S[SM_VBS]));
      const double ibdc = t * (S[SM_CBD] + S[SM_GBD] * (vbd - S[SM_VBD]));
      const double v5[5] = {vgs, vgd, vgb, vbs, vbd};
      double iq[5] = {0, 0, 0, 0, 0};
      if (S[SM_TRAN] != 0) {
        const double ag = S[SM_AG];
        for (int k = 0; k < 5; k++) {
          const double cap = k < 3 ? S[SM_CAPG0 + k] : S[SM_CAPB0 + k - 3];
          iq[k] = t * (S[SM_IQ0 + k] + ag * cap * (v5[k] - S[SM_DV0 + k]));
          o.ps += v5[k] * t * iq[k];
        }
      }
      const double id = ich - ibdc - iq[1] - iq[4], is = -ich - ibs - iq[0] - iq[3];
      const double ig = iq[0] + iq[1] + iq[2], ib = ibs + ibdc - iq[2] + iq[3] + iq[4];
      const double vd = X(e.u[0]), vs = X(e.u[1]);
      o.p = vd * id + X(e.u[2]) * ig + vs * is + X(e.u[3]) * ib;
      o.v = vd - vs; o.i = id;
      o.ext = -(o.p - o.ps);
      o.stores = true;
      // StoredEnergy, :710-731
      if (energy && (Dv[dd + DM_HASGCAP] != 0 || Dv[dd + DM_HASJCAP] != 0)) {
        for (int k = 0; k < 2; k++) {
          const double vv = v5[3 + k];
          const double cz = Dv[dd + (k == 0 ? DM_CZBS : DM_CZBD)], czsw = Dv[dd + (k == 0 ? DM_CZBSSW : DM_CZBDSW)];
          if (vv == 0 || cz + czsw == 0) continue;
          auto qf = [&](double u) {
            double q, c;
            mos_bulk_charge(V, p, Dv, dd, u, cz, czsw, &q, &c);
            return q;
          };
          o.w += vv * qf(vv) - gl16(qf, 0.0, vv, 8);
        }
        double ch[7], mc[3];
        mos_channel(e, V, Dv, v5[0], v5[0] - v5[1], v5[3], ch);
        meyer_caps(Dv, dd, v5[0], v5[1], ch[5], ch[6], ch[0], mc);
        const double ov[3] = {Dv[dd + DM_CGSO], Dv[dd + DM_CGDO], Dv[dd + DM_CGBO]};
        for (int k = 0; k < 3; k++) o.w += 0.5 * (mc[k] + ov[k]) * v5[k] * v5[k];
      }
      break;
    }
    case KS_ELEM_E: case KS_ELEM_F: case KS_ELEM_G: case KS_ELEM_H: {  // device/controlled.go:123-140
      o.v = X(e.u[0]) - X(e.u[1]);
      if (e.kind == KS_ELEM_E || e.kind == KS_ELEM_H) o.i = X(e.u[2]);
      else {
        const double ctl = e.kind == KS_ELEM_G ? X(e.u[3]) - X(e.u[4]) : X(e.u[3]);
        o.i = V[p + KS_CTL_P_GAIN] * ctl;
      }
      o.p = o.v * o.i;
      o.sup = -o.p;  // idealized: its power is model-supplied, it has no exterior port
      o.thermal = false;
      break;
    }
    case KS_ELEM_K: {  // device/mutual.go:120-133: no voltage, current or power of its own
      if (energy) o.w = Dv[dd + DK_M] * X(e.u[0]) * X(e.u[1]);
      o.stores = true;
      break;
    }
    case KS_ELEM_CN: case KS_ELEM_LN: {  // device/nonlinear_reactive.go:368-376, :577-582; StoredEnergy :410, :612
      NlLaw law(e, V, Dv);
      o.v = X(e.u[0]) - X(e.u[1]);
      o.i = nl_current(e, S, s);
      o.p = o.v * o.i;
      const double x = e.kind == KS_ELEM_LN ? o.i : o.v;
      // scalePower, :360-365: s'(t) F(x) leaves through the scale's port
      const double sp = (S[SN_TRAN] == 0 || S[SN_SDOT] == 0) ? 0.0 : S[SN_SDOT] * law.coenergy(x);
      o.ps = o.p - sp;
      if (energy) o.w = law.s(S[SN_T]) * law.energy(x);
      o.stores = true;
      o.thermal = false;  // the scale's port: mechanical
      if (e.wave != KS_WAVE_NONE) o.ext = -sp;
      break;
    }
    case KS_ELEM_S: case KS_ELEM_W: {  // device/switch.go:246-250, ExteriorPower :304-310
      o.v = X(e.u[0]) - X(e.u[1]);
      o.i = S[SW_G] * o.v + S[SW_K] * (sw_control(e, s) - S[SW_C0]);  // the current the solve used
      o.p = o.v * o.i;
      o.ext = -o.p;  // Joule heat out through the thermal port
      break;
    }
    default: break;
  }
  return o;
}

// em.Accumulator, em/energy.go:24-80.
struct LedgerAcc {
  double in, out, diss, store, sup, scale;
  __device__ __forceinline__ void zero() { in = out = diss = store = sup = scale = 0; }
  __device__ __forceinline__ void port(bool thermal, double pw) {  // AddPort :33-51
    if (pw == 0) return;
    scale += fabs(pw);
    if (thermal && pw < 0) diss += -pw;
    else if (pw > 0) in += pw;
    else out += -pw;
  }
  __device__ __forceinline__ void storage(double p) { store += p; scale += fabs(p); }  // AddStorage :54-57
  __device__ __forceinline__ void supplied(double p) {                                // AddModelSupplied :62-68
    if (p == 0) return;
    sup += p; scale += fabs(p);
  }
  __device__ __forceinline__ double residual() const { return in + sup - out - diss - store; }  // :71-73
};

constexpr double kLedgerAbsFloor = 1e-21;  // output/result.go:96
constexpr double kGrossTol = 1e-3;         // analysis/tran.go:272

// (*Sim).roundoff, analysis/op.go:275-282, of the system of the last load: every
// element is loaded once more at the last linearization point xo (with lp, the
// parameters of that load) into the thread's system, on a scratch copy of the
// circuit's device state, and 64 * 2^-52 * sum |x_i| (|A| |x| + |rhs|)_i is taken
// at the solution xn.
template <class SY, class P>
__device__ inline double roundoff_at(Thr<SY, P>& t, LoadParams lp, int64_t c, int64_t B) {
  Col Sc{t.o.res_scratch + c, B};
  for (int k = 0; k < t.prog.n_state; k++) Sc[k] = t.Sb[k];
  lp.initJct = false; lp.gmin = t.o.gmin; lp.srcStepping = false; lp.srcFact = 0;
  load_all(t.prog, t.V, t.D, Sc, t.s, lp);
  const int n = t.n();
  double sum = 0;
  for (int i = 0; i < n; i++) {
    double ab = 0;
    for (int j = 0; j < n; j++) ab += fabs(t.s.a(i, j)) * fabs(t.s.xn(j));
    sum += fabs(t.s.xn(i)) * (ab + fabs(t.s.rhs(i)));
  }
  return 64 * 0x1p-52 * sum;
}

// (*Sim).result + em.BuildLedger + em.CheckLedger (analysis/op.go:340-403,
// em/energy.go:90-128) of circuit c at its accepted operating point, before the
// Accept: element rows and the ledger into the results buffers.  Returns the
// circuit's status (KS_STATUS_LEDGER when the ledger does not balance).
template <class SY, class P>
__device__ inline int op_results(Thr<SY, P>& t, const LoadParams& lp, int64_t c, int64_t B) {
  const KOpts& o = t.o;
  const int ne = t.prog.ne;
  LedgerAcc a;
  a.zero();
  int k = 0;
  t.prog.each([&](const KElem& e) {
    ElemOp r = elem_operating(e, t.V, t.D, state_col(t.Sb, e), t.s, o.gmin, true);
    if (o.res_elem) {
      double* row = o.res_elem + ((int64_t)c * ne + k) * KS_RES_COLS;
      row[KS_RES_VOLTAGE] = r.v; row[KS_RES_CURRENT] = r.i; row[KS_RES_POWER] = r.p;
      row[KS_RES_STORAGE_POWER] = r.ps; row[KS_RES_STORED_ENERGY] = r.w; row[KS_RES_EXTERIOR_POWER] = r.ext;
      row[KS_RES_MODEL_SUPPLIED] = r.sup;
    }
    a.port(r.thermal, r.ext);
    if (r.stores) a.storage(r.ps);
    if (r.sup != 0) a.supplied(r.sup);
    k++;
  });
  const double ro = roundoff_at(t, lp, c, B);
  const double res = a.residual();
  if (o.res_ledger) {
    double* l = o.res_ledger + (int64_t)c * KS_LEDGER_COLS;
    l[KS_LEDGER_INFLOW] = a.in; l[KS_LEDGER_OUTFLOW] = a.out; l[KS_LEDGER_DISSIPATION] = a.diss;
    l[KS_LEDGER_STORAGE_RATE] = a.store; l[KS_LEDGER_MODEL_SUPPLIED] = a.sup; l[KS_LEDGER_RESIDUAL] = res;
    l[KS_LEDGER_SCALE] = a.scale; l[KS_LEDGER_ROUNDOFF] = ro;
  }
  // RelativeResidual, output/result.go:100-109
  double rr = 0;
  if (a.scale != 0 && fabs(res) > fmax(kLedgerAbsFloor, ro)) rr = fabs(res) / a.scale;
  return (o.energy_check && rr > o.ledger_tol) ? KS_STATUS_LEDGER : KS_STATUS_OK;
}

// recorder.record, analysis/tran.go:291-347, for the point at time tp of circuit c,
// before its Accept.  `slot` is the index record() stores the point at (elem and
// ledger rows laid out like the waveform: fixed-step [points][B], adaptive [B][cap];
// < 0: not stored).  Returns true when the point is out of balance by more than
// kGrossTol of the run's peak power (the transient stops there).
template <class SY, class P>
__device__ inline bool tran_point_results(Thr<SY, P>& t, TranLedger& L, const LoadParams& lp, int64_t c, int64_t B,
                                          double tp, bool imposed, bool stored_point, int64_t row) {
  const KOpts& o = t.o;
  const int ne = t.prog.ne;
  LedgerAcc a;
  a.zero();
  double stored = 0;
  // ports (element order), then the model suppliers, then the energy-storing elements
  int k = 0;
  t.prog.each([&](const KElem& e) {
    ElemOp r = elem_operating(e, t.V, t.D, state_col(t.Sb, e), t.s, o.gmin, false);
    a.port(r.thermal, r.ext);
    if (stored_point && row >= 0 && o.res_elem) {
      double* q = o.res_elem + (row * ne + k) * 2;
      q[0] = r.i; q[1] = r.p;
    }
    k++;
  });
  t.prog.each([&](const KElem& e) {  // the model suppliers: negative resistances, controlled sources
    if (e.kind != KS_ELEM_R && !(e.kind >= KS_ELEM_E && e.kind <= KS_ELEM_H)) return;
    ElemOp r = elem_operating(e, t.V, t.D, state_col(t.Sb, e), t.s, o.gmin, false);
    a.supplied(r.sup);
  });
  t.prog.each([&](const KElem& e) {  // the energy-storing elements
    if (!(e.kind == KS_ELEM_C || e.kind == KS_ELEM_L || e.kind == KS_ELEM_D || e.kind == KS_ELEM_Q ||
          e.kind == KS_ELEM_M || e.kind == KS_ELEM_K || e.kind == KS_ELEM_CN || e.kind == KS_ELEM_LN))
      return;
    ElemOp r = elem_operating(e, t.V, t.D, state_col(t.Sb, e), t.s, o.gmin, true);
    a.storage(r.ps);
    stored += r.w;
  });
  bool gross = false;
  if (a.scale > L.peakScale) L.peakScale = a.scale;
  const double res = fabs(a.residual());
  if (!imposed && res > kLedgerAbsFloor && res > roundoff_at(t, lp, c, B)) {
    if (res > L.worstAbs) L.worstAbs = res;
    if (res / L.peakScale > kGrossTol && o.energy_check) gross = true;
  }
  if (stored_point) {
    const double y[4] = {a.in, a.out, a.diss, a.sup};
    if (L.recorded == 0) { L.imposedFirst = imposed; L.storedStart = stored; }
    else
      for (int q = 0; q < 4; q++)
        L.e[q] += (L.recorded == 1 && L.imposedFirst) ? y[q] * (tp - L.tPrev) : 0.5 * (y[q] + L.yPrev[q]) * (tp - L.tPrev);
    for (int q = 0; q < 4; q++) L.yPrev[q] = y[q];
    L.tPrev = tp; L.storedEnd = stored;
    L.recorded++;
    if (row >= 0 && o.res_ledger) {
      double* l = o.res_ledger + row * KS_TPOINT_COLS;
      l[KS_TPOINT_INFLOW] = a.in; l[KS_TPOINT_OUTFLOW] = a.out; l[KS_TPOINT_DISSIPATION] = a.diss;
      l[KS_TPOINT_STORAGE_RATE] = a.store; l[KS_TPOINT_MODEL_SUPPLIED] = a.sup; l[KS_TPOINT_RESIDUAL] = a.residual();
      l[KS_TPOINT_STORED_ENERGY] = stored;
    }
  }
  return gross;
}

// recorder.finish, analysis/tran.go:350-386: the summary row of circuit c; returns
// true when the largest residual relative to the run's peak power exceeds the
// tolerance.
template <class SY, class P>
__device__ inline bool tran_finish(Thr<SY, P>& t, const TranLedger& L, int64_t c) {
  const KOpts& o = t.o;
  const double mrr = L.peakScale > 0 ? L.worstAbs / L.peakScale : 0.0;
  if (o.res_summary) {
    double* s = o.res_summary + c * KS_TSUM_COLS;
    s[KS_TSUM_MAX_RELATIVE_RESIDUAL] = mrr;
    s[KS_TSUM_ENERGY_IN] = L.e[0]; s[KS_TSUM_ENERGY_OUT] = L.e[1];
    s[KS_TSUM_ENERGY_DISSIPATED] = L.e[2]; s[KS_TSUM_ENERGY_MODEL_SUPPLIED] = L.e[3];
    s[KS_TSUM_STORED_START] = L.storedStart; s[KS_TSUM_STORED_END] = L.storedEnd;
    s[KS_TSUM_INTEGRATION_MISMATCH] = L.e[0] + L.e[3] - L.e[1] - L.e[2] - (L.storedEnd - L.storedStart);
  }
  return o.energy_check && mrr > o.ledger_tol;
}

}  // namespace ksg
