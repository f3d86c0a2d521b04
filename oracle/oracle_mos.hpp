// oracle_mos.hpp — CPU FP64 MOSFET levels 1-3 of the oracle (test infrastructure).
// Restates device/mosfet.go, device/mosfet_levels.go, device/mosfet_level23.go and the
// forward-mode dual numbers of device/dual.go.
#pragma once
#include "oracle_devices.hpp"

namespace kso {

// Dual number with three partials (vgs, vds, vbs), device/dual.go:17-106.
struct Dual {
  double v = 0, d[3] = {0, 0, 0};
  static Dual cst(double x) { Dual r; r.v = x; return r; }
  static Dual var(double x, int k) { Dual r; r.v = x; r.d[k] = 1; return r; }
  Dual add(const Dual& b) const { Dual r; r.v = v + b.v; for (int i = 0; i < 3; i++) r.d[i] = d[i] + b.d[i]; return r; }
  Dual sub(const Dual& b) const { Dual r; r.v = v - b.v; for (int i = 0; i < 3; i++) r.d[i] = d[i] - b.d[i]; return r; }
  Dual addc(double c) const { Dual r = *this; r.v += c; return r; }
  Dual neg() const { Dual r; r.v = -v; for (int i = 0; i < 3; i++) r.d[i] = -d[i]; return r; }
  Dual scale(double c) const { Dual r; r.v = v * c; for (int i = 0; i < 3; i++) r.d[i] = d[i] * c; return r; }
  Dual mul(const Dual& b) const { Dual r; r.v = v * b.v; for (int i = 0; i < 3; i++) r.d[i] = d[i] * b.v + v * b.d[i]; return r; }
  Dual div(const Dual& b) const {
    Dual r; double q = v / b.v; r.v = q;
    for (int i = 0; i < 3; i++) r.d[i] = (d[i] - q * b.d[i]) / b.v;
    return r;
  }
  Dual chain(double f, double df) const { Dual r; r.v = f; for (int i = 0; i < 3; i++) r.d[i] = df * d[i]; return r; }
  Dual sqrt() const { double s = std::sqrt(v); return chain(s, 0.5 / s); }
  Dual exp() const { double e = std::exp(v); return chain(e, e); }
  Dual log() const { return chain(std::log(v), 1 / v); }
  Dual cos() const { return chain(std::cos(v), -std::sin(v)); }
  Dual atan() const { return chain(std::atan(v), 1 / (1 + v * v)); }
  Dual abs() const { return v < 0 ? neg() : *this; }
  Dual powc(double c) const { double p = std::pow(v, c); return chain(p, c * p / v); }
};
static inline Dual dmax(const Dual& a, const Dual& b) { return b.v > a.v ? b : a; }
static inline Dual dmin(const Dual& a, const Dual& b) { return b.v < a.v ? b : a; }

constexpr double kEpsOx = 3.9 * 8.854214871e-12;   // device/mosfet.go:117
constexpr double kEpsSi = 11.7 * 8.854214871e-12;  // device/mosfet.go:118
constexpr double kNiSi = 1.45e16;                  // device/mosfet.go:119

static inline bool mgiven(uint64_t g, int k) { return (g >> k) & 1; }

// fetlim, device/mosfet.go:347-385.
static double fetlim(double vnew, double vold, double vto) {
  double vtsthi = std::fabs(2 * (vold - vto)) + 2;
  double vtstlo = vtsthi / 2 + 2;
  double vtox = vto + 3.5;
  double delv = vnew - vold;
  if (vold >= vto) {
    if (vold >= vtox) {
      if (delv <= 0) {
        if (vnew >= vtox) { if (-delv > vtstlo) vnew = vold - vtstlo; }
        else vnew = std::max(vnew, vto + 2);
      } else if (delv >= vtsthi) vnew = vold + vtsthi;
    } else if (delv <= 0) vnew = std::max(vnew, vto - 0.5);
    else vnew = std::min(vnew, vto + 4);
  } else if (delv <= 0) {
    if (-delv > vtsthi) vnew = vold - vtsthi;
  } else {
    double vtemp = vto + 0.5;
    if (vnew <= vtemp) { if (delv > vtstlo) vnew = vold + vtstlo; }
    else vnew = vtemp;
  }
  return vnew;
}

// limvds, device/mosfet.go:388-402.
static double limvds(double vnew, double vold) {
  if (vold >= 3.5) {
    if (vnew > vold) return std::min(vnew, 3 * vold + 2);
    if (vnew < 3.5) return std::max(vnew, 2.0);
    return vnew;
  }
  if (vnew > vold) return std::min(vnew, 4.0);
  return std::max(vnew, -0.5);
}

// meyer, device/mosfet.go:419-438.
static void meyer(double vgs, double vgd, double von, double vdsat, double phi, double cox, double* cgs, double* cgd, double* cgb) {
  double vgst = vgs - von;
  vdsat = std::max(vdsat, 0.0);
  if (vgst <= -phi) { *cgs = 0; *cgd = 0; *cgb = cox; return; }
  if (vgst <= -phi / 2) { *cgs = 0; *cgd = 0; *cgb = -vgst * cox / phi; return; }
  if (vgst <= 0) { *cgs = 2 * (vgst * cox / (1.5 * phi) + cox / 3); *cgd = 0; *cgb = -vgst * cox / phi; return; }
  double vds = vgs - vgd;
  if (vdsat <= vds) { *cgs = 2 * cox / 3; *cgd = 0; *cgb = 0; return; }
  double vddif = 2 * vdsat - vds, vddif1 = vdsat - vds, vddif2 = vddif * vddif;
  *cgs = 2 * cox * (1 - vddif1 * vddif1 / vddif2) / 3;
  *cgd = 2 * cox * (1 - vdsat * vdsat / vddif2) / 3;
  *cgb = 0;
}

struct MOSFET : Device {
  int level; double typ;
  double p[KS_M_NP]; uint64_t given;
  double vt, leff, weff, beta, cox = 0, oxideCap, vbi, vto, gdpr = 0, gspr = 0, isd, iss, vcritD, vcritS;
  double czbd, czbdsw, czbs, czbssw, fbt[3], fsw[3], cgso, cgdo, cgbo;
  bool hasJcap, hasGcap;
  // level constants, device/mosfet_levels.go:12-21
  double lxd = 0, lalpha = 0, lcfs = 0, lfactor = 0, lnarrow = 0, leta3 = 0, lsqrtPB = 0; bool lhasNSUB = false;
  int nd, ns_, ng, nb;
  int ud, us, g, b, dp, sp;
  double vgs = 0, vds = 0, vbs = 0, vbd = 0, vgd = 0, vgb = 0;
  double mode = 1, cdrain = 0, gm = 0, gds = 0, gmbs = 0, von = 0, vdsat = 0;
  double cbs = 0, gbs = 0, cbd = 0, gbd = 0;
  bool lim = false, tran = false;
  double ag = 0, gmin = 1e-12;
  double capG[3] = {0, 0, 0}, capB[2] = {0, 0}, iq[5] = {0, 0, 0, 0, 0}, dv[5] = {0, 0, 0, 0, 0};
  struct { double vgs = 0, vds = 0, vbs = 0, vgd = 0, vgb = 0, vbd = 0, von = 0; } acc;
  double meyerAcc[3] = {0, 0, 0}, qPrev[5] = {0, 0, 0, 0, 0}, iqPrev[5] = {0, 0, 0, 0, 0}, vPrev[5] = {0, 0, 0, 0, 0};
  History hist[5];
  bool bad = false;  // derive failed (ErrUnsupported)

  MOSFET(const double* pp, uint64_t giv, int lev, bool pmos, int d_, int s_, int g_, int b_) {
    for (int i = 0; i < KS_M_NP; i++) p[i] = pp[i];
    given = giv; level = lev; typ = pmos ? -1 : 1;
    nd = d_; ns_ = s_; ng = g_; nb = b_;
    bad = !derive();
  }
  bool derive() {  // device/mosfet.go:218-323
    vt = kBoltzmann * kTNom / kChargeQ;
    leff = p[KS_M_P_L] - 2 * p[KS_M_P_LD];
    weff = p[KS_M_P_W];
    if (level == 3) weff = p[KS_M_P_W] - 2 * p[KS_M_P_WD];
    if (!(leff > 0) || !(weff > 0)) return false;
    bool toxGiven = mgiven(given, KS_M_P_TOX) || level >= 2;
    if (toxGiven && p[KS_M_P_TOX] > 0) {
      cox = kEpsOx / p[KS_M_P_TOX];
      if (!mgiven(given, KS_M_P_KP)) p[KS_M_P_KP] = p[KS_M_P_UO] * cox * 1e-4;
      if (mgiven(given, KS_M_P_NSUB)) {
        double nsub = p[KS_M_P_NSUB] * 1e6;
        double ni = kNiSi;
        if (level == 3) {
          double eg = 1.16 - 7.02e-4 * kTNom * kTNom / (kTNom + 1108);
          double r = kTNom / 300;
          ni *= r * std::sqrt(r) * std::exp(0.5 * eg * (1.0 / 300 - 1 / kTNom) / (kBoltzmann / kChargeQ));
        }
        if (!(nsub > ni)) return false;
        if (!mgiven(given, KS_M_P_PHI)) p[KS_M_P_PHI] = std::max(0.1, 2 * vt * std::log(nsub / ni));
        if (!mgiven(given, KS_M_P_GAMMA)) p[KS_M_P_GAMMA] = std::sqrt(2 * kEpsSi * kChargeQ * nsub) / cox;
        if (!mgiven(given, KS_M_P_VTO)) {
          double eg = 1.16 - 7.02e-4 * kTNom * kTNom / (kTNom + 1108);
          double fermis = typ * 0.5 * p[KS_M_P_PHI];
          double wkfng = 3.2;
          if (p[KS_M_P_TPG] != 0) {
            double fermig = typ * p[KS_M_P_TPG] * 0.5 * eg;
            wkfng = 3.25 + 0.5 * eg - fermig;
          }
          double wkfngs = wkfng - (3.25 + 0.5 * eg + fermis);
          double vfb = wkfngs - p[KS_M_P_NSS] * 1e4 * kChargeQ / cox;
          p[KS_M_P_VTO] = vfb + typ * (p[KS_M_P_GAMMA] * std::sqrt(p[KS_M_P_PHI]) + p[KS_M_P_PHI]);
        }
        if (!mgiven(given, KS_M_P_CJ)) p[KS_M_P_CJ] = std::sqrt(kEpsSi * kChargeQ * nsub / (2 * p[KS_M_P_PB]));
      }
    }
    double M = p[KS_M_P_MULT];
    oxideCap = cox * leff * weff * M;
    beta = p[KS_M_P_KP] * weff / leff * M;
    vto = typ * p[KS_M_P_VTO];
    vbi = vto - p[KS_M_P_GAMMA] * std::sqrt(p[KS_M_P_PHI]);
    double rd = p[KS_M_P_RD], rs = p[KS_M_P_RS];
    if (!mgiven(given, KS_M_P_RD) && p[KS_M_P_RSH] > 0) rd = p[KS_M_P_RSH] * p[KS_M_P_NRD];
    if (!mgiven(given, KS_M_P_RS) && p[KS_M_P_RSH] > 0) rs = p[KS_M_P_RSH] * p[KS_M_P_NRS];
    if (rd > 0) gdpr = M / rd;
    if (rs > 0) gspr = M / rs;
    isd = iss = p[KS_M_P_IS] * M;
    if (p[KS_M_P_JS] > 0 && p[KS_M_P_AD] > 0 && p[KS_M_P_AS] > 0) {
      isd = p[KS_M_P_JS] * p[KS_M_P_AD] * M; iss = p[KS_M_P_JS] * p[KS_M_P_AS] * M;
    }
    vcritD = vt * std::log(vt / (kSqrt2 * std::max(isd, 1e-300)));
    vcritS = vt * std::log(vt / (kSqrt2 * std::max(iss, 1e-300)));
    czbd = mgiven(given, KS_M_P_CBD) ? p[KS_M_P_CBD] * M : p[KS_M_P_CJ] * p[KS_M_P_AD] * M;
    czbs = mgiven(given, KS_M_P_CBS) ? p[KS_M_P_CBS] * M : p[KS_M_P_CJ] * p[KS_M_P_AS] * M;
    czbdsw = p[KS_M_P_CJSW] * p[KS_M_P_PD] * M;
    czbssw = p[KS_M_P_CJSW] * p[KS_M_P_PS] * M;
    deplF(p[KS_M_P_PB], p[KS_M_P_MJ], p[KS_M_P_FC], &fbt[0], &fbt[1], &fbt[2]);
    deplF(p[KS_M_P_PB], p[KS_M_P_MJSW], p[KS_M_P_FC], &fsw[0], &fsw[1], &fsw[2]);
    cgso = p[KS_M_P_CGSO] * weff * M; cgdo = p[KS_M_P_CGDO] * weff * M; cgbo = p[KS_M_P_CGBO] * leff * M;
    hasJcap = czbd + czbdsw + czbs + czbssw > 0;
    hasGcap = oxideCap > 0 || cgso + cgdo + cgbo > 0;
    // deriveLevel, device/mosfet_levels.go:25-51
    if (mgiven(given, KS_M_P_NSUB)) {
      lhasNSUB = true;
      lalpha = 2 * kEpsSi / (kChargeQ * p[KS_M_P_NSUB] * 1e6);
      lxd = std::sqrt(lalpha);
    }
    if (level == 2) {
      lcfs = kChargeQ * p[KS_M_P_NFS] * 1e4 / cox;
      lfactor = p[KS_M_P_DELTA] * kPi * kEpsSi / (4 * cox * weff);
      lsqrtPB = std::sqrt(p[KS_M_P_PB]);
      if (p[KS_M_P_VMAX] > 0 && !(p[KS_M_P_NEFF] > 0)) return false;
    } else if (level == 3) {
      lcfs = kChargeQ * p[KS_M_P_NFS] * 1e4 / cox;
      lnarrow = p[KS_M_P_DELTA] * 0.5 * kPi * kEpsSi / cox;
      leta3 = p[KS_M_P_ETA] * 8.15e-22 / (cox * leff * leff * leff);
    } else if (level != 1) return false;
    acc.von = vto;
    return true;
  }
  void setup(SetupCtx& c) override {  // :326-337
    ud = c.unknown(nd); us = c.unknown(ns_);
    g = c.unknown(ng); b = c.unknown(nb);
    dp = ud; sp = us;
    if (gdpr > 0) dp = c.allocUnknown();
    if (gspr > 0) sp = c.allocUnknown();
  }
  bool nonlinear() const override { return true; }
  bool reactive() const override { return true; }
  bool limited() const override { return lim; }
  void voltages(const double* x, double* vgs_, double* vds_, double* vbs_, double* vgb_) const {  // :340-344
    double vg = at(x, n, g), vb = at(x, n, b), vdp = at(x, n, dp), vsp = at(x, n, sp);
    *vgs_ = typ * (vg - vsp); *vds_ = typ * (vdp - vsp); *vbs_ = typ * (vb - vsp); *vgb_ = typ * (vg - vb);
  }
  void bulkDiode(double v, double is, double* i, double* gg) const {  // :408-414
    if (v <= -3 * vt) { *i = gmin * v - is; *gg = gmin; return; }
    double e = std::exp(std::min(v / vt, 700.0));
    *i = is * (e - 1) + gmin * v; *gg = is * e / vt + gmin;
  }
  void meyerCaps(double vgs_, double vgd_, double von_, double vdsat_, double md, double out[3]) const {  // :441-451
    if (oxideCap == 0) { out[0] = out[1] = out[2] = 0; return; }
    double a, bb, c;
    if (md > 0) { meyer(vgs_, vgd_, von_, vdsat_, p[KS_M_P_PHI], oxideCap, &a, &bb, &c); out[0] = a; out[1] = bb; out[2] = c; }
    else { meyer(vgd_, vgs_, von_, vdsat_, p[KS_M_P_PHI], oxideCap, &a, &bb, &c); out[0] = bb; out[1] = a; out[2] = c; }
  }
  void bulkCharge(double v, double cz, double czsw, double* q, double* c) const {  // :455-460
    double q1, c1, q2, c2;
    depletion(v, cz, p[KS_M_P_PB], p[KS_M_P_MJ], p[KS_M_P_FC], fbt[0], fbt[1], fbt[2], &q1, &c1);
    depletion(v, czsw, p[KS_M_P_PB], p[KS_M_P_MJSW], p[KS_M_P_FC], fsw[0], fsw[1], fsw[2], &q2, &c2);
    *q = q1 + q2; *c = c1 + c2;
  }
  // idsLevel1, device/mosfet_levels.go:79-113
  void idsLevel1(double vg, double vd, double vb, double* cd, double* gm_, double* gds_, double* gmbs_, double* von_, double* vdsat_) const {
    double PHI = p[KS_M_P_PHI], GAMMA = p[KS_M_P_GAMMA], LAMBDA = p[KS_M_P_LAMBDA];
    double sarg;
    if (vb <= 0) sarg = std::sqrt(PHI - vb);
    else { sarg = std::sqrt(PHI); sarg = std::max(0.0, sarg - vb / (sarg + sarg)); }
    double vn = vbi + GAMMA * sarg;
    double vgst = vg - vn;
    double vs = std::max(vgst, 0.0);
    double arg = 0;
    if (sarg > 0) arg = GAMMA / (sarg + sarg);
    *von_ = vn; *vdsat_ = vs;
    if (vgst <= 0) { *cd = 0; *gm_ = 0; *gds_ = 0; *gmbs_ = 0; return; }
    double betap = beta * (1 + LAMBDA * vd);
    double c, m, ds;
    if (vgst <= vd) {
      c = betap * vgst * vgst * 0.5; m = betap * vgst; ds = LAMBDA * beta * vgst * vgst * 0.5;
    } else {
      c = betap * vd * (vgst - 0.5 * vd); m = betap * vd;
      ds = betap * (vgst - vd) + LAMBDA * beta * vd * (vgst - 0.5 * vd);
    }
    *cd = c; *gm_ = m; *gds_ = ds; *gmbs_ = m * arg;
  }
  // level2VelocitySat, device/mosfet_level23.go:202-257
  static bool level2VelocitySat(const Dual& gammad, const Dual& v1, const Dual& v2, const Dual& invxv, const Dual& sarg3, Dual* xout) {
    Dual xv = Dual::cst(1).div(invxv);
    Dual a1 = gammad.scale(1 / 0.75);
    Dual b1 = v1.add(xv).scale(-2);
    Dual c1 = gammad.mul(xv).scale(-2);
    Dual d1 = v1.mul(v2.add(xv)).scale(2).sub(v2.mul(v2)).sub(gammad.mul(sarg3).scale(4.0 / 3.0));
    Dual a = b1.neg();
    Dual bq = a1.mul(c1).sub(d1.scale(4));
    Dual c = d1.neg().mul(a1.mul(a1).sub(b1.scale(4))).sub(c1.mul(c1));
    Dual r = a.mul(a).scale(-1.0 / 3).add(bq);
    Dual s = a.mul(a).mul(a).scale(2.0 / 27).sub(a.mul(bq).scale(1.0 / 3)).add(c);
    Dual r3 = r.mul(r).mul(r);
    Dual s2 = s.mul(s);
    Dual pp = s2.scale(0.25).add(r3.scale(1.0 / 27));
    Dual p0 = pp.abs();
    Dual p2 = p0.sqrt();
    Dual y3;
    auto cbrtAbs = [](Dual z) { z = z.abs(); if (z.v == 0) return Dual(); return z.powc(1.0 / 3); };
    if (pp.v < 0) {
      Dual ro = s2.scale(0.25).add(p0).sqrt().log().scale(1.0 / 3).exp();
      Dual fi = p2.scale(-2).div(s).atan();
      y3 = ro.mul(fi.scale(1.0 / 3).cos()).scale(2).sub(a.scale(1.0 / 3));
    } else {
      y3 = cbrtAbs(s.scale(-0.5).add(p2)).add(cbrtAbs(s.scale(-0.5).sub(p2))).sub(a.scale(1.0 / 3));
    }
    Dual ra = a1.mul(a1).scale(0.25).sub(b1).add(y3);
    Dual rb = y3.mul(y3).scale(0.25).sub(d1);
    if (!(ra.v >= 0) || !(rb.v >= 0)) return false;
    Dual a3 = ra.sqrt(), b3 = rb.sqrt();
    const double sig1[4] = {1, -1, 1, -1}, sig2[4] = {1, 1, -1, -1};
    bool ok = false;
    Dual x;
    for (int i = 0; i < 4; i++) {
      Dual a4 = a1.scale(0.5).add(a3.scale(sig1[i]));
      Dual b4 = y3.scale(0.5).add(b3.scale(sig2[i]));
      Dual delta4 = a4.mul(a4).scale(0.25).sub(b4);
      if (!(delta4.v >= 0)) continue;
      Dual t = delta4.sqrt();
      Dual roots[2] = {a4.scale(-0.5).add(t), a4.scale(-0.5).sub(t)};
      for (const Dual& rr : roots) {
        if (!(rr.v > 0)) continue;
        double x2 = rr.v * rr.v;
        double poly = x2 * x2 + a1.v * x2 * rr.v + b1.v * x2 + c1.v * rr.v + d1.v;
        if (!(std::fabs(poly) <= 1e-6)) continue;
        if (!ok || rr.v < x.v) { x = rr; ok = true; }
      }
    }
    *xout = x;
    return ok;
  }
  // idsLevel2, device/mosfet_level23.go:31-194
  void idsLevel2(double vgsV, double vdsV, double vbsV, double* o) const {
    Dual G = Dual::var(vgsV, 0), D = Dual::var(vdsV, 1), B = Dual::var(vbsV, 2);
    double phi = p[KS_M_P_PHI], GAMMA = p[KS_M_P_GAMMA], XJ = p[KS_M_P_XJ], UCRIT = p[KS_M_P_UCRIT];
    double UEXP = p[KS_M_P_UEXP], UO = p[KS_M_P_UO], VMAX = p[KS_M_P_VMAX], LAMBDA = p[KS_M_P_LAMBDA];
    double NEFF = p[KS_M_P_NEFF], NFS = p[KS_M_P_NFS];
    double sphi = std::sqrt(phi), sphi3 = phi * sphi;
    Dual phiMinVbs = B.neg().addc(phi);
    Dual sarg, dsrgdb, barg, dbrgdb;
    if (B.v <= 0) { sarg = phiMinVbs.sqrt(); dsrgdb = Dual::cst(-0.5).div(sarg); }
    else { sarg = Dual::cst(sphi).div(B.scale(0.5 / phi).addc(1)); dsrgdb = sarg.mul(sarg).scale(-0.5 / sphi3); }
    if (B.v - D.v <= 0) { barg = phiMinVbs.add(D).sqrt(); dbrgdb = Dual::cst(-0.5).div(barg); }
    else { barg = Dual::cst(sphi).div(B.sub(D).scale(0.5 / phi).addc(1)); dbrgdb = barg.mul(barg).scale(-0.5 / sphi3); }
    double factor = lfactor, eta = 1 + factor;
    Dual vbin = phiMinVbs.scale(factor).addc(vbi);
    Dual gamasd = Dual::cst(GAMMA), dgddvb = Dual::cst(0);
    if (GAMMA > 0 || lhasNSUB) {
      if (XJ > 0) {
        Dual xws = sarg.scale(lxd), xwd = barg.scale(lxd);
        Dual args = xws.scale(2 / XJ).addc(1).sqrt();
        Dual argd = xwd.scale(2 / XJ).addc(1).sqrt();
        double t = 0.5 * XJ / leff;
        Dual argss = args.addc(-1).scale(t), argsd = argd.addc(-1).scale(t);
        gamasd = argss.add(argsd).neg().addc(1).scale(GAMMA);
        Dual dbargs = dsrgdb.scale(lxd).div(args).scale(0.5 / leff);
        Dual dbargd = dbrgdb.scale(lxd).div(argd).scale(0.5 / leff);
        dgddvb = dbargs.add(dbargd).scale(-GAMMA);
      }
    }
    Dual vonD = vbin.add(gamasd.mul(sarg));
    bool nfs = NFS != 0;
    Dual xn, argg;
    if (nfs) {
      Dual cdonco = gamasd.mul(dsrgdb).add(dgddvb.mul(sarg)).neg().addc(factor);
      xn = cdonco.addc(1 + lcfs);
      Dual vtxn = xn.scale(vt);
      vonD = vonD.add(vtxn);
      argg = Dual::cst(1).div(vtxn);
    } else if (G.v <= vbin.v) {
      o[0] = 0; o[1] = 0; o[2] = 0; o[3] = 0; o[4] = vonD.v; o[5] = 0; return;
    }
    Dual vgst = G.sub(vonD);
    Dual ufact = Dual::cst(1);
    double crit = UCRIT * 100 * kEpsSi / cox;
    if (vgst.v > crit) ufact = Dual::cst(crit).div(vgst).powc(UEXP);
    Dual ueff = ufact.scale(UO * 1e-4);
    Dual vgsx = G;
    if (nfs) vgsx = dmax(G, vonD);
    Dual gammad = gamasd.scale(1 / eta);
    Dual vgb_ = vgsx.sub(vbin).scale(1 / eta);
    Dual vdsatD = Dual::cst(0);
    if (gammad.v > 0) {
      Dual argv = vgb_.add(phiMinVbs);
      if (argv.v > 0) {
        Dual gammd2 = gammad.mul(gammad);
        Dual arg1 = argv.scale(4).div(gammd2).addc(1).sqrt();
        vdsatD = dmax(vgb_.add(gammd2.mul(arg1.neg().addc(1)).scale(0.5)), Dual::cst(0));
      }
    } else vdsatD = dmax(vgb_, Dual::cst(0));
    Dual sarg3 = sarg.mul(sarg).mul(sarg);
    if (VMAX > 0) {
      Dual x;
      if (level2VelocitySat(gammad, vgb_.add(phiMinVbs), phiMinVbs, ueff.scale(1 / (VMAX * leff)), sarg3, &x))
        vdsatD = x.mul(x).sub(phiMinVbs);
    }
    Dual xlamda = Dual::cst(LAMBDA);
    Dual bsarg, bodys;
    if (D.v != 0) {
      if (B.v - vdsatD.v <= 0) bsarg = vdsatD.add(phiMinVbs).sqrt();
      else bsarg = Dual::cst(sphi).div(B.sub(vdsatD).scale(0.5 / phi).addc(1));
      bodys = bsarg.mul(bsarg).mul(bsarg).sub(sarg3);
      if (lhasNSUB && !(LAMBDA > 0)) {
        if (VMAX <= 0) {
          Dual argv = D.sub(vdsatD).scale(0.25);
          Dual sargv = argv.mul(argv).addc(1).sqrt();
          xlamda = argv.add(sargv).sqrt().mul(Dual::cst(lxd).div(D.scale(leff)));
        } else {
          double xdv = lxd / std::sqrt(NEFF);
          Dual xlv = Dual::cst(VMAX * xdv * 0.5).div(ueff);
          Dual argv = dmax(D.sub(vdsatD), Dual::cst(0));
          Dual xls = xlv.mul(xlv).add(argv).sqrt();
          xlamda = xls.sub(xlv).mul(Dual::cst(xdv).div(D.scale(leff)));
        }
      }
    }
    double xwb = lxd * lsqrtPB;
    double xld = leff - xwb;
    Dual clfact = xlamda.mul(D).neg().addc(1);
    if (!lhasNSUB) xwb = 0.25e-6;
    Dual xleff = clfact.scale(leff);
    if (xleff.v < xwb) {
      Dual deltal = xlamda.mul(D).scale(leff);
      xleff = Dual::cst(xwb).div(deltal.addc(-xld).scale(1 / xwb).addc(1));
      clfact = xleff.scale(1 / leff);
    }
    Dual beta1 = ufact.scale(beta).div(clfact);
    if (D.v <= 1e-10) {
      Dual gg;
      if (G.v > vonD.v) gg = beta1.mul(G.sub(vbin).sub(gamasd.mul(sarg)));
      else if (nfs) gg = beta1.mul(vonD.sub(vbin).sub(gamasd.mul(sarg))).mul(argg.mul(G.sub(vonD)).exp());
      o[0] = 0; o[1] = 0; o[2] = gg.v; o[3] = 0; o[4] = vonD.v; o[5] = vdsatD.v; return;
    }
    Dual id;
    if (nfs && G.v <= vonD.v) {
      if (vdsatD.v <= 0) { o[0] = 0; o[1] = 0; o[2] = 0; o[3] = 0; o[4] = vonD.v; o[5] = vdsatD.v; return; }
      Dual vdson = dmin(vdsatD, D);
      Dual body = barg.mul(barg).mul(barg).sub(sarg3);
      if (D.v > vdsatD.v) body = bodys;
      Dual cdson = beta1.mul(vonD.sub(vbin).sub(vdson.scale(0.5 * eta)).mul(vdson).sub(gamasd.mul(body).scale(1 / 1.5)));
      id = cdson.mul(argg.mul(G.sub(vonD)).exp());
    } else if (D.v <= vdsatD.v) {
      Dual body = barg.mul(barg).mul(barg).sub(sarg3);
      id = beta1.mul(G.sub(vbin).sub(D.scale(0.5 * eta)).mul(D).sub(gamasd.mul(body).scale(1 / 1.5)));
    } else {
      id = beta1.mul(G.sub(vbin).sub(vdsatD.scale(0.5 * eta)).mul(vdsatD).sub(gamasd.mul(bodys).scale(1 / 1.5)));
    }
    o[0] = id.v; o[1] = id.d[0]; o[2] = id.d[1]; o[3] = id.d[2]; o[4] = vonD.v; o[5] = vdsatD.v;
  }
  // idsLevel3, device/mosfet_level23.go:277-378
  void idsLevel3(double vgsV, double vdsV, double vbsV, double* o) const {
    const double coeff0 = 0.0631353, coeff1 = 0.8013292, coeff2 = -0.01110777;
    Dual G = Dual::var(vgsV, 0), D = Dual::var(vdsV, 1), B = Dual::var(vbsV, 2);
    double phi = p[KS_M_P_PHI], XJ = p[KS_M_P_XJ], LD = p[KS_M_P_LD], GAMMA = p[KS_M_P_GAMMA];
    double THETA = p[KS_M_P_THETA], UO = p[KS_M_P_UO], VMAX = p[KS_M_P_VMAX], KAPPA = p[KS_M_P_KAPPA];
    double NFS = p[KS_M_P_NFS];
    Dual phibs, sqphbs;
    if (B.v <= 0) { phibs = B.neg().addc(phi); sqphbs = phibs.sqrt(); }
    else { sqphbs = Dual::cst(std::sqrt(phi)).div(B.scale(1 / (2 * phi)).addc(1)); phibs = sqphbs.mul(sqphbs); }
    Dual fshort = Dual::cst(1);
    if (XJ != 0 && lxd != 0) {
      Dual wponxj = sqphbs.scale(lxd / XJ);
      Dual wconxj = wponxj.mul(wponxj).scale(coeff2).add(wponxj.scale(coeff1)).addc(coeff0);
      double djonxj = LD / XJ;
      Dual arga = wconxj.addc(djonxj);
      Dual argc = wponxj.div(wponxj.addc(1));
      Dual argb = argc.mul(argc).neg().addc(1).sqrt();
      fshort = arga.mul(argb).addc(-djonxj).scale(-XJ / leff).addc(1);
    }
    Dual gammas = fshort.scale(GAMMA);
    Dual fbodys = gammas.div(sqphbs).scale(0.25);
    Dual fbody = fbodys.addc(lnarrow / weff);
    Dual qbonco = gammas.mul(sqphbs).add(phibs.scale(lnarrow / weff));
    Dual vth = D.scale(-leta3).addc(vbi).add(qbonco);
    Dual vonD = vth;
    bool nfs = NFS != 0;
    Dual xn;
    if (nfs) {
      xn = qbonco.div(phibs.scale(2)).addc(1 + lcfs);
      vonD = vth.add(xn.scale(vt));
    } else if (G.v <= vonD.v) {
      o[0] = 0; o[1] = 0; o[2] = 0; o[3] = 0; o[4] = vonD.v; o[5] = 0; return;
    }
    Dual vgsx = dmax(G, vonD);
    Dual onfg = vgsx.sub(vth).scale(THETA).addc(1);
    Dual fgate = Dual::cst(1).div(onfg);
    Dual us_ = fgate.scale(UO * 1e-4);
    Dual onfbdy = Dual::cst(1).div(fbody.addc(1));
    Dual arga = vgsx.sub(vth).mul(onfbdy);
    Dual vdsatD = arga;
    Dual vdsc;
    if (VMAX > 0) {
      vdsc = Dual::cst(leff * VMAX).div(us_);
      Dual argb = arga.mul(arga).add(vdsc.mul(vdsc)).sqrt();
      vdsatD = arga.add(vdsc).sub(argb);
    }
    Dual vdsx = dmin(D, vdsatD);
    Dual bet = fgate.scale(beta);
    if (vdsx.v == 0) {
      Dual gg = bet.mul(vgsx.sub(vth));
      if (nfs && G.v < vonD.v) gg = gg.mul(G.sub(vonD).div(xn.scale(vt)).exp());
      o[0] = 0; o[1] = 0; o[2] = gg.v; o[3] = 0; o[4] = vonD.v; o[5] = vdsatD.v; return;
    }
    Dual cdo = vgsx.sub(vth).sub(fbody.addc(1).mul(vdsx).scale(0.5));
    Dual id = bet.mul(cdo).mul(vdsx);
    Dual fdrain;
    if (VMAX > 0) {
      fdrain = Dual::cst(1).div(vdsx.div(vdsc).addc(1));
      id = id.mul(fdrain);
    }
    bool clm = false;
    Dual delxl;
    if (D.v <= vdsatD.v) {
      if (VMAX <= 0 && lalpha != 0) {
        Dual r = D.div(vdsatD);
        Dual r2 = r.mul(r);
        delxl = vdsatD.scale(KAPPA * lalpha / 8).sqrt().mul(r2.mul(r2));
        clm = true;
      }
    } else if (VMAX <= 0) {
      delxl = D.sub(vdsatD).add(vdsatD.scale(1.0 / 8)).scale(KAPPA * lalpha).sqrt();
      clm = true;
    } else if (lalpha != 0) {
      Dual gdsat = dmax(id.mul(fdrain.neg().addc(1)).div(vdsc), Dual::cst(1e-12));
      Dual emax = id.div(gdsat).scale(KAPPA / leff);
      Dual a = emax.scale(0.5 * lalpha);
      Dual argb = a.mul(a).add(D.sub(vdsatD).scale(KAPPA * lalpha)).sqrt();
      delxl = argb.sub(a);
      clm = true;
    }
    if (clm) {
      if (delxl.v > 0.5 * leff) delxl = Dual::cst(-leff * leff / 4).div(delxl).addc(leff);
      id = id.div(delxl.scale(-1 / leff).addc(1));
    }
    if (nfs && G.v < vonD.v) id = id.mul(G.sub(vonD).div(xn.scale(vt)).exp());
    o[0] = id.v; o[1] = id.d[0]; o[2] = id.d[1]; o[3] = id.d[2]; o[4] = vonD.v; o[5] = vdsatD.v;
  }
  void ids(double vg, double vd, double vb, double* o) const {  // device/mosfet_levels.go:56-64
    if (level == 2) { idsLevel2(vg, vd, vb, o); return; }
    if (level == 3) { idsLevel3(vg, vd, vb, o); return; }
    idsLevel1(vg, vd, vb, &o[0], &o[1], &o[2], &o[3], &o[4], &o[5]);
  }
  // channel, device/mosfet.go:464-473: o = {mode, cdrain, gm, gds, gmbs, von, vdsat}
  void channel(double vgs_, double vds_, double vbs_, double* o) const {
    double md = 1, vg = vgs_, vd = vds_, vb = vbs_;
    if (vds_ < 0) { md = -1; vg = vgs_ - vds_; vd = -vds_; vb = vbs_ - vds_; }
    o[0] = md;
    ids(vg, vd, vb, o + 1);
  }
  void load(LoadCtx& c) override {  // :476-551
    gmin = c.gmin;
    double vgs_, vds_, vbs_, vgb_;
    voltages(c.X, &vgs_, &vds_, &vbs_, &vgb_);
    lim = false;
    if (c.initJct) { vbs_ = -1; vgs_ = vto; vds_ = 0; lim = true; }
    else {
      double vgd_ = vgs_ - vds_;
      double vgdOld = acc.vgs - acc.vds;
      double vn = acc.von;
      if (acc.vds >= 0) {
        vgs_ = fetlim(vgs_, acc.vgs, vn);
        vds_ = vgs_ - vgd_;
        vds_ = limvds(vds_, acc.vds);
        vgd_ = vgs_ - vds_;
      } else {
        vgd_ = fetlim(vgd_, vgdOld, vn);
        vds_ = vgs_ - vgd_;
        vds_ = -limvds(-vds_, -acc.vds);
        vgs_ = vgd_ + vds_;
      }
      bool l;
      if (vds_ >= 0) vbs_ = pnjlim(vbs_, acc.vbs, vt, vcritS, &l);
      else {
        double vbd_ = pnjlim(vbs_ - vds_, acc.vbs - acc.vds, vt, vcritD, &l);
        vbs_ = vbd_ + vds_;
      }
      lim = l;
    }
    double vbd_ = vbs_ - vds_, vgd_ = vgs_ - vds_;
    double vgb2 = vgs_ - vbs_;
    vgs = vgs_; vds = vds_; vbs = vbs_; vbd = vbd_; vgd = vgd_; vgb = vgb2;
    acc.vgs = vgs_; acc.vds = vds_; acc.vbs = vbs_;
    bulkDiode(vbs_, iss, &cbs, &gbs);
    bulkDiode(vbd_, isd, &cbd, &gbd);
    double o[7];
    channel(vgs_, vds_, vbs_, o);
    mode = o[0]; cdrain = o[1]; gm = o[2]; gds = o[3]; gmbs = o[4]; von = o[5]; vdsat = o[6];
    acc.von = von;
    tran = false; ag = 0;
    for (int k = 0; k < 5; k++) iq[k] = 0;
    dv[0] = vgs_; dv[1] = vgd_; dv[2] = vgb2; dv[3] = vbs_; dv[4] = vbd_;
    if (c.mode == ModeTran && (hasGcap || hasJcap)) {
      tran = true;
      ag = c.method == TRAP ? 2 / c.h : 1 / c.h;
      double mc[3];
      meyerCaps(vgs_, vgd_, von, vdsat, mode, mc);
      double ov[3] = {cgso, cgdo, cgbo};
      for (int k = 0; k < 3; k++) capG[k] = (mc[k] + meyerAcc[k]) / 2 + ov[k];
      double qbs, cbs2, qbd, cbd2;
      bulkCharge(vbs_, czbs, czbssw, &qbs, &cbs2);
      bulkCharge(vbd_, czbd, czbdsw, &qbd, &cbd2);
      capB[0] = cbs2; capB[1] = cbd2;
      double qs[5] = {qPrev[0] + capG[0] * (vgs_ - vPrev[0]), qPrev[1] + capG[1] * (vgd_ - vPrev[1]),
                      qPrev[2] + capG[2] * (vgb2 - vPrev[2]), qbs, qbd};
      for (int k = 0; k < 5; k++) {
        iq[k] = ag * (qs[k] - qPrev[k]);
        if (c.method == TRAP) iq[k] -= iqPrev[k];
      }
    }
    stamp(c);
  }
  double cap(int k) const { return k < 3 ? capG[k] : capB[k - 3]; }
  void branch(LoadCtx& c, int a, int bb, double i0, int nn, const double* gg, const int* pk, const int* mk, const double* v0) {  // :563-578
    double ieq = i0;
    for (int k = 0; k < nn; k++) {
      if (gg[k] == 0) continue;
      c.M->add(a, pk[k], gg[k]); c.M->add(a, mk[k], -gg[k]);
      c.M->add(bb, pk[k], -gg[k]); c.M->add(bb, mk[k], gg[k]);
      ieq -= gg[k] * v0[k];
    }
    ieq *= typ;
    c.addRHS(a, -ieq); c.addRHS(bb, ieq);
  }
  void channelBranch(double* i0, double gc[3]) const {  // :582-589
    if (mode > 0) { *i0 = cdrain; gc[0] = gm; gc[1] = gds; gc[2] = gmbs; return; }
    *i0 = -cdrain; gc[0] = -gm; gc[1] = gm + gds + gmbs; gc[2] = -gmbs;
  }
  void stamp(LoadCtx& c) {  // :591-611
    double i0, gc[3];
    channelBranch(&i0, gc);
    { int pk[3] = {g, dp, b}, mk[3] = {sp, sp, sp}; double v0[3] = {vgs, vds, vbs}; branch(c, dp, sp, i0, 3, gc, pk, mk, v0); }
    { int pk[1] = {b}, mk[1] = {sp}; double gg[1] = {gbs}, v0[1] = {vbs}; branch(c, b, sp, cbs, 1, gg, pk, mk, v0); }
    { int pk[1] = {b}, mk[1] = {dp}; double gg[1] = {gbd}, v0[1] = {vbd}; branch(c, b, dp, cbd, 1, gg, pk, mk, v0); }
    if (tran) {
      int ends[5][2] = {{g, sp}, {g, dp}, {g, b}, {b, sp}, {b, dp}};
      for (int k = 0; k < 5; k++) {
        double cc[1] = {ag * cap(k)};
        int pk[1] = {ends[k][0]}, mk[1] = {ends[k][1]};
        double v0[1] = {dv[k]};
        branch(c, ends[k][0], ends[k][1], iq[k], 1, cc, pk, mk, v0);
      }
    }
    if (dp != ud) { double gg = gdpr; c.M->add(ud, ud, gg); c.M->add(dp, dp, gg); c.M->add(ud, dp, -gg); c.M->add(dp, ud, -gg); }
    if (sp != us) { double gg = gspr; c.M->add(us, us, gg); c.M->add(sp, sp, gg); c.M->add(us, sp, -gg); c.M->add(sp, us, -gg); }
  }
  bool convTest(const double* x, double reltol, double abstol) override {  // :618-631
    double vgs_, vds_, vbs_, vgb_;
    voltages(x, &vgs_, &vds_, &vbs_, &vgb_);
    double vbd_ = vbs_ - vds_;
    double i0, gc[3];
    channelBranch(&i0, gc);
    double ich = i0 + gc[0] * (vgs_ - vgs) + gc[1] * (vds_ - vds) + gc[2] * (vbs_ - vbs);
    double ibs = cbs + gbs * (vbs_ - vbs);
    double ibd = cbd + gbd * (vbd_ - vbd);
    double o[7];
    channel(vgs_, vds_, vbs_, o);
    double ichN = o[0] * o[1];
    double ibsN, ibdN, t1;
    bulkDiode(vbs_, iss, &ibsN, &t1);
    bulkDiode(vbd_, isd, &ibdN, &t1);
    auto ok = [&](double a, double bb) { return std::fabs(a - bb) <= reltol * std::max(std::fabs(a), std::fabs(bb)) + abstol; };
    return ok(ich - ibd, ichN - ibdN) && ok(ibs + ibd, ibsN + ibdN);
  }
  // terminalCurrents, :635-657: currents into drain, gate, source and bulk from
  // the linearization of the last load, and the power into storage; v5 receives
  // {vgs, vgd, vgb, vbs, vbd}.
  void terminals(const double* x, double* id, double* ig, double* is, double* ib, double* ps, double v5[5]) const {
    double vgs_, vds_, vbs_, vgb_;
    voltages(x, &vgs_, &vds_, &vbs_, &vgb_);
    double vbd_ = vbs_ - vds_, vgd_ = vgs_ - vds_;
    double t = typ;
    double i0, gc[3];
    channelBranch(&i0, gc);
    double ich = t * (i0 + gc[0] * (vgs_ - vgs) + gc[1] * (vds_ - vds) + gc[2] * (vbs_ - vbs));
    double ibs = t * (cbs + gbs * (vbs_ - vbs));
    double ibd = t * (cbd + gbd * (vbd_ - vbd));
    double iqv[5] = {0, 0, 0, 0, 0};
    double v[5] = {vgs_, vgd_, vgb_, vbs_, vbd_};
    *ps = 0;
    if (tran) {
      for (int k = 0; k < 5; k++) {
        iqv[k] = t * (iq[k] + ag * cap(k) * (v[k] - dv[k]));
        *ps += v[k] * t * iqv[k];
      }
    }
    *id = ich - ibd - iqv[1] - iqv[4];
    *is = -ich - ibs - iqv[0] - iqv[3];
    *ig = iqv[0] + iqv[1] + iqv[2];
    *ib = ibs + ibd - iqv[2] + iqv[3] + iqv[4];
    for (int k = 0; k < 5; k++) v5[k] = v[k];
  }
  double current(const double* x) override {  // Operating :660-665, drain current
    double id, ig, is, ib, ps, v5[5];
    terminals(x, &id, &ig, &is, &ib, &ps, v5);
    return id;
  }
  // StoredEnergy, :710-731: co-energy of the junction charges (quadrature on 8
  // panels) and C*v^2/2 of the gate capacitances at the present voltages.
  double storedEnergy(const double v[5]) const {
    if (!hasGcap && !hasJcap) return 0;
    double w = 0;
    const double cz[2][2] = {{czbs, czbssw}, {czbd, czbdsw}};
    for (int k = 0; k < 2; k++) {
      double vv = v[3 + k];
      if (vv == 0 || cz[k][0] + cz[k][1] == 0) continue;
      auto qf = [&](double u) { double q, c; bulkCharge(u, cz[k][0], cz[k][1], &q, &c); return q; };
      w += vv * qf(vv) - integrate(qf, 0, vv, 8);
    }
    double o[7];
    channel(v[0], v[0] - v[1], v[3], o);
    double mc[3];
    meyerCaps(v[0], v[1], o[5], o[6], o[0], mc);
    const double ov[3] = {cgso, cgdo, cgbo};
    for (int k = 0; k < 3; k++) w += 0.5 * (mc[k] + ov[k]) * v[k] * v[k];
    return w;
  }
  OpPt operating(const double* x) override {  // Operating :660-665, ExteriorPower :760-765
    double id, ig, is, ib, ps, v5[5];
    terminals(x, &id, &ig, &is, &ib, &ps, v5);
    OpPt o;
    double vd = at(x, n, ud), vs = at(x, n, us);
    o.p = vd * id + at(x, n, g) * ig + vs * is + at(x, n, b) * ib;
    o.v = vd - vs; o.i = id; o.ps = ps;
    o.ext = -(o.p - o.ps);
    o.w = storedEnergy(v5);
    o.stores = true;
    return o;
  }
  void loadAC(ACCtx& c) override {  // device/mosfet.go:779-813
    typedef std::complex<double> cx;
    double o[7];
    channel(acc.vgs, acc.vds, acc.vbs, o);
    double gch[3];
    if (o[0] > 0) { gch[0] = o[2]; gch[1] = o[3]; gch[2] = o[4]; }
    else { gch[0] = -o[2]; gch[1] = o[2] + o[3] + o[4]; gch[2] = -o[4]; }
    double ib, gbsA, gbdA;
    bulkDiode(acc.vbs, iss, &ib, &gbsA);
    bulkDiode(acc.vbd, isd, &ib, &gbdA);
    double mc[3], q, cbsA, cbdA;
    meyerCaps(acc.vgs, acc.vgd, o[5], o[6], o[0], mc);
    bulkCharge(acc.vbs, czbs, czbssw, &q, &cbsA);
    bulkCharge(acc.vbd, czbd, czbdsw, &q, &cbdA);
    double cap[5] = {mc[0] + cgso, mc[1] + cgdo, mc[2] + cgbo, cbsA, cbdA};
    int ctrlP[3] = {g, dp, b}, ctrlN[3] = {sp, sp, sp};
    for (int k = 0; k < 3; k++) c.branch(dp, sp, gch[k], ctrlP[k], ctrlN[k], 0.0, 0, 0);
    c.stampY(b, sp, gbsA);
    c.stampY(b, dp, gbdA);
    int ends[5][2] = {{g, sp}, {g, dp}, {g, b}, {b, sp}, {b, dp}};
    for (int k = 0; k < 5; k++) c.stampY(ends[k][0], ends[k][1], cx(0, c.omega * cap[k]));
    if (dp != ud) c.stampY(ud, dp, gdpr);
    if (sp != us) c.stampY(us, sp, gspr);
  }
  void accept(const double* x, double t, int md) override {  // :668-705
    double vgs_, vds_, vbs_, vgb_;
    voltages(x, &vgs_, &vds_, &vbs_, &vgb_);
    double vgd_ = vgs_ - vds_, vbd_ = vbs_ - vds_;
    double o[7];
    channel(vgs_, vds_, vbs_, o);
    acc.vgs = vgs_; acc.vds = vds_; acc.vbs = vbs_; acc.von = o[5];
    acc.vgd = vgd_; acc.vgb = vgb_; acc.vbd = vbd_;
    double mc[3];
    meyerCaps(vgs_, vgd_, o[5], o[6], o[0], mc);
    double v[5] = {vgs_, vgd_, vgb_, vbs_, vbd_};
    double qbs, qbd, tmp;
    bulkCharge(vbs_, czbs, czbssw, &qbs, &tmp);
    bulkCharge(vbd_, czbd, czbdsw, &qbd, &tmp);
    if (md == ModeTran && tran) {
      double qs[5];
      for (int k = 0; k < 3; k++) qs[k] = qPrev[k] + capG[k] * (v[k] - vPrev[k]);
      qs[3] = qbs; qs[4] = qbd;
      for (int k = 0; k < 5; k++) {
        iqPrev[k] = iq[k] + ag * cap(k) * (v[k] - dv[k]);
        qPrev[k] = qs[k];
        hist[k].push(t, qs[k]);
      }
    } else {
      double ov[3] = {cgso, cgdo, cgbo};
      for (int k = 0; k < 3; k++) qPrev[k] = (mc[k] + ov[k]) * v[k];
      qPrev[3] = qbs; qPrev[4] = qbd;
      for (int k = 0; k < 5; k++) { iqPrev[k] = 0; hist[k].reset(); hist[k].push(t, qPrev[k]); }
    }
    for (int k = 0; k < 5; k++) vPrev[k] = v[k];
    for (int k = 0; k < 3; k++) meyerAcc[k] = mc[k];
  }
  double truncate(const double* x, const TruncCtx& tc) override {  // :734-757
    if (!tran) return kInf;
    double vgs_, vds_, vbs_, vgb_;
    voltages(x, &vgs_, &vds_, &vbs_, &vgb_);
    double v[5] = {vgs_, vgs_ - vds_, vgb_, vbs_, vbs_ - vds_};
    double h = kInf;
    for (int k = 0; k < 5; k++) {
      double qk, tmp;
      if (k < 3) qk = qPrev[k] + capG[k] * (v[k] - vPrev[k]);
      else if (k == 3) bulkCharge(v[k], czbs, czbssw, &qk, &tmp);
      else bulkCharge(v[k], czbd, czbdsw, &qk, &tmp);
      if (qk == 0 && qPrev[k] == 0) continue;
      double i = iq[k] + ag * cap(k) * (v[k] - dv[k]);
      h = std::min(h, lteStep(hist[k], qk, i, iqPrev[k], tc.abstol, tc));
    }
    return h;
  }
};

}  // namespace kso
