// ks_mos.cuh — MOSFET levels 1-3 of the GB300 engine, evaluated in FP64.
// Equations: device/mosfet.go (derive, limiting, junctions, Meyer), device/mosfet_levels.go
// (level 1) and device/mosfet_level23.go (levels 2, 3 in forward-mode dual numbers,
// device/dual.go).  Per-circuit derived constants live in the DM_* block.
#pragma once
#include "ks_devices.cuh"

namespace ksg {

struct Dual {  // value and d/dvgs, d/dvds, d/dvbs (device/dual.go:17)
  double v, d0, d1, d2;
  __device__ static Dual cst(double x) { return {x, 0, 0, 0}; }
  __device__ static Dual var(double x, int k) { return {x, k == 0 ? 1.0 : 0.0, k == 1 ? 1.0 : 0.0, k == 2 ? 1.0 : 0.0}; }
  __device__ Dual add(const Dual& b) const { return {v + b.v, d0 + b.d0, d1 + b.d1, d2 + b.d2}; }
  __device__ Dual sub(const Dual& b) const { return {v - b.v, d0 - b.d0, d1 - b.d1, d2 - b.d2}; }
  __device__ Dual addc(double c) const { return {v + c, d0, d1, d2}; }
  __device__ Dual neg() const { return {-v, -d0, -d1, -d2}; }
  __device__ Dual scale(double c) const { return {v * c, d0 * c, d1 * c, d2 * c}; }
  __device__ Dual mul(const Dual& b) const { return {v * b.v, d0 * b.v + v * b.d0, d1 * b.v + v * b.d1, d2 * b.v + v * b.d2}; }
  __device__ Dual div(const Dual& b) const {
    double q = v / b.v;
    return {q, (d0 - q * b.d0) / b.v, (d1 - q * b.d1) / b.v, (d2 - q * b.d2) / b.v};
  }
  __device__ Dual chain(double f, double df) const { return {f, df * d0, df * d1, df * d2}; }
  __device__ Dual sqrt_() const { double s = sqrt(v); return chain(s, 0.5 / s); }
  __device__ Dual exp_() const { double e = exp(v); return chain(e, e); }
  __device__ Dual log_() const { return chain(log(v), 1 / v); }
  __device__ Dual cos_() const { return chain(cos(v), -sin(v)); }
  __device__ Dual atan_() const { return chain(atan(v), 1 / (1 + v * v)); }
  __device__ Dual abs_() const { return v < 0 ? neg() : *this; }
  __device__ Dual powc(double c) const { double p = pow(v, c); return chain(p, c * p / v); }
};
__device__ __forceinline__ Dual dmax(const Dual& a, const Dual& b) { return b.v > a.v ? b : a; }
__device__ __forceinline__ Dual dmin(const Dual& a, const Dual& b) { return b.v < a.v ? b : a; }

__device__ __forceinline__ bool mgiven(uint64_t g, int k) { return (g >> k) & 1ull; }

// derive + deriveLevel, device/mosfet.go:218-323 and device/mosfet_levels.go:25-51.
__device__ inline void mos_derive(const KElem& e, const Col& V, const Col& D) {
  int p = e.param, d = e.derived;
  uint64_t given = e.given;
  int level = e.level;
  double typ = (e.flags & KS_F_PTYPE) ? -1.0 : 1.0;
  double vt = kK * kTNom / kQ;
  double KP = V[p + KS_M_P_KP], PHI = V[p + KS_M_P_PHI], GAMMA = V[p + KS_M_P_GAMMA];
  double VTO = V[p + KS_M_P_VTO], CJ = V[p + KS_M_P_CJ], PB = V[p + KS_M_P_PB], TOX = V[p + KS_M_P_TOX];
  double leff = V[p + KS_M_P_L] - 2 * V[p + KS_M_P_LD];
  double weff = level == 3 ? V[p + KS_M_P_W] - 2 * V[p + KS_M_P_WD] : V[p + KS_M_P_W];
  bool bad = !(leff > 0) || !(weff > 0);
  double cox = 0;
  bool toxGiven = mgiven(given, KS_M_P_TOX) || level >= 2;
  if (!bad && toxGiven && TOX > 0) {
    cox = kEpsOx / TOX;
    if (!mgiven(given, KS_M_P_KP)) KP = V[p + KS_M_P_UO] * cox * 1e-4;
    if (mgiven(given, KS_M_P_NSUB)) {
      double nsub = V[p + KS_M_P_NSUB] * 1e6;
      double ni = kNiSi;
      double eg = 1.16 - 7.02e-4 * kTNom * kTNom / (kTNom + 1108);
      if (level == 3) {
        double r = kTNom / 300;
        ni *= r * sqrt(r) * exp(0.5 * eg * (1.0 / 300 - 1 / kTNom) / (kK / kQ));
      }
      if (!(nsub > ni)) bad = true;
      else {
        if (!mgiven(given, KS_M_P_PHI)) PHI = fmax(0.1, 2 * vt * log(nsub / ni));
        if (!mgiven(given, KS_M_P_GAMMA)) GAMMA = sqrt(2 * kEpsSi * kQ * nsub) / cox;
        if (!mgiven(given, KS_M_P_VTO)) {
          double fermis = typ * 0.5 * PHI;
          double wkfng = 3.2;
          double TPG = V[p + KS_M_P_TPG];
          if (TPG != 0) wkfng = 3.25 + 0.5 * eg - typ * TPG * 0.5 * eg;
          double wkfngs = wkfng - (3.25 + 0.5 * eg + fermis);
          double vfb = wkfngs - V[p + KS_M_P_NSS] * 1e4 * kQ / cox;
          VTO = vfb + typ * (GAMMA * sqrt(PHI) + PHI);
        }
        if (!mgiven(given, KS_M_P_CJ)) CJ = sqrt(kEpsSi * kQ * nsub / (2 * PB));
      }
    }
  }
  double M = V[p + KS_M_P_MULT];
  D[d + DM_VT] = vt; D[d + DM_RVT] = 1 / vt; D[d + DM_LEFF] = leff; D[d + DM_WEFF] = weff; D[d + DM_COX] = cox;
  D[d + DM_OXCAP] = cox * leff * weff * M;
  D[d + DM_BETA] = KP * weff / leff * M;
  double vto = typ * VTO;
  D[d + DM_VTO] = vto;
  D[d + DM_VBI] = vto - GAMMA * sqrt(PHI);
  double rd = V[p + KS_M_P_RD], rs = V[p + KS_M_P_RS], RSH = V[p + KS_M_P_RSH];
  if (!mgiven(given, KS_M_P_RD) && RSH > 0) rd = RSH * V[p + KS_M_P_NRD];
  if (!mgiven(given, KS_M_P_RS) && RSH > 0) rs = RSH * V[p + KS_M_P_NRS];
  D[d + DM_GDPR] = rd > 0 ? M / rd : 0;
  D[d + DM_GSPR] = rs > 0 ? M / rs : 0;
  double IS = V[p + KS_M_P_IS], JS = V[p + KS_M_P_JS], AD = V[p + KS_M_P_AD], AS = V[p + KS_M_P_AS];
  double isd = IS * M, iss = IS * M;
  if (JS > 0 && AD > 0 && AS > 0) { isd = JS * AD * M; iss = JS * AS * M; }
  D[d + DM_ISD] = isd; D[d + DM_ISS] = iss;
  D[d + DM_VCRITD] = vt * log(vt / (kSqrt2 * fmax(isd, 1e-300)));
  D[d + DM_VCRITS] = vt * log(vt / (kSqrt2 * fmax(iss, 1e-300)));
  double czbd = mgiven(given, KS_M_P_CBD) ? V[p + KS_M_P_CBD] * M : CJ * AD * M;
  double czbs = mgiven(given, KS_M_P_CBS) ? V[p + KS_M_P_CBS] * M : CJ * AS * M;
  double czbdsw = V[p + KS_M_P_CJSW] * V[p + KS_M_P_PD] * M, czbssw = V[p + KS_M_P_CJSW] * V[p + KS_M_P_PS] * M;
  D[d + DM_CZBD] = czbd; D[d + DM_CZBS] = czbs; D[d + DM_CZBDSW] = czbdsw; D[d + DM_CZBSSW] = czbssw;
  double FC = V[p + KS_M_P_FC], MJ = V[p + KS_M_P_MJ], MJSW = V[p + KS_M_P_MJSW];
  D[d + DM_FBT0] = PB * (1 - pow(1 - FC, 1 - MJ)) / (1 - MJ); D[d + DM_FBT1] = pow(1 - FC, 1 + MJ); D[d + DM_FBT2] = 1 - FC * (1 + MJ);
  D[d + DM_FSW0] = PB * (1 - pow(1 - FC, 1 - MJSW)) / (1 - MJSW); D[d + DM_FSW1] = pow(1 - FC, 1 + MJSW); D[d + DM_FSW2] = 1 - FC * (1 + MJSW);
  double cgso = V[p + KS_M_P_CGSO] * weff * M, cgdo = V[p + KS_M_P_CGDO] * weff * M, cgbo = V[p + KS_M_P_CGBO] * leff * M;
  D[d + DM_CGSO] = cgso; D[d + DM_CGDO] = cgdo; D[d + DM_CGBO] = cgbo;
  D[d + DM_HASJCAP] = (czbd + czbdsw + czbs + czbssw > 0) ? 1.0 : 0.0;
  D[d + DM_HASGCAP] = (cox * leff * weff * M > 0 || cgso + cgdo + cgbo > 0) ? 1.0 : 0.0;
  double xd = 0, alpha = 0;
  bool hasNSUB = mgiven(given, KS_M_P_NSUB);
  if (hasNSUB) { alpha = 2 * kEpsSi / (kQ * V[p + KS_M_P_NSUB] * 1e6); xd = sqrt(alpha); }
  double cfs = 0, factor = 0, narrow = 0, eta3 = 0, sqrtPB = 0;
  if (level == 2) {
    cfs = kQ * V[p + KS_M_P_NFS] * 1e4 / cox;
    factor = V[p + KS_M_P_DELTA] * kPi * kEpsSi / (4 * cox * weff);
    sqrtPB = sqrt(PB);
    if (V[p + KS_M_P_VMAX] > 0 && !(V[p + KS_M_P_NEFF] > 0)) bad = true;
  } else if (level == 3) {
    cfs = kQ * V[p + KS_M_P_NFS] * 1e4 / cox;
    narrow = V[p + KS_M_P_DELTA] * 0.5 * kPi * kEpsSi / cox;
    eta3 = V[p + KS_M_P_ETA] * 8.15e-22 / (cox * leff * leff * leff);
  } else if (level != 1) bad = true;
  D[d + DM_XD] = xd; D[d + DM_ALPHA] = alpha; D[d + DM_CFS] = cfs; D[d + DM_FACTOR] = factor;
  D[d + DM_NARROW] = narrow; D[d + DM_ETA3] = eta3; D[d + DM_SQRTPB] = sqrtPB; D[d + DM_HASNSUB] = hasNSUB ? 1.0 : 0.0;
  D[d + DM_KP] = KP; D[d + DM_PHI] = PHI; D[d + DM_GAMMA] = GAMMA; D[d + DM_VTOP] = VTO; D[d + DM_CJ] = CJ;
  D[d + DM_BAD] = bad ? 1.0 : 0.0;
}

// fetlim, device/mosfet.go:347-385.
__device__ inline double fetlim(double vnew, double vold, double vto) {
  double vtsthi = fabs(2 * (vold - vto)) + 2, vtstlo = vtsthi / 2 + 2, vtox = vto + 3.5, delv = vnew - vold;
  if (vold >= vto) {
    if (vold >= vtox) {
      if (delv <= 0) {
        if (vnew >= vtox) { if (-delv > vtstlo) vnew = vold - vtstlo; }
        else vnew = fmax(vnew, vto + 2);
      } else if (delv >= vtsthi) vnew = vold + vtsthi;
    } else if (delv <= 0) vnew = fmax(vnew, vto - 0.5);
    else vnew = fmin(vnew, vto + 4);
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
__device__ inline double limvds(double vnew, double vold) {
  if (vold >= 3.5) {
    if (vnew > vold) return fmin(vnew, 3 * vold + 2);
    if (vnew < 3.5) return fmax(vnew, 2.0);
    return vnew;
  }
  if (vnew > vold) return fmin(vnew, 4.0);
  return fmax(vnew, -0.5);
}

// idsLevel1, device/mosfet_levels.go:79-113.  o = {cdrain, gm, gds, gmbs, von, vdsat}
__device__ inline void ids_level1(const Col& D, int d, double lambda, double vgs, double vds, double vbs, double* o) {
  double PHI = D[d + DM_PHI], GAMMA = D[d + DM_GAMMA], beta = D[d + DM_BETA];
  double sarg;
  if (vbs <= 0) sarg = sqrt(PHI - vbs);
  else { sarg = sqrt(PHI); sarg = fmax(0.0, sarg - vbs / (sarg + sarg)); }
  double von = D[d + DM_VBI] + GAMMA * sarg;
  double vgst = vgs - von;
  o[4] = von; o[5] = fmax(vgst, 0.0);
  double arg = sarg > 0 ? GAMMA / (sarg + sarg) : 0.0;
  if (vgst <= 0) { o[0] = o[1] = o[2] = o[3] = 0; return; }
  double betap = beta * (1 + lambda * vds);
  if (vgst <= vds) {
    o[0] = betap * vgst * vgst * 0.5; o[1] = betap * vgst; o[2] = lambda * beta * vgst * vgst * 0.5;
  } else {
    o[0] = betap * vds * (vgst - 0.5 * vds); o[1] = betap * vds;
    o[2] = betap * (vgst - vds) + lambda * beta * vds * (vgst - 0.5 * vds);
  }
  o[3] = o[1] * arg;
}

// level2VelocitySat, device/mosfet_level23.go:202-257.
__device__ inline bool level2_velsat(const Dual& gammad, const Dual& v1, const Dual& v2, const Dual& invxv,
                                     const Dual& sarg3, Dual* xout) {
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
  Dual r3 = r.mul(r).mul(r), s2 = s.mul(s);
  Dual pp = s2.scale(0.25).add(r3.scale(1.0 / 27));
  Dual p0 = pp.abs_(), p2 = p0.sqrt_();
  Dual y3;
  if (pp.v < 0) {
    Dual ro = s2.scale(0.25).add(p0).sqrt_().log_().scale(1.0 / 3).exp_();
    Dual fi = p2.scale(-2).div(s).atan_();
    y3 = ro.mul(fi.scale(1.0 / 3).cos_()).scale(2).sub(a.scale(1.0 / 3));
  } else {
    Dual u1 = s.scale(-0.5).add(p2).abs_(), u2 = s.scale(-0.5).sub(p2).abs_();
    Dual c1r = u1.v == 0 ? Dual::cst(0) : u1.powc(1.0 / 3), c2r = u2.v == 0 ? Dual::cst(0) : u2.powc(1.0 / 3);
    y3 = c1r.add(c2r).sub(a.scale(1.0 / 3));
  }
  Dual ra = a1.mul(a1).scale(0.25).sub(b1).add(y3);
  Dual rb = y3.mul(y3).scale(0.25).sub(d1);
  if (!(ra.v >= 0) || !(rb.v >= 0)) return false;
  Dual a3 = ra.sqrt_(), b3 = rb.sqrt_();
  const double sig1[4] = {1, -1, 1, -1}, sig2[4] = {1, 1, -1, -1};
  bool ok = false;
  Dual x = Dual::cst(0);
  for (int i = 0; i < 4; i++) {
    Dual a4 = a1.scale(0.5).add(a3.scale(sig1[i]));
    Dual b4 = y3.scale(0.5).add(b3.scale(sig2[i]));
    Dual delta4 = a4.mul(a4).scale(0.25).sub(b4);
    if (!(delta4.v >= 0)) continue;
    Dual t = delta4.sqrt_();
    for (int j = 0; j < 2; j++) {
      Dual rr = j == 0 ? a4.scale(-0.5).add(t) : a4.scale(-0.5).sub(t);
      if (!(rr.v > 0)) continue;
      double x2 = rr.v * rr.v;
      double poly = x2 * x2 + a1.v * x2 * rr.v + b1.v * x2 + c1.v * rr.v + d1.v;
      if (!(fabs(poly) <= 1e-6)) continue;
      if (!ok || rr.v < x.v) { x = rr; ok = true; }
    }
  }
  *xout = x;
  return ok;
}

__device__ __forceinline__ void dual_out(double* o, const Dual& id, double von, double vdsat) {
  o[0] = id.v; o[1] = id.d0; o[2] = id.d1; o[3] = id.d2; o[4] = von; o[5] = vdsat;
}

// idsLevel2, device/mosfet_level23.go:31-194.
__device__ inline void ids_level2(const Col& V, int p, const Col& D, int d, double vgsV, double vdsV, double vbsV, double* o) {
  Dual G = Dual::var(vgsV, 0), Dd = Dual::var(vdsV, 1), B = Dual::var(vbsV, 2);
  double phi = D[d + DM_PHI], GAMMA = D[d + DM_GAMMA], XJ = V[p + KS_M_P_XJ], UCRIT = V[p + KS_M_P_UCRIT];
  double UEXP = V[p + KS_M_P_UEXP], UO = V[p + KS_M_P_UO], VMAX = V[p + KS_M_P_VMAX], LAMBDA = V[p + KS_M_P_LAMBDA];
  double NEFF = V[p + KS_M_P_NEFF], NFS = V[p + KS_M_P_NFS];
  double leff = D[d + DM_LEFF], cox = D[d + DM_COX], beta = D[d + DM_BETA], vt = D[d + DM_VT];
  double lxd = D[d + DM_XD], lcfs = D[d + DM_CFS];
  bool hasNSUB = D[d + DM_HASNSUB] != 0;
  double sphi = sqrt(phi), sphi3 = phi * sphi;
  Dual phiMinVbs = B.neg().addc(phi);
  Dual sarg, dsrgdb, barg, dbrgdb;
  if (B.v <= 0) { sarg = phiMinVbs.sqrt_(); dsrgdb = Dual::cst(-0.5).div(sarg); }
  else { sarg = Dual::cst(sphi).div(B.scale(0.5 / phi).addc(1)); dsrgdb = sarg.mul(sarg).scale(-0.5 / sphi3); }
  if (B.v - Dd.v <= 0) { barg = phiMinVbs.add(Dd).sqrt_(); dbrgdb = Dual::cst(-0.5).div(barg); }
  else { barg = Dual::cst(sphi).div(B.sub(Dd).scale(0.5 / phi).addc(1)); dbrgdb = barg.mul(barg).scale(-0.5 / sphi3); }
  double factor = D[d + DM_FACTOR], eta = 1 + factor;
  Dual vbin = phiMinVbs.scale(factor).addc(D[d + DM_VBI]);
  Dual gamasd = Dual::cst(GAMMA), dgddvb = Dual::cst(0);
  if ((GAMMA > 0 || hasNSUB) && XJ > 0) {
    Dual xws = sarg.scale(lxd), xwd = barg.scale(lxd);
    Dual args = xws.scale(2 / XJ).addc(1).sqrt_(), argd = xwd.scale(2 / XJ).addc(1).sqrt_();
    double t = 0.5 * XJ / leff;
    Dual argss = args.addc(-1).scale(t), argsd = argd.addc(-1).scale(t);
    gamasd = argss.add(argsd).neg().addc(1).scale(GAMMA);
    Dual dbargs = dsrgdb.scale(lxd).div(args).scale(0.5 / leff);
    Dual dbargd = dbrgdb.scale(lxd).div(argd).scale(0.5 / leff);
    dgddvb = dbargs.add(dbargd).scale(-GAMMA);
  }
  Dual vonD = vbin.add(gamasd.mul(sarg));
  bool nfs = NFS != 0;
  Dual xn = Dual::cst(0), argg = Dual::cst(0);
  if (nfs) {
    Dual cdonco = gamasd.mul(dsrgdb).add(dgddvb.mul(sarg)).neg().addc(factor);
    xn = cdonco.addc(1 + lcfs);
    Dual vtxn = xn.scale(vt);
    vonD = vonD.add(vtxn);
    argg = Dual::cst(1).div(vtxn);
  } else if (G.v <= vbin.v) {
    o[0] = o[1] = o[2] = o[3] = 0; o[4] = vonD.v; o[5] = 0; return;
  }
  Dual vgst = G.sub(vonD);
  Dual ufact = Dual::cst(1);
  double crit = UCRIT * 100 * kEpsSi / cox;
  if (vgst.v > crit) ufact = Dual::cst(crit).div(vgst).powc(UEXP);
  Dual ueff = ufact.scale(UO * 1e-4);
  Dual vgsx = nfs ? dmax(G, vonD) : G;
  Dual gammad = gamasd.scale(1 / eta);
  Dual vgb = vgsx.sub(vbin).scale(1 / eta);
  Dual vdsatD = Dual::cst(0);
  if (gammad.v > 0) {
    Dual argv = vgb.add(phiMinVbs);
    if (argv.v > 0) {
      Dual gammd2 = gammad.mul(gammad);
      Dual arg1 = argv.scale(4).div(gammd2).addc(1).sqrt_();
      vdsatD = dmax(vgb.add(gammd2.mul(arg1.neg().addc(1)).scale(0.5)), Dual::cst(0));
    }
  } else vdsatD = dmax(vgb, Dual::cst(0));
  Dual sarg3 = sarg.mul(sarg).mul(sarg);
  if (VMAX > 0) {
    Dual x;
    if (level2_velsat(gammad, vgb.add(phiMinVbs), phiMinVbs, ueff.scale(1 / (VMAX * leff)), sarg3, &x))
      vdsatD = x.mul(x).sub(phiMinVbs);
  }
  Dual xlamda = Dual::cst(LAMBDA);
  Dual bodys = Dual::cst(0);
  if (Dd.v != 0) {
    Dual bsarg;
    if (B.v - vdsatD.v <= 0) bsarg = vdsatD.add(phiMinVbs).sqrt_();
    else bsarg = Dual::cst(sphi).div(B.sub(vdsatD).scale(0.5 / phi).addc(1));
    bodys = bsarg.mul(bsarg).mul(bsarg).sub(sarg3);
    if (hasNSUB && !(LAMBDA > 0)) {
      if (VMAX <= 0) {
        Dual argv = Dd.sub(vdsatD).scale(0.25);
        Dual sargv = argv.mul(argv).addc(1).sqrt_();
        xlamda = argv.add(sargv).sqrt_().mul(Dual::cst(lxd).div(Dd.scale(leff)));
      } else {
        double xdv = lxd / sqrt(NEFF);
        Dual xlv = Dual::cst(VMAX * xdv * 0.5).div(ueff);
        Dual argv = dmax(Dd.sub(vdsatD), Dual::cst(0));
        Dual xls = xlv.mul(xlv).add(argv).sqrt_();
        xlamda = xls.sub(xlv).mul(Dual::cst(xdv).div(Dd.scale(leff)));
      }
    }
  }
  double xwb = lxd * D[d + DM_SQRTPB];
  double xld = leff - xwb;
  Dual clfact = xlamda.mul(Dd).neg().addc(1);
  if (!hasNSUB) xwb = 0.25e-6;
  Dual xleff = clfact.scale(leff);
  if (xleff.v < xwb) {
    Dual deltal = xlamda.mul(Dd).scale(leff);
    xleff = Dual::cst(xwb).div(deltal.addc(-xld).scale(1 / xwb).addc(1));
    clfact = xleff.scale(1 / leff);
  }
  Dual beta1 = ufact.scale(beta).div(clfact);
  if (Dd.v <= 1e-10) {
    Dual g = Dual::cst(0);
    if (G.v > vonD.v) g = beta1.mul(G.sub(vbin).sub(gamasd.mul(sarg)));
    else if (nfs) g = beta1.mul(vonD.sub(vbin).sub(gamasd.mul(sarg))).mul(argg.mul(G.sub(vonD)).exp_());
    o[0] = 0; o[1] = 0; o[2] = g.v; o[3] = 0; o[4] = vonD.v; o[5] = vdsatD.v; return;
  }
  Dual id;
  if (nfs && G.v <= vonD.v) {
    if (vdsatD.v <= 0) { o[0] = o[1] = o[2] = o[3] = 0; o[4] = vonD.v; o[5] = vdsatD.v; return; }
    Dual vdson = dmin(vdsatD, Dd);
    Dual body = Dd.v > vdsatD.v ? bodys : barg.mul(barg).mul(barg).sub(sarg3);
    Dual cdson = beta1.mul(vonD.sub(vbin).sub(vdson.scale(0.5 * eta)).mul(vdson).sub(gamasd.mul(body).scale(1 / 1.5)));
    id = cdson.mul(argg.mul(G.sub(vonD)).exp_());
  } else if (Dd.v <= vdsatD.v) {
    Dual body = barg.mul(barg).mul(barg).sub(sarg3);
    id = beta1.mul(G.sub(vbin).sub(Dd.scale(0.5 * eta)).mul(Dd).sub(gamasd.mul(body).scale(1 / 1.5)));
  } else {
    id = beta1.mul(G.sub(vbin).sub(vdsatD.scale(0.5 * eta)).mul(vdsatD).sub(gamasd.mul(bodys).scale(1 / 1.5)));
  }
  dual_out(o, id, vonD.v, vdsatD.v);
}

// idsLevel3, device/mosfet_level23.go:277-378.
__device__ inline void ids_level3(const Col& V, int p, const Col& D, int d, double vgsV, double vdsV, double vbsV, double* o) {
  const double coeff0 = 0.0631353, coeff1 = 0.8013292, coeff2 = -0.01110777;
  Dual G = Dual::var(vgsV, 0), Dd = Dual::var(vdsV, 1), B = Dual::var(vbsV, 2);
  double phi = D[d + DM_PHI], XJ = V[p + KS_M_P_XJ], LD = V[p + KS_M_P_LD], GAMMA = D[d + DM_GAMMA];
  double THETA = V[p + KS_M_P_THETA], UO = V[p + KS_M_P_UO], VMAX = V[p + KS_M_P_VMAX], KAPPA = V[p + KS_M_P_KAPPA];
  double NFS = V[p + KS_M_P_NFS];
  double leff = D[d + DM_LEFF], weff = D[d + DM_WEFF], vt = D[d + DM_VT], lxd = D[d + DM_XD];
  double lalpha = D[d + DM_ALPHA], lnarrow = D[d + DM_NARROW], leta3 = D[d + DM_ETA3], lcfs = D[d + DM_CFS];
  Dual phibs, sqphbs;
  if (B.v <= 0) { phibs = B.neg().addc(phi); sqphbs = phibs.sqrt_(); }
  else { sqphbs = Dual::cst(sqrt(phi)).div(B.scale(1 / (2 * phi)).addc(1)); phibs = sqphbs.mul(sqphbs); }
  Dual fshort = Dual::cst(1);
  if (XJ != 0 && lxd != 0) {
    Dual wponxj = sqphbs.scale(lxd / XJ);
    Dual wconxj = wponxj.mul(wponxj).scale(coeff2).add(wponxj.scale(coeff1)).addc(coeff0);
    double djonxj = LD / XJ;
    Dual arga = wconxj.addc(djonxj);
    Dual argc = wponxj.div(wponxj.addc(1));
    Dual argb = argc.mul(argc).neg().addc(1).sqrt_();
    fshort = arga.mul(argb).addc(-djonxj).scale(-XJ / leff).addc(1);
  }
  Dual gammas = fshort.scale(GAMMA);
  Dual fbodys = gammas.div(sqphbs).scale(0.25);
  Dual fbody = fbodys.addc(lnarrow / weff);
  Dual qbonco = gammas.mul(sqphbs).add(phibs.scale(lnarrow / weff));
  Dual vth = Dd.scale(-leta3).addc(D[d + DM_VBI]).add(qbonco);
  Dual vonD = vth;
  bool nfs = NFS != 0;
  Dual xn = Dual::cst(0);
  if (nfs) {
    xn = qbonco.div(phibs.scale(2)).addc(1 + lcfs);
    vonD = vth.add(xn.scale(vt));
  } else if (G.v <= vonD.v) {
    o[0] = o[1] = o[2] = o[3] = 0; o[4] = vonD.v; o[5] = 0; return;
  }
  Dual vgsx = dmax(G, vonD);
  Dual onfg = vgsx.sub(vth).scale(THETA).addc(1);
  Dual fgate = Dual::cst(1).div(onfg);
  Dual us = fgate.scale(UO * 1e-4);
  Dual onfbdy = Dual::cst(1).div(fbody.addc(1));
  Dual arga = vgsx.sub(vth).mul(onfbdy);
  Dual vdsatD = arga;
  Dual vdsc = Dual::cst(0);
  if (VMAX > 0) {
    vdsc = Dual::cst(leff * VMAX).div(us);
    Dual argb = arga.mul(arga).add(vdsc.mul(vdsc)).sqrt_();
    vdsatD = arga.add(vdsc).sub(argb);
  }
  Dual vdsx = dmin(Dd, vdsatD);
  Dual beta = fgate.scale(D[d + DM_BETA]);
  if (vdsx.v == 0) {
    Dual g = beta.mul(vgsx.sub(vth));
    if (nfs && G.v < vonD.v) g = g.mul(G.sub(vonD).div(xn.scale(vt)).exp_());
    o[0] = 0; o[1] = 0; o[2] = g.v; o[3] = 0; o[4] = vonD.v; o[5] = vdsatD.v; return;
  }
  Dual cdo = vgsx.sub(vth).sub(fbody.addc(1).mul(vdsx).scale(0.5));
  Dual id = beta.mul(cdo).mul(vdsx);
  Dual fdrain = Dual::cst(0);
  if (VMAX > 0) {
    fdrain = Dual::cst(1).div(vdsx.div(vdsc).addc(1));
    id = id.mul(fdrain);
  }
  bool clm = false;
  Dual delxl = Dual::cst(0);
  if (Dd.v <= vdsatD.v) {
    if (VMAX <= 0 && lalpha != 0) {
      Dual r = Dd.div(vdsatD);
      Dual r2 = r.mul(r);
      delxl = vdsatD.scale(KAPPA * lalpha / 8).sqrt_().mul(r2.mul(r2));
      clm = true;
    }
  } else if (VMAX <= 0) {
    delxl = Dd.sub(vdsatD).add(vdsatD.scale(1.0 / 8)).scale(KAPPA * lalpha).sqrt_();
    clm = true;
  } else if (lalpha != 0) {
    Dual gdsat = dmax(id.mul(fdrain.neg().addc(1)).div(vdsc), Dual::cst(1e-12));
    Dual emax = id.div(gdsat).scale(KAPPA / leff);
    Dual a = emax.scale(0.5 * lalpha);
    Dual argb = a.mul(a).add(Dd.sub(vdsatD).scale(KAPPA * lalpha)).sqrt_();
    delxl = argb.sub(a);
    clm = true;
  }
  if (clm) {
    if (delxl.v > 0.5 * leff) delxl = Dual::cst(-leff * leff / 4).div(delxl).addc(leff);
    id = id.div(delxl.scale(-1 / leff).addc(1));
  }
  if (nfs && G.v < vonD.v) id = id.mul(G.sub(vonD).div(xn.scale(vt)).exp_());
  dual_out(o, id, vonD.v, vdsatD.v);
}

// channel, device/mosfet.go:464-473.  o = {mode, cdrain, gm, gds, gmbs, von, vdsat}
__device__ inline void mos_channel(const KElem& e, const Col& V, const Col& D, double vgs, double vds, double vbs, double* o) {
  double md = 1, vg = vgs, vd = vds, vb = vbs;
  if (vds < 0) { md = -1; vg = vgs - vds; vd = -vds; vb = vbs - vds; }
  o[0] = md;
  if (e.level == 2) ids_level2(V, e.param, D, e.derived, vg, vd, vb, o + 1);
  else if (e.level == 3) ids_level3(V, e.param, D, e.derived, vg, vd, vb, o + 1);
  else ids_level1(D, e.derived, V[e.param + KS_M_P_LAMBDA], vg, vd, vb, o + 1);
}

// bulkDiode, device/mosfet.go:408-414 (rvt = 1/vt).
__device__ __forceinline__ void mos_bulk_diode(double v, double is, double vt, double rvt, double gmin, double* i,
                                               double* g) {
  if (v <= -3 * vt) { *i = gmin * v - is; *g = gmin; return; }
  double ex = exp(fmin(v * rvt, 700.0));
  *i = is * (ex - 1) + gmin * v; *g = is * ex * rvt + gmin;
}

// meyer, device/mosfet.go:419-438.
__device__ inline void meyer(double vgs, double vgd, double von, double vdsat, double phi, double cox, double* c) {
  double vgst = vgs - von;
  vdsat = fmax(vdsat, 0.0);
  if (vgst <= -phi) { c[0] = 0; c[1] = 0; c[2] = cox; return; }
  if (vgst <= -phi / 2) { c[0] = 0; c[1] = 0; c[2] = -vgst * cox / phi; return; }
  if (vgst <= 0) { c[0] = 2 * (vgst * cox / (1.5 * phi) + cox / 3); c[1] = 0; c[2] = -vgst * cox / phi; return; }
  double vds = vgs - vgd;
  if (vdsat <= vds) { c[0] = 2 * cox / 3; c[1] = 0; c[2] = 0; return; }
  double vddif = 2 * vdsat - vds, vddif1 = vdsat - vds, vddif2 = vddif * vddif;
  c[0] = 2 * cox * (1 - vddif1 * vddif1 / vddif2) / 3;
  c[1] = 2 * cox * (1 - vdsat * vdsat / vddif2) / 3;
  c[2] = 0;
}

// meyerCaps, device/mosfet.go:441-451.
__device__ inline void meyer_caps(const Col& D, int d, double vgs, double vgd, double von, double vdsat, double md, double* c) {
  double cox = D[d + DM_OXCAP];
  if (cox == 0) { c[0] = c[1] = c[2] = 0; return; }
  if (md > 0) { meyer(vgs, vgd, von, vdsat, D[d + DM_PHI], cox, c); return; }
  double t[3];
  meyer(vgd, vgs, von, vdsat, D[d + DM_PHI], cox, t);
  c[0] = t[1]; c[1] = t[0]; c[2] = t[2];
}

// bulkCharge, device/mosfet.go:455-460.
__device__ inline void mos_bulk_charge(const Col& V, int p, const Col& D, int d, double v, double cz, double czsw,
                                       double* q, double* c) {
  double q1, c1, q2, c2, PB = V[p + KS_M_P_PB], FC = V[p + KS_M_P_FC];
  depletion(v, cz, PB, V[p + KS_M_P_MJ], FC, D[d + DM_FBT0], D[d + DM_FBT1], D[d + DM_FBT2], &q1, &c1);
  depletion(v, czsw, PB, V[p + KS_M_P_MJSW], FC, D[d + DM_FSW0], D[d + DM_FSW1], D[d + DM_FSW2], &q2, &c2);
  *q = q1 + q2; *c = c1 + c2;
}

template <bool NEW, class SY>
__device__ inline void mos_voltages(const KElem& e, SY& s, double* vgs, double* vds, double* vbs, double* vgb) {
  auto X = [&](int i) { return NEW ? xn_(s, i) : xo_(s, i); };
  double t = (e.flags & KS_F_PTYPE) ? -1.0 : 1.0;  // device/mosfet.go:340-344
  double vg = X(e.u[2]), vb = X(e.u[3]), vdp = X(e.u[4]), vsp = X(e.u[5]);
  *vgs = t * (vg - vsp); *vds = t * (vdp - vsp); *vbs = t * (vb - vsp); *vgb = t * (vg - vb);
}

template <class SY>
__device__ __forceinline__ void mos_branch1(SY& s, double typ, int a, int b, double i0, double g, int pk,
                                            int mk, double v0) {  // device/mosfet.go:563-578, one control
  double ieq = i0;
  if (g != 0) {
    sadd(s, a, pk, g); sadd(s, a, mk, -g); sadd(s, b, pk, -g); sadd(s, b, mk, g);
    ieq -= g * v0;
  }
  ieq *= typ;
  srhs(s, a, -ieq); srhs(s, b, ieq);
}

// Load + stamp, device/mosfet.go:476-611.
template <class SY>
__device__ __forceinline__ void mos_load(const KElem& e, const Col& V, const Col& D, const Col& S, SY& sys,
                                const LoadParams& lp) {
  int d = e.derived, p = e.param;
  double vt = D[d + DM_VT];
  double vgs, vds, vbs, vgb0;
  mos_voltages<false>(e, sys, &vgs, &vds, &vbs, &vgb0);
  bool lim = false;
  if (lp.initJct) { vbs = -1; vgs = D[d + DM_VTO]; vds = 0; lim = true; }
  else {
    double avgs = S[SM_AVGS], avds = S[SM_AVDS], avbs = S[SM_AVBS], von = S[SM_AVON];
    double vgd = vgs - vds, vgdOld = avgs - avds;
    if (avds >= 0) {
      vgs = fetlim(vgs, avgs, von);
      vds = vgs - vgd;
      vds = limvds(vds, avds);
    } else {
      vgd = fetlim(vgd, vgdOld, von);
      vds = vgs - vgd;
      vds = -limvds(-vds, -avds);
      vgs = vgd + vds;
    }
    if (vds >= 0) vbs = pnjlim(vbs, avbs, vt, D[d + DM_RVT], D[d + DM_VCRITS], &lim);
    else {
      double vbd = pnjlim(vbs - vds, avbs - avds, vt, D[d + DM_RVT], D[d + DM_VCRITD], &lim);
      vbs = vbd + vds;
    }
  }
  double vbd = vbs - vds, vgd = vgs - vds, vgb = vgs - vbs;
  S[SM_VGS] = vgs; S[SM_VDS] = vds; S[SM_VBS] = vbs; S[SM_VBD] = vbd; S[SM_VGD] = vgd; S[SM_VGB] = vgb;
  S[SM_AVGS] = vgs; S[SM_AVDS] = vds; S[SM_AVBS] = vbs;
  double cbs, gbs, cbd, gbd;
  mos_bulk_diode(vbs, D[d + DM_ISS], vt, D[d + DM_RVT], lp.gmin, &cbs, &gbs);
  mos_bulk_diode(vbd, D[d + DM_ISD], vt, D[d + DM_RVT], lp.gmin, &cbd, &gbd);
  double o[7];
  mos_channel(e, V, D, vgs, vds, vbs, o);
  S[SM_CBS] = cbs; S[SM_GBS] = gbs; S[SM_CBD] = cbd; S[SM_GBD] = gbd;
  S[SM_MODE] = o[0]; S[SM_CDRAIN] = o[1]; S[SM_GM] = o[2]; S[SM_GDS] = o[3]; S[SM_GMBS] = o[4];
  S[SM_VON] = o[5]; S[SM_VDSAT] = o[6]; S[SM_AVON] = o[5]; S[SM_LIM] = lim ? 1.0 : 0.0;
  bool tran = lp.mode == ModeTran && (D[d + DM_HASGCAP] != 0 || D[d + DM_HASJCAP] != 0);
  double ag = 0, iq[5] = {0, 0, 0, 0, 0}, cap[5] = {0, 0, 0, 0, 0};
  double dv[5] = {vgs, vgd, vgb, vbs, vbd};
  if (tran) {
    ag = lp.method == TRAP ? 2 * lp.rh : lp.rh;
    double mc[3];
    meyer_caps(D, d, vgs, vgd, o[5], o[6], o[0], mc);
    double ov[3] = {D[d + DM_CGSO], D[d + DM_CGDO], D[d + DM_CGBO]};
    for (int k = 0; k < 3; k++) cap[k] = (mc[k] + S[SM_MEYER0 + k]) / 2 + ov[k];
    double qbs, qbd;
    mos_bulk_charge(V, p, D, d, vbs, D[d + DM_CZBS], D[d + DM_CZBSSW], &qbs, &cap[3]);
    mos_bulk_charge(V, p, D, d, vbd, D[d + DM_CZBD], D[d + DM_CZBDSW], &qbd, &cap[4]);
    double qs[5];
    for (int k = 0; k < 3; k++) qs[k] = S[SM_QPREV0 + k] + cap[k] * (dv[k] - S[SM_VPREV0 + k]);
    qs[3] = qbs; qs[4] = qbd;
    for (int k = 0; k < 5; k++) {
      iq[k] = ag * (qs[k] - S[SM_QPREV0 + k]);
      if (lp.method == TRAP) iq[k] -= S[SM_IQPREV0 + k];
    }
  }
  S[SM_TRAN] = tran ? 1.0 : 0.0; S[SM_AG] = ag;
  for (int k = 0; k < 3; k++) S[SM_CAPG0 + k] = cap[k];
  S[SM_CAPB0] = cap[3]; S[SM_CAPB0 + 1] = cap[4];
  for (int k = 0; k < 5; k++) { S[SM_IQ0 + k] = iq[k]; S[SM_DV0 + k] = dv[k]; }
  // stamp
  double typ = (e.flags & KS_F_PTYPE) ? -1.0 : 1.0;
  int g = e.u[2], b = e.u[3], dp = e.u[4], sp = e.u[5];
  double i0 = o[1], g0 = o[2], g1 = o[3], g2 = o[4];
  if (o[0] <= 0) { i0 = -o[1]; g0 = -o[2]; g1 = o[2] + o[3] + o[4]; g2 = -o[4]; }
  {  // channel branch dp -> sp controlled by vgs, vds, vbs
    double ieq = i0;
    if (g0 != 0) { sadd(sys, dp, g, g0); sadd(sys, dp, sp, -g0); sadd(sys, sp, g, -g0); sadd(sys, sp, sp, g0); ieq -= g0 * vgs; }
    if (g1 != 0) { sadd(sys, dp, dp, g1); sadd(sys, dp, sp, -g1); sadd(sys, sp, dp, -g1); sadd(sys, sp, sp, g1); ieq -= g1 * vds; }
    if (g2 != 0) { sadd(sys, dp, b, g2); sadd(sys, dp, sp, -g2); sadd(sys, sp, b, -g2); sadd(sys, sp, sp, g2); ieq -= g2 * vbs; }
    ieq *= typ;
    srhs(sys, dp, -ieq); srhs(sys, sp, ieq);
  }
  mos_branch1(sys, typ, b, sp, cbs, gbs, b, sp, vbs);
  mos_branch1(sys, typ, b, dp, cbd, gbd, b, dp, vbd);
  if (tran) {
    const int ea[5] = {g, g, g, b, b}, eb[5] = {sp, dp, b, sp, dp};
    for (int k = 0; k < 5; k++) mos_branch1(sys, typ, ea[k], eb[k], iq[k], ag * cap[k], ea[k], eb[k], dv[k]);
  }
  if (dp != e.u[0]) stamp_g(sys, e.u[0], dp, D[d + DM_GDPR]);
  if (sp != e.u[1]) stamp_g(sys, e.u[1], sp, D[d + DM_GSPR]);
}

// ConvTest, device/mosfet.go:618-631.
template <class SY>
__device__ __forceinline__ bool mos_conv(const KElem& e, const Col& V, const Col& D, const Col& S, SY& sys,
                                double reltol, double abstol, double gmin) {
  int d = e.derived;
  double vgs, vds, vbs, vgb;
  mos_voltages<true>(e, sys, &vgs, &vds, &vbs, &vgb);
  double vbd = vbs - vds;
  double i0 = S[SM_CDRAIN], g0 = S[SM_GM], g1 = S[SM_GDS], g2 = S[SM_GMBS];
  if (S[SM_MODE] <= 0) { double gm = g0; i0 = -i0; g0 = -gm; g1 = gm + g1 + g2; g2 = -g2; }
  double ich = i0 + g0 * (vgs - S[SM_VGS]) + g1 * (vds - S[SM_VDS]) + g2 * (vbs - S[SM_VBS]);
  double ibs = S[SM_CBS] + S[SM_GBS] * (vbs - S[SM_VBS]);
  double ibd = S[SM_CBD] + S[SM_GBD] * (vbd - S[SM_VBD]);
  double o[7];
  mos_channel(e, V, D, vgs, vds, vbs, o);
  double ichN = o[0] * o[1];
  double ibsN, ibdN, t;
  double vt = D[d + DM_VT];
  mos_bulk_diode(vbs, D[d + DM_ISS], vt, D[d + DM_RVT], gmin, &ibsN, &t);
  mos_bulk_diode(vbd, D[d + DM_ISD], vt, D[d + DM_RVT], gmin, &ibdN, &t);
  double a1 = ich - ibd, b1 = ichN - ibdN, a2 = ibs + ibd, b2 = ibsN + ibdN;
  return fabs(a1 - b1) <= reltol * fmax(fabs(a1), fabs(b1)) + abstol &&
         fabs(a2 - b2) <= reltol * fmax(fabs(a2), fabs(b2)) + abstol;
}

// Accept, device/mosfet.go:668-705.
template <class SY>
__device__ __forceinline__ void mos_accept(const KElem& e, const Col& V, const Col& D, const Col& S, SY& sys,
                                  double t, int mode) {
  int d = e.derived, p = e.param;
  double vgs, vds, vbs, vgb;
  mos_voltages<true>(e, sys, &vgs, &vds, &vbs, &vgb);
  double vgd = vgs - vds, vbd = vbs - vds;
  double o[7];
  mos_channel(e, V, D, vgs, vds, vbs, o);
  S[SM_AVGS] = vgs; S[SM_AVDS] = vds; S[SM_AVBS] = vbs; S[SM_AVON] = o[5];
  double mc[3];
  meyer_caps(D, d, vgs, vgd, o[5], o[6], o[0], mc);
  double v[5] = {vgs, vgd, vgb, vbs, vbd};
  double qbs, qbd, tmp;
  mos_bulk_charge(V, p, D, d, vbs, D[d + DM_CZBS], D[d + DM_CZBSSW], &qbs, &tmp);
  mos_bulk_charge(V, p, D, d, vbd, D[d + DM_CZBD], D[d + DM_CZBDSW], &qbd, &tmp);
  if (mode == ModeTran && S[SM_TRAN] != 0) {
    double qs[5];
    for (int k = 0; k < 3; k++) qs[k] = S[SM_QPREV0 + k] + S[SM_CAPG0 + k] * (v[k] - S[SM_VPREV0 + k]);
    qs[3] = qbs; qs[4] = qbd;
    double ag = S[SM_AG];
    for (int k = 0; k < 5; k++) {
      double cap = k < 3 ? S[SM_CAPG0 + k] : S[SM_CAPB0 + k - 3];
      S[SM_IQPREV0 + k] = S[SM_IQ0 + k] + ag * cap * (v[k] - S[SM_DV0 + k]);
      S[SM_QPREV0 + k] = qs[k];
      hist_push(S, SM_HIST + k * H_SIZE, t, qs[k]);
    }
  } else {
    double ov[3] = {D[d + DM_CGSO], D[d + DM_CGDO], D[d + DM_CGBO]};
    for (int k = 0; k < 3; k++) S[SM_QPREV0 + k] = (mc[k] + ov[k]) * v[k];
    S[SM_QPREV0 + 3] = qbs; S[SM_QPREV0 + 4] = qbd;
    for (int k = 0; k < 5; k++) {
      S[SM_IQPREV0 + k] = 0;
      hist_reset(S, SM_HIST + k * H_SIZE);
      hist_push(S, SM_HIST + k * H_SIZE, t, S[SM_QPREV0 + k]);
    }
  }
  for (int k = 0; k < 5; k++) S[SM_VPREV0 + k] = v[k];
  for (int k = 0; k < 3; k++) S[SM_MEYER0 + k] = mc[k];
}

}  // namespace ksg
