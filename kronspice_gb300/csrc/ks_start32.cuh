// ks_start32.cuh — FP32 Newton stage of the operating point's start (GB300 engine).
//
// GB300 issues an FP64 warp instruction once every ~64-80 cycles per SM
// sub-partition (2 FP64 lanes per clock per SM) and FP32 at 32 lanes per clock
// per sub-partition, and a lane masked off by divergence costs the FP64 pipe as
// much as an active one.  The time of a batched operating point is therefore set
// by the FP64 chain of its slowest circuit: Newton iterations times the FP64
// work of one iteration.  This stage moves the bulk of the Newton iterations to
// FP32: from the start (the learned prediction, or InitJct junction voltages) it
// runs Newton with the devices evaluated in FP32 (parameters from FP32 copies of
// the value and derived-constant columns, fast exponential and logarithm),
// limiting as the device models limit (pnjlim, fetlim, limvds), the system
// stamped and factored in FP32, until the step is at FP32 resolution.  Its point
// then becomes the start of the FP64 solve (NodeSet semantics: the limiting state
// is seeded from it, analysis/newton.go:221-243), whose Newton iterations,
// convergence test (analysis/newton.go:59-82), fallback chain and result are the
// reference's, so the FP32 stage changes how many FP64 iterations a circuit
// needs, not what it converges to.  A circuit whose FP32 stage fails (a singular
// or non-finite FP32 system, no convergence within the limit) keeps its original
// start.
//
// Covered elements: R, C, L, V, I, diodes, Gummel-Poon BJTs and level-1
// MOSFETs.  A topology with a level-2/3 MOSFET skips the stage.
#pragma once
#include "ks_solve.cuh"

namespace ksg {

// FP32 copies of a batch's SoA columns (same layouts as values / derived /
// state), made after the derived constants.
struct K32 {
  const float* values;
  const float* derived;
  float* state;
};

struct Col32 {
  float* p;
  int64_t B;
  __device__ __forceinline__ float& operator[](int k) const { return p[(int64_t)k * B]; }
};

template <class S>
__device__ __forceinline__ void sadd32(S& s, int i, int j, float v) {
  if (i < 0 || j < 0) return;
  s.a32(i, j) += v;
}
template <class S>
__device__ __forceinline__ void srhs32(S& s, int i, float v) {
  if (i < 0) return;
  s.r32(i) += v;
}
template <class S>
__device__ __forceinline__ float xo32_(S& s, int i) { return i >= 0 ? s.xo32(i) : 0.0f; }
template <class S>
__device__ __forceinline__ float xn32_(S& s, int i) { return i >= 0 ? s.x32(i) : 0.0f; }

// Exponent argument clamp: FP32 overflows above e^88.
constexpr float kExpClamp32 = 80.0f;

// pnjlim (device/diode.go:214-226) in FP32.
__device__ __forceinline__ float pnjlim32(float vnew, float vold, float vt, float rvt, float vcrit, bool* lim) {
  if (vnew > vcrit && fabsf(vnew - vold) > 2 * vt) {
    *lim = true;
    if (vold > 0) {
      float arg = 1 + (vnew - vold) * rvt;
      return arg > 0 ? vold + vt * __logf(arg) : vcrit;
    }
    return vt * __logf(vnew * rvt);
  }
  *lim = false;
  return vnew;
}

// Shockley junction with the cubic reverse tail (device/diode.go:148-162,
// device/bjt.go:272-283) in FP32.
__device__ __forceinline__ void junction32(float is, float v, float nvt, float rnvt, float* i, float* g) {
  if (is == 0) { *i = 0; *g = 0; return; }
  if (v >= -3 * nvt) {
    float e = __expf(fminf(v * rnvt, kExpClamp32));
    *i = is * (e - 1); *g = is * e * rnvt; return;
  }
  float a = 3 * nvt / (v * (float)kE); a = a * a * a;
  *i = -is * (1 + a); *g = is * 3 * a / v;
}

// ---------------------------------------------------------------- diode (OP)
template <class SY>
__device__ __forceinline__ void diode_load32(const KElem& e, const Col32& V, const Col32& D, const Col32& S, SY& s,
                                             bool initJct, float gmin) {
  const int p = e.param, dd = e.derived, a = e.u[0], k = e.u[1], ai = e.u[2];
  const bool hasBV = e.flags & KS_F_HAS_BV;
  const float vte = D[dd + DD_VTE], rvte = D[dd + DD_RVTE], vcrit = D[dd + DD_VCRIT], xbv = D[dd + DD_XBV];
  float vd;
  bool lim;
  if (initJct) { vd = vcrit; lim = true; }
  else {
    float vraw = xo32_(s, ai) - xo32_(s, k), vacc = S[SD_VDACC];
    vd = pnjlim32(vraw, vacc, vte, rvte, vcrit, &lim);
    if (hasBV && vraw < fminf(0.0f, -xbv + 10 * vte)) {
      bool l2;
      float vt = pnjlim32(-(vraw + xbv), -(vacc + xbv), vte, rvte, vcrit, &l2);
      vd = -(vt + xbv); lim = l2;
    }
  }
  S[SD_VDACC] = vd;
  S[SD_LIM] = lim ? 1.0f : 0.0f;
  const float IS = V[p + KS_D_P_IS];
  float id, g;
  if (vd >= -3 * vte) { float ex = __expf(fminf(vd * rvte, kExpClamp32)); id = IS * (ex - 1); g = IS * ex * rvte; }
  else if (!hasBV || vd >= -xbv) { float t = 3 * vte / (vd * (float)kE); t = t * t * t; id = -IS * (1 + t); g = IS * 3 * t / vd; }
  else { float ex = __expf(fminf(-(xbv + vd) * rvte, kExpClamp32)); id = -IS * ex; g = IS * ex * rvte; }
  const float gg = g + gmin, ieq = id + gmin * vd - gg * vd;
  sadd32(s, ai, ai, gg); sadd32(s, k, k, gg); sadd32(s, ai, k, -gg); sadd32(s, k, ai, -gg);
  srhs32(s, ai, -ieq); srhs32(s, k, ieq);
  const float grs = D[dd + DD_GRS];
  if (grs > 0) { sadd32(s, a, a, grs); sadd32(s, ai, ai, grs); sadd32(s, a, ai, -grs); sadd32(s, ai, a, -grs); }
}

// ---------------------------------------------------------------- BJT (OP)
template <class SY>
__device__ __forceinline__ void bjt_branch32(SY& s, float typ, int a, int b, float i0, float g1, int p1, int n1,
                                             float v10, float g2, int p2, int n2, float v20) {
  if (g1 != 0) { sadd32(s, a, p1, g1); sadd32(s, a, n1, -g1); sadd32(s, b, p1, -g1); sadd32(s, b, n1, g1); }
  if (g2 != 0) { sadd32(s, a, p2, g2); sadd32(s, a, n2, -g2); sadd32(s, b, p2, -g2); sadd32(s, b, n2, g2); }
  const float ieq = typ * (i0 - g1 * v10 - g2 * v20);
  srhs32(s, a, -ieq); srhs32(s, b, ieq);
}
template <class SY>
__device__ __forceinline__ void stamp_g32(SY& s, int a, int b, float g) {
  if (g == 0) return;
  sadd32(s, a, a, g); sadd32(s, b, b, g); sadd32(s, a, b, -g); sadd32(s, b, a, -g);
}

// Gummel-Poon DC currents (device/bjt.go:294-354) and stamps (:422-515), FP32.
template <class SY>
__device__ __forceinline__ void bjt_load32(const KElem& e, const Col32& V, const Col32& D, const Col32& S, SY& s,
                                           bool initJct, float gmin) {
  const int p = e.param, dd = e.derived;
  const float typ = (e.flags & KS_F_PTYPE) ? -1.0f : 1.0f;
  const float vt = D[dd + DQ_VT], vcrit = D[dd + DQ_VCRIT], rvt = D[dd + DQ_RVT];
  float vbe, vbc, vcs;
  if (initJct) { vbe = vcrit; vbc = 0; vcs = 0; S[SQ_LIM] = 1.0f; }
  else {
    const float vbp = xo32_(s, e.u[5]), vcp = xo32_(s, e.u[4]), vep = xo32_(s, e.u[6]);
    vbe = typ * (vbp - vep); vbc = typ * (vbp - vcp); vcs = typ * (xo32_(s, e.u[7]) - xo32_(s, e.u[8]));
    bool l1, l2;
    vbe = pnjlim32(vbe, S[SQ_VBEACC], vt, rvt, vcrit, &l1);
    vbc = pnjlim32(vbc, S[SQ_VBCACC], vt, rvt, vcrit, &l2);
    S[SQ_LIM] = (l1 || l2) ? 1.0f : 0.0f;
  }
  S[SQ_VBEACC] = vbe; S[SQ_VBCACC] = vbc;
  float cbe, gbe, cbc, gbc, cben, gben, cbcn, gbcn;
  junction32(V[p + KS_Q_P_IS], vbe, V[p + KS_Q_P_NF] * vt, D[dd + DQ_RNF], &cbe, &gbe);
  junction32(V[p + KS_Q_P_ISE], vbe, V[p + KS_Q_P_NE] * vt, D[dd + DQ_RNE], &cben, &gben);
  cben += gmin * vbe; gben += gmin;
  junction32(V[p + KS_Q_P_IS], vbc, V[p + KS_Q_P_NR] * vt, D[dd + DQ_RNR], &cbc, &gbc);
  junction32(V[p + KS_Q_P_ISC], vbc, V[p + KS_Q_P_NC] * vt, D[dd + DQ_RNC], &cbcn, &gbcn);
  cbcn += gmin * vbc; gbcn += gmin;
  const float ivaf = D[dd + DQ_IVAF], ivar = D[dd + DQ_IVAR], oik = D[dd + DQ_OIK], oikr = D[dd + DQ_OIKR];
  const float q1 = 1 / (1 - ivaf * vbc - ivar * vbe);
  float qb, dqbdve, dqbdvc;
  if (oik == 0 && oikr == 0) { qb = q1; dqbdve = q1 * qb * ivar; dqbdvc = q1 * qb * ivaf; }
  else {
    const float q2 = oik * cbe + oikr * cbc, arg = fmaxf(0.0f, 1 + 4 * q2);
    const float sq = arg != 0 ? sqrtf(arg) : 1.0f, rsq = 1 / sq;
    qb = q1 * (1 + sq) / 2;
    dqbdve = q1 * (qb * ivar + oik * gbe * rsq);
    dqbdvc = q1 * (qb * ivaf + oikr * gbc * rsq);
  }
  const float rqb = 1 / qb;
  const float it = (cbe - cbc) * rqb;
  const float itBE = (gbe - it * dqbdve) * rqb, itBC = (-gbc - it * dqbdvc) * rqb;
  const float rBF = D[dd + DQ_RBF], rBR = D[dd + DQ_RBR];
  const float ibe = cbe * rBF + cben, gpi = gbe * rBF + gben, ibc = cbc * rBR + cbcn, gmu = gbc * rBR + gbcn;
  const float rbpr = D[dd + DQ_RBPR], rbpi = D[dd + DQ_RBPI];
  float gx = rbpr + rbpi * rqb;
  const float IRB = V[p + KS_Q_P_IRB];
  if (IRB > 0 && rbpi != 0) {
    const float a1 = fmaxf((ibe + ibc) / IRB, 1e-9f);
    const float z = (-1 + sqrtf(1 + 14.59025f * a1)) / 2.4317f / sqrtf(a1), tz = tanf(z);
    gx = rbpr + 3 * rbpi * (tz - z) / z / tz / tz;
  }
  gx = gx != 0 ? 1 / gx : 0;
  float isub, gsub;
  junction32(V[p + KS_Q_P_ISS], vcs, V[p + KS_Q_P_NS] * vt, D[dd + DQ_RNS], &isub, &gsub);
  isub += gmin * vcs; gsub += gmin;
  const int b = e.u[2], cp = e.u[4], bp = e.u[5], ep = e.u[6], sa = e.u[7], sb = e.u[8];
  bjt_branch32(s, typ, cp, ep, it, itBE, bp, ep, vbe, itBC, bp, cp, vbc);
  bjt_branch32(s, typ, bp, ep, ibe, gpi, bp, ep, vbe, 0, 0, 0, 0);
  bjt_branch32(s, typ, bp, cp, ibc, gmu, bp, cp, vbc, 0, 0, 0, 0);
  bjt_branch32(s, typ, sa, sb, isub, gsub, sa, sb, vcs, 0, 0, 0, 0);
  if (bp != b) stamp_g32(s, b, bp, gx);
  if (cp != e.u[0]) stamp_g32(s, e.u[0], cp, D[dd + DQ_GCPR]);
  if (ep != e.u[1]) stamp_g32(s, e.u[1], ep, D[dd + DQ_GEPR]);
}

// ---------------------------------------------------------------- MOSFET level 1 (OP)
__device__ __forceinline__ float fetlim32(float vnew, float vold, float vto) {  // device/mosfet.go:347-385
  const float vtsthi = fabsf(2 * (vold - vto)) + 2, vtstlo = vtsthi / 2 + 2, vtox = vto + 3.5f, delv = vnew - vold;
  if (vold >= vto) {
    if (vold >= vtox) {
      if (delv <= 0) {
        if (vnew >= vtox) { if (-delv > vtstlo) vnew = vold - vtstlo; }
        else vnew = fmaxf(vnew, vto + 2);
      } else if (delv >= vtsthi) vnew = vold + vtsthi;
    } else if (delv <= 0) vnew = fmaxf(vnew, vto - 0.5f);
    else vnew = fminf(vnew, vto + 4);
  } else if (delv <= 0) {
    if (-delv > vtsthi) vnew = vold - vtsthi;
  } else {
    const float vtemp = vto + 0.5f;
    if (vnew <= vtemp) { if (delv > vtstlo) vnew = vold + vtstlo; }
    else vnew = vtemp;
  }
  return vnew;
}
__device__ __forceinline__ float limvds32(float vnew, float vold) {  // device/mosfet.go:388-402
  if (vold >= 3.5f) {
    if (vnew > vold) return fminf(vnew, 3 * vold + 2);
    if (vnew < 3.5f) return fmaxf(vnew, 2.0f);
    return vnew;
  }
  if (vnew > vold) return fminf(vnew, 4.0f);
  return fmaxf(vnew, -0.5f);
}
// idsLevel1 (device/mosfet_levels.go:79-113) in FP32: o = {cdrain, gm, gds, gmbs, von}
__device__ __forceinline__ void ids_level1_32(const Col32& D, int d, float lambda, float vgs, float vds, float vbs,
                                              float* o) {
  const float PHI = D[d + DM_PHI], GAMMA = D[d + DM_GAMMA], beta = D[d + DM_BETA];
  float sarg;
  if (vbs <= 0) sarg = sqrtf(PHI - vbs);
  else { sarg = sqrtf(PHI); sarg = fmaxf(0.0f, sarg - vbs / (sarg + sarg)); }
  const float von = D[d + DM_VBI] + GAMMA * sarg, vgst = vgs - von;
  o[4] = von;
  const float arg = sarg > 0 ? GAMMA / (sarg + sarg) : 0.0f;
  if (vgst <= 0) { o[0] = o[1] = o[2] = o[3] = 0; return; }
  const float betap = beta * (1 + lambda * vds);
  if (vgst <= vds) {
    o[0] = betap * vgst * vgst * 0.5f; o[1] = betap * vgst; o[2] = lambda * beta * vgst * vgst * 0.5f;
  } else {
    o[0] = betap * vds * (vgst - 0.5f * vds); o[1] = betap * vds;
    o[2] = betap * (vgst - vds) + lambda * beta * vds * (vgst - 0.5f * vds);
  }
  o[3] = o[1] * arg;
}
// channel (device/mosfet.go:464-473): o = {mode, cdrain, gm, gds, gmbs, von}
__device__ __forceinline__ void mos_channel32(const KElem& e, const Col32& V, const Col32& D, float vgs, float vds,
                                              float vbs, float* o) {
  float md = 1, vg = vgs, vd = vds, vb = vbs;
  if (vds < 0) { md = -1; vg = vgs - vds; vd = -vds; vb = vbs - vds; }
  o[0] = md;
  ids_level1_32(D, e.derived, V[e.param + KS_M_P_LAMBDA], vg, vd, vb, o + 1);
}
__device__ __forceinline__ void mos_bulk32(float v, float is, float vt, float rvt, float gmin, float* i, float* g) {
  if (v <= -3 * vt) { *i = gmin * v - is; *g = gmin; return; }
  const float ex = __expf(fminf(v * rvt, kExpClamp32));
  *i = is * (ex - 1) + gmin * v; *g = is * ex * rvt + gmin;
}
template <bool NEW, class SY>
__device__ __forceinline__ void mos_voltages32(const KElem& e, SY& s, float* vgs, float* vds, float* vbs) {
  auto X = [&](int i) { return NEW ? xn32_(s, i) : xo32_(s, i); };
  const float t = (e.flags & KS_F_PTYPE) ? -1.0f : 1.0f;
  const float vg = X(e.u[2]), vb = X(e.u[3]), vdp = X(e.u[4]), vsp = X(e.u[5]);
  *vgs = t * (vg - vsp); *vds = t * (vdp - vsp); *vbs = t * (vb - vsp);
}
template <class SY>
__device__ __forceinline__ void mos_branch32(SY& s, float typ, int a, int b, float i0, float g, int pk, int mk, float v0) {
  float ieq = i0;
  if (g != 0) {
    sadd32(s, a, pk, g); sadd32(s, a, mk, -g); sadd32(s, b, pk, -g); sadd32(s, b, mk, g);
    ieq -= g * v0;
  }
  ieq *= typ;
  srhs32(s, a, -ieq); srhs32(s, b, ieq);
}
// Load + stamp of a level-1 MOSFET at DC (device/mosfet.go:476-611), FP32.
template <class SY>
__device__ __forceinline__ void mos_load32(const KElem& e, const Col32& V, const Col32& D, const Col32& S, SY& s,
                                           bool initJct, float gmin) {
  const int d = e.derived;
  const float vt = D[d + DM_VT], rvt = D[d + DM_RVT];
  float vgs, vds, vbs;
  mos_voltages32<false>(e, s, &vgs, &vds, &vbs);
  bool lim = false;
  if (initJct) { vbs = -1; vgs = D[d + DM_VTO]; vds = 0; lim = true; }
  else {
    const float avgs = S[SM_AVGS], avds = S[SM_AVDS], avbs = S[SM_AVBS], von = S[SM_AVON];
    float vgd = vgs - vds;
    const float vgdOld = avgs - avds;
    if (avds >= 0) {
      vgs = fetlim32(vgs, avgs, von);
      vds = vgs - vgd;
      vds = limvds32(vds, avds);
    } else {
      vgd = fetlim32(vgd, vgdOld, von);
      vds = vgs - vgd;
      vds = -limvds32(-vds, -avds);
      vgs = vgd + vds;
    }
    if (vds >= 0) vbs = pnjlim32(vbs, avbs, vt, rvt, D[d + DM_VCRITS], &lim);
    else {
      const float vbd = pnjlim32(vbs - vds, avbs - avds, vt, rvt, D[d + DM_VCRITD], &lim);
      vbs = vbd + vds;
    }
  }
  const float vbd = vbs - vds;
  S[SM_AVGS] = vgs; S[SM_AVDS] = vds; S[SM_AVBS] = vbs;
  float cbs, gbs, cbd, gbd;
  mos_bulk32(vbs, D[d + DM_ISS], vt, rvt, gmin, &cbs, &gbs);
  mos_bulk32(vbd, D[d + DM_ISD], vt, rvt, gmin, &cbd, &gbd);
  float o[6];
  mos_channel32(e, V, D, vgs, vds, vbs, o);
  S[SM_AVON] = o[5];
  S[SM_LIM] = lim ? 1.0f : 0.0f;
  const float typ = (e.flags & KS_F_PTYPE) ? -1.0f : 1.0f;
  const int g = e.u[2], b = e.u[3], dp = e.u[4], sp = e.u[5];
  float i0 = o[1], g0 = o[2], g1 = o[3], g2 = o[4];
  if (o[0] <= 0) { i0 = -o[1]; g0 = -o[2]; g1 = o[2] + o[3] + o[4]; g2 = -o[4]; }
  float ieq = i0;
  if (g0 != 0) { sadd32(s, dp, g, g0); sadd32(s, dp, sp, -g0); sadd32(s, sp, g, -g0); sadd32(s, sp, sp, g0); ieq -= g0 * vgs; }
  if (g1 != 0) { sadd32(s, dp, dp, g1); sadd32(s, dp, sp, -g1); sadd32(s, sp, dp, -g1); sadd32(s, sp, sp, g1); ieq -= g1 * vds; }
  if (g2 != 0) { sadd32(s, dp, b, g2); sadd32(s, dp, sp, -g2); sadd32(s, sp, b, -g2); sadd32(s, sp, sp, g2); ieq -= g2 * vbs; }
  ieq *= typ;
  srhs32(s, dp, -ieq); srhs32(s, sp, ieq);
  mos_branch32(s, typ, b, sp, cbs, gbs, b, sp, vbs);
  mos_branch32(s, typ, b, dp, cbd, gbd, b, dp, vbd);
  if (dp != e.u[0]) stamp_g32(s, e.u[0], dp, D[d + DM_GDPR]);
  if (sp != e.u[1]) stamp_g32(s, e.u[1], sp, D[d + DM_GSPR]);
}

// ---------------------------------------------------------------- element dispatch
__device__ __forceinline__ bool elem_ok32(const KElem& e) {
  return e.kind <= KS_ELEM_M && (e.kind != KS_ELEM_M || e.level == 1);
}

template <class SY>
__device__ __forceinline__ void elem_load32(const KElem& e, const Col32& V, const Col32& D, const Col32& Sb, SY& s,
                                            bool initJct, float gmin, float srcFact) {
  const Col32 S{Sb.p + (int64_t)e.state * Sb.B, Sb.B};
  switch (e.kind) {
    case KS_ELEM_R: {
      const float g = D[e.derived + DR_G];
      const int a = e.u[0], b = e.u[1];
      sadd32(s, a, a, g); sadd32(s, b, b, g); sadd32(s, a, b, -g); sadd32(s, b, a, -g);
      break;
    }
    case KS_ELEM_L: {  // DC: the branch row ties the node voltages
      const int a = e.u[0], b = e.u[1], kk = e.u[2];
      sadd32(s, a, kk, 1); sadd32(s, b, kk, -1); sadd32(s, kk, a, 1); sadd32(s, kk, b, -1);
      break;
    }
    case KS_ELEM_V: {
      const int a = e.u[0], b = e.u[1], kk = e.u[2];
      sadd32(s, a, kk, 1); sadd32(s, b, kk, -1); sadd32(s, kk, a, 1); sadd32(s, kk, b, -1);
      srhs32(s, kk, S[SV_VALUE] * srcFact);
      break;
    }
    case KS_ELEM_I: {
      const float v = S[SV_VALUE] * srcFact;
      srhs32(s, e.u[0], -v); srhs32(s, e.u[1], v);
      break;
    }
    case KS_ELEM_D: diode_load32(e, V, D, S, s, initJct, gmin); break;
    case KS_ELEM_Q: bjt_load32(e, V, D, S, s, initJct, gmin); break;
    case KS_ELEM_M: mos_load32(e, V, D, S, s, initJct, gmin); break;
    default: break;  // capacitors are open at DC
  }
}

// Limiting state at a given point (the part of Accept the next load reads).
template <class SY>
__device__ __forceinline__ void elem_seed32(const KElem& e, const Col32& V, const Col32& D, const Col32& Sb, SY& s) {
  const Col32 S{Sb.p + (int64_t)e.state * Sb.B, Sb.B};
  if (e.kind == KS_ELEM_D) S[SD_VDACC] = xn32_(s, e.u[2]) - xn32_(s, e.u[1]);
  else if (e.kind == KS_ELEM_Q) {
    const float typ = (e.flags & KS_F_PTYPE) ? -1.0f : 1.0f, vbp = xn32_(s, e.u[5]);
    S[SQ_VBEACC] = typ * (vbp - xn32_(s, e.u[6]));
    S[SQ_VBCACC] = typ * (vbp - xn32_(s, e.u[4]));
  } else if (e.kind == KS_ELEM_M) {
    float vgs, vds, vbs, o[6];
    mos_voltages32<true>(e, s, &vgs, &vds, &vbs);
    mos_channel32(e, V, D, vgs, vds, vbs, o);
    S[SM_AVGS] = vgs; S[SM_AVDS] = vds; S[SM_AVBS] = vbs; S[SM_AVON] = o[5];
  }
}

// Dense FP32 LU with partial pivoting of a32, x32 = a32^-1 r32.
template <class SY>
__device__ __forceinline__ int lu_solve_f32(SY& s) {
  const int n = s.size();
#pragma unroll (SY::kUnroll)
  for (int k = 0; k < n; k++) {
    int p = k;
    float maxv = fabsf(s.a32(k, k));
#pragma unroll (SY::kUnroll)
    for (int i = k + 1; i < n; i++) {
      const float v = fabsf(s.a32(i, k));
      if (v > maxv) { maxv = v; p = i; }
    }
    if (!(maxv > 0.0f) || ks_exp32(maxv) >= 255) return SOLVE_SINGULAR;
    if constexpr (SY::kStatic) {
#pragma unroll (SY::kUnroll)
      for (int i = 0; i < n; i++)
        if (i > k && i == p) {
#pragma unroll (SY::kUnroll)
          for (int j = 0; j < n; j++) { float t = s.a32(k, j); s.a32(k, j) = s.a32(i, j); s.a32(i, j) = t; }
          float t = s.r32(k); s.r32(k) = s.r32(i); s.r32(i) = t;
        }
    } else if (p != k) {
      for (int j = 0; j < n; j++) { float t = s.a32(k, j); s.a32(k, j) = s.a32(p, j); s.a32(p, j) = t; }
      float t = s.r32(k); s.r32(k) = s.r32(p); s.r32(p) = t;
    }
    const float rp = 1.0f / s.a32(k, k);
#pragma unroll (SY::kUnroll)
    for (int i = k + 1; i < n; i++) {
      const float f = s.a32(i, k) * rp;
#pragma unroll (SY::kUnroll)
      for (int j = k + 1; j < n; j++) s.a32(i, j) = fmaf(-f, s.a32(k, j), s.a32(i, j));
      s.r32(i) = fmaf(-f, s.r32(k), s.r32(i));
    }
    s.a32(k, k) = rp;
  }
  int ex = 0;
#pragma unroll (SY::kUnroll)
  for (int i = n - 1; i >= 0; i--) {
    float acc = s.r32(i);
#pragma unroll (SY::kUnroll)
    for (int j = i + 1; j < n; j++) acc = fmaf(-s.a32(i, j), s.x32(j), acc);
    s.x32(i) = acc * s.a32(i, i);
    ex = max(ex, ks_exp32(s.x32(i)));
  }
  return ex >= 255 ? SOLVE_NONFINITE : SOLVE_OK;
}

// One FP32 Newton run from the thread's x32 (initJct: the first load at the
// junction starting voltages), with conductance g added on every voltage row
// (gmin stepping) and the sources scaled by srcFact (source stepping), for at
// most itMax iterations; *used counts them.  0: converged, 1: not converged,
// 2: singular or non-finite.  The stage solves for x itself in FP32, so its step
// does not fall below the FP32 resolution of the system (about cond(A) * 2^-24
// of x, more where a saturated transistor's collector current is the difference
// of two junction currents).  Convergence: no device limited and the largest
// node-voltage step, relative to the node's magnitude + 1 V, below 1e-5 (the
// FP64 Newton then converges in about two iterations), or a step that stops
// halving while below 1e-3 (the FP32 floor).  Branch currents follow the node
// voltages and are left to the FP64 solve.
template <class TH>
__device__ __forceinline__ int newton32(TH& t, const Col32& V, const Col32& D, const Col32& Sb, bool initJct, float g,
                                        float srcFact, int itMax, int* used) {
  typedef decltype(t.s) SY;
  typedef decltype(t.prog) P;
  SY& s = t.s;
  const int n = t.n();
  const float gmin = (float)t.o.gmin;
  float prev = 3.0e38f;
  for (int it = 0; it < itMax; it++) {
    ++*used;
#pragma unroll
    for (int i = 0; i < n; i++) {
      s.xo32(i) = s.x32(i);
#pragma unroll
      for (int j = 0; j < n; j++) s.a32(i, j) = 0.0f;
      s.r32(i) = 0.0f;
    }
    t.prog.each([&](const KElem& e) KS_INLINE_LAMBDA { elem_load32(e, V, D, Sb, s, initJct, gmin, srcFact); });
    if (g > 0) {
#pragma unroll
      for (int i = 0; i < n; i++) if (t.prog.is_v(i)) s.a32(i, i) += g;
    }
    int err = SOLVE_STATIC_FAIL;
    if constexpr (P::kStaticLU) err = t.prog.lu_f32(s);
    if (err == SOLVE_STATIC_FAIL) err = lu_solve_f32(s);
    if (err) return 2;
    if (initJct) { initJct = false; continue; }
    bool lim = false;
    t.prog.each([&](const KElem& e) KS_INLINE_LAMBDA {
      const int ls = lim_slot(e.kind);
      if (ls >= 0 && Sb[e.state + ls] != 0) lim = true;
    });
    if (lim) { prev = 3.0e38f; continue; }
    float dv = 0.0f;
#pragma unroll
    for (int i = 0; i < n; i++) {
      if (!t.prog.is_v(i)) continue;
      const float x = s.x32(i), old = s.xo32(i);
      dv = fmaxf(dv, fabsf(x - old) / (1.0f + fmaxf(fabsf(x), fabsf(old))));
    }
    if (dv <= 1e-5f || (dv <= 1e-3f && dv > 0.5f * prev)) return 0;
    prev = dv;
  }
  return 1;
}

// The FP32 stage for circuit c: x0 is the start's node voltages ([B][n], null:
// InitJct).  The stage follows dcSolve's own chain (analysis/newton.go:95-214)
// in FP32: Newton from the start (from a given start that fails, Newton from
// InitJct next); if that fails, gmin stepping from zero with the reference's
// schedule (g from 1e-2 down to gmin, the step factor growing after each
// success and shrinking after each failure); if that fails, source stepping.
// All of it within maxIt FP32 iterations.  On success the thread's FP64 iterate
// s.xn() holds the stage's point and the result is true; otherwise s.xn() is
// left undefined (the caller sets its start again).  The FP32 state columns are
// this stage's own.
template <class TH>
__device__ __forceinline__ bool start32(TH& t, const K32& k32, const double* x0, int64_t c, int64_t B, int maxIt) {
  typedef decltype(t.s) SY;
  bool ok = true;
  t.prog.each([&](const KElem& e) KS_INLINE_LAMBDA { ok = ok && elem_ok32(e); });
  if (!ok) return false;
  SY& s = t.s;
  const int n = t.n();
  const Col32 V{const_cast<float*>(k32.values) + c, B}, D{const_cast<float*>(k32.derived) + c, B};
  const Col32 Sb{k32.state + c, B};
  // source values (DC, or the waveform at t = 0) once, in FP64
  LoadParams lp;
  lp.mode = ModeOP; lp.method = BE; lp.time = 0; lp.h = 0; lp.rh = 0; lp.initJct = false; lp.gmin = t.o.gmin;
  lp.srcStepping = false; lp.srcFact = 0;
  t.prog.each([&](const KElem& e) KS_INLINE_LAMBDA {
    if (e.kind == KS_ELEM_V || e.kind == KS_ELEM_I)
      Sb[e.state + SV_VALUE] = (float)source_at(e, t.V, t.D, state_col(t.Sb, e), lp);
  });
  const int itl = t.o.itl1;
  int used = 0;
#pragma unroll
  for (int i = 0; i < n; i++) s.x32(i) = (x0 && i < t.prog.n_nodes - 1) ? (float)x0[c * n + i] : 0.0f;
  if (x0) t.prog.each([&](const KElem& e) KS_INLINE_LAMBDA { elem_seed32(e, V, D, Sb, s); });
  int res = newton32(t, V, D, Sb, x0 == nullptr, 0.0f, 1.0f, min(itl, maxIt), &used);
  if (res != 0 && x0) {  // a given start that fails: Newton from InitJct before the stepping
#pragma unroll
    for (int i = 0; i < n; i++) s.x32(i) = 0.0f;
    res = newton32(t, V, D, Sb, true, 0.0f, 1.0f, min(itl, maxIt - used), &used);
  }
  if (res != 0 && !t.o.no_gmin) {  // gmin stepping, analysis/newton.go:134-176
    const float gmin = (float)t.o.gmin;
#pragma unroll
    for (int i = 0; i < n; i++) { s.x32(i) = 0.0f; s.sv32(i) = 0.0f; }
    float g = 1e-2f, factor = 10.0f;
    bool stepped = false, initJct = true;
    for (int k = 0; k < 200 && used < maxIt; k++) {
      res = newton32(t, V, D, Sb, initJct, g, 1.0f, min(itl, maxIt - used), &used);
      initJct = false;
      if (res == 0) {
#pragma unroll
        for (int i = 0; i < n; i++) s.sv32(i) = s.x32(i);
        if (g == 0) break;
        stepped = true;
        factor = fminf(factor * sqrtf(factor), 10.0f);
        g = g / factor < gmin ? 0.0f : g / factor;
        res = 1;
      } else {
        if (!stepped) break;
#pragma unroll
        for (int i = 0; i < n; i++) s.x32(i) = s.sv32(i);
        const float prevg = g == 0 ? gmin : g * factor;
        factor = sqrtf(factor);
        if (factor < 1.00005f) break;
        g = prevg / factor;
        res = 1;
      }
    }
  }
  if (res != 0 && !t.o.no_source) {  // source stepping, analysis/newton.go:180-214
#pragma unroll
    for (int i = 0; i < n; i++) s.x32(i) = 0.0f;
    res = newton32(t, V, D, Sb, true, 0.0f, 0.0f, min(itl, maxIt - used), &used);
    if (res == 0) {
#pragma unroll
      for (int i = 0; i < n; i++) s.sv32(i) = s.x32(i);
      float done = 0.0f, step = 0.1f;
      res = 1;
      for (int k = 0; k < 1000 && used < maxIt; k++) {
        const float sf = fminf(done + step, 1.0f);
        const int r = newton32(t, V, D, Sb, false, 0.0f, sf, min(itl, maxIt - used), &used);
        if (r == 0) {
          if (sf == 1.0f) { res = 0; break; }
#pragma unroll
          for (int i = 0; i < n; i++) s.sv32(i) = s.x32(i);
          done = sf;
          step = fminf(step * 1.5f, 0.5f);
        } else {
#pragma unroll
          for (int i = 0; i < n; i++) s.x32(i) = s.sv32(i);
          step *= 0.5f;
          if (step < 1e-3f) break;
        }
      }
    }
  }
  if (res != 0) return false;
#pragma unroll
  for (int i = 0; i < n; i++) s.xn(i) = (double)s.x32(i);
  return true;
}

}  // namespace ksg
