// oracle_bjt.hpp — CPU FP64 Gummel-Poon BJT of the oracle (test infrastructure).
// Restates device/bjt.go (SPICE3 Gummel-Poon, ngspice substrate junction).
#pragma once
#include "oracle_devices.hpp"

namespace kso {

struct BJT : Device {
  // parameters (device/bjt.go:17-30), block KS_Q_P_*
  double IS, BF, NF, VAF, IKF, ISE, NE, BR, NR, VAR, IKR, ISC, NC, RB, IRB, RBM, RE, RC;
  double CJE, VJE, MJE, TF, XTF, VTF, ITF, CJC, VJC, MJC, XCJC, TR, CJS, VJS, MJS, FC, ISS, NS, SUBS, Type;
  double vt, vcrit, rbpr, rbpi, gcpr = 0, gepr = 0, ovtf = 0;
  double f1e, f2e, f3e, f1c, f2c, f3c;
  int nc, ne, nb, ns;  // circuit nodes
  int uc, ue, b, s, cp, bp, ep, sa, sb;
  double isub = 0, gsub = 0;
  double vbe = 0, vbc = 0, vbx = 0, vcs = 0;
  struct DC { double cbe, gbe, cbc, gbc, it, itBE, itBC, ibe, gpi, ibc, gmu, qb, dqbdve, dqbdvc, gx; } dc{};
  struct Ch { double q[4], c[4], dqbeDvbc; } ch{};
  double ag = 0, iq[4] = {0, 0, 0, 0};
  bool lim = false, tran = false;
  double gmin = 1e-12;
  double vbeAcc = 0, vbcAcc = 0, vbxAcc = 0, vcsAcc = 0;
  double qPrev[4] = {0, 0, 0, 0}, iqPrev[4] = {0, 0, 0, 0};
  History hist[4];
  bool hasCharge;

  BJT(const double* p, bool pnp, int c_, int e_, int b_, int s_) {
    IS = p[KS_Q_P_IS]; BF = p[KS_Q_P_BF]; NF = p[KS_Q_P_NF]; VAF = p[KS_Q_P_VAF]; IKF = p[KS_Q_P_IKF];
    ISE = p[KS_Q_P_ISE]; NE = p[KS_Q_P_NE]; BR = p[KS_Q_P_BR]; NR = p[KS_Q_P_NR]; VAR = p[KS_Q_P_VAR];
    IKR = p[KS_Q_P_IKR]; ISC = p[KS_Q_P_ISC]; NC = p[KS_Q_P_NC]; RB = p[KS_Q_P_RB]; IRB = p[KS_Q_P_IRB];
    RBM = p[KS_Q_P_RBM]; RE = p[KS_Q_P_RE]; RC = p[KS_Q_P_RC]; CJE = p[KS_Q_P_CJE]; VJE = p[KS_Q_P_VJE];
    MJE = p[KS_Q_P_MJE]; TF = p[KS_Q_P_TF]; XTF = p[KS_Q_P_XTF]; VTF = p[KS_Q_P_VTF]; ITF = p[KS_Q_P_ITF];
    CJC = p[KS_Q_P_CJC]; VJC = p[KS_Q_P_VJC]; MJC = p[KS_Q_P_MJC]; XCJC = p[KS_Q_P_XCJC]; TR = p[KS_Q_P_TR];
    CJS = p[KS_Q_P_CJS]; VJS = p[KS_Q_P_VJS]; MJS = p[KS_Q_P_MJS]; FC = p[KS_Q_P_FC]; ISS = p[KS_Q_P_ISS];
    NS = p[KS_Q_P_NS]; SUBS = p[KS_Q_P_SUBS]; Type = pnp ? -1 : 1;
    nc = c_; ne = e_; nb = b_; ns = s_;
    vt = kBoltzmann * kTNom / kChargeQ;                 // :223
    vcrit = vt * std::log(vt / (kSqrt2 * IS));          // :224
    rbpr = RBM; rbpi = RB - RBM;
    if (RC > 0) gcpr = 1 / RC;
    if (RE > 0) gepr = 1 / RE;
    if (VTF > 0) ovtf = 1 / (1.44 * VTF);
    deplF(VJE, MJE, FC, &f1e, &f2e, &f3e);
    deplF(VJC, MJC, FC, &f1c, &f2c, &f3c);
    hasCharge = CJE > 0 || CJC > 0 || CJS > 0 || TF > 0 || TR > 0;
  }
  void setup(SetupCtx& c) override {  // :250-268
    uc = c.unknown(nc); ue = c.unknown(ne);
    b = c.unknown(nb); s = c.unknown(ns);
    cp = uc; bp = b; ep = ue;
    if (RC > 0) cp = c.allocUnknown();
    if (RB > 0) bp = c.allocUnknown();
    if (RE > 0) ep = c.allocUnknown();
    sa = s; sb = cp;
    if (SUBS < 0) { sa = bp; sb = s; }
  }
  bool nonlinear() const override { return true; }
  bool reactive() const override { return true; }
  bool limited() const override { return lim; }

  void substrate(double v, double* i, double* g) const {  // :288-291
    junction(ISS, v, NS * vt, i, g);
    *i += gmin * v; *g += gmin;
  }
  DC evalDC(double vbe_, double vbc_) const {  // :294-354
    DC d{};
    junction(IS, vbe_, NF * vt, &d.cbe, &d.gbe);
    double cben, gben; junction(ISE, vbe_, NE * vt, &cben, &gben);
    cben += gmin * vbe_; gben += gmin;
    junction(IS, vbc_, NR * vt, &d.cbc, &d.gbc);
    double cbcn, gbcn; junction(ISC, vbc_, NC * vt, &cbcn, &gbcn);
    cbcn += gmin * vbc_; gbcn += gmin;
    double ivaf = 0, ivar = 0, oik = 0, oikr = 0;
    if (VAF > 0) ivaf = 1 / VAF;
    if (VAR > 0) ivar = 1 / VAR;
    if (IKF > 0) oik = 1 / IKF;
    if (IKR > 0) oikr = 1 / IKR;
    double q1 = 1 / (1 - ivaf * vbc_ - ivar * vbe_);
    if (oik == 0 && oikr == 0) {
      d.qb = q1; d.dqbdve = q1 * d.qb * ivar; d.dqbdvc = q1 * d.qb * ivaf;
    } else {
      double q2 = oik * d.cbe + oikr * d.cbc;
      double arg = std::max(0.0, 1 + 4 * q2);
      double sq = 1.0;
      if (arg != 0) sq = std::sqrt(arg);
      d.qb = q1 * (1 + sq) / 2;
      d.dqbdve = q1 * (d.qb * ivar + oik * d.gbe / sq);
      d.dqbdvc = q1 * (d.qb * ivaf + oikr * d.gbc / sq);
    }
    d.it = (d.cbe - d.cbc) / d.qb;
    d.itBE = (d.gbe - d.it * d.dqbdve) / d.qb;
    d.itBC = (-d.gbc - d.it * d.dqbdvc) / d.qb;
    d.ibe = d.cbe / BF + cben; d.gpi = d.gbe / BF + gben;
    d.ibc = d.cbc / BR + cbcn; d.gmu = d.gbc / BR + gbcn;
    double gx = rbpr + rbpi / d.qb;
    if (IRB > 0 && rbpi != 0) {
      double cb = d.ibe + d.ibc;
      double a1 = std::max(cb / IRB, 1e-9);
      double z = (-1 + std::sqrt(1 + 14.59025 * a1)) / 2.4317 / std::sqrt(a1);
      double tz = std::tan(z);
      gx = rbpr + 3 * rbpi * (tz - z) / z / tz / tz;
    }
    if (gx != 0) gx = 1 / gx;
    d.gx = gx;
    return d;
  }
  Ch charges(double vbe_, double vbc_, double vbx_, double vcs_, const DC& d) const {  // :373-412
    Ch c{};
    double cbe = d.cbe, gbe = d.gbe;
    if (TF != 0 && vbe_ > 0) {
      double argtf = 0, arg2 = 0, arg3 = 0;
      if (XTF != 0) {
        argtf = XTF;
        if (ovtf != 0) argtf *= std::exp(vbc_ * ovtf);
        arg2 = argtf;
        if (ITF != 0) {
          double t = cbe / (cbe + ITF);
          argtf *= t * t;
          arg2 = argtf * (3 - t - t);
        }
        arg3 = cbe * argtf * ovtf;
      }
      cbe = cbe * (1 + argtf) / d.qb;
      gbe = (gbe * (1 + arg2) - cbe * d.dqbdve) / d.qb;
      c.dqbeDvbc = TF * (arg3 - cbe * d.dqbdvc) / d.qb;
    }
    double qd, cd;
    depletion(vbe_, CJE, VJE, MJE, FC, f1e, f2e, f3e, &qd, &cd);
    c.q[0] = TF * cbe + qd; c.c[0] = TF * gbe + cd;
    double czbc = CJC * XCJC;
    depletion(vbc_, czbc, VJC, MJC, FC, f1c, f2c, f3c, &qd, &cd);
    c.q[1] = TR * d.cbc + qd; c.c[1] = TR * d.gbc + cd;
    depletion(vbx_, CJC - czbc, VJC, MJC, FC, f1c, f2c, f3c, &c.q[2], &c.c[2]);
    if (CJS != 0) {
      double cz = CJS;
      if (vcs_ < 0) {
        double arg = 1 - vcs_ / VJS;
        double sarg = std::exp(-MJS * std::log(arg));
        c.q[3] = VJS * cz * (1 - arg * sarg) / (1 - MJS); c.c[3] = cz * sarg;
      } else {
        c.q[3] = vcs_ * cz * (1 + MJS * vcs_ / (2 * VJS)); c.c[3] = cz * (1 + MJS * vcs_ / VJS);
      }
    }
    return c;
  }
  void voltages(const double* x, double* vbe_, double* vbc_, double* vbx_, double* vcs_) const {  // :415-419
    double t = Type;
    double vb = at(x, n, b), vbp = at(x, n, bp), vcp = at(x, n, cp), vep = at(x, n, ep);
    *vbe_ = t * (vbp - vep); *vbc_ = t * (vbp - vcp); *vbx_ = t * (vb - vcp);
    *vcs_ = t * (at(x, n, sa) - at(x, n, sb));
  }
  void load(LoadCtx& c) override {  // :422-458
    gmin = c.gmin;
    double be, bc, bx, cs;
    voltages(c.X, &be, &bc, &bx, &cs);
    lim = false;
    if (c.initJct) { be = vcrit; bc = 0; lim = true; bx = 0; cs = 0; }
    else {
      bool l1, l2;
      be = pnjlim(be, vbeAcc, vt, vcrit, &l1);
      bc = pnjlim(bc, vbcAcc, vt, vcrit, &l2);
      lim = l1 || l2;
    }
    vbeAcc = be; vbcAcc = bc;
    vbe = be; vbc = bc; vbx = bx; vcs = cs;
    dc = evalDC(be, bc);
    substrate(cs, &isub, &gsub);
    tran = false; ag = 0;
    for (int k = 0; k < 4; k++) iq[k] = 0;
    if (c.mode == ModeTran && hasCharge) {
      ch = charges(be, bc, bx, cs, dc);
      tran = true;
      if (c.method == TRAP) {
        ag = 2 / c.h;
        for (int k = 0; k < 4; k++) iq[k] = ag * (ch.q[k] - qPrev[k]) - iqPrev[k];
      } else {
        ag = 1 / c.h;
        for (int k = 0; k < 4; k++) iq[k] = ag * (ch.q[k] - qPrev[k]);
      }
    }
    stamp(c);
  }
  void branch(LoadCtx& c, int a, int bb, double i0, double g1, int p1, int n1, double v10,
              double g2, int p2, int n2, double v20) {  // :463-480
    Matrix* m = c.M;
    if (g1 != 0) { m->add(a, p1, g1); m->add(a, n1, -g1); m->add(bb, p1, -g1); m->add(bb, n1, g1); }
    if (g2 != 0) { m->add(a, p2, g2); m->add(a, n2, -g2); m->add(bb, p2, -g2); m->add(bb, n2, g2); }
    double ieq = Type * (i0 - g1 * v10 - g2 * v20);
    c.addRHS(a, -ieq); c.addRHS(bb, ieq);
  }
  static void stampG(Matrix* m, int a, int bb, double g) {  // :482-490
    if (g == 0) return;
    m->add(a, a, g); m->add(bb, bb, g); m->add(a, bb, -g); m->add(bb, a, -g);
  }
  void stamp(LoadCtx& c) {  // :492-515
    const DC& d = dc;
    branch(c, cp, ep, d.it, d.itBE, bp, ep, vbe, d.itBC, bp, cp, vbc);
    branch(c, bp, ep, d.ibe, d.gpi, bp, ep, vbe, 0, 0, 0, 0);
    branch(c, bp, cp, d.ibc, d.gmu, bp, cp, vbc, 0, 0, 0, 0);
    branch(c, sa, sb, isub, gsub, sa, sb, vcs, 0, 0, 0, 0);
    if (tran) {
      branch(c, bp, ep, iq[0], ag * ch.c[0], bp, ep, vbe, ag * ch.dqbeDvbc, bp, cp, vbc);
      branch(c, bp, cp, iq[1], ag * ch.c[1], bp, cp, vbc, 0, 0, 0, 0);
      branch(c, b, cp, iq[2], ag * ch.c[2], b, cp, vbx, 0, 0, 0, 0);
      branch(c, sa, sb, iq[3], ag * ch.c[3], sa, sb, vcs, 0, 0, 0, 0);
    }
    if (bp != b) stampG(c.M, b, bp, d.gx);
    if (cp != uc) stampG(c.M, uc, cp, gcpr);
    if (ep != ue) stampG(c.M, ue, ep, gepr);
  }
  bool convTest(const double* x, double reltol, double abstol) override {  // :522-532
    double be, bc, bx, cs;
    voltages(x, &be, &bc, &bx, &cs);
    const DC& d = dc;
    double dbe = be - vbe, dbc = bc - vbc;
    double ichat = d.it - d.ibc + d.itBE * dbe + (d.itBC - d.gmu) * dbc;
    double ibhat = d.ibe + d.ibc + d.gpi * dbe + d.gmu * dbc;
    DC nn = evalDC(be, bc);
    double ic = nn.it - nn.ibc, ib = nn.ibe + nn.ibc;
    return std::fabs(ichat - ic) <= reltol * std::max(std::fabs(ichat), std::fabs(ic)) + abstol &&
           std::fabs(ibhat - ib) <= reltol * std::max(std::fabs(ibhat), std::fabs(ib)) + abstol;
  }
  // terminalCurrents, :537-567: currents into the collector, base, emitter and
  // substrate terminals from the linearization of the last load, and the power
  // into the junction charges; v4 receives the junction voltages.
  void terminals(const double* x, double* ic, double* ib, double* ie, double* is, double* ps, double v4[4]) const {
    double be, bc, bx, cs;
    voltages(x, &be, &bc, &bx, &cs);
    double t = Type;
    const DC& d = dc;
    double dbe = be - vbe, dbc = bc - vbc;
    double it = t * (d.it + d.itBE * dbe + d.itBC * dbc);
    double ibe = t * (d.ibe + d.gpi * dbe);
    double ibc = t * (d.ibc + d.gmu * dbc);
    double iqbe = 0, iqbc = 0, iqbx = 0, iqcs = 0;
    *ps = 0;
    if (tran) {
      iqbe = t * (iq[0] + ag * ch.c[0] * dbe + ag * ch.dqbeDvbc * dbc);
      iqbc = t * (iq[1] + ag * ch.c[1] * dbc);
      iqbx = t * (iq[2] + ag * ch.c[2] * (bx - vbx));
      iqcs = t * (iq[3] + ag * ch.c[3] * (cs - vcs));
      *ps = be * t * iqbe + bc * t * iqbc + bx * t * iqbx + cs * t * iqcs;
    }
    double isb = t * (isub + gsub * (cs - vcs)) + iqcs;
    *ic = it - ibc - iqbc - iqbx;
    *ib = ibe + ibc + iqbe + iqbc + iqbx;
    *ie = -it - ibe - iqbe;
    if (SUBS > 0) { *is = isb; *ic = *ic - isb; }
    else { *ib = *ib + isb; *is = -isb; }
    v4[0] = be; v4[1] = bc; v4[2] = bx; v4[3] = cs;
  }
  double current(const double* x) override {  // Operating :571-576, collector current
    double ic, ib, ie, is, ps, v4[4];
    terminals(x, &ic, &ib, &ie, &is, &ps, v4);
    return ic;
  }
  // StoredEnergy, :630-650: co-energy of the four charges, each along its own
  // voltage with the others held (quadrature on 8 panels).
  double storedEnergy(const double v[4]) const {
    if (!hasCharge) return 0;
    double w = 0;
    for (int k = 0; k < 4; k++) {
      if (v[k] == 0) continue;
      auto qk = [&](double u) {
        double vv[4] = {v[0], v[1], v[2], v[3]};
        vv[k] = u;
        DC d = evalDC(vv[0], vv[1]);
        return charges(vv[0], vv[1], vv[2], vv[3], d).q[k];
      };
      w += v[k] * qk(v[k]) - integrate(qk, 0, v[k], 8);
    }
    return w;
  }
  OpPt operating(const double* x) override {  // Operating :571-576, ExteriorPower :675-680
    double ic, ib, ie, is, ps, v4[4];
    terminals(x, &ic, &ib, &ie, &is, &ps, v4);
    OpPt o;
    double vc = at(x, n, uc), ve = at(x, n, ue);
    o.p = vc * ic + at(x, n, b) * ib + ve * ie + at(x, n, s) * is;
    o.v = vc - ve; o.i = ic; o.ps = ps;
    o.ext = -(o.p - o.ps);
    o.w = storedEnergy(v4);
    o.stores = true;
    return o;
  }
  void loadAC(ACCtx& c) override {  // device/bjt.go:689-711
    DC d = evalDC(vbeAcc, vbcAcc);
    Ch h = charges(vbeAcc, vbcAcc, vbxAcc, vcsAcc, d);
    const double w = c.omega;
    typedef std::complex<double> cx;
    double isub, gsub;
    substrate(vcsAcc, &isub, &gsub);
    cx ybe(0, w * h.c[0]), ybeBC(0, w * h.dqbeDvbc), ybc(0, w * h.c[1]), ybx(0, w * h.c[2]), ycs(gsub, w * h.c[3]);
    c.branch(cp, ep, d.itBE, bp, ep, d.itBC, bp, cp);
    c.branch(bp, ep, cx(d.gpi) + ybe, bp, ep, ybeBC, bp, cp);
    c.branch(bp, cp, cx(d.gmu) + ybc, bp, cp, 0.0, 0, 0);
    c.branch(b, cp, ybx, b, cp, 0.0, 0, 0);
    c.branch(sa, sb, ycs, sa, sb, 0.0, 0, 0);
    if (bp != b) c.stampY(b, bp, d.gx);
    if (cp != uc) c.stampY(uc, cp, gcpr);
    if (ep != ue) c.stampY(ue, ep, gepr);
  }
  void accept(const double* x, double t, int mode) override {  // :579-601
    double be, bc, bx, cs;
    voltages(x, &be, &bc, &bx, &cs);
    vbeAcc = be; vbcAcc = bc; vbxAcc = bx; vcsAcc = cs;
    DC d = evalDC(be, bc);
    Ch c = charges(be, bc, bx, cs, d);
    double dv[4] = {be - vbe, bc - vbc, bx - vbx, cs - vcs};
    for (int k = 0; k < 4; k++) {
      if (mode == ModeTran && tran) {
        double i = iq[k] + ag * ch.c[k] * dv[k];
        if (k == 0) i += ag * ch.dqbeDvbc * (bc - vbc);
        iqPrev[k] = i;
      } else iqPrev[k] = 0;
      if (mode != ModeTran) hist[k].reset();
      qPrev[k] = c.q[k];
      hist[k].push(t, c.q[k]);
    }
  }
  double truncate(const double* x, const TruncCtx& tc) override {  // bjt.go Truncate
    if (!hasCharge || !tran) return kInf;
    double be, bc, bx, cs;
    voltages(x, &be, &bc, &bx, &cs);
    DC d = evalDC(be, bc);
    Ch c = charges(be, bc, bx, cs, d);
    double dv[4] = {be - vbe, bc - vbc, bx - vbx, cs - vcs};
    double h = kInf;
    for (int k = 0; k < 4; k++) {
      if (c.q[k] == 0 && qPrev[k] == 0) continue;
      double i = iq[k] + ag * ch.c[k] * dv[k];
      if (k == 0) i += ag * ch.dqbeDvbc * dv[1];
      h = std::min(h, lteStep(hist[k], c.q[k], i, iqPrev[k], tc.abstol, tc));
    }
    return h;
  }
};

}  // namespace kso
