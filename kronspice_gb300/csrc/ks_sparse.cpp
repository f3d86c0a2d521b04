// ks_sparse.cpp — symbolic sparse LU of one circuit's MNA system, for the
// multi-topology (warp-per-circuit) kernels.
//
// Done once per circuit on the host (the role of solver/sparse.go:154-187
// analyze and :412-452 minimumDegree, with the pivot rows of its threshold
// partial pivoting chosen once instead of at every factorization):
//   1. the reference's pattern: every entry the elements' loads stamp in the
//      analysis's modes (stamp_rows), plus every diagonal (gmin and
//      pseudo-transient stepping add to them);
//   2. columns: minimum degree on the pattern of A + A^T, ties to the lowest index;
//   3. rows: threshold partial pivoting with diagonal preference in that column
//      order on a representative matrix of the circuit's own values (at DC, or
//      with the companion models of a transient step);
//   4. the pattern of L + U for that pivot sequence (row by row, each row the
//      union of its A row and the U rows of its L entries).
// The numeric factorization on the GPU then runs on this fixed pivot sequence.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "ks_internal.h"

namespace ksh {

namespace {

struct Bits {
  int words = 0;
  std::vector<uint64_t> w;
  void init(int n) { words = (n + 63) / 64; w.assign(words, 0); }
  void set(int i) { w[i >> 6] |= 1ull << (i & 63); }
  bool get(int i) const { return (w[i >> 6] >> (i & 63)) & 1ull; }
  void clear(int i) { w[i >> 6] &= ~(1ull << (i & 63)); }
};

// The reference's pattern: every entry an element's Load stamps in the
// analysis's modes (Sparse.add keeps each new (i, j) as a slot for the rest of
// the run, solver/sparse.go:114-143), restated per device from its stamp
// sequence: passive.go:72-84, reactive.go:60-106 and :230-259, source.go:102-112,
// diode.go:229-275, bjt.go:463-515, mosfet.go:563-611.  Operating point: the
// DC stamps; transient: the union of the DC stamps (its operating point) and
// the companion stamps of the time steps.  Entries that a device stamps only
// while one of its conductances is non-zero are all included (a fixed pivot
// sequence must hold every entry any Newton iteration may stamp); entries that
// depend only on parameters follow them (the BJT's base-to-collector junction
// capacitance outside the intrinsic base: CJC (1 - XCJC) != 0).  Every diagonal
// is added too (gmin stepping and pseudo-transient continuation add to them);
// minimum degree does not look at diagonals.
void stamp_rows(const HostPlan& hp, const double* values, bool transient, std::vector<Bits>& rows) {
  auto add = [&](int i, int j) { if (i >= 0 && j >= 0) rows[i].set(j); };
  auto g4 = [&](int a, int b) { add(a, a); add(b, b); add(a, b); add(b, a); };
  // bjt.go:463-480 / mosfet.go:563-578: a current from a to b controlled by v(p) - v(n)
  auto ctl = [&](int a, int b, int p, int q) { add(a, p); add(a, q); add(b, p); add(b, q); };
  for (const KElem& e : hp.elem) {
    const int* u = e.u;
    switch (e.kind) {
      case KS_ELEM_R: g4(u[0], u[1]); break;
      case KS_ELEM_C: case KS_ELEM_CN: if (transient) g4(u[0], u[1]); break;
      case KS_ELEM_V: case KS_ELEM_L: case KS_ELEM_LN:
        add(u[0], u[2]); add(u[1], u[2]); add(u[2], u[0]); add(u[2], u[1]);
        if (e.kind != KS_ELEM_V && transient) add(u[2], u[2]);
        break;
      case KS_ELEM_I: break;
      case KS_ELEM_D:  // u = {anode, cathode, internal anode}
        g4(u[2], u[1]);
        if (u[2] != u[0]) g4(u[0], u[2]);
        break;
      case KS_ELEM_Q: {  // u = {c, e, b, s, c', b', e', sa, sb}
        const int uc = u[0], ue = u[1], b = u[2], cp = u[4], bp = u[5], ep = u[6], sa = u[7], sb = u[8];
        ctl(cp, ep, bp, ep); ctl(cp, ep, bp, cp);  // transport current on vbe and vbc
        ctl(bp, ep, bp, ep);                       // base-emitter
        ctl(bp, cp, bp, cp);                       // base-collector
        ctl(sa, sb, sa, sb);                       // substrate
        if (transient) {
          // the charge branches fall on the entries above, except the junction
          // capacitance between the external base and the collector
          const double cjc = values ? values[e.param + KS_Q_P_CJC] : 1.0;
          const double xcjc = values ? values[e.param + KS_Q_P_XCJC] : 0.0;
          if (cjc - cjc * xcjc != 0) ctl(b, cp, b, cp);
        }
        if (bp != b) g4(b, bp);
        if (cp != uc) g4(uc, cp);
        if (ep != ue) g4(ue, ep);
        break;
      }
      case KS_ELEM_M: {  // u = {d, s, g, b, d', s'}
        const int ud = u[0], us = u[1], g = u[2], b = u[3], dp = u[4], sp = u[5];
        ctl(dp, sp, g, sp); ctl(dp, sp, dp, sp); ctl(dp, sp, b, sp);  // channel on vgs, vds, vbs
        ctl(b, sp, b, sp); ctl(b, dp, b, dp);                           // bulk junctions
        if (transient) { g4(g, sp); g4(g, dp); g4(g, b); g4(b, sp); g4(b, dp); }  // Meyer and junction charges
        if (dp != ud) g4(ud, dp);
        if (sp != us) g4(us, sp);
        break;
      }
      case KS_ELEM_E: case KS_ELEM_H:  // device/controlled.go:83-100
        add(u[0], u[2]); add(u[1], u[2]); add(u[2], u[0]); add(u[2], u[1]); add(u[2], u[3]);
        if (e.kind == KS_ELEM_E) add(u[2], u[4]);
        break;
      case KS_ELEM_G: add(u[0], u[3]); add(u[0], u[4]); add(u[1], u[3]); add(u[1], u[4]); break;
      case KS_ELEM_F: add(u[0], u[3]); add(u[1], u[3]); break;
      case KS_ELEM_K: if (transient) { add(u[0], u[1]); add(u[1], u[0]); } break;  // device/mutual.go:75-118
      case KS_ELEM_S: case KS_ELEM_W: {  // device/switch.go:174-226
        g4(u[0], u[1]);
        // a smooth switch stamps its transconductance while its control is inside the band
        const bool smooth = values ? values[e.param + KS_SW_P_VH] < 0 : true;
        if (smooth) {
          if (e.kind == KS_ELEM_W) { add(u[0], u[3]); add(u[1], u[3]); }
          else ctl(u[0], u[1], u[3], u[4]);
        }
        break;
      }
      default: break;
    }
  }
  for (int i = 0; i < hp.n; i++) add(i, i);
}

}  // namespace

// The pattern stamp_rows gives, as an n x n byte matrix (the symbolic-parity tests).
void sparse_pattern(const HostPlan& hp, const double* values, bool transient, uint8_t* out) {
  const int n = hp.n;
  std::vector<Bits> A(n);
  for (auto& r : A) r.init(n);
  stamp_rows(hp, values, transient, A);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) out[(size_t)i * n + j] = A[i].get(j) ? 1 : 0;
}

int sparse_symbolic(const HostPlan& hp, const double* values, double h, SparseSym* sy, std::string* err) {
  const int n = hp.n;
  if (n < 1) { *err = "empty system"; return KS_EINVAL; }
  std::vector<Bits> A(n);
  for (auto& r : A) r.init(n);
  stamp_rows(hp, values, h > 0, A);
  // 2. columns: minimum degree on the pattern of A + A^T, ties to the lowest
  //    index (solver/sparse.go:412-452)
  std::vector<Bits> G(n);
  for (auto& r : G) r.init(n);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      if (i != j && A[i].get(j)) { G[i].set(j); G[j].set(i); }
  Bits left;
  left.init(n);
  for (int i = 0; i < n; i++) left.set(i);
  std::vector<int> q;
  q.reserve(n);
  for (int step = 0; step < n; step++) {
    int best = -1, bd = 1 << 30;
    for (int v = 0; v < n; v++) {
      if (!left.get(v)) continue;
      int d = 0;
      for (int w = 0; w < G[v].words; w++) d += __builtin_popcountll(G[v].w[w] & left.w[w]);
      if (d < bd) { bd = d; best = v; }
    }
    left.clear(best);
    std::vector<int> nb;
    for (int v = 0; v < n; v++)
      if (left.get(v) && G[best].get(v)) nb.push_back(v);
    for (int v : nb)
      for (int w = 0; w < G[v].words; w++) G[v].w[w] |= G[best].w[w] & left.w[w];
    for (int v : nb) G[v].clear(v);
    q.push_back(best);
  }
  // 3. rows: threshold partial pivoting with the reference's diagonal preference
  //    (solver/sparse.go:256-281, DiagPivotTol 1e-3) in that column order, on a
  //    representative matrix: resistors at their conductance, sources and
  //    inductors at their +-1 incidence, gmin on node diagonals, transistors
  //    conducting (on their own stamp pattern); at DC (h = 0) capacitors are open, for a transient of
  //    step h capacitors are 2C/h and inductor branches -2L/h (the trapezoidal
  //    companions).  The GPU refactors every Newton iteration on this fixed
  //    pivot sequence.
  std::vector<double> M((size_t)n * n, 0.0);
  auto at = [&](int i, int j) -> double& { return M[(size_t)i * n + j]; };
  auto madd = [&](int i, int j, double g) { if (i >= 0 && j >= 0) at(i, j) += g; };
  auto cond = [&](int a, int b, double g) { madd(a, a, g); madd(b, b, g); madd(a, b, -g); madd(b, a, -g); };
  // a current from a to b of g (v(p) - v(q))
  auto ctl = [&](int a, int b, int p, int q, double g) { madd(a, p, g); madd(a, q, -g); madd(b, p, -g); madd(b, q, g); };
  std::vector<char> branch(n, 0);
  for (const KElem& e : hp.elem) {
    const int* u = e.u;
    switch (e.kind) {
      case KS_ELEM_R: {
        double r = values ? values[e.param + KS_RCL_P_VALUE] : 1.0;
        cond(u[0], u[1], r > 0 ? 1.0 / r : 1.0);
        break;
      }
      case KS_ELEM_C: case KS_ELEM_CN: {  // a curved capacitor at 1 nF (the law's value is 0 with a curve)
        const double cv = values ? values[e.param + KS_RCL_P_VALUE] : 1e-12;
        if (h > 0) cond(u[0], u[1], 2.0 * (cv > 0 ? cv : 1e-9) / h);
        break;
      }
      case KS_ELEM_V: case KS_ELEM_L: case KS_ELEM_LN: {
        madd(u[0], u[2], 1); madd(u[1], u[2], -1); madd(u[2], u[0], 1); madd(u[2], u[1], -1);
        const double lv = values ? values[e.param + KS_RCL_P_VALUE] : 1e-9;
        if (e.kind != KS_ELEM_V && h > 0) madd(u[2], u[2], -2.0 * (lv > 0 ? lv : 1e-3) / h);
        if (u[2] >= 0) branch[u[2]] = 1;
        break;
      }
      case KS_ELEM_D:
        // junctions are left out: their conductance spans twelve decades over a
        // Newton solve, and a node row they feed stays diagonally dominant
        // whatever it is (their stamp is +g on the diagonal, -g beside it), so
        // the pivots are chosen on the parts that do not move
        if (u[2] != u[0]) {
          double rs = values ? values[e.param + KS_D_P_RS] : 0.0;
          cond(u[0], u[2], rs > 0 ? 1.0 / rs : 1.0);
        }
        break;
      case KS_ELEM_Q: {  // a forward-active transistor: gm 40 mS, gpi 1 mS, gmu 1 uS, series resistances
        const int uc = u[0], ue = u[1], b = u[2], cp = u[4], bp = u[5], ep = u[6];
        ctl(cp, ep, bp, ep, 4e-2);
        cond(bp, ep, 1e-3);
        cond(bp, cp, 1e-6);
        auto rser = [&](int k) { double r = values ? values[e.param + k] : 0.0; return r > 0 ? 1.0 / r : 1.0; };
        if (bp != b) cond(b, bp, rser(KS_Q_P_RB));
        if (cp != uc) cond(uc, cp, rser(KS_Q_P_RC));
        if (ep != ue) cond(ue, ep, rser(KS_Q_P_RE));
        break;
      }
      case KS_ELEM_M: {  // a conducting channel: gm 1 mS, gds 0.1 mS; at a step of h, 1 pF gate capacitances
        const int ud = u[0], us = u[1], g = u[2], b = u[3], dp = u[4], sp = u[5];
        ctl(dp, sp, g, sp, 1e-3);
        cond(dp, sp, 1e-4);
        if (h > 0) { cond(g, sp, 2e-12 / h); cond(g, dp, 2e-12 / h); cond(g, b, 2e-12 / h); }
        if (dp != ud) cond(ud, dp, 1.0);
        if (sp != us) cond(us, sp, 1.0);
        break;
      }
      case KS_ELEM_E: case KS_ELEM_H: {  // the output branch row at its gain
        const double g = values ? values[e.param + KS_CTL_P_GAIN] : 1.0;
        madd(u[0], u[2], 1); madd(u[1], u[2], -1); madd(u[2], u[0], 1); madd(u[2], u[1], -1);
        madd(u[2], u[3], -g);
        if (e.kind == KS_ELEM_E) madd(u[2], u[4], g);
        if (u[2] >= 0) branch[u[2]] = 1;
        break;
      }
      case KS_ELEM_G: {
        const double g = values ? values[e.param + KS_CTL_P_GAIN] : 1.0;
        madd(u[0], u[3], g); madd(u[0], u[4], -g); madd(u[1], u[3], -g); madd(u[1], u[4], g);
        break;
      }
      case KS_ELEM_F: {
        const double g = values ? values[e.param + KS_CTL_P_GAIN] : 1.0;
        madd(u[0], u[3], g); madd(u[1], u[3], -g);
        break;
      }
      // switches are left out like the junctions: RON and ROFF lie six to twelve
      // decades apart, and which one a Newton iteration stamps is not known here
      case KS_ELEM_K:  // the trapezoidal coupling 2M/h of a time step
        if (h > 0 && values) {
          const double m = values[e.param + KS_K_P_COUPLING] *
                           std::sqrt(values[u[2] + KS_RCL_P_VALUE] * values[u[3] + KS_RCL_P_VALUE]);
          madd(u[0], u[1], -2 * m / h); madd(u[1], u[0], -2 * m / h);
        }
        break;
      default: break;
    }
  }
  for (int i = 0; i < n; i++)
    if (!branch[i]) at(i, i) += 1e-12;
  for (int i = 0; i < n; i++)  // every stamp above falls on the pattern; keep it so
    for (int j = 0; j < n; j++)
      if (!A[i].get(j)) at(i, j) = 0;
  std::vector<int> pr(n, -1);  // pr[column] = pivot row
  std::vector<char> used(n, 0);
  for (int k = 0; k < n; k++) {
    const int c = q[k];
    int piv = -1;
    double best = -1;
    for (int r = 0; r < n; r++) {  // every row left, fill included
      if (used[r]) continue;
      double v = std::fabs(at(r, c));
      if (v > 0 && (v > best || (v == best && r < piv))) { best = v; piv = r; }
    }
    if (piv < 0) {  // numerically empty column: any free row (the factorization reports it singular)
      for (int r = 0; r < n; r++) if (!used[r]) { piv = r; break; }
    } else if (!used[c] && std::fabs(at(c, c)) >= 1e-3 * best && std::fabs(at(c, c)) > 0) {
      piv = c;
    }
    used[piv] = 1;
    pr[c] = piv;
    const double pv = at(piv, c);
    if (pv == 0) continue;
    for (int r = 0; r < n; r++) {
      if (used[r]) continue;
      const double f = at(r, c) / pv;
      if (f == 0) continue;
      for (int l = k + 1; l < n; l++) {
        const int cl = q[l];
        at(r, cl) -= f * at(piv, cl);
      }
      at(r, c) = 0;
    }
  }
  sy->n = n;
  sy->q = q;
  sy->prow.resize(n);
  sy->qinv.assign(n, 0);
  sy->pinv.assign(n, 0);
  for (int k = 0; k < n; k++) {
    sy->prow[k] = pr[q[k]];
    sy->qinv[q[k]] = k;
  }
  for (int k = 0; k < n; k++) sy->pinv[sy->prow[k]] = k;
  // 4. pattern of L + U in step coordinates, row by row
  std::vector<Bits> C(n);
  for (auto& r : C) r.init(n);
  for (int k = 0; k < n; k++) {
    for (int l = 0; l < n; l++)
      if (A[sy->prow[k]].get(q[l])) C[k].set(l);
    C[k].set(k);  // every pivot has a slot (zero where the matching found none)
  }
  sy->rp.assign(n + 1, 0);
  sy->ci.clear();
  sy->in_a.clear();
  sy->dg.assign(n, 0);
  int64_t flops = 0;
  for (int i = 0; i < n; i++) {
    for (int k = 0; k < i; k++) {  // in ascending order, fill included
      if (!C[i].get(k)) continue;
      for (int w = 0; w < C[i].words; w++) {
        uint64_t mask = C[k].w[w];
        int base = w * 64;  // only columns > k
        if (base + 63 <= k) continue;
        if (base <= k) mask &= ~((k - base == 63) ? ~0ull : ((2ull << (k - base)) - 1));
        C[i].w[w] |= mask;
      }
    }
    sy->rp[i] = (int)sy->ci.size();
    for (int l = 0; l < n; l++) {
      if (!C[i].get(l)) continue;
      if (l == i) sy->dg[i] = (int)sy->ci.size();
      sy->ci.push_back(l);
      sy->in_a.push_back(A[sy->prow[i]].get(q[l]) ? 1 : 0);
    }
  }
  sy->rp[n] = (int)sy->ci.size();
  for (int i = 0; i < n; i++)
    for (int p = sy->rp[i]; p < sy->dg[i]; p++) {
      int k = sy->ci[p];
      flops += 1 + 2 * (sy->rp[k + 1] - sy->dg[k] - 1);
    }
  sy->flops = flops;
  return KS_OK;
}

}  // namespace ksh
