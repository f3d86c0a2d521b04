// ks_sparse.cpp — symbolic sparse LU of one circuit's MNA system, for the
// multi-topology (warp-per-circuit) kernels.
//
// Done once per circuit on the host (the role of solver/sparse.go:154-187
// analyze and :412-452 minimumDegree, with the pivot rows of its threshold
// partial pivoting chosen once instead of at every factorization):
//   1. the structural pattern: every entry any element stamps in any mode
//      (devices as dense blocks over their terminals) plus every diagonal (gmin
//      and pseudo-transient stepping add to them);
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

void stamp_rows(const HostPlan& hp, std::vector<Bits>& rows) {
  auto add = [&](int i, int j) { if (i >= 0 && j >= 0) rows[i].set(j); };
  auto block = [&](const int* u, int k) {
    for (int a = 0; a < k; a++)
      for (int b = 0; b < k; b++) add(u[a], u[b]);
  };
  for (const KElem& e : hp.elem) {
    const int* u = e.u;
    switch (e.kind) {
      case KS_ELEM_R: case KS_ELEM_C: block(u, 2); break;
      case KS_ELEM_V: case KS_ELEM_L:
        add(u[0], u[2]); add(u[1], u[2]); add(u[2], u[0]); add(u[2], u[1]); add(u[2], u[2]); break;
      case KS_ELEM_I: break;
      case KS_ELEM_D: block(u, 3); break;
      case KS_ELEM_Q: block(u, 9); break;
      case KS_ELEM_M: block(u, 6); break;
      default: break;
    }
  }
  for (int i = 0; i < hp.n; i++) add(i, i);
}

}  // namespace

int sparse_symbolic(const HostPlan& hp, const double* values, double h, SparseSym* sy, std::string* err) {
  const int n = hp.n;
  if (n < 1) { *err = "empty system"; return KS_EINVAL; }
  std::vector<Bits> A(n);
  for (auto& r : A) r.init(n);
  stamp_rows(hp, A);
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
  //    inductors at their +-1 incidence, gmin on node diagonals, transistor
  //    terminals at 1 mS; at DC (h = 0) capacitors are open, for a transient of
  //    step h capacitors are 2C/h and inductor branches -2L/h (the trapezoidal
  //    companions).  The GPU refactors every Newton iteration on this fixed
  //    pivot sequence.
  std::vector<double> M((size_t)n * n, 0.0);
  auto at = [&](int i, int j) -> double& { return M[(size_t)i * n + j]; };
  auto madd = [&](int i, int j, double g) { if (i >= 0 && j >= 0) at(i, j) += g; };
  auto cond = [&](int a, int b, double g) { madd(a, a, g); madd(b, b, g); madd(a, b, -g); madd(b, a, -g); };
  std::vector<char> branch(n, 0);
  for (const KElem& e : hp.elem) {
    const int* u = e.u;
    switch (e.kind) {
      case KS_ELEM_R: {
        double r = values ? values[e.param + KS_RCL_P_VALUE] : 1.0;
        cond(u[0], u[1], r > 0 ? 1.0 / r : 1.0);
        break;
      }
      case KS_ELEM_C:
        if (h > 0) cond(u[0], u[1], 2.0 * (values ? values[e.param + KS_RCL_P_VALUE] : 1e-12) / h);
        break;
      case KS_ELEM_V: case KS_ELEM_L:
        madd(u[0], u[2], 1); madd(u[1], u[2], -1); madd(u[2], u[0], 1); madd(u[2], u[1], -1);
        if (e.kind == KS_ELEM_L && h > 0) madd(u[2], u[2], -2.0 * (values ? values[e.param + KS_RCL_P_VALUE] : 1e-9) / h);
        if (u[2] >= 0) branch[u[2]] = 1;
        break;
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
      case KS_ELEM_Q:
        for (int t = 0; t < 9; t++)
          for (int v = t + 1; v < 9; v++) if (u[t] >= 0 && u[v] >= 0 && u[t] != u[v]) cond(u[t], u[v], 1e-3);
        break;
      case KS_ELEM_M:
        for (int t = 0; t < 6; t++)
          for (int v = t + 1; v < 6; v++) if (u[t] >= 0 && u[v] >= 0 && u[t] != u[v]) cond(u[t], u[v], 1e-3);
        break;
      default: break;
    }
  }
  for (int i = 0; i < n; i++)
    if (!branch[i]) at(i, i) += 1e-12;
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
