// oracle_torn.hpp — TEST INFRASTRUCTURE: restatement of the reference's torn
// linear solver, kron.JacobianTearing (kron/jacobian.go), as a Matrix backend
// of the oracle's Sim.  Only the oracle uses it; the engine never does.
//
//   pieces      union-find over J's pattern with the torn node pairs removed
//               (buildPlan, kron/jacobian.go:296-389)
//   per piece   equilibrated dense LU with partial pivoting (denseLU,
//               :609-712), reused while its block is unchanged (or within
//               ReuseTol of its largest entry), W_k = B^-1 e_row per port
//   join        dense interconnection I + M.Q.B^-1.P, factored every solve
//               (:468-507)
//   apply       z = B^-1 b; (I + M.Q.B^-1.P) w = M.Q.z; x = z - B^-1.P.w (:508-550)
//   refinement  against the whole J until the componentwise backward error is
//               <= 1e-14, accepted at <= 1e-12 (:551-589)
//   fallback    stale factors that do not refine: refactor once more; then an
//               untorn LU of the whole J (:391-434)
#ifndef KS_ORACLE_TORN_HPP
#define KS_ORACLE_TORN_HPP

#include <cmath>
#include <memory>
#include <unordered_map>
#include <vector>

#include "oracle_solver.hpp"

namespace kso {

struct TornStats {
  int64_t solves = 0, factors = 0, reuses = 0, stale = 0, fallbacks = 0, refines = 0, maxPieces = 0;
};

// denseLU, kron/jacobian.go:609-712 (rows and columns equilibrated to unit maximum).
struct EqLU {
  int n = 0;
  std::vector<double> lu, rs, cs, col;
  std::vector<int> piv;
  void init(int n_) { n = n_; lu.assign((size_t)n * n, 0); rs.assign(n, 0); cs.assign(n, 0); col.assign(n, 0); piv.assign(n, 0); }
  struct Ent { int32_t i, j; double v; };
  bool factor(const std::vector<Ent>& ent) {
    std::fill(lu.begin(), lu.end(), 0.0);
    std::fill(rs.begin(), rs.end(), 0.0);
    std::fill(cs.begin(), cs.end(), 0.0);
    std::fill(col.begin(), col.end(), 0.0);
    for (auto& e : ent) rs[e.i] = std::max(rs[e.i], std::fabs(e.v));
    for (int i = 0; i < n; i++) {
      if (rs[i] == 0) return false;  // an empty equation
      rs[i] = 1 / rs[i];
    }
    for (auto& e : ent) cs[e.j] = std::max(cs[e.j], std::fabs(e.v) * rs[e.i]);
    for (int j = 0; j < n; j++) {
      if (cs[j] == 0) return false;  // an unknown in no equation
      cs[j] = 1 / cs[j];
    }
    for (auto& e : ent) lu[(size_t)e.i * n + e.j] += e.v * rs[e.i] * cs[e.j];
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++) col[j] = std::max(col[j], std::fabs(lu[(size_t)i * n + j]));
    for (int k = 0; k < n; k++) {
      int p = k;
      double maxv = std::fabs(lu[(size_t)k * n + k]);
      for (int i = k + 1; i < n; i++) {
        double v = std::fabs(lu[(size_t)i * n + k]);
        if (v > maxv) { maxv = v; p = i; }
      }
      if (maxv <= col[k] * (double)n * 1e-14) return false;
      piv[k] = p;
      if (p != k)
        for (int j = 0; j < n; j++) std::swap(lu[(size_t)k * n + j], lu[(size_t)p * n + j]);
      const double pivot = lu[(size_t)k * n + k];
      for (int i = k + 1; i < n; i++) {
        double f = lu[(size_t)i * n + k] / pivot;
        lu[(size_t)i * n + k] = f;
        if (f == 0) continue;
        for (int j = k + 1; j < n; j++) lu[(size_t)i * n + j] -= f * lu[(size_t)k * n + j];
      }
    }
    return true;
  }
  // x = A^-1 b (b and x distinct)
  void solve(const double* b, double* x) const {
    for (int i = 0; i < n; i++) x[i] = b[i] * rs[i];
    for (int k = 0; k < n; k++) if (piv[k] != k) std::swap(x[k], x[piv[k]]);
    for (int i = 0; i < n; i++) {
      double s = x[i];
      for (int j = 0; j < i; j++) s -= lu[(size_t)i * n + j] * x[j];
      x[i] = s;
    }
    for (int i = n - 1; i >= 0; i--) {
      double s = x[i];
      for (int j = i + 1; j < n; j++) s -= lu[(size_t)i * n + j] * x[j];
      x[i] = s / lu[(size_t)i * n + i];
    }
    for (int j = 0; j < n; j++) x[j] *= cs[j];
  }
};

// tornMat, kron/jacobian.go:226-589 (real systems).
struct Torn : Matrix {
  static constexpr int kMaxRefine = 12;       // maxRefine
  static constexpr double kRefineDone = 1e-14, kRefineAccept = 1e-12;
  static constexpr int kMaxDense = 4096;      // solver.MaxDense
  int n;
  std::vector<std::pair<int, int>> cuts;      // node unknowns of the torn elements
  double reuseTol;
  TornStats* stats;
  std::unordered_map<int64_t, int32_t> slot;
  std::vector<int32_t> ri, ci;
  std::vector<double> val;
  bool havePlan = false;
  struct Piece {
    std::vector<int32_t> idx, slots, li, lj, ports;
    EqLU lu;
    std::vector<double> last;
    bool have = false;
    std::vector<std::vector<double>> W;
    std::vector<EqLU::Ent> ent;
    std::vector<double> b, xl;
  };
  std::vector<Piece> pieces;
  std::vector<int32_t> pieceOf, local, off, rows, rowIdx;
  EqLU ic;
  std::vector<EqLU::Ent> icEnt;
  std::vector<double> z, r, h, w, dx, den;
  std::unique_ptr<Matrix> fallback;

  Torn(int n_, const std::vector<std::pair<int, int>>& c, double tol, TornStats* st)
      : n(n_), cuts(c), reuseTol(tol), stats(st) {}
  int size() const override { return n; }
  void clear() override { std::fill(val.begin(), val.end(), 0.0); }
  void add(int i, int j, double v) override {
    if (i < 0 || j < 0 || i >= n || j >= n) return;
    int64_t k = (int64_t)i * n + j;
    auto it = slot.find(k);
    int32_t s;
    if (it == slot.end()) {
      s = (int32_t)val.size();
      slot[k] = s;
      ri.push_back(i); ci.push_back(j); val.push_back(0);
      havePlan = false;
    } else s = it->second;
    val[s] += v;
  }
  double at(int i, int j) const override {
    auto it = slot.find((int64_t)i * n + j);
    return it == slot.end() ? 0.0 : val[it->second];
  }
  void absProduct(const double* x, double* y) override {
    for (int i = 0; i < n; i++) y[i] = 0;
    for (size_t s = 0; s < val.size(); s++) y[ri[s]] += std::fabs(val[s]) * std::fabs(x[ci[s]]);
  }

  // buildPlan, kron/jacobian.go:296-389
  bool buildPlan() {
    std::unordered_map<int64_t, bool> cut;
    for (auto& c : cuts)
      if (c.first < n && c.second < n && c.first >= 0 && c.second >= 0) {
        cut[(int64_t)c.first * n + c.second] = true;
        cut[(int64_t)c.second * n + c.first] = true;
      }
    std::vector<int32_t> parent(n);
    for (int i = 0; i < n; i++) parent[i] = i;
    auto find = [&](int32_t i) {
      while (parent[i] != i) { parent[i] = parent[parent[i]]; i = parent[i]; }
      return i;
    };
    for (size_t s = 0; s < val.size(); s++) {
      int32_t i = ri[s], j = ci[s];
      if (i == j || cut.count((int64_t)i * n + j)) continue;
      int32_t a = find(i), b = find(j);
      if (a != b) { if (a < b) parent[b] = a; else parent[a] = b; }
    }
    pieces.clear();
    pieceOf.assign(n, 0); local.assign(n, 0); rowIdx.assign(n, -1);
    off.clear(); rows.clear();
    std::vector<int32_t> root(n, -1);
    for (int32_t i = 0; i < n; i++) {
      int32_t r = find(i);
      if (root[r] < 0) { root[r] = (int32_t)pieces.size(); pieces.emplace_back(); }
      Piece& pc = pieces[root[r]];
      pieceOf[i] = root[r]; local[i] = (int32_t)pc.idx.size();
      pc.idx.push_back(i);
    }
    for (size_t s = 0; s < val.size(); s++) {
      int32_t i = ri[s], j = ci[s];
      if (pieceOf[i] == pieceOf[j]) {
        Piece& pc = pieces[pieceOf[i]];
        pc.slots.push_back((int32_t)s); pc.li.push_back(local[i]); pc.lj.push_back(local[j]);
        continue;
      }
      off.push_back((int32_t)s);
      if (rowIdx[i] < 0) {
        rowIdx[i] = (int32_t)rows.size();
        rows.push_back(i);
        pieces[pieceOf[i]].ports.push_back(rowIdx[i]);
      }
    }
    for (auto& pc : pieces) {
      int nl = (int)pc.idx.size();
      if (nl > kMaxDense) return false;
      pc.lu.init(nl);
      pc.last.assign(pc.slots.size(), 0);
      pc.ent.resize(pc.slots.size());
      pc.W.assign(pc.ports.size(), std::vector<double>(nl, 0));
      pc.b.assign(nl, 0); pc.xl.assign(nl, 0);
      pc.have = false;
    }
    if (!rows.empty()) ic.init((int)rows.size());
    z.assign(n, 0); r.assign(n, 0); dx.assign(n, 0); den.assign(n, 0);
    h.assign(rows.size(), 0); w.assign(rows.size(), 0);
    if (stats && (int64_t)pieces.size() > stats->maxPieces) stats->maxPieces = (int64_t)pieces.size();
    havePlan = true;
    return true;
  }

  void apply(const double* rhs, double* out) {
    for (auto& pc : pieces) {
      bool nz = false;
      for (size_t li = 0; li < pc.idx.size(); li++) { pc.b[li] = rhs[pc.idx[li]]; nz = nz || pc.b[li] != 0; }
      if (!nz) { for (int32_t g : pc.idx) out[g] = 0; continue; }
      pc.lu.solve(pc.b.data(), pc.xl.data());
      for (size_t li = 0; li < pc.idx.size(); li++) out[pc.idx[li]] = pc.xl[li];
    }
    if (rows.empty()) return;
    std::fill(h.begin(), h.end(), 0.0);
    for (int32_t s : off) h[rowIdx[ri[s]]] += val[s] * out[ci[s]];
    ic.solve(h.data(), w.data());
    for (auto& pc : pieces)
      for (size_t k = 0; k < pc.ports.size(); k++) {
        double wk = w[pc.ports[k]];
        if (wk == 0) continue;
        for (size_t li = 0; li < pc.idx.size(); li++) out[pc.idx[li]] -= wk * pc.W[k][li];
      }
  }

  // torn, kron/jacobian.go:438-589: (ok, usedStale)
  std::pair<bool, bool> torn(const double* b, double* x, bool allowStale) {
    bool usedStale = false;
    for (auto& pc : pieces) {
      bool same = pc.have, small = pc.have && allowStale && reuseTol > 0;
      double mx = 0, dmax = 0;
      for (size_t k = 0; k < pc.slots.size(); k++) {
        double v = val[pc.slots[k]];
        if (v != pc.last[k]) {
          same = false;
          if (small) dmax = std::max(dmax, std::fabs(v - pc.last[k]));
        }
        if (small) mx = std::max(mx, std::fabs(v));
      }
      if (same) { if (stats) stats->reuses++; continue; }
      if (small && dmax <= reuseTol * mx) { if (stats) stats->stale++; usedStale = true; continue; }
      for (size_t k = 0; k < pc.slots.size(); k++) {
        pc.ent[k] = EqLU::Ent{pc.li[k], pc.lj[k], val[pc.slots[k]]};
        pc.last[k] = val[pc.slots[k]];
      }
      pc.have = false;
      if (!pc.lu.factor(pc.ent)) return {false, usedStale};
      if (stats) stats->factors++;
      for (size_t k = 0; k < pc.ports.size(); k++) {
        std::fill(pc.b.begin(), pc.b.end(), 0.0);
        pc.b[local[rows[pc.ports[k]]]] = 1;
        pc.lu.solve(pc.b.data(), pc.W[k].data());
      }
      pc.have = true;
    }
    if (!rows.empty()) {
      icEnt.clear();
      for (size_t a = 0; a < rows.size(); a++) icEnt.push_back(EqLU::Ent{(int32_t)a, (int32_t)a, 1.0});
      for (int32_t s : off) {
        int32_t rr = ri[s], cc = ci[s];
        double v = val[s];
        if (v == 0) continue;
        Piece& pc = pieces[pieceOf[cc]];
        int32_t lc = local[cc];
        for (size_t k = 0; k < pc.ports.size(); k++) {
          double g = pc.W[k][lc];
          if (g != 0) icEnt.push_back(EqLU::Ent{rowIdx[rr], pc.ports[k], v * g});
        }
      }
      if (!ic.factor(icEnt)) return {false, usedStale};
    }
    apply(b, x);
    double berr = INFINITY;
    for (int pass = 0; pass <= kMaxRefine; pass++) {
      for (int i = 0; i < n; i++) { r[i] = b[i]; den[i] = std::fabs(b[i]); }
      for (size_t s = 0; s < val.size(); s++) {
        double t = val[s] * x[ci[s]];
        r[ri[s]] -= t;
        den[ri[s]] += std::fabs(t);
      }
      berr = 0;
      for (int i = 0; i < n; i++) {
        if (den[i] > 0) berr = std::max(berr, std::fabs(r[i]) / den[i]);
        else if (r[i] != 0) berr = INFINITY;
      }
      if (berr <= kRefineDone || pass == kMaxRefine) break;
      apply(r.data(), dx.data());
      for (int i = 0; i < n; i++) x[i] += dx[i];
      if (stats) stats->refines++;
    }
    if (!(berr <= kRefineAccept)) return {false, usedStale};
    for (int i = 0; i < n; i++) if (!finite(x[i])) return {false, usedStale};
    return {true, usedStale};
  }

  int untorn(const double* b, double* x, std::string* msg) {  // :418-434
    if (stats) stats->fallbacks++;
    if (!fallback) {
      if (n < 30) fallback.reset(new Dense(n)); else fallback.reset(new Sparse(n));
    }
    fallback->clear();
    for (size_t s = 0; s < val.size(); s++) fallback->add(ri[s], ci[s], val[s]);
    return fallback->solve(b, x, msg);
  }

  int solve(const double* b, double* x, std::string* msg) override {  // :391-416
    if (stats) stats->solves++;
    for (double v : val) if (!finite(v)) return SOLVE_NONFINITE;
    if (!havePlan && !buildPlan()) { havePlan = false; return untorn(b, x, msg); }
    auto res = torn(b, x, true);
    if (!res.first && res.second) res = torn(b, x, false);
    if (!res.first) return untorn(b, x, msg);
    return SOLVE_OK;
  }
};

}  // namespace kso

#endif
