// oracle_solver.hpp — CPU FP64 linear solvers of the oracle (test infrastructure).
//
// Restates the reference's two real backends:
//   Dense  : solver/dense.go:80-177  (Doolittle, partial pivoting, column-relative
//            singularity test maxv <= col[k]*n*1e-14, non-finite checks)
//   Sparse : solver/sparse.go:114-452 (stamp-order slot replay, minimum degree on
//            A+A^T with ties to the lowest index, left-looking Gilbert-Peierls with
//            threshold pivoting and KLU diagonal preference DiagPivotTol = 1e-3)
// Auto picks Dense below 30 unknowns (solver/matrix.go:74-85).
#pragma once
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <map>
#include <set>
#include <algorithm>
#include <unordered_map>
#include <vector>
#include <string>
#include <limits>

namespace kso {

enum SolveErr { SOLVE_OK = 0, SOLVE_SINGULAR = 1, SOLVE_NONFINITE = 2 };

struct Matrix {
  virtual ~Matrix() {}
  virtual int size() const = 0;
  virtual void clear() = 0;
  virtual void add(int i, int j, double v) = 0;
  virtual int solve(const double* b, double* x, std::string* msg) = 0;
  virtual void absProduct(const double* x, double* y) = 0;
  virtual double at(int i, int j) const = 0;
};

static inline bool finite(double v) { return !std::isnan(v) && !std::isinf(v); }

// Dense LU (solver/dense.go).
struct Dense : Matrix {
  int n;
  std::vector<double> a, lu, y, col;
  std::vector<int> piv;
  explicit Dense(int n_) : n(n_), a(n_ * n_), lu(n_ * n_), y(n_), col(n_), piv(n_) {}
  int size() const override { return n; }
  void clear() override { std::fill(a.begin(), a.end(), 0.0); }
  void add(int i, int j, double v) override {
    if (i < 0 || j < 0 || i >= n || j >= n) return;
    a[i * n + j] += v;
  }
  double at(int i, int j) const override { return a[i * n + j]; }
  void absProduct(const double* x, double* yy) override {
    for (int i = 0; i < n; i++) {
      double s = 0;
      for (int j = 0; j < n; j++) s += std::fabs(a[i * n + j]) * std::fabs(x[j]);
      yy[i] = s;
    }
  }
  int solve(const double* b, double* x, std::string* msg) override {
    lu = a;
    double scale = 0;
    for (double v : lu) {
      if (!finite(v)) return SOLVE_NONFINITE;
      scale = std::max(scale, std::fabs(v));
    }
    if (scale == 0) return SOLVE_SINGULAR;
    std::fill(col.begin(), col.end(), 0.0);
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++) col[j] = std::max(col[j], std::fabs(lu[i * n + j]));
    for (int k = 0; k < n; k++) {
      int p = k;
      double maxv = std::fabs(lu[k * n + k]);
      for (int i = k + 1; i < n; i++) {
        double v = std::fabs(lu[i * n + k]);
        if (v > maxv) { maxv = v; p = i; }
      }
      if (maxv <= col[k] * double(n) * 1e-14) {
        if (msg) { char buf[96]; snprintf(buf, sizeof buf, ": pivot %d is %.3g", k, maxv); *msg = buf; }
        return SOLVE_SINGULAR;
      }
      piv[k] = p;
      if (p != k)
        for (int j = 0; j < n; j++) std::swap(lu[k * n + j], lu[p * n + j]);
      double pivot = lu[k * n + k];
      for (int i = k + 1; i < n; i++) {
        double f = lu[i * n + k] / pivot;
        lu[i * n + k] = f;
        if (f == 0) continue;
        for (int j = k + 1; j < n; j++) lu[i * n + j] -= f * lu[k * n + j];
      }
    }
    for (int i = 0; i < n; i++) y[i] = b[i];
    for (int k = 0; k < n; k++) if (piv[k] != k) std::swap(y[k], y[piv[k]]);
    for (int i = 0; i < n; i++) {
      double s = y[i];
      for (int j = 0; j < i; j++) s -= lu[i * n + j] * y[j];
      y[i] = s;
    }
    for (int i = n - 1; i >= 0; i--) {
      double s = y[i];
      for (int j = i + 1; j < n; j++) s -= lu[i * n + j] * x[j];
      x[i] = s / lu[i * n + i];
    }
    for (int i = 0; i < n; i++) if (!finite(x[i])) return SOLVE_NONFINITE;
    return SOLVE_OK;
  }
};

// Minimum degree on the pattern of A + A^T, ties to the lowest index
// (solver/sparse.go:412-452).
static std::vector<int> minimumDegree(int n, const std::vector<int32_t>& ri, const std::vector<int32_t>& ci) {
  std::vector<std::set<int32_t>> adj(n);
  for (size_t k = 0; k < ri.size(); k++) {
    int32_t i = ri[k], j = ci[k];
    if (i != j) { adj[i].insert(j); adj[j].insert(i); }
  }
  std::vector<char> gone(n, 0);
  std::vector<int> order;
  order.reserve(n);
  std::vector<int32_t> nbr;
  while ((int)order.size() < n) {
    int v = -1;
    size_t best = std::numeric_limits<size_t>::max();
    for (int i = 0; i < n; i++)
      if (!gone[i] && adj[i].size() < best) { v = i; best = adj[i].size(); }
    gone[v] = 1;
    order.push_back(v);
    nbr.assign(adj[v].begin(), adj[v].end());
    for (int32_t u : nbr) {
      adj[u].erase(v);
      for (int32_t w : nbr) if (w != u) adj[u].insert(w);
    }
    adj[v].clear();
  }
  return order;
}

// Sparse Gilbert-Peierls LU (solver/sparse.go).
struct Sparse : Matrix {
  int n;
  std::unordered_map<int64_t, int32_t> slot;
  std::vector<int32_t> ri, ci;
  std::vector<double> val;
  bool dirty = true;
  std::vector<int64_t> seqKey;
  std::vector<int32_t> seqSlot;
  size_t cursor = 0;
  std::vector<int32_t> q, qinv, ap, arow, aslot;
  std::vector<int32_t> lp, li, up, ui, pinv, prow;
  std::vector<double> lx, ux, udiag;
  std::vector<double> xw, w;
  std::vector<int32_t> xi, pstack, mark;
  int32_t gen = 0;
  bool valid = false;
  static constexpr double DiagPivotTol = 1e-3;

  explicit Sparse(int n_) : n(n_), q(n_), qinv(n_), ap(n_ + 1), lp(n_ + 1), up(n_ + 1),
      pinv(n_), prow(n_), udiag(n_), xw(n_), w(n_), xi(2 * n_), pstack(n_), mark(n_) {}
  int size() const override { return n; }
  void clear() override { std::fill(val.begin(), val.end(), 0.0); valid = false; cursor = 0; }
  void add(int i, int j, double v) override {
    if (i < 0 || j < 0 || i >= n || j >= n) return;
    int64_t key = int64_t(i) * n + j;
    size_t c = cursor++;
    if (c < seqKey.size() && seqKey[c] == key) { val[seqSlot[c]] += v; valid = false; return; }
    int32_t k;
    auto it = slot.find(key);
    if (it == slot.end()) {
      k = (int32_t)val.size();
      slot[key] = k;
      ri.push_back(i); ci.push_back(j); val.push_back(0);
      dirty = true;
    } else k = it->second;
    if (c < seqKey.size()) { seqKey[c] = key; seqSlot[c] = k; }
    else { seqKey.push_back(key); seqSlot.push_back(k); }
    val[k] += v;
    valid = false;
  }
  double at(int i, int j) const override {
    auto it = slot.find(int64_t(i) * n + j);
    return it == slot.end() ? 0.0 : val[it->second];
  }
  void absProduct(const double* x, double* y) override {
    for (int i = 0; i < n; i++) y[i] = 0;
    for (size_t k = 0; k < val.size(); k++) y[ri[k]] += std::fabs(val[k]) * std::fabs(x[ci[k]]);
  }
  void analyze() {
    std::vector<int> order = minimumDegree(n, ri, ci);
    for (int k = 0; k < n; k++) { q[k] = order[k]; qinv[order[k]] = k; }
    std::vector<int32_t> cnt(n + 1, 0);
    for (size_t k = 0; k < val.size(); k++) cnt[qinv[ci[k]] + 1]++;
    for (int k = 0; k < n; k++) cnt[k + 1] += cnt[k];
    for (int k = 0; k <= n; k++) ap[k] = cnt[k];
    size_t nz = val.size();
    arow.assign(nz, 0); aslot.assign(nz, 0);
    std::vector<int32_t> next(cnt.begin(), cnt.begin() + n);
    for (size_t k = 0; k < nz; k++) {
      int32_t c = qinv[ci[k]];
      int32_t p = next[c]++;
      arow[p] = qinv[ri[k]];
      aslot[p] = (int32_t)k;
    }
    for (int c = 0; c < n; c++) {
      std::vector<std::pair<int32_t, int32_t>> col;
      for (int32_t p = ap[c]; p < ap[c + 1]; p++) col.push_back({arow[p], aslot[p]});
      std::sort(col.begin(), col.end());
      for (int32_t p = ap[c], t = 0; p < ap[c + 1]; p++, t++) { arow[p] = col[t].first; aslot[p] = col[t].second; }
    }
    dirty = false;
  }
  bool marked(int32_t r) const { return mark[r] == gen; }
  int reach(int k) {
    gen++;
    if (gen == std::numeric_limits<int32_t>::max()) { std::fill(mark.begin(), mark.end(), 0); gen = 1; }
    int top = n;
    int32_t* stack = xi.data();
    for (int32_t p = ap[k]; p < ap[k + 1]; p++) {
      int32_t r = arow[p];
      if (mark[r] == gen) continue;
      int head = 0;
      stack[0] = r;
      while (head >= 0) {
        int32_t v = stack[head];
        int32_t j = pinv[v];
        if (mark[v] != gen) {
          mark[v] = gen;
          if (j >= 0) pstack[head] = lp[j];
        }
        bool done = true;
        if (j >= 0) {
          int32_t end = lp[j + 1];
          for (int32_t qq = pstack[head]; qq < end; qq++) {
            int32_t wv = li[qq];
            if (mark[wv] == gen) continue;
            pstack[head] = qq + 1;
            head++;
            stack[head] = wv;
            done = false;
            break;
          }
        }
        if (done) { head--; top--; xi[top] = v; }
      }
    }
    return top;
  }
  int factor(std::string* msg) {
    if (dirty) analyze();
    double scale = 0;
    for (double v : val) {
      if (!finite(v)) return SOLVE_NONFINITE;
      scale = std::max(scale, std::fabs(v));
    }
    if (scale == 0) return SOLVE_SINGULAR;
    std::fill(pinv.begin(), pinv.end(), -1);
    li.clear(); lx.clear(); ui.clear(); ux.clear();
    double* x = xw.data();
    for (int k = 0; k < n; k++) {
      lp[k] = (int32_t)li.size();
      up[k] = (int32_t)ui.size();
      int top = reach(k);
      for (int p = top; p < n; p++) x[xi[p]] = 0;
      double colMax = 0;
      for (int32_t p = ap[k]; p < ap[k + 1]; p++) {
        double v = val[aslot[p]];
        x[arow[p]] = v;
        colMax = std::max(colMax, std::fabs(v));
      }
      double tiny = colMax * double(n) * 1e-14;
      for (int p = top; p < n; p++) {
        int32_t r = xi[p];
        int32_t j = pinv[r];
        if (j < 0) continue;
        double xj = x[r];
        if (xj == 0) continue;
        for (int32_t qq = lp[j]; qq < lp[j + 1]; qq++) x[li[qq]] -= lx[qq] * xj;
      }
      int32_t piv = -1;
      double best = -1;
      for (int p = top; p < n; p++) {
        int32_t r = xi[p];
        if (pinv[r] >= 0) { ui.push_back(pinv[r]); ux.push_back(x[r]); continue; }
        double a = std::fabs(x[r]);
        if (a > best || (a == best && r < piv)) { best = a; piv = r; }
      }
      if (piv < 0 || best <= tiny) {
        lp[k + 1] = (int32_t)li.size(); up[k + 1] = (int32_t)ui.size();
        if (msg) { char buf[96]; snprintf(buf, sizeof buf, ": pivot %d is %.3g", k, std::max(best, 0.0)); *msg = buf; }
        return SOLVE_SINGULAR;
      }
      if (pinv[k] < 0 && marked(k) && std::fabs(x[k]) >= DiagPivotTol * best && std::fabs(x[k]) > tiny) piv = k;
      double pv = x[piv];
      udiag[k] = pv;
      pinv[piv] = k;
      prow[k] = piv;
      for (int p = top; p < n; p++) {
        int32_t r = xi[p];
        if (pinv[r] < 0) { li.push_back(r); lx.push_back(x[r] / pv); }
      }
    }
    lp[n] = (int32_t)li.size(); up[n] = (int32_t)ui.size();
    valid = true;
    return SOLVE_OK;
  }
  int solve(const double* b, double* x, std::string* msg) override {
    if (!valid) { int e = factor(msg); if (e) return e; }
    for (int i = 0; i < n; i++) w[qinv[i]] = b[i];
    double* y = xw.data();
    for (int k = 0; k < n; k++) {
      double yk = w[prow[k]];
      y[k] = yk;
      if (yk == 0) continue;
      for (int32_t p = lp[k]; p < lp[k + 1]; p++) w[li[p]] -= lx[p] * yk;
    }
    for (int k = n - 1; k >= 0; k--) {
      double zk = y[k] / udiag[k];
      y[k] = zk;
      if (zk == 0) continue;
      for (int32_t p = up[k]; p < up[k + 1]; p++) y[ui[p]] -= ux[p] * zk;
    }
    for (int k = 0; k < n; k++) {
      if (!finite(y[k])) return SOLVE_NONFINITE;
      x[q[k]] = y[k];
    }
    return SOLVE_OK;
  }
};

// CDense, solver/cdense.go:77-193: complex LU with partial pivoting on |entry|
// (hypot), the column-relative singular test of Dense, non-finite checks.
inline int cdense_solve(int n, std::vector<std::complex<double>> lu, const std::vector<std::complex<double>>& b,
                        std::vector<std::complex<double>>& x) {
  auto finite = [](std::complex<double> v) { return std::isfinite(v.real()) && std::isfinite(v.imag()); };
  double scale = 0;
  for (auto& v : lu) {
    if (!finite(v)) return SOLVE_NONFINITE;
    scale = std::max(scale, std::abs(v));
  }
  if (scale == 0) return SOLVE_SINGULAR;
  std::vector<double> col(n, 0.0);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) col[j] = std::max(col[j], std::abs(lu[(size_t)i * n + j]));
  std::vector<int> piv(n);
  for (int k = 0; k < n; k++) {
    int p = k;
    double maxv = std::abs(lu[(size_t)k * n + k]);
    for (int i = k + 1; i < n; i++) {
      double v = std::abs(lu[(size_t)i * n + k]);
      if (v > maxv) { maxv = v; p = i; }
    }
    if (maxv <= col[k] * (double)n * 1e-14) return SOLVE_SINGULAR;
    piv[k] = p;
    if (p != k)
      for (int j = 0; j < n; j++) std::swap(lu[(size_t)k * n + j], lu[(size_t)p * n + j]);
    std::complex<double> pivot = lu[(size_t)k * n + k];
    for (int i = k + 1; i < n; i++) {
      std::complex<double> f = lu[(size_t)i * n + k] / pivot;
      lu[(size_t)i * n + k] = f;
      if (f == 0.0) continue;
      for (int j = k + 1; j < n; j++) lu[(size_t)i * n + j] -= f * lu[(size_t)k * n + j];
    }
  }
  x = b;
  for (int k = 0; k < n; k++) if (piv[k] != k) std::swap(x[k], x[piv[k]]);
  for (int i = 0; i < n; i++) {
    std::complex<double> s = x[i];
    for (int j = 0; j < i; j++) s -= lu[(size_t)i * n + j] * x[j];
    x[i] = s;
  }
  for (int i = n - 1; i >= 0; i--) {
    std::complex<double> s = x[i];
    for (int j = i + 1; j < n; j++) s -= lu[(size_t)i * n + j] * x[j];
    x[i] = s / lu[(size_t)i * n + i];
  }
  for (auto& v : x) if (!finite(v)) return SOLVE_NONFINITE;
  return SOLVE_OK;
}

}  // namespace kso
