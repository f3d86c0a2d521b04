// ks_oracle.cpp — CPU FP64 oracle: simulation driver and C API (test infrastructure).
//
// Restates the reference's analysis package for the hot path:
//   (*Sim).solve            analysis/op.go:289-322
//   (*Sim).newton/converged analysis/newton.go:36-82
//   dcSolve + fallbacks     analysis/newton.go:95-311
//   (*Sim).OP               analysis/op.go:340-357
//   DC                      analysis/dc.go:51-130
//   (*Sim).tran             analysis/tran.go:95-243 (and the fixed-step mode of
//                           ks_tran_spec: steps of exactly `step`, no LTE control,
//                           no breakpoint landing, h/8 retry on Newton failure)
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
#include "ks_oracle.h"
#include "oracle_devices.hpp"
#include "oracle_bjt.hpp"
#include "oracle_mos.hpp"
#include "oracle_torn.hpp"

#include <atomic>
#include <chrono>
#include <cstdio>
#include <memory>
#include <thread>

namespace kso {

enum Err { E_OK = 0, E_SINGULAR = KS_STATUS_SINGULAR, E_NONFINITE = KS_STATUS_NONFINITE,
           E_NOCONV = KS_STATUS_NO_CONVERGENCE, E_TSTEP = KS_STATUS_TIMESTEP_TOO_SMALL,
           E_TOOMANY = KS_STATUS_TOO_MANY_STEPS, E_INTR = KS_STATUS_INTERRUPTED, E_LEDGER = KS_STATUS_LEDGER,
           E_BAD = 100 };

// em.Accumulator, em/energy.go:24-80: one set of classification rules for the
// operating point's ledger and every transient point's.
struct Acc {
  double in = 0, out = 0, diss = 0, store = 0, sup = 0, scale = 0;
  void port(int ch, double pw) {  // AddPort :33-51
    if (pw == 0) return;
    scale += std::fabs(pw);
    if (ch == CH_THERMAL && pw < 0) diss += -pw;
    else if (pw > 0) in += pw;
    else out += -pw;
  }
  void storage(double p) { store += p; scale += std::fabs(p); }  // AddStorage :54-57
  void supplied(double p) {  // AddModelSupplied :62-68
    if (p == 0) return;
    sup += p; scale += std::fabs(p);
  }
  double residual() const { return in + sup - out - diss - store; }  // :71-73
};

constexpr double kLedgerAbsFloor = 1e-21;  // output/result.go:96
constexpr double kGrossTol = 1e-3;         // analysis/tran.go:272

struct Opts {  // analysis.Options with defaults, analysis/op.go:91-110
  double reltol, abstol, vntol, gmin;
  int itl1, itl4;
  bool noGmin, noSource, noPT;
  int backend;
  double deadline;  // absolute steady-clock seconds, 0 = none
  explicit Opts(const ks_options* o) {
    reltol = o && o->reltol > 0 ? o->reltol : 1e-3;
    abstol = o && o->abstol > 0 ? o->abstol : 1e-12;
    vntol = o && o->vntol > 0 ? o->vntol : 1e-6;
    gmin = o && o->gmin > 0 ? o->gmin : 1e-12;
    itl1 = o && o->itl1 > 0 ? o->itl1 : 100;
    itl4 = o && o->itl4 > 0 ? o->itl4 : 10;
    noGmin = o && o->no_gmin_stepping; noSource = o && o->no_source_stepping; noPT = o && o->no_pseudo_transient;
    backend = o ? o->backend : 0;
    deadline = 0;
    if (o && o->deadline_s > 0) deadline = now() + o->deadline_s;
  }
  static double now() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
  }
  bool interrupted() const { return deadline > 0 && now() > deadline; }
};

struct Sim {
  std::vector<std::unique_ptr<Device>> devs;
  std::vector<int> reactive, nonlin, breakp, limiters;
  std::vector<char> isV;
  int n = 0, numNodes = 0;
  std::vector<double> x, xOld, rhs, ptPrev;
  double diagGmin = 0, ptG = 0;
  bool warm = false;
  std::unique_ptr<Matrix> M;
  LoadCtx lc;
  int iters = 0;  // total Newton iterations (solves)
  std::string msg;

  // newSim, analysis/op.go:160-208
  // kron.JacobianTearing as the linear solver (Options.Solver), when set
  const std::vector<std::pair<int, int>>* tornCuts = nullptr;
  double tornReuseTol = 0;
  TornStats tornStats;

  int build(const ks_topology* t, const double* v, double step, double stop, int backend) {
    numNodes = t->n_nodes;
    for (int e = 0; e < t->n_elem; e++) {
      const ks_element& el = t->elem[e];
      const double* p = v + el.param;
      Device* d = nullptr;
      switch (el.kind) {
        case KS_ELEM_R: { auto* r = new Resistor(p[0]); r->nodes[0] = el.node[0]; r->nodes[1] = el.node[1]; d = r; break; }
        case KS_ELEM_C: { auto* c = new Capacitor(p[0], p[1], el.flags & KS_F_HAS_IC); c->nodes[0] = el.node[0]; c->nodes[1] = el.node[1]; d = c; break; }
        case KS_ELEM_L: { auto* l = new Inductor(p[0], p[1], el.flags & KS_F_HAS_IC); l->nodes[0] = el.node[0]; l->nodes[1] = el.node[1]; d = l; break; }
        case KS_ELEM_V: case KS_ELEM_I: {
          SourceValue sv;
          sv.dc = p[KS_SRC_P_DC]; sv.hasDC = el.flags & KS_F_HAS_DC; sv.wkind = el.wave;
          sv.ac = std::polar(p[KS_SRC_P_ACMAG], p[KS_SRC_P_ACPHASE] * M_PI / 180);  // device/source.go:34
          sv.args.assign(p + KS_SRC_P_ARGS, p + KS_SRC_P_ARGS + el.nargs);
          if (el.kind == KS_ELEM_V) { auto* s = new VSource(); s->src = sv; s->nodes[0] = el.node[0]; s->nodes[1] = el.node[1]; d = s; }
          else { auto* s = new ISource(); s->src = sv; s->nodes[0] = el.node[0]; s->nodes[1] = el.node[1]; d = s; }
          break;
        }
        case KS_ELEM_D: { auto* dd = new Diode(p, el.flags & KS_F_HAS_BV); dd->nodes[0] = el.node[0]; dd->nodes[1] = el.node[1]; d = dd; break; }
        case KS_ELEM_Q: d = new BJT(p, el.flags & KS_F_PTYPE, el.node[0], el.node[1], el.node[2], el.node[3]); break;
        case KS_ELEM_M: {
          auto* m = new MOSFET(p, el.given, el.level, el.flags & KS_F_PTYPE, el.node[0], el.node[1], el.node[2], el.node[3]);
          if (m->bad) { delete m; msg = "device: unsupported element kind: MOSFET parameters"; return E_BAD; }
          d = m; break;
        }
        case KS_ELEM_E: case KS_ELEM_F: case KS_ELEM_G: case KS_ELEM_H: {
          auto* c = new Controlled(el.kind, p[KS_CTL_P_GAIN]);
          c->nodes[0] = el.node[0]; c->nodes[1] = el.node[1];
          if (el.kind == KS_ELEM_E || el.kind == KS_ELEM_G) { c->cn[0] = el.node[2]; c->cn[1] = el.node[3]; }
          else c->ctrlElem = el.node[2];
          d = c; break;
        }
        case KS_ELEM_K: {
          if (el.node[0] < 0 || el.node[0] >= t->n_elem || el.node[1] < 0 || el.node[1] >= t->n_elem ||
              t->elem[el.node[0]].kind != KS_ELEM_L || t->elem[el.node[1]].kind != KS_ELEM_L) {
            msg = "device: unsupported element kind: inductor not found"; return E_BAD;
          }
          const double l1 = v[t->elem[el.node[0]].param + KS_RCL_P_VALUE], l2 = v[t->elem[el.node[1]].param + KS_RCL_P_VALUE];
          auto* m = new Mutual(p[KS_K_P_COUPLING], l1, l2);
          m->l[0] = el.node[0]; m->l[1] = el.node[1];
          d = m; break;
        }
        case KS_ELEM_CN: case KS_ELEM_LN: {  // NewNonlinearCapacitor / NewNonlinearInductor
          const double* curve = p + KS_NL_P_ARGS + el.nargs;
          if (el.kind == KS_ELEM_CN) {
            auto* c = new NonlinearCapacitor(p[KS_NL_P_IC], el.flags & KS_F_HAS_IC);
            c->law.init(p[KS_NL_P_VALUE], curve, el.level, el.wave, p + KS_NL_P_ARGS, el.nargs);
            c->nodes[0] = el.node[0]; c->nodes[1] = el.node[1];
            d = c;
          } else {
            auto* l = new NonlinearInductor(p[KS_NL_P_IC], el.flags & KS_F_HAS_IC);
            l->law.init(p[KS_NL_P_VALUE], curve, el.level, el.wave, p + KS_NL_P_ARGS, el.nargs);
            l->nodes[0] = el.node[0]; l->nodes[1] = el.node[1];
            d = l;
          }
          break;
        }
        case KS_ELEM_S: case KS_ELEM_W: {
          auto* w = new Switch(el.kind == KS_ELEM_W, p);
          w->nodes[0] = el.node[0]; w->nodes[1] = el.node[1];
          if (el.kind == KS_ELEM_S) { w->cn[0] = el.node[2]; w->cn[1] = el.node[3]; }
          else w->ctrlElem = el.node[2];
          d = w; break;
        }
        default: msg = "device: unsupported element kind"; return E_BAD;
      }
      devs.emplace_back(d);
    }
    SetupCtx sc;
    sc.numNodes = numNodes; sc.step = step; sc.stop = stop;
    for (size_t i = 0; i < devs.size(); i++) {
      devs[i]->setup(sc);
      if (devs[i]->reactive()) reactive.push_back((int)i);
      if (devs[i]->nonlinear()) nonlin.push_back((int)i);
      if (devs[i]->breakpointer()) breakp.push_back((int)i);
      if (devs[i]->limiter()) limiters.push_back((int)i);
    }
    // Link, device/controlled.go:69-80 and device/mutual.go:54-70: the branches
    // a CCCS / CCVS senses and a mutual inductance couples
    for (size_t i = 0; i < devs.size(); i++) {
      if (auto* c = dynamic_cast<Controlled*>(devs[i].get())) {
        if (c->ctrlElem >= 0) {
          auto* vs = c->ctrlElem < (int)devs.size() ? dynamic_cast<VSource*>(devs[c->ctrlElem].get()) : nullptr;
          if (!vs) { msg = "device: unsupported element kind: controlling source not found"; return E_BAD; }
          c->ck = vs->branch;
        }
      } else if (auto* w = dynamic_cast<Switch*>(devs[i].get())) {  // Link, device/switch.go:120-130
        if (w->currentCtl) {
          auto* vs = w->ctrlElem >= 0 && w->ctrlElem < (int)devs.size() ? dynamic_cast<VSource*>(devs[w->ctrlElem].get()) : nullptr;
          if (!vs) { msg = "device: unsupported element kind: controlling source not found"; return E_BAD; }
          w->ck = vs->branch;
        }
      } else if (auto* m = dynamic_cast<Mutual*>(devs[i].get())) {
        auto* a = dynamic_cast<Inductor*>(devs[m->l[0]].get());
        auto* b = dynamic_cast<Inductor*>(devs[m->l[1]].get());
        if (!a || !b) { msg = "device: unsupported element kind: inductor not found"; return E_BAD; }
        m->k1 = a->branch; m->k2 = b->branch;
      }
    }
    n = sc.size();
    for (auto& d : devs) d->n = n;
    int be = backend == KS_BACKEND_AUTO ? (n < 30 ? KS_BACKEND_DENSE : KS_BACKEND_SPARSE) : backend;
    if (tornCuts) M.reset(new Torn(n, *tornCuts, tornReuseTol, &tornStats));
    else if (be == KS_BACKEND_SPARSE) M.reset(new Sparse(n));
    else M.reset(new Dense(n));
    x.assign(n, 0); xOld.assign(n, 0); rhs.assign(n, 0);
    isV.assign(n, 0);
    for (int i = 0; i < numNodes - 1; i++) isV[i] = 1;
    for (int i : sc.internal) isV[i] = 1;
    lc.M = M.get(); lc.rhs = rhs.data(); lc.n = n; lc.X = xOld.data(); lc.gmin = 1e-12;
    return E_OK;
  }

  int solve() {  // analysis/op.go:289-322
    iters++;
    xOld = x;
    lc.X = xOld.data();
    M->clear();
    std::fill(rhs.begin(), rhs.end(), 0.0);
    for (auto& d : devs) d->load(lc);
    if (ptG > 0) {
      double g = ptG;
      for (int i = 0; i < n; i++) {
        if (isV[i]) { M->add(i, i, g); rhs[i] += g * ptPrev[i]; }
        else { M->add(i, i, -g); rhs[i] -= g * ptPrev[i]; }
      }
    }
    if (diagGmin > 0) for (int i = 0; i < n; i++) if (isV[i]) M->add(i, i, diagGmin);
    std::string m;
    int e = M->solve(rhs.data(), x.data(), &m);
    if (e == SOLVE_SINGULAR) { msg = "solver: singular matrix" + m; return E_SINGULAR; }
    if (e == SOLVE_NONFINITE) { msg = "solver: non-finite value in system"; return E_NONFINITE; }
    return E_OK;
  }
  void accept(double t, int mode) { for (auto& d : devs) d->accept(x.data(), t, mode); }

  bool converged(const Opts& o) {  // analysis/newton.go:59-82
    for (int i : nonlin) if (devs[i]->limited()) return false;
    for (int i = 0; i < n; i++) {
      double tol = isV[i] ? o.vntol : o.abstol;
      tol += o.reltol * std::max(std::fabs(x[i]), std::fabs(xOld[i]));
      if (std::fabs(x[i] - xOld[i]) > tol) return false;
    }
    for (int i : nonlin) if (!devs[i]->convTest(x.data(), o.reltol, o.abstol)) return false;
    return true;
  }
  static bool retryable(int e) { return e == E_NOCONV || e == E_NONFINITE || e == E_SINGULAR; }

  int newton(int maxIter, const Opts& o) {  // analysis/newton.go:36-57
    lc.gmin = o.gmin;
    for (int it = 0; it < maxIter; it++) {
      if (o.interrupted()) { msg = "analysis interrupted: context deadline exceeded"; return E_INTR; }
      int e = solve();
      if (e) return e;
      if (nonlin.empty()) return E_OK;
      if (lc.initJct) { lc.initJct = false; continue; }
      if (converged(o)) return E_OK;
    }
    char buf[96]; snprintf(buf, sizeof buf, "analysis: no convergence after %d iterations", maxIter);
    msg = buf;
    return E_NOCONV;
  }

  int dcSolve(const Opts& o, const double* nodeset) {  // analysis/newton.go:95-128
    lc.initJct = !warm;
    if (!warm && nodeset) {  // applyNodeSet, analysis/newton.go:221-243
      std::fill(x.begin(), x.end(), 0.0);
      for (int i = 0; i < numNodes - 1; i++) x[i] = nodeset[i];
      for (int i : nonlin) devs[i]->accept(x.data(), 0, ModeOP);
      lc.initJct = false;
    }
    int err = newton(o.itl1, o);
    if (err == E_OK || nonlin.empty() || !retryable(err)) {
      warm = warm || err == E_OK;
      return err;
    }
    std::string first = msg;
    int firstErr = err;
    if (!o.noGmin) { err = gminStepping(o); if (err == E_OK) { warm = true; return E_OK; } }
    if (!o.noSource) { err = sourceStepping(o); if (err == E_OK) { warm = true; return E_OK; } }
    if (!o.noPT) { err = pseudoTransient(o); if (err == E_OK) { warm = true; return E_OK; } }
    msg = first + " (fallbacks failed: " + msg + ")";
    return firstErr;
  }

  int gminStepping(const Opts& o) {  // analysis/newton.go:134-176
    struct Reset { Sim* s; ~Reset() { s->diagGmin = 0; } } reset{this};
    std::vector<double> save(n, 0.0);
    std::fill(x.begin(), x.end(), 0.0);
    lc.initJct = true;
    double g = 1e-2, factor = 10.0;
    bool ok = false;
    for (int k = 0; k < 200; k++) {
      diagGmin = g;
      int err = newton(o.itl1, o);
      if (err == E_OK) {
        save = x;
        if (g == 0) return E_OK;
        ok = true;
        factor = std::min(factor * std::sqrt(factor), 10.0);
        if (g / factor < o.gmin) g = 0; else g /= factor;
        continue;
      } else if (!retryable(err)) return err;
      if (!ok) { msg = "analysis: no convergence: gmin stepping failed at its first step"; return E_NOCONV; }
      x = save;
      double prev = g * factor;
      if (g == 0) prev = o.gmin;
      factor = std::sqrt(factor);
      if (factor < 1.00005) {
        char buf[128]; snprintf(buf, sizeof buf, "analysis: no convergence: gmin stepping stalled at %g S", prev);
        msg = buf; return E_NOCONV;
      }
      g = prev / factor;
    }
    msg = "analysis: no convergence: gmin stepping exceeded 200 steps";
    return E_NOCONV;
  }

  int sourceStepping(const Opts& o) {  // analysis/newton.go:180-214
    struct Reset { Sim* s; ~Reset() { s->lc.srcStepping = false; s->lc.srcFact = 0; } } reset{this};
    std::vector<double> save(n, 0.0);
    std::fill(x.begin(), x.end(), 0.0);
    lc.srcStepping = true;
    double done = 0.0, step = 0.1;
    lc.srcFact = 0;
    int err = newton(o.itl1, o);
    if (err) return err;
    save = x;
    for (int k = 0; k < 1000; k++) {
      double f = std::min(done + step, 1.0);
      lc.srcFact = f;
      err = newton(o.itl1, o);
      if (err == E_OK) {
        if (f == 1) return E_OK;
        save = x;
        done = f; step = std::min(step * 1.5, 0.5);
        continue;
      } else if (!retryable(err)) return err;
      x = save;
      step /= 2;
      if (step < 1e-3) {
        char buf[128]; snprintf(buf, sizeof buf, "analysis: no convergence: source stepping stalled at %.4g of full value", done);
        msg = buf; return E_NOCONV;
      }
    }
    msg = "analysis: no convergence: source stepping exceeded 1000 steps";
    return E_NOCONV;
  }

  int pseudoTransient(const Opts& o) {  // analysis/newton.go:260-311
    struct Reset { Sim* s; ~Reset() { s->ptG = 0; } } reset{this};
    ptPrev.assign(n, 0.0);
    std::fill(x.begin(), x.end(), 0.0);
    lc.initJct = true;
    double h = 1e-6;
    int quiet = 0;
    for (int k = 0; k < 2000; k++) {
      ptG = 1 / h;
      int err = newton(o.itl1, o);
      if (err) {
        if (!retryable(err)) return err;
        x = ptPrev;
        h /= 4;
        if (h < 1e-15) { msg = "analysis: no convergence: pseudo-transient step too small"; return E_NOCONV; }
        continue;
      }
      bool moved = false;
      for (int i = 0; i < n; i++) {
        double tol = isV[i] ? o.vntol : o.abstol;
        if (std::fabs(x[i] - ptPrev[i]) > o.reltol * std::fabs(x[i]) + tol) { moved = true; break; }
      }
      ptPrev = x;
      if (!moved) quiet++; else quiet = 0;
      if (quiet >= 3 && h >= 1e6) { ptG = 0; return newton(o.itl1, o); }
      h = std::min(h * 2, 1e12);
    }
    msg = "analysis: no convergence: pseudo-transient exceeded 2000 steps";
    return E_NOCONV;
  }

  // polish, analysis/op.go:251-271: up to two more solves at the operating point.
  int polish() {
    if (nonlin.empty()) return E_OK;
    for (int k = 0; k < 2; k++) {
      int e = solve();
      if (e) return e;
      bool done = true;
      for (int i = 0; i < n; i++)
        if (std::fabs(x[i] - xOld[i]) > 1e-12 * std::max(1.0, std::fabs(x[i]))) done = false;
      if (done) break;
    }
    accept(0, ModeOP);
    return E_OK;
  }

  // AC, analysis/ac.go:76-150 (phasors only; the power ledger is not built):
  // the operating point, polish, then one complex solve per frequency.
  int ac(const Opts& o, const double* freqs, int nf, std::complex<double>* xout) {
    int e = op(o, nullptr);
    if (e) { msg = "AC operating point: " + msg; return e; }
    e = polish();
    if (e) { msg = "AC operating point: " + msg; return e; }
    std::vector<std::complex<double>> A((size_t)n * n), rhs(n), xc(n);
    ACCtx c;
    c.n = n; c.A = &A; c.rhs = &rhs;
    for (int k = 0; k < nf; k++) {
      std::fill(A.begin(), A.end(), 0.0);
      std::fill(rhs.begin(), rhs.end(), 0.0);
      c.omega = 2 * M_PI * freqs[k];
      for (auto& d : devs) d->loadAC(c);
      int se = cdense_solve(n, A, rhs, xc);
      if (se == SOLVE_SINGULAR) { msg = "solver: singular matrix"; return E_SINGULAR; }
      if (se == SOLVE_NONFINITE) { msg = "solver: non-finite value in system"; return E_NONFINITE; }
      for (int i = 0; i < n; i++) xout[(size_t)k * n + i] = xc[i];
    }
    return E_OK;
  }

  // roundoff, analysis/op.go:275-282: the residual round-off alone can make,
  // from the last linear system and the solution.
  double roundoff() {
    std::vector<double> ab(n);
    M->absProduct(x.data(), ab.data());
    double sum = 0;
    for (int i = 0; i < n; i++) sum += std::fabs(x[i]) * (ab[i] + std::fabs(rhs[i]));
    return 64 * 0x1p-52 * sum;
  }

  // result + em.BuildLedger, analysis/op.go:361-403 and em/energy.go:90-121:
  // element rows [ne][KS_RES_COLS] and the ledger [KS_LEDGER_COLS].
  void opResult(double* elem, double* ledger) {
    Acc a;
    for (size_t k = 0; k < devs.size(); k++) {
      OpPt o = devs[k]->operating(x.data());
      if (elem) {
        double* r = elem + k * KS_RES_COLS;
        r[KS_RES_VOLTAGE] = o.v; r[KS_RES_CURRENT] = o.i; r[KS_RES_POWER] = o.p; r[KS_RES_STORAGE_POWER] = o.ps;
        r[KS_RES_STORED_ENERGY] = o.w; r[KS_RES_EXTERIOR_POWER] = o.ext; r[KS_RES_MODEL_SUPPLIED] = o.sup;
      }
      a.port(o.ch, o.ext);
      if (o.stores) a.storage(o.ps);
      if (o.sup != 0) a.supplied(o.sup);
    }
    ledger[KS_LEDGER_INFLOW] = a.in; ledger[KS_LEDGER_OUTFLOW] = a.out; ledger[KS_LEDGER_DISSIPATION] = a.diss;
    ledger[KS_LEDGER_STORAGE_RATE] = a.store; ledger[KS_LEDGER_MODEL_SUPPLIED] = a.sup;
    ledger[KS_LEDGER_RESIDUAL] = a.residual(); ledger[KS_LEDGER_SCALE] = a.scale;
    ledger[KS_LEDGER_ROUNDOFF] = roundoff();
  }

  int op(const Opts& o, const double* nodeset) {  // analysis/op.go:340-357 (ledger: opResult)
    lc.mode = ModeOP; lc.time = 0;
    int e = dcSolve(o, nodeset);
    if (e) return e;
    accept(0, ModeOP);
    return E_OK;
  }

  double nextBreakpoint(double t) {  // analysis/tran.go:233-243
    double nb = kInf;
    for (int i : breakp) nb = std::min(nb, devs[i]->nextBreakpoint(t));
    return nb;
  }

  struct Rec {
    int cap = 0, npts = 0;
    double *t = nullptr, *x = nullptr, *i = nullptr;
    int n = 0, ne = 0;
    double start = 0;
    // the energy ledger of every point (recorder, analysis/tran.go:248-386); on
    // when `ledger` is set.  ip [cap][ne][2] current and absorbed power, lp
    // [cap][KS_TPOINT_COLS].
    bool ledger = false, check = true;
    double *ip = nullptr, *lp = nullptr;
    double peakScale = 0, worstAbs = 0, worstT = 0, tol = 1e-9;
    bool imposedFirst = false;
    int recorded = 0;  // points recorded (capacity aside)
    double tPrev = 0, yPrev[4] = {0, 0, 0, 0}, e[4] = {0, 0, 0, 0};  // trapezoid sums: in, out, dissipated, supplied
    double storedStart = 0, storedEnd = 0;
  };
  // recorder.record, analysis/tran.go:291-347.  Returns E_LEDGER when the
  // point is out of balance by more than kGrossTol of the run's peak power.
  int record(Rec& r, double t, bool imposed = false) {
    int err = E_OK;
    std::vector<OpPt> ops;
    Acc a;
    double stored = 0;
    if (r.ledger) {
      ops.resize(devs.size());
      for (size_t k = 0; k < devs.size(); k++) ops[k] = devs[k]->operating(x.data());
      for (size_t k = 0; k < devs.size(); k++) a.port(ops[k].ch, ops[k].ext);  // s.ports, element order
      for (size_t k = 0; k < devs.size(); k++) a.supplied(ops[k].sup);        // s.supply
      for (int k : reactive) { a.storage(ops[k].ps); stored += ops[k].w; }    // s.reactive
      if (a.scale > r.peakScale) r.peakScale = a.scale;
      double res = std::fabs(a.residual());
      if (!imposed && res > std::max(kLedgerAbsFloor, roundoff())) {
        if (res > r.worstAbs) { r.worstAbs = res; r.worstT = t; }
        double rr = res / r.peakScale;
        if (rr > kGrossTol && r.check) {
          char buf[192];
          snprintf(buf, sizeof buf, "em: energy ledger does not balance at t = %g s: residual %.3g W (relative %.3g)", t,
                   a.residual(), rr);
          msg = buf;
          err = E_LEDGER;
        }
      }
    }
    if (t < r.start) return err;
    if (r.ledger) {  // the running trapezoid sums of recorder.finish, :362-381
      double y[4] = {a.in, a.out, a.diss, a.sup};
      if (r.recorded == 0) { r.imposedFirst = imposed; r.storedStart = stored; }
      else
        for (int q = 0; q < 4; q++)
          r.e[q] += (r.recorded == 1 && r.imposedFirst) ? y[q] * (t - r.tPrev) : 0.5 * (y[q] + r.yPrev[q]) * (t - r.tPrev);
      for (int q = 0; q < 4; q++) r.yPrev[q] = y[q];
      r.tPrev = t; r.storedEnd = stored;
    }
    r.recorded++;
    if (r.npts >= r.cap) { r.npts++; return err; }
    int k = r.npts++;
    if (r.t) r.t[k] = t;
    if (r.x) for (int j = 0; j < n; j++) r.x[(size_t)k * n + j] = x[j];
    if (r.i) for (int j = 0; j < (int)devs.size(); j++) r.i[(size_t)k * devs.size() + j] = devs[j]->current(x.data());
    if (r.ledger && r.ip)
      for (size_t j = 0; j < devs.size(); j++) {
        r.ip[((size_t)k * devs.size() + j) * 2] = ops[j].i;
        r.ip[((size_t)k * devs.size() + j) * 2 + 1] = ops[j].p;
      }
    if (r.ledger && r.lp) {
      double* l = r.lp + (size_t)k * KS_TPOINT_COLS;
      l[KS_TPOINT_INFLOW] = a.in; l[KS_TPOINT_OUTFLOW] = a.out; l[KS_TPOINT_DISSIPATION] = a.diss;
      l[KS_TPOINT_STORAGE_RATE] = a.store; l[KS_TPOINT_MODEL_SUPPLIED] = a.sup; l[KS_TPOINT_RESIDUAL] = a.residual();
      l[KS_TPOINT_STORED_ENERGY] = stored;
    }
    return err;
  }
  // recorder.finish, analysis/tran.go:350-386: summary [KS_TSUM_COLS]; E_LEDGER
  // when the largest residual relative to the run's peak power exceeds tol.
  int finish(Rec& r, double* sum) {
    int err = E_OK;
    double mrr = 0;
    if (r.peakScale > 0) {
      mrr = r.worstAbs / r.peakScale;
      if (mrr > r.tol && r.check) {
        char buf[192];
        snprintf(buf, sizeof buf, "em: energy ledger does not balance at t = %g s: residual %.3g W (relative to the run's peak power %.3g)",
                 r.worstT, r.worstAbs, mrr);
        msg = buf;
        err = E_LEDGER;
      }
    }
    if (sum) {
      sum[KS_TSUM_MAX_RELATIVE_RESIDUAL] = mrr;
      sum[KS_TSUM_ENERGY_IN] = r.e[0]; sum[KS_TSUM_ENERGY_OUT] = r.e[1];
      sum[KS_TSUM_ENERGY_DISSIPATED] = r.e[2]; sum[KS_TSUM_ENERGY_MODEL_SUPPLIED] = r.e[3];
      sum[KS_TSUM_STORED_START] = r.storedStart; sum[KS_TSUM_STORED_END] = r.storedEnd;
      sum[KS_TSUM_INTEGRATION_MISMATCH] = r.e[0] + r.e[3] - r.e[1] - r.e[2] - (r.storedEnd - r.storedStart);
    }
    return err;
  }

  // analysis/tran.go:95-231 (adaptive) and the fixed-step mode.
  int tran(const ks_tran_spec& sp, const Opts& o, Rec& rec, int* stepsOut) {
    int method = sp.method == KS_METHOD_BE ? BE : TRAP;
    double chgtol = sp.chgtol > 0 ? sp.chgtol : 1e-14, trtol = sp.trtol > 0 ? sp.trtol : 7;
    double minStep = sp.min_step > 0 ? sp.min_step : 1e-12 * sp.stop;
    int maxSteps = sp.max_steps > 0 ? sp.max_steps : 1000000;
    bool fixed = sp.fixed_step != 0;
    double maxStep = sp.max_step;
    if (maxStep == 0) maxStep = std::min(sp.step, (sp.stop - sp.start) / 50);
    if (fixed) maxStep = sp.step;
    rec.start = sp.start;
    if (sp.uic) {
      for (auto& d : devs) d->setInitialCondition();
      lc.mode = ModeUICInit; lc.time = 0; lc.initJct = true;
      int e = newton(o.itl1, o);
      if (e) { msg = "initial conditions: " + msg; return e; }
      accept(0, ModeUICInit);
    } else {
      lc.mode = ModeTranOP; lc.time = 0;
      int e = dcSolve(o, nullptr);
      if (e) { msg = "transient operating point: " + msg; return e; }
      accept(0, ModeTranOP);
    }
    if (int le = record(rec, 0, sp.uic != 0)) { *stepsOut = 0; return le; }  // the UIC point is imposed: not checked
    TruncCtx tc{0, 0, BE, o.reltol, o.abstol, o.vntol, chgtol, trtol};
    double t = 0;
    double h = fixed ? sp.step : std::min(maxStep, std::min(sp.step, sp.stop / 100)) / 10;
    int order = BE;
    int accepted = 0;
    double eps = 1e-12 * sp.stop;
    std::vector<double> xAcc = x;
    long kgrid = 1;
    long ngrid = fixed ? std::lround(sp.stop / sp.step) : 0;
    auto reject = [&](double hNew) -> int {
      x = xAcc;
      if (hNew < minStep) {
        char buf[128]; snprintf(buf, sizeof buf, "analysis: timestep too small: %.3g s at t = %g s", hNew, t);
        msg = buf; return E_TSTEP;
      }
      return E_OK;
    };
    while (fixed ? kgrid <= ngrid : t < sp.stop - eps) {
      if (o.interrupted()) { msg = "analysis interrupted: context deadline exceeded"; *stepsOut = accepted; return E_INTR; }
      if (accepted >= maxSteps) {
        char buf[128]; snprintf(buf, sizeof buf, "analysis: too many time steps: %d accepted steps at t = %g s", accepted, t);
        msg = buf; *stepsOut = accepted; return E_TOOMANY;
      }
      double tn;
      bool hitBreak = false, onGrid = false;
      if (fixed) {
        double target = double(kgrid) * sp.step;
        tn = t + h;
        if (tn >= target - eps) { tn = target; onGrid = true; }
      } else {
        double nb = nextBreakpoint(t);
        tn = t + h;
        if (tn >= nb - eps) { tn = nb; hitBreak = true; }
        if (tn >= sp.stop - eps) { tn = sp.stop; hitBreak = false; }
      }
      h = tn - t;
      lc.mode = ModeTran; lc.time = tn; lc.h = h; lc.method = order;
      int e = newton(o.itl4, o);
      if (e) {
        if (!retryable(e) || nonlin.empty()) {
          char buf[64]; snprintf(buf, sizeof buf, "t = %g s: ", tn);
          msg = buf + msg; *stepsOut = accepted; return e;
        }
        h /= 8;
        int r = reject(h);
        if (r) { msg += " (Newton did not converge: analysis: no convergence)"; *stepsOut = accepted; return r; }
        order = BE;
        continue;
      }
      double proposal = kInf;
      if (!fixed) {
        tc.time = tn; tc.h = h; tc.method = order;
        for (int i : reactive) proposal = std::min(proposal, devs[i]->truncate(x.data(), tc));
        for (int i : limiters) proposal = std::min(proposal, devs[i]->limitStep(x.data(), tc));  // :186-190
        if (proposal < 0.9 * h) {
          h = std::max(proposal, h / 8);
          int r = reject(h);
          if (r) { *stepsOut = accepted; return r; }
          continue;
        }
      }
      accept(tn, ModeTran);
      if (!fixed || onGrid) {
        if (int le = record(rec, tn)) { *stepsOut = accepted; return le; }
      }
      xAcc = x;
      accepted++;
      t = tn;
      if (fixed) {
        if (onGrid) kgrid++;
        order = method;
        h = std::max(std::min(2 * h, maxStep), minStep);
        continue;
      }
      double next = std::min(proposal, 2 * h);
      next = std::min(next, maxStep);
      order = method;
      for (int i : limiters)  // :213-217: a switch changed state: restart like a corner
        if (devs[i]->restart()) hitBreak = true;
      if (hitBreak) {
        order = BE;
        double nb2 = nextBreakpoint(t);
        next = std::min(next, 0.1 * std::min(maxStep, nb2 - t));
      }
      h = std::max(next, minStep);
    }
    *stepsOut = accepted;
    return E_OK;
  }
};

static void copyMsg(const std::string& m, char* err, int errlen) {
  if (!err || errlen <= 0) return;
  snprintf(err, errlen, "%s", m.c_str());
}

}  // namespace kso

using namespace kso;

extern "C" int kso_unknowns(const ks_topology* t, const double* values, int32_t* n, int32_t* is_v) {
  Sim s;
  if (s.build(t, values, 0, 0, 0)) return KS_EINVAL;
  *n = s.n;
  if (is_v) for (int i = 0; i < s.n; i++) is_v[i] = s.isV[i];
  return KS_OK;
}

extern "C" int kso_op(const ks_topology* t, const double* values, const ks_options* o, const double* x0,
                      double* x_out, double* i_out, int32_t* iters, char* err, int errlen) {
  Sim s;
  Opts opt(o);
  if (s.build(t, values, 0, 0, opt.backend)) { copyMsg(s.msg, err, errlen); return KS_STATUS_NOT_RUN; }
  int e = s.op(opt, x0);
  if (iters) *iters = s.iters;
  if (x_out) for (int i = 0; i < s.n; i++) x_out[i] = s.x[i];
  if (i_out && e == E_OK) for (size_t i = 0; i < s.devs.size(); i++) i_out[i] = s.devs[i]->current(s.x.data());
  copyMsg(e ? s.msg : std::string(), err, errlen);
  return e;
}

// analysis.OP with its *output.Result: element rows, the ledger, and
// em.CheckLedger (analysis/op.go:340-357).
extern "C" int kso_op_results(const ks_topology* t, const double* values, const ks_options* o, const double* x0,
                              double* x_out, double* elem_out, double* ledger_out, int32_t* iters, char* err,
                              int errlen) {
  Sim s;
  Opts opt(o);
  if (s.build(t, values, 0, 0, opt.backend)) { copyMsg(s.msg, err, errlen); return KS_STATUS_NOT_RUN; }
  int e = s.op(opt, x0);
  if (iters) *iters = s.iters;
  if (x_out) for (int i = 0; i < s.n; i++) x_out[i] = s.x[i];
  if (e == E_OK) {
    double led[KS_LEDGER_COLS];
    s.opResult(elem_out, led);
    if (ledger_out) for (int i = 0; i < KS_LEDGER_COLS; i++) ledger_out[i] = led[i];
    // RelativeResidual (output/result.go:100-109) against the tolerance, CheckLedger em/energy.go:123-128
    double res = std::fabs(led[KS_LEDGER_RESIDUAL]), rr = 0;
    if (led[KS_LEDGER_SCALE] != 0 && res > std::max(kLedgerAbsFloor, led[KS_LEDGER_ROUNDOFF])) rr = res / led[KS_LEDGER_SCALE];
    double tol = o && o->ledger_tol > 0 ? o->ledger_tol : 1e-9;
    if (rr > tol && !(o && o->skip_energy_check)) {
      char buf[160];
      snprintf(buf, sizeof buf, "em: energy ledger does not balance: residual %.3g W (relative %.3g > %.3g)",
               led[KS_LEDGER_RESIDUAL], rr, tol);
      s.msg = buf;
      e = E_LEDGER;
    }
  }
  copyMsg(e ? s.msg : std::string(), err, errlen);
  return e;
}

extern "C" int kso_ac(const ks_topology* t, const double* values, const ks_options* o, const double* freqs, int nf,
                      double* x_out, char* err, int errlen) {
  Sim s;
  Opts opt(o);
  if (s.build(t, values, 0, 0, opt.backend)) { copyMsg(s.msg, err, errlen); return KS_STATUS_NOT_RUN; }
  std::vector<std::complex<double>> xc((size_t)nf * s.n);
  int e = s.ac(opt, freqs, nf, xc.data());
  if (x_out)
    for (size_t i = 0; i < xc.size(); i++) { x_out[2 * i] = xc[i].real(); x_out[2 * i + 1] = xc[i].imag(); }
  copyMsg(e ? s.msg : std::string(), err, errlen);
  return e;
}

// The left-looking LU's reach sets (solver/sparse.go:301-352: the depth-first
// search of Gilbert & Peierls from the rows of A(:, q[k]), pivotal rows leading on
// to the rows of their L column) for a fixed pivot sequence: prow[k] pivots at
// step k.  A is n x n row-major (A rows, A columns); out[i * n + k] = 1 when the
// row pivoting at step i is in the reach of step k (U above the diagonal, L
// below).  Returns the first step whose pivot row is outside its reach, or -1.
extern "C" int kso_reach_pattern(int n, const uint8_t* A, const int32_t* q, const int32_t* prow, uint8_t* out) {
  std::vector<int> pinv(n, -1), mark(n, -1), stack(n), pstack(n);
  for (int k = 0; k < n; k++) pinv[prow[k]] = k;
  std::vector<std::vector<int>> lcol(n);  // rows of L(:, j): its reach's rows pivoting after j
  std::fill(out, out + (size_t)n * n, 0);
  int bad = -1;
  for (int k = 0; k < n; k++) {
    std::vector<int> reach;
    for (int r = 0; r < n; r++) {
      if (!A[(size_t)r * n + q[k]] || mark[r] == k) continue;
      int head = 0;  // non-recursive DFS from r, as reach does
      stack[0] = r;
      while (head >= 0) {
        const int v = stack[head];
        const int j = pinv[v] < k ? pinv[v] : -1;  // pivotal before step k
        if (mark[v] != k) { mark[v] = k; pstack[head] = 0; }
        bool done = true;
        if (j >= 0) {
          for (int& p = pstack[head]; p < (int)lcol[j].size(); ) {
            const int w = lcol[j][p++];
            if (mark[w] == k) continue;
            stack[++head] = w;
            done = false;
            break;
          }
        }
        if (done) { head--; reach.push_back(v); }
      }
    }
    bool has_pivot = false;
    for (int v : reach) {
      out[(size_t)pinv[v] * n + k] = 1;
      if (pinv[v] > k) lcol[k].push_back(v);
      has_pivot = has_pivot || v == prow[k];
    }
    if (!has_pivot && bad < 0) bad = k;
  }
  return bad;
}

extern "C" int kso_dc2(const ks_topology* t, const double* values, const ks_options* o, int src,
                       const double* vals, int npts, int src2, const double* vals2, int npts2, double* x_out,
                       double* i_out, char* err, int errlen) {
  Sim s;
  Opts opt(o);
  if (s.build(t, values, 0, 0, opt.backend)) { copyMsg(s.msg, err, errlen); return KS_STATUS_NOT_RUN; }
  if (src < 0 || src >= (int)s.devs.size() || src2 >= (int)s.devs.size()) {
    copyMsg("analysis: swept source not found", err, errlen);
    return KS_STATUS_NOT_RUN;
  }
  const int total = npts * (src2 >= 0 ? npts2 : 1);
  for (int k = 0; k < total; k++) {  // analysis/dc.go:104-128: one OP per point, warm-started
    if (src2 >= 0) s.devs[src2]->setDCOverride(vals2[k / npts]);  // the outer sweep, :105-108
    s.devs[src]->setDCOverride(vals[k % npts]);
    int e = s.op(opt, nullptr);
    if (e) {
      char buf[64]; snprintf(buf, sizeof buf, "sweep = %g: ", vals[k % npts]);
      copyMsg(buf + s.msg, err, errlen);
      return e;
    }
    if (x_out) for (int i = 0; i < s.n; i++) x_out[(size_t)k * s.n + i] = s.x[i];
    if (i_out) for (size_t i = 0; i < s.devs.size(); i++) i_out[(size_t)k * s.devs.size() + i] = s.devs[i]->current(s.x.data());
  }
  s.devs[src]->clearDCOverride();
  if (src2 >= 0) s.devs[src2]->clearDCOverride();
  return E_OK;
}

extern "C" int kso_dc(const ks_topology* t, const double* values, const ks_options* o, int src,
                      const double* vals, int npts, double* x_out, double* i_out, char* err, int errlen) {
  return kso_dc2(t, values, o, src, vals, npts, -1, nullptr, 0, x_out, i_out, err, errlen);
}

extern "C" int kso_tran(const ks_topology* t, const double* values, const ks_tran_spec* spec,
                        const ks_options* o, int capacity, double* t_out, double* x_out, double* i_out,
                        int32_t* npts, int32_t* steps, int32_t* iters, char* err, int errlen) {
  Sim s;
  Opts opt(o);
  if (s.build(t, values, spec->step, spec->stop, opt.backend)) { copyMsg(s.msg, err, errlen); return KS_STATUS_NOT_RUN; }
  Sim::Rec rec;
  rec.cap = capacity; rec.t = t_out; rec.x = x_out; rec.i = i_out; rec.n = s.n; rec.ne = (int)s.devs.size();
  int st = 0;
  int e = s.tran(*spec, opt, rec, &st);
  if (npts) *npts = std::min(rec.npts, capacity);
  if (steps) *steps = st;
  if (iters) *iters = s.iters;
  copyMsg(e ? s.msg : std::string(), err, errlen);
  return e;
}

// The sparse backend's column order after an analysis (solver/sparse.go:154-187:
// minimumDegree of the pattern every load of the run stamped) and that pattern.
extern "C" int kso_sparse_order(const ks_topology* t, const double* values, const ks_tran_spec* spec,
                                const ks_options* o, int32_t* n_out, int32_t* order, uint8_t* pattern,
                                int32_t* pivots) {
  Sim s;
  ks_options oo = o ? *o : ks_options{};
  oo.backend = KS_BACKEND_SPARSE;
  Opts opt(&oo);
  if (s.build(t, values, spec ? spec->step : 0, spec ? spec->stop : 0, KS_BACKEND_SPARSE)) return KS_STATUS_NOT_RUN;
  int e;
  if (spec) {
    Sim::Rec rec;
    int st = 0;
    e = s.tran(*spec, opt, rec, &st);
  } else {
    e = s.op(opt, nullptr);
  }
  Sparse* sp = dynamic_cast<Sparse*>(s.M.get());
  if (!sp) return KS_STATUS_NOT_RUN;
  if (n_out) *n_out = s.n;
  if (order) for (int k = 0; k < s.n; k++) order[k] = sp->q[k];
  // the pivot rows of the run's last factorization, as A rows (the factor holds
  // rows in the column order's symmetric permutation)
  if (pivots) for (int k = 0; k < s.n; k++) pivots[k] = sp->valid ? sp->q[sp->prow[k]] : -1;
  if (pattern) {
    std::fill(pattern, pattern + (size_t)s.n * s.n, 0);
    for (size_t k = 0; k < sp->ri.size(); k++) pattern[(size_t)sp->ri[k] * s.n + sp->ci[k]] = 1;
  }
  return e;
}

// minimumDegree (solver/sparse.go:412-452) of an n x n byte pattern.
extern "C" void kso_min_degree(int n, const uint8_t* pattern, int32_t* order) {
  std::vector<int32_t> ri, ci;
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++)
      if (pattern[(size_t)i * n + j]) { ri.push_back(i); ci.push_back(j); }
  std::vector<int> q = minimumDegree(n, ri, ci);
  for (int k = 0; k < n; k++) order[k] = q[k];
}

// analysis.Tran with the Waveform's element series and ledger (recorder,
// analysis/tran.go:248-386).
extern "C" int kso_tran_results(const ks_topology* t, const double* values, const ks_tran_spec* spec,
                                const ks_options* o, int capacity, double* t_out, double* x_out, double* elem_out,
                                double* ledger_out, double* summary_out, int32_t* npts, int32_t* steps,
                                int32_t* iters, char* err, int errlen) {
  Sim s;
  Opts opt(o);
  if (s.build(t, values, spec->step, spec->stop, opt.backend)) { copyMsg(s.msg, err, errlen); return KS_STATUS_NOT_RUN; }
  Sim::Rec rec;
  rec.cap = capacity; rec.t = t_out; rec.x = x_out; rec.n = s.n; rec.ne = (int)s.devs.size();
  rec.ledger = true; rec.ip = elem_out; rec.lp = ledger_out;
  rec.check = !(o && o->skip_energy_check);
  rec.tol = o && o->ledger_tol > 0 ? o->ledger_tol : 1e-9;
  int st = 0;
  int e = s.tran(*spec, opt, rec, &st);
  int fe = s.finish(rec, summary_out);
  if (e == E_OK) e = fe;
  if (npts) *npts = std::min(rec.npts, capacity);
  if (steps) *steps = st;
  if (iters) *iters = s.iters;
  copyMsg(e ? s.msg : std::string(), err, errlen);
  return e;
}

// tearTerminals + NewJacobianTearing, kron/jacobian.go:92-232: the node-unknown
// pairs of the torn elements, with the reference's refusals.
extern "C" int kso_torn_cuts(const ks_topology* t, const int32_t* elems, int n_elems, int32_t* pairs, int cap,
                             int32_t* n_pairs, char* err, int errlen) {
  std::vector<std::pair<int, int>> out;
  std::vector<char> seen(t->n_elem, 0);
  for (int k = 0; k < n_elems; k++) {
    int e = elems[k];
    if (e < 0 || e >= t->n_elem) { copyMsg("kron: unsupported: no element", err, errlen); return KS_EINVAL; }
    char name[32];
    snprintf(name, sizeof name, "element %d", e);
    if (seen[e]) { copyMsg(std::string("kron: unsupported: ") + name + " is torn twice", err, errlen); return KS_EINVAL; }
    seen[e] = 1;
    const ks_element& el = t->elem[e];
    if (el.kind == KS_ELEM_V || el.kind == KS_ELEM_L || el.kind == KS_ELEM_E || el.kind == KS_ELEM_F ||
        el.kind == KS_ELEM_H || el.kind == KS_ELEM_K || el.kind == KS_ELEM_W || el.kind == KS_ELEM_LN) {  // tearTerminals, kron/jacobian.go:143-147
      copyMsg(std::string("kron: unsupported: tearing ") + name +
              ": its coupling runs through a branch-current unknown; tear a neighbouring element", err, errlen);
      return KS_EINVAL;
    }
    // a VCCS and an S switch: their control nodes too (:160-163)
    int nn = el.kind == KS_ELEM_Q || el.kind == KS_ELEM_M || el.kind == KS_ELEM_G || el.kind == KS_ELEM_S ? 4 : 2;
    std::vector<int> terms;
    for (int a = 0; a < nn; a++) {
      int node = el.node[a];
      if (node == 0) continue;
      bool dup = false;
      for (int m : terms) dup = dup || m == node;
      if (!dup) terms.push_back(node);
    }
    if (terms.size() < 2) {
      copyMsg(std::string("kron: unsupported: tearing ") + name + ": it connects to ground, so tearing it separates nothing",
              err, errlen);
      return KS_EINVAL;
    }
    for (size_t x = 0; x < terms.size(); x++)
      for (size_t y = x + 1; y < terms.size(); y++)
        if (terms[x] != terms[y]) out.push_back({terms[x] - 1, terms[y] - 1});
  }
  *n_pairs = (int32_t)out.size();
  for (size_t i = 0; i < out.size() && (int)i < cap; i++) { pairs[2 * i] = out[i].first; pairs[2 * i + 1] = out[i].second; }
  copyMsg(std::string(), err, errlen);
  return KS_OK;
}

static std::vector<std::pair<int, int>> cut_pairs(const int32_t* pairs, int n) {
  std::vector<std::pair<int, int>> c;
  for (int i = 0; i < n; i++) c.push_back({pairs[2 * i], pairs[2 * i + 1]});
  return c;
}

static void torn_stats_out(const TornStats& s, int64_t* out) {
  if (!out) return;
  out[0] = s.solves; out[1] = s.factors; out[2] = s.reuses; out[3] = s.stale;
  out[4] = s.fallbacks; out[5] = s.refines; out[6] = s.maxPieces;
}

extern "C" int kso_op_torn(const ks_topology* t, const double* values, const ks_options* o, const int32_t* pairs,
                           int n_pairs, double reuse_tol, double* x_out, int32_t* iters, int64_t* stats, char* err,
                           int errlen) {
  Sim s;
  Opts opt(o);
  auto cuts = cut_pairs(pairs, n_pairs);
  s.tornCuts = &cuts;
  s.tornReuseTol = reuse_tol;
  if (s.build(t, values, 0, 0, opt.backend)) { copyMsg(s.msg, err, errlen); return KS_STATUS_NOT_RUN; }
  int e = s.op(opt, nullptr);
  if (x_out) for (int i = 0; i < s.n; i++) x_out[i] = s.x[i];
  if (iters) *iters = s.iters;
  torn_stats_out(s.tornStats, stats);
  copyMsg(e ? s.msg : std::string(), err, errlen);
  return e;
}

extern "C" int kso_tran_torn(const ks_topology* t, const double* values, const ks_tran_spec* spec,
                             const ks_options* o, const int32_t* pairs, int n_pairs, double reuse_tol, int capacity,
                             double* t_out, double* x_out, int32_t* npts, int32_t* steps, int32_t* iters,
                             int64_t* stats, char* err, int errlen) {
  Sim s;
  Opts opt(o);
  auto cuts = cut_pairs(pairs, n_pairs);
  s.tornCuts = &cuts;
  s.tornReuseTol = reuse_tol;
  if (s.build(t, values, spec->step, spec->stop, opt.backend)) { copyMsg(s.msg, err, errlen); return KS_STATUS_NOT_RUN; }
  Sim::Rec rec;
  rec.cap = capacity; rec.t = t_out; rec.x = x_out; rec.i = nullptr; rec.n = s.n; rec.ne = (int)s.devs.size();
  int st = 0;
  int e = s.tran(*spec, opt, rec, &st);
  if (npts) *npts = std::min(rec.npts, capacity);
  if (steps) *steps = st;
  if (iters) *iters = s.iters;
  torn_stats_out(s.tornStats, stats);
  copyMsg(e ? s.msg : std::string(), err, errlen);
  return e;
}

// The plan buildPlan (kron/jacobian.go:296-389) makes for the Jacobian of one
// backward-Euler step of length h (the transient pattern): piece of each
// unknown and the coupling rows in the reference's order.
extern "C" int kso_torn_plan(const ks_topology* t, const double* values, const int32_t* pairs, int n_pairs, double h,
                             int32_t* piece_of, int32_t* n_pieces, int32_t* rows, int cap, int32_t* n_rows) {
  Sim s;
  Opts opt(nullptr);
  auto cuts = cut_pairs(pairs, n_pairs);
  s.tornCuts = &cuts;
  ks_tran_spec sp{};
  sp.step = h; sp.stop = h; sp.method = KS_METHOD_BE; sp.fixed_step = 1;
  if (s.build(t, values, sp.step, sp.stop, 0)) return KS_EINVAL;
  Sim::Rec rec;
  int st = 0;
  int e = s.tran(sp, opt, rec, &st);
  Torn* T = dynamic_cast<Torn*>(s.M.get());
  if (e || !T || !T->havePlan) return KS_EINVAL;
  for (int i = 0; i < s.n; i++) piece_of[i] = T->pieceOf[i];
  *n_pieces = (int32_t)T->pieces.size();
  *n_rows = (int32_t)T->rows.size();
  for (size_t a = 0; a < T->rows.size() && (int)a < cap; a++) rows[a] = T->rows[a];
  return KS_OK;
}

template <class F>
static void parallelFor(int nc, int nthreads, F f) {
  if (nthreads <= 0) nthreads = (int)std::thread::hardware_concurrency();
  if (nthreads < 1) nthreads = 1;
  std::atomic<int> next(0);
  auto worker = [&]() {
    for (;;) {
      int c = next.fetch_add(1);
      if (c >= nc) break;
      f(c);
    }
  };
  std::vector<std::thread> th;
  for (int i = 1; i < nthreads; i++) th.emplace_back(worker);
  worker();
  for (auto& x : th) x.join();
}

extern "C" int kso_batch_op(const ks_topology* t, const double* values, int nc, const ks_options* o,
                            const double* x0, int nthreads, double* x_out, int32_t* status, int32_t* iters) {
  int32_t n = 0;
  if (kso_unknowns(t, values, &n, nullptr)) return KS_EINVAL;
  parallelFor(nc, nthreads, [&](int c) {
    int32_t it = 0;
    status[c] = kso_op(t, values + (size_t)c * t->n_values, o, x0 ? x0 + (size_t)c * n : nullptr,
                       x_out ? x_out + (size_t)c * n : nullptr, nullptr, &it, nullptr, 0);
    if (iters) iters[c] = it;
  });
  return KS_OK;
}

extern "C" int kso_batch_tran(const ks_topology* t, const double* values, int nc, const ks_tran_spec* spec,
                              const ks_options* o, int nthreads, double* x_out, int32_t* status,
                              int32_t* steps, int32_t* iters) {
  int32_t n = 0;
  if (kso_unknowns(t, values, &n, nullptr)) return KS_EINVAL;
  if (!spec->fixed_step) return KS_EINVAL;
  int npts = (int)std::lround(spec->stop / spec->step) + 1;
  parallelFor(nc, nthreads, [&](int c) {
    std::vector<double> xs(x_out ? (size_t)npts * n : 0);
    int32_t np = 0, st = 0, it = 0;
    status[c] = kso_tran(t, values + (size_t)c * t->n_values, spec, o, x_out ? npts : 0, nullptr,
                         x_out ? xs.data() : nullptr, nullptr, &np, &st, &it, nullptr, 0);
    if (x_out)
      for (int k = 0; k < np; k++)
        for (int i = 0; i < n; i++) x_out[((size_t)k * nc + c) * n + i] = xs[(size_t)k * n + i];
    if (steps) steps[c] = st;
    if (iters) iters[c] = it;
  });
  return KS_OK;
}
