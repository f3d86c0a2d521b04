// oracle_devices.hpp — CPU FP64 device models of the oracle (test infrastructure).
//
// Each device restates the reference's Go device of the same name; the file:line
// of the reference function follows every method.  Element values arrive in the
// value-block layouts of include/kronspice_gpu.h (defaults and area scaling
// already applied, as NewDiode/NewBJT/NewMOSFET do when they read a model card).
#pragma once
#include "oracle_solver.hpp"
#include "../include/kronspice_gpu.h"

namespace kso {

constexpr double kChargeQ = 1.602176634e-19;  // device/diode.go:15
constexpr double kBoltzmann = 1.380649e-23;   // device/diode.go:16
constexpr double kTNom = 300.15;              // device/diode.go:18
constexpr double kInf = std::numeric_limits<double>::infinity();
constexpr double kE = 2.718281828459045235360287;
constexpr double kSqrt2 = 1.41421356237309504880168872;
constexpr double kPi = 3.14159265358979323846264338;

enum Mode { ModeOP = 0, ModeTranOP = 1, ModeUICInit = 2, ModeTran = 3 };  // device/device.go:103-116
enum Method { BE = 1, TRAP = 2 };                                         // device/device.go:119-124

struct LoadCtx {  // device/device.go:127-148
  Matrix* M = nullptr;
  double* rhs = nullptr;
  int n = 0;
  int mode = ModeOP;
  double time = 0, h = 0;
  int method = BE;
  const double* X = nullptr;
  bool initJct = false;
  double gmin = 1e-12;
  bool srcStepping = false;
  double srcFact = 0;
  void addRHS(int i, double v) { if (i >= 0 && i < n) rhs[i] += v; }
};

struct TruncCtx { double time, h; int method; double reltol, abstol, vntol, chgtol, trtol; };  // device/lte.go:10-19

struct History {  // device/lte.go:23-37
  double t[3] = {0, 0, 0}, q[3] = {0, 0, 0};
  int n = 0;
  void push(double tt, double qq) {
    t[2] = t[1]; t[1] = t[0]; t[0] = tt;
    q[2] = q[1]; q[1] = q[0]; q[0] = qq;
    if (n < 3) n++;
  }
  void reset() { n = 0; }
};

// lteStep, device/lte.go:50-85.
static double lteStep(const History& hist, double qn, double in, double inPrev, double absTol, const TruncCtx& tc) {
  int k = tc.method;
  if (k < 1 || k > 2 || hist.n < k + 1) return kInf;
  double ts[4] = {tc.time, hist.t[0], hist.t[1], hist.t[2]};
  double qs[4] = {qn, hist.q[0], hist.q[1], hist.q[2]};
  double dd[4] = {0, 0, 0, 0};
  for (int i = 0; i < k + 2; i++) dd[i] = qs[i];
  for (int order = 1; order <= k + 1; order++) {
    for (int i = 0; i + order <= k + 1; i++) {
      double den = ts[i] - ts[i + order];
      if (den == 0) return kInf;
      dd[i] = (dd[i] - dd[i + 1]) / den;
    }
  }
  double deriv = dd[0];
  double fact = 2.0, c = 0.5;
  if (k == 2) { fact = 6; c = 1.0 / 12; }
  double h = tc.h;
  double errI = c * std::pow(h, double(k)) * std::fabs(deriv * fact);
  if (errI == 0 || std::isnan(errI)) return kInf;
  double qmax = std::max(std::fabs(qn), std::fabs(hist.q[0]));
  double allowed = tc.trtol * std::max(tc.reltol * std::max(std::fabs(in), std::fabs(inPrev)) + absTol,
                                       tc.reltol * std::max(qmax, tc.chgtol) / h);
  return h * std::pow(allowed / errI, 1 / double(k));
}

static inline double at(const double* x, int n, int i) { return (i < 0 || i >= n) ? 0.0 : x[i]; }

// pnjlim, device/diode.go:214-226.
static double pnjlim(double vnew, double vold, double vt, double vcrit, bool* lim) {
  if (vnew > vcrit && std::fabs(vnew - vold) > 2 * vt) {
    *lim = true;
    if (vold > 0) {
      double arg = 1 + (vnew - vold) / vt;
      if (arg > 0) return vold + vt * std::log(arg);
      return vcrit;
    }
    return vt * std::log(vnew / vt);
  }
  *lim = false;
  return vnew;
}

struct SetupCtx {  // device/device.go:36-100
  int numNodes = 0, branches = 0;
  std::vector<int> internal;
  double step = 0, stop = 0;
  int unknown(int node) const { return node - 1; }
  int allocBranch() { return numNodes - 1 + branches++; }
  int allocUnknown() { int i = allocBranch(); internal.push_back(i); return i; }
  int size() const { return numNodes - 1 + branches; }
};

// Complex small-signal stamping, device.ACContext (device/device.go): Y = G + jwC and
// the AC source phasors.
struct ACCtx {
  int n = 0;
  double omega = 0;
  std::vector<std::complex<double>>* A = nullptr;  // row-major n x n
  std::vector<std::complex<double>>* rhs = nullptr;
  void add(int i, int j, std::complex<double> v) { if (i >= 0 && j >= 0) (*A)[(size_t)i * n + j] += v; }
  void addRHS(int i, std::complex<double> v) { if (i >= 0) (*rhs)[i] += v; }
  void stampY(int a, int b, std::complex<double> y) { add(a, a, y); add(b, b, y); add(a, b, -y); add(b, a, -y); }  // device/device.go:333-338
  // acBranch, device/bjt.go:713-726
  void branch(int a, int b, std::complex<double> y1, int p1, int n1, std::complex<double> y2, int p2, int n2) {
    if (y1 != 0.0) { add(a, p1, y1); add(a, n1, -y1); add(b, p1, -y1); add(b, n1, y1); }
    if (y2 != 0.0) { add(a, p2, y2); add(a, n2, -y2); add(b, p2, -y2); add(b, n2, y2); }
  }
};

// One element's operating point (device.OperatingPoint, device/device.go) with its
// ledger entries: ExteriorPower on its one modeled exterior port (channel ch; 0
// when the port is not modeled), ModelSuppliedPower (device.ModelSupplier),
// StoredEnergy and whether it is a device.Reactive element (its storage power
// enters the ledger).
enum { CH_ELECTRICAL = 0, CH_THERMAL = 1, CH_MECHANICAL = 2 };
struct OpPt {
  double v = 0, i = 0, p = 0, ps = 0;  // Voltage, Current, PowerAbsorbed, StoragePower
  double w = 0;                        // StoredEnergy
  double ext = 0;                      // ExteriorPower on channel ch
  double sup = 0;                      // ModelSuppliedPower
  int ch = CH_THERMAL;
  bool stores = false;
};

// integrate, device/bjt.go:607-627: 16-point Gauss-Legendre on n equal panels
// (nodes and weights of Abramowitz & Stegun, Table 25.4).
template <class F>
static double integrate(F&& f, double a, double b, int n) {
  static const double gx[8] = {0.0950125098376374, 0.2816035507792589, 0.4580167776572274, 0.6178762444026438,
                               0.7554044083550030, 0.8656312023878318, 0.9445750230732326, 0.9894009349916499};
  static const double gw[8] = {0.1894506104550685, 0.1826034150449236, 0.1691565193950025, 0.1495959888165767,
                               0.1246289712555339, 0.0951585116824928, 0.0622535239386479, 0.0271524594117541};
  double h = (b - a) / n, s = 0;
  for (int p = 0; p < n; p++) {
    double mid = a + (p + 0.5) * h, half = h / 2;
    for (int k = 0; k < 8; k++) s += gw[k] * (f(mid - half * gx[k]) + f(mid + half * gx[k]));
  }
  return s * h / 2;
}

struct Device {
  int n = 0;  // system size (set after setup)
  virtual void loadAC(ACCtx& c) {}
  virtual ~Device() {}
  virtual void setup(SetupCtx& c) = 0;
  virtual void load(LoadCtx& c) = 0;
  virtual double current(const double* x) = 0;  // Operating(x).Current
  virtual OpPt operating(const double* x) = 0;  // Operating, ExteriorPower, ModelSuppliedPower, StoredEnergy
  virtual void accept(const double* x, double t, int mode) {}
  virtual bool nonlinear() const { return false; }
  virtual bool limited() const { return false; }
  virtual bool convTest(const double* x, double reltol, double abstol) { return true; }
  virtual bool reactive() const { return false; }
  virtual double truncate(const double* x, const TruncCtx& tc) { return kInf; }
  virtual bool breakpointer() const { return false; }
  virtual double nextBreakpoint(double t) { return kInf; }
  virtual void setInitialCondition() {}
  virtual void setDCOverride(double v) {}
  virtual void clearDCOverride() {}
  // device.StepLimiter (device/switch.go:14-26)
  virtual bool limiter() const { return false; }
  virtual double limitStep(const double* x, const TruncCtx& tc) { return kInf; }
  virtual bool restart() const { return false; }
};

struct TwoTerm : Device {
  int nodes[2] = {0, 0}, u[2] = {-1, -1};
  void setupNodes(SetupCtx& c) { u[0] = c.unknown(nodes[0]); u[1] = c.unknown(nodes[1]); }
  double voltage(const double* x) const {  // device/device.go:310-319
    double v = 0;
    if (u[0] >= 0) v += x[u[0]];
    if (u[1] >= 0) v -= x[u[1]];
    return v;
  }
};

// Resistor, device/passive.go:65-95 (no ECE terms).
struct Resistor : TwoTerm {
  double R, g = 0;
  explicit Resistor(double r) : R(r) {}
  void setup(SetupCtx& c) override { setupNodes(c); g = 1 / R; }
  void load(LoadCtx& c) override {
    int a = u[0], b = u[1];
    c.M->add(a, a, g); c.M->add(b, b, g); c.M->add(a, b, -g); c.M->add(b, a, -g);
  }
  double current(const double* x) override { return voltage(x) * g; }
  OpPt operating(const double* x) override {  // device/passive.go:86-113
    OpPt o;
    o.v = voltage(x); o.i = o.v * g; o.p = o.v * o.i;
    if (R > 0) o.ext = -o.p;  // Joule heat out through the thermal port
    else o.sup = -o.p;        // negative resistance: model-supplied, thermal port not modeled
    return o;
  }
  void loadAC(ACCtx& c) override { c.stampY(u[0], u[1], g); }  // device/passive.go:116-123
};

// Capacitor, device/reactive.go:43-181.
struct Capacitor : TwoTerm {
  double C, ic; bool hasIC;
  double geq = 0, ihist = 0; bool tran = false;
  double vPrev = 0, iPrev = 0;
  History hist;
  Capacitor(double c, double ic_, bool has) : C(c), ic(ic_), hasIC(has) {}
  void setup(SetupCtx& c) override { setupNodes(c); }
  bool reactive() const override { return true; }
  void load(LoadCtx& c) override {
    int a = u[0], b = u[1];
    switch (c.mode) {
      case ModeOP: case ModeTranOP: tran = false; geq = 0; ihist = 0; return;
      case ModeUICInit: {
        tran = false;
        double g = 1e9;  // uicConductance, device/reactive.go:70
        c.M->add(a, a, g); c.M->add(b, b, g); c.M->add(a, b, -g); c.M->add(b, a, -g);
        c.addRHS(a, g * vPrev); c.addRHS(b, -g * vPrev);
        geq = 0; ihist = 0;
        return;
      }
    }
    tran = true;
    if (c.method == TRAP) { geq = 2 * C / c.h; ihist = -(geq * vPrev + iPrev); }
    else { geq = C / c.h; ihist = -geq * vPrev; }
    double g = geq;
    c.M->add(a, a, g); c.M->add(b, b, g); c.M->add(a, b, -g); c.M->add(b, a, -g);
    c.addRHS(a, -ihist); c.addRHS(b, ihist);
  }
  double current(const double* x) override { return tran ? geq * voltage(x) + ihist : 0.0; }
  OpPt operating(const double* x) override {  // :109-130, StoredEnergy :172-175
    OpPt o;
    o.v = voltage(x); o.i = current(x); o.p = o.v * o.i; o.ps = o.v * o.i;
    o.w = 0.5 * C * o.v * o.v;
    o.stores = true;
    return o;
  }
  void accept(const double* x, double t, int mode) override {  // :144-161
    if (mode == ModeUICInit) { iPrev = 0; hist.reset(); }
    else if (mode == ModeOP || mode == ModeTranOP) { vPrev = voltage(x); iPrev = 0; hist.reset(); }
    else { double v = voltage(x); double i = current(x); vPrev = v; iPrev = i; }
    hist.push(t, C * vPrev);
  }
  void setInitialCondition() override { vPrev = 0; iPrev = 0; if (hasIC) vPrev = ic; }
  void loadAC(ACCtx& c) override { c.stampY(u[0], u[1], std::complex<double>(0, c.omega * C)); }  // reactive.go:355-363
  double truncate(const double* x, const TruncCtx& tc) override {  // :178-181
    double v = voltage(x), i = current(x);
    return lteStep(hist, C * v, i, iPrev, tc.abstol, tc);
  }
};

// Inductor, device/reactive.go:198-352.
struct Inductor : TwoTerm {
  double L, ic; bool hasIC;
  int branch = -1;
  double vPrev = 0, iPrev = 0;
  History hist;
  Inductor(double l, double ic_, bool has) : L(l), ic(ic_), hasIC(has) {}
  void setup(SetupCtx& c) override { setupNodes(c); branch = c.allocBranch(); }
  bool reactive() const override { return true; }
  void load(LoadCtx& c) override {
    int a = u[0], b = u[1], k = branch;
    c.M->add(a, k, 1); c.M->add(b, k, -1);
    switch (c.mode) {
      case ModeOP: case ModeTranOP: c.M->add(k, a, 1); c.M->add(k, b, -1); return;
      case ModeUICInit: c.M->add(k, k, 1); c.addRHS(k, iPrev); return;
    }
    double req = L / c.h, r = -req * iPrev;
    if (c.method == TRAP) { req = 2 * L / c.h; r = -req * iPrev - vPrev; }
    c.M->add(k, a, 1); c.M->add(k, b, -1); c.M->add(k, k, -req);
    c.addRHS(k, r);
  }
  double current(const double* x) override { return x[branch]; }
  OpPt operating(const double* x) override {  // :289-300, StoredEnergy :340-342
    OpPt o;
    o.v = voltage(x); o.i = x[branch]; o.p = o.v * o.i; o.ps = o.v * o.i;
    o.w = 0.5 * L * o.i * o.i;
    o.stores = true;
    return o;
  }
  void accept(const double* x, double t, int mode) override {  // :312-329
    if (mode == ModeUICInit) { vPrev = 0; hist.reset(); }
    else if (mode == ModeOP || mode == ModeTranOP) { vPrev = 0; iPrev = x[branch]; hist.reset(); }
    else { vPrev = voltage(x); iPrev = x[branch]; }
    hist.push(t, L * iPrev);
  }
  void setInitialCondition() override { vPrev = 0; iPrev = 0; if (hasIC) iPrev = ic; }
  void loadAC(ACCtx& c) override {  // device/reactive.go:377-393
    int a = u[0], b = u[1], k = branch;
    c.add(a, k, 1); c.add(b, k, -1); c.add(k, a, 1); c.add(k, b, -1);
    c.add(k, k, std::complex<double>(0, -c.omega * L));
  }
  double truncate(const double* x, const TruncCtx& tc) override {  // :346-349
    return lteStep(hist, L * x[branch], voltage(x), vPrev, tc.vntol, tc);
  }
};

// Source waveform, device/waveform.go:10-239.
struct Wave {
  int kind = KS_WAVE_NONE;
  double a[7] = {0, 0, 0, 0, 0, 0, 0};
  std::vector<double> pwl;
  void resolve(int k, const double* args, int nargs, double step, double stop) {  // :25-66
    kind = k;
    if (step <= 0) step = 1e-9;
    if (stop <= 0) stop = 1e-6;
    auto arg = [&](int i, double def) { return i < nargs ? args[i] : def; };
    switch (k) {
      case KS_WAVE_PULSE: {
        double v[7] = {arg(0, 0), arg(1, 0), arg(2, 0), arg(3, step), arg(4, step), arg(5, stop), arg(6, stop)};
        for (int i = 0; i < 7; i++) a[i] = v[i];
        if (a[3] == 0) a[3] = step;
        if (a[4] == 0) a[4] = step;
        break;
      }
      case KS_WAVE_SIN: {
        double v[7] = {arg(0, 0), arg(1, 0), arg(2, 1 / stop), arg(3, 0), arg(4, 0), arg(5, 0), 0};
        for (int i = 0; i < 7; i++) a[i] = v[i];
        break;
      }
      case KS_WAVE_EXP: {
        double td1 = arg(2, 0);
        double v[7] = {arg(0, 0), arg(1, 0), td1, arg(3, step), arg(4, td1 + step), arg(5, step), 0};
        for (int i = 0; i < 7; i++) a[i] = v[i];
        if (a[3] == 0) a[3] = step;
        if (a[5] == 0) a[5] = step;
        break;
      }
      case KS_WAVE_PWL: pwl.assign(args, args + nargs); break;
    }
  }
  double value(double t) const {  // :69-126
    switch (kind) {
      case KS_WAVE_PULSE: {
        double v1 = a[0], v2 = a[1], td = a[2], tr = a[3], tf = a[4], pw = a[5], per = a[6];
        if (t < td) return v1;
        double tt = t - td;
        if (per > 0) tt = std::fmod(tt, per);
        if (tt < tr) return v1 + (v2 - v1) * tt / tr;
        if (tt < tr + pw) return v2;
        if (tt < tr + pw + tf) return v2 + (v1 - v2) * (tt - tr - pw) / tf;
        return v1;
      }
      case KS_WAVE_SIN: {
        double vo = a[0], va = a[1], f = a[2], td = a[3], theta = a[4], ph = a[5] * kPi / 180;
        if (t < td) return vo + va * std::sin(ph);
        double tt = t - td;
        return vo + va * std::exp(-tt * theta) * std::sin(2 * kPi * f * tt + ph);
      }
      case KS_WAVE_EXP: {
        double v1 = a[0], v2 = a[1], td1 = a[2], tau1 = a[3], td2 = a[4], tau2 = a[5];
        if (t < td1) return v1;
        if (t < td2) return v1 + (v2 - v1) * (1 - std::exp(-(t - td1) / tau1));
        return v1 + (v2 - v1) * (1 - std::exp(-(t - td1) / tau1)) + (v1 - v2) * (1 - std::exp(-(t - td2) / tau2));
      }
      case KS_WAVE_PWL: {
        const std::vector<double>& p = pwl;
        int n = (int)p.size() / 2;
        if (t <= p[0]) return p[1];
        if (t >= p[2 * (n - 1)]) return p[2 * n - 1];
        int k = 0;
        while (k < n && !(p[2 * k] > t)) k++;
        double t0 = p[2 * (k - 1)], v0 = p[2 * (k - 1) + 1], t1 = p[2 * k], v1 = p[2 * k + 1];
        if (t1 == t0) return v1;
        return v0 + (v1 - v0) * (t - t0) / (t1 - t0);
      }
    }
    return 0;
  }
  double slope(double t) const {  // :131-186
    switch (kind) {
      case KS_WAVE_PULSE: {
        double v1 = a[0], v2 = a[1], td = a[2], tr = a[3], tf = a[4], pw = a[5], per = a[6];
        if (t <= td) return 0;
        double tt = t - td;
        if (per > 0) {
          tt = std::fmod(tt, per);
          if (tt == 0) tt = per;  // the end of the previous period
        }
        if (tt <= tr) return (v2 - v1) / tr;
        if (tt <= tr + pw) return 0;
        if (tt <= tr + pw + tf) return (v1 - v2) / tf;
        return 0;
      }
      case KS_WAVE_SIN: {
        double va = a[1], f = a[2], td = a[3], theta = a[4], ph = a[5] * kPi / 180;
        if (t <= td) return 0;
        double tt = t - td, om = 2 * kPi * f;
        return va * std::exp(-tt * theta) * (om * std::cos(om * tt + ph) - theta * std::sin(om * tt + ph));
      }
      case KS_WAVE_EXP: {
        double v1 = a[0], v2 = a[1], td1 = a[2], tau1 = a[3], td2 = a[4], tau2 = a[5];
        if (t <= td1) return 0;
        double d = (v2 - v1) / tau1 * std::exp(-(t - td1) / tau1);
        if (t > td2) d += (v1 - v2) / tau2 * std::exp(-(t - td2) / tau2);
        return d;
      }
      case KS_WAVE_PWL: {
        const std::vector<double>& p = pwl;
        int n = (int)p.size() / 2;
        if (t <= p[0] || t > p[2 * (n - 1)]) return 0;
        int k = 0;  // segment k-1 -> k ends at or after t
        while (k < n && !(p[2 * k] >= t)) k++;
        double t0 = p[2 * (k - 1)], v0 = p[2 * (k - 1) + 1], t1 = p[2 * k], v1 = p[2 * k + 1];
        if (t1 == t0) return 0;
        return (v1 - v0) / (t1 - t0);
      }
    }
    return 0;
  }
  double nextBreakpoint(double t) const {  // :190-239
    const double rel = 1e-12;
    auto after = [&](double b) { return b > t + rel * std::max(std::fabs(t), 1e-15); };
    switch (kind) {
      case KS_WAVE_PULSE: {
        double td = a[2], tr = a[3], tf = a[4], pw = a[5], per = a[6];
        double edges[4] = {0, tr, tr + pw, tr + pw + tf};
        if (per <= 0) {
          for (double e : edges) if (after(td + e)) return td + e;
          return kInf;
        }
        double k = std::floor((t - td) / per);
        if (k < 0) k = 0;
        for (double kk = k; kk <= k + 1; kk++) {
          double base = td + kk * per;
          for (double e : edges) if (after(base + e)) return base + e;
        }
        return td + (k + 2) * per;
      }
      case KS_WAVE_SIN: if (after(a[3])) return a[3]; break;
      case KS_WAVE_EXP:
        if (after(a[2])) return a[2];
        if (after(a[4])) return a[4];
        break;
      case KS_WAVE_PWL: {
        int n = (int)pwl.size() / 2;
        for (int k = 0; k < n; k++) if (after(pwl[2 * k])) return pwl[2 * k];
        break;
      }
    }
    return kInf;
  }
};

// sourceValue, device/source.go:21-73.
struct SourceValue {
  double dc; bool hasDC;
  std::complex<double> ac = 0;  // AC phasor, magnitude at phase (degrees): device/source.go:34
  int wkind; std::vector<double> args;
  Wave w;
  double override_ = 0; bool overridden = false;
  void setup(const SetupCtx& c) { w.resolve(wkind, args.data(), (int)args.size(), c.step, c.stop); }
  double raw(const LoadCtx& c) const {
    if (overridden && c.mode == ModeOP) return override_;
    if (wkind == KS_WAVE_NONE) return dc;
    if (c.mode == ModeOP && hasDC) return dc;
    double t = c.mode == ModeTran ? c.time : 0;
    return w.value(t);
  }
  double at(const LoadCtx& c) const {
    double v = raw(c);
    if (c.srcStepping && c.mode != ModeTran) v *= c.srcFact;
    return v;
  }
  double nextBreakpoint(double t) const { return wkind == KS_WAVE_NONE ? kInf : w.nextBreakpoint(t); }
};

struct VSource : TwoTerm {  // device/source.go:75-121
  SourceValue src; int branch = -1; double value = 0;
  void setup(SetupCtx& c) override { setupNodes(c); branch = c.allocBranch(); src.setup(c); }
  void load(LoadCtx& c) override {
    int a = u[0], b = u[1], k = branch;
    value = src.at(c);
    c.M->add(a, k, 1); c.M->add(b, k, -1); c.M->add(k, a, 1); c.M->add(k, b, -1);
    c.addRHS(k, value);
  }
  double current(const double* x) override { return x[branch]; }
  OpPt operating(const double* x) override {  // :114-129: delivered power enters from the electrical exterior
    OpPt o;
    o.v = voltage(x); o.i = x[branch]; o.p = o.v * o.i; o.ext = -o.p; o.ch = CH_ELECTRICAL;
    return o;
  }
  bool breakpointer() const override { return true; }
  double nextBreakpoint(double t) override { return src.nextBreakpoint(t); }
  void setDCOverride(double v) override { src.override_ = v; src.overridden = true; }
  void clearDCOverride() override { src.overridden = false; }
  void loadAC(ACCtx& c) override {  // device/source.go:186-194
    int a = u[0], b = u[1], k = branch;
    c.add(a, k, 1); c.add(b, k, -1); c.add(k, a, 1); c.add(k, b, -1);
    c.addRHS(k, src.ac);
  }
};

struct ISource : TwoTerm {  // device/source.go:131-177
  SourceValue src; double value = 0;
  void loadAC(ACCtx& c) override { c.addRHS(u[0], -src.ac); c.addRHS(u[1], src.ac); }  // :208-212
  void setup(SetupCtx& c) override { setupNodes(c); src.setup(c); }
  void load(LoadCtx& c) override { value = src.at(c); c.addRHS(u[0], -value); c.addRHS(u[1], value); }
  double current(const double*) override { return value; }
  OpPt operating(const double* x) override {  // :163-177
    OpPt o;
    o.v = voltage(x); o.i = value; o.p = o.v * value; o.ext = -o.p; o.ch = CH_ELECTRICAL;
    return o;
  }
  bool breakpointer() const override { return true; }
  double nextBreakpoint(double t) override { return src.nextBreakpoint(t); }
  void setDCOverride(double v) override { src.override_ = v; src.overridden = true; }
  void clearDCOverride() override { src.overridden = false; }
};

// Controlled, device/controlled.go:29-162: E (VCVS), F (CCCS), G (VCCS), H (CCVS).
struct Controlled : TwoTerm {
  int kind;
  double gain;
  int cn[2] = {0, 0}, cu[2] = {-1, -1};  // control nodes and their unknowns (E, G)
  int ctrlElem = -1, ck = -1;            // controlling voltage source and its branch (F, H)
  int branch = -1;                       // own branch (E, H)
  Controlled(int k, double g) : kind(k), gain(g) {}
  bool voltageOutput() const { return kind == KS_ELEM_E || kind == KS_ELEM_H; }
  bool voltageControlled() const { return kind == KS_ELEM_E || kind == KS_ELEM_G; }
  void setup(SetupCtx& c) override {  // :55-66
    setupNodes(c);
    if (voltageControlled()) { cu[0] = c.unknown(cn[0]); cu[1] = c.unknown(cn[1]); }
    if (voltageOutput()) branch = c.allocBranch();
  }
  template <class ADD>
  void stamp(ADD add) const {  // :83-110
    const int p = u[0], nn = u[1];
    if (voltageOutput()) {
      const int k = branch;
      add(p, k, 1); add(nn, k, -1); add(k, p, 1); add(k, nn, -1);
      if (kind == KS_ELEM_E) { add(k, cu[0], -gain); add(k, cu[1], gain); }
      else add(k, ck, -gain);
      return;
    }
    if (kind == KS_ELEM_G) { add(p, cu[0], gain); add(p, cu[1], -gain); add(nn, cu[0], -gain); add(nn, cu[1], gain); }
    else { add(p, ck, gain); add(nn, ck, -gain); }
  }
  void load(LoadCtx& c) override { stamp([&](int i, int j, double v) { c.M->add(i, j, v); }); }
  void loadAC(ACCtx& c) override { stamp([&](int i, int j, double v) { c.add(i, j, v); }); }  // :143-148
  double control(const double* x) const {
    return voltageControlled() ? at(x, n, cu[0]) - at(x, n, cu[1]) : at(x, n, ck);
  }
  double current(const double* x) override { return voltageOutput() ? at(x, n, branch) : gain * control(x); }
  OpPt operating(const double* x) override {  // :123-140: model-supplied, no exterior port
    OpPt o;
    o.v = voltage(x); o.i = current(x); o.p = o.v * o.i; o.sup = -o.p; o.ch = CH_ELECTRICAL;
    return o;
  }
};

// Mutual, device/mutual.go:30-157 (no torsion terms): M = k sqrt(L1 L2) between
// the branch rows of two inductors.
struct Mutual : Device {
  double k, m;
  int l[2] = {-1, -1};  // the inductors' element indices
  int k1 = -1, k2 = -1;
  double i1Prev = 0, i2Prev = 0;
  Mutual(double kc, double l1, double l2) : k(kc), m(kc * std::sqrt(l1 * l2)) {}
  void setup(SetupCtx&) override {}
  bool reactive() const override { return true; }
  void load(LoadCtx& c) override {  // :75-118
    if (c.mode == ModeOP || c.mode == ModeTranOP || c.mode == ModeUICInit) return;
    double f = m / c.h;
    if (c.method == TRAP) f = 2 * m / c.h;
    c.M->add(k1, k2, -f); c.M->add(k2, k1, -f);
    c.addRHS(k1, -f * i2Prev); c.addRHS(k2, -f * i1Prev);
  }
  double current(const double*) override { return 0; }
  OpPt operating(const double* x) override {  // :120-133, StoredEnergy :137
    OpPt o;
    o.w = m * at(x, n, k1) * at(x, n, k2);
    o.stores = true;
    return o;
  }
  void accept(const double* x, double, int) override { i1Prev = at(x, n, k1); i2Prev = at(x, n, k2); }  // :134-137
  void loadAC(ACCtx& c) override {  // :146-151
    c.add(k1, k2, std::complex<double>(0, -c.omega * m));
    c.add(k2, k1, std::complex<double>(0, -c.omega * m));
  }
};

// stateLaw, device/nonlinear_reactive.go:15-249: y(x, t) = s(t) f(x) with f a
// piecewise-linear curve through the origin (or lin x) and s a scale waveform.
struct StateLaw {
  double lin = 0;
  std::vector<double> xs, ys, pre;  // knots, and the integral of f from xs[0] to each knot
  double g0 = 0, maxStep = 0, knotT = 0;
  int skind = KS_WAVE_NONE;
  std::vector<double> sargs;
  Wave scale;
  bool varies = false;
  void init(double value, const double* curve, int ncurve, int wk, const double* args, int nargs) {  // :47-64
    lin = value; skind = wk; varies = wk != KS_WAVE_NONE;
    sargs.assign(args, args + nargs);
    const int n = ncurve / 2;
    if (n < 2) return;
    xs.resize(n); ys.resize(n); pre.assign(n, 0.0);
    for (int i = 0; i < n; i++) { xs[i] = curve[2 * i]; ys[i] = curve[2 * i + 1]; }
    for (int k = 1; k < n; k++) pre[k] = pre[k - 1] + 0.5 * (ys[k - 1] + ys[k]) * (xs[k] - xs[k - 1]);
    g0 = cum(0);
    maxStep = 4 * (xs[n - 1] - xs[0]) / double(n - 1);
  }
  void resolve(double step, double stop) {  // :69-90 (the EXP bound is the host's)
    if (varies) scale.resolve(skind, sargs.data(), (int)sargs.size(), step, stop);
  }
  int segment(double x) const {  // :93-104
    const int n = (int)xs.size();
    const int k = (int)(std::lower_bound(xs.begin(), xs.end(), x) - xs.begin());
    if (k <= 0) return 1;
    if (k >= n) return n - 1;
    return k;
  }
  void f(double x, double* y, double* dy) const {  // :107-115
    if (xs.empty()) { *y = lin * x; *dy = lin; return; }
    const int k = segment(x);
    const double g = (ys[k] - ys[k - 1]) / (xs[k] - xs[k - 1]);
    *y = ys[k - 1] + g * (x - xs[k - 1]);
    *dy = g;
  }
  double cum(double x) const {  // :118-123
    const int k = segment(x);
    const double g = (ys[k] - ys[k - 1]) / (xs[k] - xs[k - 1]);
    const double d = x - xs[k - 1];
    return pre[k - 1] + ys[k - 1] * d + 0.5 * g * d * d;
  }
  double coenergy(double x) const { return xs.empty() ? 0.5 * lin * x * x : cum(x) - g0; }  // :126-131
  double energy(double x) const { double y, dy; f(x, &y, &dy); return x * y - coenergy(x); }  // :134-137
  double s(double t) const { return varies ? scale.value(t) : 1.0; }
  double sdot(double t) const { return varies ? scale.slope(t) : 0.0; }
  double limit(double x, double prev, bool* lim) const {  // :150-159
    *lim = false;
    if (maxStep == 0 || std::fabs(x - prev) <= maxStep) return x;
    const double lo = xs.front(), hi = xs.back();
    if ((x <= lo && prev <= lo) || (x >= hi && prev >= hi)) return x;
    *lim = true;
    return prev + std::copysign(maxStep, x - prev);
  }
  double knotStep(double x0, double x1, double h) const {  // :171-206
    if (xs.empty() || x0 == x1) return kInf;
    const int n = (int)xs.size();
    int k = (int)(std::lower_bound(xs.begin(), xs.end(), x0) - xs.begin());  // first knot >= x0
    double xk;
    if (x1 > x0) {
      while (k < n && xs[k] <= x0) k++;
      if (k == n || xs[k] >= x1) return kInf;
      xk = xs[k];
    } else {
      if (--k < 0 || xs[k] <= x1) return kInf;
      xk = xs[k];
    }
    double w = kInf;
    if (k > 0) w = xs[k] - xs[k - 1];
    if (k < n - 1) w = std::min(w, xs[k + 1] - xs[k]);
    if (std::fabs(xk - x0) <= 1e-3 * w) return kInf;
    const double fr = (xk - x0) / (x1 - x0);
    if (fr > 0.9) return kInf;
    return fr * h;
  }
  double truncate(double x0, double x1, const TruncCtx& tc) {  // :213-219
    const double p = knotStep(x0, x1, tc.h);
    if (p < kInf) knotT = tc.time - tc.h + p;
    return p;
  }
  void accepted(double t) { if (knotT != 0 && t >= knotT) knotT = 0; }  // :222-226
  double nextBreakpoint(double t) const {  // :228-237
    double b = varies ? scale.nextBreakpoint(t) : kInf;
    if (knotT > t && knotT < b) b = knotT;
    return b;
  }
};

// NonlinearCapacitor, device/nonlinear_reactive.go:263-465: q = s(t) Q(v), the
// charge integrated by the companion models.
struct NonlinearCapacitor : TwoTerm {
  StateLaw law;
  double ic; bool hasIC;
  double v0 = 0, iq = 0, geq = 0, a = 0, b = 0, sn = 1, sd = 0, t = 0, vIter = 0, omega = 0;
  bool tran = false, lim = false;
  double vPrev = 0, qPrev = 0, iPrev = 0, vAcc = 0, sAcc = 1;
  History hist;
  NonlinearCapacitor(double ic_, bool has) : ic(ic_), hasIC(has) {}
  void setup(SetupCtx& c) override { setupNodes(c); law.resolve(c.step, c.stop); }
  bool reactive() const override { return true; }
  bool nonlinear() const override { return !law.xs.empty(); }  // curvedCapacitor
  bool limited() const override { return lim; }
  bool breakpointer() const override { return true; }
  double nextBreakpoint(double tt) override { return law.nextBreakpoint(tt); }
  void load(LoadCtx& c) override {  // :318-357
    const int p = u[0], nn = u[1];
    lim = false; t = c.time; tran = false; geq = 0; iq = 0;
    if (c.mode == ModeOP || c.mode == ModeTranOP) return;
    if (c.mode == ModeUICInit) {
      const double g = 1e9;  // uicConductance
      c.M->add(p, p, g); c.M->add(nn, nn, g); c.M->add(p, nn, -g); c.M->add(nn, p, -g);
      c.addRHS(p, g * vPrev); c.addRHS(nn, -g * vPrev);
      return;
    }
    tran = true;
    const double v = law.limit(voltage(c.X), vIter, &lim);
    vIter = v; v0 = v;
    sn = law.s(c.time); sd = law.sdot(c.time);
    if (c.method == TRAP) { a = 2 / c.h; b = -2 * qPrev / c.h - iPrev; }
    else { a = 1 / c.h; b = -qPrev / c.h; }
    double q, dq;
    law.f(v, &q, &dq);
    iq = a * sn * q + b;
    geq = a * sn * dq;
    const double g = geq;
    c.M->add(p, p, g); c.M->add(nn, nn, g); c.M->add(p, nn, -g); c.M->add(nn, p, -g);
    const double ieq = iq - g * v;
    c.addRHS(p, -ieq); c.addRHS(nn, ieq);
  }
  double scalePower(double v) const { return (!tran || sd == 0) ? 0.0 : sd * law.coenergy(v); }  // :360-365
  double current(const double* x) override { return tran ? iq + geq * (voltage(x) - v0) : 0.0; }
  OpPt operating(const double* x) override {  // :368-376, StoredEnergy :410-413, ExteriorPower :432-437
    OpPt o;
    o.v = voltage(x); o.i = current(x); o.p = o.v * o.i;
    const double sp = scalePower(o.v);
    o.ps = o.p - sp;
    o.w = law.s(t) * law.energy(o.v);
    o.stores = true;
    o.ch = CH_MECHANICAL;
    if (law.varies) o.ext = -sp;
    return o;
  }
  void accept(const double* x, double tt, int mode) override {  // :379-399
    double v = voltage(x);
    if (mode == ModeUICInit) { v = vPrev; iPrev = 0; hist.reset(); }
    else if (mode == ModeOP || mode == ModeTranOP) { iPrev = 0; hist.reset(); }
    else iPrev = iq + geq * (v - v0);
    vPrev = vIter = vAcc = v;
    sAcc = law.s(tt);
    double q, dq;
    law.f(v, &q, &dq);
    qPrev = sAcc * q;
    hist.push(tt, qPrev);
    law.accepted(tt);
  }
  void setInitialCondition() override { vPrev = 0; iPrev = 0; if (hasIC) vPrev = ic; }  // :402-407
  double truncate(const double* x, const TruncCtx& tc) override {  // :417-424
    const double v = voltage(x), i = current(x);
    double q, dq;
    law.f(v, &q, &dq);
    const double h = lteStep(hist, law.s(tc.time) * q, i, iPrev, tc.abstol, tc);
    return std::min(h, law.truncate(vAcc, v, tc));
  }
  bool convTest(const double* x, double reltol, double abstol) override {  // :458-468
    if (!tran) return true;
    const double v = voltage(x), ihat = iq + geq * (v - v0);
    double q, dq;
    law.f(v, &q, &dq);
    const double i = a * sn * q + b;
    return std::fabs(ihat - i) <= reltol * std::max(std::fabs(i), std::fabs(ihat)) + abstol;
  }
  void loadAC(ACCtx& c) override {  // :440-449
    double q, dq;
    law.f(vAcc, &q, &dq);
    c.stampY(u[0], u[1], std::complex<double>(0, c.omega * sAcc * dq));
  }
};

// NonlinearInductor, device/nonlinear_reactive.go:470-682: flux linkage
// s(t) L(i) with a branch current, the flux integrated by the companion models.
struct NonlinearInductor : TwoTerm {
  StateLaw law;
  double ic; bool hasIC;
  int branch = -1;
  double i0 = 0, lam0 = 0, ld = 0, a = 0, b = 0, sn = 1, sd = 0, t = 0, iIter = 0;
  bool tran = false, lim = false;
  double vPrev = 0, iPrev = 0, lamPrev = 0, iAcc = 0, sAcc = 1;
  History hist;
  NonlinearInductor(double ic_, bool has) : ic(ic_), hasIC(has) {}
  void setup(SetupCtx& c) override { setupNodes(c); branch = c.allocBranch(); law.resolve(c.step, c.stop); }
  bool reactive() const override { return true; }
  bool nonlinear() const override { return !law.xs.empty(); }  // curvedInductor
  bool limited() const override { return lim; }
  bool breakpointer() const override { return true; }
  double nextBreakpoint(double tt) override { return law.nextBreakpoint(tt); }
  void load(LoadCtx& c) override {  // :531-566
    const int p = u[0], nn = u[1], k = branch;
    lim = false; t = c.time; tran = false;
    c.M->add(p, k, 1); c.M->add(nn, k, -1);
    if (c.mode == ModeOP || c.mode == ModeTranOP) { c.M->add(k, p, 1); c.M->add(k, nn, -1); return; }
    if (c.mode == ModeUICInit) { c.M->add(k, k, 1); c.addRHS(k, iPrev); return; }
    tran = true;
    const double i = law.limit(at(c.X, n, k), iIter, &lim);
    iIter = i; i0 = i;
    sn = law.s(c.time); sd = law.sdot(c.time);
    if (c.method == TRAP) { a = 2 / c.h; b = -2 * lamPrev / c.h - vPrev; }
    else { a = 1 / c.h; b = -lamPrev / c.h; }
    double lam, dl;
    law.f(i, &lam, &dl);
    lam0 = sn * lam; ld = sn * dl;
    c.M->add(k, p, 1); c.M->add(k, nn, -1); c.M->add(k, k, -a * ld);
    c.addRHS(k, a * (lam0 - ld * i0) + b);
  }
  double scalePower(double i) const { return (!tran || sd == 0) ? 0.0 : sd * law.coenergy(i); }  // :569-574
  double current(const double* x) override { return at(x, n, branch); }
  OpPt operating(const double* x) override {  // :577-582, StoredEnergy :612-615, ExteriorPower :632-637
    OpPt o;
    o.v = voltage(x); o.i = at(x, n, branch); o.p = o.v * o.i;
    const double sp = scalePower(o.i);
    o.ps = o.p - sp;
    o.w = law.s(t) * law.energy(o.i);
    o.stores = true;
    o.ch = CH_MECHANICAL;
    if (law.varies) o.ext = -sp;
    return o;
  }
  void accept(const double* x, double tt, int mode) override {  // :585-602
    double i = at(x, n, branch), v = voltage(x);
    if (mode == ModeUICInit) { i = iPrev; v = 0; hist.reset(); }
    else if (mode == ModeOP || mode == ModeTranOP) { v = 0; hist.reset(); }
    iPrev = iIter = iAcc = i; vPrev = v;
    sAcc = law.s(tt);
    double lam, dl;
    law.f(i, &lam, &dl);
    lamPrev = sAcc * lam;
    hist.push(tt, lamPrev);
    law.accepted(tt);
  }
  void setInitialCondition() override { vPrev = 0; iPrev = 0; if (hasIC) iPrev = ic; }  // :605-610
  double truncate(const double* x, const TruncCtx& tc) override {  // :620-625
    const double i = at(x, n, branch), v = voltage(x);
    double lam, dl;
    law.f(i, &lam, &dl);
    const double h = lteStep(hist, law.s(tc.time) * lam, v, vPrev, tc.vntol, tc);
    return std::min(h, law.truncate(iAcc, i, tc));
  }
  bool convTest(const double* x, double reltol, double) override {  // :672-682 (vntol 1e-6)
    if (!tran) return true;
    const double i = at(x, n, branch), vhat = a * (lam0 + ld * (i - i0)) + b;
    double lam, dl;
    law.f(i, &lam, &dl);
    const double v = a * sn * lam + b;
    return std::fabs(vhat - v) <= reltol * std::max(std::fabs(v), std::fabs(vhat)) + 1e-6;
  }
  void loadAC(ACCtx& c) override {  // :640-651
    const int p = u[0], nn = u[1], k = branch;
    double lam, dl;
    law.f(iAcc, &lam, &dl);
    c.add(p, k, 1); c.add(nn, k, -1); c.add(k, p, 1); c.add(k, nn, -1);
    c.add(k, k, std::complex<double>(0, -c.omega * sAcc * dl));
  }
};

// Switch, device/switch.go:28-332: S (voltage-controlled) and W (current-
// controlled).  Abrupt (VH >= 0): RON or ROFF with hysteresis about VT, the
// state referred to the last accepted solution, held through a transient step;
// smooth (VH < 0): ln R a cubic in the control between VT - |VH| and VT + |VH|.
struct Switch : TwoTerm {
  bool currentCtl;
  int cn[2] = {0, 0}, cu[2] = {-1, -1};  // control nodes and their unknowns (S)
  int ctrlElem = -1, ck = -1;            // controlling voltage source and its branch (W)
  double vt, vh, ron, roff;
  bool smooth = false;
  double lmean = 0, lratio = 0;  // ln sqrt(RON ROFF), ln(RON / ROFF)
  bool initOn, on, accOn, accepted = false, frozen = false, flipped = false;
  double g = 0, k = 0, c0 = 0, cAcc = 0;  // linearization i = g v + k (c - c0)
  Switch(bool cur, const double* p) : currentCtl(cur) {  // NewSwitch, :92-108
    vt = p[KS_SW_P_VT]; vh = p[KS_SW_P_VH]; ron = p[KS_SW_P_RON]; roff = p[KS_SW_P_ROFF];
    if (vh < 0) {
      smooth = true;
      vh = -vh;
      lmean = std::log(std::sqrt(ron * roff));
      lratio = std::log(ron / roff);
    }
    initOn = p[KS_SW_P_ON] == 1;
    on = accOn = initOn;
  }
  void setup(SetupCtx& c) override {  // :111-117
    setupNodes(c);
    if (!currentCtl) { cu[0] = c.unknown(cn[0]); cu[1] = c.unknown(cn[1]); }
  }
  bool nonlinear() const override { return true; }
  bool limiter() const override { return true; }
  double control(const double* x) const {  // :132-137
    return currentCtl ? at(x, n, ck) : at(x, n, cu[0]) - at(x, n, cu[1]);
  }
  bool next(double c, bool prev) const {  // :140-148
    if (c > vt + vh) return true;
    if (c < vt - vh) return false;
    return prev;
  }
  void smoothG(double c, double* gg, double* dg) const {  // :151-162
    double xx = (c - vt) / vh;
    if (xx >= 1) { *gg = 1 / ron; *dg = 0; return; }
    if (xx <= -1) { *gg = 1 / roff; *dg = 0; return; }
    *gg = std::exp(-(lmean + lratio * (3 * xx - xx * xx * xx) / 4));
    *dg = -*gg * lratio * 3 * (1 - xx * xx) / (4 * vh);
  }
  double vab(const double* x) const { return at(x, n, u[0]) - at(x, n, u[1]); }
  template <class ADD>
  void stampCtrl(ADD add, double kk) const {  // :214-226
    const int a = u[0], b = u[1];
    if (currentCtl) { add(a, ck, kk); add(b, ck, -kk); return; }
    add(a, cu[0], kk); add(a, cu[1], -kk); add(b, cu[0], -kk); add(b, cu[1], kk);
  }
  void load(LoadCtx& c) override {  // :174-212
    const int a = u[0], b = u[1];
    if (smooth) {
      double cc = control(c.X), v = vab(c.X);
      if (c.initJct) { cc = initOn ? vt + vh : vt - vh; v = 0; }
      double gg, dg;
      smoothG(cc, &gg, &dg);
      g = gg; k = dg * v; c0 = cc;
      c.M->add(a, a, g); c.M->add(b, b, g); c.M->add(a, b, -g); c.M->add(b, a, -g);
      if (k != 0) {
        stampCtrl([&](int i, int j, double vv) { c.M->add(i, j, vv); }, k);
        const double j0 = -k * cc;
        c.addRHS(a, -j0); c.addRHS(b, j0);
      }
      return;
    }
    frozen = c.mode == ModeTran;
    if (c.initJct || frozen) on = accOn;
    else on = next(control(c.X), accOn);
    g = on ? 1 / ron : 1 / roff;
    k = 0;
    c.M->add(a, a, g); c.M->add(b, b, g); c.M->add(a, b, -g); c.M->add(b, a, -g);
  }
  bool convTest(const double* x, double reltol, double abstol) override {  // :231-243
    const double cc = control(x);
    if (!smooth) return frozen || next(cc, accOn) == on;
    const double v = vab(x);
    double gg, dg;
    smoothG(cc, &gg, &dg);
    const double ihat = g * v + k * (cc - c0), i = gg * v;
    return std::fabs(ihat - i) <= reltol * std::max(std::fabs(i), std::fabs(ihat)) + abstol;
  }
  double current(const double* x) override { return g * vab(x) + k * (control(x) - c0); }
  OpPt operating(const double* x) override {  // :246-250, ExteriorPower :304-310
    OpPt o;
    o.v = vab(x); o.i = current(x); o.p = o.v * o.i;
    o.ext = -o.p;  // Joule heat out through the thermal port
    return o;
  }
  void accept(const double* x, double, int) override {  // :253-261
    const double c = control(x);
    cAcc = c; accepted = true;
    if (!smooth) {
      const bool o = next(c, accOn);
      flipped = o != accOn;
      accOn = on = o;
    }
  }
  bool restart() const override { return flipped; }  // :264
  double limitStep(const double* x, const TruncCtx& tc) override {  // :268-285
    if (smooth || !accepted) return kInf;
    const double c = control(x);
    if (next(c, accOn) == accOn || c == cAcc) return kInf;
    const double th = accOn ? vt - vh : vt + vh;
    const double frac = (th - cAcc) / (c - cAcc);
    if (!(frac > 0) || frac >= 0.99) return kInf;
    return tc.h * std::min(frac + 0.005, 1.0);
  }
  void loadAC(ACCtx& c) override {  // :314-329
    c.stampY(u[0], u[1], std::complex<double>(g, 0));
    if (smooth && k != 0) stampCtrl([&](int i, int j, double v) { c.add(i, j, v); }, k);
  }
};

// Diode, device/diode.go:61-397.
struct Diode : TwoTerm {
  double IS, N, RS, CJO, VJ, M, TT, BV, IBV, FC; bool hasBV;
  double vte, vcrit, xbv = 0, grs = 0; int ai = -1;
  double vd = 0, cd = 0, gd = 0, iq = 0, geq = 0; bool tran = false, lim = false, hasCharge;
  double gmin = 1e-12, qPrev = 0, iqPrev = 0, vdAcc = 0;
  History hist;
  Diode(const double* p, bool hasBV_) {
    IS = p[KS_D_P_IS]; N = p[KS_D_P_N]; RS = p[KS_D_P_RS]; CJO = p[KS_D_P_CJO]; VJ = p[KS_D_P_VJ];
    M = p[KS_D_P_M]; TT = p[KS_D_P_TT]; BV = p[KS_D_P_BV]; IBV = p[KS_D_P_IBV]; FC = p[KS_D_P_FC];
    hasBV = hasBV_;
    vte = N * kBoltzmann * kTNom / kChargeQ;            // :116
    vcrit = vte * std::log(vte / (kSqrt2 * IS));        // :117
    if (RS > 0) grs = 1 / RS;
    hasCharge = CJO > 0 || TT > 0;
    if (hasBV) xbv = breakdownVoltage(IS, BV, IBV, kBoltzmann * kTNom / kChargeQ);
  }
  static double breakdownVoltage(double is, double bv, double ibv, double vt) {  // :166-187
    if (ibv < is * bv / vt) return bv;
    auto g = [&](double x) { return is * (std::exp(std::min((bv - x) / vt, 700.0)) - 1 + x / vt) - ibv; };
    double lo = std::min(0.0, bv - vt * std::log1p(ibv / is)) - 10 * vt, hi = bv;
    for (int i = 0; i < 200 && g(lo) <= 0; i++) lo -= 10 * vt;
    for (int i = 0; i < 200; i++) {
      double mid = 0.5 * (lo + hi);
      if (mid == lo || mid == hi) break;
      if (g(mid) > 0) lo = mid; else hi = mid;
    }
    return 0.5 * (lo + hi);
  }
  void setup(SetupCtx& c) override { setupNodes(c); ai = u[0]; if (grs > 0) ai = c.allocUnknown(); }
  bool nonlinear() const override { return true; }
  bool reactive() const override { return true; }
  bool limited() const override { return lim; }
  void curr(double v, double* id, double* g) const {  // :148-162
    if (v >= -3 * vte) {
      double e = std::exp(std::min(v / vte, 700.0));
      *id = IS * (e - 1); *g = IS * e / vte; return;
    }
    if (!hasBV || v >= -xbv) {
      double a = 3 * vte / (v * kE); a = a * a * a;
      *id = -IS * (1 + a); *g = IS * 3 * a / v; return;
    }
    double e = std::exp(std::min(-(xbv + v) / vte, 700.0));
    *id = -IS * e; *g = IS * e / vte;
  }
  void loadAC(ACCtx& c) override {  // device/diode.go:409-421
    double id, gd, q, cap;
    curr(vdAcc, &id, &gd);
    charge(vdAcc, id, gd, &q, &cap);
    c.stampY(ai, u[1], std::complex<double>(gd + gmin, c.omega * cap));
    if (grs > 0) c.stampY(u[0], ai, grs);
  }
  void charge(double v, double id, double g, double* q, double* c) const {  // :191-211
    *q = TT * id; *c = TT * g;
    if (CJO == 0) return;
    double fcv = FC * VJ;
    if (v < fcv) {
      double arg = 1 - v / VJ, sarg = std::pow(arg, -M);
      *q += CJO * VJ * (1 - arg * sarg) / (1 - M);
      *c += CJO * sarg;
      return;
    }
    double f1 = VJ * (1 - std::pow(1 - FC, 1 - M)) / (1 - M);
    double f2 = std::pow(1 - FC, 1 + M);
    double f3 = 1 - FC * (1 + M);
    *q += CJO * f1 + CJO / f2 * (f3 * (v - fcv) + M / (2 * VJ) * (v * v - fcv * fcv));
    *c += CJO / f2 * (f3 + M * v / VJ);
  }
  void load(LoadCtx& c) override {  // :229-275
    int a = u[0], k = u[1];
    gmin = c.gmin;
    double vraw = at(c.X, n, ai) - at(c.X, n, k);
    if (c.initJct) { vd = vcrit; lim = true; }
    else {
      vd = pnjlim(vraw, vdAcc, vte, vcrit, &lim);
      if (hasBV && vraw < std::min(0.0, -xbv + 10 * vte)) {
        bool l2;
        double vt = pnjlim(-(vraw + xbv), -(vdAcc + xbv), vte, vcrit, &l2);
        vd = -(vt + xbv); lim = l2;
      }
    }
    vdAcc = vd;
    double id, g0;
    curr(vd, &id, &g0);
    cd = id + gmin * vd; gd = g0 + gmin;
    tran = false; iq = 0; geq = 0;
    if (c.mode == ModeTran && hasCharge) {
      double q, cc;
      charge(vd, id, g0, &q, &cc);
      tran = true;
      if (c.method == TRAP) { iq = 2 * (q - qPrev) / c.h - iqPrev; geq = 2 * cc / c.h; }
      else { iq = (q - qPrev) / c.h; geq = cc / c.h; }
    }
    double g = gd + geq;
    double ieq = cd + iq - g * vd;
    c.M->add(ai, ai, g); c.M->add(k, k, g); c.M->add(ai, k, -g); c.M->add(k, ai, -g);
    c.addRHS(ai, -ieq); c.addRHS(k, ieq);
    if (grs > 0) { c.M->add(a, a, grs); c.M->add(ai, ai, grs); c.M->add(a, ai, -grs); c.M->add(ai, a, -grs); }
  }
  bool convTest(const double* x, double reltol, double abstol) override {  // :282-289
    double v = at(x, n, ai) - at(x, n, u[1]);
    double cdhat = cd + gd * (v - vd);
    double id, g;
    curr(v, &id, &g);
    double cdn = id + gmin * v;
    double tol = reltol * std::max(std::fabs(cdhat), std::fabs(cdn)) + abstol;
    return std::fabs(cdhat - cdn) <= tol;
  }
  double current(const double* x) override {  // :293-301
    double v = at(x, n, ai) - at(x, n, u[1]);
    return (cd + gd * (v - vd)) + (iq + geq * (v - vd));
  }
  // intDepletion, :340-361: integral of the depletion charge from 0 to v.
  double intDepletion(double v) const {
    if (CJO == 0) return 0;
    double fcv = FC * VJ;
    auto below = [&](double w) { return CJO * VJ / (1 - M) * (w + VJ / (2 - M) * (std::pow(1 - w / VJ, 2 - M) - 1)); };
    if (v < fcv) return below(v);
    double f1 = VJ * (1 - std::pow(1 - FC, 1 - M)) / (1 - M), f2 = std::pow(1 - FC, 1 + M), f3 = 1 - FC * (1 + M);
    double dv = v - fcv;
    return below(fcv) + CJO * f1 * dv + CJO / f2 * (f3 * dv * dv / 2 + M / (2 * VJ) * ((v * v * v - fcv * fcv * fcv) / 3 - fcv * fcv * dv));
  }
  // intCurrent, :363-387: integral of the junction current (no gmin) from 0 to v.
  double intCurrent(double v) const {
    auto fwd = [&](double w) { return IS * (vte * std::expm1(std::min(w / vte, 700.0)) - w); };
    double v1 = -3 * vte;
    if (v >= v1) return fwd(v);
    double total = fwd(v1);
    double a3 = std::pow(3 * vte / kE, 3);
    auto rev = [&](double w) { return -IS * (w - a3 / (2 * w * w)); };
    double v2 = v;
    if (hasBV && v < -xbv) v2 = -xbv;
    total += rev(v2) - rev(v1);
    if (v2 == v) return total;
    auto brk = [&](double w) { return IS * vte * std::exp(std::min(-(xbv + w) / vte, 700.0)); };
    return total + brk(v) - brk(v2);
  }
  OpPt operating(const double* x) override {  // Operating :293-301, StoredEnergy :329-334, ExteriorPower :400-405
    OpPt o;
    double vj = at(x, n, ai) - at(x, n, u[1]);
    double ir = cd + gd * (vj - vd), ic = iq + geq * (vj - vd);
    o.i = ir + ic; o.v = voltage(x); o.p = o.v * o.i; o.ps = vj * ic;
    o.ext = -(o.p - o.ps);
    o.stores = true;
    if (hasCharge) {
      double id, g, q, cc;
      curr(vj, &id, &g);
      charge(vj, id, g, &q, &cc);
      o.w = vj * q - intDepletion(vj) - TT * intCurrent(vj);
    }
    return o;
  }
  void accept(const double* x, double t, int mode) override {  // :304-322
    double v = at(x, n, ai) - at(x, n, u[1]);
    vdAcc = v;
    double id, g, q, cc;
    curr(v, &id, &g);
    charge(v, id, g, &q, &cc);
    if (mode == ModeTran) iqPrev = tran ? iq + geq * (v - vd) : 0;
    else { iqPrev = 0; hist.reset(); }
    qPrev = q;
    hist.push(t, q);
  }
  double truncate(const double* x, const TruncCtx& tc) override {  // :388-397
    if (!hasCharge) return kInf;
    double v = at(x, n, ai) - at(x, n, u[1]);
    double id, g, q, cc;
    curr(v, &id, &g);
    charge(v, id, g, &q, &cc);
    double ic = iq + geq * (v - vd);
    return lteStep(hist, q, ic, iqPrev, tc.abstol, tc);
  }
};

static void deplF(double vj, double m, double fc, double* f1, double* f2, double* f3) {  // device/bjt.go:245-247
  *f1 = vj * (1 - std::pow(1 - fc, 1 - m)) / (1 - m);
  *f2 = std::pow(1 - fc, 1 + m);
  *f3 = 1 - fc * (1 + m);
}

// junction, device/bjt.go:272-283.
static void junction(double is, double v, double nvt, double* i, double* g) {
  if (is == 0) { *i = 0; *g = 0; return; }
  if (v >= -3 * nvt) {
    double e = std::exp(std::min(v / nvt, 700.0));
    *i = is * (e - 1); *g = is * e / nvt; return;
  }
  double a = 3 * nvt / (v * kE); a = a * a * a;
  *i = -is * (1 + a); *g = is * 3 * a / v;
}

// depletion, device/bjt.go:358-370.
static void depletion(double v, double cz, double vj, double m, double fc, double f1, double f2, double f3,
                      double* q, double* c) {
  if (cz == 0) { *q = 0; *c = 0; return; }
  double fcv = fc * vj;
  if (v < fcv) {
    double arg = 1 - v / vj;
    double sarg = std::exp(-m * std::log(arg));
    *q = vj * cz * (1 - arg * sarg) / (1 - m); *c = cz * sarg; return;
  }
  double czf2 = cz / f2;
  *q = cz * f1 + czf2 * (f3 * (v - fcv) + (m / (vj + vj)) * (v * v - fcv * fcv));
  *c = czf2 * (f3 + m * v / vj);
}

}  // namespace kso
