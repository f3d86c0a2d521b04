// ks_host.cpp — host symbolic pass of the GB300 engine: unknown layout and validation.
//
// plan_layout restates device Setup (device/device.go:36-100 and the Setup of each
// device kind) once per topology: node k -> unknown k-1, then branch currents and
// internal nodes allocated in element order from one counter.  validate restates
// circuit.Validate (circuit/circuit.go:368-557) and checkPaths (:704-804) for the
// engine's element kinds, with the same sentinel texts.
#include "ks_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>

namespace ksh {

static thread_local std::string g_err;
void set_error(const std::string& s) { g_err = s; }

int plan_layout(const ks_topology* t, HostPlan* hp, std::string* err) {
  if (!t || !t->elem || t->n_elem <= 0 || t->n_nodes <= 0) { *err = "circuit: no elements"; return KS_EINVAL; }
  hp->n_nodes = t->n_nodes;
  hp->n_elem = t->n_elem;
  hp->n_values = t->n_values;
  hp->src.assign(t->elem, t->elem + t->n_elem);
  hp->elem.assign(t->n_elem, KElem{});
  int next = t->n_nodes - 1;
  std::vector<int> internal;
  auto alloc_branch = [&]() { return next++; };
  auto alloc_unknown = [&]() { int i = next++; internal.push_back(i); return i; };
  int nd = 0, ns = 0;
  for (int k = 0; k < t->n_elem; k++) {
    const ks_element& s = t->elem[k];
    KElem& e = hp->elem[k];
    e.kind = s.kind; e.flags = s.flags; e.level = s.level; e.wave = s.wave;
    e.nargs = s.nargs; e.param = s.param; e.given = s.given;
    for (int i = 0; i < 10; i++) e.u[i] = -1;
    // F, H: node[2] and K: node[0..1] index elements (linked below), not nodes
    for (int i = 0; i < 4; i++) {
      const bool elem_ref = (s.kind == KS_ELEM_K && i < 2) ||
                            ((s.kind == KS_ELEM_F || s.kind == KS_ELEM_H || s.kind == KS_ELEM_W) && i == 2);
      if (elem_ref) continue;
      if (s.node[i] < 0 || s.node[i] >= t->n_nodes) {
        char buf[128];
        snprintf(buf, sizeof buf, "circuit: invalid element value: element %d has node index %d out of range", k, s.node[i]);
        *err = buf;
        return KS_EINVAL;
      }
    }
    const bool ctl = s.kind >= KS_ELEM_E && s.kind <= KS_ELEM_K;
    const bool sw = s.kind == KS_ELEM_S || s.kind == KS_ELEM_W;
    const bool nl = s.kind == KS_ELEM_CN || s.kind == KS_ELEM_LN;
    if (nl && (s.level < 0 || s.level > 1 << 20 || s.level % 2 != 0 || s.level == 2)) {
      *err = "ks_topology: a curve needs two or more (x, y) pairs";
      return KS_EINVAL;
    }
    int need = s.kind == KS_ELEM_D ? KS_D_NP : s.kind == KS_ELEM_Q ? KS_Q_NP : s.kind == KS_ELEM_M ? KS_M_NP
             : (s.kind == KS_ELEM_V || s.kind == KS_ELEM_I) ? KS_SRC_P_ARGS + s.nargs : ctl ? KS_CTL_NP
             : sw ? KS_SW_NP : nl ? KS_NL_P_ARGS + s.nargs + s.level : KS_RCL_NP;
    if (s.nargs < 0 || s.nargs > 1 << 20 || s.param < 0 || (int64_t)s.param + need > t->n_values) {
      *err = "ks_topology: element value block outside the value vector";
      return KS_EINVAL;
    }
    int u0 = s.node[0] - 1, u1 = s.node[1] - 1;
    e.derived = nd;
    e.state = ns;
    switch (s.kind) {
      case KS_ELEM_R: e.u[0] = u0; e.u[1] = u1; nd += DR_N; break;
      case KS_ELEM_C: e.u[0] = u0; e.u[1] = u1; ns += SC_N; hp->n_reactive++; break;
      case KS_ELEM_L: e.u[0] = u0; e.u[1] = u1; e.u[2] = alloc_branch(); ns += SL_N; hp->n_reactive++; break;
      case KS_ELEM_V:
        e.u[0] = u0; e.u[1] = u1; e.u[2] = alloc_branch();
        nd += DS_N; ns += SV_N; hp->n_breakpointer++;
        break;
      case KS_ELEM_I: e.u[0] = u0; e.u[1] = u1; nd += DS_N; ns += SV_N; hp->n_breakpointer++; break;
      case KS_ELEM_D:
        e.u[0] = u0; e.u[1] = u1; e.u[2] = u0;
        if (s.flags & KS_F_INT_A) e.u[2] = alloc_unknown();
        nd += DD_N; ns += SD_N; hp->n_nonlin++; hp->n_reactive++;
        break;
      case KS_ELEM_Q: {  // device/bjt.go:250-268
        int c = s.node[0] - 1, em = s.node[1] - 1, b = s.node[2] - 1, sub = s.node[3] - 1;
        e.u[0] = c; e.u[1] = em; e.u[2] = b; e.u[3] = sub;
        int cp = c, bp = b, ep = em;
        if (s.flags & KS_F_INT_C) cp = alloc_unknown();
        if (s.flags & KS_F_INT_B) bp = alloc_unknown();
        if (s.flags & KS_F_INT_E) ep = alloc_unknown();
        e.u[4] = cp; e.u[5] = bp; e.u[6] = ep;
        e.u[7] = sub; e.u[8] = cp;
        if (s.flags & KS_F_LATERAL) { e.u[7] = bp; e.u[8] = sub; }
        nd += DQ_N; ns += SQ_N; hp->n_nonlin++; hp->n_reactive++;
        break;
      }
      case KS_ELEM_M: {  // device/mosfet.go:326-337
        int d = s.node[0] - 1, so = s.node[1] - 1, g = s.node[2] - 1, b = s.node[3] - 1;
        e.u[0] = d; e.u[1] = so; e.u[2] = g; e.u[3] = b;
        e.u[4] = (s.flags & KS_F_INT_D) ? alloc_unknown() : d;
        e.u[5] = (s.flags & KS_F_INT_S) ? alloc_unknown() : so;
        if (s.level < 1 || s.level > 3) { *err = "circuit: bad model: LEVEL must be 1, 2 or 3"; return KS_EINVAL; }
        nd += DM_N; ns += SM_N; hp->n_nonlin++; hp->n_reactive++;
        break;
      }
      case KS_ELEM_E: case KS_ELEM_H:  // device/controlled.go:55-66: a voltage output has a branch
        e.u[0] = u0; e.u[1] = u1; e.u[2] = alloc_branch();
        if (s.kind == KS_ELEM_E) { e.u[3] = s.node[2] - 1; e.u[4] = s.node[3] - 1; }
        break;
      case KS_ELEM_G:
        e.u[0] = u0; e.u[1] = u1; e.u[3] = s.node[2] - 1; e.u[4] = s.node[3] - 1;
        break;
      case KS_ELEM_F: e.u[0] = u0; e.u[1] = u1; break;
      case KS_ELEM_K: nd += DK_N; ns += SK_N; hp->n_reactive++; break;
      case KS_ELEM_CN: case KS_ELEM_LN:  // device/nonlinear_reactive.go:311-314, :522-527
        e.u[0] = u0; e.u[1] = u1;
        if (s.kind == KS_ELEM_LN) e.u[2] = alloc_branch();
        nd += DN_PRE + s.level / 2; ns += SN_N; hp->n_reactive++; hp->n_breakpointer++;
        if (s.level > 0) hp->n_nonlin++;  // curvedCapacitor / curvedInductor
        break;
      case KS_ELEM_S: case KS_ELEM_W:  // device/switch.go:111-117: nonlinear (ConvTest), no branch
        e.u[0] = u0; e.u[1] = u1;
        if (s.kind == KS_ELEM_S) { e.u[3] = s.node[2] - 1; e.u[4] = s.node[3] - 1; }
        nd += DW_N; ns += SW_N; hp->n_nonlin++;
        break;
      default:
        *err = "device: unsupported element kind";
        return KS_EUNSUPPORTED;
    }
  }
  // Link (device/controlled.go:69-80, device/mutual.go:54-70): the branches a
  // CCCS / CCVS senses and a mutual inductance couples, once every branch exists
  for (int k = 0; k < t->n_elem; k++) {
    const ks_element& s = t->elem[k];
    KElem& e = hp->elem[k];
    auto branch_of = [&](int j, int want) -> int {
      if (j < 0 || j >= t->n_elem || t->elem[j].kind != want) return -1;
      return hp->elem[j].u[2];
    };
    if (s.kind == KS_ELEM_F || s.kind == KS_ELEM_H || s.kind == KS_ELEM_W) {  // W: device/switch.go:120-130
      e.u[3] = branch_of(s.node[2], KS_ELEM_V);
      if (e.u[3] < 0) { *err = "device: unsupported element kind: controlling source not found"; return KS_EUNSUPPORTED; }
    } else if (s.kind == KS_ELEM_K) {
      e.u[0] = branch_of(s.node[0], KS_ELEM_L);
      e.u[1] = branch_of(s.node[1], KS_ELEM_L);
      if (e.u[0] < 0 || e.u[1] < 0) { *err = "device: unsupported element kind: inductor not found"; return KS_EUNSUPPORTED; }
      e.u[2] = t->elem[s.node[0]].param;
      e.u[3] = t->elem[s.node[1]].param;
    }
  }
  hp->n = next;
  hp->n_derived = nd;
  hp->n_state = ns;
  hp->is_v.assign(hp->n, 0);
  for (int i = 0; i < t->n_nodes - 1; i++) hp->is_v[i] = 1;
  for (int i : internal) hp->is_v[i] = 1;
  return KS_OK;
}

static bool finite(double v) { return std::isfinite(v); }

// validateWave, circuit/circuit.go:647-700.
static bool validate_wave(const ks_element& e, const double* a, std::string* err) {
  int n = e.nargs;
  for (int i = 0; i < n; i++)
    if (!finite(a[i])) { *err = "circuit: invalid source waveform: non-finite argument"; return false; }
  switch (e.wave) {
    case KS_WAVE_NONE: if (n != 0) { *err = "circuit: invalid source waveform"; return false; } break;
    case KS_WAVE_PULSE:
      if (n < 2 || n > 7) { *err = "circuit: invalid source waveform: PULSE needs 2-7 arguments"; return false; }
      for (int i = 2; i < n; i++) if (a[i] < 0) { *err = "circuit: invalid source waveform: PULSE argument is negative"; return false; }
      break;
    case KS_WAVE_SIN:
      if (n < 2 || n > 6) { *err = "circuit: invalid source waveform: SIN needs 2-6 arguments"; return false; }
      if ((n > 2 && a[2] < 0) || (n > 3 && a[3] < 0)) { *err = "circuit: invalid source waveform: SIN frequency and delay must not be negative"; return false; }
      break;
    case KS_WAVE_EXP:
      if (n < 2 || n > 6) { *err = "circuit: invalid source waveform: EXP needs 2-6 arguments"; return false; }
      for (int i = 2; i < n; i++) if (a[i] < 0) { *err = "circuit: invalid source waveform: EXP argument is negative"; return false; }
      break;
    case KS_WAVE_PWL:
      if (n < 2 || n % 2 != 0 || n / 2 > 100000) { *err = "circuit: invalid source waveform: PWL needs time/value pairs"; return false; }
      for (int i = 2; i < n; i += 2) if (a[i] < a[i - 2]) { *err = "circuit: invalid source waveform: PWL times must not decrease"; return false; }
      if (a[0] < 0) { *err = "circuit: invalid source waveform: PWL times must not be negative"; return false; }
      break;
    default: *err = "circuit: invalid source waveform: unknown waveform"; return false;
  }
  return true;
}

int validate(const ks_topology* t, const double* v, bool transient, std::string* err) {
  if (!t || t->n_elem <= 0) { *err = "circuit: no elements"; return KS_EVALIDATE; }
  if (t->n_nodes > 100000 || t->n_elem > 1000000) { *err = "circuit: too many nodes or elements"; return KS_EVALIDATE; }
  bool groundUsed = false;
  std::vector<std::pair<int, int>> coupled;  // validateMutual's pairs
  for (int k = 0; k < t->n_elem; k++) {
    const ks_element& e = t->elem[k];
    if (e.kind == KS_ELEM_K) {  // validateMutual, circuit/circuit.go:807-831 (no nodes of its own)
      const double kc = v[e.param + KS_K_P_COUPLING];
      if (!(kc > 0 && kc <= 1)) {
        char buf[128]; snprintf(buf, sizeof buf, "circuit: invalid element value: element %d: coupling coefficient %g must be in (0, 1]", k, kc);
        *err = buf; return KS_EVALIDATE;
      }
      int a = e.node[0], b = e.node[1];
      if (a == b) { *err = "circuit: invalid element value: a mutual inductance couples an inductor with itself"; return KS_EVALIDATE; }
      for (int j : {a, b})
        if (j < 0 || j >= t->n_elem || t->elem[j].kind != KS_ELEM_L) {
          *err = "circuit: invalid element value: a mutual inductance couples an element that is not a linear inductor";
          return KS_EVALIDATE;
        }
      if (a > b) std::swap(a, b);
      for (auto& pr : coupled)
        if (pr.first == a && pr.second == b) { *err = "circuit: invalid element value: the inductors are already coupled"; return KS_EVALIDATE; }
      coupled.push_back({a, b});
      if (!finite(kc)) { *err = "circuit: invalid element value: non-finite value"; return KS_EVALIDATE; }
      continue;
    }
    int nn = (e.kind == KS_ELEM_Q || e.kind == KS_ELEM_M) ? 4 : 2;
    for (int i = 0; i < nn; i++) {
      if (e.node[i] < 0 || e.node[i] >= t->n_nodes) { *err = "circuit: invalid element value: node index out of range"; return KS_EVALIDATE; }
      if (e.node[i] == 0 && !(e.kind == KS_ELEM_Q && i == 3)) groundUsed = true;
    }
    if (e.node[0] == e.node[1] && e.kind != KS_ELEM_Q && e.kind != KS_ELEM_M) {
      char buf[96]; snprintf(buf, sizeof buf, "circuit: element connects a node to itself: element %d", k);
      *err = buf; return KS_EVALIDATE;
    }
    const double* p = v + e.param;
    switch (e.kind) {
      case KS_ELEM_R: case KS_ELEM_C: case KS_ELEM_L:
        if (!finite(p[0]) || !finite(p[1])) { *err = "circuit: invalid element value: non-finite value"; return KS_EVALIDATE; }
        if (p[0] == 0 || (p[0] < 0 && e.kind != KS_ELEM_R)) {
          char buf[128]; snprintf(buf, sizeof buf, "circuit: invalid element value: element %d must be > 0, got %g", k, p[0]);
          *err = buf; return KS_EVALIDATE;
        }
        break;
      case KS_ELEM_V: case KS_ELEM_I:
        for (int i = 0; i < 3; i++) if (!finite(p[i])) { *err = "circuit: invalid element value: non-finite value"; return KS_EVALIDATE; }
        if (!validate_wave(e, p + KS_SRC_P_ARGS, err)) return KS_EVALIDATE;
        break;
      case KS_ELEM_D: case KS_ELEM_Q: case KS_ELEM_M: {
        const int np = e.kind == KS_ELEM_D ? (int)KS_D_NP : e.kind == KS_ELEM_Q ? (int)KS_Q_NP : (int)KS_M_NP;
        for (int i = 0; i < np; i++) if (!finite(p[i])) { *err = "circuit: bad model: parameter is not finite"; return KS_EVALIDATE; }
        if (e.kind == KS_ELEM_M) {  // validateMOSInstance, circuit/circuit.go:845-862
          for (int i = KS_M_P_L; i <= KS_M_P_MULT; i++) {
            double x = p[i];
            bool lwm = i == KS_M_P_L || i == KS_M_P_W || i == KS_M_P_MULT;
            if (x < 0 || (lwm && x == 0) || x > 1e6) { *err = "circuit: invalid element value: MOSFET instance parameter"; return KS_EVALIDATE; }
          }
          if (e.level < 1 || e.level > 3) { *err = "circuit: bad model: LEVEL must be 1, 2 or 3"; return KS_EVALIDATE; }
        }
        break;
      }
      case KS_ELEM_E: case KS_ELEM_G:  // validateControl, circuit/circuit.go:865-876
        if (!finite(p[0])) { *err = "circuit: invalid element value: non-finite value"; return KS_EVALIDATE; }
        for (int i = 2; i < 4; i++)
          if (e.node[i] < 0 || e.node[i] >= t->n_nodes) { *err = "circuit: invalid element value: control node index out of range"; return KS_EVALIDATE; }
        if (e.node[2] == e.node[3]) {
          char buf[128]; snprintf(buf, sizeof buf, "circuit: invalid element value: element %d is controlled by a voltage that is always 0", k);
          *err = buf; return KS_EVALIDATE;
        }
        break;
      case KS_ELEM_F: case KS_ELEM_H:  // validateControl, :877-881
        if (!finite(p[0])) { *err = "circuit: invalid element value: non-finite value"; return KS_EVALIDATE; }
        if (e.node[2] < 0 || e.node[2] >= t->n_elem || t->elem[e.node[2]].kind != KS_ELEM_V) {
          char buf[128]; snprintf(buf, sizeof buf, "circuit: invalid element value: element %d is controlled by an element that is not a voltage source", k);
          *err = buf; return KS_EVALIDATE;
        }
        break;
      case KS_ELEM_CN: case KS_ELEM_LN: {  // validateStateLaw, circuit/circuit.go:890-942
        const int nc = e.level, na = e.nargs;
        for (int i = 0; i < KS_NL_P_ARGS + na + nc; i++)
          if (!finite(p[i])) { *err = "circuit: invalid element value: non-finite value"; return KS_EVALIDATE; }
        const double* c = p + KS_NL_P_ARGS + na;
        if (nc == 0) {
          if (!(p[KS_NL_P_VALUE] > 0)) {
            char buf[128]; snprintf(buf, sizeof buf, "circuit: invalid element value: element %d must be > 0, got %g", k, p[0]);
            *err = buf; return KS_EVALIDATE;
          }
        } else {
          if (p[KS_NL_P_VALUE] != 0) { *err = "circuit: invalid element value: an element has both a value and a curve"; return KS_EVALIDATE; }
          if (nc < 4 || nc % 2 != 0 || nc > 200000) { *err = "circuit: invalid element value: a curve needs 2 to 100000 (x, y) points"; return KS_EVALIDATE; }
          double ymax = 0;
          for (int i = 0; i < nc; i++) {
            if (i >= 2 && !(c[i] > c[i - 2])) {
              *err = "circuit: invalid element value: a curve must strictly increase in x and y"; return KS_EVALIDATE;
            }
            if (i % 2 == 1) ymax = std::max(ymax, std::fabs(c[i]));
          }
          // curveAt(curve, 0), :944-961: the end segments extend
          const int n = nc / 2;
          int j = 0;
          while (j < n && c[2 * j] < 0) j++;
          const int lo = j <= 0 ? 0 : j >= n ? n - 2 : j - 1;
          const double y0 = c[2 * lo + 1] + (c[2 * lo + 3] - c[2 * lo + 1]) / (c[2 * lo + 2] - c[2 * lo]) * (0 - c[2 * lo]);
          if (std::fabs(y0) > 1e-12 * ymax) { *err = "circuit: invalid element value: a curve must pass through the origin"; return KS_EVALIDATE; }
        }
        if (e.wave != KS_WAVE_NONE) {  // the scale: a valid waveform that stays > 0 (scaleLowerBound, :963-986)
          ks_element w = e;
          w.param = 0;
          if (!validate_wave(w, p + KS_NL_P_ARGS, err)) return KS_EVALIDATE;
          const double* a = p + KS_NL_P_ARGS;
          auto arg = [&](int i) { return i < na ? a[i] : 0.0; };
          double lo = 0;
          bool ok = true;
          if (e.wave == KS_WAVE_PULSE || e.wave == KS_WAVE_EXP) lo = std::min(arg(0), arg(1));
          else if (e.wave == KS_WAVE_SIN) { ok = arg(4) >= 0; lo = arg(0) - std::fabs(arg(1)); }
          else {
            lo = 1e300;
            for (int i = 1; i < na; i += 2) lo = std::min(lo, a[i]);
            for (int i = 2; i < na; i += 2)
              if (!(a[i] > a[i - 2])) { *err = "circuit: invalid source waveform: scale PWL times must strictly increase"; return KS_EVALIDATE; }
          }
          if (!ok || !(lo > 0)) { *err = "circuit: invalid source waveform: scale must stay > 0"; return KS_EVALIDATE; }
        }
        break;
      }
      case KS_ELEM_S: case KS_ELEM_W: {  // validateSwitch, circuit/switch.go:52-72
        for (int i = 0; i < KS_SW_NP; i++)
          if (!finite(p[i])) { *err = "circuit: invalid element value: non-finite value"; return KS_EVALIDATE; }
        if (!(p[KS_SW_P_RON] > 0) || !(p[KS_SW_P_ROFF] > 0)) {  // swParams: ron, roff pos
          *err = "circuit: bad model: switch RON and ROFF must be > 0"; return KS_EVALIDATE;
        }
        if (p[KS_SW_P_VH] < 0 && p[KS_SW_P_RON] == p[KS_SW_P_ROFF]) {
          *err = "circuit: bad model: a smooth switch (negative hysteresis) needs RON != ROFF"; return KS_EVALIDATE;
        }
        if (p[KS_SW_P_ON] != 0 && p[KS_SW_P_ON] != 1) {
          char buf[128]; snprintf(buf, sizeof buf, "circuit: invalid element value: element %d initial state must be ON (1) or OFF (0)", k);
          *err = buf; return KS_EVALIDATE;
        }
        if (e.kind == KS_ELEM_S) {  // validateControl, circuit/circuit.go:865-876
          for (int i = 2; i < 4; i++)
            if (e.node[i] < 0 || e.node[i] >= t->n_nodes) { *err = "circuit: invalid element value: control node index out of range"; return KS_EVALIDATE; }
          if (e.node[2] == e.node[3]) {
            char buf[128]; snprintf(buf, sizeof buf, "circuit: invalid element value: element %d is controlled by a voltage that is always 0", k);
            *err = buf; return KS_EVALIDATE;
          }
        } else if (e.node[2] < 0 || e.node[2] >= t->n_elem || t->elem[e.node[2]].kind != KS_ELEM_V) {  // :877-881
          char buf[128]; snprintf(buf, sizeof buf, "circuit: invalid element value: element %d is controlled by an element that is not a voltage source", k);
          *err = buf; return KS_EVALIDATE;
        }
        break;
      }
      default: *err = "circuit: unknown element kind"; return KS_EVALIDATE;
    }
  }
  if (!groundUsed) { *err = "circuit: no ground node (0 or gnd)"; return KS_EVALIDATE; }
  // checkPaths, circuit/circuit.go:704-804: union-find over DC paths.
  std::vector<int> parent(t->n_nodes);
  std::iota(parent.begin(), parent.end(), 0);
  auto find = [&](int x) {
    while (parent[x] != x) { parent[x] = parent[parent[x]]; x = parent[x]; }
    return x;
  };
  auto unite = [&](int a, int b) { a = find(a); b = find(b); if (a != b) parent[a] = b; };
  for (int k = 0; k < t->n_elem; k++) {
    const ks_element& e = t->elem[k];
    // current sources, mutual inductances and controlled current outputs are no path
    if (e.kind == KS_ELEM_I || e.kind == KS_ELEM_K || e.kind == KS_ELEM_F || e.kind == KS_ELEM_G ||
        ((e.kind == KS_ELEM_C || e.kind == KS_ELEM_CN) && !transient))
      continue;
    unite(e.node[0], e.node[1]);
    if (e.kind == KS_ELEM_M) unite(e.node[3], e.node[0]);
    if (e.kind == KS_ELEM_Q) unite(e.node[2], e.node[0]);
  }
  int g = find(0);
  std::string floating;
  int nf = 0;
  for (int i = 1; i < t->n_nodes; i++) {
    if (find(i) != g) {
      if (nf < 10) { if (nf) floating += ", "; floating += "node " + std::to_string(i); }
      nf++;
    }
  }
  if (nf) {
    *err = std::string("circuit: node has no path to ground (") + (transient ? "" : "DC ") + "path): " + floating;
    return KS_EVALIDATE;
  }
  return KS_OK;
}

}  // namespace ksh

extern "C" const char* ks_version(void) { return "kronspice-gb300 0.1 (sm_103a)"; }
extern "C" const char* ks_last_error(void) { return ksh::g_err.c_str(); }

extern "C" int ks_validate(const ks_topology* topo, const double* values, int transient) {
  std::string err;
  int rc = ksh::validate(topo, values, transient != 0, &err);
  ksh::set_error(rc ? err : std::string());
  return rc;
}

extern "C" int ks_unknowns(const ks_topology* topo, int32_t* n_unknowns, int32_t* is_voltage) {
  ksh::HostPlan hp;
  std::string err;
  int rc = ksh::plan_layout(topo, &hp, &err);
  if (rc) { ksh::set_error(err); return rc; }
  if (n_unknowns) *n_unknowns = hp.n;
  if (is_voltage) for (int i = 0; i < hp.n; i++) is_voltage[i] = hp.is_v[i];
  return KS_OK;
}

extern "C" int ks_tran_points(const ks_tran_spec* spec, int32_t* n_points) {
  if (!spec || !(spec->step > 0) || !(spec->stop > 0)) return KS_EINVAL;
  *n_points = (int32_t)std::lround(spec->stop / spec->step) + 1;
  return KS_OK;
}
