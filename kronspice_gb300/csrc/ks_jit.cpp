// ks_jit.cpp — per-topology kernels of the GB300 engine.
//
// Every circuit of a plan has the same topology, so the element program of the
// generic kernels (an element table read from shared memory and a kind switch
// per element per Newton iteration) is known before the batch runs.  For large
// batches the host writes that program out as CUDA source: each element becomes
// a compile-time constant KElem, so the kind switch folds away, every unknown
// index is an immediate, and systems of up to KS_JIT_REG_MAX unknowns live in
// registers (larger ones in shared memory at constant offsets).  The device code
// is the same set of templates the generic kernels instantiate (ks_tran.cuh and
// below, embedded in the library at build time), so both kernels follow the same
// arithmetic; only the program and the system storage differ.
//
// NVRTC compiles the source for the device's own architecture; the cubin is kept
// in memory per process and on disk (KS_JIT_CACHE_DIR, else
// $XDG_CACHE_HOME/kronspice_gb300, else ~/.cache/kronspice_gb300; "off" disables)
// under a hash of the source, the embedded headers, the options and the NVRTC
// version, and is loaded as a context-independent CUDA library (cudaLibrary_t)
// whose kernels the runtime launches like any other.
#include <cuda_runtime.h>
#include <nvrtc.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "ks_internal.h"

// Generated at build time from the device headers (kronspice_gb300/build.py).
extern const int ks_jit_n_headers;
extern const char* const ks_jit_header_names[];
extern const char* const ks_jit_header_srcs[];

namespace ksj {

int reg_max() {
  const char* e = getenv("KS_JIT_REG_MAX");
  return e ? atoi(e) : 6;
}

static void append_elem(std::string& s, const KElem& e) {
  char buf[512];
  snprintf(buf, sizeof buf, "    { const KElem e{%d, %d, %d, %d, %d, %d, %d, %d, {", e.kind, e.flags, e.level, e.wave,
           e.nargs, e.param, e.derived, e.state);
  s += buf;
  for (int i = 0; i < 10; i++) {
    snprintf(buf, sizeof buf, "%s%d", i ? ", " : "", e.u[i]);
    s += buf;
  }
  snprintf(buf, sizeof buf, "}, 0x%llxull}; f(e); }\n", (unsigned long long)e.given);
  s += buf;
}


// ---------------------------------------------------------------- fixed pivot sequence
// A symbolic LU of the plan's MNA pattern, emitted as straight-line code over the
// structurally non-zero entries only:
//   1. the pattern: every entry any element stamps in any mode (devices as dense
//      blocks over their terminals), and every diagonal (gmin and
//      pseudo-transient stepping add to them);
//   2. rows: the branch row of each voltage source / inductor trades places with
//      the row of one of its nodes, so both pivots are the source's +-1
//      incidence entries instead of the branch row's structural zero;
//   3. columns: minimum degree on the pattern of B + B^T (ties to the lowest
//      index), as solver/sparse.go's minimumDegree orders its columns;
//   4. fill of the LU with diagonal pivots in that order.
// At run time each pivot must pass a threshold (within 2^-10 of the largest
// entry left in its column, and not below 2^-30 of the column's largest input
// entry, both on exponent bits); a failed check returns SOLVE_STATIC_FAIL and
// the solve falls back to partial pivoting, which also owns the singular test.
namespace {

struct Symbolic {
  int n = 0;
  std::vector<int> prow;          // prow[k]: A row pivoting in step k
  std::vector<int> q;             // q[k]: A column eliminated in step k
  std::vector<uint32_t> Amask;    // structural pattern of A, by A row (bit = A column)
  std::vector<uint64_t> Cmask;    // pattern of the factors, by step (bit = step), fill included
};

void stamp_pattern(const ksh::HostPlan& hp, std::vector<uint32_t>& m) {
  auto add = [&](int i, int j) { if (i >= 0 && j >= 0) m[i] |= 1u << j; };
  auto block = [&](const int* u, int k) {
    for (int a = 0; a < k; a++)
      for (int b = 0; b < k; b++) add(u[a], u[b]);
  };
  for (const KElem& e : hp.elem) {
    const int* u = e.u;
    switch (e.kind) {
      case KS_ELEM_R: case KS_ELEM_C: case KS_ELEM_CN: block(u, 2); break;
      case KS_ELEM_V: case KS_ELEM_L: case KS_ELEM_LN:
        add(u[0], u[2]); add(u[1], u[2]); add(u[2], u[0]); add(u[2], u[1]); add(u[2], u[2]); break;
      case KS_ELEM_I: break;
      case KS_ELEM_D: block(u, 3); break;
      case KS_ELEM_Q: block(u, 9); break;
      case KS_ELEM_M: block(u, 6); break;
      case KS_ELEM_E: case KS_ELEM_H:  // device/controlled.go:83-100
        add(u[0], u[2]); add(u[1], u[2]); add(u[2], u[0]); add(u[2], u[1]); add(u[2], u[3]);
        if (e.kind == KS_ELEM_E) add(u[2], u[4]);
        break;
      case KS_ELEM_G: add(u[0], u[3]); add(u[0], u[4]); add(u[1], u[3]); add(u[1], u[4]); break;
      case KS_ELEM_F: add(u[0], u[3]); add(u[1], u[3]); break;
      case KS_ELEM_K: add(u[0], u[1]); add(u[1], u[0]); break;  // device/mutual.go:110-113
      case KS_ELEM_S:  // device/switch.go:174-226 (the smooth switch's transconductance too)
        block(u, 2); add(u[0], u[3]); add(u[0], u[4]); add(u[1], u[3]); add(u[1], u[4]); break;
      case KS_ELEM_W: block(u, 2); add(u[0], u[3]); add(u[1], u[3]); break;
      default: break;
    }
  }
  for (int i = 0; i < hp.n; i++) add(i, i);
}

bool symbolic(const ksh::HostPlan& hp, Symbolic* sy) {
  const int n = hp.n;
  if (n < 1 || n > 32) return false;
  sy->n = n;
  sy->Amask.assign(n, 0);
  stamp_pattern(hp, sy->Amask);
  auto has = [&](int r, int c) { return (sy->Amask[r] >> c) & 1u; };
  // 2. row pairing: pivot row of each A column
  std::vector<int> pr(n);
  for (int i = 0; i < n; i++) pr[i] = i;
  for (const KElem& e : hp.elem) {
    if (e.kind != KS_ELEM_V && e.kind != KS_ELEM_L) continue;
    int j = e.u[2];
    for (int t = 0; t < 2; t++) {
      int a = e.u[t];
      if (a < 0 || pr[a] != a || pr[j] != j || a == j) continue;
      if (!has(j, a) || !has(a, j)) continue;
      pr[a] = j;
      pr[j] = a;
      break;
    }
  }
  // B(k, c) = A(pr[k], c): minimum degree on the pattern of B + B^T
  std::vector<uint32_t> G(n, 0);
  for (int k = 0; k < n; k++)
    for (int c = 0; c < n; c++)
      if (k != c && has(pr[k], c)) { G[k] |= 1u << c; G[c] |= 1u << k; }
  std::vector<int> q;
  uint32_t left = n == 32 ? 0xffffffffu : ((1u << n) - 1);
  while (left) {
    int best = -1, bd = 1 << 30;
    for (int v = 0; v < n; v++) {
      if (!((left >> v) & 1u)) continue;
      int d = __builtin_popcount(G[v] & left);
      if (d < bd) { bd = d; best = v; }
    }
    uint32_t nb = G[best] & left & ~(1u << best);
    for (int v = 0; v < n; v++)
      if ((nb >> v) & 1u) G[v] |= nb & ~(1u << v);
    left &= ~(1u << best);
    q.push_back(best);
  }
  sy->q = q;
  sy->prow.resize(n);
  for (int k = 0; k < n; k++) sy->prow[k] = pr[q[k]];
  // C(k, l) = A(prow[k], q[l]) and its fill
  sy->Cmask.assign(n, 0);
  for (int k = 0; k < n; k++)
    for (int l = 0; l < n; l++)
      if (has(sy->prow[k], q[l])) sy->Cmask[k] |= 1ull << l;
  for (int k = 0; k < n; k++) {
    if (!((sy->Cmask[k] >> k) & 1ull)) return false;  // structurally zero pivot
    for (int i = k + 1; i < n; i++) {
      if (!((sy->Cmask[i] >> k) & 1ull)) continue;
      sy->Cmask[i] |= sy->Cmask[k] & ~((2ull << k) - 1);
    }
  }
  return true;
}

// Straight-line factor + solve in type T ("double" or "float"), reading A from
// the system.  mode LU_FP64: x = A^-1 rhs in FP64; LU_MIXED: FP32 factor of the
// FP64 matrix with FP64-residual refinement; LU_F32: the FP32 start stage's
// system, x32 = a32^-1 r32 entirely in FP32.
enum { LU_FP64 = 0, LU_MIXED = 1, LU_F32 = 2 };
std::string emit_lu(const Symbolic& sy, int mode) {
  const int n = sy.n;
  const bool mixed = mode != LU_FP64;
  const char* T = mixed ? "float" : "double";
  auto C = [&](int k, int l) { return (sy.Cmask[k] >> l) & 1ull; };
  std::string o;
  char b[512];
  auto f = [&](int k, int l) { snprintf(b, sizeof b, "f%d_%d", k, l); return std::string(b); };
  // load (fill entries start at zero) and the column scales of the input
  for (int k = 0; k < n; k++)
    for (int l = 0; l < n; l++) {
      if (!C(k, l)) continue;
      bool inA = (sy.Amask[sy.prow[k]] >> sy.q[l]) & 1u;
      if (inA && mode == LU_F32) snprintf(b, sizeof b, "    float %s = s.a32(%d, %d);\n", f(k, l).c_str(), sy.prow[k], sy.q[l]);
      else if (inA) snprintf(b, sizeof b, "    %s %s = (%s)s.a(%d, %d);\n", T, f(k, l).c_str(), T, sy.prow[k], sy.q[l]);
      else snprintf(b, sizeof b, "    %s %s = 0;\n", T, f(k, l).c_str());
      o += b;
    }
  // exponent field of |v| as an int (float or double)
  const char* ex = mixed ? "ks_exp32" : "ks_exp64";
  for (int l = 0; l < n; l++) {
    snprintf(b, sizeof b, "    int cs%d = 0;", l);
    o += b;
    for (int k = 0; k < n; k++)
      if (C(k, l) && ((sy.Amask[sy.prow[k]] >> sy.q[l]) & 1u)) {
        snprintf(b, sizeof b, " cs%d = max(cs%d, %s(%s));", l, l, ex, f(k, l).c_str());
        o += b;
      }
    o += "\n";
  }
  const int big = mixed ? 255 : 2047;  // exponent field of infinities and NaNs
  for (int k = 0; k < n; k++) {
    // threshold on exponents: pivot within 2^-10 of the column's largest remaining entry
    snprintf(b, sizeof b, "    { int ep = %s(%s), em = ep;", ex, f(k, k).c_str());
    o += b;
    for (int i = k + 1; i < n; i++)
      if (C(i, k)) { snprintf(b, sizeof b, " em = max(em, %s(%s));", ex, f(i, k).c_str()); o += b; }
    snprintf(b, sizeof b,
             "\n      if (em >= %d || ep == 0 || ep + 10 < em || ep + 30 < cs%d) return SOLVE_STATIC_FAIL;"
             " }\n",
             big, k);
    o += b;
    snprintf(b, sizeof b, "    const %s r%d = %s / %s;\n", T, k, mixed ? "1.0f" : "1.0", f(k, k).c_str());
    o += b;
    for (int i = k + 1; i < n; i++) {
      if (!C(i, k)) continue;
      snprintf(b, sizeof b, "    %s *= r%d;\n", f(i, k).c_str(), k);
      o += b;
      for (int l = k + 1; l < n; l++)
        if (C(k, l)) {
          snprintf(b, sizeof b, "    %s = %s(-%s, %s, %s);\n", f(i, l).c_str(), mixed ? "fmaf" : "fma",
                   f(i, k).c_str(), f(k, l).c_str(), f(i, l).c_str());
          o += b;
        }
    }
  }
  // y = C^-1 v for a right-hand side v given per A row: forward, then back substitution
  auto solve = [&](const char* vin, const char* yout) {
    std::string r;
    for (int k = 0; k < n; k++) {
      snprintf(b, sizeof b, "      %s y%d = (%s)(%s);\n", T, k, T,
               (std::string(vin) + "(" + std::to_string(sy.prow[k]) + ")").c_str());
      r += b;
    }
    for (int k = 0; k < n; k++)
      for (int i = k + 1; i < n; i++)
        if (C(i, k)) {
          snprintf(b, sizeof b, "      y%d = %s(-%s, y%d, y%d);\n", i, mixed ? "fmaf" : "fma", f(i, k).c_str(), k, i);
          r += b;
        }
    for (int k = n - 1; k >= 0; k--) {
      for (int l = k + 1; l < n; l++)
        if (C(k, l)) {
          snprintf(b, sizeof b, "      y%d = %s(-%s, y%d, y%d);\n", k, mixed ? "fmaf" : "fma", f(k, l).c_str(), l, k);
          r += b;
        }
      snprintf(b, sizeof b, "      y%d *= r%d;\n", k, k);
      r += b;
    }
    for (int k = 0; k < n; k++) {
      snprintf(b, sizeof b, "      %s(%d) = y%d;\n", yout, sy.q[k], k);
      r += b;
    }
    return r;
  };
  if (mode == LU_F32) {
    o += "    {\n" + solve("s.r32", "s.x32") + "    }\n";
    o += "    int kx = 0;\n";
    for (int i = 0; i < n; i++) { snprintf(b, sizeof b, "    kx = max(kx, ks_exp32(s.x32(%d)));\n", i); o += b; }
    o += "    return kx >= 255 ? SOLVE_NONFINITE : SOLVE_OK;\n";
    return o;
  }
  if (!mixed) {
    o += "    {\n" + solve("s.rhs", "s.xn") + "    }\n";
    o += "    long long kx = 0;\n";
    for (int i = 0; i < n; i++) { snprintf(b, sizeof b, "    kx = key_max(kx, mag_key(s.xn(%d)));\n", i); o += b; }
    o += "    return kx >= KS_INF_KEY ? SOLVE_NONFINITE : SOLVE_OK;\n";
    return o;
  }
  // refinement from x_old: r = rhs - A x in FP64 over A's pattern, d = C^-1 r in FP32
  for (int i = 0; i < n; i++) { snprintf(b, sizeof b, "    s.xn(%d) = s.xo(%d);\n", i, i); o += b; }
  o += "    double prev = KS_INF;\n    for (int pass = 0; pass < passes; pass++) {\n";
  for (int i = 0; i < n; i++) {
    snprintf(b, sizeof b, "      { double r = s.rhs(%d);", i);
    o += b;
    for (int j = 0; j < n; j++)
      if ((sy.Amask[i] >> j) & 1u) { snprintf(b, sizeof b, " r = fma(-s.a(%d, %d), s.xn(%d), r);", i, j, j); o += b; }
    snprintf(b, sizeof b, " s.col(%d) = r; }\n", i);
    o += b;
  }
  o += "      {\n" + solve("s.col", "s.col") + "      }\n";
  o += "      long long kd = 0, kx = 0;\n";
  for (int i = 0; i < n; i++) {
    snprintf(b, sizeof b,
             "      { double v = s.xn(%d) + s.col(%d); s.xn(%d) = v; kd = key_max(kd, mag_key(s.col(%d))); "
             "kx = key_max(kx, mag_key(v)); }\n", i, i, i, i);
    o += b;
  }
  o += "      if (kx >= KS_INF_KEY || kd >= KS_INF_KEY) return SOLVE_NONFINITE;\n"
       "      const double dmax = key_mag(kd), xmax = key_mag(kx);\n"
       "      if (dmax <= rtol * xmax || dmax == 0) break;\n"
       "      if (pass > 0 && dmax > 0.5 * prev) return SOLVE_FP32_FAIL;\n"
       "      if (pass == passes - 1 && passes > 1) return SOLVE_FP32_FAIL;\n"
       "      prev = dmax;\n    }\n    return SOLVE_OK;\n";
  return o;
}

}  // namespace

std::string source(const ksh::HostPlan& hp, int T, int kind, bool* reg_out) {
  const int n = hp.n;
  const bool reg = n <= reg_max();
  if (reg_out) *reg_out = reg;
  uint32_t isv = 0;
  for (int i = 0; i < n; i++)
    if (hp.is_v[i]) isv |= 1u << i;
  std::string s;
  char buf[512];
  s += "// per-topology kernels: " + std::to_string(hp.n_elem) + " elements, " + std::to_string(n) + " unknowns\n";
  s += "#include \"ks_tran.cuh\"\nusing namespace ksg;\n\nstruct GenProg {\n";
  snprintf(buf, sizeof buf,
           "  static constexpr int ne = %d, n_nodes = %d, n_state = %d;\n"
           "  static constexpr bool nonlin_empty = %s;\n"
           "  template <class F>\n  __device__ __forceinline__ void each(F&& f) const {\n",
           hp.n_elem, hp.n_nodes, hp.n_state, hp.n_nonlin == 0 ? "true" : "false");
  s += buf;
  for (const KElem& e : hp.elem) append_elem(s, e);
  snprintf(buf, sizeof buf, "  }\n  __device__ __forceinline__ bool is_v(int i) const { return (0x%xu >> i) & 1u; }\n",
           isv);
  s += buf;
  s += "  static constexpr bool kWarp = false;\n"
       "  __device__ __forceinline__ static int64_t x_base(int64_t c, int n) { return c * n; }\n"
       "  __device__ __forceinline__ static int64_t wave_base(int64_t c, int64_t B, int n, int k) {\n"
       "    return ((int64_t)k * B + c) * n;\n  }\n";
  Symbolic sy;
  if (getenv("KS_JIT_STATIC_LU") && atoi(getenv("KS_JIT_STATIC_LU")) == 0) {
    s += "  static constexpr bool kStaticLU = false;\n";
  } else if (symbolic(hp, &sy)) {
    s += "  static constexpr bool kStaticLU = true;\n";
    s += "  // factor and solve on the fixed pivot sequence (steps: A rows";
    for (int k = 0; k < hp.n; k++) s += " " + std::to_string(sy.prow[k]);
    s += "; A columns";
    for (int k = 0; k < hp.n; k++) s += " " + std::to_string(sy.q[k]);
    s += ")\n  template <class SY>\n  __device__ __forceinline__ int lu_fp64(SY& s) const {\n";
    s += emit_lu(sy, LU_FP64);
    s += "  }\n  template <class SY>\n  __device__ __forceinline__ int lu_mixed(SY& s, int passes, double rtol) const {\n";
    s += emit_lu(sy, LU_MIXED);
    s += "  }\n  template <class SY>\n  __device__ __forceinline__ int lu_f32(SY& s) const {\n";
    s += emit_lu(sy, LU_F32);
    s += "  }\n";
  } else {
    s += "  static constexpr bool kStaticLU = false;  // a structurally zero pivot: partial pivoting\n";
  }
  s += "};\n\n";
  snprintf(buf, sizeof buf, "#define KS_T %d\n#define KS_N %d\n", T, n);
  s += buf;
  if (reg) {
    s += "typedef RegSys<KS_N> Sys;\n#define KS_BIND(t)\n";
  } else {
    s += "typedef SmemSys<KS_T, KS_N> Sys;\n"
         "#define KS_BIND(t) extern __shared__ __align__(16) unsigned char smem[]; "
         "smem_layout_static<KS_T, KS_N>(t.s, smem);\n";
  }
  if (kind == KIND_OP) s += R"(
extern "C" __global__ void __launch_bounds__(KS_T)
ks_spec_op(KOpts o, const double* __restrict__ values, const double* __restrict__ derived, double* state,
           double* work, int64_t B, const double* __restrict__ x0, double* out_x, int32_t* out_status,
           int32_t* out_iters, uint64_t deadline_ns, unsigned long long* queue, K32 k32) {
  Thr<Sys, GenProg> t;
  KS_BIND(t)
  t.o = o;
  op_persistent(t, values, derived, state, work, B, x0, out_x, out_status, out_iters, deadline_ns, queue,
                k32.values ? &k32 : nullptr);
}
)";
  else s += R"(
extern "C" __global__ void __launch_bounds__(KS_T)
ks_spec_tran(KOpts o, TranSpecK sp, const double* __restrict__ values, const double* __restrict__ derived,
             double* state, double* work, int64_t B, double* out_time, double* out_wave, int32_t* out_npts,
             int32_t* out_status, int32_t* out_steps, int32_t* out_iters, uint64_t deadline_ns,
             unsigned long long* queue) {
  Thr<Sys, GenProg> t;
  KS_BIND(t)
  t.o = o;
  tran_persistent(t, sp, values, derived, state, work, B, out_time, out_wave, out_npts, out_status, out_steps,
                  out_iters, deadline_ns, queue);
}
)";
  return s;
}

static uint64_t fnv1a(uint64_t h, const void* p, size_t len) {
  const unsigned char* b = static_cast<const unsigned char*>(p);
  for (size_t i = 0; i < len; i++) { h ^= b[i]; h *= 1099511628211ull; }
  return h;
}

static std::string cache_dir() {
  const char* d = getenv("KS_JIT_CACHE_DIR");
  if (d) return strcmp(d, "off") == 0 ? std::string() : std::string(d);
  const char* x = getenv("XDG_CACHE_HOME");
  if (x && *x) return std::string(x) + "/kronspice_gb300";
  const char* h = getenv("HOME");
  if (h && *h) return std::string(h) + "/.cache/kronspice_gb300";
  return std::string();
}

static bool read_file(const std::string& path, std::string* out) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) return false;
  std::string s;
  char buf[65536];
  size_t r;
  while ((r = fread(buf, 1, sizeof buf, f)) > 0) s.append(buf, r);
  fclose(f);
  *out = s;
  return !s.empty();
}

static void write_file(const std::string& dir, const std::string& path, const std::string& data) {
  std::string cur;
  for (size_t i = 1; i <= dir.size(); i++)  // mkdir -p
    if (i == dir.size() || dir[i] == '/') mkdir(dir.substr(0, i).c_str(), 0755);
  std::string tmp = path + ".tmp" + std::to_string(getpid());
  FILE* f = fopen(tmp.c_str(), "wb");
  if (!f) return;
  bool ok = fwrite(data.data(), 1, data.size(), f) == data.size();
  ok = (fclose(f) == 0) && ok;
  if (ok) rename(tmp.c_str(), path.c_str());
  else remove(tmp.c_str());
}

struct Compiled {
  std::string cubin;
  double seconds = 0;
  bool from_disk = false;
};

static std::mutex g_mu;
static std::map<uint64_t, Compiled> g_cubins;
static std::map<uint64_t, cudaLibrary_t> g_libs;

static int compile(const std::string& src, const std::string& arch, uint64_t key, Compiled* out, std::string* err) {
  std::string dir = cache_dir();
  char name[64];
  snprintf(name, sizeof name, "/spec_%016llx_%s.cubin", (unsigned long long)key, arch.c_str());
  if (!dir.empty() && read_file(dir + name, &out->cubin)) { out->from_disk = true; return 0; }
  struct timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  nvrtcProgram prog;
  if (nvrtcCreateProgram(&prog, src.c_str(), "ks_spec.cu", ks_jit_n_headers, ks_jit_header_srcs,
                         ks_jit_header_names) != NVRTC_SUCCESS) {
    *err = "nvrtcCreateProgram failed";
    return -1;
  }
  std::string archopt = "--gpu-architecture=" + arch;
  const char* opts[] = {archopt.c_str(), "-std=c++17", "--generate-line-info", "-DKS_JIT=1"};
  nvrtcResult rc = nvrtcCompileProgram(prog, 4, opts);
  if (rc != NVRTC_SUCCESS) {
    size_t ls = 0;
    nvrtcGetProgramLogSize(prog, &ls);
    std::string log(ls, '\0');
    if (ls) nvrtcGetProgramLog(prog, &log[0]);
    *err = std::string("NVRTC: ") + nvrtcGetErrorString(rc) + "\n" + log.substr(0, 4000);
    nvrtcDestroyProgram(&prog);
    return -1;
  }
  size_t cs = 0;
  nvrtcGetCUBINSize(prog, &cs);
  out->cubin.resize(cs);
  if (cs == 0 || nvrtcGetCUBIN(prog, &out->cubin[0]) != NVRTC_SUCCESS) {
    nvrtcDestroyProgram(&prog);
    *err = "NVRTC produced no cubin for " + arch;
    return -1;
  }
  nvrtcDestroyProgram(&prog);
  clock_gettime(CLOCK_MONOTONIC, &t1);
  out->seconds = (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);
  if (!dir.empty()) write_file(dir, dir + name, out->cubin);
  return 0;
}

static std::string device_arch(int dev, std::string* err) {
  int major = 0, minor = 0;
  if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev) != cudaSuccess) {
    *err = "cannot read the device's compute capability";
    return std::string();
  }
  // architecture-specific targets (sm_90a, sm_100a, sm_103a, ...) from compute capability 9.0 on
  return "sm_" + std::to_string(major) + std::to_string(minor) + (major >= 9 ? "a" : "");
}

#define RT_OK(call, what)                                                        \
  do {                                                                           \
    cudaError_t r_ = (call);                                                     \
    if (r_ != cudaSuccess) {                                                     \
      *err = std::string(what) + ": " + cudaGetErrorString(r_);                  \
      return -1;                                                                 \
    }                                                                            \
  } while (0)

// Per-topology kernel of hp (KIND_OP or KIND_TRAN) for the current device,
// compiled or loaded once.
int get(const ksh::HostPlan& hp, int kind, KsSpec* out, std::string* err) {
  if (hp.n > KS_MAX_DENSE) { *err = "system larger than the thread-per-circuit kernels take"; return -1; }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaFree(0) != cudaSuccess) { *err = "no CUDA device"; return -1; }
  std::string arch = device_arch(dev, err);
  if (arch.empty()) return -1;
  // threads per block: 32 for register systems (a few thousand circuits then
  // spread over every SM), 64 for shared-memory ones (measured faster)
  const int T = hp.n <= reg_max() ? 32 : 64;
  bool reg = false;
  std::string src = source(hp, T, kind, &reg);
  int ver[2] = {0, 0};
  nvrtcVersion(&ver[0], &ver[1]);
  uint64_t key = 1469598103934665603ull;
  key = fnv1a(key, src.data(), src.size());
  for (int i = 0; i < ks_jit_n_headers; i++) key = fnv1a(key, ks_jit_header_srcs[i], strlen(ks_jit_header_srcs[i]));
  key = fnv1a(key, ver, sizeof ver);
  key = fnv1a(key, arch.data(), arch.size());

  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_cubins.find(key);
  if (it == g_cubins.end()) {
    Compiled c;
    if (compile(src, arch, key, &c, err)) return -1;
    it = g_cubins.emplace(key, std::move(c)).first;
  }
  cudaLibrary_t lib = nullptr;
  auto li = g_libs.find(key);
  if (li != g_libs.end()) {
    lib = li->second;
  } else {
    RT_OK(cudaLibraryLoadData(&lib, it->second.cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0),
          "loading the per-topology kernels");
    g_libs[key] = lib;
  }
  cudaKernel_t k = nullptr;
  RT_OK(cudaLibraryGetKernel(&k, lib, kind == KIND_OP ? "ks_spec_op" : "ks_spec_tran"), "per-topology kernel");
  const void* fn = reinterpret_cast<const void*>(k);
  size_t smem = reg ? 0 : ks_sys_smem(hp.n, 0, T);
  int maxSmem = 0;
  cudaDeviceGetAttribute(&maxSmem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (smem > (size_t)maxSmem) { *err = "per-thread systems exceed shared memory"; return -1; }
  RT_OK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "shared memory size");
  int per = 0, sms = 0;
  RT_OK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, T, smem), "occupancy");
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  out->fn = const_cast<void*>(fn);
  out->T = T;
  out->smem = smem;
  out->reg = reg;
  out->device = dev;
  out->blocks = sms * (per > 0 ? per : 1);
  out->compile_s = it->second.seconds;
  out->from_disk = it->second.from_disk;
  out->key = key;
  return 0;
}

}  // namespace ksj

int circuits_per_thread() {
  static int v = [] {
    const char* e = getenv("KS_CIRCUITS_PER_THREAD");
    int k = e ? atoi(e) : 1;
    return k < 1 ? 1 : k;
  }();
  return v;
}

namespace ksj {

int launch(void* fn, unsigned grid, int T, size_t smem, void* stream, void** args, std::string* err) {
  RT_OK(cudaLaunchKernel(fn, dim3(grid), dim3(T), args, smem, (cudaStream_t)stream), "launching a per-topology kernel");
  return 0;
}

}  // namespace ksj
