/*
 * kronspice_gpu.h — C ABI of the GB300 batched circuit-solve engine.
 *
 * The engine replaces, for a whole batch of circuits in one call, the
 * per-circuit hot path of kronspice's analysis package:
 *
 *   analysis.OP            analysis/op.go:331        -> ks_op
 *   (*Sim).dcSolve         analysis/newton.go:95     -> ks_op (fallback chain on device)
 *   analysis.Tran          analysis/tran.go:70       -> ks_tran
 *   analysis.DC            analysis/dc.go:51         -> ks_dc_sweep (the points chained per
 *                                                       circuit), or ks_op with the points as circuits
 *   analysis.AC            analysis/ac.go:76         -> ks_ac
 *   analysis.Options       analysis/op.go:22-62      -> ks_options
 *   analysis.TranSpec/TranOptions analysis/tran.go:26-40 -> ks_tran_spec
 *   solver sentinels       solver/matrix.go:15-20,
 *   analysis sentinels     analysis/newton.go:20, analysis/tran.go:18-22 -> ks_status
 *
 * A Go caller binds these through cgo; a Python caller
 * through ctypes (kronspice_gb300/_lib.py).  Every pointer argument is plain
 * host memory unless the name ends in _dev (device memory).  No function keeps
 * a caller pointer after it returns.  Every function returns a ks_rc.
 *
 * Circuits enter as a topology (element kinds and node connections, shared by
 * every circuit of a batch) plus one value vector per circuit (element values
 * and model parameters).  This is the "one call x N circuits" boundary: the
 * symbolic work (unknown layout, stamp map, matrix pattern, ordering) is done
 * once per topology on the host, the numeric work for all circuits on the GPU.
 */
#ifndef KRONSPICE_GPU_H
#define KRONSPICE_GPU_H

#ifndef __CUDACC_RTC__
#include <stddef.h>
#include <stdint.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- return codes of the API calls ------------------------------------- */
typedef enum {
  KS_OK = 0,
  KS_EINVAL = -1,   /* bad argument, bad topology or value vector            */
  KS_ENOMEM = -2,   /* device or host allocation failed                      */
  KS_ECUDA = -3,    /* a CUDA call failed (message in ks_last_error)         */
  KS_EUNSUPPORTED = -4, /* element or analysis not built into this engine    */
  KS_EVALIDATE = -5 /* structural validation failed (ks_validate's message)  */
} ks_rc;

/* ---- per-circuit status: 1:1 with the Go sentinels --------------------- */
typedef enum {
  KS_STATUS_OK = 0,
  KS_STATUS_SINGULAR = 1,          /* solver.ErrSingularMatrix     solver/matrix.go:17 */
  KS_STATUS_NONFINITE = 2,         /* solver.ErrNonFinite          solver/matrix.go:19 */
  KS_STATUS_NO_CONVERGENCE = 3,    /* analysis.ErrNoConvergence    analysis/newton.go:20 */
  KS_STATUS_TIMESTEP_TOO_SMALL = 4,/* analysis.ErrTimestepTooSmall analysis/tran.go:19 */
  KS_STATUS_TOO_MANY_STEPS = 5,    /* analysis.ErrTooManySteps     analysis/tran.go:20 */
  KS_STATUS_INTERRUPTED = 6,       /* context deadline / cancel    analysis/op.go:81-89 */
  KS_STATUS_NOT_RUN = 7,           /* circuit was not solved (earlier error)          */
  KS_STATUS_LEDGER = 8             /* em.ErrLedgerResidual         em/energy.go:18    */
} ks_status;

/* ---- element kinds (circuit/circuit.go:41-99) --------------------------- */
typedef enum {
  KS_ELEM_R = 1,  /* resistor          device/passive.go:32   */
  KS_ELEM_C = 2,  /* capacitor         device/reactive.go:24  */
  KS_ELEM_L = 3,  /* inductor          device/reactive.go:198 */
  KS_ELEM_V = 4,  /* voltage source    device/source.go:77    */
  KS_ELEM_I = 5,  /* current source    device/source.go:133   */
  KS_ELEM_D = 6,  /* junction diode    device/diode.go:61     */
  KS_ELEM_Q = 7,  /* Gummel-Poon BJT   device/bjt.go:78       */
  KS_ELEM_M = 8,  /* MOSFET level 1-3  device/mosfet.go:43    */
  KS_ELEM_E = 9,  /* VCVS              device/controlled.go:29 */
  KS_ELEM_F = 10, /* CCCS              device/controlled.go:29 */
  KS_ELEM_G = 11, /* VCCS              device/controlled.go:29 */
  KS_ELEM_H = 12, /* CCVS              device/controlled.go:29 */
  KS_ELEM_K = 13, /* mutual inductance device/mutual.go:30     */
  KS_ELEM_S = 14, /* voltage-controlled switch device/switch.go:57 */
  KS_ELEM_W = 15, /* current-controlled switch device/switch.go:57 */
  KS_ELEM_CN = 16, /* nonlinear / time-varying capacitor device/nonlinear_reactive.go:291 */
  KS_ELEM_LN = 17  /* nonlinear / time-varying inductor  device/nonlinear_reactive.go:500 */
} ks_elem_kind;

/* source waveforms (circuit/circuit.go WaveKind; device/waveform.go) */
typedef enum {
  KS_WAVE_NONE = 0,
  KS_WAVE_PULSE = 1,
  KS_WAVE_SIN = 2,
  KS_WAVE_EXP = 3,
  KS_WAVE_PWL = 4
} ks_wave_kind;

/* element flags */
enum {
  KS_F_HAS_DC = 1 << 0,   /* source: DC value given explicitly (Element.HasDC) */
  KS_F_HAS_IC = 1 << 1,   /* C, L: initial condition given (Element.HasIC)      */
  KS_F_HAS_BV = 1 << 2,   /* diode: BV given (DiodeParams.HasBV)                */
  KS_F_PTYPE = 1 << 3,    /* BJT: PNP; MOSFET: PMOS                             */
  KS_F_INT_A = 1 << 4,    /* diode: internal anode node (RS > 0)                */
  KS_F_INT_C = 1 << 5,    /* BJT: internal collector (RC > 0)                   */
  KS_F_INT_B = 1 << 6,    /* BJT: internal base (RB > 0)                        */
  KS_F_INT_E = 1 << 7,    /* BJT: internal emitter (RE > 0)                     */
  KS_F_INT_D = 1 << 8,    /* MOSFET: internal drain (conductance 1/RD > 0)      */
  KS_F_INT_S = 1 << 9,    /* MOSFET: internal source (conductance 1/RS > 0)     */
  KS_F_LATERAL = 1 << 10  /* BJT: SUBS < 0, substrate junction to the base      */
};

/*
 * One circuit element.  node[] holds circuit node indices (0 = ground):
 *   R C L V I D : node[0] = n+ (anode), node[1] = n- (cathode)
 *   Q (BJT)     : node[0] = collector, node[1] = emitter, node[2] = base,
 *                 node[3] = substrate (0 = ground when absent)
 *                 -- Element.Nodes/Extra of circuit/builder.go:101
 *   M (MOSFET)  : node[0] = drain, node[1] = source, node[2] = gate,
 *                 node[3] = bulk    -- circuit/builder.go:108
 *   E, G        : node[0] = n+, node[1] = n-, node[2] = nc+, node[3] = nc-
 *                 (the controlling voltage, Element.CtrlNodes)
 *   F, H        : node[0] = n+, node[1] = n-, node[2] = index in elem[] of
 *                 the controlling voltage source (Element.CtrlSource; its
 *                 branch current, positive into its n+ terminal)
 *   K           : node[0], node[1] = indices in elem[] of the two coupled
 *                 inductors (Element.Couples); no circuit nodes
 *   S           : node[0] = n+, node[1] = n-, node[2] = nc+, node[3] = nc-
 *                 (the controlling voltage, Element.CtrlNodes)
 *   W           : node[0] = n+, node[1] = n-, node[2] = index in elem[] of
 *                 the controlling voltage source (Element.CtrlSource)
 *   CN, LN      : node[0] = n+, node[1] = n-; wave = the SCALE waveform
 *                 (KS_WAVE_NONE: s = 1), nargs = its arguments, level = the
 *                 number of curve values (2 x knots of Q=pwl / FLUX=pwl;
 *                 0: the linear law value * x)
 * param is the offset of the element's block in the per-circuit value vector;
 * the block layouts are the KS_*_P_* enums below.
 */
typedef struct {
  int32_t kind;
  int32_t node[4];
  int32_t flags;
  int32_t level;     /* MOSFET level 1..3                                    */
  int32_t wave;      /* source waveform kind                                 */
  int32_t nargs;     /* source waveform arguments given (PULSE 2..7, SIN 2..6, EXP 2..6, PWL even) */
  int32_t param;     /* offset of the element's value block                  */
  uint64_t given;    /* MOSFET: bit KS_M_P_x set when model parameter x was given */
} ks_element;

typedef struct {
  int32_t n_nodes;   /* circuit nodes including ground                      */
  int32_t n_elem;
  int32_t n_values;  /* length of each circuit's value vector               */
  int32_t reserved;
  const ks_element* elem;
} ks_topology;

/* value blocks -------------------------------------------------------------*/
/* R: [R]   C: [C, IC]   L: [L, IC] */
enum { KS_RCL_P_VALUE = 0, KS_RCL_P_IC = 1, KS_RCL_NP = 2 };
/* E, F, G, H: [gain]   K: [coupling coefficient k] */
enum { KS_CTL_P_GAIN = 0, KS_K_P_COUPLING = 0, KS_CTL_NP = 1 };
/* S, W: [threshold VT (S, volts) or IT (W, amperes), hysteresis VH or IH
 * (negative: the smooth switch), RON, ROFF, initial state (1 = ON, 0 = OFF)]:
 * circuit.SwitchParams of circuit/switch.go:36-50 after defaults */
enum { KS_SW_P_VT = 0, KS_SW_P_VH = 1, KS_SW_P_RON = 2, KS_SW_P_ROFF = 3, KS_SW_P_ON = 4, KS_SW_NP = 5 };
/* CN, LN: [value (C or L of the linear law, 0 with a curve), IC, SCALE
 * arguments (nargs), curve x0, y0, x1, y1, ... (level values)]: the charge
 * q = s(t) Q(v) or flux linkage s(t) L(i) of circuit.NonlinearCapacitor /
 * NonlinearInductor (Element.Value, IC, Scale, Curve) */
enum { KS_NL_P_VALUE = 0, KS_NL_P_IC = 1, KS_NL_P_ARGS = 2 };
/* V, I: [dc, ac_mag, ac_phase_deg, arg0 .. arg(nargs-1)] */
enum { KS_SRC_P_DC = 0, KS_SRC_P_ACMAG = 1, KS_SRC_P_ACPHASE = 2, KS_SRC_P_ARGS = 3 };
/* D: DiodeParams of device/diode.go:23 after defaults and area scaling */
enum {
  KS_D_P_IS, KS_D_P_N, KS_D_P_RS, KS_D_P_CJO, KS_D_P_VJ, KS_D_P_M, KS_D_P_TT,
  KS_D_P_BV, KS_D_P_IBV, KS_D_P_FC, KS_D_NP
};
/* Q: BJTParams of device/bjt.go:17 after defaults, RBM <= RB, SUBS and area */
enum {
  KS_Q_P_IS, KS_Q_P_BF, KS_Q_P_NF, KS_Q_P_VAF, KS_Q_P_IKF, KS_Q_P_ISE, KS_Q_P_NE,
  KS_Q_P_BR, KS_Q_P_NR, KS_Q_P_VAR, KS_Q_P_IKR, KS_Q_P_ISC, KS_Q_P_NC,
  KS_Q_P_RB, KS_Q_P_IRB, KS_Q_P_RBM, KS_Q_P_RE, KS_Q_P_RC,
  KS_Q_P_CJE, KS_Q_P_VJE, KS_Q_P_MJE, KS_Q_P_TF, KS_Q_P_XTF, KS_Q_P_VTF,
  KS_Q_P_ITF, KS_Q_P_CJC, KS_Q_P_VJC, KS_Q_P_MJC, KS_Q_P_XCJC, KS_Q_P_TR,
  KS_Q_P_CJS, KS_Q_P_VJS, KS_Q_P_MJS, KS_Q_P_FC, KS_Q_P_ISS, KS_Q_P_NS,
  KS_Q_P_SUBS, KS_Q_NP
};
/* M: mosParams of device/mosfet.go:97 (model defaults of :140-149 applied)
 * followed by the instance parameters */
enum {
  KS_M_P_VTO, KS_M_P_KP, KS_M_P_GAMMA, KS_M_P_PHI, KS_M_P_LAMBDA, KS_M_P_RD,
  KS_M_P_RS, KS_M_P_CBD, KS_M_P_CBS, KS_M_P_IS, KS_M_P_PB, KS_M_P_CGSO,
  KS_M_P_CGDO, KS_M_P_CGBO, KS_M_P_RSH, KS_M_P_CJ, KS_M_P_MJ, KS_M_P_CJSW,
  KS_M_P_MJSW, KS_M_P_JS, KS_M_P_TOX, KS_M_P_NSUB, KS_M_P_NSS, KS_M_P_NFS,
  KS_M_P_TPG, KS_M_P_XJ, KS_M_P_LD, KS_M_P_UO, KS_M_P_UCRIT, KS_M_P_UEXP,
  KS_M_P_UTRA, KS_M_P_VMAX, KS_M_P_NEFF, KS_M_P_FC, KS_M_P_DELTA,
  KS_M_P_THETA, KS_M_P_ETA, KS_M_P_KAPPA, KS_M_P_WD,
  KS_M_P_L, KS_M_P_W, KS_M_P_AD, KS_M_P_AS, KS_M_P_PD, KS_M_P_PS,
  KS_M_P_NRD, KS_M_P_NRS, KS_M_P_MULT, KS_M_NP
};

/* ---- analysis options (analysis/op.go:22-62, defaults :91-110) ---------- */
enum { KS_PREC_FP64 = 0, KS_PREC_MIXED = 1 };
/* backend: DENSE / SPARSE pick the CPU oracle's linear solver; on the GPU,
 * GENERIC forces the generic thread-per-circuit kernels, SPECIALIZED the
 * per-topology kernels (compiled at run time, ks_plan_specialize), and AUTO
 * takes the per-topology kernels for large batches. */
enum { KS_BACKEND_AUTO = 0, KS_BACKEND_DENSE = 1, KS_BACKEND_SPARSE = 2, KS_BACKEND_GENERIC = 3,
       KS_BACKEND_SPECIALIZED = 4 };
/* Kernel of a batch's last analysis (ks_batch_last_kernel). */
enum { KS_KERNEL_GENERIC = 0, KS_KERNEL_SPEC_REG = 1, KS_KERNEL_SPEC_SMEM = 2 };

typedef struct {
  double reltol;   /* <= 0: 1e-3  */
  double abstol;   /* <= 0: 1e-12 */
  double vntol;    /* <= 0: 1e-6  */
  double gmin;     /* <= 0: 1e-12 */
  int32_t itl1;    /* <= 0: 100   */
  int32_t itl4;    /* <= 0: 10    */
  int32_t no_gmin_stepping;
  int32_t no_source_stepping;
  int32_t no_pseudo_transient;
  int32_t precision;      /* KS_PREC_FP64 (plain) or KS_PREC_MIXED          */
  int32_t backend;        /* KS_BACKEND_*                                   */
  int32_t max_iter_total; /* device-side bound on all Newton iterations of one
                             circuit, fallbacks included (0: unbounded by it) */
  double deadline_s;      /* > 0: per-call wall-clock limit, the context
                             deadline of Options.Context (KS_STATUS_INTERRUPTED) */
  int32_t mixed_passes;   /* KS_PREC_MIXED: most FP64-residual refinement passes
                             per linear solve (<= 0: 6).  Refinement stops at a
                             correction below 1e-3 reltol of the solution (1e-11
                             for linear circuits); a solve that does not get
                             there, or whose refinement stops contracting, goes
                             to FP64.  1: one unchecked pass, each Newton step
                             the FP32 solve of the FP64 residual
                             (well-conditioned systems only). */
  int32_t fp32_start_iters; /* operating points (ks_op, ks_ac): > 0 runs an FP32
                             stage of at most this many Newton iterations from the
                             start (x0, or InitJct without one), with the devices
                             evaluated and the system factored in FP32 and
                             dcSolve's gmin / source stepping when Newton fails,
                             and starts the FP64 solve from the point it reaches
                             (NodeSet semantics).  The FP64 Newton, its convergence
                             test and its fallback chain are unchanged, so the
                             stage changes how many FP64 iterations a circuit
                             takes, not its result.  Circuits whose stage fails
                             keep their start.  Covers R, C, L, V, I, diodes, BJTs
                             and level-1 MOSFETs; other topologies skip it.
                             0: off. */
  double start_check;     /* operating points with x0: > 0 solves a circuit again
                             from the standard start (InitJct and the full dcSolve
                             chain) when its solution ends farther than this many
                             volts from x0 at any node: the check a learned start
                             uses to catch a prediction that led Newton to another
                             operating point.  Its iterations count in out_iters.
                             0: no check. */
  double ledger_tol;      /* ks_op_results / ks_tran_results: relative ledger
                             residual above which a circuit gets KS_STATUS_LEDGER
                             (Options.LedgerTolerance; <= 0: 1e-9,
                             em.DefaultTolerance em/energy.go:21) */
  int32_t skip_energy_check; /* Options.SkipEnergyCheck: build the ledger, never
                             fail a circuit on it */
  int32_t step_predictor; /* transients: > 0 starts each time step's Newton from
                             the extrapolation of the accepted history (the
                             polynomial through the last three accepted points,
                             two before there are three) instead of from the
                             last one (analysis/tran.go:164); never across a
                             breakpoint.  The Newton, its convergence test, the
                             device limiting (from the accepted junction
                             voltages) and the step control are the reference's,
                             so the start changes how many iterations a step
                             takes.  0: off. */
  int32_t autotune;       /* ks_op / ks_op_async: > 0 times the operating-point
                             kernels this batch can run (the per-topology kernel
                             when the plan has one, the generic kernel; each with
                             1, 2 or 4 circuits per thread of the persistent grid)
                             on the first call for the plan, analysis and batch
                             size (to the power of two), keeps the fastest in the
                             plan and runs it then and on later calls (the tuning
                             call synchronizes its stream).  The kernels run the
                             same algorithm, so the choice changes the time, not
                             the result beyond the Newton tolerance.  0: the
                             fixed rules (KS_JIT_MIN_BATCH, KS_CIRCUITS_PER_THREAD). */
} ks_options;

/* ---- transient request (analysis/tran.go:26-59) ------------------------- */
enum { KS_METHOD_BE = 1, KS_METHOD_TRAP = 2 };

typedef struct {
  double step, stop, start, max_step; /* TranSpec                              */
  int32_t uic;
  int32_t method;     /* 0: trapezoidal                                       */
  int32_t fixed_step; /* 1: steps of exactly `step`, no LTE control, no
                         breakpoint landing (the batch mode of the configs)   */
  int32_t max_steps;  /* <= 0: 1,000,000                                      */
  double chgtol;      /* <= 0: 1e-14 */
  double trtol;       /* <= 0: 7     */
  double min_step;    /* <= 0: 1e-12 * stop */
} ks_tran_spec;

#ifndef __CUDACC_RTC__ /* the device code compiled at run time needs only the layout above */
/* ---- library ------------------------------------------------------------ */
const char* ks_version(void);
/* Message of the last failed call on this host thread ("" if none). */
const char* ks_last_error(void);

/*
 * Structural check of one circuit, the equivalent of circuit.Validate
 * (circuit/circuit.go:368, checkPaths :704-804) for the element kinds above.
 * Returns KS_OK or KS_EVALIDATE with the reason (ErrFloatingNode, ErrBadValue,
 * ErrSelfConnected, ...) in ks_last_error.  transient != 0 gives
 * ValidateTransient (capacitors count as paths, for UIC).
 */
int ks_validate(const ks_topology* topo, const double* values, int transient);

/* Number of MNA unknowns of the topology (node voltages, branch currents,
 * internal nodes: the layout of device/device.go:36-100) and, if is_voltage is
 * not NULL, whether each unknown is a voltage (1) or a current (0). */
int ks_unknowns(const ks_topology* topo, int32_t* n_unknowns, int32_t* is_voltage);

/* ---- plans and batches --------------------------------------------------- */
typedef struct ks_plan ks_plan;   /* one topology, symbolic analysis done   */
typedef struct ks_batch ks_batch; /* n circuits of one plan, values on device */
typedef struct ks_multi ks_multi; /* n circuits of different topologies       */

/* Analyse a topology: unknown layout, stamp map, matrix pattern.  The plan
 * owns copies of everything it needs. */
int ks_plan_create(const ks_topology* topo, ks_plan** out);
void ks_plan_destroy(ks_plan* plan);
int ks_plan_info(const ks_plan* plan, int32_t* n_unknowns, int32_t* n_values, int32_t* n_state);

/* Per-topology kernels (engine-specific, no counterpart in the reference): the
 * plan's element program written out as CUDA source with every element a
 * compile-time constant, compiled by NVRTC for the current device, one kernel
 * per analysis (KS_ANALYSIS_OP: ks_op, KS_ANALYSIS_TRAN: ks_tran).  Compiles
 * (or loads from the cubin cache) now instead of at the first large analysis;
 * *kernel receives KS_KERNEL_SPEC_REG or KS_KERNEL_SPEC_SMEM, *compile_s the
 * NVRTC time (0 when cached).  KS_EUNSUPPORTED with the compiler log in
 * ks_last_error when it does not compile. */
enum { KS_ANALYSIS_OP = 0, KS_ANALYSIS_TRAN = 1 };
int ks_plan_specialize(ks_plan* plan, int32_t analysis, int32_t* kernel, double* compile_s);
/* The generated source of one analysis' kernel (NUL-terminated, truncated to
 * cap-1 bytes; *len = full size). */
int ks_plan_kernel_source(const ks_plan* plan, int32_t analysis, char* buf, size_t cap, size_t* len);

/* Allocate device storage for n_circ circuits of a plan and upload their
 * value vectors (row-major [n_circ][n_values], host memory). */
int ks_batch_create(ks_plan* plan, int32_t n_circ, const double* values, ks_batch** out);
/* Replace the value vectors of an existing batch (same n_circ); host memory,
 * or device memory when values_are_device != 0 (then `values` is a device
 * pointer to [n_circ][n_values] doubles). */
int ks_batch_set_values(ks_batch* b, const double* values, int values_are_device, void* stream);
/* KS_KERNEL_* that ran the batch's last analysis (-1 before the first). */
int ks_batch_last_kernel(const ks_batch* b);
/* The batch's cancel word, the context cancellation of Options.Context
 * (analysis/op.go:81-89, checked per Newton iteration, step and frequency there):
 * an int32 in page-locked host memory mapped into the device's address space,
 * allocated by the first call and valid until ks_batch_destroy.  While it is
 * non-zero, the batch's operating-point, AC and transient kernels end every
 * unfinished circuit with KS_STATUS_INTERRUPTED, the running ones included: each
 * circuit reads the word before its first Newton iteration and every eighth one
 * after.  The host writes it from any thread while the kernels run (the Go
 * wrapper on ctx.Done()); reset it to 0 before the next analysis. */
int ks_batch_cancel_word(ks_batch* b, volatile int32_t** word);

/* ---- batches of different topologies --------------------------------------
 * analysis.OP / analysis.Tran for n_circ circuits that share nothing: each has
 * its own topology and size (thousands of unknowns each at most by memory),
 * the way a caller runs a pool of goroutines over unrelated circuits
 * (evo/engine.go:519-543).  One warp per circuit on the GPU; the host computes
 * each circuit's sparse pattern, fill and fixed pivot sequence once, at
 * creation (solver/sparse.go:154-187, :412-452).  topos[c] / values +
 * value_offsets[c] are circuit c's topology and value vector (host memory).
 * Results are concatenated per circuit in circuit order: x [sum n_c], fixed-step
 * waveforms [sum over c of n_points * n_c], each circuit's block [n_points][n_c]. */
/* The host's analysis of one circuit (no GPU work; values: its value vector,
 * which picks the pivot rows at DC when step = 0, else with the trapezoidal
 * companions of that time step): unknowns, slots of L + U with fill,
 * multiply-adds of one numeric factorization, the fixed pivot sequence (step k
 * pivots A row prow[k] on A column pcol[k]; [n] each) and the pattern of L + U
 * in step coordinates (rowptr [n + 1], cols [slots], columns ascending in each
 * row).  Output pointers are optional. */
int ks_sparse_analyze(const ks_topology* topo, const double* values, double step, int32_t* n, int64_t* slots, int64_t* lu_flops, int32_t* prow,
                      int32_t* pcol, int32_t* rowptr, int32_t* cols);
/* The pattern the analysis above orders (solver/sparse.go:114-143: every entry
 * the elements' loads stamp over an operating point (transient = 0) or a
 * transient, plus every diagonal), as an n x n byte matrix, row-major.  The
 * column order (pcol of ks_sparse_analyze) is minimumDegree of it
 * (solver/sparse.go:412-452). */
int ks_sparse_pattern(const ks_topology* topo, const double* values, int32_t transient, int32_t* n, uint8_t* pattern);
int ks_multi_create(int32_t n_circ, const ks_topology* topos, const double* values, const int64_t* value_offsets,
                    ks_multi** out);
void ks_multi_destroy(ks_multi* m);
/* Totals, and each circuit's unknown count (n_per_circuit [n_circ], optional). */
int ks_multi_info(const ks_multi* m, int64_t* total_unknowns, int64_t* factor_slots, int64_t* lu_flops,
                  int32_t* n_per_circuit);
int ks_multi_op(ks_multi* m, const ks_options* opt, double* out_x, int32_t* out_status, int32_t* out_iters);
int ks_multi_op_async(ks_multi* m, const ks_options* opt, double* out_x_dev, int32_t* out_status_dev,
                      int32_t* out_iters_dev, void* stream);
/* Fixed-step transients only (spec->fixed_step = 1). */
int ks_multi_tran(ks_multi* m, const ks_tran_spec* spec, const ks_options* opt, double* out_wave,
                  int32_t* out_status, int32_t* out_steps, int32_t* out_iters);
int ks_multi_tran_async(ks_multi* m, const ks_tran_spec* spec, const ks_options* opt, double* out_wave_dev,
                        int32_t* out_npts_dev, int32_t* out_status_dev, int32_t* out_steps_dev,
                        int32_t* out_iters_dev, void* stream);

/* ---- operating point without device allocation --------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory when they solve (a memory pool or arena that owns the device, a path
 * where an allocation could synchronise the device or fail under pressure):
 * ks_op for n_circ circuits of one topology with every intermediate array in a
 * fixed scratch area of KS_NOALLOC_SCRATCH_BYTES that the library holds on each
 * GPU that loads it, and no cudaMalloc / cudaFree.  values_dev: device memory
 * [n_circ][n_values] row-major; out_x_dev [n_circ][n], out_status_dev and
 * out_iters_dev [n_circ]: device memory.  Returns KS_EINVAL when the batch needs
 * more scratch than that (ks_op_noalloc_scratch_bytes gives the need).  Runs the
 * generic kernel from the standard start without the FP32 start stage; a
 * request for the per-topology kernels (KS_BACKEND_SPECIALIZED) is refused with
 * KS_EUNSUPPORTED, since loading their code allocates device memory.  All calls
 * share the scratch: calls that overlap on the GPU race.  The first call on a
 * device looks up the scratch address; make it before any stream capture.  The
 * call copies the element table to the device on `stream` and waits for that
 * copy (so it also waits for the work queued on `stream` before it); the solve
 * itself is queued on `stream` and the call returns without waiting for it. */
#define KS_NOALLOC_SCRATCH_BYTES (64u << 20)
int ks_op_noalloc(const ks_topology* topo, int32_t n_circ, const double* values_dev, const ks_options* opt,
                  double* out_x_dev, int32_t* out_status_dev, int32_t* out_iters_dev, void* stream);
int ks_op_noalloc_scratch_bytes(const ks_topology* topo, int32_t n_circ, size_t* bytes);
void ks_batch_destroy(ks_batch* b);

/*
 * DC operating point of every circuit of the batch (analysis.OP for each):
 * Newton with the SPICE3 convergence test, then gmin stepping, source
 * stepping and pseudo-transient continuation on the circuits that fail.
 *   x0        NULL (cold start: InitJct) or [n_circ][n_unknowns] starting
 *             points (Options.NodeSet semantics: device limiting state is
 *             seeded from the guess, analysis/newton.go:221-243)
 *   out_x     [n_circ][n_unknowns] solutions
 *   out_status[n_circ] ks_status, out_iters[n_circ] Newton iterations used
 * All host buffers; the call returns when the results are in them.
 */
int ks_op(ks_batch* b, const ks_options* opt, const double* x0, double* out_x,
          int32_t* out_status, int32_t* out_iters, void* stream);

/* Same, on device buffers, asynchronous on `stream` (NULL: the batch's own
 * stream).  x0_dev may be NULL. */
int ks_op_async(ks_batch* b, const ks_options* opt, const double* x0_dev, double* out_x_dev,
                int32_t* out_status_dev, int32_t* out_iters_dev, void* stream);

/*
 * AC small-signal sweep of every circuit of the batch (analysis.AC,
 * analysis/ac.go:76-150): the operating point (as ks_op, followed by the
 * polish of analysis/op.go:251-271: up to two more FP64 solves), then for each
 * frequency f the complex system (G + j*2*pi*f*C) x = b of the devices' LoadAC
 * stamps, solved as solver/cdense.go does.  freqs [n_freq] in Hz, the list of
 * ACSpec.Frequencies (analysis/ac.go:33-72; made by the caller).
 * out_x [n_circ][n_freq][n][2]: every unknown's phasor (real, imaginary), node
 * voltages first (x[i] is node i+1), zeros at a frequency whose solve failed
 * and at every frequency of a circuit whose operating point failed.
 * out_status [n_circ]: the operating point's status, else that of the first
 * failing frequency (KS_STATUS_SINGULAR: "f = %g Hz: singular matrix",
 * KS_STATUS_NONFINITE).  out_iters [n_circ]: Newton solves of the operating point.
 * ks_options.precision chooses the operating point's LU as in ks_op; the polish
 * and the AC solves are FP64.  Replaces analysis.AC per circuit (ledger and
 * element currents are the caller's post-processing of the phasors).
 */
int ks_ac(ks_batch* b, const ks_options* opt, const double* x0, const double* freqs, int32_t n_freq,
          double* out_x, int32_t* out_status, int32_t* out_iters, void* stream);

/* Same, on device buffers (freqs_dev, out_x_dev, out_status_dev, out_iters_dev;
 * x0_dev, out_status_dev and out_iters_dev may be NULL), asynchronous on
 * `stream` (NULL: the batch's own stream). */
int ks_ac_async(ks_batch* b, const ks_options* opt, const double* x0_dev, const double* freqs_dev,
                int32_t n_freq, double* out_x_dev, int32_t* out_status_dev, int32_t* out_iters_dev, void* stream);

/*
 * DC sweep of every circuit of the batch (analysis.DC, analysis/dc.go:51-133):
 * element `src` (a V or I source) takes values[0 .. npts-1] in order as its DC
 * value, for each of values2[0 .. npts2-1] of a second, outer source src2 in
 * turn (src2 < 0: one sweep), and each point is an operating point
 * warm-started from the previous point's solution and device state (no
 * InitJct once a point has converged; a switch's state and the junctions'
 * limiting history carry over), as the reference chains a sweep.  A circuit's
 * sweep stops at its first failing point.  At most 1,000,000 points.
 *   out_x      [n_circ][npts2][npts][n_unknowns]   (after a failure: untouched)
 *   out_status [n_circ]  KS_STATUS_OK, or the failing point's status
 *   out_points [n_circ]  points solved
 *   out_iters  [n_circ]  Newton iterations over the sweep
 * Host buffers; synchronous.  Replaces analysis.DC per circuit (no ledger
 * check per point).
 */
int ks_dc_sweep(ks_batch* b, const ks_options* opt, int32_t src, const double* values, int32_t npts,
                int32_t src2, const double* values2, int32_t npts2, double* out_x, int32_t* out_status,
                int32_t* out_points, int32_t* out_iters, void* stream);

/* The sweep alone, about operating points the caller already has (device
 * buffers): x_op_dev [n_circ][n] (a ks_op / ks_op_async result; the small-signal
 * model is taken at exactly these values, so pass polished points for results
 * independent of the Newton tolerance), status_dev [n_circ] (NULL: all solved;
 * circuits with a non-zero status are skipped).  out_status_dev receives
 * status_dev updated with each circuit's first failing frequency.  Only
 * ks_options.gmin is read. */
int ks_ac_at(ks_batch* b, const ks_options* opt, const double* x_op_dev, const int32_t* status_dev,
             const double* freqs_dev, int32_t n_freq, double* out_x_dev, int32_t* out_status_dev, void* stream);

/*
 * Transient analysis of every circuit of the batch (analysis.Tran for each).
 * Fixed-step mode (spec->fixed_step) records n_points = round((stop)/step)+1
 * points t_k = k*step for every circuit:
 *   out_wave  [n_points][n_circ][n_unknowns]  (NULL: not recorded)
 * Adaptive mode records up to `capacity` accepted points per circuit:
 *   out_time  [n_circ][capacity], out_wave [n_circ][capacity][n_unknowns],
 *   out_npts  [n_circ]
 * out_status[n_circ], out_steps[n_circ] accepted steps, out_iters[n_circ]
 * total Newton iterations.
 */
int ks_tran(ks_batch* b, const ks_tran_spec* spec, const ks_options* opt,
            int32_t capacity, double* out_time, double* out_wave, int32_t* out_npts,
            int32_t* out_status, int32_t* out_steps, int32_t* out_iters, void* stream);

/* Same, on device buffers, asynchronous on `stream` (NULL: the batch's own
 * stream); any output pointer may be NULL. */
int ks_tran_async(ks_batch* b, const ks_tran_spec* spec, const ks_options* opt, int32_t capacity,
                  double* out_time_dev, double* out_wave_dev, int32_t* out_npts_dev,
                  int32_t* out_status_dev, int32_t* out_steps_dev, int32_t* out_iters_dev, void* stream);

/* Number of points a fixed-step transient records. */
int ks_tran_points(const ks_tran_spec* spec, int32_t* n_points);

/* ---- element results and the energy ledger -------------------------------
 * What the reference's analyses return beside the solution: each element's
 * operating point and power, and the open-system energy ledger.  Computed on
 * the device at the accepted solution, from the linearization of each device's
 * last load, as (*Sim).result (analysis/op.go:361-403) and the transient
 * recorder (analysis/tran.go:291-386) do; the ledger sums follow
 * em.Accumulator (em/energy.go:24-80): a port's power goes to dissipation when
 * it leaves through the thermal port, else to inflow or outflow; storage
 * powers and model-supplied powers in their own columns.  Round-off estimate:
 * 64 * 2^-52 * sum |x_i| (|A| |x| + |rhs|)_i of the last linear system
 * (analysis/op.go:275-282).  These calls run on the generic kernels.
 *
 * Columns of one element's row (output.ElementResult): */
enum { KS_RES_VOLTAGE = 0,        /* Voltage (terminal 1 - terminal 2)            */
       KS_RES_CURRENT = 1,        /* Current (into terminal 1)                    */
       KS_RES_POWER = 2,          /* PowerAbsorbed                                */
       KS_RES_STORAGE_POWER = 3,  /* StoragePower (energy-storing elements)       */
       KS_RES_STORED_ENERGY = 4,  /* StoredEnergy                                 */
       KS_RES_EXTERIOR_POWER = 5, /* ExteriorPower through the element's modeled
                                     exterior port: thermal for R > 0, D, Q, M;
                                     electrical for V and I; none for C, L and
                                     R < 0 (0)                                    */
       KS_RES_MODEL_SUPPLIED = 6, /* ModelSuppliedPower (R < 0)                   */
       KS_RES_COLS = 7 };
/* Columns of an operating point's ledger (output.Ledger, em.BuildLedger
 * em/energy.go:90-121): */
enum { KS_LEDGER_INFLOW = 0, KS_LEDGER_OUTFLOW = 1, KS_LEDGER_DISSIPATION = 2, KS_LEDGER_STORAGE_RATE = 3,
       KS_LEDGER_MODEL_SUPPLIED = 4, KS_LEDGER_RESIDUAL = 5, KS_LEDGER_SCALE = 6, KS_LEDGER_ROUNDOFF = 7,
       KS_LEDGER_COLS = 8 };
/* Columns of one transient point's ledger (the Waveform's Ledger series,
 * analysis/tran.go:336-345): */
enum { KS_TPOINT_INFLOW = 0, KS_TPOINT_OUTFLOW = 1, KS_TPOINT_DISSIPATION = 2, KS_TPOINT_STORAGE_RATE = 3,
       KS_TPOINT_MODEL_SUPPLIED = 4, KS_TPOINT_RESIDUAL = 5, KS_TPOINT_STORED_ENERGY = 6, KS_TPOINT_COLS = 7 };
/* Columns of a transient's ledger summary (recorder.finish, analysis/tran.go:350-386): */
enum { KS_TSUM_MAX_RELATIVE_RESIDUAL = 0, KS_TSUM_ENERGY_IN = 1, KS_TSUM_ENERGY_OUT = 2,
       KS_TSUM_ENERGY_DISSIPATED = 3, KS_TSUM_ENERGY_MODEL_SUPPLIED = 4, KS_TSUM_STORED_START = 5,
       KS_TSUM_STORED_END = 6, KS_TSUM_INTEGRATION_MISMATCH = 7, KS_TSUM_COLS = 8 };

/* The operating point of every circuit (as ks_op) with its results:
 *   out_elem   [n_circ][n_elem][KS_RES_COLS]   (NULL: not written)
 *   out_ledger [n_circ][KS_LEDGER_COLS]        (NULL: not written)
 * and em.CheckLedger (em/energy.go:123-128) on each solved circuit: a relative
 * residual above ks_options.ledger_tol gives KS_STATUS_LEDGER unless
 * skip_energy_check.  Rows of circuits that did not solve are zeros.
 * Replaces analysis.OP's *output.Result (analysis/op.go:340-357). */
int ks_op_results(ks_batch* b, const ks_options* opt, const double* x0, double* out_x, int32_t* out_status,
                  int32_t* out_iters, double* out_elem, double* out_ledger, void* stream);
int ks_op_results_async(ks_batch* b, const ks_options* opt, const double* x0_dev, double* out_x_dev,
                        int32_t* out_status_dev, int32_t* out_iters_dev, double* out_elem_dev,
                        double* out_ledger_dev, void* stream);

/* A transient (as ks_tran) with the Waveform's element series and ledger at
 * every recorded point, laid out as out_wave (fixed-step: [n_points][n_circ][...],
 * adaptive: [n_circ][capacity][...]):
 *   out_elem   [...][n_elem][2]  current and absorbed power (Waveform.I, .P)
 *   out_ledger [...][KS_TPOINT_COLS]
 *   out_summary [n_circ][KS_TSUM_COLS]
 * Every point is checked as recorder.record does (analysis/tran.go:291-318):
 * a point out of balance by more than 1e-3 of the run's peak power stops the
 * circuit with KS_STATUS_LEDGER, and so does a largest relative residual above
 * ks_options.ledger_tol at the end (unless skip_energy_check).  The imposed
 * first point of a UIC run is recorded, not checked.  In fixed-step mode the
 * recorded (grid) points are the checked points.  Any output may be NULL. */
int ks_tran_results(ks_batch* b, const ks_tran_spec* spec, const ks_options* opt, int32_t capacity,
                    double* out_time, double* out_wave, double* out_elem, double* out_ledger, double* out_summary,
                    int32_t* out_npts, int32_t* out_status, int32_t* out_steps, int32_t* out_iters, void* stream);
int ks_tran_results_async(ks_batch* b, const ks_tran_spec* spec, const ks_options* opt, int32_t capacity,
                          double* out_time_dev, double* out_wave_dev, double* out_elem_dev, double* out_ledger_dev,
                          double* out_summary_dev, int32_t* out_npts_dev, int32_t* out_status_dev,
                          int32_t* out_steps_dev, int32_t* out_iters_dev, void* stream);

/* ---- learned Newton start ------------------------------------------------
 * A BF16 MLP in -> H -> H -> H -> out (ReLU) on the GPU's tensor cores that
 * predicts each circuit's Newton starting point from its parameter vector.
 * It plays the role of Options.NodeSet (analysis/op.go:39-43, applied by
 * analysis/newton.go:221-243): plain Newton corrects the prediction, and the
 * gmin/source-stepping chain takes over when Newton from it fails. */
typedef struct ks_mlp ks_mlp;

int ks_mlp_create(int32_t in_dim, int32_t hidden, int32_t out_dim, uint64_t seed, ks_mlp** out);
void ks_mlp_destroy(ks_mlp* m);
int ks_mlp_num_params(const ks_mlp* m, int64_t* n);
/* FP32 parameters, layout per layer l: W_l [out][in] row-major, then b_l [out]. */
int ks_mlp_get_params(const ks_mlp* m, float* host);
int ks_mlp_set_params(ks_mlp* m, const float* host);
/* Features: value-vector columns `cols[in_dim]`, log-transformed where bit j of
 * logmask is set, standardized by fmean/fstd; targets: unknowns 0..out_dim-1
 * divided by value column scale_col (-1: not divided), standardized by
 * tmean/tstd. */
int ks_mlp_set_io(ks_mlp* m, const int32_t* cols, uint64_t logmask, const float* fmean, const float* fstd,
                  const float* tmean, const float* tstd, int32_t scale_col);
/* One forward and backward pass on host data (standardized X [rows][in],
 * T [rows][out]); FP32 gradients in the parameter layout and the MSE loss. */
int ks_mlp_grad(ks_mlp* m, const float* X, const float* T, int32_t rows, float* grads, float* loss);
/* Adam training on the circuits idx_dev[0..n_train) of a batch, with solutions
 * x_dev [n_circ][n] (device memory), `epochs` passes of minibatches of `mb`
 * rows (a multiple of 64). */
int ks_mlp_train(ks_mlp* m, ks_batch* b, const double* x_dev, const int32_t* idx_dev, int32_t n_train,
                 int32_t epochs, int32_t mb, float lr, float* last_loss, void* stream);
/*
 * Torn solves of large circuits, batched over variants of one topology
 * (kron.JacobianTearing as analysis.Options.Solver, kron/jacobian.go:92-589,
 * under analysis.OP and analysis.Tran).  ks_torn_create takes the topology,
 * n_variants value vectors ([n_variants][n_values], row-major) and the indices
 * of the torn elements (kron.Tearing.Torn; refused as NewJacobianTearing
 * refuses: a voltage source or inductor, an element to ground, one torn twice,
 * KS_EINVAL with the reference's message).  The pieces are the connected
 * components of the Jacobian's pattern without the torn node pairs
 * (buildPlan, :296-389); each is factored as a band matrix, the
 * interconnection I + M.Q.B^-1.P of each variant as a dense matrix.
 * reuse = KS_TORN_REUSE keeps factors while the refinement against the exact
 * Jacobian (backward error <= 1e-14, accepted at 1e-12) converges on them
 * (ReuseTol without a bound); KS_TORN_REFACTOR refactors at every solve;
 * KS_TORN_UNTORN solves every system untorn (one band LU per connected
 * component of the whole Jacobian: the analysis without Options.Solver, for
 * torn-versus-untorn comparisons).  A variant whose torn solve is not accepted
 * after a fresh refactor is solved untorn, as the reference falls back to a
 * plain LU of the whole system (kron/jacobian.go:412-434); a system whose
 * connected component is too large for one band piece (12,000 unknowns) has
 * no untorn solver and such a variant ends with KS_STATUS_SINGULAR.  Errors
 * per variant as ks_status.  stats [15]: solves, refactors, refinement steps,
 * most refinement steps of one solve, torn solves not accepted, pieces,
 * coupling rows, largest band (kl + ku), band-factor doubles per variant,
 * kernel launches of the call, the device time (microseconds, CUDA events) of
 * the refactors, the applications of the factors, the loads and the
 * residuals, then the variant solves that went untorn.
 */
enum { KS_TORN_REFACTOR = 0, KS_TORN_REUSE = 1, KS_TORN_UNTORN = 2 };
typedef struct ks_torn ks_torn;
int ks_torn_create(const ks_topology* topo, int32_t n_variants, const double* values, const int32_t* torn_elems,
                   int32_t n_torn, ks_torn** out);
void ks_torn_destroy(ks_torn* t);
/* The tearing alone, on the host (no GPU): piece_of [n] (pieces numbered in
 * order of their first unknown, as buildPlan numbers them), the coupling rows
 * (up to rows_cap), the largest piece and band (kl + ku).  Any output may be
 * NULL. */
int ks_torn_plan(const ks_topology* topo, const int32_t* torn_elems, int32_t n_torn, int32_t* piece_of,
                 int32_t* n_pieces, int32_t* rows, int32_t rows_cap, int32_t* n_rows, int32_t* max_piece,
                 int32_t* max_band);
/* Stream of the later calls (NULL: the one ks_torn_create made).  The calls
 * still return only when their results are on the host. */
int ks_torn_set_stream(ks_torn* t, void* stream);
int ks_torn_info(const ks_torn* t, int32_t* n_unknowns, int32_t* n_pieces, int32_t* n_coupling_rows,
                 int32_t* max_piece, int32_t* max_band);
/* analysis.OP of every variant (Newton from zero, InitJct; no gmin / source
 * stepping fallback).  out_x [n_variants][n]. */
int ks_torn_op(ks_torn* t, const ks_options* opt, int32_t reuse, double* out_x, int32_t* out_status,
               int32_t* out_iters, int64_t* stats);
/* Fixed-step analysis.Tran of every variant from its transient operating
 * point: n_points = round(stop / step) + 1, backward Euler at the first step,
 * then spec->method.  out_wave [n_points][n_variants][n_probes] holds the
 * unknowns listed in probes; out_x [n_variants][n] the last point. */
int ks_torn_tran(ks_torn* t, const ks_tran_spec* spec, const ks_options* opt, int32_t reuse, const int32_t* probes,
                 int32_t n_probes, double* out_wave, double* out_x, int32_t* out_status, int32_t* out_steps,
                 int32_t* out_iters, int64_t* stats);

/* The autotuner's choice for operating points of `n_circ` circuits on this plan
 * (the power-of-two bucket of n_circ): *kernel a KS_KERNEL_* value, *cpt the
 * circuits per thread of the persistent grid, *ms the winning trial's kernel
 * time.  KS_EINVAL when no ks_options.autotune call has tuned that bucket. */
int ks_plan_tuned(const ks_plan* plan, int32_t analysis, int64_t n_circ, int32_t* kernel, int32_t* cpt, double* ms);

/* Predicted starting points x0_dev [n_circ][n] (device memory) for ks_op_async. */
int ks_mlp_predict(ks_mlp* m, ks_batch* b, double* x0_dev, void* stream);

/* ---- measurement ----------------------------------------------------------
 * No counterpart in the reference.  FP64 throughput of the current device: FMA
 * chains on every SM (16 warps, eight independent chains per lane), the fastest
 * of three timed runs.  *flops_per_s counts an FMA as two operations;
 * *fma_per_clk_per_sm (optional) is FMA lanes per SM clock at the device's
 * rated clock.  The denominator of FP64 roofline fractions. */
int ks_fp64_peak(double* flops_per_s, double* fma_per_clk_per_sm);
#endif /* __CUDACC_RTC__ */

#ifdef __cplusplus
}
#endif
#endif /* KRONSPICE_GPU_H */
