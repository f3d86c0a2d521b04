// ks_engine.h — internal layout shared by the host planner and the GB300 kernels.
//
// A plan is one topology after the symbolic work the host does once: the MNA
// unknown layout of device Setup (device/device.go:36-100, per-kind Setup in
// device/passive.go:65, reactive.go:184,355, source.go:93,148, diode.go:131,
// bjt.go:250, mosfet.go:326) compiled into one KElem record per element.
//
// Per-circuit data lives on the device in structure-of-arrays form, one column
// per circuit, so that the threads of a warp (one circuit each, all running the
// same element program) touch consecutive addresses:
//   values  [n_values][B]  element values and model parameters
//   derived [n_derived][B] per-circuit constants (setup kernel)
//   state   [n_state][B]   device linearization and accepted state
#pragma once
#ifdef __CUDACC_RTC__
typedef signed char int8_t;
typedef int int32_t;
typedef long long int64_t;
typedef unsigned int uint32_t;
typedef unsigned long long uint64_t;
#else
#include <stddef.h>
#include <stdint.h>
#endif

#define KS_MAX_DENSE 32  // largest system of the thread-per-circuit kernels

struct KElem {
  int32_t kind, flags, level, wave;
  int32_t nargs, param, derived, state;
  int32_t u[10];   // unknown indices (-1 = ground), per kind below
  uint64_t given;
};

// u[] per kind:
//   R, C, I : u[0] = n+, u[1] = n-
//   L, V    : u[0] = n+, u[1] = n-, u[2] = branch
//   D       : u[0] = anode, u[1] = cathode, u[2] = internal anode ai (= u[0] without RS)
//   Q       : u[0] = c, u[1] = e, u[2] = b, u[3] = s, u[4] = cp, u[5] = bp, u[6] = ep, u[7] = sa, u[8] = sb
//   M       : u[0] = d, u[1] = s, u[2] = g, u[3] = b, u[4] = dp, u[5] = sp
//   E       : u[0] = n+, u[1] = n-, u[2] = branch, u[3] = nc+, u[4] = nc-
//   G       : u[0] = n+, u[1] = n-, u[3] = nc+, u[4] = nc-
//   F       : u[0] = n+, u[1] = n-, u[3] = the controlling source's branch
//   H       : u[0] = n+, u[1] = n-, u[2] = branch, u[3] = the controlling source's branch
//   K       : u[0], u[1] = the coupled inductors' branches, u[2], u[3] = their value blocks
//   CN      : u[0] = n+, u[1] = n-
//   LN      : u[0] = n+, u[1] = n-, u[2] = branch
//   S       : u[0] = n+, u[1] = n-, u[3] = nc+, u[4] = nc-
//   W       : u[0] = n+, u[1] = n-, u[3] = the controlling source's branch

// Derived constants per kind (offsets within the element's derived block).
enum { DR_G = 0, DR_N = 1 };
enum { DS_A0 = 0, DS_N = 7 };  // resolved waveform arguments a[0..6]
// The R* entries are reciprocals of per-circuit constants, so that the Newton
// loop multiplies where the model equations divide by a parameter.
enum { DD_VTE = 0, DD_VCRIT, DD_XBV, DD_GRS, DD_RVTE, DD_N };
enum { DQ_VT = 0, DQ_VCRIT, DQ_RBPR, DQ_RBPI, DQ_GCPR, DQ_GEPR, DQ_OVTF, DQ_F1E, DQ_F2E, DQ_F3E,
       DQ_F1C, DQ_F2C, DQ_F3C,
       DQ_RVT, DQ_RNF, DQ_RNE, DQ_RNR, DQ_RNC, DQ_RNS,  // 1/vt, 1/(N* vt)
       DQ_IVAF, DQ_IVAR, DQ_OIK, DQ_OIKR,             // 1/VAF, 1/VAR, 1/IKF, 1/IKR (0 when not given)
       DQ_RBF, DQ_RBR, DQ_N };
enum { DM_VT = 0, DM_LEFF, DM_WEFF, DM_BETA, DM_COX, DM_OXCAP, DM_VBI, DM_VTO, DM_GDPR, DM_GSPR,
       DM_ISD, DM_ISS, DM_VCRITD, DM_VCRITS, DM_CZBD, DM_CZBDSW, DM_CZBS, DM_CZBSSW,
       DM_FBT0, DM_FBT1, DM_FBT2, DM_FSW0, DM_FSW1, DM_FSW2, DM_CGSO, DM_CGDO, DM_CGBO,
       DM_HASJCAP, DM_HASGCAP, DM_XD, DM_ALPHA, DM_CFS, DM_FACTOR, DM_NARROW, DM_ETA3, DM_SQRTPB,
       DM_HASNSUB, DM_KP, DM_PHI, DM_GAMMA, DM_VTOP, DM_CJ, DM_BAD, DM_RVT, DM_N };

// History of accepted charges for LTE (device/lte.go:23-37): t[3], q[3], n.
enum { H_T0 = 0, H_T1, H_T2, H_Q0, H_Q1, H_Q2, H_N, H_SIZE };

// State per kind.
enum { SC_GEQ = 0, SC_IHIST, SC_VPREV, SC_IPREV, SC_TRAN, SC_HIST, SC_N = SC_HIST + H_SIZE };
enum { SL_VPREV = 0, SL_IPREV, SL_HIST, SL_N = SL_HIST + H_SIZE };
enum { SV_VALUE = 0, SV_OVR, SV_OVRON, SV_N };
enum { SK_I1PREV = 0, SK_I2PREV, SK_N };  // mutual inductance: the accepted branch currents
enum { DK_M = 0, DK_N = 1 };              // mutual inductance M = k sqrt(L1 L2)
// switch: |VH|, smooth (VH < 0), ln sqrt(RON ROFF), ln(RON/ROFF), initial state ON
enum { DW_VH = 0, DW_SMOOTH, DW_LMEAN, DW_LRATIO, DW_INIT, DW_N };
// switch: stamped state, accepted state, a solution accepted, state held by the
// last load (transient step), the last Accept changed the state, and the
// linearization i = g v + k (c - c0) of the last load; the accepted control
enum { SW_ON = 0, SW_ACC, SW_ACCEPTED, SW_FROZEN, SW_FLIP, SW_G, SW_K, SW_C0, SW_CACC, SW_N };
// nonlinear / time-varying C and L (the state law y = s(t) f(x)): the resolved
// SCALE arguments a[0..6], the integral of f from the first knot to 0, the
// Newton step limit, then the integral of f from the first knot to each knot
enum { DN_A0 = 0, DN_G0 = 7, DN_MAXSTEP = 8, DN_PRE = 9 };
// the last load's linearization (x0 and the law's value and slope there: the
// capacitor's iq and geq, the inductor's lam0 and ld), the companion's a and b,
// s and ds/dt at the load's time, that time, a companion stamped, the load
// limited its update, the limited iterate; the accepted voltage, current and
// charge (flux), the accepted x and s, a knot crossing's landing time, history
enum { SN_X0 = 0, SN_Y0, SN_G, SN_A, SN_B, SN_SN, SN_SDOT, SN_T, SN_TRAN, SN_LIM, SN_XITER,
       SN_VPREV, SN_IPREV, SN_QPREV, SN_XACC, SN_SACC, SN_KNOTT, SN_HIST, SN_N = SN_HIST + H_SIZE };
enum { SD_VD = 0, SD_CD, SD_GD, SD_IQ, SD_GEQ, SD_QPREV, SD_IQPREV, SD_VDACC, SD_LIM, SD_TRAN,
       SD_HIST, SD_N = SD_HIST + H_SIZE };
enum { SQ_VBE = 0, SQ_VBC, SQ_VBX, SQ_VCS,
       SQ_CBE, SQ_GBE, SQ_CBC, SQ_GBC, SQ_IT, SQ_ITBE, SQ_ITBC, SQ_IBE, SQ_GPI, SQ_IBC, SQ_GMU,
       SQ_QB, SQ_DQBDVE, SQ_DQBDVC, SQ_GX, SQ_ISUB, SQ_GSUB, SQ_AG, SQ_IQ0, SQ_IQ1, SQ_IQ2, SQ_IQ3,
       SQ_C0, SQ_C1, SQ_C2, SQ_C3, SQ_DQBEDVBC, SQ_LIM, SQ_TRAN, SQ_VBEACC, SQ_VBCACC,
       SQ_QPREV0, SQ_IQPREV0 = SQ_QPREV0 + 4, SQ_HIST = SQ_IQPREV0 + 4, SQ_N = SQ_HIST + 4 * H_SIZE };
enum { SM_VGS = 0, SM_VDS, SM_VBS, SM_VBD, SM_VGD, SM_VGB, SM_MODE, SM_CDRAIN, SM_GM, SM_GDS, SM_GMBS,
       SM_VON, SM_VDSAT, SM_CBS, SM_GBS, SM_CBD, SM_GBD, SM_LIM, SM_TRAN, SM_AG,
       SM_CAPG0, SM_CAPB0 = SM_CAPG0 + 3, SM_IQ0 = SM_CAPB0 + 2, SM_DV0 = SM_IQ0 + 5,
       SM_AVGS = SM_DV0 + 5, SM_AVDS, SM_AVBS, SM_AVON, SM_MEYER0,
       SM_QPREV0 = SM_MEYER0 + 3, SM_IQPREV0 = SM_QPREV0 + 5, SM_VPREV0 = SM_IQPREV0 + 5,
       SM_HIST = SM_VPREV0 + 5, SM_N = SM_HIST + 5 * H_SIZE };

// Options after defaults (analysis/op.go:91-110), as the kernels read them.
struct KOpts {
  double reltol, abstol, vntol, gmin;
  int32_t itl1, itl4;
  int32_t no_gmin, no_source, no_pt;
  int32_t mixed;           // FP32 LU + FP64 residual
  int32_t max_iter_total;  // bound on all solves of one circuit (0 = default)
  int32_t passes;          // mixed: most refinement passes per solve
  double refine_tol;       // mixed: refinement stops when the correction is below this fraction of x
  int32_t polish;          // OP: the polish of analysis/op.go:251-271 (AC operating points)
  int32_t start32;         // OP: most iterations of the FP32 start stage (0: no FP32 stage)
  double start_check;      // OP with a given start: a circuit whose solution ends farther than this (volts, any
                           // node) from its start is solved again from the standard start (0: no check)
  const int32_t* cancel;   // the batch's cancel word (page-locked host memory mapped for the device), or null
  int32_t predict;         // transients: start each step's Newton from the extrapolated accepted history
  // element results and the energy ledger (read by the generic kernels' results instantiation only)
  double* res_elem;        // op: [B][ne][KS_RES_COLS]; transient: per recorded point [..][ne][2]
  double* res_ledger;      // op: [B][KS_LEDGER_COLS]; transient: per recorded point [..][KS_TPOINT_COLS]
  double* res_summary;     // transient: [B][KS_TSUM_COLS]
  double* res_scratch;     // [n_state][B]: the device-state copy the round-off load runs on
  double ledger_tol;       // relative residual limit (em.DefaultTolerance 1e-9)
  int32_t energy_check;    // 0: Options.SkipEnergyCheck
  int32_t cpt;             // circuits per thread the persistent grid is sized for (0: KS_CIRCUITS_PER_THREAD)
};

#ifndef __CUDACC_RTC__
// Bytes of dynamic shared memory of T per-thread dense systems of n unknowns,
// behind an element table of ne entries and its is-voltage flags (ne = 0: no
// table, the per-topology kernels).
inline size_t ks_sys_smem(int n, int ne, int T) {
  size_t off = ne ? (size_t)ne * sizeof(KElem) + ((n + 15) / 16) * 16 : 0;
  size_t per = (size_t)(n * n + 4 * n) * 8 + (size_t)n * 4 + 8 + (size_t)n * n * 4 + 8;
  return off + per * T;
}
#endif

struct KPlan {  // device-side view of a plan
  int32_t n, n_elem, n_values, n_derived, n_state, n_nodes;
  int32_t n_nonlin, n_reactive;
  const KElem* elem;  // device pointer
  const int8_t* is_v; // device pointer [n]
};
