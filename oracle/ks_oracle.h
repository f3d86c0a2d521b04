/*
 * ks_oracle.h — CPU FP64 oracle of the batched circuit-solve engine.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a line-by-line C++ restatement of the
 * reference's (fdamador/kronspice, pure Go) hot path for the element kinds of
 * include/kronspice_gpu.h: device Setup/Load/Accept/ConvTest/Truncate, the
 * dense and sparse LU backends, Newton with the SPICE3 convergence test, the
 * DC fallback chain and the transient loop.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load it; the engine never does.
 *
 * Parity pin: tests/test_oracle_golden.py checks it against the reference's
 * golden vectors (the testdata/golden CSV files, committed as fixtures under
 * tests/golden/) with the reference's tolerances (internal/golden/golden.go:22-27).
 */
#ifndef KS_ORACLE_H
#define KS_ORACLE_H
#include "../include/kronspice_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* One operating point (analysis.OP).  x0 (nullable) gives NodeSet voltages for
 * unknowns 0..n_nodes-2.  Returns a ks_status; err gets the Go error text. */
int kso_op(const ks_topology* t, const double* values, const ks_options* o, const double* x0,
           double* x_out, double* i_out, int32_t* iters, char* err, int errlen);

/* DC sweep of source element `src` over vals[npts] (analysis.DC, one sweep).
 * x_out [npts][n], i_out [npts][n_elem] (nullable).  Returns a ks_status. */
/* AC small-signal sweep (analysis/ac.go): x_out [nf][n] complex, interleaved re/im. */
int kso_ac(const ks_topology* t, const double* values, const ks_options* o, const double* freqs, int nf,
           double* x_out, char* err, int errlen);
int kso_reach_pattern(int n, const uint8_t* A, const int32_t* q, const int32_t* prow, uint8_t* out);
int kso_dc2(const ks_topology* t, const double* values, const ks_options* o, int src, const double* vals,
            int npts, int src2, const double* vals2, int npts2, double* x_out, double* i_out, char* err, int errlen);
int kso_dc(const ks_topology* t, const double* values, const ks_options* o, int src,
           const double* vals, int npts, double* x_out, double* i_out, char* err, int errlen);

/* Transient (analysis.Tran, or the fixed-step mode of ks_tran_spec).  Up to
 * `capacity` recorded points: t_out[cap], x_out[cap][n], i_out[cap][n_elem]
 * (nullable).  npts gets the number recorded. */
int kso_tran(const ks_topology* t, const double* values, const ks_tran_spec* spec,
             const ks_options* o, int capacity, double* t_out, double* x_out, double* i_out,
             int32_t* npts, int32_t* steps, int32_t* iters, char* err, int errlen);

/* analysis.OP with its result (analysis/op.go:340-403): elem_out [n_elem][KS_RES_COLS],
 * ledger_out [KS_LEDGER_COLS] (nullable), and em.CheckLedger: KS_STATUS_LEDGER when
 * the relative residual exceeds o->ledger_tol (1e-9) unless o->skip_energy_check. */
int kso_op_results(const ks_topology* t, const double* values, const ks_options* o, const double* x0,
                   double* x_out, double* elem_out, double* ledger_out, int32_t* iters, char* err, int errlen);

/* analysis.Tran with the Waveform's element series and ledger (analysis/tran.go:248-386):
 * elem_out [cap][n_elem][2] current and absorbed power, ledger_out [cap][KS_TPOINT_COLS],
 * summary_out [KS_TSUM_COLS] (all nullable).  KS_STATUS_LEDGER as recorder.record
 * and recorder.finish decide it. */
int kso_tran_results(const ks_topology* t, const double* values, const ks_tran_spec* spec,
                     const ks_options* o, int capacity, double* t_out, double* x_out, double* elem_out,
                     double* ledger_out, double* summary_out, int32_t* npts, int32_t* steps, int32_t* iters,
                     char* err, int errlen);

/* Batches over host threads (the timed CPU baseline).  values [nc][n_values];
 * x0 nullable [nc][n]; x_out [nc][n]. */
int kso_batch_op(const ks_topology* t, const double* values, int nc, const ks_options* o,
                 const double* x0, int nthreads, double* x_out, int32_t* status, int32_t* iters);
/* Fixed-step transients of a batch: x_out [npts][nc][n] (nullable). */
int kso_batch_tran(const ks_topology* t, const double* values, int nc, const ks_tran_spec* spec,
                   const ks_options* o, int nthreads, double* x_out, int32_t* status,
                   int32_t* steps, int32_t* iters);

/* kron.JacobianTearing (kron/jacobian.go) as the linear solver.  kso_torn_cuts
 * turns torn element indices into node-unknown pairs (tearTerminals, with the
 * reference's refusals as KS_EINVAL + message); kso_op_torn / kso_tran_torn run
 * the analyses with every linear system solved torn (reuse_tol: ReuseTol).
 * stats [7]: solves, pieces factored, reused, stale reuses, untorn fallbacks,
 * refinement steps, most pieces. */
int kso_torn_cuts(const ks_topology* t, const int32_t* elems, int n_elems, int32_t* pairs, int cap,
                  int32_t* n_pairs, char* err, int errlen);
int kso_op_torn(const ks_topology* t, const double* values, const ks_options* o, const int32_t* pairs,
                int n_pairs, double reuse_tol, double* x_out, int32_t* iters, int64_t* stats, char* err, int errlen);
int kso_tran_torn(const ks_topology* t, const double* values, const ks_tran_spec* spec, const ks_options* o,
                  const int32_t* pairs, int n_pairs, double reuse_tol, int capacity, double* t_out, double* x_out,
                  int32_t* npts, int32_t* steps, int32_t* iters, int64_t* stats, char* err, int errlen);

/* buildPlan's pieces and coupling rows for the Jacobian of one backward-Euler
 * step of length h: piece_of [n], rows [cap]. */
int kso_torn_plan(const ks_topology* t, const double* values, const int32_t* pairs, int n_pairs, double h,
                  int32_t* piece_of, int32_t* n_pieces, int32_t* rows, int cap, int32_t* n_rows);

/* The sparse backend's column order after an operating point (spec NULL) or a
 * transient, with the pattern it ordered (every entry the run's loads stamped,
 * n x n bytes); returns the analysis's status.  kso_min_degree: minimumDegree
 * (solver/sparse.go:412-452) of a given pattern. */
int kso_sparse_order(const ks_topology* t, const double* values, const ks_tran_spec* spec, const ks_options* o,
                     int32_t* n, int32_t* order, uint8_t* pattern,
                     int32_t* pivots);
void kso_min_degree(int n, const uint8_t* pattern, int32_t* order);

/* Unknown count and layout of one circuit (device Setup), for the tests. */
int kso_unknowns(const ks_topology* t, const double* values, int32_t* n, int32_t* is_v);

#ifdef __cplusplus
}
#endif
#endif
