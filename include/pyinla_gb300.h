/*
 * pyinla_gb300 -- C ABI of the GB300-native block-tridiagonal-arrowhead (BTA) solver.
 *
 * The entry points replace the arithmetic that the reference reaches through the
 * third-party Serinv package (`serinv.algs`), called from
 * src/pyinla/solvers/structured_solver.py of lisa-gm/pyINLA:
 *
 *   reference call (structured_solver.py)               entry point here
 *   pobtaf(D, L, R, T)               :83-88             gbta_pobtaf
 *   pobtf(D, L)                      :90-93             gbta_pobtf
 *   pobtas(D, L, R, T, rhs, trans)   :112-127           gbta_pobtas
 *   pobts(D, L, rhs, trans)          :129-140           gbta_pobts
 *   logdet(sparsity)                 :151-166           gbta_logdet
 *   pobtasi(D, L, R, T)              :176-181           gbta_pobtasi
 *   pobtsi(D, L)                     :183-186           gbta_pobtsi
 *
 * Storage is the reference's (structured_solver.py:37-61): FP64, C-contiguous,
 *   D (nt, b, b)      diagonal blocks
 *   L (nt-1, b, b)    L[i] = block (i+1, i)
 *   R (nt, a, b)      arrow bottom blocks (row block nt, column block i)
 *   T (a, a)          arrow tip
 * All matrix pointers are DEVICE pointers; every routine works in place like Serinv.
 * After a factorization the diagonal blocks hold the lower Cholesky factor with an
 * exactly-zero strict upper triangle; after a selected inversion the buffers hold
 * Sigma = Q^{-1} on the BTA pattern, with D and T full symmetric.
 *
 * Right-hand sides: B is (N, nrhs) row-major with N = nt*b + a (N = nt*b for the
 * "bt" variants); the reference passes nrhs = 1.  trans = 0 solves L y = b
 * (Serinv trans="N"), trans = 1 solves L^T x = y (trans="C").
 *
 * Return codes (int): 0 success; > 0 LAPACK-style info: the 1-based global row whose
 * pivot was not positive (non-SPD input, or NaN); < 0 an error (see gbta_last_error).
 * Routines without the _async suffix synchronise the solver's stream before they
 * return their status; the _async forms only enqueue, and gbta_status() later
 * synchronises and returns (and clears) the first status recorded since the last call.
 */
#ifndef PYINLA_GB300_H
#define PYINLA_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBTA_OK 0
#define GBTA_ERR_ARG (-1)
#define GBTA_ERR_CUDA (-2)
#define GBTA_ERR_TIMEOUT (-3)
#define GBTA_ERR_ALLOC (-5)

typedef struct gbta_solver gbta_solver;

/* Version of this ABI (major*10000 + minor*100 + patch). */
int gbta_version(void);

/* Text of the last error raised on the calling thread ("" if none). */
const char* gbta_last_error(void);

/* Geometry of a solver (any output may be NULL); *stream receives the cudaStream_t
 * the solver enqueues on. */
int gbta_geometry(const gbta_solver* s, int* b, int* nt, int* a, void** stream);

/* Record `msg` as the calling thread's last error and return `code`. */
int gbta_set_error(int code, const char* msg);

/* Create a solver for nt diagonal blocks of size b and an arrowhead of size a
 * (a may be 0).  Replaces SerinvSolver.__init__ (structured_solver.py:22-70) minus
 * the block buffers, which the caller owns.  Allocates the solver's device
 * workspace (tile flags, task lists) and a private CUDA stream. */
int gbta_create(int b, int nt, int a, gbta_solver** out);
int gbta_destroy(gbta_solver* s);

/* Make the solver enqueue its work on `stream` (a cudaStream_t; NULL restores the
 * private stream). */
int gbta_set_stream(gbta_solver* s, void* stream);

/* Limit, in milliseconds, on any inter-CTA wait inside a kernel; after it the
 * kernel records GBTA_ERR_TIMEOUT and returns instead of waiting further. */
int gbta_set_wait_limit_ms(gbta_solver* s, double ms);

/* Bytes of device workspace held by the solver (SerinvSolver.get_solver_memory,
 * structured_solver.py:540-550, minus the caller-owned block buffers). */
size_t gbta_workspace_bytes(const gbta_solver* s);

/* Synchronise the stream and return (then clear) the first recorded status. */
int gbta_status(gbta_solver* s);

/* ---- factorization: Serinv pobtaf / pobtf -------------------------------- */
int gbta_pobtaf(gbta_solver* s, double* D, double* L, double* R, double* T);
int gbta_pobtf(gbta_solver* s, double* D, double* L);
int gbta_pobtaf_async(gbta_solver* s, double* D, double* L, double* R, double* T);
int gbta_pobtf_async(gbta_solver* s, double* D, double* L);

/* ---- triangular sweeps: Serinv pobtas / pobts ---------------------------- */
int gbta_pobtas(gbta_solver* s, const double* D, const double* L, const double* R,
                const double* T, double* B, int nrhs, int trans);
int gbta_pobts(gbta_solver* s, const double* D, const double* L, double* B, int nrhs,
               int trans);
int gbta_pobtas_async(gbta_solver* s, const double* D, const double* L, const double* R,
                      const double* T, double* B, int nrhs, int trans);

/* ---- logdet from the factor (structured_solver.py:151-166) ---------------- */
/* with_tip = 1 for "bta", 0 for "bt" (tip excluded).  *out is a HOST double.
 * Returns GBTA_ERR_ARG with message "Logdet is NaN" when the sum is NaN. */
int gbta_logdet(gbta_solver* s, const double* D, const double* T, int with_tip, double* out);

/* ---- selected inversion: Serinv pobtasi / pobtsi ------------------------- */
int gbta_pobtasi(gbta_solver* s, double* D, double* L, double* R, double* T);
int gbta_pobtsi(gbta_solver* s, double* D, double* L);
int gbta_pobtasi_async(gbta_solver* s, double* D, double* L, double* R, double* T);

/* ---- sparse <-> BTA mapping --------------------------------------------- */
/* Zero-fill D, L (and R, T when with_arrow) and scatter the COO entries (int64 rows,
 * cols; device pointers) of a symmetric N x N matrix into them: entries of the
 * diagonal blocks (both triangles), of the lower off-diagonal blocks, of the arrow
 * bottom and of the tip are kept, the upper blocks are implied by symmetry.
 * Replaces SerinvSolver._spmatrix_to_structured (structured_solver.py:192-250) and
 * its CuPy mapping (:252-468).  Asynchronous on the solver's stream. */
int gbta_scatter_coo(gbta_solver* s, const long long* rows, const long long* cols, const double* vals,
                     long long nnz, double* D, double* L, double* R, double* T, int with_arrow);

/* Gather the BTA-stored values at (rows[k], cols[k]) (lower pattern) into vals[k]
 * (device pointers).  Replaces the block gather of SerinvSolver._structured_to_spmatrix
 * (structured_solver.py:470-538).  Asynchronous on the solver's stream. */
int gbta_gather_coo(gbta_solver* s, const long long* rows, const long long* cols, long long nnz,
                    const double* D, const double* L, const double* R, const double* T, int with_arrow,
                    double* vals);

#ifdef __cplusplus
}
#endif

#endif /* PYINLA_GB300_H */
