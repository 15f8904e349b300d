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
 * (Serinv trans="N"), trans = 1 solves L^T x = y (trans="C"), and trans = 2 does both,
 * N then C, in one launch (the reference's solve, structured_solver.py:102-149: the
 * backward sweep's tasks follow the forward sweep's as soon as their tiles are solved).
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

/* How the factorization computes its tile products (gbta_set_method).
 * GBTA_METHOD_FP64: FP64 FMAs on the CUDA cores.
 * GBTA_METHOD_OZAKI (default): error-free splitting of each FP64 tile into eight
 * balanced base-128 integer digit planes (per-row exponents from the matrix diagonal)
 * multiplied on the tensor cores (43 plane pairs) with exact fp32 accumulation and
 * folded into FP64; the product error is bounded like an FP64 product's (a few units
 * of 2^-53 of the operands' magnitudes).  The selected inversion uses the same scheme
 * for its products (factor tiles sliced once per inversion with per-column exponents,
 * every Sigma tile sliced once by the task that produces it).  Tile Cholesky factors,
 * tile inverses / triangular solves and the sweeps stay FP64. */
#define GBTA_METHOD_FP64 0
#define GBTA_METHOD_OZAKI 1

typedef struct gbta_solver gbta_solver;

/* Version of this ABI (major*10000 + minor*100 + patch). */
int gbta_version(void);

/* Number of kernels this library has launched in the process so far. */
long long gbta_kernel_launches(void);

/* Measure the chip's FP64 FMA throughput (TFLOP/s) with a DFMA-bound kernel on every
 * SM (`iters` FMA rounds per thread); the roofline denominator of the FP64 kernels. */
int gbta_probe_fp64_peak(int iters, double* tflops);

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

/* Make the solver enqueue its work on `stream` (a cudaStream_t, used as given: NULL
 * is the CUDA default stream).  A new solver uses a private non-blocking stream. */
int gbta_set_stream(gbta_solver* s, void* stream);

/* Limit, in milliseconds, on any inter-CTA wait inside a kernel; after it the
 * kernel records GBTA_ERR_TIMEOUT and returns instead of waiting further.  The default
 * is 20 s, or GBTA_WAIT_LIMIT_MS from the environment when the solver is created. */
int gbta_set_wait_limit_ms(gbta_solver* s, double ms);

/* Select / query the product method of the factorization (see GBTA_METHOD_*). */
int gbta_set_method(gbta_solver* s, int method);
int gbta_get_method(const gbta_solver* s);

/* Elimination order of the block recurrences (no reference counterpart: the factor
 * blocks between gbta_pobtaf and the sweeps / inversion are internal state).  With
 * twist = 1 (the default for nt >= 3) the blocks are eliminated from both ends towards
 * the middle block m = nt/2 -- blocks 0..m-1 top-down and nt-1..m+1 bottom-up, side
 * by side, then m -- which halves the longest chain of dependent work at the same
 * flop count; twist = 0 is the top-down order of Serinv's recurrence.  The logdet,
 * the solutions and the selected inverse are the same either way (to rounding); the
 * factor itself differs: after a twisted factorization D_i holds the Cholesky factor
 * of the partially eliminated block i, and for j >= m the L buffer's block j holds the
 * factor's coupling of block j to block j+1 in the orientation Q(j, j+1) (the
 * transpose of the reference's L_j).  A factor is valid input only to sweeps and
 * inversions under the same setting; gbta_pobtasi restores the reference's layout of
 * Sigma in every buffer. */
int gbta_set_twist(gbta_solver* s, int twist);
int gbta_get_twist(const gbta_solver* s);

/* Overlapped selected inversion (off by default; no reference counterpart: the reference
 * runs its calls one after the other).  With it on, a tensor-core gbta_pobtasi that follows
 * this solver's gbta_pobtaf runs its whole pre-pass and inversion on a second stream from
 * the factorization's completion, concurrently with the work enqueued on the solver's
 * stream in between (the sweeps of gbta_pobtas), and writes Sigma into a workspace of the
 * size of the blocks; the write-back into the caller's blocks is enqueued on the solver's
 * stream, after that work and the inversion.  The blocks must hold the factor that
 * gbta_pobtaf left until then (the sweeps only read them).  The sweeps keep one CTA per
 * SM and the inversion's CTAs fill the rest of each SM.  An inversion called when no
 * sweep enqueued since the factorization is still in flight runs in place on the
 * solver's stream as without the option (there is nothing to overlap).  Status words
 * of both streams are read by gbta_status. */
int gbta_set_selinv_overlap(gbta_solver* s, int enable);

/* Persistent CTAs per SM of the dataflow launches (0, the default: as many as the
 * kernel's registers and shared memory allow for the factorization and the selected
 * inversion, one for the sweeps, whose latency-bound chain runs fastest so;
 * GBTA_CTAS_PER_SM in the environment sets the initial value).  No reference
 * counterpart (a launch-shape setting). */
int gbta_set_ctas_per_sm(gbta_solver* s, int n);

/* Task tracing (off by default).  When enabled, every dataflow kernel launched by
 * the solver records one entry of 8 int64 per task: [ticket, (CTA index << 32) |
 * (task type << 16) | SM id, start ns, end ns, m0, m1, m2, m3] (GPU global timer;
 * m0..m3 are intermediate
 * marks of the task's phases, 0 where a kernel sets none).  gbta_get_trace copies the
 * records (out: 8 * max_records int64) of the last traced launch to host memory and
 * returns how many were copied. */
int gbta_set_trace(gbta_solver* s, int enable);
long long gbta_get_trace(gbta_solver* s, long long* out, long long max_records);
/* The task list of the factorization (which = 0) or of the selected inversion of the
 * solver's current product method (which = 1), as the dataflow kernel takes it: one
 * (type, block, row, column) int quadruple per ticket (out: 4 * max_tasks ints; the
 * type word carries the split flags of the factorization's tasks).  Returns the number
 * copied.  A measurement aid for reading traces (no reference counterpart). */
long long gbta_get_task_list(gbta_solver* s, int which, int* out, long long max_tasks);

/* Kernel timing (off by default; a measurement aid with no reference counterpart).
 * When enabled, the solver records CUDA events on its stream around the dataflow
 * kernel of each factorization (k_factor / k_factor_oz, without the exponent and flag
 * preparation), each selected inversion (k_selinv / k_selinv_oz, without the pre-pass
 * and the write-back) and each solve call (all its sweep launches).  gbta_kernel_ms
 * waits for the last recorded events and writes ms[0] factorization, ms[1] selected
 * inversion, ms[2] solve call, in milliseconds (-1 where none was recorded since
 * timing was enabled). */
int gbta_set_kernel_timing(gbta_solver* s, int enable);
int gbta_kernel_ms(gbta_solver* s, double* ms);
/* With kernel timing on: the tile-pair products (one 32 x 32 x 32 fp16 MMA of two digit
 * planes each, 2 * 32^3 flops) that the tensor-core product loops of the last timed
 * factorization (pairs[0]) and selected inversion (pairs[1]) issued, after the
 * products of zero tiles and zero digit planes were left out; -1 where none was
 * recorded (or the FP64 method ran: 0).  Synchronizes the solver's stream. */
int gbta_kernel_pairs(gbta_solver* s, long long* pairs);

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

/* ---- factorization without device allocation ----------------------------- */
/* No counterpart in the reference.  For callers that cannot allocate device memory
 * when they factor -- hosts that own a fixed device-memory pool and forbid
 * allocations outside it, or loops that cannot afford the implicit device
 * synchronisation of cudaMalloc/cudaFree -- gbta_pobtaf_noalloc factors D, L, R, T in
 * place without a solver object and without calling cudaMalloc, cudaFree or any
 * allocating routine.  It runs the FP64-product factorization kernel (the kernel of
 * gbta_pobtaf under GBTA_METHOD_FP64, with a task list that leaves out the feeder
 * row-group split), so its results agree with gbta_pobtaf to rounding (both product
 * methods), and its return codes are gbta_pobtaf's.  It is synchronous: it returns
 * after the work enqueued on `stream` (NULL = the CUDA default stream) has finished
 * and its status has been read back.
 *
 * Its scratch (control words, ready flags, the task list, the arrow-tip partials)
 * lives in one fixed array of GBTA_NOALLOC_SCRATCH_BYTES (64 MiB) of device memory
 * inside the library.  Problems whose scratch (gbta_noalloc_scratch_bytes) exceeds it
 * are rejected with GBTA_ERR_ARG before any device work.  All calls on a device share
 * the array and it keeps the last call's contents (each call clears what must start
 * at zero): calls that overlap on the GPU race.
 *
 * The array and the code of this path occupy device memory from the moment the part
 * of the library that holds them is loaded on a GPU until the process exits.  Under
 * CUDA's default lazy module loading that happens during the FIRST call on each
 * device, which also looks up the array's device address (with that device current):
 * that first call does take device memory (the 64 MiB plus kernel code), so make it --
 * any small problem will do -- before the caller reserves its memory pool, and before
 * any stream capture.  With CUDA_MODULE_LOADING=EAGER in the environment the memory is
 * taken when the process creates its CUDA context instead.  If the load fails for lack
 * of memory, the call returns GBTA_ERR_CUDA with a message that says so. */
#define GBTA_NOALLOC_SCRATCH_BYTES (64u << 20)
size_t gbta_noalloc_scratch_bytes(int b, int nt, int a);
int gbta_pobtaf_noalloc(int b, int nt, int a, double* D, double* L, double* R, double* T, void* stream);

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

/* ---- on-device assembly of Kronecker-sum precisions ----------------------- */
/* Largest number of variates (coregional components) a model may have. */
#define GBTA_MAX_VARIATES 8

/* Overwrite D, L (R, T) with the BTA blocks of
 *     Q = sum_k  M_k(theta) (x) S_k  +  sum_v lik_scale[v] * A_v^T A_v  +  tip_diag * I_a
 * where S_k are fixed ns x ns spatial matrices placed at variate block (v_k, w_k) of
 * the b = nv * ns diagonal block, with temporal coefficients
 *     D_t += alpha[k*nt + t] * S_k,     L_t += beta[k*(nt-1) + t] * S_k.
 * The S_k share one union pattern (CSR upat_rowptr[ns+1], upat_col); uval[e*nterms + k]
 * is S_k's value at union entry e (0 when absent); term_vw[2k], term_vw[2k+1] = (v_k, w_k).
 * A^T A (theta-independent) is given as CSR rows of the diagonal blocks (lik_rowptr
 * [nt*b+1] over block rows t*b + rho, lik_col block-local) plus dense arrow parts
 * lik_R (nt, a, b) and lik_T (a, a); any of them may be NULL.  A_v^T A_v is the part
 * of A^T A that belongs to the observations of variate v: diagonal-block rows and R
 * columns of variate v's nodes, T rows of the fixed effects with arrow_variate[i] == v
 * (arrow_variate: device [a], NULL = every fixed effect belongs to variate 0).
 * lik_scale is a DEVICE array of nv noise precisions, read when the kernel runs (so a
 * captured graph picks up new values); required when any A^T A part is given.
 * All arrays are device pointers.  Replaces the per-evaluation Q construction of the
 * reference (src/pyinla/submodels/spatio_temporal.py:114-149, src/pyinla/core/model.py:
 * 306-423, src/pyinla/models/coregional_model.py:274-643) and the sparse-to-BTA
 * scatter (structured_solver.py:192-468).  Deterministic.  Asynchronous on the
 * solver's stream. */
int gbta_assemble_kron(gbta_solver* s, int ns, int nv, int nterms, const int* upat_rowptr,
                       const int* upat_col, const double* uval, const int* term_vw, const double* alpha,
                       const double* beta, const long long* lik_rowptr, const int* lik_col,
                       const double* lik_val, const double* lik_R, const double* lik_T, const double* lik_scale,
                       const int* arrow_variate, double tip_diag, double* D, double* L, double* R, double* T);

/* Contractions for the adjoint theta-gradient (no counterpart in the reference, which
 * differentiates by central finite differences, src/pyinla/core/pyinla.py:512-600):
 * with Sigma given by SD, SL, SR, ST (selected inverse blocks, any may be NULL) and
 * mu (N vector, may be NULL), writes out[4*K*nt + 2*nv*(nt+1)] (K = nterms):
 *   out[0*K*nt + k*nt + t] = <Sigma_tt, S_k>       out[1*K*nt + k*nt + t] = <Sigma_{t+1,t}, S_k>
 *   out[2*K*nt + k*nt + t] = mu_t' S_k mu_t        out[3*K*nt + k*nt + t] = mu_{t+1}' S_k mu_t
 *   out[4*K*nt + v*2*(nt+1) + t]          = <Sigma, A_v^T A_v> on block t (t = nt: tip part)
 *   out[4*K*nt + v*2*(nt+1) + nt+1 + t]   = the same with mu mu'.
 * Deterministic.  Asynchronous on the solver's stream. */
int gbta_contract_kron(gbta_solver* s, int ns, int nv, int nterms, const int* upat_rowptr,
                       const int* upat_col, const double* uval, const int* term_vw,
                       const long long* lik_rowptr, const int* lik_col, const double* lik_val,
                       const double* lik_R, const double* lik_T, const int* arrow_variate, const double* SD,
                       const double* SL, const double* SR, const double* ST, const double* mu, double* out);

/* ---- marginal variances from a selected inverse --------------------------- */
/* Latent marginal variances out[nt*b + a] = diag(Sigma) in latent order, from the
 * diagonal blocks SD and the tip ST of a selected inverse (gbta_pobtasi output).
 * Replaces PyINLA.get_marginal_variances_latent_parameters
 * (src/pyinla/core/pyinla.py:940-964: _structured_to_spmatrix on the identity's
 * pattern, structured_solver.py:470-538, then extract_diagonal,
 * src/pyinla/utils/spmatrix_utils.py:46-63).  Asynchronous on the solver's stream. */
int gbta_sigma_diagonal(gbta_solver* s, const double* SD, const double* ST, double* out);

/* Observation marginal variances out[r] = (A Sigma A^T)_rr for the nrows rows of the
 * CSR observation matrix A (device arrays: A_rowptr[nrows + 1], A_col, A_val; columns
 * in latent order), read from the Sigma blocks SD, SL, SR, ST.  Replaces
 * PyINLA.get_marginal_variances_observations (src/pyinla/core/pyinla.py:966-1018: Sigma
 * on the pattern of Q_cond, then the diagonal of the dense product a @ Sigma @ a.T).
 * Pairs of columns farther apart than neighbouring time blocks are outside the BTA
 * pattern and contribute 0; a row with a column outside [0, nt*b + a) gets NaN.
 * Deterministic.  Asynchronous on the solver's stream. */
int gbta_obs_variances(gbta_solver* s, long long nrows, const long long* A_rowptr, const int* A_col,
                       const double* A_val, const double* SD, const double* SL, const double* SR,
                       const double* ST, double* out);

/* ---- inner Newton iteration for non-Gaussian likelihoods ----------------- */
/* out[e] = sum_{k = seg[e] .. seg[e+1]-1} w[obs[k]] * coef[k] for e < n_out (device
 * arrays; fixed order, deterministic): the entries of A^T W A that gbta_assemble_kron
 * takes as its likelihood part (diagonal-block CSR values, then the dense arrow rows,
 * then the tip), from the per-entry lists of (observation, A_rp A_rq) pairs.  Replaces
 * the product A^T D A of Model.construct_Q_conditional (src/pyinla/core/model.py:384-423)
 * for the inner iteration of PyINLA._inner_iteration (src/pyinla/core/pyinla.py:1025-1074).
 * Asynchronous on the solver's stream. */
int gbta_weighted_gram(gbta_solver* s, long long n_out, const long long* seg, const int* obs, const double* coef,
                       const double* w, double* out);

/* y = Q x for the symmetric BTA matrix in the Serinv layout (D full symmetric blocks,
 * L_t = block (t+1, t), R_t = arrow rows of column block t, T the tip; use_arrow = 0
 * ignores R, T and the last a entries).  Device pointers, N = nt*b + a.  The product
 * Q_prior x of the information vector (src/pyinla/core/model.py:425-449) and of the
 * prior term x^T Q_prior x (src/pyinla/core/pyinla.py:1076-1110).  Fixed summation
 * order (deterministic).  Asynchronous on the solver's stream. */
int gbta_bta_symv(gbta_solver* s, const double* D, const double* L, const double* R, const double* T,
                  int use_arrow, const double* x, double* y);

/* ---- many instances in one persistent launch per phase -------------------- */
/* A batch holds n independent BTA instances of arbitrary geometry (b[k], nt[k], a[k];
 * a[k] = 0: block tridiagonal) -- the Q(theta) of a gradient's central-difference
 * points, a Hessian or a theta grid (the reference evaluates them one at a time,
 * src/pyinla/core/pyinla.py:512-600, 747-910), including coregional instances of other
 * block sizes.  Each phase of all instances runs as ONE persistent launch that hands
 * out the tasks of every instance from a merged ticket order.  No reference
 * counterpart as an interface: per instance the results equal gbta_pobtaf /
 * gbta_logdet / gbta_pobtas (N then C, one right-hand side) / gbta_pobtasi.
 * methods[k] (NULL = all GBTA_METHOD_OZAKI) fixes each instance's product method and
 * is chosen at creation because it sizes the workspace.  The batch owns its workspace
 * and a non-blocking stream. */
typedef struct gbta_batch gbta_batch;

#define GBTA_PHASE_FACTOR 1   /* pobtaf (pobtf when a = 0) */
#define GBTA_PHASE_LOGDET 2   /* logdet of the factor into logdet_out[k] (device) */
#define GBTA_PHASE_SOLVE 4    /* pobtas N then C on rhs[k] (one column, in place) */
#define GBTA_PHASE_SELINV 8   /* pobtasi: the factor blocks become Sigma */

/* Ticket order of the merged task lists. */
#define GBTA_BATCH_ORDER_PROPORTIONAL 0   /* every instance advances at the same fraction */
#define GBTA_BATCH_ORDER_ROUND_ROBIN 1    /* one task of each instance in turn */
#define GBTA_BATCH_ORDER_SEQUENTIAL 2     /* instance after instance */

int gbta_batch_create(int n, const int* b, const int* nt, const int* a, const int* methods, gbta_batch** out);
int gbta_batch_destroy(gbta_batch* bt);
size_t gbta_batch_workspace_bytes(const gbta_batch* bt);
/* Work goes to `stream` (NULL = CUDA default stream; graph launches need another). */
int gbta_batch_set_stream(gbta_batch* bt, void* stream);
int gbta_batch_set_order(gbta_batch* bt, int policy);
/* Persistent CTAs per SM of the batch's launches (0, the default: as many as fit). */
int gbta_batch_set_ctas_per_sm(gbta_batch* bt, int n);
int gbta_batch_set_wait_limit_ms(gbta_batch* bt, double ms);
/* Bind the instances' device blocks: arrays (host) of n device pointers in the
 * Serinv layout; R, T may be NULL (or hold NULL) for a[k] = 0; rhs may be NULL when
 * the solve phase is not used.  The pointers must stay valid for every later run and
 * every replay of a captured graph. */
int gbta_batch_bind(gbta_batch* bt, double* const* D, double* const* L, double* const* R, double* const* T,
                    double* const* rhs);
/* Enqueue the phases (GBTA_PHASE_* bits) of every instance on the batch stream, in
 * the order factor, logdet, solve, selected inversion.  No host synchronisation. */
int gbta_batch_run_async(gbta_batch* bt, int phases, double* logdet_out);
/* The same, captured once into a CUDA graph (re-captured when phases or logdet_out
 * change) and launched: one graph launch per call. */
int gbta_batch_graph_launch(gbta_batch* bt, int phases, double* logdet_out);
/* Kernels one replay of the captured graph launches. */
long long gbta_batch_graph_kernels(const gbta_batch* bt);
/* Wait for the stream.  Returns 0, GBTA_ERR_TIMEOUT, or the pivot row (> 0) of the
 * first instance that is not positive definite; info[k] (host, may be NULL) receives
 * every instance's pivot row (0 = fine). */
int gbta_batch_status(gbta_batch* bt, int* info);

#ifdef __cplusplus
}
#endif

#endif /* PYINLA_GB300_H */
