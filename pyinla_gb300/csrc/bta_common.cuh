// Shared device machinery of the BTA dataflow kernels.
//
// Every kernel of this library is a persistent "task" kernel: one CTA per SM pulls
// task tickets from a global counter in a topological order of the tile DAG, waits
// (bounded) on per-tile ready flags, runs the task on TS x TS FP64 tiles and
// publishes its output tile with a release store of the flag.  Because a CTA only
// waits for tasks with smaller tickets, and a ticket is only handed to a CTA that
// is already running, the kernels make progress without co-residency guarantees.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "bta_internal.h"

namespace gbta {

constexpr int NT = 128;          // threads per CTA
constexpr int LDS = TS + 1;      // shared-memory row stride (odd: column reads hit distinct banks)
constexpr int TILE_SMEM = TS * LDS;
constexpr int PER_THREAD = TS * TS / NT;   // tile elements staged per thread (8)

// Control block (ints) shared by all kernels of a solver.
enum {
  CTRL_TICKET = 0,   // next task ticket
  CTRL_ABORT = 1,    // set when any task fails; every wait returns early
  CTRL_INFO = 2,     // sticky: 1-based global row of the first non-positive pivot
  CTRL_ERR = 3,      // sticky: ERR_* code
  CTRL_N = 8
};
enum { ERR_NONE = 0, ERR_TIMEOUT = 1 };

struct Ctl {
  int* ctrl;
  int* flags;
  int epoch;
  unsigned long long wait_ns;
  long long* trace;   // optional: 4 int64 per task (see trace_task), or null
};

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_relaxed(const int* p) {
  return *(volatile const int*)p;
}
__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned smid() {
  unsigned r;
  asm volatile("mov.u32 %0, %%smid;" : "=r"(r));
  return r;
}
// Task trace record (thread 0): [ticket, (type << 16) | sm, t_start, t_end] in
// globaltimer nanoseconds; written only when tracing is enabled.
__device__ __forceinline__ void trace_task(const Ctl& c, int ticket, int type, unsigned long long t0) {
  if (c.trace && threadIdx.x == 0) {
    long long* r = c.trace + 4ll * ticket;
    r[0] = ticket;
    r[1] = ((long long)type << 16) | smid();
    r[2] = (long long)t0;
    r[3] = (long long)gtimer();
  }
}

__device__ __forceinline__ void raise_abort(const Ctl& c) { atomicExch(c.ctrl + CTRL_ABORT, 1); }

// Thread-0 helper: spin (bounded in time) until flag >= epoch.  Returns false on
// abort or timeout (timeout also records ERR_TIMEOUT and aborts the launch).
// Only thread 0 of a CTA polls, and a persistent kernel runs one CTA per SM, so the
// first SPIN_NS of a wait are a tight acquire-load loop (the hop latency of the
// dependency chains is what bounds these kernels); longer waits back off with a
// short sleep.
constexpr unsigned long long SPIN_NS = 200000;

static __device__ bool spin_ready(const Ctl& c, const int* flag) {
  if (ld_acquire(flag) >= c.epoch) return true;
  const unsigned long long t0 = gtimer();
  for (unsigned it = 1;; ++it) {
    if (ld_acquire(flag) >= c.epoch) return true;
    if ((it & 63) == 0) {
      if (ld_relaxed(c.ctrl + CTRL_ABORT)) return false;
      const unsigned long long dt = gtimer() - t0;
      if (dt > c.wait_ns) {
        atomicCAS(c.ctrl + CTRL_ERR, ERR_NONE, ERR_TIMEOUT);
        raise_abort(c);
        return false;
      }
      if (dt > SPIN_NS) __nanosleep(256);
    }
  }
}

// CTA-wide wait on up to two flags (nullptr = no flag).  All threads return the
// same value.  Contains __syncthreads().
static __device__ bool cta_wait(const Ctl& c, const int* f0, const int* f1, int* s_ok) {
  if (threadIdx.x == 0) {
    bool ok = true;
    if (f0) ok = spin_ready(c, f0);
    if (ok && f1) ok = spin_ready(c, f1);
    *s_ok = ok ? 1 : 0;
  }
  __syncthreads();
  const bool ok = *s_ok != 0;
  __syncthreads();
  return ok;
}

// Readiness scan for pipelined product loops.  Thread 0 advances *s_ready (the
// number of leading steps whose operand flags are all set) by checking up to
// SCAN_AHEAD further steps with independent relaxed loads and a single acquire fence,
// so one memory round trip covers many steps.  `flags_of(s, f0, f1)` returns the
// step's flags (nullptr = none).  The caller synchronises the CTA afterwards.
constexpr int SCAN_AHEAD = 8;

__device__ __forceinline__ int ld_relaxed_gpu(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void fence_acquire_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

template <class FlagsOf>
__device__ __forceinline__ void scan_ready(const Ctl& c, int nsteps, FlagsOf flags_of, int* s_ready) {
  if (threadIdx.x == 0) {
    const int r0 = *s_ready;
    int v[SCAN_AHEAD];
#pragma unroll
    for (int k = 0; k < SCAN_AHEAD; ++k) {
      v[k] = 1;
      if (r0 + k < nsteps) {
        const int* f0;
        const int* f1;
        flags_of(r0 + k, f0, f1);
        const int a = f0 ? ld_relaxed_gpu(f0) : c.epoch;
        const int b = f1 ? ld_relaxed_gpu(f1) : c.epoch;
        v[k] = (a >= c.epoch) && (b >= c.epoch);
      }
    }
    fence_acquire_gpu();
    int r = r0;
#pragma unroll
    for (int k = 0; k < SCAN_AHEAD; ++k)
      if (r == r0 + k && r < nsteps && v[k]) ++r;
    *s_ready = r;
  }
}

// CTA-wide non-blocking poll of up to two flags.  Contains __syncthreads().
static __device__ bool cta_poll(const Ctl& c, const int* f0, const int* f1, int* s_ok) {
  if (threadIdx.x == 0) {
    bool ok = true;
    if (f0) ok = ld_acquire(f0) >= c.epoch;
    if (ok && f1) ok = ld_acquire(f1) >= c.epoch;
    *s_ok = ok ? 1 : 0;
  }
  __syncthreads();
  const bool ok = *s_ok != 0;
  __syncthreads();
  return ok;
}

// Publish a tile: every thread's stores are ordered before the flag release.
__device__ __forceinline__ void cta_publish(const Ctl& c, int* flag) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    st_release(flag, c.epoch);
  }
}

// Pull the next ticket (CTA-uniform).
__device__ __forceinline__ int cta_ticket(const Ctl& c, int* s_t) {
  __syncthreads();
  if (threadIdx.x == 0) *s_t = ld_relaxed(c.ctrl + CTRL_ABORT) ? -1 : atomicAdd(c.ctrl + CTRL_TICKET, 1);
  __syncthreads();
  return *s_t;
}

// A tile view into a row-major matrix: rows x cols valid elements (<= TS each).
struct Tile {
  const double* p;
  int ld;
  int rows;
  int cols;
};

__device__ __forceinline__ Tile make_tile(const double* base, int ld, int row0, int col0, int nrows_total,
                                          int ncols_total) {
  Tile t;
  t.p = base + (size_t)row0 * ld + col0;
  t.ld = ld;
  t.rows = min(TS, nrows_total - row0);
  t.cols = min(TS, ncols_total - col0);
  return t;
}

// Register staging of one tile: element k of this thread is (r, c) with
// idx = threadIdx.x + k*NT, r = idx / TS, c = idx % TS (a warp reads one 256-B row).
// Loads bypass L1 (ld.global.cg): tiles are produced by other SMs inside the launch.
__device__ __forceinline__ void tile_ldg(double (&v)[PER_THREAD], const Tile& t) {
#pragma unroll
  for (int k = 0; k < PER_THREAD; ++k) {
    const int idx = threadIdx.x + k * NT;
    const int r = idx / TS, c = idx % TS;
    v[k] = (r < t.rows && c < t.cols) ? __ldcg(t.p + (size_t)r * t.ld + c) : 0.0;
  }
}
__device__ __forceinline__ void tile_sts(double* S, const double (&v)[PER_THREAD]) {
#pragma unroll
  for (int k = 0; k < PER_THREAD; ++k) {
    const int idx = threadIdx.x + k * NT;
    S[(idx / TS) * LDS + (idx % TS)] = v[k];
  }
}
// Transposed store: S[c][r] = element (r, c).
__device__ __forceinline__ void tile_sts_t(double* S, const double (&v)[PER_THREAD]) {
#pragma unroll
  for (int k = 0; k < PER_THREAD; ++k) {
    const int idx = threadIdx.x + k * NT;
    S[(idx % TS) * LDS + (idx / TS)] = v[k];
  }
}
__device__ __forceinline__ void tile_sts_op(double* S, const double (&v)[PER_THREAD], bool trans) {
  if (trans)
    tile_sts_t(S, v);
  else
    tile_sts(S, v);
}
// Direct global -> shared tile load (used outside the pipelined loops).
__device__ __forceinline__ void tile_load(double* S, const Tile& t) {
  double v[PER_THREAD];
  tile_ldg(v, t);
  tile_sts(S, v);
}
// Set the padded part of a diagonal tile's diagonal to one (rows/cols >= n).
__device__ __forceinline__ void tile_pad_identity(double* S, int n) {
  for (int j = n + threadIdx.x; j < TS; j += NT) S[j * LDS + j] = 1.0;
}
// Store the valid part of a shared tile.
__device__ __forceinline__ void tile_store(double* dst, int ld, int rows, int cols, const double* S) {
#pragma unroll
  for (int k = 0; k < PER_THREAD; ++k) {
    const int idx = threadIdx.x + k * NT;
    const int r = idx / TS, c = idx % TS;
    if (r < rows && c < cols) dst[(size_t)r * ld + c] = S[r * LDS + c];
  }
}
__device__ __forceinline__ void tile_store_zero(double* dst, int ld, int rows, int cols) {
#pragma unroll
  for (int k = 0; k < PER_THREAD; ++k) {
    const int idx = threadIdx.x + k * NT;
    const int r = idx / TS, c = idx % TS;
    if (r < rows && c < cols) dst[(size_t)r * ld + c] = 0.0;
  }
}

// ---------------------------------------------------------------------------
// Tile GEMM micro-kernel: acc (+|-)= op(A) * op(B) on TS x TS shared tiles.
// Thread (ty, tx) = (tid / 8, tid % 8) owns rows {2ty, 2ty+1} and columns
// {tx, tx+8, tx+16, tx+24}.
// ---------------------------------------------------------------------------
struct Acc {
  double v[2][4];
};

__device__ __forceinline__ void acc_zero(Acc& a) {
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int q = 0; q < 4; ++q) a.v[i][q] = 0.0;
}
__device__ __forceinline__ int acc_row(int i) { return (threadIdx.x / 8) * 2 + i; }
__device__ __forceinline__ int acc_col(int q) { return (threadIdx.x % 8) + 8 * q; }

__device__ __forceinline__ void acc_from_smem(Acc& a, const double* S) {
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int q = 0; q < 4; ++q) a.v[i][q] = S[acc_row(i) * LDS + acc_col(q)];
}
__device__ __forceinline__ void acc_to_smem(const Acc& a, double* S) {
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int q = 0; q < 4; ++q) S[acc_row(i) * LDS + acc_col(q)] = a.v[i][q];
}

// acc (+|-)= A * B with A(i,m) = As[i][m], B(m,j) = Bs[m][j] (transposes are applied
// when the tiles are staged into shared memory).
template <bool SUB>
__device__ __forceinline__ void tile_mma(Acc& acc, const double* As, const double* Bs) {
  const int i0 = (threadIdx.x / 8) * 2;
  const int j0 = threadIdx.x % 8;
#pragma unroll 8
  for (int m = 0; m < TS; ++m) {
    const double a0 = As[i0 * LDS + m];
    const double a1 = As[(i0 + 1) * LDS + m];
    double bq[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) bq[q] = Bs[m * LDS + j0 + 8 * q];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (SUB) {
        acc.v[0][q] = fma(-a0, bq[q], acc.v[0][q]);
        acc.v[1][q] = fma(-a1, bq[q], acc.v[1][q]);
      } else {
        acc.v[0][q] = fma(a0, bq[q], acc.v[0][q]);
        acc.v[1][q] = fma(a1, bq[q], acc.v[1][q]);
      }
    }
  }
}

// One step of a tile K-loop: operand tiles, whether each is staged transposed, and
// the ready flags to wait on (nullptr: no wait).
struct Step {
  Tile a, b;
  bool ta, tb;
  const int* fa;
  const int* fb;
};

// Pipelined K-loop: acc (+|-)= sum_s op(A_s) op(B_s).  The next step's tiles are
// fetched into registers while the current step computes, when their flags are
// already set (otherwise after the compute, with a bounded wait).  `bufs` holds
// four shared tiles.  Returns false (uniformly) on abort/timeout.
template <bool SUB, class StepFn>
static __device__ bool kloop(Acc& acc, int nsteps, StepFn step_of, const Ctl& c, double* bufs, int* s_ok) {
  if (nsteps <= 0) return true;
  double ra[PER_THREAD], rb[PER_THREAD];
  Step st = step_of(0);
  if (!cta_wait(c, st.fa, st.fb, s_ok)) return false;
  tile_ldg(ra, st.a);
  tile_ldg(rb, st.b);
  tile_sts_op(bufs, ra, st.ta);
  tile_sts_op(bufs + TILE_SMEM, rb, st.tb);
  __syncthreads();
  for (int s = 0; s < nsteps; ++s) {
    double* cur = bufs + (s & 1) * 2 * TILE_SMEM;
    double* nxt = bufs + ((s + 1) & 1) * 2 * TILE_SMEM;
    const bool more = s + 1 < nsteps;
    bool pre = false;
    if (more) {
      st = step_of(s + 1);
      pre = cta_poll(c, st.fa, st.fb, s_ok);
      if (pre) {
        tile_ldg(ra, st.a);
        tile_ldg(rb, st.b);
      }
    }
    tile_mma<SUB>(acc, cur, cur + TILE_SMEM);
    if (more) {
      if (!pre) {
        if (!cta_wait(c, st.fa, st.fb, s_ok)) return false;
        tile_ldg(ra, st.a);
        tile_ldg(rb, st.b);
      }
      tile_sts_op(nxt, ra, st.ta);
      tile_sts_op(nxt + TILE_SMEM, rb, st.tb);
    }
    __syncthreads();
  }
  return true;
}

// ---------------------------------------------------------------------------
// Small dense kernels on shared tiles (whole CTA).
// ---------------------------------------------------------------------------

// Scalar FP64 helpers.  On GB300 one warp-wide FP64 instruction occupies an SM
// sub-partition's FP64 unit for ~64 cycles, so the sequential per-column work of the
// small tile kernels is kept to a few FP64 instructions: reciprocals and inverse
// square roots are Newton-Raphson refinements (y <- y (2 - x y), resp.
// y <- y (3 - x y^2) / 2, each doubling the correct bits) of the hardware
// approximations rcp.approx / rsqrt.approx, computed once per tile or per pivot.
__device__ __forceinline__ double nr_recip(double x) {
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  double e = fma(-x, y, 1.0);
  y = fma(y, e, y);
  e = fma(-x, y, 1.0);
  y = fma(y, e, y);
  e = fma(-x, y, 1.0);
  return fma(y, e, y);
}
__device__ __forceinline__ double nr_rsqrt(double x) {
  double y;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  const double h = 0.5 * x;
  double r = fma(-h * y, y, 0.5);
  y = fma(y, r, y);
  r = fma(-h * y, y, 0.5);
  y = fma(y, r, y);
  r = fma(-h * y, y, 0.5);
  return fma(y, r, y);
}

// sqrt(x) and 1/sqrt(x) together by Goldschmidt's iteration (R. E. Goldschmidt,
// "Applications of division by convergence", MIT thesis, 1964): from y0 ~ 1/sqrt(x)
// (rsqrt.approx, ~20 correct bits), g = x y0, h = y0/2 and r = 1/2 - g h,
// g <- g + g r, h <- h + h r doubles the correct bits per step; g and h update in
// parallel, so two steps are a chain of five FP64 operations instead of the eleven
// of three dependent Newton steps.
__device__ __forceinline__ void gs_sqrt_rsqrt(double x, double& sq, double& rs) {
  double y;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  double g = x * y, h = 0.5 * y;
  double r = fma(-g, h, 0.5);
  g = fma(g, r, g);
  h = fma(h, r, h);
  r = fma(-g, h, 0.5);
  g = fma(g, r, g);
  h = fma(h, r, h);
  sq = g;
  rs = 2.0 * h;
}

// rd[j] = 1 / F[j][j] for the TS diagonal entries (one lane each).  Caller syncs.
__device__ __forceinline__ void tile_diag_recip(const double* F, double* rd) {
  if (threadIdx.x < TS) rd[threadIdx.x] = nr_recip(F[threadIdx.x * LDS + threadIdx.x]);
}

// In-place lower Cholesky of S (TS x TS; entries past n must already be identity).
// Returns 0, or the 1-based column of the first non-positive (or NaN) pivot.
// One barrier per column: step j updates the trailing matrix with the unscaled
// column j and 1/d_j; the columns are scaled by 1/sqrt(d_j) in a final pass (column
// j is not modified after step j).  The strict upper triangle is zeroed on success.
// `ybuf` is a TS-double shared scratch.
static __device__ int smem_potrf(double* S, double* ybuf) {
  for (int j = 0; j < TS; ++j) {
    __syncthreads();
    const double d = S[j * LDS + j];
    if (!(d > 0.0)) {
      __syncthreads();
      return j + 1;
    }
    double sq, y;
    gs_sqrt_rsqrt(d, sq, y);
    const double inv = y * y;
    if (threadIdx.x == 0) ybuf[j] = y;
    const int m = TS - 1 - j;
    for (int idx = threadIdx.x; idx < m * m; idx += NT) {
      const int rr = j + 1 + idx / m, kk = j + 1 + idx % m;
      if (kk <= rr) S[rr * LDS + kk] = fma(-S[rr * LDS + j] * inv, S[kk * LDS + j], S[rr * LDS + kk]);
    }
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < TS * TS; idx += NT) {
    const int r = idx / TS, c = idx % TS;
    S[r * LDS + c] = (c > r) ? 0.0 : S[r * LDS + c] * ybuf[c];
  }
  __syncthreads();
  return 0;
}

// X <- X * F^{-T} with F lower triangular; rd = 1/diag(F) (tile_diag_recip, synced).
// One barrier per column: column j stays unscaled until a final pass, updates use
// X[r][j] * rd[j].
static __device__ void smem_trsm_rlt(double* X, const double* F, const double* rd) {
  for (int j = 0; j < TS - 1; ++j) {
    __syncthreads();
    const double rj = rd[j];
    const int m = TS - 1 - j;
    for (int idx = threadIdx.x; idx < TS * m; idx += NT) {
      const int r = idx / m, col = j + 1 + idx % m;
      X[r * LDS + col] = fma(-X[r * LDS + j] * rj, F[col * LDS + j], X[r * LDS + col]);
    }
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < TS * TS; idx += NT) X[(idx / TS) * LDS + idx % TS] *= rd[idx % TS];
  __syncthreads();
}

// X <- X * F^{-1} with F lower triangular (solve X F = X, backward column sweep);
// rd = 1/diag(F).  Same one-barrier-per-column scheme.
static __device__ void smem_trsm_rln(double* X, const double* F, const double* rd) {
  for (int j = TS - 1; j > 0; --j) {
    __syncthreads();
    const double rj = rd[j];
    for (int idx = threadIdx.x; idx < TS * j; idx += NT) {
      const int r = idx / j, col = idx % j;
      X[r * LDS + col] = fma(-X[r * LDS + j] * rj, F[j * LDS + col], X[r * LDS + col]);
    }
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < TS * TS; idx += NT) X[(idx / TS) * LDS + idx % TS] *= rd[idx % TS];
  __syncthreads();
}

}  // namespace gbta
