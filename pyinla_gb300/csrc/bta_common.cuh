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
  CTRL_MMA = 4,      // words 4-5: tile-pair products issued by the launch (one 64-bit count)
  CTRL_N = 8
};
enum { ERR_NONE = 0, ERR_TIMEOUT = 1 };

struct Ctl {
  int* ctrl;
  int* flags;
  int epoch;
  unsigned long long wait_ns;
  long long* trace;   // optional: TRACE_WORDS int64 per task (see trace_task), or null
};

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// Release-add at GPU scope without a return value (no round trip for the issuer).
__device__ __forceinline__ void red_add_release(int* p, int v) {
  asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// Atomic add with acquire-release semantics at GPU scope; returns the old value.
__device__ __forceinline__ int atom_add_acq_rel(int* p, int v) {
  int old;
  asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
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
// Task trace record (thread 0): [ticket, (type << 16) | sm, t_start, t_end, m0..m3] in
// globaltimer nanoseconds, m0..m3 optional intermediate marks (0 when unused);
// written only when tracing is enabled.
constexpr int TRACE_WORDS = 8;
__device__ __forceinline__ void trace_task(const Ctl& c, int ticket, int type, unsigned long long t0) {
  if (c.trace && threadIdx.x == 0) {
    long long* r = c.trace + (long long)TRACE_WORDS * ticket;
    r[0] = ticket;
    r[1] = ((long long)blockIdx.x << 32) | ((long long)type << 16) | smid();
    r[2] = (long long)t0;
    r[3] = (long long)gtimer();
  }
}
__device__ __forceinline__ void trace_clear_marks(const Ctl& c, int ticket) {
  if (c.trace && threadIdx.x == 0)
    for (int k = 4; k < TRACE_WORDS; ++k) c.trace[(long long)TRACE_WORDS * ticket + k] = 0;
}
__device__ __forceinline__ void trace_mark(const Ctl& c, int ticket, int k) {
  if (c.trace && threadIdx.x == 0) c.trace[(long long)TRACE_WORDS * ticket + 4 + k] = (long long)gtimer();
}
__device__ __forceinline__ void trace_put(const Ctl& c, int ticket, int k, long long v) {
  if (c.trace && threadIdx.x == 0) c.trace[(long long)TRACE_WORDS * ticket + 4 + k] = v;
}

__device__ __forceinline__ void raise_abort(const Ctl& c) { atomicExch(c.ctrl + CTRL_ABORT, 1); }

// Thread-0 helper: spin (bounded in time) until flag >= epoch.  Returns false on
// abort or timeout (timeout also records ERR_TIMEOUT and aborts the launch).
// Only thread 0 of a CTA polls, and a persistent kernel runs one CTA per SM, so the
// first SPIN_NS of a wait are a tight acquire-load loop (the hop latency of the
// dependency chains is what bounds these kernels); longer waits back off with a
// short sleep.
constexpr unsigned long long SPIN_NS = 200000;

static __device__ bool spin_ready(const Ctl& c, const int* flag, int* seen = nullptr, int plus = 0) {
  const int want = c.epoch + plus;
  int v = ld_acquire(flag);
  if (v >= want) {
    if (seen) *seen = v;
    return true;
  }
  const unsigned long long t0 = gtimer();
  for (unsigned it = 1;; ++it) {
    v = ld_acquire(flag);
    if (v >= want) {
      if (seen) *seen = v;
      return true;
    }
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

// CTA-wide wait on one flag that also returns the flag word seen (epoch + payload) to
// every thread through *s_val.  Contains __syncthreads().
static __device__ bool cta_wait_val(const Ctl& c, const int* f, int* s_ok, int* s_val) {
  if (threadIdx.x == 0) *s_ok = spin_ready(c, f, s_val) ? 1 : 0;
  __syncthreads();
  const bool ok = *s_ok != 0;
  __syncthreads();
  return ok;
}

// Wait until *f >= epoch + plus: a flag that was published (epoch) and then raised by
// `plus` with cta_raise for a second product of the same task.
static __device__ bool cta_wait_plus(const Ctl& c, const int* f, int plus, int* s_ok) {
  if (threadIdx.x == 0) *s_ok = spin_ready(c, f, nullptr, plus) ? 1 : 0;
  __syncthreads();
  const bool ok = *s_ok != 0;
  __syncthreads();
  return ok;
}

// Publish a tile with a payload in its flag word (see EPOCH_SHIFT).  The barrier
// orders every thread's writes before thread 0's release store, which is cumulative,
// so no separate fence is needed.
__device__ __forceinline__ void cta_publish_val(const Ctl& c, int* flag, int payload) {
  __syncthreads();
  if (threadIdx.x == 0) st_release(flag, c.epoch + payload);
}

// Readiness scan for pipelined product loops.  Warp 0 advances *s_ready (the number of
// leading steps whose operand flags are all set) by checking up to SCAN_AHEAD further
// steps at once: lane 2k loads the first flag of step *s_ready + k and lane 2k+1 its
// second, each with an acquire load, so one memory round trip covers all of them and
// no GPU-scope fence is needed (a fence waits for the CTA's own outstanding writes,
// which costs thousands of cycles in a busy kernel).  `flags_of(s, f0, f1)` returns the
// step's flags (nullptr = none).  The caller synchronises the CTA before the call (the
// other warps decide from *s_ready whether to call it, so they must have read it before
// warp 0 rewrites it; a warp that read the new value would skip the call and its
// barriers) and afterwards, which extends the acquires to all its threads.
constexpr int SCAN_AHEAD = 16;
static_assert(2 * SCAN_AHEAD <= 32, "one lane per flag");

__device__ __forceinline__ int ld_relaxed_gpu(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// With `ring` (SCAN_RING ints), the first flag word of every step found ready is kept
// at ring[step % SCAN_RING] (read while step - *s_ready < SCAN_RING - SCAN_AHEAD).
constexpr int SCAN_RING = 2 * SCAN_AHEAD;
template <class FlagsOf>
__device__ __forceinline__ void scan_ready(const Ctl& c, int nsteps, FlagsOf flags_of, int* s_ready,
                                           int* ring = nullptr) {
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    const int r0 = *s_ready;
    const int k = lane >> 1;
    int word = c.epoch;
    bool ready = true;
    if (k < SCAN_AHEAD) {
      if (r0 + k < nsteps) {
        const int* f0;
        const int* f1;
        flags_of(r0 + k, f0, f1);
        const int* f = (lane & 1) ? f1 : f0;
        if (f) {
          word = ld_acquire(f);
          ready = word >= c.epoch;
        }
      } else {
        ready = false;
      }
    }
    const unsigned ok = __ballot_sync(0xffffffffu, ready);
    int r = r0;
#pragma unroll
    for (int kk = 0; kk < SCAN_AHEAD; ++kk) {
      const int w0 = __shfl_sync(0xffffffffu, word, 2 * kk);
      if (r == r0 + kk && ((ok >> (2 * kk)) & 3u) == 3u) {
        if (ring && lane == 0) ring[r % SCAN_RING] = w0;
        ++r;
      }
    }
    if (lane == 0) *s_ready = r;
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
  __syncthreads();   // every thread's writes before thread 0's (cumulative) release store
  if (threadIdx.x == 0) st_release(flag, c.epoch);
}

// Raise a published flag by v (< 512, so it stays below the next launch's epoch) once
// every thread's writes since the publication are done; the barrier and the cumulative
// release order them as in cta_publish.
__device__ __forceinline__ void cta_raise(int* flag, int v) {
  __syncthreads();
  if (threadIdx.x == 0) red_add_release(flag, v);
}

// Thread 0: add a task's tile-pair products (32 x 32 x 32 fp16 MMAs of two digit planes)
// to the launch's count.
__device__ __forceinline__ void count_pairs(const Ctl& c, unsigned long long n) {
  if (threadIdx.x == 0 && n) atomicAdd(reinterpret_cast<unsigned long long*>(c.ctrl + CTRL_MMA), n);
}

// Pull the next ticket (CTA-uniform).
// Between tasks every thread also orders its generic shared-memory writes (a task's
// FP64 scratch) before the bulk copies (async proxy) that a later task issues into the
// same bytes.
__device__ __forceinline__ int cta_ticket(const Ctl& c, int* s_t) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
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

// Scalar FP64 helpers.  On GB300 a warp-wide FP64 instruction occupies its SM
// sub-partition's FP64 unit for ~64-76 cycles, whether it is dependent, independent or
// even predicated off, so the sequential work of the tile routines below is counted in
// FP64 instructions.  Reciprocals and inverse square roots start from the hardware
// approximations rcp.approx / rsqrt.approx (~20 correct bits) and take ONE third-order
// correction (a truncated binomial series, i.e. a third-order Householder step), which
// leaves a truncation error of order e^3 ~ 2^-57:
//   1/d:       e = 1 - d y,    y <- y (1 + e + e^2)
//   1/sqrt(d): e = 1 - d y^2,  y <- y (1 + e/2 + 3 e^2 / 8)
__device__ __forceinline__ double rcp3(double d) {
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(d));
  const double e = fma(-d, y, 1.0);
  const double p = 1.0 + e;
  const double ye = y * e;
  return fma(ye, p, y);
}
__device__ __forceinline__ double rsqrt3(double d) {
  double y;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(d));
  const double dy = d * y;
  const double e = fma(-dy, y, 1.0);
  const double p = fma(e, 0.375, 0.5);
  const double ye = y * e;
  return fma(ye, p, y);
}

// rd[j] = 1 / F[j][j] for the TS diagonal entries (one lane each).  Caller syncs.
__device__ __forceinline__ void tile_diag_recip(const double* F, double* rd) {
  if (threadIdx.x < TS) rd[threadIdx.x] = rcp3(F[threadIdx.x * LDS + threadIdx.x]);
}

// ---- register-resident tile factorization and triangular solves ------------------
// In the triangular solves, thread (lane r, warp g) holds row r of the tile at the
// eight columns c = g + 4q (q = 0..7) in registers, so every FP64 instruction has 32
// useful lanes.  Columns are processed in order; the warp owning the current column
// finalises it and publishes it through shared memory with one CTA barrier per column,
// and every warp then updates its later columns with one FMA per element (the
// Cholesky, smem_potrf below, splits the work differently).  The loops over
// columns and register slots are fully unrolled: the conditions "column c = g + 4q
// is after column j" are written as a compile-time part plus a runtime part that
// only the one boundary slot needs, because an FP64 instruction issued under a false
// predicate still costs a full pipe slot.
__device__ __forceinline__ bool col_after(int q, int j, int g) {   // g + 4q > j
  return 4 * q > j || (4 * q + 3 > j && g > j - 4 * q);
}
__device__ __forceinline__ bool col_before(int q, int j, int g) {  // g + 4q < j
  return 4 * q + 3 < j || (4 * q < j && g < j - 4 * q);
}

// Named CTA barriers (ids 1 .. 15; id 0 is __syncthreads) for a producer warp that
// hands shared-memory data to the other warps: the producer arrives (release), the
// consumers sync (acquire); NT threads take part.
__device__ __forceinline__ void nbar_arrive(int id) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "n"(NT) : "memory");
}
__device__ __forceinline__ void nbar_sync(int id) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "n"(NT) : "memory");
}

// Named barriers with a thread count other than NT (both sides must agree on N).
template <int N> __device__ __forceinline__ void nbar_arrive_n(int id) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "n"(N) : "memory");
}
template <int N> __device__ __forceinline__ void nbar_sync_n(int id) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "n"(N) : "memory");
}

// Barrier ids of smem_potrf: POTRF_BAR_L + (j & 7) hands pivot j from the pivot warp
// to the three update warps (NT threads); POTRF_BAR_C + (j & 3) hands column j+2,
// updated through pivot j, from its owner to the pivot warp (64 threads).
constexpr int POTRF_BAR_L = 1, POTRF_BAR_C = 9;

// x > 0 (false for zeros and NaN, true for +inf) by integer compares on the bits: a
// double compare is an FP64-unit instruction, and on the pivot chain it would occupy
// that unit for a full slot per pivot.
__device__ __forceinline__ bool positive_bits(double x) {
  const long long b = __double_as_longlong(x);
  return b > 0 && b <= 0x7ff0000000000000ll;
}

// 1/d with the third-order refinement in three dependent FMAs (for a chain that counts
// FP64 instructions): e = 1 - d y, y <- y + y (e + e^2).
__device__ __forceinline__ double rcp3_fma(double d) {
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(d));
  const double e = fma(-d, y, 1.0);
  return fma(y, fma(e, e, e), y);
}

// Register slots of the update warps of smem_potrf.  Slot s < 14 holds column s + 2
// (lane = row); slot s >= 14 holds the pair of columns c0 = 16 + 2 (s - 14) and c0 + 1,
// rows 16..31 only (lane l: row 16 + (l & 15), column c0 + (l >> 4)): a column c needs
// rows c..31, so for c >= 16 half a warp covers it.  Owners rotate over the three warps
// (any seven consecutive columns have all three owners).
constexpr int POTRF_SLOTS = 22, POTRF_FULL = 14;
__host__ __device__ constexpr int potrf_slot_col(int s) { return s < POTRF_FULL ? s + 2 : 16 + 2 * (s - POTRF_FULL); }
__host__ __device__ constexpr int potrf_slot_last(int s) { return s < POTRF_FULL ? s + 2 : 17 + 2 * (s - POTRF_FULL); }
__host__ __device__ constexpr int potrf_slot_owner(int s) { return s < POTRF_FULL ? s % 3 : (s - 12) % 3; }

// Update warp W (0..2; warp W + 1) of smem_potrf.  For every pivot j it first applies
// pivot j to column j + 2 if it owns it and hands that column to the pivot warp, then
// applies pivot j to its slots whose columns come later: a_rc -= w_rj u_cj (w_rj =
// u_rj / d_j from the pivot warp's ring, u_cj from S).  Slot tests are compile-time, so
// no predicated-off FMA is issued.
template <int W>
__device__ __forceinline__ void potrf_update_warp(double* S, const double (*wring)[TS], int lane) {
  const int prow = 16 + (lane & 15), half = lane >> 4;
  double acc[POTRF_SLOTS];
#pragma unroll
  for (int s = 0; s < POTRF_SLOTS; ++s)
    if (potrf_slot_owner(s) == W)
      acc[s] = s < POTRF_FULL ? S[lane * LDS + potrf_slot_col(s)] : S[prow * LDS + potrf_slot_col(s) + half];
#pragma unroll
  for (int j = 0; j < TS - 2; ++j) {
    nbar_sync(POTRF_BAR_L + (j & 7));
    const double wf = wring[j & 7][lane];   // w of this lane's row (full slots)
    const double wp = wring[j & 7][prow];   // w of the pair slots' row
#pragma unroll
    for (int s = 0; s < POTRF_SLOTS; ++s) {   // the look-ahead column j + 2 first
      if (potrf_slot_owner(s) != W) continue;
      if (s < POTRF_FULL && potrf_slot_col(s) == j + 2) {
        acc[s] = fma(-wf, S[(j + 2) * LDS + j], acc[s]);
        S[lane * LDS + j + 2] = acc[s];
        nbar_arrive_n<64>(POTRF_BAR_C + (j & 3));
      } else if (s >= POTRF_FULL && (potrf_slot_col(s) == j + 2 || potrf_slot_col(s) + 1 == j + 2)) {
        acc[s] = fma(-wp, S[(potrf_slot_col(s) + half) * LDS + j], acc[s]);
        if (potrf_slot_col(s) + half == j + 2) S[prow * LDS + j + 2] = acc[s];
        nbar_arrive_n<64>(POTRF_BAR_C + (j & 3));
      }
    }
#pragma unroll
    for (int s = 0; s < POTRF_SLOTS; ++s) {
      if (potrf_slot_owner(s) != W || potrf_slot_last(s) <= j + 2) continue;
      if (s < POTRF_FULL) acc[s] = fma(-wf, S[potrf_slot_col(s) * LDS + j], acc[s]);
      else if (potrf_slot_col(s) > j + 2) acc[s] = fma(-wp, S[(potrf_slot_col(s) + half) * LDS + j], acc[s]);
    }
  }
}

// In-place lower Cholesky of S (TS x TS; entries past n must already be identity).
// Returns 0, or the 1-based column of the first non-positive (or NaN) pivot (the
// tile then holds NaNs).  The strict upper triangle is zeroed.
// The elimination runs in the square-root-free form S = U D^-1 U^T (u_rk: column k
// after pivots 0..k-1, d_k = u_kk), and L = U D^{-1/2} is formed at the end, all
// columns at once.  Warp 0 does nothing but the pivot chain: for pivot k it takes
// column k, already updated through pivot k-2 by its owner (awaited and loaded while
// pivot k-1's reciprocal was formed), applies pivot k-1 itself
// (it holds w_{:,k-1} = u_{:,k-1} / d_{k-1} in registers, the multiplier u_{k,k-1} is
// one shuffle), stores u_{:,k} to S, forms 1/d_k and w_{:,k}, and hands w_{:,k} to the
// update warps through an eight-slot ring.  That is five FP64 instructions per pivot on
// the chain (GB300 issues one FP64 warp instruction per ~64 cycles on a sub-partition),
// against seven for l_rk = a_rk / sqrt(d_k) with a refined reciprocal square root.
// Warps 1-3 apply every pivot to the later columns (potrf_update_warp), the column that
// the pivot warp needs next first; each entry receives its updates in pivot order.
// Barrier ids rotate over 8 (pivots) and 4 (look-ahead columns): before the pivot warp
// publishes pivot p+8 (and overwrites ring slot p & 7), each update warp has handed it
// one of columns p+2 .. p+8 (seven consecutive columns have all three owners) and so
// consumed pivot p; the pivot warp consumes look-ahead column p before it can publish
// the pivot that look-ahead column p+4 needs.
static __device__ int smem_potrf(double* S) {
  __shared__ int s_info;
  __shared__ double s_wring[8][TS];
  __shared__ double s_y[TS];
  const int r = threadIdx.x & 31, g = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_info = TS + 1;
  __syncthreads();
  if (g == 0) {
    const double u0 = S[r * LDS];       // column 0 of U is column 0 of S
    const double a1 = S[r * LDS + 1];   // column 1 takes no update before pivot 0
    double dk = __shfl_sync(0xffffffffu, u0, 0);   // lane k keeps d_k
    if (r == 0 && !positive_bits(dk)) atomicMin(&s_info, 1);
    double wp = u0 * rcp3_fma(dk);
    s_wring[0][r] = wp;
    nbar_arrive(POTRF_BAR_L);
    double a = a1;
    double ub = __shfl_sync(0xffffffffu, u0, 1);   // u_{1,0}
#pragma unroll
    for (int k = 1; k < TS; ++k) {
      a = fma(-wp, ub, a);   // column k through pivot k-1
      const double u = (r >= k) ? a : 0.0;
      const double d = __shfl_sync(0xffffffffu, a, k);
      if (r == k) dk = d;
      S[r * LDS + k] = u;
      if (r == 0 && !positive_bits(d)) atomicMin(&s_info, k + 1);
      if (k < TS - 1) {
        const double sk = rcp3_fma(d);
        // Column k+1, updated through pivot k-1 by its owner, is awaited and loaded
        // while this pivot's reciprocal is formed, off the chain.
        nbar_sync_n<64>(POTRF_BAR_C + ((k - 1) & 3));
        const double an = S[r * LDS + k + 1];
        const double w = u * sk;
        ub = __shfl_sync(0xffffffffu, u, k + 1);   // u_{k+1,k}
        if (k < TS - 2) {
          s_wring[k & 7][r] = w;
          nbar_arrive(POTRF_BAR_L + (k & 7));
        }
        wp = w;
        a = an;
      }
    }
    s_y[r] = rsqrt3(dk);
  } else if (g == 1) {
    potrf_update_warp<0>(S, s_wring, r);
  } else if (g == 2) {
    potrf_update_warp<1>(S, s_wring, r);
  } else {
    potrf_update_warp<2>(S, s_wring, r);
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < 8; ++q) {   // L = U D^{-1/2}: warp g scales columns g + 4q
    const int cc = g + 4 * q;
    S[r * LDS + cc] *= s_y[cc];
  }
  __syncthreads();
  const int info = s_info;
  __syncthreads();
  return info > TS ? 0 : info;
}

// X <- X * F^{-T} with F lower triangular; rd = 1/diag(F) (tile_diag_recip).  Row r
// solves x_r F^T = X_r by forward substitution over the columns.
static __device__ void smem_trsm_rlt(double* X, const double* F, const double* rd) {
  __shared__ double xs[2 * TS];
  const int r = threadIdx.x & 31, g = threadIdx.x >> 5;
  __syncthreads();
  double acc[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) acc[q] = X[r * LDS + g + 4 * q];
#pragma unroll
  for (int j = 0; j < TS; ++j) {
    double* xb = xs + (j & 1) * TS;
    if (g == (j & 3)) {
      const double x = acc[j >> 2] * rd[j];
      acc[j >> 2] = x;
      xb[r] = x;
    }
    __syncthreads();
    const double xr = xb[r];
#pragma unroll
    for (int q = 0; q < 8; ++q)
      if (col_after(q, j, g)) acc[q] = fma(-xr, F[(g + 4 * q) * LDS + j], acc[q]);
  }
#pragma unroll
  for (int q = 0; q < 8; ++q) X[r * LDS + g + 4 * q] = acc[q];
  __syncthreads();
}

// Rows row0 .. row0 + 7 of X <- X * F^{-T} (F lower triangular, identity padded).
// Warp w solves rows row0 + 2w and row0 + 2w + 1: lane l holds columns (l & 15) and
// (l & 15) + 16 of row row0 + 2w + (l >> 4).  Column j is finished on the lane that
// holds it and broadcast to its row's 16 lanes with one shuffle, so the sweep needs no
// barrier; the later columns are updated with one FMA each.  With FS (a copy of F
// whose row j is scaled by 1/F_jj, see tile_scale_rows_by_recip) and X's columns
// pre-scaled the same way, no multiplication is left on the column chain.
static __device__ void smem_trsm_rlt_rows8(double* X, const double* FS, const double* rd, int row0) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int row = row0 + 2 * w + (lane >> 4), cg = lane & 15, base = lane & 16;
  __syncthreads();
  double a0 = X[row * LDS + cg] * rd[cg], a1 = X[row * LDS + cg + 16] * rd[cg + 16];
#pragma unroll
  for (int j = 0; j < TS; ++j) {
    const double xj = __shfl_sync(0xffffffffu, j < 16 ? a0 : a1, base | (j & 15));
    if (j < 15) {
      const double f0 = FS[cg * LDS + j];
      if (cg > j) a0 = fma(-xj, f0, a0);
    }
    const double f1 = FS[(cg + 16) * LDS + j];
    if (j < 16 || cg + 16 > j) a1 = fma(-xj, f1, a1);
  }
  __syncthreads();
  X[row * LDS + cg] = a0;
  X[row * LDS + cg + 16] = a1;
  __syncthreads();
}

// FS <- F with row j scaled by rd[j] = 1/F_jj (the strict lower part is what the
// row solves read).  Caller syncs before and after.
__device__ __forceinline__ void tile_scale_rows_by_recip(double* FS, const double* F, const double* rd) {
#pragma unroll
  for (int k = 0; k < PER_THREAD; ++k) {
    const int idx = threadIdx.x + k * NT;
    const int r = idx / TS, c = idx % TS;
    FS[r * LDS + c] = F[r * LDS + c] * rd[r];
  }
}

// X <- X * F^{-1} with F lower triangular; rd = 1/diag(F).  Row r solves x_r F = X_r
// by backward substitution over the columns.
static __device__ void smem_trsm_rln(double* X, const double* F, const double* rd) {
  __shared__ double xs[2 * TS];
  const int r = threadIdx.x & 31, g = threadIdx.x >> 5;
  __syncthreads();
  double acc[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) acc[q] = X[r * LDS + g + 4 * q];
#pragma unroll
  for (int j = TS - 1; j >= 0; --j) {
    double* xb = xs + (j & 1) * TS;
    if (g == (j & 3)) {
      const double x = acc[j >> 2] * rd[j];
      acc[j >> 2] = x;
      xb[r] = x;
    }
    __syncthreads();
    const double xr = xb[r];
#pragma unroll
    for (int q = 0; q < 8; ++q)
      if (col_before(q, j, g)) acc[q] = fma(-xr, F[j * LDS + g + 4 * q], acc[q]);
  }
#pragma unroll
  for (int q = 0; q < 8; ++q) X[r * LDS + g + 4 * q] = acc[q];
  __syncthreads();
}

}  // namespace gbta
