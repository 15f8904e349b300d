// Per-task bodies of the BTA selected inversion, shared by the single-instance kernels
// (bta_selinv.cu, bta_selinv_oz.cu) and the multi-instance kernel (bta_batch.cu).
//
// Replaces the backward block recurrence the reference runs through Serinv
// (src/pyinla/solvers/structured_solver.py:176-186), which overwrites the factor
// blocks with Sigma = Q^{-1} on the BTA pattern.  Here the recurrence is taken to
// tile level.  With F the (tile-banded) Cholesky factor, Sigma F = F^{-T} gives for
// tile column k and its below-diagonal pattern P_k:
//   Sigma(j,k) = -( sum_{l in P_k} Sigma(j,l) F(l,k) ) F(k,k)^{-1}      (j in P_k)
//   Sigma(k,k) =  ( F(k,k)^{-T} - sum_{l in P_k} Sigma(l,k)^T F(l,k) ) F(k,k)^{-1}
// The factor is fixed during the inversion, so a pre-pass (launch_selinv_prepare)
// forms, off the critical path, G(l,k) = F(l,k) F(k,k)^{-1} in place of every pattern
// tile and C_k = F(k,k)^{-T} F(k,k)^{-1} per diagonal tile; then
//   Sigma(j,k) = -sum_l Sigma(j,l) G(l,k),   Sigma(k,k) = C_k - sum_l Sigma(l,k)^T G(l,k)
// and no task ends in a triangular solve.
// P_k of tile column c of block i is: tiles of D_i below c, all tiles of block i's
// coupling slot lslot(i) (block row nxt(i), the neighbour eliminated after i; see Geom)
// and the arrow tile.  Every Sigma(j,l) needed lies in a column eliminated later, so
// tasks run column by column in reverse elimination order: the tip, the separator
// block, then the two chains outwards; a task of column k starts its products while
// the column before it is still finishing.  Sigma of a coupling slot below the
// separator is produced as Sigma(j, j+1) and transposed by the write-back.
//
// Sigma is written to a separate workspace (the factor tiles F(l,k) of a column are
// read by all tasks of that column) and copied back into the caller's buffers by
// launch_selinv_writeback, which also mirrors D_i and T to full symmetric blocks.
//
// Two ways to compute the product loops (SelinvArgs::method):
//  * FP64: FP64 FMAs on staged FP64 tiles (selinv_fp64_task);
//  * OZAKI: tensor-core digit-plane products (selinv_oz_task, see bta_ozaki.cuh):
//    the right operand F(l,c) is fixed during the inversion, so every factor tile is
//    sliced once (k_fac_digits_t) relative to per-column exponents
//    (k_fac_col_exponents: max over the column's pattern) and stored transposed for
//    the ldmatrix layout; every Sigma tile is sliced once, by the task that produces
//    it, against its own exponent (a multiple of 7), and its consumers stage those
//    planes shifted to the task's running exponent E (the largest tile exponent seen
//    so far in the task); when a tile raises E, the exact partial sums are first
//    folded into FP64 with the old E.  Tile inverses and triangular solves stay in FP64.
#pragma once

#include "bta_ozaki.cuh"

namespace gbta {

// Arguments of one selected-inversion instance (both product methods).
struct SelinvArgs {
  const double* D;
  const double* L;
  const double* R;
  const double* T;
  double* SD;
  double* SL;
  double* SR;
  double* ST;
  Geom g;
  int use_arrow;
  int method;           // GBTA_METHOD_FP64 / GBTA_METHOD_OZAKI
  const int4* tasks;
  int ntasks;
  const __half* fdig;   // Ozaki: transposed digits of the G tiles per flag slot
  const int* fdz;       // Ozaki: leading zero digit planes of each G tile (per flag slot; 8 =
                        // zero tile), or null; steps with a zero G tile are dropped
  const int* ecol;      // Ozaki: per global column (nt*b) exponent of the G column pattern
  const double* cinv;   // [nt*B][TS*TS]: F_cc^{-T} F_cc^{-1} of every diagonal factor tile
  __half* sdig;         // Ozaki: digit planes of every Sigma tile per flag slot (their
                        // exponents ride in the tiles' flag words, see sig_exp_code)
  double* part;         // Ozaki, merged task list: [nt*B][TS*TS] partial sums of the
  int* part_flag;       // sub-diagonal tiles and their epoch-stamped flags [nt*B]
  int merged;           // the task list is selinv_task_list(g, true)
  Ctl c;
};

// Row descriptor of a tile row in the pattern of column (i, c):
//   code in [0, B): block i row tile; [B, 2B): block nxt(i) row tile; 2B: arrow.
struct SigTile {
  Tile t;
  bool trans;
  const int* flag;
};

static __device__ __forceinline__ int rows_of(const Geom& g, int code) {
  return code == 2 * g.B ? g.a : g.vrows(code % g.B);
}

// Sigma tile at (row j, col l) of the global matrix, both given as row codes
// relative to block column i.  Stored in lower storage; trans = stored transposed.
static __device__ SigTile sig_tile(const SelinvArgs& p, int i, int j, int l) {
  const Geom& g = p.g;
  const int B = g.B, A = 2 * B;
  const size_t bb = (size_t)g.b * g.b, ab = (size_t)g.a * g.b;
  const int* F = p.c.flags;
  SigTile s;
  auto dtile = [&](int blk, int r, int c) {   // lower tile of SD[blk]
    return make_tile(p.SD + blk * bb, g.b, r * TS, c * TS, g.b, g.b);
  };
  if (j == A && l == A) {
    s.t = make_tile(p.ST, g.a, 0, 0, g.a, g.a);
    s.trans = false;
    s.flag = F + g.fT();
  } else if (j == A || l == A) {
    const int other = (j == A) ? l : j;
    const int blk = other < B ? i : g.nxt(i);
    const int r = other % B;
    s.t = make_tile(p.SR + blk * ab, g.b, 0, r * TS, g.a, g.b);
    s.trans = (l == A);
    s.flag = F + g.fR(blk, r);
  } else if (j < B && l < B) {   // both in block i
    const int hi = max(j, l), lo = min(j, l);
    s.t = dtile(i, hi, lo);
    s.trans = j < l;
    s.flag = F + g.fD(i, hi, lo);
  } else if (j >= B && l >= B) {   // both in block nxt(i)
    const int hi = max(j, l) - B, lo = min(j, l) - B, nx = g.nxt(i);
    s.t = dtile(nx, hi, lo);
    s.trans = j < l;
    s.flag = F + g.fD(nx, hi, lo);
  } else {   // one in block nxt(i) (rows of the coupling slot), one in block i (its cols)
    const int rl = (j >= B ? j : l) - B, cd = (j >= B ? l : j), ls = g.lslot(i);
    s.t = make_tile(p.SL + ls * bb, g.b, rl * TS, cd * TS, g.b, g.b);
    s.trans = j < B;
    s.flag = F + g.fL(ls, rl, cd);
  }
  return s;
}

// Factor tile F(l, c) of block column i (l a row code); no wait needed.
static __device__ __forceinline__ Tile fac_tile(const SelinvArgs& p, int i, int l, int c) {
  const Geom& g = p.g;
  const size_t bb = (size_t)g.b * g.b, ab = (size_t)g.a * g.b;
  const int B = g.B;
  if (l == 2 * B) return make_tile(p.R + i * ab, g.b, 0, c * TS, g.a, g.b);
  if (l >= B) return make_tile(p.L + g.lslot(i) * bb, g.b, (l - B) * TS, c * TS, g.b, g.b);
  return make_tile(p.D + i * bb, g.b, l * TS, c * TS, g.b, g.b);
}

// Destination of Sigma(j, c) (j a row code of column (i, c)).
static __device__ __forceinline__ SigTile sig_dest(const SelinvArgs& p, int i, int j, int c) {
  const Geom& g = p.g;
  const size_t bb = (size_t)g.b * g.b, ab = (size_t)g.a * g.b;
  const int B = g.B;
  SigTile s;
  s.trans = false;
  if (j == 2 * B) {
    s.t = make_tile(p.SR + i * ab, g.b, 0, c * TS, g.a, g.b);
    s.flag = p.c.flags + g.fR(i, c);
  } else if (j >= B) {
    s.t = make_tile(p.SL + g.lslot(i) * bb, g.b, (j - B) * TS, c * TS, g.b, g.b);
    s.flag = p.c.flags + g.fL(g.lslot(i), j - B, c);
  } else {
    s.t = make_tile(p.SD + i * bb, g.b, j * TS, c * TS, g.b, g.b);
    s.flag = p.c.flags + g.fD(i, j, c);
  }
  return s;
}

// Pattern of column (i, c), ordered so that the most recently produced Sigma tiles
// come last: arrow, block nxt(i) rows descending, block i rows descending (> c).
static __device__ __forceinline__ int pat_size(const SelinvArgs& p, int i, int c) {
  const Geom& g = p.g;
  return (p.use_arrow ? 1 : 0) + (g.nxt(i) >= 0 ? g.B : 0) + (g.B - 1 - c);
}
static __device__ __forceinline__ int pat_code(const SelinvArgs& p, int i, int c, int s) {
  const Geom& g = p.g;
  if (p.use_arrow) {
    if (s == 0) return 2 * g.B;
    --s;
  }
  if (g.nxt(i) >= 0) {
    if (s < g.B) return 2 * g.B - 1 - s;
    s -= g.B;
  }
  return g.B - 1 - s;
}

// X <- (F^{-T} - X) F^{-1} (diagonal tile of Sigma), then symmetrise; rd = 1/diag(F).
static __device__ void diag_finish(double* X, double* W, const double* F, const double* rd) {
  // W = I * F^{-T}
  for (int idx = threadIdx.x; idx < TS * TS; idx += NT) {
    const int r = idx / TS, cc = idx % TS;
    W[r * LDS + cc] = (r == cc) ? 1.0 : 0.0;
  }
  smem_trsm_rlt(W, F, rd);
  for (int idx = threadIdx.x; idx < TS * TS; idx += NT) {
    const int r = idx / TS, cc = idx % TS;
    W[r * LDS + cc] -= X[r * LDS + cc];
  }
  smem_trsm_rln(W, F, rd);
  for (int idx = threadIdx.x; idx < TS * TS; idx += NT) {
    const int r = idx / TS, cc = idx % TS;
    X[r * LDS + cc] = 0.5 * (W[r * LDS + cc] + W[cc * LDS + r]);
  }
  __syncthreads();
}

// X <- C + X, symmetrised (C = F^{-T} F^{-1} of the diagonal factor tile, X = -Z).
static __device__ void diag_from_cinv(double* X, const double* C) {
  double v[PER_THREAD];
#pragma unroll
  for (int k = 0; k < PER_THREAD; ++k) {
    const int idx = threadIdx.x + k * NT;
    const int r = idx / TS, cc = idx % TS;
    v[k] = 0.5 * ((C[r * LDS + cc] + X[r * LDS + cc]) + (C[cc * LDS + r] + X[cc * LDS + r]));
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < PER_THREAD; ++k) {
    const int idx = threadIdx.x + k * NT;
    X[(idx / TS) * LDS + idx % TS] = v[k];
  }
  __syncthreads();
}

// Shared memory of the FP64 selected-inversion task: 4 tiles (K-loop double buffer;
// X, F, W alias its first three) and the TS reciprocals of the diagonal factor tile.
constexpr size_t FP64S_SMEM = 4 * TILE_SMEM * sizeof(double) + TS * sizeof(double);

// Task t of a FP64-product selected-inversion instance.  `raw` is FP64S_SMEM bytes of
// shared memory.  Returns false when the launch is aborted.
static __device__ __forceinline__ bool selinv_fp64_task(const SelinvArgs& p, int t, unsigned char* raw, int* s_okp) {
  double* sm = reinterpret_cast<double*>(raw);
  double* rd = sm + 4 * TILE_SMEM;
  double* bufs = sm;
  double* X = sm;
  double* F = sm + TILE_SMEM;
  double* W = sm + 2 * TILE_SMEM;
  int& s_ok = *s_okp;
  const Geom& g = p.g;
  const Ctl& c = p.c;
  {
    const unsigned long long t_task0 = c.trace ? gtimer() : 0ull;
    const int4 tk = p.tasks[t];
    const int type = tk.x, i = tk.y, j = tk.z, col = tk.w;
    if (!p.use_arrow && (type == ST_TIP || (type == ST_OFF && j == 2 * g.B))) return true;

    if (type == ST_TIP) {
      // Sigma_T = T^{-T} T^{-1} from the tip factor.
      tile_load(F, make_tile(p.T, g.a, 0, 0, g.a, g.a));
      __syncthreads();
      tile_pad_identity(F, g.a);
      for (int idx = threadIdx.x; idx < TS * TS; idx += NT) X[idx / TS * LDS + idx % TS] = 0.0;
      __syncthreads();
      tile_diag_recip(F, rd);
      __syncthreads();
      diag_finish(X, W, F, rd);
      tile_store(p.ST, g.a, g.a, g.a, X);
      cta_publish(c, c.flags + g.fT());
      trace_task(c, t, type, t_task0);
      return true;
    }

    const int np = pat_size(p, i, col);
    Acc acc;
    acc_zero(acc);
    if (type == ST_OFF) {
      // Sigma(j,col) = -sum_l Sigma(j,l) G(l,col)
      auto step_of = [&](int s) -> Step {
        const int l = pat_code(p, i, col, s);
        const SigTile st_ = sig_tile(p, i, j, l);
        Step st;
        st.a = st_.t;
        st.ta = st_.trans;
        st.fa = st_.flag;
        st.b = fac_tile(p, i, l, col);
        st.tb = false;
        st.fb = nullptr;
        return st;
      };
      if (!kloop<true>(acc, np, step_of, c, bufs, &s_ok)) return false;   // acc = -Y = Sigma(j,col)
      acc_to_smem(acc, X);
      __syncthreads();
      const SigTile d = sig_dest(p, i, j, col);
      tile_store(const_cast<double*>(d.t.p), d.t.ld, d.t.rows, d.t.cols, X);
      cta_publish(c, const_cast<int*>(d.flag));
      trace_task(c, t, type, t_task0);
    } else {   // ST_DIAG
      // Z = sum_l Sigma(l,col)^T G(l,col); Sigma(col,col) = F^{-T} F^{-1} - Z
      auto step_of = [&](int s) -> Step {
        const int l = pat_code(p, i, col, s);
        const SigTile st_ = sig_dest(p, i, l, col);
        Step st;
        st.a = st_.t;
        st.ta = true;
        st.fa = st_.flag;
        st.b = fac_tile(p, i, l, col);
        st.tb = false;
        st.fb = nullptr;
        return st;
      };
      if (!kloop<true>(acc, np, step_of, c, bufs, &s_ok)) return false;   // acc = -Z
      acc_to_smem(acc, X);
      tile_load(F, make_tile(p.cinv + (size_t)(i * g.B + col) * TS * TS, TS, 0, 0, TS, TS));
      __syncthreads();
      diag_from_cinv(X, F);
      const SigTile d = sig_dest(p, i, col, col);
      tile_store(const_cast<double*>(d.t.p), d.t.ld, d.t.rows, d.t.cols, X);
      cta_publish(c, const_cast<int*>(d.flag));
      trace_task(c, t, type, t_task0);
    }
  }
  return true;
}

// flag slot of the factor tile F(l, c) of block column i
static __device__ __forceinline__ int fac_slot(const Geom& g, int i, int l, int c) {
  const int B = g.B;
  if (l == 2 * B) return g.fR(i, c);
  if (l >= B) return g.fL(g.lslot(i), l - B, c);
  return g.fD(i, l, c);
}
// Exponent value of an all-zero tile.
constexpr int NO_EXP = -100000;

// Exponent of the valid part of a shared tile for its Sigma digit planes: the smallest
// multiple of 7 with |x| < 2^E (so that tiles of one product loop differ by whole
// planes), or NO_EXP for an all-zero tile.  Integer max of the magnitude bits.
static __device__ __forceinline__ int smem_tile_exponent7(const double* X, int rows, int cols, double* red4) {
  unsigned long long m = 0;
#pragma unroll
  for (int k = 0; k < PER_THREAD; ++k) {
    const int idx = threadIdx.x + k * NT;
    const int r = idx / TS, cc = idx % TS;
    if (r < rows && cc < cols) {
      const unsigned long long a = (unsigned long long)__double_as_longlong(X[r * LDS + cc]) & 0x7fffffffffffffffull;
      m = a > m ? a : m;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_xor_sync(0xffffffffu, m, o);
    m = x > m ? x : m;
  }
  unsigned long long* red = reinterpret_cast<unsigned long long*>(red4);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  unsigned long long r = red[0];
#pragma unroll
  for (int w = 1; w < NT / 32; ++w) r = red[w] > r ? red[w] : r;
  __syncthreads();
  if (!r) return NO_EXP;
  const int e = ilogb_bits(r) + 1;   // |x| < 2^e
  return e >= 0 ? 7 * ((e + 6) / 7) : -7 * ((-e) / 7);
}

// The same exponent for a tile held in the OzAcc register layout (v), valid part rows x
// cols.  Writes red (NT / 32 words) and contains one __syncthreads(): the caller's
// earlier reads of red must be behind a barrier, and shared-memory writes made before
// the call are visible to every thread after it.
static __device__ __forceinline__ int acc_tile_exponent7(const double (&v)[2][4], int rows, int cols,
                                                         unsigned long long* red) {
  unsigned long long m = 0;
#pragma unroll
  for (int n = 0; n < 2; ++n)
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (oz_row(n, q) < rows && oz_col(n, q) < cols) {
        const unsigned long long a = (unsigned long long)__double_as_longlong(v[n][q]) & 0x7fffffffffffffffull;
        m = a > m ? a : m;
      }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_xor_sync(0xffffffffu, m, o);
    m = x > m ? x : m;
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  unsigned long long r = red[0];
#pragma unroll
  for (int w = 1; w < NT / 32; ++w) r = red[w] > r ? red[w] : r;
  if (!r) return NO_EXP;
  const int e = ilogb_bits(r) + 1;   // |x| < 2^e
  return e >= 0 ? 7 * ((e + 6) / 7) : -7 * ((-e) / 7);
}

// A Sigma tile's exponent (a multiple of 7 in [-1071, 1029], or NO_EXP) as the payload
// of its flag word (below 2^EPOCH_SHIFT), and back.
static __device__ __forceinline__ int sig_exp_code(int E) { return E == NO_EXP ? 0 : E / 7 + 256; }
static __device__ __forceinline__ int sig_exp_decode(int flag_word, int epoch) {
  const int code = flag_word - epoch;
  return code ? (code - 256) * 7 : NO_EXP;
}

// Digit planes of a finished Sigma tile (shared X, rows x cols valid), written to its
// slot before the tile is published; returns the flag payload of its exponent.
static __device__ __forceinline__ int sig_store_digits(const SelinvArgs& p, int slot, const double* X, int rows,
                                                       int cols, double* red4) {
  const int E = smem_tile_exponent7(X, rows, cols, red4);
  oz_store_digits_uniform(p.sdig + (size_t)slot * OZ_TILE, X, rows, cols, E == NO_EXP ? 0 : E);
  return sig_exp_code(E);
}

// Plane shift of a left operand with exponent En in the frame of the running
// exponent E >= En (both multiples of 7, or NO_EXP): OZ_S drops the whole tile.
static __device__ __forceinline__ int sig_shift(int E, int En) {
  if (En == NO_EXP) return E == NO_EXP ? 0 : OZ_S;
  const int q = (E - En) / 7;
  return q < OZ_S ? q : OZ_S;
}

// OZS_STAGE: halves per stage (A, B digit planes), two stages.  The FP64 tiles of the
// epilogues live in the stages, used only when no copy is in flight: X, F and the
// merged finish's X2 in the second, W (the tip task) and the merged finish's digit
// planes in the first.  That keeps a CTA at 67 KB, so that three fit on an SM (with
// the 168 registers of k_selinv_oz's launch bounds).
constexpr int OZS_STAGE = 2 * OZ_OPER;
static_assert(3 * TILE_SMEM * sizeof(double) <= OZS_STAGE * sizeof(__half), "X, F and X2 fit in a stage");
// Step descriptors of a task's product loop, computed once per task (larger loops
// compute the rest on the fly): left tile slot << 1 | transposed, right tile slot.
// 256 cover the loops of blocks up to 4096 rows (at most 2 B steps).
constexpr int OZS_DESC = 256;
constexpr size_t OZS_SMEM = 2 * OZS_STAGE * sizeof(__half) + TS * sizeof(double) + TS * sizeof(int) +
                            4 * sizeof(double) + (SCAN_RING + 2) * sizeof(int) + OZS_DESC * sizeof(int2);
constexpr int OZS_CTAS_PER_SM = 3;
static_assert(OZS_CTAS_PER_SM * (OZS_SMEM + 2048) <= 228 * 1024, "three CTAs per SM");

// Task t of a tensor-core selected-inversion instance.  `raw` is OZS_SMEM bytes of
// (16-byte aligned) shared memory.  Returns false when the launch is aborted.
//
// Both operands arrive as digit planes: the right one (G) sliced by the pre-pass, the
// left one (a Sigma tile) sliced once by the task that produced it, against its own
// exponent E_t (a multiple of 7).  The product loop keeps a running exponent E (the
// largest E_t so far) and stages each left tile shifted down by (E - E_t) / 7 planes;
// a tile that raises E first folds the exact partial sums with the old E.
static __device__ __forceinline__ bool selinv_oz_task(const SelinvArgs& p, int t, unsigned char* raw, int* s_okp,
                                                      int* s_readyp, OzPipe* pp) {
  __half* stages = reinterpret_cast<__half*>(raw);
  double* X = reinterpret_cast<double*>(raw + OZS_STAGE * sizeof(__half));   // stage 1
  double* F = X + TILE_SMEM;                                                 // stage 1
  double* W = reinterpret_cast<double*>(raw);   // stage 0 (the tip task)
  double* rd = reinterpret_cast<double*>(raw + 2 * OZS_STAGE * sizeof(__half));
  int* ecol_t = reinterpret_cast<int*>(rd + TS);
  double* red4 = reinterpret_cast<double*>(ecol_t + TS);
  int* ring = reinterpret_cast<int*>(red4 + 4);   // flag words of the steps found ready
  int* s_val = ring + SCAN_RING;                  // flag word of the last blocking wait
  int2* sdesc = reinterpret_cast<int2*>(ring + SCAN_RING + 2);   // step descriptors (8-byte aligned)
  int& s_ok = *s_okp;
  int& s_ready = *s_readyp;
  const Geom& g = p.g;
  const Ctl& c = p.c;
  {
    const unsigned long long t_task0 = c.trace ? gtimer() : 0ull;
    const int4 tk = p.tasks[t];
    const int type = tk.x, i = tk.y, j = tk.z, col = tk.w;
    if (!p.use_arrow && (type == ST_TIP || (type == ST_OFF && j == 2 * g.B))) return true;

    if (type == ST_TIP) {
      tile_load(F, make_tile(p.T, g.a, 0, 0, g.a, g.a));
      __syncthreads();
      tile_pad_identity(F, g.a);
      for (int idx = threadIdx.x; idx < TS * TS; idx += NT) X[idx / TS * LDS + idx % TS] = 0.0;
      __syncthreads();
      tile_diag_recip(F, rd);
      __syncthreads();
      diag_finish(X, W, F, rd);
      tile_store(p.ST, g.a, g.a, g.a, X);
      const int code = sig_store_digits(p, g.fT(), X, g.a, g.a, red4);
      cta_publish_val(c, c.flags + g.fT(), code);
      trace_task(c, t, type, t_task0);
      return true;
    }

    // a partial task (ST_PART) leaves out its last step: the diagonal tile j itself
    int np = pat_size(p, i, col) - (type == ST_PART ? 1 : 0);
    if (threadIdx.x < TS) {
      const int cc = col * TS + threadIdx.x;
      ecol_t[threadIdx.x] = cc < g.b ? p.ecol[(size_t)i * g.b + cc] : 0;
    }
    __syncthreads();
    // ST_OFF / ST_PART: acc.v = -(sum of the products) = Sigma(j, col) (or its partial);
    // ST_DIAG starts from C_col = F^{-T} F^{-1} (identity-padded): acc.v = C_col - Z =
    // Sigma(col, col), symmetrised after the loop
    OzAcc acc;
    oz_clear_partials(acc);
    {
      const double* cinv_t = p.cinv + (size_t)(i * g.B + col) * TS * TS;
#pragma unroll
      for (int n = 0; n < 2; ++n)
#pragma unroll
        for (int q = 0; q < 4; ++q)
          acc.v[n][q] = type == ST_DIAG ? __ldcg(cinv_t + oz_row(n, q) * TS + oz_col(n, q)) : 0.0;
    }
    int E = NO_EXP;   // running exponent of the left operand (unset)
    int esum[2][4];
    auto set_esum = [&]() {
#pragma unroll
      for (int n = 0; n < 2; ++n)
#pragma unroll
        for (int q = 0; q < 4; ++q) esum[n][q] = E + ecol_t[oz_col(n, q)];
    };
    // step s: left tile (Sigma digits, its flag slot and orientation) and right tile
    // (G digits), as a descriptor (left slot << 1 | transposed, right slot | the right
    // tile's leading zero planes << 24)
    auto compute_desc = [&](int s) -> int2 {
      const int l = pat_code(p, i, col, s);
      int slot;
      bool tr;
      if (type == ST_OFF || type == ST_PART) {
        const SigTile st_ = sig_tile(p, i, j, l);
        slot = (int)(st_.flag - c.flags);
        tr = st_.trans;
      } else {   // Sigma(l, col), used transposed
        slot = (int)(sig_dest(p, i, l, col).flag - c.flags);
        tr = true;
      }
      const int rs = fac_slot(g, i, l, col);
      return make_int2((slot << 1) | (tr ? 1 : 0), rs | ((p.fdz ? p.fdz[rs] : 0) << 24));
    };
    for (int s = threadIdx.x; s < np && s < OZS_DESC; s += NT) sdesc[s] = compute_desc(s);
    __syncthreads();
    // Steps whose right tile is zero contribute nothing: drop them up front (in order,
    // by warp 0), so their left tiles are not even waited for.
    const int np_all = np;
    if (p.fdz && np <= OZS_DESC) {
      if (threadIdx.x < 32) {
        int cnt = 0;
        for (int base = 0; base < np; base += 32) {
          const int s = base + threadIdx.x;
          const int2 d = s < np ? sdesc[s] : make_int2(0, OZ_S << 24);
          const bool live = (d.y >> 24) < OZ_S;
          const unsigned m = __ballot_sync(0xffffffffu, live);
          __syncwarp();
          if (live) sdesc[cnt + __popc(m & ((1u << threadIdx.x) - 1u))] = d;
          cnt += __popc(m);
          __syncwarp();
        }
        if (threadIdx.x == 0) s_val[1] = cnt;
      }
      __syncthreads();
      np = s_val[1];
    }
    auto desc_of = [&](int s) -> int2 { return np_all <= OZS_DESC ? sdesc[s] : compute_desc(s); };
    auto left_of = [&](int s) -> SigTile {
      const int2 d = desc_of(s);
      SigTile st_;
      st_.flag = c.flags + (d.x >> 1);
      st_.trans = (d.x & 1) != 0;
      return st_;
    };
    auto right_of = [&](int s) -> const __half* { return p.fdig + (size_t)(desc_of(s).y & 0xffffff) * OZ_TILE; };
    auto zero_planes_of = [&](int s) -> int { return desc_of(s).y >> 24; };
    // stage step s's operands into stage buffer st with the left tile shifted by q
    // planes: bulk copies of its leading OZ_S - q planes and of the right tile, the
    // q planes below the shift zeroed by the CTA
    unsigned ph = pp->phase;
    int qst[2] = {0, 0};   // plane shift of the left tile in each stage buffer
    int zst[2] = {0, 0};   // leading zero planes of the right tile in each stage buffer
    auto stage = [&](int st, const SigTile& lt, int q, int s) {
      qst[st] = q;
      zst[st] = zero_planes_of(s);
      __half* dst = stages + st * OZS_STAGE;
      const int slot = (int)(lt.flag - c.flags);
      const unsigned abytes = q < OZ_S ? (unsigned)((OZ_S - q) * OZ_PLANE * sizeof(__half)) : 0u;
      if (threadIdx.x == 0) {
        oz_bulk_expect(pp, st, abytes + (unsigned)(OZ_TILE * sizeof(__half)));
        if (abytes) oz_bulk_copy(pp, st, dst + q * OZ_PLANE, p.sdig + (size_t)slot * OZ_TILE, abytes);
        oz_bulk_copy(pp, st, dst + OZ_OPER, right_of(s), (unsigned)(OZ_TILE * sizeof(__half)));
      }
      for (int idx = threadIdx.x; idx < q * (OZ_PLANE / 8); idx += NT)
        reinterpret_cast<uint4*>(dst)[idx] = make_uint4(0u, 0u, 0u, 0u);
      if (q) fence_async_smem();   // a later copy into this stage may cover these planes
    };
    // wait for stage st; a copy that never lands aborts the launch
    auto stage_wait = [&](int st) -> bool {
      const bool late = !oz_stage_wait(pp, st, ph);
      if (__syncthreads_or(late)) {
        if (threadIdx.x == 0) {
          atomicCAS(c.ctrl + CTRL_ERR, ERR_NONE, ERR_TIMEOUT);
          raise_abort(c);
        }
        oz_stage_wait(pp, st, ph);   // give the copy one more bounded wait before leaving
        return false;
      }
      return true;
    };

    bool ok = true;
    int since_fold = 0;
    unsigned long long npairs = 0;   // tile-pair products issued (thread 0's count is used)
    // trace marks: m0 first operand ready, m1 end of the last blocking wait in the
    // product loop, m2 ns spent in those waits, m3 product steps (a diagonal task
    // overwrites m2 and m3 with the times its product loop ended and it published the
    // next column's sub-diagonal tile)
    unsigned long long waited = 0;
    trace_clear_marks(c, t);
    auto flags_of = [&](int s, const int*& f0, const int*& f1) {
      f0 = left_of(s).flag;
      f1 = nullptr;
    };
    if (np > 0) {
      SigTile lt = left_of(0);
      ok = cta_wait_val(c, lt.flag, &s_ok, s_val);
      trace_mark(c, t, 0);
      bool tcur = lt.trans;
      if (ok) {
        if (threadIdx.x == 0) s_ready = 1;
        E = sig_exp_decode(*s_val, c.epoch);
        set_esum();
        stage(0, lt, 0, 0);
      }
      for (int s = 0; s < np && ok; ++s) {
        __half* cur = stages + (s & 1) * OZS_STAGE;
        const int nst = (s + 1) & 1;
        if (!(ok = stage_wait(s & 1))) break;   // contains the barrier that frees the other stage
        const bool more = s + 1 < np;
        bool have = false;
        SigTile nt_;
        int En = NO_EXP;
        if (more) {
          nt_ = left_of(s + 1);
          if (s_ready <= s + 1) {   // uniform: read after the barrier, rewritten after the next one
            __syncthreads();   // every warp has read s_ready before warp 0 advances it
            scan_ready(c, np, flags_of, &s_ready, ring);
            __syncthreads();
          }
          if (s_ready > s + 1) {
            En = sig_exp_decode(ring[(s + 1) % SCAN_RING], c.epoch);
            stage(nst, nt_, En > E ? 0 : sig_shift(E, En), s + 1);
            have = true;
          }
        }
        // the left tile was staged qcur planes down: its planes below qcur are zero
        // (all of them from OZ_S on: nothing to add)
        const int qcur = qst[s & 1], zcur = zst[s & 1];
        npairs += oz_pairs_issued(qcur, zcur);
        if (oz_pairs_vanish(qcur, zcur)) {
        } else if (tcur) {
          oz_step_z<true>(acc, cur, cur + OZ_OPER, qcur, zcur);
        } else {
          oz_step_z<false>(acc, cur, cur + OZ_OPER, qcur, zcur);
        }
        ++since_fold;
        if (more) {
          if (!have) {
            const unsigned long long w0 = c.trace ? gtimer() : 0ull;
            if (!(ok = cta_wait_val(c, nt_.flag, &s_ok, s_val))) break;
            if (c.trace) {
              waited += gtimer() - w0;
              trace_mark(c, t, 1);
            }
            if (threadIdx.x == 0) s_ready = s + 2;
            En = sig_exp_decode(*s_val, c.epoch);
          }
          if ((En > E && En != NO_EXP) || since_fold == OZ_CHUNK) {
            if (E > NO_EXP) oz_fold_sub_steps(acc, esum, since_fold);
            since_fold = 0;
            if (En > E && En != NO_EXP) {
              E = En;
              set_esum();
            }
          }
          if (!have) stage(nst, nt_, sig_shift(E, En), s + 1);
          tcur = nt_.trans;
        }
      }
    }
    if (!ok) return false;   // no copy is in flight here
    if (np > 0 && E > NO_EXP) oz_fold_sub_steps(acc, esum, since_fold);   // acc.v = -(sum)
    if (threadIdx.x == 0) pp->phase = ph;
    count_pairs(c, npairs);
    trace_put(c, t, 2, (long long)waited);
    trace_put(c, t, 3, np);
    __syncthreads();
    unsigned long long* red = reinterpret_cast<unsigned long long*>(red4);
    auto acc_to_x = [&](double* Y, const double (&v)[2][4]) {
#pragma unroll
      for (int n = 0; n < 2; ++n)
#pragma unroll
        for (int q = 0; q < 4; ++q) Y[oz_row(n, q) * LDS + oz_col(n, q)] = v[n][q];
    };
    // A finished Sigma tile leaves through its digit planes, which are all that the
    // inversion's consumers read: they are written and the tile published first, the
    // FP64 tile stored after (for the caller).
    if (type == ST_OFF) {
      const SigTile d = sig_dest(p, i, j, col);
      acc_to_x(X, acc.v);
      const int E = acc_tile_exponent7(acc.v, d.t.rows, d.t.cols, red);   // (its barrier covers X)
      oz_store_digits_uniform(p.sdig + (size_t)(d.flag - c.flags) * OZ_TILE, X, d.t.rows, d.t.cols,
                              E == NO_EXP ? 0 : E);
      cta_publish_val(c, const_cast<int*>(d.flag), sig_exp_code(E));
      tile_store(const_cast<double*>(d.t.p), d.t.ld, d.t.rows, d.t.cols, X);
    } else if (type == ST_PART) {   // the partial sum, for the diagonal task that finishes the tile
      acc_to_x(X, acc.v);
      __syncthreads();
      tile_store(p.part + (size_t)(i * g.B + col) * TS * TS, TS, TS, TS, X);
      cta_publish(c, p.part_flag + i * g.B + col);
    } else {
      trace_mark(c, t, 2);   // (diagonal task) product loop done
      const SigTile d = sig_dest(p, i, col, col);
      // The merged finish below (Sigma(j2, c2) of block column i2) reads its right tile's
      // digit planes, column exponents and zero-plane count from global memory: all three
      // are copied into shared memory asynchronously from here (stage 0 is free after the
      // loop), so that their latency passes under the symmetrisation instead of on the
      // column chain.
      // (the target's indices are recomputed after the symmetrisation rather than kept
      // live across it: the kernel runs at its register limit)
      auto merged_target = [&](int& i2, int& c2, int& j2) {
        i2 = col > 0 ? i : (g.nprev(i) == 1 ? g.prev(i, 0) : -1);
        c2 = col > 0 ? col - 1 : g.B - 1;
        j2 = col > 0 ? col : g.B;
        return p.merged && i2 >= 0;
      };
      int i2, c2, j2;
      if (merged_target(i2, c2, j2)) {
        oz_load_async(stages + OZ_OPER, p.fdig + (size_t)fac_slot(g, i2, j2, c2) * OZ_TILE);
        if (threadIdx.x < TS) {
          const int cc = c2 * TS + threadIdx.x;
          if (cc < g.b)
            cp_async4(ecol_t + threadIdx.x, p.ecol + (size_t)i2 * g.b + cc);
          else
            ecol_t[threadIdx.x] = 0;
        }
        if (threadIdx.x == 0) {   // (s_val[1] is free once the task has read its step count)
          if (p.fdz)
            cp_async4(s_val + 1, p.fdz + fac_slot(g, i2, j2, c2));
          else
            s_val[1] = 0;
        }
        cp_async_commit();
      }
      // symmetrise: the lower triangle mirrored into the upper one, through X (selects
      // only: no FP64 instruction on the chain)
      acc_to_x(X, acc.v);
      __syncthreads();
#pragma unroll
      for (int n = 0; n < 2; ++n)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int r = oz_row(n, q), cc = oz_col(n, q);
          if (r < cc) acc.v[n][q] = X[cc * LDS + r];
        }
      __syncthreads();
      acc_to_x(X, acc.v);
      const int Ed = acc_tile_exponent7(acc.v, d.t.rows, d.t.cols, red);   // (its barrier covers X)
      // Merged task list: this task also finishes the sub-diagonal tile of the next
      // column, Sigma(j2, c2) of block column i2, whose last product needs this tile:
      // Sigma(j2, c2) = partial - Sigma(col, col) G(j2, c2) (the tile is symmetric, so
      // it is its own left operand untransposed).  That tile is the next link of the
      // column chain, so it is published first; this tile's store, digits and flag
      // follow (its other consumers are later columns' products).  After column (i, 0)
      // the chain goes on in the one neighbour eliminated before i (none for the first
      // block of a chain; two for the separator, whose next tiles ordinary tasks form).
      if (merged_target(i2, c2, j2)) {
        __half* A0 = stages;   // stage 0: this tile's digits (no copy is in flight after the loop)
        __half* B0 = stages + OZ_OPER;   // (its copy was issued above)
        double* X2 = F + TILE_SMEM;   // stage 1, after X and F: Sigma(j2, c2)
        if (!cta_wait(c, p.part_flag + i2 * g.B + c2, nullptr, &s_ok)) return false;
        OzAcc a2;   // starts from the partial (its loads overlap the slicing below)
        oz_clear_partials(a2);
        {
          const double* P = p.part + (size_t)(i2 * g.B + c2) * TS * TS;
#pragma unroll
          for (int n = 0; n < 2; ++n)
#pragma unroll
            for (int q = 0; q < 4; ++q) a2.v[n][q] = __ldcg(P + oz_row(n, q) * TS + oz_col(n, q));
        }
        oz_store_digits_uniform(A0, X, d.t.rows, d.t.cols, Ed == NO_EXP ? 0 : Ed);
        cp_async_wait_all();
        __syncthreads();
        const int z2 = s_val[1];
        int es[2][4];
#pragma unroll
        for (int n = 0; n < 2; ++n)
#pragma unroll
          for (int q = 0; q < 4; ++q) es[n][q] = Ed + ecol_t[oz_col(n, q)];
        if (Ed > NO_EXP && !oz_pairs_vanish(0, z2)) {
          count_pairs(c, oz_pairs_issued(0, z2));
          oz_step_z<false>(a2, A0, B0, 0, z2);
          oz_fold_sub_short(a2, es);   // (one step)
        }
        const SigTile d2 = sig_dest(p, i2, j2, c2);
        acc_to_x(X2, a2.v);
        const int E2 = acc_tile_exponent7(a2.v, d2.t.rows, d2.t.cols, red);   // (its barrier covers X2)
        oz_store_digits_uniform(p.sdig + (size_t)(d2.flag - c.flags) * OZ_TILE, X2, d2.t.rows, d2.t.cols,
                                E2 == NO_EXP ? 0 : E2);
        cta_publish_val(c, const_cast<int*>(d2.flag), sig_exp_code(E2));
        trace_mark(c, t, 3);   // (diagonal task) next column's sub-diagonal tile published
        tile_store(const_cast<double*>(d2.t.p), d2.t.ld, d2.t.rows, d2.t.cols, X2);
        // this tile: its digits are the ones in A0
        {
          const uint4* src = reinterpret_cast<const uint4*>(A0);
          uint4* dst = reinterpret_cast<uint4*>(p.sdig + (size_t)(d.flag - c.flags) * OZ_TILE);
          for (int k = threadIdx.x; k < OZ_CHUNKS16; k += NT) dst[k] = src[k];
        }
        cta_publish_val(c, const_cast<int*>(d.flag), sig_exp_code(Ed));
        tile_store(const_cast<double*>(d.t.p), d.t.ld, d.t.rows, d.t.cols, X);
        fence_async_smem();   // stages 0 and 1 are refilled by bulk copies later
      } else {
        oz_store_digits_uniform(p.sdig + (size_t)(d.flag - c.flags) * OZ_TILE, X, d.t.rows, d.t.cols,
                                Ed == NO_EXP ? 0 : Ed);
        cta_publish_val(c, const_cast<int*>(d.flag), sig_exp_code(Ed));
        tile_store(const_cast<double*>(d.t.p), d.t.ld, d.t.rows, d.t.cols, X);
      }
    }
    trace_task(c, t, type, t_task0);
  }
  return true;
}

}  // namespace gbta
