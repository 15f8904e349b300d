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
// P_k of tile column c of block i is: tiles of D_i below c, all tiles of L_i (block
// row i+1) and the arrow tile.  Every Sigma(j,l) needed lies in a later column, so
// tasks run column by column from the tip backwards; a task of column k starts its
// products while column k+1 is still finishing.
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
//    the ldmatrix layout; the left operand Sigma tiles are sliced while staged,
//    relative to the task's running exponent E (the largest tile exponent seen so far
//    in the task); when a tile raises E, the exact partial sums are first folded into
//    FP64 with the old E.  Tile inverses and triangular solves stay in FP64.
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
  const int* ecol;      // Ozaki: per global column (nt*b) exponent of the G column pattern
  const double* cinv;   // [nt*B][TS*TS]: F_cc^{-T} F_cc^{-1} of every diagonal factor tile
  Ctl c;
};

// Row descriptor of a tile row in the pattern of column (i, c):
//   code in [0, B): block i row tile; [B, 2B): block i+1 row tile; 2B: arrow.
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
    const int blk = other < B ? i : i + 1;
    const int r = other % B;
    s.t = make_tile(p.SR + blk * ab, g.b, 0, r * TS, g.a, g.b);
    s.trans = (l == A);
    s.flag = F + g.fR(blk, r);
  } else if (j < B && l < B) {   // both in block i
    const int hi = max(j, l), lo = min(j, l);
    s.t = dtile(i, hi, lo);
    s.trans = j < l;
    s.flag = F + g.fD(i, hi, lo);
  } else if (j >= B && l >= B) {   // both in block i+1
    const int hi = max(j, l) - B, lo = min(j, l) - B;
    s.t = dtile(i + 1, hi, lo);
    s.trans = j < l;
    s.flag = F + g.fD(i + 1, hi, lo);
  } else {   // one in block i+1 (rows of SL_i), one in block i (cols of SL_i)
    const int rl = (j >= B ? j : l) - B, cd = (j >= B ? l : j);
    s.t = make_tile(p.SL + i * bb, g.b, rl * TS, cd * TS, g.b, g.b);
    s.trans = j < B;
    s.flag = F + g.fL(i, rl, cd);
  }
  return s;
}

// Factor tile F(l, c) of block column i (l a row code); no wait needed.
static __device__ __forceinline__ Tile fac_tile(const SelinvArgs& p, int i, int l, int c) {
  const Geom& g = p.g;
  const size_t bb = (size_t)g.b * g.b, ab = (size_t)g.a * g.b;
  const int B = g.B;
  if (l == 2 * B) return make_tile(p.R + i * ab, g.b, 0, c * TS, g.a, g.b);
  if (l >= B) return make_tile(p.L + i * bb, g.b, (l - B) * TS, c * TS, g.b, g.b);
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
    s.t = make_tile(p.SL + i * bb, g.b, (j - B) * TS, c * TS, g.b, g.b);
    s.flag = p.c.flags + g.fL(i, j - B, c);
  } else {
    s.t = make_tile(p.SD + i * bb, g.b, j * TS, c * TS, g.b, g.b);
    s.flag = p.c.flags + g.fD(i, j, c);
  }
  return s;
}

// Pattern of column (i, c), ordered so that the most recently produced Sigma tiles
// come last: arrow, block i+1 rows descending, block i rows descending (> c).
static __device__ __forceinline__ int pat_size(const SelinvArgs& p, int i, int c) {
  const Geom& g = p.g;
  return (p.use_arrow ? 1 : 0) + (i < g.nt - 1 ? g.B : 0) + (g.B - 1 - c);
}
static __device__ __forceinline__ int pat_code(const SelinvArgs& p, int i, int c, int s) {
  const Geom& g = p.g;
  if (p.use_arrow) {
    if (s == 0) return 2 * g.B;
    --s;
  }
  if (i < g.nt - 1) {
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
  if (l >= B) return g.fL(i, l - B, c);
  return g.fD(i, l, c);
}
// ---- consumer-side slicing of a staged FP64 tile ------------------------------------
// The left-operand tile is staged in registers as element pairs that are adjacent in
// the k dimension of the A operand, so that each digit plane gets one 32-bit shared
// store per pair:
//   not transposed (A(m, k) = X(m, k)):  pair (X(r, c), X(r, c+1)), c even;
//   transposed     (A(m, k) = X(k, m)):  pair (X(r, c), X(r+1, c)), r even.
// Pair p = threadIdx.x + q * NT (q = 0..3); a warp reads whole 256-byte rows.
static __device__ __forceinline__ void pair_coords(int p, bool trans, int& r, int& c) {
  if (trans) {
    c = p % TS;
    r = 2 * (p / TS);
  } else {
    r = p / (TS / 2);
    c = 2 * (p % (TS / 2));
  }
}
static __device__ __forceinline__ void tile_ldg_pairs(double (&v)[PER_THREAD], const Tile& t, bool trans) {
#pragma unroll
  for (int q = 0; q < PER_THREAD / 2; ++q) {
    int r, c;
    pair_coords(threadIdx.x + q * NT, trans, r, c);
    const int r1 = trans ? r + 1 : r, c1 = trans ? c : c + 1;
    v[2 * q] = (r < t.rows && c < t.cols) ? __ldcg(t.p + (size_t)r * t.ld + c) : 0.0;
    v[2 * q + 1] = (r1 < t.rows && c1 < t.cols) ? __ldcg(t.p + (size_t)r1 * t.ld + c1) : 0.0;
  }
}

// Exponent for slicing the register-staged tile: ilogb(max |v|) + 1 over the CTA, or
// NO_EXP for an all-zero tile (all threads return it).  The max is an integer max of
// the sign-cleared bit patterns (ordered like the magnitudes), so that no FP64
// instruction is spent on it.
constexpr int NO_EXP = -100000;
static __device__ __forceinline__ int cta_tile_exponent(const double (&v)[PER_THREAD], double* red4) {
  unsigned long long m = 0;
#pragma unroll
  for (int k = 0; k < PER_THREAD; ++k) {
    const unsigned long long a = (unsigned long long)__double_as_longlong(v[k]) & 0x7fffffffffffffffull;
    m = a > m ? a : m;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_xor_sync(0xffffffffu, m, o);
    m = x > m ? x : m;
  }
  unsigned long long* red = reinterpret_cast<unsigned long long*>(red4);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  unsigned long long r = red[0];
#pragma unroll
  for (int w = 1; w < NT / 32; ++w) r = red[w] > r ? red[w] : r;
  __syncthreads();
  return r ? ilogb_bits(r) + 1 : NO_EXP;
}

// Write the digit planes of the register-staged pairs relative to 2^E into the shared
// A operand ([plane][row][k], padded rows).
static __device__ __forceinline__ void oz_slice_to_smem(__half* As, const double (&v)[PER_THREAD], int E, bool trans) {
#pragma unroll
  for (int q = 0; q < PER_THREAD / 2; ++q) {
    int r, c;
    pair_coords(threadIdx.x + q * NT, trans, r, c);
    const int row = trans ? c : r, kk = trans ? r : c;
    int d0[OZ_S], d1[OZ_S];
    oz_digits(v[2 * q], E, d0);
    oz_digits(v[2 * q + 1], E, d1);
    unsigned* dst = reinterpret_cast<unsigned*>(As + row * OZ_LD + kk);
#pragma unroll
    for (int s = 0; s < OZ_S; ++s) dst[s * (OZ_PLANE / 2)] = oz_digit_pair(d0[s], d1[s]);
  }
}

constexpr int OZS_STAGE = 2 * OZ_OPER;   // halves per stage (A, B)
// X and F follow the two stages; W (used only by the epilogue and the tip task, when
// no stage is in flight) reuses the first stage, so that two CTAs fit on one SM.
constexpr size_t OZS_SMEM = 2 * OZS_STAGE * sizeof(__half) + 2 * TILE_SMEM * sizeof(double) + TS * sizeof(double) +
                            TS * sizeof(int) + 4 * sizeof(double);

// Task t of a tensor-core selected-inversion instance.  `raw` is OZS_SMEM bytes of
// (16-byte aligned) shared memory.  Returns false when the launch is aborted.
static __device__ __forceinline__ bool selinv_oz_task(const SelinvArgs& p, int t, unsigned char* raw, int* s_okp,
                                                      int* s_readyp) {
  __half* stages = reinterpret_cast<__half*>(raw);
  double* X = reinterpret_cast<double*>(raw + 2 * OZS_STAGE * sizeof(__half));
  double* F = X + TILE_SMEM;
  double* W = reinterpret_cast<double*>(raw);   // aliases stage 0 (free in the epilogue)
  double* rd = F + TILE_SMEM;
  int* ecol_t = reinterpret_cast<int*>(rd + TS);
  double* red4 = reinterpret_cast<double*>(ecol_t + TS);
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
      cta_publish(c, c.flags + g.fT());
      trace_task(c, t, type, t_task0);
      return true;
    }

    const int np = pat_size(p, i, col);
    if (threadIdx.x < TS) {
      const int cc = col * TS + threadIdx.x;
      ecol_t[threadIdx.x] = cc < g.b ? p.ecol[(size_t)i * g.b + cc] : 0;
    }
    __syncthreads();
    OzAcc acc;
    oz_clear_partials(acc);
#pragma unroll
    for (int n = 0; n < 2; ++n)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc.v[n][q] = 0.0;
    int E = NO_EXP;   // running exponent of the left operand (unset)
    int esum[2][4];
    auto set_esum = [&]() {
#pragma unroll
      for (int n = 0; n < 2; ++n)
#pragma unroll
        for (int q = 0; q < 4; ++q) esum[n][q] = E + ecol_t[oz_col(n, q)];
    };
    // step s: left tile (FP64) and right digits
    auto left_of = [&](int s) -> SigTile {
      const int l = pat_code(p, i, col, s);
      if (type == ST_OFF) return sig_tile(p, i, j, l);
      SigTile st_ = sig_dest(p, i, l, col);   // Sigma(l, col), used transposed
      st_.trans = true;
      return st_;
    };
    auto right_of = [&](int s) -> const __half* {
      return p.fdig + (size_t)fac_slot(g, i, pat_code(p, i, col, s), col) * OZ_TILE;
    };

    bool ok = true;
    double vreg[PER_THREAD];
    int since_fold = 0;
    // trace marks: m0 first operand ready, m1 end of the last blocking wait in the
    // product loop, m2 ns spent in those waits, m3 product steps
    unsigned long long waited = 0;
    trace_clear_marks(c, t);
    auto flags_of = [&](int s, const int*& f0, const int*& f1) {
      f0 = left_of(s).flag;
      f1 = nullptr;
    };
    if (np > 0) {
      SigTile lt = left_of(0);
      ok = cta_wait(c, lt.flag, nullptr, &s_ok);
      trace_mark(c, t, 0);
      if (ok) {
        if (threadIdx.x == 0) s_ready = 1;
        tile_ldg_pairs(vreg, lt.t, lt.trans);
        oz_load_async(stages + OZ_OPER, right_of(0));
        cp_async_commit();
        E = cta_tile_exponent(vreg, red4);
        set_esum();
        oz_slice_to_smem(stages, vreg, E, lt.trans);
      }
      for (int s = 0; s < np && ok; ++s) {
        __half* cur = stages + (s & 1) * OZS_STAGE;
        __half* nxt = stages + ((s + 1) & 1) * OZS_STAGE;
        cp_async_wait_all();
        __syncthreads();
        const bool more = s + 1 < np;
        bool have = false;
        SigTile nt_;
        if (more) {
          nt_ = left_of(s + 1);
          if (s_ready <= s + 1) {   // uniform: read after the barrier
            scan_ready(c, np, flags_of, &s_ready);
            __syncthreads();
          }
          if (s_ready > s + 1) {
            tile_ldg_pairs(vreg, nt_.t, nt_.trans);
            oz_load_async(nxt + OZ_OPER, right_of(s + 1));
            cp_async_commit();
            have = true;
          }
        }
        oz_step(acc, cur, cur + OZ_OPER);
        ++since_fold;
        if (more) {
          if (!have) {
            const unsigned long long w0 = c.trace ? gtimer() : 0ull;
            if (!(ok = cta_wait(c, nt_.flag, nullptr, &s_ok))) break;
            if (c.trace) {
              waited += gtimer() - w0;
              trace_mark(c, t, 1);
            }
            if (threadIdx.x == 0) s_ready = s + 2;
            tile_ldg_pairs(vreg, nt_.t, nt_.trans);
            oz_load_async(nxt + OZ_OPER, right_of(s + 1));
            cp_async_commit();
          }
          const int En = cta_tile_exponent(vreg, red4);
          if (En > E || since_fold == OZ_CHUNK) {
            if (E > NO_EXP) oz_fold_sub(acc, esum);
            since_fold = 0;
            if (En > E) E = En;
            set_esum();
          }
          oz_slice_to_smem(nxt, vreg, E, nt_.trans);
        } else if (E > NO_EXP) {
          oz_fold_sub(acc, esum);   // acc.v = -(sum)
        }
      }
    }
    if (!ok) {
      cp_async_wait_all();
      return false;
    }
    trace_put(c, t, 2, (long long)waited);
    trace_put(c, t, 3, np);
    __syncthreads();
    // acc.v = -(sum of the products): ST_OFF: Sigma(j,col); ST_DIAG: -Z
#pragma unroll
    for (int n = 0; n < 2; ++n)
#pragma unroll
      for (int q = 0; q < 4; ++q) X[oz_row(n, q) * LDS + oz_col(n, q)] = acc.v[n][q];
    if (type == ST_OFF) {
      __syncthreads();
      const SigTile d = sig_dest(p, i, j, col);
      tile_store(const_cast<double*>(d.t.p), d.t.ld, d.t.rows, d.t.cols, X);
      cta_publish(c, const_cast<int*>(d.flag));
    } else {
      tile_load(F, make_tile(p.cinv + (size_t)(i * g.B + col) * TS * TS, TS, 0, 0, TS, TS));
      __syncthreads();
      diag_from_cinv(X, F);
      const SigTile d = sig_dest(p, i, col, col);
      tile_store(const_cast<double*>(d.t.p), d.t.ld, d.t.rows, d.t.cols, X);
      cta_publish(c, const_cast<int*>(d.flag));
    }
    trace_task(c, t, type, t_task0);
  }
  return true;
}

}  // namespace gbta
