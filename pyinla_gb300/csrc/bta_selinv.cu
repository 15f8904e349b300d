// BTA selected inversion (Serinv pobtasi / pobtsi) as one persistent dataflow kernel.
//
// Replaces the backward block recurrence the reference runs through Serinv
// (src/pyinla/solvers/structured_solver.py:176-186), which overwrites the factor
// blocks with Sigma = Q^{-1} on the BTA pattern.  Here the recurrence is taken to
// tile level.  With F the (tile-banded) Cholesky factor, Sigma F = F^{-T} gives for
// tile column k and its below-diagonal pattern P_k:
//   Sigma(j,k) = -( sum_{l in P_k} Sigma(j,l) F(l,k) ) F(k,k)^{-1}      (j in P_k)
//   Sigma(k,k) =  ( F(k,k)^{-T} - sum_{l in P_k} Sigma(l,k)^T F(l,k) ) F(k,k)^{-1}
// P_k of tile column c of block i is: tiles of D_i below c, all tiles of L_i (block
// row i+1) and the arrow tile.  Every Sigma(j,l) needed lies in a later column, so
// tasks run column by column from the tip backwards; a task of column k starts its
// products while column k+1 is still finishing.
//
// Sigma is written to a separate workspace (the factor tiles F(l,k) of a column are
// read by all tasks of that column) and copied back into the caller's buffers by
// launch_selinv_writeback, which also mirrors D_i and T to full symmetric blocks.
#include "bta_common.cuh"

namespace gbta {

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
  const int4* tasks;
  int ntasks;
  Ctl c;
};

// Row descriptor of a tile row in the pattern of column (i, c):
//   code in [0, B): block i row tile; [B, 2B): block i+1 row tile; 2B: arrow.
struct SigTile {
  Tile t;
  bool trans;
  const int* flag;
};

__device__ __forceinline__ int rows_of(const Geom& g, int code) {
  return code == 2 * g.B ? g.a : g.vrows(code % g.B);
}

// Sigma tile at (row j, col l) of the global matrix, both given as row codes
// relative to block column i.  Stored in lower storage; trans = stored transposed.
__device__ SigTile sig_tile(const SelinvArgs& p, int i, int j, int l) {
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
__device__ __forceinline__ Tile fac_tile(const SelinvArgs& p, int i, int l, int c) {
  const Geom& g = p.g;
  const size_t bb = (size_t)g.b * g.b, ab = (size_t)g.a * g.b;
  const int B = g.B;
  if (l == 2 * B) return make_tile(p.R + i * ab, g.b, 0, c * TS, g.a, g.b);
  if (l >= B) return make_tile(p.L + i * bb, g.b, (l - B) * TS, c * TS, g.b, g.b);
  return make_tile(p.D + i * bb, g.b, l * TS, c * TS, g.b, g.b);
}

// Destination of Sigma(j, c) (j a row code of column (i, c)).
__device__ __forceinline__ SigTile sig_dest(const SelinvArgs& p, int i, int j, int c) {
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
__device__ __forceinline__ int pat_size(const SelinvArgs& p, int i, int c) {
  const Geom& g = p.g;
  return (p.use_arrow ? 1 : 0) + (i < g.nt - 1 ? g.B : 0) + (g.B - 1 - c);
}
__device__ __forceinline__ int pat_code(const SelinvArgs& p, int i, int c, int s) {
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
__device__ void diag_finish(double* X, double* W, const double* F, const double* rd) {
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

__global__ void __launch_bounds__(NT, 1) k_selinv(SelinvArgs p) {
  __shared__ double sm[4 * TILE_SMEM];
  __shared__ double rd[TS];   // reciprocals of the diagonal factor tile's diagonal
  __shared__ int s_ok, s_t;
  double* bufs = sm;
  double* X = sm;
  double* F = sm + TILE_SMEM;
  double* W = sm + 2 * TILE_SMEM;
  const Geom& g = p.g;
  const Ctl& c = p.c;

  while (true) {
    const int t = cta_ticket(c, &s_t);
    const unsigned long long t_task0 = c.trace ? gtimer() : 0ull;
    if (t < 0 || t >= p.ntasks) break;
    const int4 tk = p.tasks[t];
    const int type = tk.x, i = tk.y, j = tk.z, col = tk.w;
    if (!p.use_arrow && (type == ST_TIP || (type == ST_OFF && j == 2 * g.B))) continue;

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
      continue;
    }

    const int np = pat_size(p, i, col);
    Acc acc;
    acc_zero(acc);
    if (type == ST_OFF) {
      // Y = sum_l Sigma(j,l) F(l,col); Sigma(j,col) = -Y F(col,col)^{-1}
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
      if (!kloop<true>(acc, np, step_of, c, bufs, &s_ok)) break;   // acc = -Y
      acc_to_smem(acc, X);
      __syncthreads();
      tile_load(F, fac_tile(p, i, col, col));
      __syncthreads();
      tile_pad_identity(F, g.vrows(col));
      __syncthreads();
      tile_diag_recip(F, rd);
      smem_trsm_rln(X, F, rd);
      const SigTile d = sig_dest(p, i, j, col);
      tile_store(const_cast<double*>(d.t.p), d.t.ld, d.t.rows, d.t.cols, X);
      cta_publish(c, const_cast<int*>(d.flag));
      trace_task(c, t, type, t_task0);
    } else {   // ST_DIAG
      // Z = sum_l Sigma(l,col)^T F(l,col)
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
      if (!kloop<false>(acc, np, step_of, c, bufs, &s_ok)) break;
      acc_to_smem(acc, X);
      __syncthreads();
      tile_load(F, fac_tile(p, i, col, col));
      __syncthreads();
      tile_pad_identity(F, g.vrows(col));
      __syncthreads();
      tile_diag_recip(F, rd);
      __syncthreads();
      diag_finish(X, W, F, rd);
      const SigTile d = sig_dest(p, i, col, col);
      tile_store(const_cast<double*>(d.t.p), d.t.ld, d.t.rows, d.t.cols, X);
      cta_publish(c, const_cast<int*>(d.flag));
      trace_task(c, t, type, t_task0);
    }
  }
}

// Copy Sigma back into the caller's buffers; D_i and T become full symmetric.
__global__ void k_writeback(const double* SD, const double* SL, const double* SR, const double* ST, double* D,
                            double* L, double* R, double* T, Geom g, int use_arrow) {
  const size_t bb = (size_t)g.b * g.b;
  const size_t nD = g.nt * bb, nL = (g.nt - 1) * bb, nR = use_arrow ? (size_t)g.nt * g.a * g.b : 0;
  const size_t nT = use_arrow ? (size_t)g.a * g.a : 0;
  const size_t total = nD + nL + nR + nT;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    if (e < nD) {
      const size_t blk = e / bb, rem = e % bb;
      const int r = (int)(rem / g.b), cc = (int)(rem % g.b);
      const bool lower = (r / TS) >= (cc / TS);   // tiles on/below the diagonal are stored
      D[e] = lower ? SD[blk * bb + (size_t)r * g.b + cc] : SD[blk * bb + (size_t)cc * g.b + r];
    } else if (e < nD + nL) {
      L[e - nD] = SL[e - nD];
    } else if (e < nD + nL + nR) {
      R[e - nD - nL] = SR[e - nD - nL];
    } else {
      T[e - nD - nL - nR] = ST[e - nD - nL - nR];
    }
  }
}

void launch_selinv(const Geom& g, const double* D, const double* L, const double* R, const double* T, double* SD,
                   double* SL, double* SR, double* ST, int use_arrow, const int4* tasks, int ntasks,
                   const LaunchCtl& lc) {
  SelinvArgs p;
  p.D = D;
  p.L = L;
  p.R = R;
  p.T = T;
  p.SD = SD;
  p.SL = SL;
  p.SR = SR;
  p.ST = ST;
  p.g = g;
  p.use_arrow = use_arrow;
  p.tasks = tasks;
  p.ntasks = ntasks;
  p.c.ctrl = lc.ctrl;
  p.c.flags = lc.flags;
  p.c.epoch = lc.epoch;
  p.c.wait_ns = lc.wait_ns;
  p.c.trace = lc.trace;
  k_selinv<<<lc.grid, NT, 0, lc.stream>>>(p);
  count_launches(1);
}

void launch_selinv_writeback(const Geom& g, const double* SD, const double* SL, const double* SR, const double* ST,
                             double* D, double* L, double* R, double* T, int use_arrow, cudaStream_t stream) {
  k_writeback<<<1024, 256, 0, stream>>>(SD, SL, SR, ST, D, L, R, T, g, use_arrow);
  count_launches(1);
}

}  // namespace gbta
