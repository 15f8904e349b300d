// BTA Cholesky factorization (Serinv pobtaf / pobtf) as one persistent dataflow kernel.
//
// Replaces the sequential block recurrence that the reference runs through Serinv
// (src/pyinla/solvers/structured_solver.py:83-93):
//   D_i <- chol(D_i); L_i <- L_i D_i^{-T}; R_i <- R_i D_i^{-T};
//   D_{i+1} -= L_i L_i^T; R_{i+1} -= R_i L_i^T; T -= R_i R_i^T; T <- chol(T)
// by a left-looking tile Cholesky of the banded tile matrix.  One task finalises one
// TS x TS tile of D_i (lower), L_i or R_i: it subtracts the products of already
// final tiles to its left (including the previous block column, which is the
// Schur update D_{i+1} -= L_i L_i^T / R_{i+1} -= R_i L_i^T), then factors (diagonal
// tile) or solves against the diagonal tile of its column.  Tiles of the next
// block start as soon as the panels they need are final, so consecutive diagonal
// blocks overlap instead of running one after the other.
#include "bta_common.cuh"

namespace gbta {

struct FactorArgs {
  double* D;
  double* L;
  double* R;
  double* T;
  Geom g;
  int use_arrow;
  const int4* tasks;
  int ntasks;
  double* tip_part;   // [nt*B] tiles of R_i(c) R_i(c)^T (a x a used)
  Ctl c;
};

__device__ __forceinline__ const double* Dblk(const FactorArgs& p, int i) {
  return p.D + (size_t)i * p.g.b * p.g.b;
}
__device__ __forceinline__ const double* Lblk(const FactorArgs& p, int i) {
  return p.L + (size_t)i * p.g.b * p.g.b;
}
__device__ __forceinline__ const double* Rblk(const FactorArgs& p, int i) {
  return p.R + (size_t)i * p.g.a * p.g.b;
}

// Tile (r, c) of a b x b block / column tile c of an a x b arrow block.
__device__ __forceinline__ Tile btile(const double* blk, const Geom& g, int r, int c) {
  return make_tile(blk, g.b, r * TS, c * TS, g.b, g.b);
}
__device__ __forceinline__ Tile atile(const double* blk, const Geom& g, int c) {
  return make_tile(blk, g.b, 0, c * TS, g.a, g.b);
}

// Stage the diagonal factor tile D_i(c, c) (identity padded) after waiting for it.
__device__ bool load_diag_factor(const FactorArgs& p, int i, int c, double* F, int* s_ok) {
  if (!cta_wait(p.c, p.c.flags + p.g.fD(i, c, c), nullptr, s_ok)) return false;
  tile_load(F, btile(Dblk(p, i), p.g, c, c));
  __syncthreads();
  tile_pad_identity(F, p.g.vrows(c));
  __syncthreads();
  return true;
}

__global__ void __launch_bounds__(NT, 1) k_factor(FactorArgs p) {
  __shared__ double sm[4 * TILE_SMEM];
  __shared__ double vec[TS];            // pivots' 1/sqrt, or reciprocals of a factor tile's diagonal
  __shared__ int s_ok, s_t;
  double* bufs = sm;                    // 4 tiles: K-loop double buffer
  double* X = sm;                       // target tile (aliases the K-loop buffers:
  double* F = sm + TILE_SMEM;           // used only before / after the loop)
  const Geom& g = p.g;
  const Ctl& c = p.c;

  while (true) {
    const int t = cta_ticket(c, &s_t);
    const unsigned long long t_task0 = c.trace ? gtimer() : 0ull;
    if (t < 0 || t >= p.ntasks) break;
    const int4 tk = p.tasks[t];
    const int type = tk.x, i = tk.y, r = tk.z, col = tk.w;
    if (!p.use_arrow && (type == FT_ARW || type == FT_TIP)) continue;

    Acc acc;
    if (type == FT_TIP) {
      // T -= sum_{i,c} R_i(c) R_i(c)^T in a fixed order, then chol(T) (a <= TS).
      tile_load(X, make_tile(p.T, g.a, 0, 0, g.a, g.a));
      __syncthreads();
      acc_from_smem(acc, X);
      bool ok = true;
      for (int k = 0; k < g.nt * g.B && ok; ++k) {
        ok = cta_wait(c, c.flags + g.fR(k / g.B, k % g.B), nullptr, &s_ok);
        if (!ok) break;
        const double* P = p.tip_part + (size_t)k * TS * TS;
#pragma unroll
        for (int ii = 0; ii < 2; ++ii)
#pragma unroll
          for (int q = 0; q < 4; ++q) acc.v[ii][q] -= __ldcg(P + acc_row(ii) * TS + acc_col(q));
      }
      if (!ok) break;
      acc_to_smem(acc, X);
      __syncthreads();
      for (int idx = threadIdx.x; idx < TS * TS; idx += NT) {   // zero padding, identity diagonal
        const int rr = idx / TS, cc = idx % TS;
        if (rr >= g.a || cc >= g.a) X[rr * LDS + cc] = (rr == cc) ? 1.0 : 0.0;
      }
      const int info = smem_potrf(X, vec);
      if (info) {
        if (threadIdx.x == 0) {
          atomicCAS(c.ctrl + CTRL_INFO, 0, g.nt * g.b + info);
          raise_abort(c);
        }
        break;
      }
      tile_store(p.T, g.a, g.a, g.a, X);
      cta_publish(c, c.flags + g.fT());
      trace_task(c, t, type, t_task0);
      continue;
    }

    // ---- K-loop: subtract products of final tiles left of the target.
    // Target row operand source for within-block (k < col) and previous-block terms.
    const double* tgt_blk;
    Tile tgt;
    int* tgt_flag;
    if (type == FT_DIAG || type == FT_OFFD) {
      tgt_blk = Dblk(p, i);
      tgt = btile(tgt_blk, g, r, col);
      tgt_flag = c.flags + g.fD(i, r, col);
    } else if (type == FT_LOW) {
      tgt_blk = Lblk(p, i);
      tgt = btile(tgt_blk, g, r, col);
      tgt_flag = c.flags + g.fL(i, r, col);
    } else {   // FT_ARW
      tgt_blk = Rblk(p, i);
      tgt = atile(tgt_blk, g, col);
      tgt_flag = c.flags + g.fR(i, col);
    }
    tile_load(X, tgt);
    __syncthreads();
    acc_from_smem(acc, X);
    __syncthreads();

    const bool prev = (i > 0) && (type != FT_LOW);
    const int nprev = prev ? g.B : 0;
    const int nsteps = nprev + col;
    auto step_of = [&](int s) -> Step {
      Step st;
      st.ta = false;
      st.tb = true;
      if (s < nprev) {   // previous block column: Schur terms with L_{i-1}
        const int k = s;
        if (type == FT_ARW) {
          st.a = atile(Rblk(p, i - 1), g, k);
          st.fa = c.flags + g.fR(i - 1, k);
        } else {
          st.a = btile(Lblk(p, i - 1), g, r, k);
          st.fa = c.flags + g.fL(i - 1, r, k);
        }
        st.b = btile(Lblk(p, i - 1), g, col, k);
        st.fb = c.flags + g.fL(i - 1, col, k);
      } else {           // within the block column: tiles k < col of the same row
        const int k = s - nprev;
        if (type == FT_ARW) {
          st.a = atile(Rblk(p, i), g, k);
          st.fa = c.flags + g.fR(i, k);
        } else if (type == FT_LOW) {
          st.a = btile(Lblk(p, i), g, r, k);
          st.fa = c.flags + g.fL(i, r, k);
        } else {
          st.a = btile(Dblk(p, i), g, r, k);
          st.fa = c.flags + g.fD(i, r, k);
        }
        st.b = btile(Dblk(p, i), g, col, k);
        st.fb = c.flags + g.fD(i, col, k);
        if (st.fa == st.fb) st.fb = nullptr;
      }
      return st;
    };
    if (!kloop<true>(acc, nsteps, step_of, c, bufs, &s_ok)) break;
    acc_to_smem(acc, X);
    __syncthreads();

    if (type == FT_DIAG) {
      tile_pad_identity(X, g.vrows(col));
      const int info = smem_potrf(X, vec);
      if (info) {
        if (threadIdx.x == 0) {
          atomicCAS(c.ctrl + CTRL_INFO, 0, i * g.b + col * TS + info);
          raise_abort(c);
        }
        break;
      }
      tile_store(const_cast<double*>(tgt.p), g.b, tgt.rows, tgt.cols, X);
      cta_publish(c, tgt_flag);
      trace_task(c, t, type, t_task0);
      continue;
    }

    // Off-diagonal targets: X <- X * D_i(col,col)^{-T}.
    if (!load_diag_factor(p, i, col, F, &s_ok)) break;
    tile_diag_recip(F, vec);
    smem_trsm_rlt(X, F, vec);
    tile_store(const_cast<double*>(tgt.p), tgt.ld, tgt.rows, tgt.cols, X);
    if (type == FT_OFFD) {
      // The factor's strict upper triangle is zero: clear the mirrored tile.
      const Tile up = btile(Dblk(p, i), g, col, r);
      tile_store_zero(const_cast<double*>(up.p), g.b, up.rows, up.cols);
    }
    if (type == FT_ARW) {
      // Partial tip update P = X X^T, consumed in order by the tip task.
      __syncthreads();
      for (int idx = threadIdx.x; idx < TS * TS; idx += NT) F[(idx % TS) * LDS + idx / TS] = X[(idx / TS) * LDS + idx % TS];
      __syncthreads();
      Acc pacc;
      acc_zero(pacc);
      tile_mma<false>(pacc, X, F);
      double* P = p.tip_part + (size_t)(i * g.B + col) * TS * TS;
#pragma unroll
      for (int ii = 0; ii < 2; ++ii)
#pragma unroll
        for (int q = 0; q < 4; ++q) P[acc_row(ii) * TS + acc_col(q)] = pacc.v[ii][q];
    }
    cta_publish(c, tgt_flag);
    trace_task(c, t, type, t_task0);
  }
}

void launch_factor(const Geom& g, double* D, double* L, double* R, double* T, int use_arrow, const int4* tasks,
                   int ntasks, double* tip_part, const LaunchCtl& lc) {
  FactorArgs p;
  p.D = D;
  p.L = L;
  p.R = R;
  p.T = T;
  p.g = g;
  p.use_arrow = use_arrow;
  p.tasks = tasks;
  p.ntasks = ntasks;
  p.tip_part = tip_part;
  p.c.ctrl = lc.ctrl;
  p.c.flags = lc.flags;
  p.c.epoch = lc.epoch;
  p.c.wait_ns = lc.wait_ns;
  p.c.trace = lc.trace;
  k_factor<<<lc.grid, NT, 0, lc.stream>>>(p);
  count_launches(1);
}

}  // namespace gbta
