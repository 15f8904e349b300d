// Per-task bodies of the BTA factorization, shared by the single-instance kernels
// (bta_factor.cu, bta_factor_oz.cu) and the multi-instance kernel (bta_batch.cu).
//
// BTA Cholesky factorization (Serinv pobtaf / pobtf) as one persistent dataflow kernel.
//
// Replaces the sequential block recurrence that the reference runs through Serinv
// (src/pyinla/solvers/structured_solver.py:83-93):
//   D_i <- chol(D_i); L_i <- L_i D_i^{-T}; R_i <- R_i D_i^{-T};
//   D_{i+1} -= L_i L_i^T; R_{i+1} -= R_i L_i^T; T -= R_i R_i^T; T <- chol(T)
// by a left-looking tile Cholesky of the banded tile matrix.  One task finalises one
// TS x TS tile of D_i (lower), of block i's coupling slot in L, or of R_i: it subtracts
// the products of already final tiles to its left (including the block columns of the
// neighbours eliminated before block i, which is the Schur update D_{i+1} -= L_i L_i^T /
// R_{i+1} -= R_i L_i^T), then factors (diagonal tile) or solves against the diagonal
// tile of its column.  The blocks are eliminated in the order of Geom (top-down, or
// from both ends towards the separator block).  Tiles of the next
// block start as soon as the panels they need are final, so consecutive diagonal
// blocks overlap instead of running one after the other.
//
// Two ways to compute the tile products of the left-looking loop (FactorArgs::method):
//  * FP64: FP64 FMAs on staged FP64 tiles (factor_fp64_task);
//  * OZAKI: the tiles' digit planes (written by the tasks that finalised them) go
//    through mma.sync with exact fp32 accumulation, folded into FP64 every OZ_CHUNK
//    steps (factor_oz_task, see bta_ozaki.cuh).
// Both share the task DAG, the ordering and the FP64 epilogues: tile factorizations
// (POTRF), triangular solves (TRSM) and the arrow-tip partials.
#pragma once

#include "bta_ozaki.cuh"

namespace gbta {

// Arguments of one factorization instance (both product methods).
struct FactorArgs {
  double* D;
  double* L;
  double* R;
  double* T;
  Geom g;
  int use_arrow;
  int method;           // GBTA_METHOD_FP64 / GBTA_METHOD_OZAKI
  const int4* tasks;
  int ntasks;
  double* tip_part;     // [nt*B] tiles of R_i(c) R_i(c)^T (a x a used)
  __half* digits;       // Ozaki: [nflags][OZ_TILE] digit planes of the final tiles
  const int* erow;      // Ozaki: [nt*b + a] row exponents
  int* info;            // where a failed pivot is recorded (null: the control block)
  int* feed_pre;        // [nt*B] flag: the feeder of diagonal tile (i, c) has its products
  int* diag_pre;        // [2*nt*B] flags: diagonal tile (i, c), then the feeder of column
                        // (i, c), holds its partial products (split loops; see FT_PART)
  const int* kf;        // [(nt-1)*B] first column tile of each coupling-slot row tile that
                        // can be nonzero (launch_coupling_kfirst), or null
  Ctl c;
};

// Product steps of a task's left-looking loop: the (one or two) neighbour blocks'
// columns first (prev = true, neighbour pb, column k), then the columns k < col of its
// own block.  A diagonal tile's loop and its column's feeder loop are split into a
// partial (every step but the last: k = col - 1, or k = B - 1 of each neighbour when
// col = 0) and a tail (those last steps) when the task list splits them (FT_PART /
// FT_TAIL).
struct StepRange {
  int n;       // steps
  int mode;    // 0 full, 1 partial, 2 tail
  int nprev;   // leading steps that are neighbour-block terms
  int n0;      // of those, the first neighbour's (the rest are the second's)
  int ka, kb;  // column of the first neighbour's first term, and of the second's
  int kin;     // column of the first own-block term
};
// First column tile of coupling slot ls's row tile r that can be nonzero (FactorArgs::kf).
static __device__ __forceinline__ int kfirst(const FactorArgs& p, int ls, int r) {
  return p.kf ? __ldg(p.kf + ls * p.g.B + r) : 0;
}
// The steps of a task (type, mode) on target row tile r, column col of block i.  A
// neighbour's term k multiplies its coupling tiles (r, k) and (col, k) (the arrow's
// only (col, k)); an L target's own-block term k its own tile (r, k): terms on a
// structurally zero tile are left out, so each neighbour's terms and the own block's
// are a contiguous run of columns.
static __device__ __forceinline__ StepRange step_range(const FactorArgs& p, int type, int mode, int i, int r,
                                                       int col) {
  const Geom& g = p.g;
  StepRange sr;
  sr.mode = mode;
  sr.nprev = 0;
  sr.n0 = 0;
  sr.ka = sr.kb = 0;
  const int np = (type != FT_LOW) ? g.nprev(i) : 0;
  for (int q = 0; q < np; ++q) {
    const int ls = g.lslot(g.prev(i, q));
    int k0 = kfirst(p, ls, col), k1 = g.B;
    if (type != FT_ARW) k0 = max(k0, kfirst(p, ls, r));
    if (mode == 1 && col == 0) k1 = g.B - 1;           // all but each neighbour's last column
    if (mode == 2) k0 = col == 0 ? max(k0, g.B - 1) : g.B;   // only those (col 0), none (col > 0)
    const int cnt = max(0, k1 - k0);
    if (q == 0) {
      sr.ka = k0;
      sr.n0 = cnt;
    } else {
      sr.kb = k0;
    }
    sr.nprev += cnt;
  }
  int kin = (type == FT_LOW) ? kfirst(p, g.lslot(i), r) : 0, kend = col;
  if (mode == 1) kend = col - 1;                        // all but the last own column
  if (mode == 2) kin = col == 0 ? col : max(kin, col - 1);   // only that one
  sr.kin = kin;
  sr.n = sr.nprev + max(0, kend - kin);
  return sr;
}
// Step s of a range: a neighbour-block term (prev: neighbour pb, its column k) or a term
// of the task's own block (column k).
static __device__ __forceinline__ void step_src(const Geom& g, const StepRange& sr, int i, int s, bool& prev,
                                                int& pb, int& k) {
  prev = s < sr.nprev;
  if (prev) {
    const bool first = s < sr.n0;
    pb = g.prev(i, first ? 0 : 1);
    k = first ? sr.ka + s : sr.kb + (s - sr.n0);
  } else {
    pb = i;
    k = sr.kin + (s - sr.nprev);
  }
}

static __device__ __forceinline__ const double* Dblk(const FactorArgs& p, int i) {
  return p.D + (size_t)i * p.g.b * p.g.b;
}
static __device__ __forceinline__ const double* Lblk(const FactorArgs& p, int i) {
  return p.L + (size_t)i * p.g.b * p.g.b;
}
static __device__ __forceinline__ const double* Rblk(const FactorArgs& p, int i) {
  return p.R + (size_t)i * p.g.a * p.g.b;
}

// Tile (r, c) of a b x b block / column tile c of an a x b arrow block.
static __device__ __forceinline__ Tile btile(const double* blk, const Geom& g, int r, int c) {
  return make_tile(blk, g.b, r * TS, c * TS, g.b, g.b);
}
static __device__ __forceinline__ Tile atile(const double* blk, const Geom& g, int c) {
  return make_tile(blk, g.b, 0, c * TS, g.a, g.b);
}

// The feeder tile of diagonal tile (i, c) (Geom::feeder_kind), its flag slot and the
// global row of its first row.
static __device__ __forceinline__ Tile feeder_tile(const FactorArgs& p, int i, int c, int& slot, long long& row0) {
  const Geom& g = p.g;
  if (g.feeder_kind(i, c) == 1) {
    slot = g.fD(i, c + 1, c);
    row0 = (long long)i * g.b + (c + 1) * TS;
    return btile(Dblk(p, i), g, c + 1, c);
  }
  const int ls = g.lslot(i);
  slot = g.fL(ls, 0, c);
  row0 = (long long)g.nxt(i) * g.b;
  return btile(Lblk(p, ls), g, 0, c);
}

// FT_FEEDQ task: rows FEED_ROWS q .. of the feeder of diagonal tile (i, col) <- their
// products (left there by the FT_PRE task) times D_i(col, col)^{-T}, plus their digit
// planes (tensor-core method).  Each group adds its share of the epoch to the
// feeder's ready flag, which reaches the epoch when the last group has written.  X, F, FS: shared tiles; rd: TS doubles; erow_t: TS ints (digits only).
static __device__ bool factor_feed_rows(const FactorArgs& p, int t, int i, int q, int col, double* X, double* F,
                                        double* FS, double* rd, int* erow_t, int* s_ok, unsigned long long t_task0) {
  const Geom& g = p.g;
  const Ctl& c = p.c;
  int slot;
  long long grow0;
  const Tile ft = feeder_tile(p, i, col, slot, grow0);
  const int gc = i * g.B + col, row0 = q * FEED_ROWS;
  trace_clear_marks(c, t);
  const bool digits = p.method == GBTA_METHOD_OZAKI && p.digits;
  // the group's rows (their products were formed ahead of the diagonal tile) are
  // loaded while the diagonal tile is awaited
  if (!cta_wait(c, p.feed_pre + gc, nullptr, s_ok)) return false;
  constexpr int RPT = FEED_ROWS * TS / NT;
  double xv[RPT];
#pragma unroll
  for (int k = 0; k < RPT; ++k) {
    const int idx = threadIdx.x + k * NT, rr = row0 + idx / TS, cc = idx % TS;
    xv[k] = (rr < ft.rows && cc < ft.cols) ? __ldcg(ft.p + (size_t)rr * ft.ld + cc) : 0.0;
  }
  if (digits && threadIdx.x < TS) erow_t[threadIdx.x] = threadIdx.x < ft.rows ? p.erow[grow0 + threadIdx.x] : 0;
  if (!cta_wait(c, c.flags + g.fD(i, col, col), nullptr, s_ok)) return false;
  trace_mark(c, t, 0);   // diagonal factor tile ready
  {
    double fv[PER_THREAD];
    tile_ldg(fv, btile(Dblk(p, i), g, col, col));
    tile_sts(F, fv);
#pragma unroll
    for (int k = 0; k < RPT; ++k) {
      const int idx = threadIdx.x + k * NT;
      X[(row0 + idx / TS) * LDS + idx % TS] = xv[k];
    }
  }
  __syncthreads();
  tile_pad_identity(F, g.vrows(col));
  __syncthreads();
  tile_diag_recip(F, rd);
  __syncthreads();
  tile_scale_rows_by_recip(FS, F, rd);
  trace_mark(c, t, 1);   // operands staged
  smem_trsm_rlt_rows8(X, FS, rd, row0);
  trace_mark(c, t, 2);   // rows solved
  for (int idx = threadIdx.x; idx < FEED_ROWS * TS; idx += NT) {
    const int rr = row0 + idx / TS, cc = idx % TS;
    if (rr < ft.rows && cc < ft.cols) const_cast<double*>(ft.p)[(size_t)rr * ft.ld + cc] = X[rr * LDS + cc];
  }
  if (digits) {
    __half* dst = p.digits + (size_t)slot * OZ_TILE;
    oz_store_digits_rows(dst, X, row0, ft.rows, ft.cols, erow_t);
    if (q == g.feeder_quarters(i, col) - 1)   // rows past the last group: zero digits
      for (int idx = threadIdx.x; idx < OZ_S * (TS - row0 - FEED_ROWS) * TS / 2; idx += NT) {
        const int per = (TS - row0 - FEED_ROWS) * TS / 2;
        const int sp = idx / per, w = idx % per;
        reinterpret_cast<unsigned*>(dst + sp * TS * TS + (row0 + FEED_ROWS) * TS)[w] = 0u;
      }
  }
  __syncthreads();
  trace_mark(c, t, 3);   // rows and digits written
  if (threadIdx.x == 0) {
    // The feeder's flag starts the launch at zero (launch_clear_feeders) and every row
    // group adds its share of the epoch with a release-add (no round trip): the flag
    // reads >= epoch exactly when all groups have written their rows.
    const int nq = g.feeder_quarters(i, col), share = c.epoch / nq;
    red_add_release(c.flags + slot, q < nq - 1 ? share : c.epoch - (nq - 1) * share);
  }
  trace_task(c, t, FT_FEEDQ, t_task0);
  return true;
}

// Stage the diagonal factor tile D_i(c, c) (identity padded) after waiting for it.
static __device__ bool load_diag_factor(const FactorArgs& p, int i, int c, double* F, int* s_ok) {
  if (!cta_wait(p.c, p.c.flags + p.g.fD(i, c, c), nullptr, s_ok)) return false;
  tile_load(F, btile(Dblk(p, i), p.g, c, c));
  __syncthreads();
  tile_pad_identity(F, p.g.vrows(c));
  __syncthreads();
  return true;
}

// X <- X * F^{-T} for the target of an off-diagonal task (F: the padded diagonal factor
// tile, rd: TS doubles).  An arrow tile has only a rows of the factor, so for a <= 16 the
// 8-row solve (lane = column, no barrier per column) runs on those rows alone; FS is a
// free tile of shared memory for the row-scaled copy of F it reads.
static __device__ __forceinline__ void offdiag_trsm(double* X, const double* F, double* FS, double* rd,
                                                    bool arrow, int a) {
  tile_diag_recip(F, rd);
  if (arrow && a <= 2 * FEED_ROWS) {
    __syncthreads();
    tile_scale_rows_by_recip(FS, F, rd);
    for (int row0 = 0; row0 < a; row0 += FEED_ROWS) smem_trsm_rlt_rows8(X, FS, rd, row0);
  } else {
    smem_trsm_rlt(X, F, rd);
  }
}

// Tip partial P = X X^T of an arrow tile (F is scratch), written for the tip task.
static __device__ __forceinline__ void arrow_tip_partial(const FactorArgs& p, int i, int col, const double* X,
                                                         double* F) {
  __syncthreads();
  for (int idx = threadIdx.x; idx < TS * TS; idx += NT) F[(idx % TS) * LDS + idx / TS] = X[(idx / TS) * LDS + idx % TS];
  __syncthreads();
  Acc pacc;
  acc_zero(pacc);
  tile_mma<false>(pacc, X, F);
  double* P = p.tip_part + (size_t)(i * p.g.B + col) * TS * TS;
#pragma unroll
  for (int ii = 0; ii < 2; ++ii)
#pragma unroll
    for (int q = 0; q < 4; ++q) P[acc_row(ii) * TS + acc_col(q)] = pacc.v[ii][q];
}

// Shared memory of the FP64 factor task: 4 tiles (K-loop double buffer; the target X
// and the diagonal factor F alias its first two, used only before / after the loop),
// TS pivots, and the wait flag.
constexpr size_t FP64F_SMEM = 4 * TILE_SMEM * sizeof(double) + TS * sizeof(double);

// Task t of a FP64-product factorization instance.  `raw` is FP64F_SMEM bytes of
// shared memory.  Returns false when the launch is aborted.
static __device__ __forceinline__ bool factor_fp64_task(const FactorArgs& p, int t, unsigned char* raw, int* s_okp) {
  double* sm = reinterpret_cast<double*>(raw);
  double* vec = sm + 4 * TILE_SMEM;     // pivots' 1/sqrt, or reciprocals of a factor tile's diagonal
  double* bufs = sm;
  double* X = sm;
  double* F = sm + TILE_SMEM;
  int& s_ok = *s_okp;
  const Geom& g = p.g;
  const Ctl& c = p.c;
  int* info_slot = p.info ? p.info : c.ctrl + CTRL_INFO;
  {
    const unsigned long long t_task0 = c.trace ? gtimer() : 0ull;
    const int4 tk = p.tasks[t];
    const int type = tk.x & 7, i = tk.y, r = tk.z, col = tk.w;
    const bool pre_only = (tk.x & FT_PRE) != 0;
    // split loops (FT_PART / FT_TAIL on a diagonal task or a feeder's FT_PRE task)
    const int dmode = (tk.x & FT_PART) ? 1 : ((tk.x & FT_TAIL) ? 2 : 0);
    int* part_flag = (type == FT_DIAG ? p.diag_pre : p.diag_pre + g.nt * g.B) + i * g.B + col;
    if (!p.use_arrow && (type == FT_ARW || type == FT_TIP)) return true;
    if (type == FT_FEEDQ) return factor_feed_rows(p, t, i, r, col, X, F, sm + 2 * TILE_SMEM, vec, nullptr, &s_ok, t_task0);

    Acc acc;
    if (type == FT_TIP) {
      // T -= sum_{i,c} R_i(c) R_i(c)^T in a fixed order, then chol(T) (a <= TS).
      tile_load(X, make_tile(p.T, g.a, 0, 0, g.a, g.a));
      __syncthreads();
      acc_from_smem(acc, X);
      bool ok = true;
      for (int k = 0; k < g.nt * g.B && ok; ++k) {
        ok = cta_wait_plus(c, c.flags + g.fR(k / g.B, k % g.B), 1, &s_ok);   // partial written
        if (!ok) break;
        const double* P = p.tip_part + (size_t)k * TS * TS;
#pragma unroll
        for (int ii = 0; ii < 2; ++ii)
#pragma unroll
          for (int q = 0; q < 4; ++q) acc.v[ii][q] -= __ldcg(P + acc_row(ii) * TS + acc_col(q));
      }
      if (!ok) return false;
      acc_to_smem(acc, X);
      __syncthreads();
      for (int idx = threadIdx.x; idx < TS * TS; idx += NT) {   // zero padding, identity diagonal
        const int rr = idx / TS, cc = idx % TS;
        if (rr >= g.a || cc >= g.a) X[rr * LDS + cc] = (rr == cc) ? 1.0 : 0.0;
      }
      const int info = smem_potrf(X);
      if (info) {
        if (threadIdx.x == 0) {
          atomicCAS(info_slot, 0, g.nt * g.b + info);
          raise_abort(c);
        }
        return false;
      }
      tile_store(p.T, g.a, g.a, g.a, X);
      cta_publish(c, c.flags + g.fT());
      trace_task(c, t, type, t_task0);
      return true;
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
      tgt_blk = Lblk(p, g.lslot(i));
      tgt = btile(tgt_blk, g, r, col);
      tgt_flag = c.flags + g.fL(g.lslot(i), r, col);
    } else {   // FT_ARW
      tgt_blk = Rblk(p, i);
      tgt = atile(tgt_blk, g, col);
      tgt_flag = c.flags + g.fR(i, col);
    }
    // a tail starts from the partial its FT_PART task stored
    if (dmode == 2 && !cta_wait(c, part_flag, nullptr, &s_ok)) return false;
    tile_load(X, tgt);
    __syncthreads();
    acc_from_smem(acc, X);
    __syncthreads();

    // previous block columns: the Schur terms of the (one or two) neighbours eliminated
    // before block i, through their coupling slots (L tiles have none: Q(nxt(i), p) = 0)
    const StepRange sr = step_range(p, type, dmode, i, r, col);
    const int nsteps = sr.n;
    const int lsi = g.lslot(i);
    auto step_of = [&](int s) -> Step {
      Step st;
      st.ta = false;
      st.tb = true;
      bool isprev;
      int pb, k;
      step_src(g, sr, i, s, isprev, pb, k);
      if (isprev) {
        const int ls = g.lslot(pb);
        if (type == FT_ARW) {
          st.a = atile(Rblk(p, pb), g, k);
          st.fa = c.flags + g.fR(pb, k);
        } else {
          st.a = btile(Lblk(p, ls), g, r, k);
          st.fa = c.flags + g.fL(ls, r, k);
        }
        st.b = btile(Lblk(p, ls), g, col, k);
        st.fb = c.flags + g.fL(ls, col, k);
      } else {           // within the block column: tiles k < col of the same row
        if (type == FT_ARW) {
          st.a = atile(Rblk(p, i), g, k);
          st.fa = c.flags + g.fR(i, k);
        } else if (type == FT_LOW) {
          st.a = btile(Lblk(p, lsi), g, r, k);
          st.fa = c.flags + g.fL(lsi, r, k);
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
    if (!kloop<true>(acc, nsteps, step_of, c, bufs, &s_ok)) return false;
    acc_to_smem(acc, X);
    __syncthreads();

    if (dmode == 1) {   // a partial: stored for its tail task
      tile_store(const_cast<double*>(tgt.p), tgt.ld, tgt.rows, tgt.cols, X);
      cta_publish(c, part_flag);
      trace_task(c, t, type, t_task0);
      return true;
    }
    if (pre_only) {   // feeder products: the FT_FEEDQ tasks finish the tile
      tile_store(const_cast<double*>(tgt.p), tgt.ld, tgt.rows, tgt.cols, X);
      cta_publish(c, p.feed_pre + i * g.B + col);
      if (type == FT_OFFD) {
        const Tile up = btile(Dblk(p, i), g, col, r);
        tile_store_zero(const_cast<double*>(up.p), g.b, up.rows, up.cols);
      }
      trace_task(c, t, type, t_task0);
      return true;
    }

    if (type == FT_DIAG) {
      tile_pad_identity(X, g.vrows(col));
      const int info = smem_potrf(X);
      if (info) {
        if (threadIdx.x == 0) {
          atomicCAS(info_slot, 0, i * g.b + col * TS + info);
          raise_abort(c);
        }
        return false;
      }
      tile_store(const_cast<double*>(tgt.p), g.b, tgt.rows, tgt.cols, X);
      cta_publish(c, tgt_flag);
      trace_task(c, t, type, t_task0);
      return true;
    }

    // Off-diagonal targets: X <- X * D_i(col,col)^{-T}; a structurally zero coupling tile
    // (no products, zero input) stays zero without the solve, so without its wait.
    if (!(type == FT_LOW && col < kfirst(p, lsi, r))) {
      if (!load_diag_factor(p, i, col, F, &s_ok)) return false;
      offdiag_trsm(X, F, sm + 2 * TILE_SMEM, vec, type == FT_ARW, g.a);
    }
    tile_store(const_cast<double*>(tgt.p), tgt.ld, tgt.rows, tgt.cols, X);
    if (type == FT_OFFD) {
      // The factor's strict upper triangle is zero: clear the mirrored tile.
      const Tile up = btile(Dblk(p, i), g, col, r);
      tile_store_zero(const_cast<double*>(up.p), g.b, up.rows, up.cols);
    }
    cta_publish(c, tgt_flag);
    if (type == FT_ARW) {
      // The next arrow tile of the row needs this one: the tip partial P = X X^T comes
      // after the publication and raises the flag by one when written (the tip task
      // consumes the partials in order).
      arrow_tip_partial(p, i, col, X, F);
      cta_raise(tgt_flag, 1);
    }
    trace_task(c, t, type, t_task0);
  }
  return true;
}

// dynamic shared memory layout
constexpr int OZF_STAGE_HALVES = 2 * OZ_OPER;   // A and B operand of one stage
constexpr size_t OZF_SMEM = 2 * OZF_STAGE_HALVES * sizeof(__half) + 2 * TILE_SMEM * sizeof(double) +
                            TS * sizeof(double) + 2 * TS * sizeof(int);

// Shared-memory views of one CTA (carved from the dynamic buffer by oz_factor_smem).
struct OzFactorSmem {
  __half* stages;
  double* X;
  double* F;
  double* vec;
  int* erow_t;   // exponents of the target's rows
  int* ecol_t;   // exponents of the target's columns
  int* s_ok;
  int* s_ready;
  OzPipe* pipe;   // bulk-copy barriers of the two stage buffers
};

static __device__ __forceinline__ OzFactorSmem oz_factor_smem(unsigned char* raw, int* s_ok, int* s_ready,
                                                              OzPipe* pipe) {
  OzFactorSmem m;
  m.pipe = pipe;
  m.stages = reinterpret_cast<__half*>(raw);
  m.X = reinterpret_cast<double*>(raw + 2 * OZF_STAGE_HALVES * sizeof(__half));
  m.F = m.X + TILE_SMEM;
  m.vec = m.F + TILE_SMEM;
  m.erow_t = reinterpret_cast<int*>(m.vec + TS);
  m.ecol_t = m.erow_t + TS;
  m.s_ok = s_ok;
  m.s_ready = s_ready;
  return m;
}

// Task t of the instance described by p.  Returns false when the launch is aborted
// (a failed pivot or a wait that ran out).
static __device__ __forceinline__ bool factor_oz_task(const FactorArgs& p, int t, const OzFactorSmem& sm) {
  __half* stages = sm.stages;
  double* X = sm.X;
  double* F = sm.F;
  double* vec = sm.vec;
  int* erow_t = sm.erow_t;
  int* ecol_t = sm.ecol_t;
  int& s_ok = *sm.s_ok;
  int& s_ready = *sm.s_ready;
  const Geom& g = p.g;
  const Ctl& c = p.c;
  int* info_slot = p.info ? p.info : c.ctrl + CTRL_INFO;
  {
    const unsigned long long t_task0 = c.trace ? gtimer() : 0ull;
    const int4 tk = p.tasks[t];
    const int type = tk.x & 7, i = tk.y, r = tk.z, col = tk.w;
    const bool pre_only = (tk.x & FT_PRE) != 0;
    // split loops (FT_PART / FT_TAIL on a diagonal task or a feeder's FT_PRE task)
    const int dmode = (tk.x & FT_PART) ? 1 : ((tk.x & FT_TAIL) ? 2 : 0);
    int* part_flag = (type == FT_DIAG ? p.diag_pre : p.diag_pre + g.nt * g.B) + i * g.B + col;
    if (!p.use_arrow && (type == FT_ARW || type == FT_TIP)) return true;
    if (type == FT_FEEDQ)
      return factor_feed_rows(p, t, i, r, col, X, F, reinterpret_cast<double*>(stages), vec, erow_t, &s_ok, t_task0);
    const size_t bb = (size_t)g.b * g.b, ab = (size_t)g.a * g.b;

    if (type == FT_TIP) {
      // T -= sum_{i,c} R_i(c) R_i(c)^T in a fixed order, then chol(T) (a <= TS).
      Acc acc;
      tile_load(X, make_tile(p.T, g.a, 0, 0, g.a, g.a));
      __syncthreads();
      acc_from_smem(acc, X);
      bool ok = true;
      for (int k = 0; k < g.nt * g.B && ok; ++k) {
        ok = cta_wait_plus(c, c.flags + g.fR(k / g.B, k % g.B), 1, &s_ok);   // partial written
        if (!ok) break;
        const double* P = p.tip_part + (size_t)k * TS * TS;
#pragma unroll
        for (int ii = 0; ii < 2; ++ii)
#pragma unroll
          for (int q = 0; q < 4; ++q) acc.v[ii][q] -= __ldcg(P + acc_row(ii) * TS + acc_col(q));
      }
      if (!ok) return false;
      acc_to_smem(acc, X);
      __syncthreads();
      for (int idx = threadIdx.x; idx < TS * TS; idx += NT) {
        const int rr = idx / TS, cc = idx % TS;
        if (rr >= g.a || cc >= g.a) X[rr * LDS + cc] = (rr == cc) ? 1.0 : 0.0;
      }
      const int info = smem_potrf(X);
      if (info) {
        if (threadIdx.x == 0) {
          atomicCAS(info_slot, 0, g.nt * g.b + info);
          raise_abort(c);
        }
        return false;
      }
      tile_store(p.T, g.a, g.a, g.a, X);
      cta_publish(c, c.flags + g.fT());
      trace_task(c, t, type, t_task0);
      return true;
    }

    // ---- target tile, its flag / digit slot, and the global rows of its rows
    Tile tgt;
    int tgt_slot;
    long long row_base;
    if (type == FT_DIAG || type == FT_OFFD) {
      tgt = make_tile(p.D + i * bb, g.b, r * TS, col * TS, g.b, g.b);
      tgt_slot = g.fD(i, r, col);
      row_base = (long long)i * g.b + r * TS;
    } else if (type == FT_LOW) {
      tgt = make_tile(p.L + g.lslot(i) * bb, g.b, r * TS, col * TS, g.b, g.b);
      tgt_slot = g.fL(g.lslot(i), r, col);
      row_base = (long long)g.nxt(i) * g.b + r * TS;
    } else {
      tgt = make_tile(p.R + i * ab, g.b, 0, col * TS, g.a, g.b);
      tgt_slot = g.fR(i, col);
      row_base = (long long)g.nt * g.b;
    }
    const long long col_base = (long long)i * g.b + col * TS;   // rows of the diagonal tile (i, col)
    if (threadIdx.x < TS) {
      erow_t[threadIdx.x] = (threadIdx.x < tgt.rows) ? p.erow[row_base + threadIdx.x] : 0;
      ecol_t[threadIdx.x] = (threadIdx.x < tgt.cols) ? p.erow[col_base + threadIdx.x] : 0;
    }
    // a tail starts from the partial its FT_PART task stored
    if (dmode == 2 && !cta_wait(c, part_flag, nullptr, &s_ok)) return false;
    tile_load(X, tgt);
    __syncthreads();
    OzAcc acc;
    int esum[2][4];
#pragma unroll
    for (int n = 0; n < 2; ++n)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        acc.v[n][j] = X[oz_row(n, j) * LDS + oz_col(n, j)];
        esum[n][j] = erow_t[oz_row(n, j)] + ecol_t[oz_col(n, j)];
      }
    oz_clear_partials(acc);

    // ---- product loop over the final tiles left of the target (previous block
    //      column first, then columns k < col of this block)
    const StepRange sr = step_range(p, type, dmode, i, r, col);
    const int nsteps = sr.n;
    const int lsi = g.lslot(i);
    auto slots = [&](int s, int& sa, int& sb) {
      bool isprev;
      int pb, k;
      step_src(g, sr, i, s, isprev, pb, k);
      if (isprev) {
        const int ls = g.lslot(pb);
        sa = (type == FT_ARW) ? g.fR(pb, k) : g.fL(ls, r, k);
        sb = g.fL(ls, col, k);
      } else {
        sa = (type == FT_ARW) ? g.fR(i, k) : (type == FT_LOW) ? g.fL(lsi, r, k) : g.fD(i, r, k);
        sb = g.fD(i, col, k);
      }
    };
    bool ok = true;
    OzPipe* pp = sm.pipe;
    unsigned ph = pp->phase;
    unsigned long long t_alldeps = 0;   // (trace) when the last operand was known ready
    // stage the operand tiles (slots a, b) of a step into stage buffer st (bulk copies)
    auto stage = [&](int st, int a_slot, int b_slot) {
      if (threadIdx.x == 0) {
        __half* dst = stages + st * OZF_STAGE_HALVES;
        constexpr unsigned tb = (unsigned)(OZ_TILE * sizeof(__half));
        oz_bulk_expect(pp, st, 2 * tb);
        oz_bulk_copy(pp, st, dst, p.digits + (size_t)a_slot * OZ_TILE, tb);
        oz_bulk_copy(pp, st, dst + OZ_OPER, p.digits + (size_t)b_slot * OZ_TILE, tb);
      }
    };
    if (nsteps > 0) {
      auto flags_of = [&](int s, const int*& f0, const int*& f1) {
        int sa, sb;
        slots(s, sa, sb);
        f0 = c.flags + sa;
        f1 = (sa == sb) ? nullptr : c.flags + sb;
      };
      int sa, sb;
      slots(0, sa, sb);
      ok = cta_wait(c, c.flags + sa, sa == sb ? nullptr : c.flags + sb, &s_ok);
      if (ok) {
        if (threadIdx.x == 0) s_ready = 1;
        stage(0, sa, sb);
      }
      for (int s = 0; s < nsteps && ok; ++s) {
        __half* cur = stages + (s & 1) * OZF_STAGE_HALVES;
        const int nst = (s + 1) & 1;
        {   // stage s has landed; the barrier frees stage s-1's buffers
          const bool late = !oz_stage_wait(pp, s & 1, ph);
          if (__syncthreads_or(late)) {
            if (threadIdx.x == 0) {
              atomicCAS(c.ctrl + CTRL_ERR, ERR_NONE, ERR_TIMEOUT);
              raise_abort(c);
            }
            oz_stage_wait(pp, s & 1, ph);   // one more bounded wait for the copy before leaving
            ok = false;
            break;
          }
        }
        const bool more = s + 1 < nsteps;
        bool issued = false;
        int na = 0, nb = 0;
        if (more) {
          if (s_ready <= s + 1) {   // uniform: read after the barrier, rewritten after the next one
            __syncthreads();   // every warp has read s_ready before warp 0 advances it
            scan_ready(c, nsteps, flags_of, &s_ready);
            __syncthreads();
            if (c.trace && s_ready >= nsteps && !t_alldeps) t_alldeps = gtimer();
          }
          if (s_ready > s + 1) {
            slots(s + 1, na, nb);
            stage(nst, na, nb);
            issued = true;
          }
        }
        oz_step(acc, cur, cur + OZ_OPER);
        if ((s + 1) % OZ_CHUNK == 0) oz_fold_sub(acc, esum);   // (the last fold follows the loop)
        if (more && !issued) {
          slots(s + 1, na, nb);
          if (!(ok = cta_wait(c, c.flags + na, na == nb ? nullptr : c.flags + nb, &s_ok))) break;
          if (threadIdx.x == 0) s_ready = s + 2;
          if (c.trace && s + 2 >= nsteps) t_alldeps = gtimer();
          stage(nst, na, nb);
        }
      }
    }
    if (!ok) return false;   // no copy is in flight here
    {
      // the steps since the last fold, folded out of the loop: the short form when there
      // are at most OZ_SHORT of them (a diagonal tail's last fold is on the column chain)
      const int rest = nsteps % OZ_CHUNK;
      if (rest != 0) {
        if (rest <= OZ_SHORT)
          oz_fold_sub_short(acc, esum);
        else
          oz_fold_sub(acc, esum);
      }
    }
    if (threadIdx.x == 0) pp->phase = ph;
    count_pairs(c, (unsigned long long)nsteps * oz_pairs_from(0, 0));
    __syncthreads();
    trace_clear_marks(c, t);
    trace_mark(c, t, 0);   // product loop done
    trace_put(c, t, 3, (long long)t_alldeps);   // last operand ready
#pragma unroll
    for (int n = 0; n < 2; ++n)
#pragma unroll
      for (int j = 0; j < 4; ++j) X[oz_row(n, j) * LDS + oz_col(n, j)] = acc.v[n][j];
    __syncthreads();

    if (dmode == 1) {   // a partial: stored for its tail task
      tile_store(const_cast<double*>(tgt.p), tgt.ld, tgt.rows, tgt.cols, X);
      cta_publish(c, part_flag);
      trace_task(c, t, type, t_task0);
      return true;
    }
    if (pre_only) {   // feeder products: the FT_FEEDQ tasks finish the tile and its digits
      tile_store(const_cast<double*>(tgt.p), tgt.ld, tgt.rows, tgt.cols, X);
      cta_publish(c, p.feed_pre + i * g.B + col);
      if (type == FT_OFFD) {
        const Tile up = make_tile(p.D + i * bb, g.b, col * TS, r * TS, g.b, g.b);
        tile_store_zero(const_cast<double*>(up.p), g.b, up.rows, up.cols);
      }
      trace_task(c, t, type, t_task0);
      return true;
    }

    if (type == FT_DIAG) {
      tile_pad_identity(X, g.vrows(col));
      const int info = smem_potrf(X);
      if (info) {
        if (threadIdx.x == 0) {
          atomicCAS(info_slot, 0, i * g.b + col * TS + info);
          raise_abort(c);
        }
        return false;
      }
      trace_mark(c, t, 1);   // tile factored
      // (diagonal tiles are never operands of the product loops: no digit planes)
      tile_store(const_cast<double*>(tgt.p), g.b, tgt.rows, tgt.cols, X);
      trace_mark(c, t, 2);   // tile written
      cta_publish(c, c.flags + tgt_slot);
      trace_task(c, t, type, t_task0);
      return true;
    }

    // Off-diagonal targets: X <- X * D_i(col,col)^{-T}; a structurally zero coupling tile
    // (no products, zero input) stays zero without the solve, so without its wait.
    if (!(type == FT_LOW && col < kfirst(p, lsi, r))) {
      if (!cta_wait(c, c.flags + g.fD(i, col, col), nullptr, &s_ok)) return false;
      trace_mark(c, t, 1);   // diagonal factor tile ready
      tile_load(F, make_tile(p.D + i * bb, g.b, col * TS, col * TS, g.b, g.b));
      __syncthreads();
      tile_pad_identity(F, g.vrows(col));
      __syncthreads();
      offdiag_trsm(X, F, reinterpret_cast<double*>(stages), vec, type == FT_ARW, g.a);
      trace_mark(c, t, 2);   // triangular solve done
    }
    tile_store(const_cast<double*>(tgt.p), tgt.ld, tgt.rows, tgt.cols, X);
    oz_store_digits(p.digits + (size_t)tgt_slot * OZ_TILE, X, tgt.rows, tgt.cols, erow_t);
    trace_mark(c, t, 3);   // tile and digits written
    cta_publish(c, c.flags + tgt_slot);
    if (type == FT_ARW) {   // tip partial after the publication, as in factor_fp64_task
      arrow_tip_partial(p, i, col, X, F);
      cta_raise(c.flags + tgt_slot, 1);
    }
    if (type == FT_OFFD) {
      // The factor's strict upper triangle is zero: clear the mirrored tile (read by
      // no task of the factorization, so after the publication).
      const Tile up = make_tile(p.D + i * bb, g.b, col * TS, r * TS, g.b, g.b);
      tile_store_zero(const_cast<double*>(up.p), g.b, up.rows, up.cols);
    }
    trace_task(c, t, type, t_task0);
  }
  return true;
}

}  // namespace gbta
