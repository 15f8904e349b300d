// BTA Cholesky factorization with tensor-core products (see bta_ozaki.cuh).
//
// Same task DAG, ordering and epilogues as k_factor (bta_factor.cu): one task
// finalises one 32 x 32 tile of D_i (lower), L_i or R_i.  The difference is the
// left-looking product loop: instead of FP64 FMAs on the FP64 tiles it streams the
// tiles' digit planes (written by the tasks that finalised them) through mma.sync
// with exact fp32 accumulation, folding into FP64 every OZ_CHUNK steps.  Tile
// factorizations (POTRF), triangular solves (TRSM) and the arrow-tip partials stay
// in FP64.  The per-row exponents come from the input matrix's diagonal
// (k_row_exponents), computed before the factorization overwrites it.
#include "bta_ozaki.cuh"

namespace gbta {

struct FactorOzArgs {
  double* D;
  double* L;
  double* R;
  double* T;
  Geom g;
  int use_arrow;
  const int4* tasks;
  int ntasks;
  double* tip_part;
  __half* digits;      // [nflags][OZ_TILE]
  const int* erow;     // [nt*b + a] row exponents
  Ctl c;
};

__global__ void k_row_exponents(const double* D, const double* T, Geom g, int use_arrow, int* erow) {
  const long long n = (long long)g.nt * g.b + (use_arrow ? g.a : 0);
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    double q;
    if (e < (long long)g.nt * g.b) {
      const long long i = e / g.b, r = e % g.b;
      q = D[(i * g.b + r) * g.b + r];
    } else {
      const long long r = e - (long long)g.nt * g.b;
      q = T[r * g.a + r];
    }
    erow[e] = oz_row_exponent(q);
  }
}

// dynamic shared memory layout
constexpr int OZF_STAGE_HALVES = 2 * OZ_OPER;   // A and B operand of one stage
constexpr size_t OZF_SMEM = 2 * OZF_STAGE_HALVES * sizeof(__half) + 2 * TILE_SMEM * sizeof(double) +
                            TS * sizeof(double) + 2 * TS * sizeof(int);

__global__ void __launch_bounds__(NT, 1) k_factor_oz(FactorOzArgs p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __half* stages = reinterpret_cast<__half*>(smem_raw);
  double* X = reinterpret_cast<double*>(smem_raw + 2 * OZF_STAGE_HALVES * sizeof(__half));
  double* F = X + TILE_SMEM;
  double* vec = F + TILE_SMEM;
  int* erow_t = reinterpret_cast<int*>(vec + TS);   // exponents of the target's rows
  int* ecol_t = erow_t + TS;                        // exponents of the target's columns
  __shared__ int s_ok, s_t, s_ready;
  const Geom& g = p.g;
  const Ctl& c = p.c;

  while (true) {
    const int t = cta_ticket(c, &s_t);
    if (t < 0 || t >= p.ntasks) break;
    const unsigned long long t_task0 = c.trace ? gtimer() : 0ull;
    const int4 tk = p.tasks[t];
    const int type = tk.x, i = tk.y, r = tk.z, col = tk.w;
    if (!p.use_arrow && (type == FT_ARW || type == FT_TIP)) continue;
    const size_t bb = (size_t)g.b * g.b, ab = (size_t)g.a * g.b;

    if (type == FT_TIP) {
      // T -= sum_{i,c} R_i(c) R_i(c)^T in a fixed order, then chol(T) (a <= TS).
      Acc acc;
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
      for (int idx = threadIdx.x; idx < TS * TS; idx += NT) {
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

    // ---- target tile, its flag / digit slot, and the global rows of its rows
    Tile tgt;
    int tgt_slot;
    long long row_base;
    if (type == FT_DIAG || type == FT_OFFD) {
      tgt = make_tile(p.D + i * bb, g.b, r * TS, col * TS, g.b, g.b);
      tgt_slot = g.fD(i, r, col);
      row_base = (long long)i * g.b + r * TS;
    } else if (type == FT_LOW) {
      tgt = make_tile(p.L + i * bb, g.b, r * TS, col * TS, g.b, g.b);
      tgt_slot = g.fL(i, r, col);
      row_base = (long long)(i + 1) * g.b + r * TS;
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
    const bool prev = (i > 0) && (type != FT_LOW);
    const int nprev = prev ? g.B : 0;
    const int nsteps = nprev + col;
    auto slots = [&](int s, int& sa, int& sb) {
      if (s < nprev) {
        const int k = s;
        sa = (type == FT_ARW) ? g.fR(i - 1, k) : g.fL(i - 1, r, k);
        sb = g.fL(i - 1, col, k);
      } else {
        const int k = s - nprev;
        sa = (type == FT_ARW) ? g.fR(i, k) : (type == FT_LOW) ? g.fL(i, r, k) : g.fD(i, r, k);
        sb = g.fD(i, col, k);
      }
    };
    bool ok = true;
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
        oz_load_async(stages, p.digits + (size_t)sa * OZ_TILE);
        oz_load_async(stages + OZ_OPER, p.digits + (size_t)sb * OZ_TILE);
        cp_async_commit();
      }
      for (int s = 0; s < nsteps && ok; ++s) {
        __half* cur = stages + (s & 1) * OZF_STAGE_HALVES;
        __half* nxt = stages + ((s + 1) & 1) * OZF_STAGE_HALVES;
        cp_async_wait_all();
        __syncthreads();   // stage s is in shared memory; stage s-1 buffers are free
        const bool more = s + 1 < nsteps;
        bool issued = false;
        int na = 0, nb = 0;
        if (more) {
          if (s_ready <= s + 1) {   // uniform: read after the barrier
            scan_ready(c, nsteps, flags_of, &s_ready);
            __syncthreads();
          }
          if (s_ready > s + 1) {
            slots(s + 1, na, nb);
            oz_load_async(nxt, p.digits + (size_t)na * OZ_TILE);
            oz_load_async(nxt + OZ_OPER, p.digits + (size_t)nb * OZ_TILE);
            cp_async_commit();
            issued = true;
          }
        }
        oz_step(acc, cur, cur + OZ_OPER);
        if ((s + 1) % OZ_CHUNK == 0 || !more) oz_fold_sub(acc, esum);
        if (more && !issued) {
          slots(s + 1, na, nb);
          if (!(ok = cta_wait(c, c.flags + na, na == nb ? nullptr : c.flags + nb, &s_ok))) break;
          if (threadIdx.x == 0) s_ready = s + 2;
          oz_load_async(nxt, p.digits + (size_t)na * OZ_TILE);
          oz_load_async(nxt + OZ_OPER, p.digits + (size_t)nb * OZ_TILE);
          cp_async_commit();
        }
      }
    }
    if (!ok) {
      cp_async_wait_all();
      break;
    }
    __syncthreads();
#pragma unroll
    for (int n = 0; n < 2; ++n)
#pragma unroll
      for (int j = 0; j < 4; ++j) X[oz_row(n, j) * LDS + oz_col(n, j)] = acc.v[n][j];
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
      oz_store_digits(p.digits + (size_t)tgt_slot * OZ_TILE, X, tgt.rows, tgt.cols, erow_t);
      cta_publish(c, c.flags + tgt_slot);
      trace_task(c, t, type, t_task0);
      continue;
    }

    // Off-diagonal targets: X <- X * D_i(col,col)^{-T}.
    if (!cta_wait(c, c.flags + g.fD(i, col, col), nullptr, &s_ok)) break;
    tile_load(F, make_tile(p.D + i * bb, g.b, col * TS, col * TS, g.b, g.b));
    __syncthreads();
    tile_pad_identity(F, g.vrows(col));
    __syncthreads();
    tile_diag_recip(F, vec);
    smem_trsm_rlt(X, F, vec);
    tile_store(const_cast<double*>(tgt.p), tgt.ld, tgt.rows, tgt.cols, X);
    oz_store_digits(p.digits + (size_t)tgt_slot * OZ_TILE, X, tgt.rows, tgt.cols, erow_t);
    if (type == FT_OFFD) {
      const Tile up = make_tile(p.D + i * bb, g.b, col * TS, r * TS, g.b, g.b);
      tile_store_zero(const_cast<double*>(up.p), g.b, up.rows, up.cols);
    }
    if (type == FT_ARW) {
      // tip partial P = X X^T in FP64 (consumed in order by the tip task)
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
    cta_publish(c, c.flags + tgt_slot);
    trace_task(c, t, type, t_task0);
  }
}

size_t factor_oz_digit_bytes(const Geom& g) { return (size_t)g.nflags() * OZ_TILE * sizeof(__half); }

void launch_factor_oz(const Geom& g, double* D, double* L, double* R, double* T, int use_arrow, const int4* tasks,
                      int ntasks, double* tip_part, __half* digits, int* erow, const LaunchCtl& lc) {
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(k_factor_oz, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)OZF_SMEM);
    attr_set = true;
  }
  const long long n = (long long)g.nt * g.b + (use_arrow ? g.a : 0);
  k_row_exponents<<<(unsigned)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096), 256, 0, lc.stream>>>(D, T, g, use_arrow,
                                                                                                      erow);
  FactorOzArgs p;
  p.D = D;
  p.L = L;
  p.R = R;
  p.T = T;
  p.g = g;
  p.use_arrow = use_arrow;
  p.tasks = tasks;
  p.ntasks = ntasks;
  p.tip_part = tip_part;
  p.digits = digits;
  p.erow = erow;
  p.c.ctrl = lc.ctrl;
  p.c.flags = lc.flags;
  p.c.epoch = lc.epoch;
  p.c.wait_ns = lc.wait_ns;
  p.c.trace = lc.trace;
  k_factor_oz<<<lc.grid, NT, OZF_SMEM, lc.stream>>>(p);
  count_launches(2);
}

}  // namespace gbta
