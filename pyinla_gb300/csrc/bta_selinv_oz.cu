// BTA selected inversion with tensor-core products (see bta_ozaki.cuh).
//
// Same tile Takahashi DAG, ordering and epilogues as k_selinv (bta_selinv.cu); the
// product loops  Y = sum_l Sigma(j,l) F(l,c)  and  Z = sum_l Sigma(l,c)^T F(l,c)
// run on mma.sync with exact integer digit planes:
//  * right operand F(l,c): the factor is fixed during the inversion, so every tile
//    F(l,c) of every column pattern is sliced once (k_fac_digits_t) relative to
//    per-column exponents (k_fac_col_exponents: max over the column's pattern), and
//    stored transposed ([plane][column][row]) for the ldmatrix layout;
//  * left operand Sigma tiles: sliced while staged, relative to the task's running
//    exponent E (the largest tile exponent seen so far in the task); when a tile
//    raises E, the exact partial sums are first folded into FP64 with the old E.
// Tile inverses and triangular solves of the epilogues stay in FP64.
#include "bta_ozaki.cuh"

namespace gbta {

struct SelinvOzArgs {
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
  const __half* fdig;   // transposed factor digits per flag slot
  const int* ecol;      // per global column (nt*b) exponent of the factor column pattern
  Ctl c;
};

// ---- pattern helpers (same as bta_selinv.cu) ---------------------------------------
struct SigTileOz {
  Tile t;
  bool trans;
  const int* flag;
};

__device__ SigTileOz sig_tile_oz(const SelinvOzArgs& p, int i, int j, int l) {
  const Geom& g = p.g;
  const int B = g.B, A = 2 * B;
  const size_t bb = (size_t)g.b * g.b, ab = (size_t)g.a * g.b;
  const int* F = p.c.flags;
  SigTileOz s;
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
  } else if (j < B && l < B) {
    const int hi = max(j, l), lo = min(j, l);
    s.t = make_tile(p.SD + i * bb, g.b, hi * TS, lo * TS, g.b, g.b);
    s.trans = j < l;
    s.flag = F + g.fD(i, hi, lo);
  } else if (j >= B && l >= B) {
    const int hi = max(j, l) - B, lo = min(j, l) - B;
    s.t = make_tile(p.SD + (i + 1) * bb, g.b, hi * TS, lo * TS, g.b, g.b);
    s.trans = j < l;
    s.flag = F + g.fD(i + 1, hi, lo);
  } else {
    const int rl = (j >= B ? j : l) - B, cd = (j >= B ? l : j);
    s.t = make_tile(p.SL + i * bb, g.b, rl * TS, cd * TS, g.b, g.b);
    s.trans = j < B;
    s.flag = F + g.fL(i, rl, cd);
  }
  return s;
}

__device__ __forceinline__ SigTileOz sig_dest_oz(const SelinvOzArgs& p, int i, int j, int c) {
  const Geom& g = p.g;
  const size_t bb = (size_t)g.b * g.b, ab = (size_t)g.a * g.b;
  const int B = g.B;
  SigTileOz s;
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

// flag slot of the factor tile F(l, c) of block column i
__device__ __forceinline__ int fac_slot(const Geom& g, int i, int l, int c) {
  const int B = g.B;
  if (l == 2 * B) return g.fR(i, c);
  if (l >= B) return g.fL(i, l - B, c);
  return g.fD(i, l, c);
}
__device__ __forceinline__ int pat_size_oz(const SelinvOzArgs& p, int i, int c) {
  return (p.use_arrow ? 1 : 0) + (i < p.g.nt - 1 ? p.g.B : 0) + (p.g.B - 1 - c);
}
__device__ __forceinline__ int pat_code_oz(const SelinvOzArgs& p, int i, int c, int s) {
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

// ---- pre-passes over the factor ---------------------------------------------------
// One CTA per (block i, column tile c): ecol[i*b + c*TS + j] = exponent of
// max |F(m, j)| over the rows m of the column's pattern (D_i below tile c, L_i, R_i).
__global__ void __launch_bounds__(NT) k_fac_col_exponents(const double* D, const double* L, const double* R, Geom g,
                                                          int use_arrow, int* ecol) {
  __shared__ double red[NT];
  const int ic = blockIdx.x;
  const int i = ic / g.B, c = ic % g.B;
  const size_t bb = (size_t)g.b * g.b, ab = (size_t)g.a * g.b;
  const int j = threadIdx.x % TS, r0 = threadIdx.x / TS;   // 4 row groups
  const int col = c * TS + j;
  double m = 0.0;
  if (col < g.b) {
    for (int row = (c + 1) * TS + r0; row < g.b; row += NT / TS) m = fmax(m, fabs(D[i * bb + (size_t)row * g.b + col]));
    if (i < g.nt - 1)
      for (int row = r0; row < g.b; row += NT / TS) m = fmax(m, fabs(L[i * bb + (size_t)row * g.b + col]));
    if (use_arrow)
      for (int row = r0; row < g.a; row += NT / TS) m = fmax(m, fabs(R[i * ab + (size_t)row * g.b + col]));
  }
  red[threadIdx.x] = m;
  __syncthreads();
  if (threadIdx.x < TS) {
    double mm = fmax(fmax(red[threadIdx.x], red[threadIdx.x + TS]), fmax(red[threadIdx.x + 2 * TS], red[threadIdx.x + 3 * TS]));
    if (col < g.b) ecol[(size_t)i * g.b + col] = (mm > 0.0 && isfinite(mm)) ? ilogb(mm) + 1 : 0;
  }
}

// One CTA per flag slot that is a factor tile of some column pattern: digits relative
// to the column exponents, stored transposed: dst[s][j][m] = digit s of F[m][j].
__global__ void __launch_bounds__(NT) k_fac_digits_t(const double* D, const double* L, const double* R, Geom g,
                                                     int use_arrow, const int* ecol, __half* dig) {
  const int slot = blockIdx.x;
  const int B = g.B;
  const size_t bb = (size_t)g.b * g.b, ab = (size_t)g.a * g.b;
  int i, r, c;
  Tile t;
  if (slot < g.nt * B * B) {
    i = slot / (B * B);
    r = (slot / B) % B;
    c = slot % B;
    if (r <= c) return;
    t = make_tile(D + i * bb, g.b, r * TS, c * TS, g.b, g.b);
  } else if (slot < (2 * g.nt - 1) * B * B) {
    const int s2 = slot - g.nt * B * B;
    i = s2 / (B * B);
    r = (s2 / B) % B;
    c = s2 % B;
    t = make_tile(L + i * bb, g.b, r * TS, c * TS, g.b, g.b);
  } else if (slot < (2 * g.nt - 1) * B * B + g.nt * B) {
    if (!use_arrow) return;
    const int s3 = slot - (2 * g.nt - 1) * B * B;
    i = s3 / B;
    c = s3 % B;
    t = make_tile(R + i * ab, g.b, 0, c * TS, g.a, g.b);
  } else {
    return;
  }
  __half* dst = dig + (size_t)slot * OZ_TILE;
#pragma unroll
  for (int k = 0; k < PER_THREAD; ++k) {
    const int idx = threadIdx.x + k * NT;
    const int m = idx / TS, jj = idx % TS;   // element (m, jj) of the tile
    int d[OZ_S];
    if (m < t.rows && jj < t.cols) {
      oz_digits(t.p[(size_t)m * t.ld + jj], ecol[(size_t)i * g.b + c * TS + jj], d);
    } else {
#pragma unroll
      for (int s = 0; s < OZ_S; ++s) d[s] = 0;
    }
#pragma unroll
    for (int s = 0; s < OZ_S; ++s) dst[s * TS * TS + jj * TS + m] = __int2half_rn(d[s]);
  }
}

// ---- consumer-side slicing of a staged FP64 tile ------------------------------------
// CTA max |v| of the register-staged tile (all threads return it).
__device__ __forceinline__ double cta_absmax(const double (&v)[PER_THREAD], double* red4) {
  double m = 0.0;
#pragma unroll
  for (int k = 0; k < PER_THREAD; ++k) m = fmax(m, fabs(v[k]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red4[threadIdx.x >> 5] = m;
  __syncthreads();
  m = fmax(fmax(red4[0], red4[1]), fmax(red4[2], red4[3]));
  __syncthreads();
  return m;
}

// Write the digit planes of the register-staged tile relative to 2^E into the shared
// A operand ([plane][row][k], padded rows); trans: element (r, c) is A(c, r).
__device__ __forceinline__ void oz_slice_to_smem(__half* As, const double (&v)[PER_THREAD], int E, bool trans) {
#pragma unroll
  for (int k = 0; k < PER_THREAD; ++k) {
    const int idx = threadIdx.x + k * NT;
    const int r = idx / TS, c = idx % TS;
    const int row = trans ? c : r, kk = trans ? r : c;
    int d[OZ_S];
    oz_digits(v[k], E, d);
#pragma unroll
    for (int s = 0; s < OZ_S; ++s) As[s * OZ_PLANE + row * OZ_LD + kk] = __int2half_rn(d[s]);
  }
}

constexpr int OZS_STAGE = 2 * OZ_OPER;   // halves per stage (A, B)
constexpr size_t OZS_SMEM = 2 * OZS_STAGE * sizeof(__half) + 3 * TILE_SMEM * sizeof(double) + TS * sizeof(double) +
                            TS * sizeof(int) + 4 * sizeof(double);

__device__ __forceinline__ void oz_diag_finish(double* X, double* W, const double* F, const double* rd) {
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

__global__ void __launch_bounds__(NT, 1) k_selinv_oz(SelinvOzArgs p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __half* stages = reinterpret_cast<__half*>(smem_raw);
  double* X = reinterpret_cast<double*>(smem_raw + 2 * OZS_STAGE * sizeof(__half));
  double* F = X + TILE_SMEM;
  double* W = F + TILE_SMEM;
  double* rd = W + TILE_SMEM;
  int* ecol_t = reinterpret_cast<int*>(rd + TS);
  double* red4 = reinterpret_cast<double*>(ecol_t + TS);
  __shared__ int s_ok, s_t, s_ready;
  const Geom& g = p.g;
  const Ctl& c = p.c;

  while (true) {
    const int t = cta_ticket(c, &s_t);
    if (t < 0 || t >= p.ntasks) break;
    const unsigned long long t_task0 = c.trace ? gtimer() : 0ull;
    const int4 tk = p.tasks[t];
    const int type = tk.x, i = tk.y, j = tk.z, col = tk.w;
    if (!p.use_arrow && (type == ST_TIP || (type == ST_OFF && j == 2 * g.B))) continue;

    if (type == ST_TIP) {
      tile_load(F, make_tile(p.T, g.a, 0, 0, g.a, g.a));
      __syncthreads();
      tile_pad_identity(F, g.a);
      for (int idx = threadIdx.x; idx < TS * TS; idx += NT) X[idx / TS * LDS + idx % TS] = 0.0;
      __syncthreads();
      tile_diag_recip(F, rd);
      __syncthreads();
      oz_diag_finish(X, W, F, rd);
      tile_store(p.ST, g.a, g.a, g.a, X);
      cta_publish(c, c.flags + g.fT());
      trace_task(c, t, type, t_task0);
      continue;
    }

    const int np = pat_size_oz(p, i, col);
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
    int E = -100000;   // running exponent of the left operand (unset)
    int esum[2][4];
    auto set_esum = [&]() {
#pragma unroll
      for (int n = 0; n < 2; ++n)
#pragma unroll
        for (int q = 0; q < 4; ++q) esum[n][q] = E + ecol_t[oz_col(n, q)];
    };
    // step s: left tile (FP64) and right digits
    auto left_of = [&](int s) -> SigTileOz {
      const int l = pat_code_oz(p, i, col, s);
      if (type == ST_OFF) return sig_tile_oz(p, i, j, l);
      SigTileOz st_ = sig_dest_oz(p, i, l, col);   // Sigma(l, col), used transposed
      st_.trans = true;
      return st_;
    };
    auto right_of = [&](int s) -> const __half* {
      return p.fdig + (size_t)fac_slot(g, i, pat_code_oz(p, i, col, s), col) * OZ_TILE;
    };

    bool ok = true;
    double vreg[PER_THREAD];
    int since_fold = 0;
    auto flags_of = [&](int s, const int*& f0, const int*& f1) {
      f0 = left_of(s).flag;
      f1 = nullptr;
    };
    if (np > 0) {
      SigTileOz lt = left_of(0);
      ok = cta_wait(c, lt.flag, nullptr, &s_ok);
      if (ok) {
        if (threadIdx.x == 0) s_ready = 1;
        tile_ldg(vreg, lt.t);
        oz_load_async(stages + OZ_OPER, right_of(0));
        cp_async_commit();
        const double mx = cta_absmax(vreg, red4);
        if (mx > 0.0) E = ilogb(mx) + 1;
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
        SigTileOz nt_;
        if (more) {
          nt_ = left_of(s + 1);
          if (s_ready <= s + 1) {   // uniform: read after the barrier
            scan_ready(c, np, flags_of, &s_ready);
            __syncthreads();
          }
          if (s_ready > s + 1) {
            tile_ldg(vreg, nt_.t);
            oz_load_async(nxt + OZ_OPER, right_of(s + 1));
            cp_async_commit();
            have = true;
          }
        }
        oz_step(acc, cur, cur + OZ_OPER);
        ++since_fold;
        if (more) {
          if (!have) {
            if (!(ok = cta_wait(c, nt_.flag, nullptr, &s_ok))) break;
            if (threadIdx.x == 0) s_ready = s + 2;
            tile_ldg(vreg, nt_.t);
            oz_load_async(nxt + OZ_OPER, right_of(s + 1));
            cp_async_commit();
          }
          const double mx = cta_absmax(vreg, red4);
          const int En = mx > 0.0 ? ilogb(mx) + 1 : -100000;
          if (En > E || since_fold == OZ_CHUNK) {
            if (E > -100000) oz_fold_sub(acc, esum);
            since_fold = 0;
            if (En > E) E = En;
            set_esum();
          }
          oz_slice_to_smem(nxt, vreg, E, nt_.trans);
        } else if (E > -100000) {
          oz_fold_sub(acc, esum);   // acc.v = -(sum)
        }
      }
    }
    if (!ok) {
      cp_async_wait_all();
      break;
    }
    __syncthreads();
    // ST_OFF: X = -Y ; ST_DIAG: X = Z = -acc.v
#pragma unroll
    for (int n = 0; n < 2; ++n)
#pragma unroll
      for (int q = 0; q < 4; ++q)
        X[oz_row(n, q) * LDS + oz_col(n, q)] = (type == ST_OFF) ? acc.v[n][q] : -acc.v[n][q];
    __syncthreads();
    const size_t bb = (size_t)g.b * g.b;
    tile_load(F, make_tile(p.D + i * bb, g.b, col * TS, col * TS, g.b, g.b));
    __syncthreads();
    tile_pad_identity(F, g.vrows(col));
    __syncthreads();
    tile_diag_recip(F, rd);
    if (type == ST_OFF) {
      smem_trsm_rln(X, F, rd);
      const SigTileOz d = sig_dest_oz(p, i, j, col);
      tile_store(const_cast<double*>(d.t.p), d.t.ld, d.t.rows, d.t.cols, X);
      cta_publish(c, const_cast<int*>(d.flag));
    } else {
      __syncthreads();
      oz_diag_finish(X, W, F, rd);
      const SigTileOz d = sig_dest_oz(p, i, col, col);
      tile_store(const_cast<double*>(d.t.p), d.t.ld, d.t.rows, d.t.cols, X);
      cta_publish(c, const_cast<int*>(d.flag));
    }
    trace_task(c, t, type, t_task0);
  }
}

size_t selinv_oz_digit_bytes(const Geom& g) { return (size_t)g.nflags() * OZ_TILE * sizeof(__half); }

void launch_selinv_oz(const Geom& g, const double* D, const double* L, const double* R, const double* T, double* SD,
                      double* SL, double* SR, double* ST, int use_arrow, const int4* tasks, int ntasks, __half* fdig,
                      int* ecol, const LaunchCtl& lc) {
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(k_selinv_oz, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)OZS_SMEM);
    attr_set = true;
  }
  k_fac_col_exponents<<<g.nt * g.B, NT, 0, lc.stream>>>(D, L, R, g, use_arrow, ecol);
  k_fac_digits_t<<<g.nflags(), NT, 0, lc.stream>>>(D, L, R, g, use_arrow, ecol, fdig);
  SelinvOzArgs p;
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
  p.fdig = fdig;
  p.ecol = ecol;
  p.c.ctrl = lc.ctrl;
  p.c.flags = lc.flags;
  p.c.epoch = lc.epoch;
  p.c.wait_ns = lc.wait_ns;
  p.c.trace = lc.trace;
  k_selinv_oz<<<lc.grid, NT, OZS_SMEM, lc.stream>>>(p);
  count_launches(3);
}

}  // namespace gbta
