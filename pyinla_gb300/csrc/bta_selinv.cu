// Single-instance BTA selected-inversion kernel with FP64 tile products (the task body
// is selinv_fp64_task in bta_selinv_task.cuh), and the write-back of Sigma into the
// caller's blocks.
#include "../../include/pyinla_gb300.h"
#include "bta_selinv_task.cuh"

namespace gbta {

__global__ void __launch_bounds__(NT, 1) k_selinv(SelinvArgs p) {
  __shared__ __align__(16) unsigned char raw[FP64S_SMEM];
  __shared__ int s_ok, s_t;
  while (true) {
    const int t = cta_ticket(p.c, &s_t);
    if (t < 0 || t >= p.ntasks) break;
    if (!selinv_fp64_task(p, t, raw, &s_ok)) break;
  }
}

// ---- pre-pass: G tiles and the diagonal inverses ------------------------------------
// "column c is not after column k" for the register layout of the tile routines (c = g + 4q).
__device__ __forceinline__ bool col_upto(int q, int k, int g) { return !col_after(q, k, g); }

// X <- X W with W lower triangular (rows of X: lane, columns: warp + 4 q).
static __device__ void smem_gemm_lower_right(double* X, const double* W) {
  const int r = threadIdx.x & 31, g = threadIdx.x >> 5;
  __syncthreads();
  double out[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) out[q] = 0.0;
#pragma unroll
  for (int k = 0; k < TS; ++k) {
    const double xv = X[r * LDS + k];
#pragma unroll
    for (int q = 0; q < 8; ++q)
      if (col_upto(q, k, g)) out[q] = fma(xv, W[k * LDS + g + 4 * q], out[q]);
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < 8; ++q) X[r * LDS + g + 4 * q] = out[q];
  __syncthreads();
}

// C <- W^T W with W lower triangular.
static __device__ void smem_gram_lower(double* C, const double* W) {
  const int r = threadIdx.x & 31, g = threadIdx.x >> 5;
  __syncthreads();
  double out[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) out[q] = 0.0;
#pragma unroll
  for (int k = 0; k < TS; ++k) {
    const double wr = W[k * LDS + r];   // W(k, r): zero for k < r
#pragma unroll
    for (int q = 0; q < 8; ++q)
      if (col_upto(q, k, g)) out[q] = fma(wr, W[k * LDS + g + 4 * q], out[q]);
  }
#pragma unroll
  for (int q = 0; q < 8; ++q) C[r * LDS + g + 4 * q] = out[q];
  __syncthreads();
}

// One CTA per diagonal factor tile F = D_i(c, c): finv = F^{-1}, cinv = F^{-T} F^{-1}
// (identity-padded past the block edge); with wdig, also the digit planes of W^T =
// F^{-T} (row n of W^T relative to ew[n], the exponent of column n of W), the right
// operand of the tensor-core G tiles.
__global__ void __launch_bounds__(NT) k_diag_inverses(const double* D, Geom g, double* finv, double* cinv,
                                                      __half* wdig, int* ew) {
  __shared__ double F[TILE_SMEM], W[TILE_SMEM], rd[TS];
  __shared__ int es[TS];
  const int ic = blockIdx.x;
  const int i = ic / g.B, c = ic % g.B;
  const size_t bb = (size_t)g.b * g.b;
  tile_load(F, make_tile(D + i * bb, g.b, c * TS, c * TS, g.b, g.b));
  for (int idx = threadIdx.x; idx < TS * TS; idx += NT) W[(idx / TS) * LDS + idx % TS] = (idx / TS == idx % TS);
  __syncthreads();
  tile_pad_identity(F, g.vrows(c));
  __syncthreads();
  tile_diag_recip(F, rd);
  smem_trsm_rln(W, F, rd);   // W = F^{-1}
  if (!wdig) tile_store(finv + (size_t)ic * TS * TS, TS, TS, TS, W);
  smem_gram_lower(F, W);
  tile_store(cinv + (size_t)ic * TS * TS, TS, TS, TS, F);
  if (wdig) {
    __syncthreads();
    if (threadIdx.x < TS) {
      const int n = threadIdx.x;
      double m = 0.0;
      for (int k = n; k < TS; ++k) m = fmax(m, fabs(W[k * LDS + n]));   // lower triangular
      es[n] = (m > 0.0 && isfinite(m)) ? ilogb(m) + 1 : 0;
      ew[(size_t)ic * TS + n] = es[n];
    }
    for (int idx = threadIdx.x; idx < TS * TS; idx += NT) {
      const int n = idx / TS, k = idx % TS;
      F[n * LDS + k] = W[k * LDS + n];
    }
    __syncthreads();
    oz_store_digits(wdig + (size_t)ic * OZ_TILE, F, TS, TS, es);
  }
}

// One CTA per off-diagonal pattern tile (the slots of k_g_tiles): G = F(l, c) F(c, c)^{-1}
// on the tensor cores, from the digit planes the factorization left for F(l, c) (rows
// relative to the row exponents erow) and those of F(c, c)^{-T} (k_diag_inverses): one
// 43-pair tile step folded into FP64, written into the blocks D, L, R (the factor's
// own, in place, or a separate set; the kernel reads no FP64 factor tile).  Coupling
// tiles that are structurally zero (kf, launch_coupling_kfirst) are zero in place and
// written as zeros into a separate set (zero_skipped).
__global__ void __launch_bounds__(NT, 3) k_g_tiles_oz(double* D, double* L, double* R, Geom g, int use_arrow,
                                                   const __half* fdig, const int* erow, const __half* wdig,
                                                   const int* ew, const int* kf, int zero_skipped) {
  __shared__ __align__(16) __half As[OZ_OPER];
  __shared__ __align__(16) __half Bs[OZ_OPER];
  __shared__ double X[TILE_SMEM];
  __shared__ int er[TS], ec[TS];
  const int slot = blockIdx.x;
  const int B = g.B;
  const size_t bb = (size_t)g.b * g.b, ab = (size_t)g.a * g.b;
  int i, c;
  double* base;
  int row0, rows;
  long long grow0;   // global row of the tile's first row (row exponents)
  if (slot < g.nt * B * B) {
    i = slot / (B * B);
    const int r = (slot / B) % B;
    c = slot % B;
    if (r <= c) return;
    base = D + i * bb;
    row0 = r * TS;
    rows = g.b;
    grow0 = (long long)i * g.b + r * TS;
  } else if (slot < (2 * g.nt - 1) * B * B) {
    const int s2 = slot - g.nt * B * B;
    const int j = s2 / (B * B);   // L slot j: columns of block lcol(j), rows of the block after it
    const int r = (s2 / B) % B;
    c = s2 % B;
    if (kf && c < kf[j * B + r]) {
      if (zero_skipped) tile_store_zero(L + j * bb + (size_t)r * TS * g.b + c * TS, g.b, min(TS, g.b - r * TS),
                                        min(TS, g.b - c * TS));
      return;
    }
    i = g.lcol(j);
    base = L + j * bb;
    row0 = r * TS;
    rows = g.b;
    grow0 = (long long)g.nxt(i) * g.b + r * TS;
  } else if (slot < (2 * g.nt - 1) * B * B + g.nt * B) {
    if (!use_arrow) return;
    const int s3 = slot - (2 * g.nt - 1) * B * B;
    i = s3 / B;
    c = s3 % B;
    base = R + i * ab;
    row0 = 0;
    rows = g.a;
    grow0 = (long long)g.nt * g.b;
  } else {
    return;
  }
  const Tile t = make_tile(base, g.b, row0, c * TS, rows, g.b);
  oz_load_async(As, fdig + (size_t)slot * OZ_TILE);
  oz_load_async(Bs, wdig + (size_t)(i * B + c) * OZ_TILE);
  cp_async_commit();
  if (threadIdx.x < TS) {
    er[threadIdx.x] = threadIdx.x < t.rows ? erow[grow0 + threadIdx.x] : 0;
    ec[threadIdx.x] = ew[(size_t)(i * B + c) * TS + threadIdx.x];
  }
  cp_async_wait_all();
  __syncthreads();
  OzAcc acc;
  oz_clear_partials(acc);
  int esum[2][4];
#pragma unroll
  for (int n = 0; n < 2; ++n)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      acc.v[n][q] = 0.0;
      esum[n][q] = er[oz_row(n, q)] + ec[oz_col(n, q)];
    }
  oz_step(acc, As, Bs);
  oz_fold_sub_short(acc, esum);   // acc.v = -G (one step)
#pragma unroll
  for (int n = 0; n < 2; ++n)
#pragma unroll
    for (int q = 0; q < 4; ++q) X[oz_row(n, q) * LDS + oz_col(n, q)] = -acc.v[n][q];
  __syncthreads();
  tile_store(const_cast<double*>(t.p), g.b, t.rows, t.cols, X);
}

// One CTA per off-diagonal pattern tile F(l, c) of block column i (the slots of D_i
// below the diagonal, block i's coupling slot lslot(i) and R_i): G = F(l, c) F(c, c)^{-1},
// in place.  A zero tile (half the coupling tiles of a banded coupling) stays as it is.
__global__ void __launch_bounds__(NT) k_g_tiles(double* D, double* L, double* R, Geom g, int use_arrow,
                                                const double* finv) {
  __shared__ double X[TILE_SMEM], W[TILE_SMEM];
  const int slot = blockIdx.x;
  const int B = g.B;
  const size_t bb = (size_t)g.b * g.b, ab = (size_t)g.a * g.b;
  int i, c;
  double* base;
  int row0, rows;
  if (slot < g.nt * B * B) {
    i = slot / (B * B);
    const int r = (slot / B) % B;
    c = slot % B;
    if (r <= c) return;
    base = D + i * bb;
    row0 = r * TS;
    rows = g.b;
  } else if (slot < (2 * g.nt - 1) * B * B) {
    const int s2 = slot - g.nt * B * B;
    const int j = s2 / (B * B);   // L slot j: columns of block lcol(j)
    const int r = (s2 / B) % B;
    c = s2 % B;
    i = g.lcol(j);
    base = L + j * bb;
    row0 = r * TS;
    rows = g.b;
  } else if (slot < (2 * g.nt - 1) * B * B + g.nt * B) {
    if (!use_arrow) return;
    const int s3 = slot - (2 * g.nt - 1) * B * B;
    i = s3 / B;
    c = s3 % B;
    base = R + i * ab;
    row0 = 0;
    rows = g.a;
  } else {
    return;
  }
  const Tile t = make_tile(base, g.b, row0, c * TS, rows, g.b);
  {
    double v[PER_THREAD];
    tile_ldg(v, t);
    bool nz = false;
#pragma unroll
    for (int k = 0; k < PER_THREAD; ++k) nz |= v[k] != 0.0;
    if (!__syncthreads_or(nz)) return;
    tile_sts(X, v);
  }
  tile_load(W, make_tile(finv + (size_t)(i * B + c) * TS * TS, TS, 0, 0, TS, TS));
  smem_gemm_lower_right(X, W);
  tile_store(const_cast<double*>(t.p), g.b, t.rows, t.cols, X);
}

// Workspace per diagonal tile: F^{-1} (FP64), C = F^{-T} F^{-1} (FP64), the digit planes of
// F^{-T} and its column exponents.
size_t selinv_prepare_bytes(const Geom& g) {
  return (size_t)g.nt * g.B * (2 * TS * TS * sizeof(double) + OZ_TILE * sizeof(__half) + TS * sizeof(int));
}

void launch_selinv_prepare(const Geom& g, const double* D, double* L, double* R, int use_arrow, double* ws,
                           cudaStream_t stream, const __half* fdig, const int* erow, const int* kf, double* GD,
                           double* GL, double* GR) {
  static bool attr_set = false;   // the largest shared-memory carveout (see launch_solve)
  if (!attr_set) {
    cudaFuncSetAttribute(k_diag_inverses, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    cudaFuncSetAttribute(k_g_tiles_oz, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    cudaFuncSetAttribute(k_g_tiles, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    attr_set = true;
  }
  const size_t ntile = (size_t)g.nt * g.B;
  double* finv = ws;
  double* cinv = ws + ntile * TS * TS;
  __half* wdig = reinterpret_cast<__half*>(cinv + ntile * TS * TS);
  int* ew = reinterpret_cast<int*>(wdig + ntile * OZ_TILE);
  if (fdig) {
    k_diag_inverses<<<g.nt * g.B, NT, 0, stream>>>(D, g, finv, cinv, wdig, ew);
    const bool sep = GD != nullptr;
    k_g_tiles_oz<<<g.nflags(), NT, 0, stream>>>(sep ? GD : const_cast<double*>(D), sep ? GL : L, sep ? GR : R, g,
                                                use_arrow, fdig, erow, wdig, ew, kf, sep ? 1 : 0);
  } else {
    k_diag_inverses<<<g.nt * g.B, NT, 0, stream>>>(D, g, finv, cinv, nullptr, nullptr);
    k_g_tiles<<<g.nflags(), NT, 0, stream>>>(const_cast<double*>(D), L, R, g, use_arrow, finv);
  }
  count_launches(2);
}

// Copy Sigma back into the caller's buffers; D_i and T become full symmetric, and the
// coupling slots below the separator (Sigma(j, j+1)) are transposed to the caller's
// Sigma(j+1, j).  One 32 x 32 destination tile per step of a CTA (256 threads, four
// rows each): a tile that is a transpose of a stored tile (above a diagonal block's
// diagonal, or a coupling slot past the separator) is staged through shared memory so
// that reads and writes both run along rows; the arrow rows and the tip, which are
// plain copies, are spread over all threads after the tiles.
__global__ void __launch_bounds__(256) k_writeback(const double* SD, const double* SL, const double* SR,
                                                   const double* ST, double* D, double* L, double* R, double* T,
                                                   Geom g, int use_arrow) {
  __shared__ double A[TS][TS + 1];
  const int B = g.B, b = g.b;
  const size_t bb = (size_t)b * b;
  const long long perblk = (long long)B * B;
  const long long nDt = (long long)g.nt * perblk, nLt = (long long)(g.nt - 1) * perblk;
  const int cc = threadIdx.x & 31, r8 = threadIdx.x >> 5;
  for (long long t = blockIdx.x; t < nDt + nLt; t += gridDim.x) {
    const bool isD = t < nDt;
    const long long u = isD ? t : t - nDt;
    const int blk = (int)(u / perblk), q = (int)(u % perblk);
    const int Rt = q / B, Ct = q % B;
    const double* src = (isD ? SD : SL) + (size_t)blk * bb;
    double* dst = (isD ? D : L) + (size_t)blk * bb;
    const bool trans = isD ? Rt < Ct : blk >= g.sep();   // uniform over the CTA
    if (!trans) {
      const int c = Ct * TS + cc;
      double v[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int r = Rt * TS + r8 + 8 * k;
        v[k] = (r < b && c < b) ? __ldcs(src + (size_t)r * b + c) : 0.0;
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int r = Rt * TS + r8 + 8 * k;
        if (r < b && c < b) __stcs(dst + (size_t)r * b + c, v[k]);
      }
    } else {
      // destination tile (Rt, Ct) = transpose of source tile (Ct, Rt)
      __syncthreads();   // the previous transposed tile's reads of A are done
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int r = Ct * TS + r8 + 8 * k, c = Rt * TS + cc;
        A[r8 + 8 * k][cc] = (r < b && c < b) ? __ldcs(src + (size_t)r * b + c) : 0.0;
      }
      __syncthreads();
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int r = Rt * TS + r8 + 8 * k, c = Ct * TS + cc;
        if (r < b && c < b) __stcs(dst + (size_t)r * b + c, A[cc][r8 + 8 * k]);
      }
    }
  }
  const size_t nR = use_arrow ? (size_t)g.nt * g.a * g.b : 0;
  const size_t nT = use_arrow ? (size_t)g.a * g.a : 0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < nR + nT; e += (size_t)gridDim.x * blockDim.x) {
    if (e < nR)
      R[e] = SR[e];
    else
      T[e - nR] = ST[e - nR];
  }
}

// In-place finish of a tensor-core selected inversion (Sigma written over the factor):
// one CTA per tile pair R > C of a diagonal block writes upper tile (C, R) as the
// transpose of lower tile (R, C), so D_i becomes full symmetric (reads and writes touch
// disjoint tiles).
__global__ void __launch_bounds__(256) k_mirror_upper(double* D, Geom g) {
  __shared__ double A[TS][TS + 1];
  const int B = g.B, pairs = B * (B - 1) / 2;
  const int blk = blockIdx.x / pairs, q = blockIdx.x % pairs;
  int R = (int)((1.f + sqrtf(1.f + 8.f * q)) * 0.5f);   // R (R - 1) / 2 <= q < R (R + 1) / 2
  while (R * (R - 1) / 2 > q) --R;
  while ((R + 1) * R / 2 <= q) ++R;
  const int C = q - R * (R - 1) / 2;
  double* d = D + (size_t)blk * g.b * g.b;
  const int r0 = R * TS, c0 = C * TS;
  for (int idx = threadIdx.x; idx < TS * TS; idx += blockDim.x) {
    const int rr = idx / TS, cc = idx % TS;
    if (r0 + rr < g.b && c0 + cc < g.b) A[rr][cc] = d[(size_t)(r0 + rr) * g.b + c0 + cc];
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < TS * TS; idx += blockDim.x) {
    const int rr = idx / TS, cc = idx % TS;   // element (c0 + rr, r0 + cc) of tile (C, R)
    if (c0 + rr < g.b && r0 + cc < g.b) d[(size_t)(c0 + rr) * g.b + r0 + cc] = A[cc][rr];
  }
}

void launch_selinv_finish_inplace(const Geom& g, double* D, double* L, cudaStream_t stream) {
  const long long blocks = (long long)g.nt * (g.B * (g.B - 1) / 2);
  if (blocks > 0) {
    k_mirror_upper<<<(unsigned)blocks, 256, 0, stream>>>(D, g);
    count_launches(1);
  }
  if (g.nt > 1) launch_transpose_lslots(g, L, stream);
}

void launch_selinv(const Geom& g, const double* D, const double* L, const double* R, const double* T, double* SD,
                   double* SL, double* SR, double* ST, int use_arrow, const int4* tasks, int ntasks,
                   const double* cinv, const LaunchCtl& lc) {
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
  p.method = GBTA_METHOD_FP64;
  p.tasks = tasks;
  p.ntasks = ntasks;
  p.fdig = nullptr;
  p.fdz = nullptr;
  p.ecol = nullptr;
  p.cinv = cinv;
  p.sdig = nullptr;
  p.part = nullptr;
  p.part_flag = nullptr;
  p.merged = 0;
  p.c.ctrl = lc.ctrl;
  p.c.flags = lc.flags;
  p.c.epoch = lc.epoch;
  p.c.wait_ns = lc.wait_ns;
  p.c.trace = lc.trace;
  k_selinv<<<launch_grid((const void*)k_selinv, NT, 0, lc), NT, 0, lc.stream>>>(p);
  count_launches(1);
}

void launch_selinv_writeback(const Geom& g, const double* SD, const double* SL, const double* SR, const double* ST,
                             double* D, double* L, double* R, double* T, int use_arrow, cudaStream_t stream) {
  k_writeback<<<152 * 8, 256, 0, stream>>>(SD, SL, SR, ST, D, L, R, T, g, use_arrow);
  count_launches(1);
}

}  // namespace gbta
