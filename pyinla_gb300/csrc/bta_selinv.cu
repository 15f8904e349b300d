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
// (identity-padded past the block edge).
__global__ void __launch_bounds__(NT) k_diag_inverses(const double* D, Geom g, double* finv, double* cinv) {
  __shared__ double F[TILE_SMEM], W[TILE_SMEM], rd[TS];
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
  tile_store(finv + (size_t)ic * TS * TS, TS, TS, TS, W);
  smem_gram_lower(F, W);
  tile_store(cinv + (size_t)ic * TS * TS, TS, TS, TS, F);
}

// One CTA per off-diagonal pattern tile F(l, c) of block column i (the slots of D_i
// below the diagonal, block i's coupling slot lslot(i) and R_i): G = F(l, c) F(c, c)^{-1},
// in place.
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
  tile_load(X, t);
  tile_load(W, make_tile(finv + (size_t)(i * B + c) * TS * TS, TS, 0, 0, TS, TS));
  smem_gemm_lower_right(X, W);
  tile_store(const_cast<double*>(t.p), g.b, t.rows, t.cols, X);
}

size_t selinv_prepare_bytes(const Geom& g) { return 2 * (size_t)g.nt * g.B * TS * TS * sizeof(double); }

void launch_selinv_prepare(const Geom& g, const double* D, double* L, double* R, int use_arrow, double* ws,
                           cudaStream_t stream) {
  double* finv = ws;
  double* cinv = ws + (size_t)g.nt * g.B * TS * TS;
  k_diag_inverses<<<g.nt * g.B, NT, 0, stream>>>(D, g, finv, cinv);
  k_g_tiles<<<g.nflags(), NT, 0, stream>>>(const_cast<double*>(D), L, R, g, use_arrow, finv);
  count_launches(2);
}

// Copy Sigma back into the caller's buffers; D_i and T become full symmetric, and the
// coupling slots below the separator (Sigma(j, j+1)) are transposed to the caller's
// Sigma(j+1, j).
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
      const size_t blk = (e - nD) / bb, rem = (e - nD) % bb;
      if ((int)blk >= g.sep()) {
        const int r = (int)(rem / g.b), cc = (int)(rem % g.b);
        L[e - nD] = SL[blk * bb + (size_t)cc * g.b + r];
      } else {
        L[e - nD] = SL[e - nD];
      }
    } else if (e < nD + nL + nR) {
      R[e - nD - nL] = SR[e - nD - nL];
    } else {
      T[e - nD - nL - nR] = ST[e - nD - nL - nR];
    }
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
  k_writeback<<<1024, 256, 0, stream>>>(SD, SL, SR, ST, D, L, R, T, g, use_arrow);
  count_launches(1);
}

}  // namespace gbta
