// Building blocks of the inner Newton iteration for non-Gaussian likelihoods.
//
// The reference runs, per objective evaluation with a Poisson or Binomial likelihood,
// a Newton iteration on the latent field (src/pyinla/core/pyinla.py:1025-1074):
//   eta = A x;  Q_cond = Q_prior + A^T W(eta) A  (W = -diag l''(eta), model.py:384-423);
//   rhs = -Q_prior x + A^T l'(eta)  (model.py:425-449);  dx = Q_cond^{-1} rhs.
// Two pieces are new relative to the Gaussian path:
//   * gbta_weighted_gram: the entries of A^T W A that the BTA assembly consumes (the
//     diagonal-block CSR entries, the dense arrow rows and the tip), each a fixed-order
//     sum over a precomputed list of (observation, A_rp A_rq) pairs, so that W can
//     change every iteration without a sparse product and the result is deterministic;
//   * gbta_bta_symv: y = Q x for a symmetric BTA matrix held in the Serinv layout
//     (D full symmetric blocks, L_t = block (t+1, t), R_t = block (arrow, t), T),
//     here the unfactored prior, also in a fixed summation order.
#include <cuda_runtime.h>

#include "../../include/pyinla_gb300.h"
#include "bta_internal.h"

namespace gbta {

__global__ void k_weighted_gram(long long n_out, const long long* __restrict__ seg, const int* __restrict__ obs,
                                const double* __restrict__ coef, const double* __restrict__ w,
                                double* __restrict__ out) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n_out;
       e += (long long)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (long long k = seg[e]; k < seg[e + 1]; ++k) s = fma(w[obs[k]], coef[k], s);
    out[e] = s;
  }
}

constexpr int SV_WARPS = 8;

// One CTA per (block t, 32-column tile c0): the 32 rows c0 .. c0+31 of block t of y.
// Column sums of D_t, L_t and R_t (lanes = columns: coalesced rows; warps take rows
// j = w mod SV_WARPS; the eight partials are added in warp order) and row dot products
// of L_{t-1} (one warp per row, lanes over the row, a fixed shuffle tree).
__global__ void __launch_bounds__(SV_WARPS * 32) k_bta_symv_blocks(Geom g, const double* __restrict__ D,
                                                                   const double* __restrict__ L,
                                                                   const double* __restrict__ R, int use_arrow,
                                                                   const double* __restrict__ x,
                                                                   double* __restrict__ y) {
  __shared__ double part[SV_WARPS][TS];
  __shared__ double rowdot[TS];
  const int t = blockIdx.x / g.B, c0 = (blockIdx.x % g.B) * TS;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int c = c0 + lane;
  const size_t bb = (size_t)g.b * g.b;
  const long long nb = (long long)g.nt * g.b;
  double s = 0.0;
  if (c < g.b) {
    const double* Dt = D + (size_t)t * bb;
    const double* xt = x + (size_t)t * g.b;
    for (int j = w; j < g.b; j += SV_WARPS) s = fma(Dt[(size_t)j * g.b + c], xt[j], s);
    if (t + 1 < g.nt) {   // L_t^T x_{t+1}
      const double* Lt = L + (size_t)t * bb;
      const double* xn = x + (size_t)(t + 1) * g.b;
      for (int j = w; j < g.b; j += SV_WARPS) s = fma(Lt[(size_t)j * g.b + c], xn[j], s);
    }
    if (use_arrow) {      // R_t^T x_a
      const double* Rt = R + (size_t)t * g.a * g.b;
      const double* xa = x + nb;
      for (int j = w; j < g.a; j += SV_WARPS) s = fma(Rt[(size_t)j * g.b + c], xa[j], s);
    }
  }
  part[w][lane] = s;
  // L_{t-1} x_{t-1}: rows c0 .. c0+31 of block (t, t-1)
  for (int rr = w; rr < TS; rr += SV_WARPS) {
    double d = 0.0;
    const int row = c0 + rr;
    if (t > 0 && row < g.b) {
      const double* Lrow = L + (size_t)(t - 1) * bb + (size_t)row * g.b;
      const double* xp = x + (size_t)(t - 1) * g.b;
      for (int k = lane; k < g.b; k += 32) d = fma(Lrow[k], xp[k], d);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
    if (lane == 0) rowdot[rr] = d;
  }
  __syncthreads();
  if (w == 0 && c < g.b) {
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < SV_WARPS; ++k) acc += part[k][lane];
    y[(size_t)t * g.b + c] = acc + rowdot[lane];
  }
}

// The arrow rows: y_a[j] = sum_t R_t[j] . x_t + T[j] . x_a (one CTA per row; per-thread
// partials in index order, then a fixed tree).
__global__ void __launch_bounds__(256) k_bta_symv_arrow(Geom g, const double* __restrict__ R,
                                                        const double* __restrict__ T,
                                                        const double* __restrict__ x, double* __restrict__ y) {
  __shared__ double red[256];
  const int j = blockIdx.x;
  const long long nb = (long long)g.nt * g.b;
  double s = 0.0;
  for (long long k = threadIdx.x; k < nb; k += blockDim.x) {
    const long long t = k / g.b, cc = k - t * g.b;
    s = fma(R[((size_t)t * g.a + j) * g.b + cc], x[k], s);
  }
  for (int k = threadIdx.x; k < g.a; k += blockDim.x) s = fma(T[(size_t)j * g.a + k], x[nb + k], s);
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) y[nb + j] = red[0];
}

}  // namespace gbta

extern "C" int gbta_weighted_gram(gbta_solver* s, long long n_out, const long long* seg, const int* obs,
                                  const double* coef, const double* w, double* out) {
  int b, nt, a;
  void* st;
  if (int r = gbta_geometry(s, &b, &nt, &a, &st)) return r;
  if (n_out < 0) return gbta_set_error(GBTA_ERR_ARG, "weighted_gram: n_out < 0");
  if (n_out == 0) return GBTA_OK;
  if (!seg || !obs || !coef || !w || !out) return gbta_set_error(GBTA_ERR_ARG, "weighted_gram: null pointer");
  const long long blocks = (n_out + 255) / 256;
  gbta::k_weighted_gram<<<(unsigned)(blocks < 152 * 32 ? blocks : 152 * 32), 256, 0, (cudaStream_t)st>>>(
      n_out, seg, obs, coef, w, out);
  gbta::count_launches(1);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GBTA_OK : gbta_set_error(GBTA_ERR_CUDA, cudaGetErrorString(e));
}

extern "C" int gbta_bta_symv(gbta_solver* s, const double* D, const double* L, const double* R, const double* T,
                             int use_arrow, const double* x, double* y) {
  int b, nt, a;
  void* st;
  if (int r = gbta_geometry(s, &b, &nt, &a, &st)) return r;
  if (!D || (nt > 1 && !L) || !x || !y) return gbta_set_error(GBTA_ERR_ARG, "bta_symv: null pointer");
  use_arrow = use_arrow && a > 0;
  if (use_arrow && (!R || !T)) return gbta_set_error(GBTA_ERR_ARG, "bta_symv: R/T required with the arrow");
  gbta::Geom g{b, nt, a, (b + gbta::TS - 1) / gbta::TS};
  gbta::k_bta_symv_blocks<<<nt * g.B, gbta::SV_WARPS * 32, 0, (cudaStream_t)st>>>(g, D, L, R, use_arrow, x, y);
  int launches = 1;
  if (use_arrow) {
    gbta::k_bta_symv_arrow<<<a, 256, 0, (cudaStream_t)st>>>(g, R, T, x, y);
    ++launches;
  }
  gbta::count_launches(launches);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GBTA_OK : gbta_set_error(GBTA_ERR_CUDA, cudaGetErrorString(e));
}
