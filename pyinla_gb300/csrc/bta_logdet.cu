// logdet from the factor: 2 * sum(log diag) over D_i (and the tip for "bta").
// Replaces SerinvSolver.logdet (src/pyinla/solvers/structured_solver.py:151-166).
// Deterministic: one fixed-order tree reduction per block, then an ordered sum.
#include "bta_internal.h"

namespace gbta {

constexpr int LD_THREADS = 256;

__global__ void __launch_bounds__(LD_THREADS) k_logdet_blocks(const double* D, const double* T, Geom g, int with_tip,
                                                                double* partial) {
  __shared__ double red[LD_THREADS];
  const int blk = blockIdx.x;   // 0..nt-1: D blocks; nt: tip
  double s = 0.0;
  if (blk < g.nt) {
    const double* Di = D + (size_t)blk * g.b * g.b;
    for (int j = threadIdx.x; j < g.b; j += LD_THREADS) s += log(Di[(size_t)j * g.b + j]);
  } else if (with_tip) {
    for (int j = threadIdx.x; j < g.a; j += LD_THREADS) s += log(T[(size_t)j * g.a + j]);
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = LD_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blk] = red[0];
}

__global__ void k_logdet_final(const double* partial, int n, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += partial[i];
    *out = 2.0 * s;
  }
}

void launch_logdet(const Geom& g, const double* D, const double* T, int with_tip, double* partial, double* out,
                   cudaStream_t stream) {
  k_logdet_blocks<<<g.nt + 1, LD_THREADS, 0, stream>>>(D, T, g, with_tip, partial);
  k_logdet_final<<<1, 32, 0, stream>>>(partial, g.nt + 1, out);
  count_launches(2);
}

}  // namespace gbta
