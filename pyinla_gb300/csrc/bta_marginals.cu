// Marginal variances from a selected inverse (the BTA blocks of Sigma).
//
// The reference returns, after an INLA run (src/pyinla/core/pyinla.py:303-311):
//   latent:       diag(Sigma), taken from the selected inverse mapped onto the
//                 identity's pattern (get_marginal_variances_latent_parameters,
//                 pyinla.py:940-964, with extract_diagonal of
//                 src/pyinla/utils/spmatrix_utils.py:46-63);
//   observations: diag(A Sigma_Q A^T), Sigma restricted to the pattern of Q_cond and
//                 the product formed densely (get_marginal_variances_observations,
//                 pyinla.py:966-1018).
// Here both are read straight from the BTA blocks.  For observation row r with
// nonzeros (c_j, a_j) the variance is sum_{j,k} a_j a_k Sigma(c_j, c_k); every pair
// lies in the pattern of A^T A, hence of Q_cond, so the restriction removes nothing.
// One warp per row: the lanes take the row's ordered pairs and the warp sums them
// with a fixed shuffle tree (deterministic).  The Sigma entries a row needs sit in
// one diagonal block (plus the arrow rows and the tip, and a neighbouring block for
// a row that touches two time steps), so consecutive rows of one time step hit L2.
#include <cuda_runtime.h>

#include <cmath>

#include "../../include/pyinla_gb300.h"
#include "bta_internal.h"

namespace gbta {

struct SigmaBlocks {
  const double* D;   // [nt][b][b]
  const double* L;   // [nt-1][b][b], L_t = Sigma(block t+1, block t)
  const double* R;   // [nt][a][b],  R_t = Sigma(arrow, block t)
  const double* T;   // [a][a]
  int b, nt, a;
};

// Sigma(p, q) for 0 <= p, q < nt*b + a; 0 for blocks farther apart than neighbours
// (outside the BTA pattern).
__device__ __forceinline__ double sigma_at(const SigmaBlocks& s, long long p, long long q) {
  const long long nb = (long long)s.nt * s.b;
  if (p >= nb) {
    if (q >= nb) return s.T[(p - nb) * s.a + (q - nb)];
    const long long t = q / s.b;
    return s.R[(t * s.a + (p - nb)) * s.b + (q - t * s.b)];
  }
  if (q >= nb) {
    const long long t = p / s.b;
    return s.R[(t * s.a + (q - nb)) * s.b + (p - t * s.b)];
  }
  const long long tp = p / s.b, tq = q / s.b;
  const long long ip = p - tp * s.b, iq = q - tq * s.b;
  if (tp == tq) return s.D[(tp * s.b + ip) * s.b + iq];
  if (tp == tq + 1) return s.L[(tq * s.b + ip) * s.b + iq];
  if (tq == tp + 1) return s.L[(tp * s.b + iq) * s.b + ip];
  return 0.0;
}

__global__ void k_sigma_diagonal(SigmaBlocks s, double* __restrict__ out) {
  const long long nb = (long long)s.nt * s.b;
  const long long n = nb + s.a;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    if (i < nb) {
      const long long t = i / s.b, r = i - t * s.b;
      out[i] = s.D[(t * s.b + r) * s.b + r];
    } else {
      const long long j = i - nb;
      out[i] = s.T[j * s.a + j];
    }
  }
}

constexpr int OV_WARPS = 8;   // warps (rows in flight) per CTA

__global__ void __launch_bounds__(OV_WARPS * 32) k_obs_variances(SigmaBlocks s, long long nrows,
                                                                  const long long* __restrict__ rowptr,
                                                                  const int* __restrict__ col,
                                                                  const double* __restrict__ val,
                                                                  double* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const long long n = (long long)s.nt * s.b + s.a;
  const long long warps = (long long)gridDim.x * OV_WARPS;
  for (long long r = blockIdx.x * (long long)OV_WARPS + (threadIdx.x >> 5); r < nrows; r += warps) {
    const long long beg = rowptr[r];
    const long long m = rowptr[r + 1] - beg;
    double acc = 0.0;
    bool bad = false;
    for (long long e = lane; e < m * m; e += 32) {
      const long long j = e / m, k = e - j * m;
      const long long cj = col[beg + j], ck = col[beg + k];
      if (cj < 0 || cj >= n || ck < 0 || ck >= n) {
        bad = true;
        continue;
      }
      acc = fma(val[beg + j] * val[beg + k], sigma_at(s, cj, ck), acc);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    bad = __any_sync(0xffffffffu, bad);
    if (lane == 0) out[r] = bad ? NAN : acc;
  }
}

}  // namespace gbta

namespace {

int finish_launch() {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return gbta_set_error(GBTA_ERR_CUDA, cudaGetErrorString(e));
  return GBTA_OK;
}

}  // namespace

extern "C" int gbta_sigma_diagonal(gbta_solver* s, const double* SD, const double* ST, double* out) {
  int b, nt, a;
  void* st;
  if (int r = gbta_geometry(s, &b, &nt, &a, &st)) return r;
  if (!SD || !out || (a > 0 && !ST)) return gbta_set_error(GBTA_ERR_ARG, "sigma_diagonal: null pointer");
  gbta::SigmaBlocks sb{SD, nullptr, nullptr, ST, b, nt, a};
  const long long n = (long long)nt * b + a;
  const unsigned grid = (unsigned)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
  gbta::k_sigma_diagonal<<<grid, 256, 0, (cudaStream_t)st>>>(sb, out);
  gbta::count_launches(1);
  return finish_launch();
}

extern "C" int gbta_obs_variances(gbta_solver* s, long long nrows, const long long* A_rowptr, const int* A_col,
                                  const double* A_val, const double* SD, const double* SL, const double* SR,
                                  const double* ST, double* out) {
  int b, nt, a;
  void* st;
  if (int r = gbta_geometry(s, &b, &nt, &a, &st)) return r;
  if (nrows < 0) return gbta_set_error(GBTA_ERR_ARG, "obs_variances: nrows < 0");
  if (nrows == 0) return GBTA_OK;
  if (!A_rowptr || !A_col || !A_val || !out) return gbta_set_error(GBTA_ERR_ARG, "obs_variances: null A or out");
  if (!SD || (nt > 1 && !SL) || (a > 0 && (!SR || !ST)))
    return gbta_set_error(GBTA_ERR_ARG, "obs_variances: null Sigma block");
  gbta::SigmaBlocks sb{SD, SL, SR, ST, b, nt, a};
  const long long ctas = (nrows + gbta::OV_WARPS - 1) / gbta::OV_WARPS;
  const unsigned grid = (unsigned)(ctas < 152 * 16 ? ctas : 152 * 16);
  gbta::k_obs_variances<<<grid, gbta::OV_WARPS * 32, 0, (cudaStream_t)st>>>(sb, nrows, A_rowptr, A_col, A_val, out);
  gbta::count_launches(1);
  return finish_launch();
}
