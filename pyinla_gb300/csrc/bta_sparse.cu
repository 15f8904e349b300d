// Sparse <-> BTA block mapping on the device.
//
// gbta_scatter_coo replaces SerinvSolver._spmatrix_to_structured
// (src/pyinla/solvers/structured_solver.py:192-250, CPU slicing loop) and its CuPy
// path _spmatrix_to_bta / _spmatrix_to_bt (:252-468, which needs (nt+1)^2 mask
// launches of pyinla/kernels/blockmapping.py:12-37 plus per-block fancy indexing):
// one zero-fill and one scatter launch, each COO entry routed to its block by
// integer division.  gbta_gather_coo replaces the per-block gather of
// SerinvSolver._structured_to_spmatrix (:470-538).
#include <cuda_runtime.h>

#include "../../include/pyinla_gb300.h"
#include "bta_internal.h"

namespace gbta {

struct BtaPtrs {
  double* D;
  double* L;
  double* R;
  double* T;
};

// Where a (row, col) entry of the symmetric N x N matrix lives in BTA storage;
// nullptr if it is outside the stored lower pattern (upper blocks are implied).
__device__ __forceinline__ double* locate(const Geom& g, const BtaPtrs& p, int with_arrow, long long row,
                                          long long col) {
  const long long nb = (long long)g.nt * g.b;
  const long long n = nb + ((with_arrow && g.a > 0) ? g.a : 0);
  if (row < 0 || col < 0 || row >= n || col >= n) return nullptr;   // outside the matrix
  if (row < nb && col < nb) {
    const int br = (int)(row / g.b), bc = (int)(col / g.b);
    const int rr = (int)(row % g.b), cc = (int)(col % g.b);
    if (br == bc) return p.D + ((size_t)br * g.b + rr) * g.b + cc;
    if (br == bc + 1) return p.L + ((size_t)bc * g.b + rr) * g.b + cc;
    return nullptr;
  }
  if (!with_arrow || g.a == 0) return nullptr;
  if (row >= nb && col < nb) {
    const int bc = (int)(col / g.b), cc = (int)(col % g.b);
    return p.R + ((size_t)bc * g.a + (row - nb)) * g.b + cc;
  }
  if (row >= nb && col >= nb) return p.T + (size_t)(row - nb) * g.a + (col - nb);
  return nullptr;
}

__global__ void k_zero(double* p, size_t n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) p[e] = 0.0;
}

__global__ void k_scatter(Geom g, BtaPtrs p, int with_arrow, const long long* rows, const long long* cols,
                          const double* vals, long long nnz) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nnz; e += (long long)gridDim.x * blockDim.x) {
    double* dst = locate(g, p, with_arrow, rows[e], cols[e]);
    if (dst) *dst = vals[e];
  }
}

__global__ void k_gather(Geom g, BtaPtrs p, int with_arrow, const long long* rows, const long long* cols, double* vals,
                         long long nnz) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nnz; e += (long long)gridDim.x * blockDim.x) {
    const double* src = locate(g, p, with_arrow, rows[e], cols[e]);
    vals[e] = src ? *src : 0.0;
  }
}

}  // namespace gbta

// Internal helpers implemented in bta_api.cu.
extern "C" int gbta_set_error(int code, const char* msg);

extern "C" int gbta_scatter_coo(gbta_solver* s, const long long* rows, const long long* cols, const double* vals,
                                long long nnz, double* D, double* L, double* R, double* T, int with_arrow) {
  int b, nt, a;
  void* st;
  if (int r = gbta_geometry(s, &b, &nt, &a, &st)) return r;
  if (!D || (nt > 1 && !L) || (with_arrow && a > 0 && (!R || !T)) || (nnz > 0 && (!rows || !cols || !vals)))
    return gbta_set_error(GBTA_ERR_ARG, "scatter: null device pointer");
  gbta::Geom g{b, nt, a, (b + gbta::TS - 1) / gbta::TS};
  gbta::BtaPtrs p{D, L, R, T};
  cudaStream_t stream = (cudaStream_t)st;
  const size_t bb = (size_t)b * b;
  gbta::k_zero<<<1024, 256, 0, stream>>>(D, nt * bb);
  if (nt > 1) gbta::k_zero<<<1024, 256, 0, stream>>>(L, (nt - 1) * bb);
  if (with_arrow && a > 0) {
    gbta::k_zero<<<256, 256, 0, stream>>>(R, (size_t)nt * a * b);
    gbta::k_zero<<<1, 256, 0, stream>>>(T, (size_t)a * a);
  }
  if (nnz > 0) {
    const long long blocks = (nnz + 255) / 256;
    gbta::k_scatter<<<(unsigned)(blocks < 4096 ? blocks : 4096), 256, 0, stream>>>(g, p, with_arrow, rows, cols, vals,
                                                                                  nnz);
  }
  gbta::count_launches(1 + (nt > 1) + 2 * (with_arrow && a > 0) + (nnz > 0));
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return gbta_set_error(GBTA_ERR_CUDA, cudaGetErrorString(e));
  return GBTA_OK;
}

extern "C" int gbta_gather_coo(gbta_solver* s, const long long* rows, const long long* cols, long long nnz,
                               const double* D, const double* L, const double* R, const double* T, int with_arrow,
                               double* vals) {
  int b, nt, a;
  void* st;
  if (int r = gbta_geometry(s, &b, &nt, &a, &st)) return r;
  if (nnz <= 0) return GBTA_OK;
  if (!D || !rows || !cols || !vals || (nt > 1 && !L) || (with_arrow && a > 0 && (!R || !T)))
    return gbta_set_error(GBTA_ERR_ARG, "gather: null device pointer");
  gbta::Geom g{b, nt, a, (b + gbta::TS - 1) / gbta::TS};
  gbta::BtaPtrs p{const_cast<double*>(D), const_cast<double*>(L), const_cast<double*>(R), const_cast<double*>(T)};
  const long long blocks = (nnz + 255) / 256;
  gbta::k_gather<<<(unsigned)(blocks < 4096 ? blocks : 4096), 256, 0, (cudaStream_t)st>>>(g, p, with_arrow, rows, cols,
                                                                                         vals, nnz);
  gbta::count_launches(1);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return gbta_set_error(GBTA_ERR_CUDA, cudaGetErrorString(e));
  return GBTA_OK;
}
