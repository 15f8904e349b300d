// Single-instance BTA factorization kernel with tensor-core (Ozaki digit-plane) tile
// products; the task body is factor_oz_task in bta_factor_task.cuh.  The per-row
// exponents come from the input matrix's diagonal (k_row_exponents), computed before
// the factorization overwrites it.
#include "../../include/pyinla_gb300.h"
#include "bta_factor_task.cuh"

namespace gbta {

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

__global__ void __launch_bounds__(NT, 1) k_factor_oz(FactorArgs p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_ok, s_t, s_ready;
  __shared__ OzPipe pipe;
  oz_pipe_init(&pipe);
  const OzFactorSmem sm = oz_factor_smem(smem_raw, &s_ok, &s_ready, &pipe);
  while (true) {
    const int t = cta_ticket(p.c, &s_t);
    if (t < 0 || t >= p.ntasks) break;
    if (!factor_oz_task(p, t, sm)) break;
  }
}

void launch_row_exponents(const Geom& g, const double* D, const double* T, int use_arrow, int* erow,
                          cudaStream_t stream) {
  const long long n = (long long)g.nt * g.b + (use_arrow ? g.a : 0);
  const long long blocks = (n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096;
  k_row_exponents<<<(unsigned)blocks, 256, 0, stream>>>(D, T, g, use_arrow, erow);
  count_launches(1);
}

size_t factor_oz_digit_bytes(const Geom& g) { return (size_t)g.nflags() * OZ_TILE * sizeof(__half); }

void launch_factor_oz(const Geom& g, double* D, double* L, double* R, double* T, int use_arrow, const int4* tasks,
                      int ntasks, double* tip_part, __half* digits, int* erow, const LaunchCtl& lc,
                      int* feed_aux, int* diag_pre, const int* kf) {
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(k_factor_oz, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)OZF_SMEM);
    cudaFuncSetAttribute(k_factor_oz, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    attr_set = true;
  }
  launch_row_exponents(g, D, T, use_arrow, erow, lc.stream);
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
  p.digits = digits;
  p.method = GBTA_METHOD_OZAKI;
  p.erow = erow;
  p.info = nullptr;
  p.feed_pre = feed_aux;
  p.diag_pre = diag_pre;
  p.kf = kf;
  p.c.ctrl = lc.ctrl;
  p.c.flags = lc.flags;
  p.c.epoch = lc.epoch;
  p.c.wait_ns = lc.wait_ns;
  p.c.trace = lc.trace;
  k_factor_oz<<<launch_grid((const void*)k_factor_oz, NT, OZF_SMEM, lc), NT, OZF_SMEM, lc.stream>>>(p);
  count_launches(1);
}

}  // namespace gbta
