// Single-instance BTA factorization kernel with FP64 tile products (the task body is
// factor_fp64_task in bta_factor_task.cuh).
#include "../../include/pyinla_gb300.h"
#include "bta_factor_task.cuh"

namespace gbta {

__global__ void __launch_bounds__(NT, 1) k_factor(FactorArgs p) {
  __shared__ __align__(16) unsigned char raw[FP64F_SMEM];
  __shared__ int s_ok, s_t;
  while (true) {
    const int t = cta_ticket(p.c, &s_t);
    if (t < 0 || t >= p.ntasks) break;
    if (!factor_fp64_task(p, t, raw, &s_ok)) break;
  }
}

__global__ void k_clear_feeders(Geom g, int* flags) {
  const int n = g.nt * g.B;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int i = k / g.B, c = k - i * g.B;
    const int fk = g.feeder_kind(i, c);
    if (fk == 1) flags[g.fD(i, c + 1, c)] = 0;
    if (fk == 2) flags[g.fL(i, 0, c)] = 0;
  }
}

void launch_clear_feeders(const Geom& g, int* flags, cudaStream_t stream) {
  const int n = g.nt * g.B;
  const int blocks = (n + 255) / 256;
  k_clear_feeders<<<blocks < 1216 ? blocks : 1216, 256, 0, stream>>>(g, flags);
  count_launches(1);
}

void launch_factor(const Geom& g, double* D, double* L, double* R, double* T, int use_arrow, const int4* tasks,
                   int ntasks, double* tip_part, const LaunchCtl& lc, int* feed_aux) {
  FactorArgs p;
  p.D = D;
  p.L = L;
  p.R = R;
  p.T = T;
  p.g = g;
  p.use_arrow = use_arrow;
  p.tasks = tasks;
  p.ntasks = ntasks;
  p.method = GBTA_METHOD_FP64;
  p.tip_part = tip_part;
  p.digits = nullptr;
  p.erow = nullptr;
  p.info = nullptr;
  p.feed_pre = feed_aux;
  p.c.ctrl = lc.ctrl;
  p.c.flags = lc.flags;
  p.c.epoch = lc.epoch;
  p.c.wait_ns = lc.wait_ns;
  p.c.trace = lc.trace;
  k_factor<<<launch_grid((const void*)k_factor, NT, 0, lc), NT, 0, lc.stream>>>(p);
  count_launches(1);
}

}  // namespace gbta
