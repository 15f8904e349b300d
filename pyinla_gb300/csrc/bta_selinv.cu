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

// Copy Sigma back into the caller's buffers; D_i and T become full symmetric.
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
      L[e - nD] = SL[e - nD];
    } else if (e < nD + nL + nR) {
      R[e - nD - nL] = SR[e - nD - nL];
    } else {
      T[e - nD - nL - nR] = ST[e - nD - nL - nR];
    }
  }
}

void launch_selinv(const Geom& g, const double* D, const double* L, const double* R, const double* T, double* SD,
                   double* SL, double* SR, double* ST, int use_arrow, const int4* tasks, int ntasks,
                   const LaunchCtl& lc) {
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
  p.ecol = nullptr;
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
