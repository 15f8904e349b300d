// Single-instance BTA triangular-sweep kernel (Serinv pobtas / pobts); the task body
// is solve_task in bta_solve_task.cuh.
#include "bta_solve_task.cuh"

namespace gbta {

__global__ void __launch_bounds__(NT, 1) k_solve(SolveArgs p) {
  __shared__ __align__(16) unsigned char raw[SOLVE_SMEM];
  __shared__ int s_ok, s_t;
  while (true) {
    const int t = cta_ticket(p.c, &s_t);
    if (t < 0 || t >= p.ntasks) break;
    if (!solve_task(p, t, raw, &s_ok)) break;
  }
}

void launch_solve(const Geom& g, const double* D, const double* L, const double* R, const double* T, double* Bv,
                  int ldb, int nc, int trans, int use_arrow, double* arrow_part, const LaunchCtl& lc, int both) {
  // One launch covers nc <= NC right-hand-side columns starting at Bv (row stride ldb).
  // The largest shared-memory carveout, as the other dataflow kernels: an SM keeps its
  // split while any CTA is resident, so a sweep CTA on the default split would keep the
  // selected inversion's CTAs (overlapped with the sweeps) off that SM.
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(k_solve, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    attr_set = true;
  }
  SolveArgs p;
  p.D = D;
  p.L = L;
  p.R = R;
  p.T = T;
  p.B = Bv;
  p.ldb = ldb;
  p.nc = nc;
  p.g = g;
  p.use_arrow = use_arrow;
  p.trans = trans;
  p.part = arrow_part;
  p.ntasks = (g.nt * g.B + (use_arrow ? 1 : 0)) * (both ? 2 : 1);
  p.both = both;
  p.bflag0 = 2 * g.nt * g.B + 1;   // after the tiles' and the forward partials' flags
  p.c.ctrl = lc.ctrl;
  p.c.flags = lc.flags;
  p.c.epoch = lc.epoch;
  p.c.wait_ns = lc.wait_ns;
  p.c.trace = lc.trace;
  k_solve<<<launch_grid((const void*)k_solve, NT, 0, lc), NT, 0, lc.stream>>>(p);
  count_launches(1);
}

}  // namespace gbta
