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
    if (fk == 2) flags[g.fL(g.lslot(i), 0, c)] = 0;
  }
}

// One CTA per pair of tiles (R, C), (C, R) with R >= C of one L slot below the separator:
// both are read, then written back transposed (a tile on the diagonal is its own pair).
__global__ void __launch_bounds__(256) k_transpose_lslots(double* L, Geom g, int j0) {
  __shared__ double A[TS][TS + 1], At[TS][TS + 1];
  const int B = g.B, pairs = B * (B + 1) / 2;
  const int slot = j0 + blockIdx.x / pairs;
  const int q = blockIdx.x % pairs;
  int R = (int)((sqrtf(8.f * q + 1.f) - 1.f) * 0.5f);
  while ((R + 1) * (R + 2) / 2 <= q) ++R;
  while (R * (R + 1) / 2 > q) --R;
  const int C = q - R * (R + 1) / 2;
  double* blk = L + (size_t)slot * g.b * g.b;
  const int r0 = R * TS, c0 = C * TS;
  for (int idx = threadIdx.x; idx < TS * TS; idx += blockDim.x) {
    const int rr = idx / TS, cc = idx % TS;
    if (r0 + rr < g.b && c0 + cc < g.b) A[rr][cc] = blk[(size_t)(r0 + rr) * g.b + c0 + cc];
    if (c0 + rr < g.b && r0 + cc < g.b) At[rr][cc] = blk[(size_t)(c0 + rr) * g.b + r0 + cc];
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < TS * TS; idx += blockDim.x) {
    const int rr = idx / TS, cc = idx % TS;
    if (r0 + rr < g.b && c0 + cc < g.b) blk[(size_t)(r0 + rr) * g.b + c0 + cc] = At[cc][rr];
    if (c0 + rr < g.b && r0 + cc < g.b) blk[(size_t)(c0 + rr) * g.b + r0 + cc] = A[cc][rr];
  }
}

void launch_transpose_lslots(const Geom& g, double* L, cudaStream_t stream) {
  const int j0 = g.sep(), nslots = g.nt - 1 - j0;
  if (nslots <= 0) return;
  const long long blocks = (long long)nslots * (g.B * (g.B + 1) / 2);
  k_transpose_lslots<<<(unsigned)blocks, 256, 0, stream>>>(L, g, j0);
  count_launches(1);
}

// One CTA per (L slot j, row tile r): scan the row tile's column tiles left to right
// until one holds a nonzero (a NaN counts as nonzero).
__global__ void __launch_bounds__(NT) k_coupling_kfirst(const double* __restrict__ L, Geom g, int* kf) {
  const int j = blockIdx.x / g.B, r = blockIdx.x % g.B;
  const double* rows = L + (size_t)j * g.b * g.b + (size_t)r * TS * g.b;
  const int nr = min(TS, g.b - r * TS);
  int k = 0;
  for (; k < g.B; ++k) {
    const int nc = min(TS, g.b - k * TS);
    bool nz = false;
    for (int idx = threadIdx.x; idx < nr * TS; idx += NT) {
      const int rr = idx / TS, cc = idx % TS;
      if (cc < nc && __ldg(rows + (size_t)rr * g.b + k * TS + cc) != 0.0) nz = true;
    }
    if (__syncthreads_or(nz)) break;
  }
  if (threadIdx.x == 0) kf[blockIdx.x] = k;
}

void launch_coupling_kfirst(const Geom& g, const double* L, int* kf, cudaStream_t stream) {
  if (g.nt < 2) return;
  k_coupling_kfirst<<<(g.nt - 1) * g.B, NT, 0, stream>>>(L, g, kf);
  count_launches(1);
}

void launch_clear_feeders(const Geom& g, int* flags, cudaStream_t stream) {
  const int n = g.nt * g.B;
  const int blocks = (n + 255) / 256;
  k_clear_feeders<<<blocks < 1216 ? blocks : 1216, 256, 0, stream>>>(g, flags);
  count_launches(1);
}

void launch_factor(const Geom& g, double* D, double* L, double* R, double* T, int use_arrow, const int4* tasks,
                   int ntasks, double* tip_part, const LaunchCtl& lc, int* feed_aux, int* diag_pre,
                   const int* kf) {
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
  p.diag_pre = diag_pre;
  p.kf = kf;
  p.c.ctrl = lc.ctrl;
  p.c.flags = lc.flags;
  p.c.epoch = lc.epoch;
  p.c.wait_ns = lc.wait_ns;
  p.c.trace = lc.trace;
  k_factor<<<launch_grid((const void*)k_factor, NT, 0, lc), NT, 0, lc.stream>>>(p);
  count_launches(1);
}

}  // namespace gbta
