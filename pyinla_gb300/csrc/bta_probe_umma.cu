// Check and timing of the tcgen05 digit-plane tile step (bta_umma.cuh) against the
// mma.sync tile step (bta_ozaki.cuh) on one CTA: pseudo-random digits in [-64, 64]
// for a left and a right tile, every combination of orientation and plane shift the
// selected inversion uses, the exact partial sums of all nine diagonals compared
// element by element, the FP64 fold compared bit for bit, accumulation over two steps,
// and cycles per tile step of both paths.
#include <cuda_runtime.h>

#include "../../include/pyinla_gb300.h"
#include "bta_umma.cuh"

namespace gbta {

constexpr int PU_CONFIGS = 7;
constexpr int PU_STAGE_H = UMMA_STAGE_PLANES * OZ_PLANE;
constexpr size_t PU_SMEM = 512 + PU_STAGE_H * sizeof(__half) + OZ_OPER * sizeof(__half) +
                           OZ_ND * TS * TS * sizeof(float) + OZ_ND * 8 * 32 * sizeof(float) +
                           2 * TS * TS * sizeof(double);

__device__ __forceinline__ __half pu_digit(unsigned idx, unsigned salt) {
  unsigned h = idx * 2654435761u + salt * 40503u;
  h ^= h >> 15;
  h *= 2246822519u;
  h ^= h >> 13;
  return __int2half_rn((int)(h % 129u) - 64);
}

__global__ void __launch_bounds__(NT, 1) k_probe_umma(int* mism, long long* cyc, int iters) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ UmmaState us;
  __shared__ int s_mis;
  unsigned char* raw = smem_align512(smem_raw);
  __half* stage = reinterpret_cast<__half*>(raw);
  __half* L = stage;
  __half* R = stage + UMMA_RIGHT_PLANE * OZ_PLANE;
  __half* Ash = stage + PU_STAGE_H;
  float* ref = reinterpret_cast<float*>(Ash + OZ_OPER);
  float* xch = ref + OZ_ND * TS * TS;
  double* vref = reinterpret_cast<double*>(xch + OZ_ND * 8 * 32);
  double* vu = vref + TS * TS;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  umma_init(&us);
  umma_zero_planes(stage, 1);
  for (int idx = threadIdx.x; idx < OZ_OPER; idx += NT) {
    L[idx] = pu_digit(idx, 1);
    R[idx] = pu_digit(idx, 2);
  }
  fence_async_smem();
  __syncthreads();
  const unsigned tl = us.tmem + ((unsigned)(32 * w) << 16);
  const int cfg_t[PU_CONFIGS] = {0, 1, 0, 1, 0, 1, 0};
  const int cfg_q[PU_CONFIGS] = {0, 0, 2, 3, 5, 7, 8};
  int st = 0;   // stage barrier of the next step (the two alternate)

  // reference partial sums of one mma.sync step into ref[d][m][n]
  auto reference = [&](int q, bool trans) {
    for (int idx = threadIdx.x; idx < OZ_OPER; idx += NT) {
      const int s = idx / OZ_PLANE;
      Ash[idx] = s >= q ? L[idx - q * OZ_PLANE] : __int2half_rn(0);
    }
    __syncthreads();
    OzAcc acc;
    oz_clear_partials(acc);
    if (trans)
      oz_step_t<true>(acc, Ash, R);
    else
      oz_step_t<false>(acc, Ash, R);
#pragma unroll
    for (int d = 0; d < OZ_ND; ++d)
#pragma unroll
      for (int n = 0; n < 2; ++n)
#pragma unroll
        for (int j = 0; j < 4; ++j) ref[(d * TS + oz_row(n, j)) * TS + oz_col(n, j)] = acc.p[d][n][j];
    __syncthreads();
  };
  // accumulator groups against scale * ref; returns the CTA's mismatch count
  auto compare = [&](unsigned written, float scale) -> int {
    if (threadIdx.x == 0) s_mis = 0;
    tmem_fence_after();
    __syncthreads();
    int bad = 0;
#pragma unroll
    for (int gi = 0; gi < UMMA_GROUPS; ++gi) {
      if (gi == 0 && w != 0) continue;
      const int d = umma_group_d0(gi) + w;
      if ((written >> gi) & 1u) {
        float pv[32];
        tmem_ld32(tl + 32 * gi, pv);
        for (int m = 0; m < TS; ++m) bad += pv[m] != scale * ref[(d * TS + m) * TS + lane];
      } else {
        for (int m = 0; m < TS; ++m) bad += ref[(d * TS + m) * TS + lane] != 0.f;
      }
    }
    atomicAdd(&s_mis, bad);
    tmem_fence_before();
    __syncthreads();
    const int r = s_mis;
    __syncthreads();
    return r;
  };
  auto step = [&](int q, bool trans, unsigned& fresh) {
    if (threadIdx.x == 0) {
      umma_drain_stage(&us, st);
      umma_oz_step(&us, st, stage, q, trans, fresh);
    }
    st ^= 1;
  };
  auto drain_all = [&]() -> bool {
    bool ok = true;
    if (threadIdx.x == 0) ok = umma_drain_stage(&us, 0) & umma_drain_stage(&us, 1);
    return __syncthreads_and(ok);
  };

  for (int k = 0; k < PU_CONFIGS; ++k) {
    const int q = cfg_q[k];
    const bool trans = cfg_t[k] != 0;
    reference(q, trans);
    unsigned fresh = 7;
    step(q, trans, fresh);
    const bool ok = drain_all();
    const int bad = compare(umma_groups_written(q), 1.f);
    if (threadIdx.x == 0) mism[k] = ok ? bad : -1;
  }

  // fold: exact sums to FP64, both paths, bit for bit (q = 0, not transposed)
  {
    reference(0, false);
    OzAcc acc;
    oz_clear_partials(acc);
    oz_step_t<false>(acc, Ash, R);
    int es[2][4];
#pragma unroll
    for (int n = 0; n < 2; ++n)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        es[n][j] = 40;
        acc.v[n][j] = 0.0;
      }
    oz_fold_sub(acc, es);
#pragma unroll
    for (int n = 0; n < 2; ++n)
#pragma unroll
      for (int j = 0; j < 4; ++j) vref[oz_row(n, j) * TS + oz_col(n, j)] = acc.v[n][j];
    unsigned fresh = 7;
    step(0, false, fresh);
    const bool ok = drain_all();
    tmem_fence_before();
    __syncthreads();
    double v[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) v[e] = 0.0;
    umma_fold_sub(&us, 7u, 40, v, xch);
#pragma unroll
    for (int e = 0; e < 8; ++e) vu[umma_row(e) * TS + umma_col()] = v[e];
    if (threadIdx.x == 0) s_mis = 0;
    __syncthreads();
    int bad = 0;
    for (int idx = threadIdx.x; idx < TS * TS; idx += NT)
      bad += __double_as_longlong(vref[idx]) != __double_as_longlong(vu[idx]);
    atomicAdd(&s_mis, bad);
    __syncthreads();
    if (threadIdx.x == 0) mism[PU_CONFIGS] = ok ? s_mis : -1;
    __syncthreads();
  }

  // two steps into the same accumulators
  {
    reference(0, true);
    unsigned fresh = 7;
    step(0, true, fresh);
    step(0, true, fresh);
    const bool ok = drain_all();
    const int bad = compare(7u, 2.f);
    if (threadIdx.x == 0) mism[PU_CONFIGS + 1] = ok ? bad : -1;
  }

  // cycles per tile step: tcgen05 (issue with two steps in flight, then drain) and mma.sync
  {
    unsigned fresh = 7;
    __syncthreads();
    long long t0 = clock64();
    for (int it = 0; it < iters; ++it) step(0, false, fresh);
    drain_all();
    long long t1 = clock64();
    if (threadIdx.x == 0) cyc[0] = (t1 - t0) / iters;
    OzAcc acc;
    oz_clear_partials(acc);
    __syncthreads();
    t0 = clock64();
    for (int it = 0; it < iters; ++it) oz_step_t<false>(acc, Ash, R);
    __syncthreads();
    t1 = clock64();
    if (threadIdx.x == 0) cyc[1] = (t1 - t0) / iters;
    float sink = 0.f;
#pragma unroll
    for (int d = 0; d < OZ_ND; ++d) sink += acc.p[d][0][0];
    if (sink == 12345.f) cyc[2] = 1;   // keeps the products live
  }
  umma_release(&us);
}

}  // namespace gbta

extern "C" int gbta_set_error(int code, const char* msg);

extern "C" int gbta_probe_umma(int iters, int* mismatches, long long* cycles) {
  if (!mismatches || !cycles || iters < 1) return gbta_set_error(GBTA_ERR_ARG, "probe_umma: need iters >= 1 and outputs");
  int* d_mis = nullptr;
  long long* d_cyc = nullptr;
  if (cudaMalloc(&d_mis, (gbta::PU_CONFIGS + 2) * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&d_cyc, 3 * sizeof(long long)) != cudaSuccess) {
    cudaFree(d_mis);
    return gbta_set_error(GBTA_ERR_ALLOC, "probe_umma: cudaMalloc failed");
  }
  cudaFuncSetAttribute(gbta::k_probe_umma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gbta::PU_SMEM);
  gbta::k_probe_umma<<<1, gbta::NT, gbta::PU_SMEM>>>(d_mis, d_cyc, iters);
  gbta::count_launches(1);
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(mismatches, d_mis, (gbta::PU_CONFIGS + 2) * sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(cycles, d_cyc, 2 * sizeof(long long), cudaMemcpyDeviceToHost);
  cudaFree(d_mis);
  cudaFree(d_cyc);
  if (e != cudaSuccess) return gbta_set_error(GBTA_ERR_CUDA, cudaGetErrorString(e));
  return GBTA_OK;
}
