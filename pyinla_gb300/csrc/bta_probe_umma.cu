// Check and timing of the tcgen05 digit-plane tile step (bta_umma.cuh) against the
// mma.sync tile step (bta_ozaki.cuh) on one CTA: pseudo-random digits in [-64, 64]
// for a left and a right tile, every combination of orientation and plane shift the
// selected inversion uses, the FP64 fold of both paths compared bit for bit (the
// partial sums are exact integers, so the results must agree in every bit), two
// accumulated steps, and cycles per tile step of both paths, of issuing one step and
// of one fold.  Also: residency of CTAs that hold tensor memory.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "../../include/pyinla_gb300.h"
#include "bta_umma.cuh"

namespace gbta {

constexpr int PU_CONFIGS = 7;
constexpr int PU_OUT = PU_CONFIGS + 3;
constexpr int PU_STAGE_H = UMMA_STAGE_PLANES * OZ_PLANE;
constexpr size_t PU_XCH = NT * 64 * sizeof(float);
constexpr size_t PU_SMEM = 512 + PU_STAGE_H * sizeof(__half) + 2 * OZ_OPER * sizeof(__half) + PU_XCH +
                           TS * TS * sizeof(float) + 2 * TS * TS * sizeof(double);

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
  __half* L = stage;                                   // shifted left planes
  __half* R = stage + UMMA_RIGHT_PLANE * OZ_PLANE;
  __half* Lorig = stage + PU_STAGE_H;                  // unshifted left planes
  __half* Ash = Lorig + OZ_OPER;                       // shifted left planes for mma.sync
  float* xch = reinterpret_cast<float*>(Ash + OZ_OPER);
  float* x44 = reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(xch) + PU_XCH);
  double* vref = reinterpret_cast<double*>(x44 + TS * TS);
  double* vu = vref + TS * TS;
  umma_init(&us);
  for (int idx = threadIdx.x; idx < OZ_OPER; idx += NT) {
    Lorig[idx] = pu_digit(idx, 1);
    R[idx] = pu_digit(idx, 2);
  }
  __syncthreads();
  int st = 0;   // completion barrier of the next step (they rotate)

  // left planes shifted by q into L (tensor core) and Ash (mma.sync)
  auto shift_left = [&](int q) {
    for (int idx = threadIdx.x; idx < OZ_OPER; idx += NT) {
      const __half x = (idx / OZ_PLANE) >= q ? Lorig[idx - q * OZ_PLANE] : __int2half_rn(0);
      L[idx] = x;
      Ash[idx] = x;
    }
    fence_async_smem();
    __syncthreads();
  };
  // reference: `nsteps` mma.sync steps folded into vref
  auto reference = [&](bool trans, int nsteps) {
    OzAcc acc;
    oz_clear_partials(acc);
    for (int k = 0; k < nsteps; ++k) {
      if (trans)
        oz_step_t<true>(acc, Ash, R);
      else
        oz_step_t<false>(acc, Ash, R);
    }
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
  };
  auto drain_all = [&]() -> bool {
    bool ok = true;
    if (threadIdx.x == 0)
      for (int k = 0; k < UMMA_NSTAGE; ++k) ok = umma_drain_stage(&us, k) && ok;
    return __syncthreads_and(ok);
  };
  float p44[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
  auto issue = [&](bool trans, bool swap, bool& fresh) {
    if (threadIdx.x == 0) {
      umma_drain_stage(&us, st);
      umma_oz_step(&us, st, stage, trans, fresh, swap);
    }
    oz_pair44(p44, stage, trans);
    st = (st + 1) % UMMA_NSTAGE;
  };
  // `nsteps` tensor-core steps folded into vu; mismatching bits against vref (-1: a
  // completion wait ran out)
  auto check = [&](bool trans, bool swap, int nsteps) -> int {
    bool fresh = true;
    for (int k = 0; k < nsteps; ++k) issue(trans, swap, fresh);
    const bool ok = drain_all();
    tmem_fence_before();
    __syncthreads();
    double v[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) v[e] = 0.0;
    umma_fold_sub(&us, 40, v, p44, xch, x44);
#pragma unroll
    for (int e = 0; e < 8; ++e) vu[umma_row(e) * TS + umma_col()] = v[e];
    if (threadIdx.x == 0) s_mis = 0;
    __syncthreads();
    int bad = 0;
    for (int idx = threadIdx.x; idx < TS * TS; idx += NT)
      bad += __double_as_longlong(vref[idx]) != __double_as_longlong(vu[idx]);
    atomicAdd(&s_mis, bad);
    __syncthreads();
    const int r = ok ? s_mis : -1;
    __syncthreads();
    return r;
  };

  const int cfg_t[PU_CONFIGS] = {0, 1, 0, 1, 0, 1, 0};
  const int cfg_q[PU_CONFIGS] = {0, 0, 2, 3, 5, 7, 7};
  for (int k = 0; k < PU_CONFIGS; ++k) {
    shift_left(cfg_q[k]);
    reference(cfg_t[k] != 0, 1);
    const int r = check(cfg_t[k] != 0, false, 1);
    if (threadIdx.x == 0) mism[k] = r;
  }
  // transposed left tile with the two MN-major offsets in the other descriptor fields
  shift_left(0);
  reference(true, 1);
  {
    const int r = check(true, true, 1);
    if (threadIdx.x == 0) mism[PU_CONFIGS] = r;
  }
  // two steps into the same accumulators, both orientations
  reference(true, 2);
  {
    const int r = check(true, false, 2);
    if (threadIdx.x == 0) mism[PU_CONFIGS + 1] = r;
  }
  reference(false, 2);
  {
    const int r = check(false, false, 2);
    if (threadIdx.x == 0) mism[PU_CONFIGS + 2] = r;
  }

  // cycles per tile step: tcgen05 (steps in flight up to the stage count, then drain)
  // and mma.sync
  {
    bool fresh = true;
    __syncthreads();
    long long t0 = clock64();
    for (int it = 0; it < iters; ++it) issue(false, false, fresh);
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
    if (sink == 12345.f) cyc[4] = 1;   // keeps the products live
  }
  // cycles of thread 0 issuing one step (no MMA in flight), and of one fold (MMAs done)
  {
    bool fresh = true;
    drain_all();
    long long t0 = clock64();
    if (threadIdx.x == 0) {
      umma_oz_step(&us, st, stage, false, fresh);
      cyc[2] = clock64() - t0;
    }
    st = (st + 1) % UMMA_NSTAGE;
    drain_all();
    tmem_fence_before();
    __syncthreads();
    double v[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) v[e] = 0.0;
    t0 = clock64();
    umma_fold_sub(&us, 40, v, p44, xch, x44);
    const long long t1 = clock64();
    if (threadIdx.x == 0) cyc[3] = t1 - t0;
    if (v[0] == 12345.0) cyc[4] = 2;
  }
  umma_release(&us);
}

// Residency of CTAs that hold tensor memory: every CTA allocates UMMA_TMEM_COLS
// columns, holds them for hold_ns and records its SM, start, allocation and end times.
__global__ void __launch_bounds__(NT, 1) k_probe_tmem_pairs(long long* rec, unsigned long long hold_ns) {
  __shared__ unsigned taddr;
  const unsigned long long t0 = gtimer();
  if (threadIdx.x < 32) tmem_alloc(&taddr);
  tmem_fence_before();
  __syncthreads();
  tmem_fence_after();
  const unsigned long long t1 = gtimer();
  while (gtimer() - t1 < hold_ns) {
  }
  tmem_fence_before();
  __syncthreads();
  tmem_fence_after();
  if (threadIdx.x < 32) tmem_dealloc(taddr);
  if (threadIdx.x == 0) {
    long long* r = rec + 4 * blockIdx.x;
    r[0] = smid();
    r[1] = (long long)t0;
    r[2] = (long long)t1;
    r[3] = (long long)gtimer();
  }
}

}  // namespace gbta

extern "C" int gbta_set_error(int code, const char* msg);

extern "C" int gbta_probe_umma(int iters, int* mismatches, long long* cycles) {
  if (!mismatches || !cycles || iters < 1) return gbta_set_error(GBTA_ERR_ARG, "probe_umma: need iters >= 1 and outputs");
  int* d_mis = nullptr;
  long long* d_cyc = nullptr;
  if (cudaMalloc(&d_mis, gbta::PU_OUT * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&d_cyc, 5 * sizeof(long long)) != cudaSuccess) {
    cudaFree(d_mis);
    return gbta_set_error(GBTA_ERR_ALLOC, "probe_umma: cudaMalloc failed");
  }
  cudaFuncSetAttribute(gbta::k_probe_umma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gbta::PU_SMEM);
  gbta::k_probe_umma<<<1, gbta::NT, gbta::PU_SMEM>>>(d_mis, d_cyc, iters);
  gbta::count_launches(1);
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(mismatches, d_mis, gbta::PU_OUT * sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(cycles, d_cyc, 4 * sizeof(long long), cudaMemcpyDeviceToHost);
  cudaFree(d_mis);
  cudaFree(d_cyc);
  if (e != cudaSuccess) return gbta_set_error(GBTA_ERR_CUDA, cudaGetErrorString(e));
  return GBTA_OK;
}

// out[0]: CTAs per SM the occupancy calculator allows for the probe kernel (100 KB of
// shared memory, UMMA_TMEM_COLS tensor-memory columns per CTA); out[1]: SMs that ran
// two such CTAs at once; out[2]: SMs that got two CTAs; out[3]: the longest wait of a
// CTA for its tensor memory (ns); out[4]: CTAs per SM that fit its registers, shared
// and tensor memory (resident_ctas, the grid rule of tensor-memory kernels).
extern "C" int gbta_probe_tmem_pairs(long long* out) {
  if (!out) return gbta_set_error(GBTA_ERR_ARG, "probe_tmem_pairs: null output");
  int nsm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, 0);
  const int grid = 2 * nsm;
  const size_t smem = 100 * 1024;   // two CTAs per SM at most
  cudaFuncSetAttribute(gbta::k_probe_tmem_pairs, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaFuncSetAttribute(gbta::k_probe_tmem_pairs, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  {
    int calc = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&calc, gbta::k_probe_tmem_pairs, gbta::NT, smem) != cudaSuccess)
      calc = -1;
    out[0] = calc;
    out[4] = gbta::resident_ctas((const void*)gbta::k_probe_tmem_pairs, gbta::NT, smem, gbta::UMMA_TMEM_COLS);
  }
  long long* d_rec = nullptr;
  if (cudaMalloc(&d_rec, (size_t)grid * 4 * sizeof(long long)) != cudaSuccess)
    return gbta_set_error(GBTA_ERR_ALLOC, "probe_tmem_pairs: cudaMalloc failed");
  cudaFuncSetAttribute(gbta::k_probe_tmem_pairs, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaFuncSetAttribute(gbta::k_probe_tmem_pairs, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  gbta::k_probe_tmem_pairs<<<grid, gbta::NT, smem>>>(d_rec, 200000ull);
  gbta::count_launches(1);
  cudaError_t e = cudaDeviceSynchronize();
  std::vector<long long> rec((size_t)grid * 4);
  if (e == cudaSuccess) e = cudaMemcpy(rec.data(), d_rec, rec.size() * sizeof(long long), cudaMemcpyDeviceToHost);
  cudaFree(d_rec);
  if (e != cudaSuccess) return gbta_set_error(GBTA_ERR_CUDA, cudaGetErrorString(e));
  long long both = 0, pairs = 0, maxwait = 0;
  for (int a = 0; a < grid; ++a) {
    maxwait = std::max(maxwait, rec[4 * a + 2] - rec[4 * a + 1]);
    for (int b = a + 1; b < grid; ++b) {
      if (rec[4 * a] != rec[4 * b]) continue;
      ++pairs;
      if (rec[4 * a + 2] < rec[4 * b + 3] && rec[4 * b + 2] < rec[4 * a + 3]) ++both;
    }
  }
  out[1] = both;
  out[2] = pairs;
  out[3] = maxwait;
  return GBTA_OK;
}
