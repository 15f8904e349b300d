// FP64 peak probe, launch-shape helpers and kernel-launch accounting.
//
// GB300 has no FP64 tensor-core rate worth using (its DMMA path measures below the
// CUDA-core DFMA rate), so the roofline denominator of the FP64 kernels is the DFMA
// throughput of the whole chip, measured here with independent FMA chains on every SM.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>

#include "../../include/pyinla_gb300.h"
#include "bta_internal.h"

namespace gbta {

std::atomic<long long> g_launches{0};

void count_launches(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

int resident_ctas(const void* kernel, int threads, size_t smem, int tmem_cols) {
  cudaFuncAttributes fa;
  int dev = 0;
  if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess || cudaGetDevice(&dev) != cudaSuccess) return 1;
  int regs_sm = 0, smem_sm = 0, resv = 0, thr_sm = 0, blk_sm = 0;
  cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&resv, cudaDevAttrReservedSharedMemoryPerBlock, dev);
  cudaDeviceGetAttribute(&thr_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev);
  cudaDeviceGetAttribute(&blk_sm, cudaDevAttrMaxBlocksPerMultiprocessor, dev);
  const long long warps = (threads + 31) / 32;
  const long long regs_warp = ((long long)fa.numRegs * 32 + 255) / 256 * 256;   // 256-register units
  const long long smem_cta = (long long)smem + (long long)fa.sharedSizeBytes + resv;
  long long n = blk_sm;
  if (regs_warp > 0) n = std::min(n, (long long)regs_sm / (regs_warp * warps));
  n = std::min(n, (long long)thr_sm / threads);
  if (smem_cta > 0) n = std::min(n, (long long)smem_sm / smem_cta);
  if (tmem_cols > 0) n = std::min(n, (long long)(512 / tmem_cols));
  return n < 1 ? 1 : (int)n;
}

int launch_grid(const void* kernel, int threads, size_t smem, const LaunchCtl& lc) {
  if (lc.nsm <= 0) return lc.grid;
  int occ = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, threads, smem) != cudaSuccess || occ < 1) occ = 1;
  const int per = lc.ctas_per_sm > 0 ? (lc.ctas_per_sm < occ ? lc.ctas_per_sm : occ) : occ;
  long long g = (long long)lc.nsm * per;
  if (lc.ntasks > 0 && g > lc.ntasks) g = lc.ntasks;
  return g < 1 ? 1 : (int)g;
}

__global__ void __launch_bounds__(256) k_dfma_peak(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-9, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
         x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b);
    x1 = fma(x1, a, b);
    x2 = fma(x2, a, b);
    x3 = fma(x3, a, b);
    x4 = fma(x4, a, b);
    x5 = fma(x5, a, b);
    x6 = fma(x6, a, b);
    x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

}  // namespace gbta

extern "C" int gbta_set_error(int code, const char* msg);

extern "C" long long gbta_kernel_launches(void) { return gbta::g_launches.load(std::memory_order_relaxed); }

extern "C" int gbta_probe_fp64_peak(int iters, double* tflops) {
  if (!tflops || iters < 1) return gbta_set_error(GBTA_ERR_ARG, "probe: need iters >= 1 and an output");
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return gbta_set_error(GBTA_ERR_CUDA, "probe: no device");
  const int blocks = nsm * 2, threads = 256;
  double* out = nullptr;
  cudaEvent_t e0, e1;
  if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess)
    return gbta_set_error(GBTA_ERR_ALLOC, "probe: cudaMalloc failed");
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  gbta::k_dfma_peak<<<blocks, threads>>>(out, 64, 1.0000001, 1e-7);   // warm-up
  cudaEventRecord(e0);
  gbta::k_dfma_peak<<<blocks, threads>>>(out, iters, 1.0000001, 1e-7);
  cudaEventRecord(e1);
  const cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  gbta::count_launches(2);
  if (e != cudaSuccess) return gbta_set_error(GBTA_ERR_CUDA, cudaGetErrorString(e));
  *tflops = 2.0 * 8.0 * (double)iters * blocks * threads / (ms * 1e-3) / 1e12;
  return GBTA_OK;
}
