// FP64 peak probe and kernel-launch accounting.
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

// Chip-wide throughput of the candidate arithmetic paths for FP64 tile products,
// 2 CTAs of 256 threads per SM, register-only loops timed with CUDA events:
// [0] DMMA mma.sync.m8n8k4.f64, [1] HMMA mma.sync.m16n8k16 f16 -> f32, [2] FFMA.
namespace gbta {
__global__ void __launch_bounds__(256) k_rate_dmma(double* out, int iters) {
  double a = 1.0 + threadIdx.x * 1e-9, b = 0.5;
  double c[8][2];
#pragma unroll
  for (int k = 0; k < 8; ++k) c[k][0] = c[k][1] = k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                   : "+d"(c[k][0]), "+d"(c[k][1])
                   : "d"(a), "d"(b));
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += c[k][0] + c[k][1];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
__global__ void __launch_bounds__(256) k_rate_hmma(double* out, int iters) {
  const unsigned a0 = 0x3c003c00u, b0 = 0x3c003c00u;   // fp16 ones
  float c[8][4];
#pragma unroll
  for (int k = 0; k < 8; ++k) c[k][0] = c[k][1] = c[k][2] = c[k][3] = 0.f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k)
      asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                   "{%0,%1,%2,%3};"
                   : "+f"(c[k][0]), "+f"(c[k][1]), "+f"(c[k][2]), "+f"(c[k][3])
                   : "r"(a0), "r"(a0), "r"(a0), "r"(a0), "r"(b0), "r"(b0));
  }
  float s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += c[k][0] + c[k][1] + c[k][2] + c[k][3];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
__global__ void __launch_bounds__(256) k_rate_ffma(double* out, int iters) {
  float x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-6f + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fmaf(x[k], 0.9999f, 1e-7f);
  }
  float s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace gbta

extern "C" int gbta_probe_tensor_rates(int iters, double* tflops) {
  if (!tflops || iters < 1) return gbta_set_error(GBTA_ERR_ARG, "probe: need iters >= 1 and an output");
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return gbta_set_error(GBTA_ERR_CUDA, "probe: no device");
  const int blocks = nsm * 2, threads = 256;
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess)
    return gbta_set_error(GBTA_ERR_ALLOC, "probe: cudaMalloc failed");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // flops per thread and iteration: DMMA 8 x (8*8*4*2)/32, HMMA 8 x (16*8*16*2)/32, FFMA 8 x 2
  const double per_thread_iter[3] = {8.0 * 512 / 32, 8.0 * 4096 / 32, 16.0};
  cudaError_t err = cudaSuccess;
  for (int k = 0; k < 3 && err == cudaSuccess; ++k) {
    for (int rep = 0; rep < 2; ++rep) {   // the first run warms up
      cudaEventRecord(e0);
      if (k == 0) gbta::k_rate_dmma<<<blocks, threads>>>(out, iters);
      if (k == 1) gbta::k_rate_hmma<<<blocks, threads>>>(out, iters);
      if (k == 2) gbta::k_rate_ffma<<<blocks, threads>>>(out, iters);
      cudaEventRecord(e1);
      err = cudaEventSynchronize(e1);
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    tflops[k] = per_thread_iter[k] * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
  }
  gbta::count_launches(6);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return gbta_set_error(GBTA_ERR_CUDA, cudaGetErrorString(err));
  return GBTA_OK;
}
