// BTA Cholesky factorization that allocates no device memory.
//
// Some callers cannot allocate device memory at the point where they need a
// factorization: hosts that own a fixed device-memory pool and forbid allocations
// outside it (custom-call hooks of other frameworks, long-running services that
// reserve their whole arena up front), and latency-sensitive loops where the implicit
// device-wide synchronisation of cudaMalloc/cudaFree is not acceptable.  For them,
// gbta_pobtaf_noalloc runs the FP64-product dataflow factorization kernel (k_factor) in
// the elimination order of gbta_pobtaf (so the sweeps and the inversion of a solver
// accept its factor),
// with every piece of its scratch -- control words, per-tile ready flags, the task
// list and the arrow-tip partial products -- placed in one file-scope __device__ array
// of GBTA_NOALLOC_SCRATCH_BYTES (64 MiB).  The caller passes only the block buffers.
//
// The array is part of this file's device module.  The library is built with one
// module per source file, and CUDA loads modules lazily by default, so the array (and
// the code of this path) takes device memory when the module is first used on a GPU
// -- the first call there -- and keeps it until the process exits; with
// CUDA_MODULE_LOADING=EAGER the load happens at context creation instead.  A caller
// that reserves a memory pool makes its first call before reserving it.
//
// All calls on a device share the array and it keeps the previous call's contents:
// each call clears the part that must start at zero (control words and ready flags)
// and regenerates the rest, and calls whose work overlaps on the GPU (different
// streams, or different host threads, at the same time) race on it.
//
// In host code the array's name is only a host-side stand-in, not a device address,
// so its device address is looked up with cudaGetSymbolAddress, once per device with
// that device current, the first time the entry point runs there; that first call
// should therefore come before any stream capture.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/pyinla_gb300.h"
#include "bta_internal.h"

namespace gbta {

static __device__ __align__(256) unsigned char g_noalloc_scratch[GBTA_NOALLOC_SCRATCH_BYTES];

// Writes the factorization task list without the feeder split (no FT_PRE products and
// no FT_FEEDQ row groups, which k_factor accepts when it is given no feeder flags), in
// the elimination order of the regular path: the columns of the two chains interleaved
// one for one (Geom::interleave), then the separator's columns, then TIP (a > 0).  Per
// column (i, c): DIAG, OFFD (r > c), LOW (every block but the separator), ARW (a > 0).
// Every task waits only for tasks earlier in this order.  One thread per column; its
// offset is the number of tasks of the columns before it, in closed form: a column c of
// a chain has f(c) = 2B + ab - c tasks, one of the separator B + ab - c.
__device__ __forceinline__ long long noalloc_chain_tasks(long long n, int B, int ab) {   // sum_{k<n} f(k % B)
  const long long full = n / B, q = n % B;
  const long long fb = (long long)B * (2 * B + ab) - (long long)B * (B - 1) / 2;
  return full * fb + q * (2 * B + ab) - q * (q - 1) / 2;
}

__global__ void k_gen_factor_tasks(Geom g, int4* tasks) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= g.nt * g.B) return;
  const int B = g.B, ab = g.a > 0 ? 1 : 0, sp = g.sep();
  const int n1 = sp * B, n2 = (g.nt - 1 - sp) * B, mn = n1 < n2 ? n1 : n2;
  int i, c;
  long long off;
  if (q < n1 + n2) {
    int k;
    const int ch = Geom::interleave(n1, n2, q, &k);
    i = ch == 0 ? k / B : g.nt - 1 - k / B;
    c = k % B;
    if (q < 2 * mn)
      off = 2 * noalloc_chain_tasks(q >> 1, B, ab) + ((q & 1) ? 2 * B + ab - c : 0);
    else
      off = noalloc_chain_tasks(mn, B, ab) + noalloc_chain_tasks(k, B, ab);
  } else {
    i = sp;
    c = q - (n1 + n2);
    const long long osep = noalloc_chain_tasks(mn, B, ab) + noalloc_chain_tasks(n1 + n2 - mn, B, ab);
    off = osep + (long long)c * (B + ab) - (long long)c * (c - 1) / 2;
  }
  tasks[off++] = make_int4(FT_DIAG, i, c, c);
  for (int r = c + 1; r < B; ++r) tasks[off++] = make_int4(FT_OFFD, i, r, c);
  if (g.nxt(i) >= 0)
    for (int r = 0; r < B; ++r) tasks[off++] = make_int4(FT_LOW, i, r, c);
  if (ab) tasks[off++] = make_int4(FT_ARW, i, 0, c);
  if (ab && q == g.nt * B - 1) tasks[off] = make_int4(FT_TIP, 0, 0, 0);
}

}  // namespace gbta

extern "C" int gbta_set_error(int code, const char* msg);

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {};

size_t align256(size_t n) { return (n + 255) & ~size_t(255); }

}  // namespace

extern "C" size_t gbta_noalloc_scratch_bytes(int b, int nt, int a) {
  if (b < 1 || nt < 1 || a < 0) return 0;
  const long long B = (b + gbta::TS - 1) / gbta::TS;
  const long long nflags = (2LL * nt - 1) * B * B + (long long)nt * B + 1;
  const long long per_block = B * (1 + (nt > 1 ? B : 0) + (a > 0 ? 1 : 0)) + B * (B - 1) / 2;
  const long long ntasks = nt * per_block - (nt > 1 ? B * B : 0) + (a > 0 ? 1 : 0);
  size_t bytes = align256(8 * sizeof(int));
  bytes += align256((size_t)nflags * sizeof(int));
  bytes += align256((size_t)ntasks * sizeof(int4));
  bytes += align256((size_t)nt * B * gbta::TS * gbta::TS * sizeof(double));
  return bytes;
}

extern "C" int gbta_pobtaf_noalloc(int b, int nt, int a, double* D, double* L, double* R, double* T, void* stream) {
  if (b < 1 || nt < 1 || a < 0) return gbta_set_error(GBTA_ERR_ARG, "noalloc pobtaf: require b >= 1, nt >= 1, a >= 0");
  if (a > gbta::TS) return gbta_set_error(GBTA_ERR_ARG, "noalloc pobtaf: arrowhead block size above 32 is not supported");
  if (!D || (nt > 1 && !L) || (a > 0 && (!R || !T)))
    return gbta_set_error(GBTA_ERR_ARG, "noalloc pobtaf: D/L (and R/T when a > 0) must be device pointers");
  const size_t need = gbta_noalloc_scratch_bytes(b, nt, a);
  if (need > (size_t)GBTA_NOALLOC_SCRATCH_BYTES)
    return gbta_set_error(GBTA_ERR_ARG, ("noalloc pobtaf: this problem needs " + std::to_string(need) +
                                         " bytes of scratch, above the fixed limit of " +
                                         std::to_string((size_t)GBTA_NOALLOC_SCRATCH_BYTES) + " bytes")
                                            .c_str());
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return gbta_set_error(GBTA_ERR_CUDA, "noalloc pobtaf: no usable current device");
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
      const cudaError_t e = cudaGetSymbolAddress(&g_addr[dev], gbta::g_noalloc_scratch);
      if (e != cudaSuccess) {
        g_addr[dev] = nullptr;
        return gbta_set_error(GBTA_ERR_CUDA, (std::string("noalloc pobtaf: loading the library's fixed ") +
                                              std::to_string((size_t)GBTA_NOALLOC_SCRATCH_BYTES >> 20) +
                                              " MiB scratch array on this device failed (" + cudaGetErrorString(e) +
                                              (e == cudaErrorMemoryAllocation
                                                   ? "): the first call on a device loads it; make that call "
                                                     "before reserving the device memory pool, or set "
                                                     "CUDA_MODULE_LOADING=EAGER"
                                                   : ")"))
                                                 .c_str());
      }
    }
    base = g_addr[dev];
  }
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return gbta_set_error(GBTA_ERR_CUDA, "noalloc pobtaf: cannot query the SM count");

  gbta::Geom g{b, nt, a, (b + gbta::TS - 1) / gbta::TS};
  g.m = gbta::default_sep(nt);   // the elimination order of gbta_pobtaf
  const long long nflags = (2LL * nt - 1) * g.B * g.B + (long long)nt * g.B + 1;
  const long long per_block = (long long)g.B * (1 + (nt > 1 ? g.B : 0) + (a > 0 ? 1 : 0)) + (long long)g.B * (g.B - 1) / 2;
  const long long ntasks = nt * per_block - (nt > 1 ? (long long)g.B * g.B : 0) + (a > 0 ? 1 : 0);
  unsigned char* p = static_cast<unsigned char*>(base);
  int* ctrl = reinterpret_cast<int*>(p);
  p += align256(8 * sizeof(int));
  int* flags = reinterpret_cast<int*>(p);
  p += align256((size_t)nflags * sizeof(int));
  int4* tasks = reinterpret_cast<int4*>(p);
  p += align256((size_t)ntasks * sizeof(int4));
  double* tip_part = reinterpret_cast<double*>(p);

  cudaStream_t st = (cudaStream_t)stream;
  // Control words and ready flags must start at zero; the task list is regenerated;
  // the tip partials are fully written before they are read.
  cudaError_t e = cudaMemsetAsync(ctrl, 0, (size_t)(reinterpret_cast<unsigned char*>(tasks) -
                                                     reinterpret_cast<unsigned char*>(ctrl)), st);
  if (e != cudaSuccess) return gbta_set_error(GBTA_ERR_CUDA, cudaGetErrorString(e));
  const int ncol = nt * g.B;
  gbta::k_gen_factor_tasks<<<(ncol + 127) / 128, 128, 0, st>>>(g, tasks);
  if (nt > 1) gbta::launch_transpose_lslots(g, L, st);
  gbta::LaunchCtl lc;
  lc.ctrl = ctrl;
  lc.flags = flags;
  lc.epoch = 1 << gbta::EPOCH_SHIFT;
  lc.wait_ns = 20ull * 1000 * 1000 * 1000;
  lc.grid = (int)(ntasks < nsm ? ntasks : nsm);
  lc.stream = st;
  gbta::launch_factor(g, D, L, R, T, a > 0 ? 1 : 0, tasks, (int)ntasks, tip_part, lc);
  gbta::count_launches(1);
  if ((e = cudaGetLastError()) != cudaSuccess)
    return gbta_set_error(GBTA_ERR_CUDA, (std::string("noalloc pobtaf: launch failed (") + cudaGetErrorString(e) +
                                          (e == cudaErrorMemoryAllocation
                                               ? "): loading the factorization kernel's code on its first use "
                                                 "needs device memory; make the first call before reserving the "
                                                 "device memory pool, or set CUDA_MODULE_LOADING=EAGER"
                                               : ")"))
                                             .c_str());
  int h_ctrl[8] = {0};
  if ((e = cudaMemcpyAsync(h_ctrl, ctrl, sizeof(h_ctrl), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return gbta_set_error(GBTA_ERR_CUDA, cudaGetErrorString(e));
  if (h_ctrl[3] != 0) return gbta_set_error(GBTA_ERR_TIMEOUT, "noalloc pobtaf: a kernel wait exceeded its limit");
  if (h_ctrl[2] > 0)
    return gbta_set_error(h_ctrl[2], ("matrix is not positive definite (non-positive pivot at global row " +
                                      std::to_string(h_ctrl[2]) + ")").c_str());
  return GBTA_OK;
}
