// Digit-plane products on the 5th-generation tensor cores (tcgen05.mma, kind::f16,
// fp32 accumulators in tensor memory).
//
// One tile step adds P_d(m, n) = sum_{s+t=d} sum_k X_s(m, k) Y_t(n, k) (d = 0 .. 8, the
// 43 pairs s + t <= 8 of the digit planes X_s of the left tile and Y_t of the right
// tile) to nine fp32 accumulators, as 32 x 32 x 32 integer products (see
// bta_ozaki.cuh for the digit scheme and why fp32 accumulation is exact).
//
// The diagonal sums are formed by the tensor core itself.  For a group of four
// consecutive diagonals d0 .. d0+3 and one left plane s, the A operand (M = 128 rows)
// is the right tile's planes t = d0 - s .. d0 - s + 3 stacked (row 32 j + n = row n of
// plane d0 + j - s), and the B operand (N = 32) is the left plane s: accumulator row
// 32 j + n, column m then collects P_{d0+j}(m, n) over s.  The planes of a tile are
// contiguous 2 KB blocks, so the stacked operand is one shared-memory descriptor whose
// start moves by one plane per s; zero planes before and after the right tile supply
// t < 0 and t = 8.  Three groups cover the nine diagonals: {0} (s = 0), {1..4}
// (s = 0..4) and {5..8} (s = 0..7): 14 left planes x 2 K-halves = 28 MMAs of
// 128 x 32 x 16 per tile step, 96 accumulator columns.
//
// A left tile in the frame of a larger exponent is shifted down by q planes (its
// plane s is global plane s - q): the shift only skips the MMAs with s < q and moves
// the B descriptor, no data is moved.  A transposed left tile (stored [k][m]) is read
// as an MN-major operand.
//
// Layouts: every plane is 32 rows of 64 bytes with the 16-byte chunks of row r
// permuted by (r >> 1) & 3 (oz_swz), which is the 64-byte swizzle of the tensor core
// when the plane starts on a 512-byte boundary.
#pragma once

#include "bta_ozaki.cuh"

namespace gbta {

constexpr int UMMA_TMEM_COLS = 128;   // accumulator columns allocated per CTA (96 used)
constexpr int UMMA_GROUPS = 3;
constexpr int UMMA_ZLEAD = 3;         // zero planes before the right tile
// Planes of one stage buffer: left tile (8), zero planes (3), right tile (8), zero (1).
constexpr int UMMA_STAGE_PLANES = OZ_S + UMMA_ZLEAD + OZ_S + 1;
constexpr int UMMA_RIGHT_PLANE = OZ_S + UMMA_ZLEAD;

__device__ __forceinline__ int umma_group_d0(int gi) { return gi == 0 ? 0 : (gi == 1 ? 1 : 5); }
__device__ __forceinline__ int umma_group_smax(int gi) { return gi == 0 ? 0 : (gi == 1 ? 4 : 7); }
// Accumulator groups written by a step whose left tile is shifted by q planes.
__device__ __forceinline__ unsigned umma_groups_written(int q) {
  return (q == 0 ? 1u : 0u) | (q <= 4 ? 2u : 0u) | (q <= 7 ? 4u : 0u);
}

// Shared-memory matrix descriptor: 64-byte swizzle, 8-row groups 512 bytes apart (both
// offset fields; only one is used for the K-major and MN-major 32-wide operands here).
__device__ __forceinline__ unsigned long long umma_sdesc(unsigned saddr) {
  return (unsigned long long)((saddr >> 4) & 0x3fffu) | ((unsigned long long)(512 >> 4) << 16) |
         ((unsigned long long)(512 >> 4) << 32) | (1ull << 46) | (4ull << 61);
}
// Instruction descriptor: fp32 accumulator, fp16 A and B, A K-major, B K-major or
// MN-major, N = 32, M = 128.
__device__ __forceinline__ unsigned umma_idesc(bool b_mn_major) {
  return (1u << 4) | ((b_mn_major ? 1u : 0u) << 16) | ((32u >> 3) << 17) | ((128u >> 4) << 24);
}

__device__ __forceinline__ void umma_f16(unsigned dtmem, unsigned long long a, unsigned long long b, unsigned idesc,
                                         unsigned accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(dtmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}
// Arrive once on the barrier when every MMA issued so far by this thread has finished.
__device__ __forceinline__ void umma_commit(unsigned long long* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tmem_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Warp-wide: allocate / free UMMA_TMEM_COLS columns (the address goes to *s_addr).
__device__ __forceinline__ void tmem_alloc(unsigned* s_addr) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(s_addr)),
               "n"(UMMA_TMEM_COLS)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(unsigned taddr) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "n"(UMMA_TMEM_COLS)
               : "memory");
}

// Warp-wide: 32 consecutive accumulator columns of the warp's 32 lanes.
__device__ __forceinline__ void tmem_ld32(unsigned taddr, float (&v)[32]) {
  unsigned r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
      "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 32; ++k) v[k] = __uint_as_float(r[k]);
}

// Warp-wide: 8 consecutive accumulator columns of the warp's 32 lanes.
__device__ __forceinline__ void tmem_ld8(unsigned taddr, float (&v)[8]) {
  unsigned r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr)
               : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k] = __uint_as_float(r[k]);
}

// Bounded wait for the next completion (parity) of an mbarrier; false if it ran out.
__device__ __forceinline__ bool mbar_wait_parity(unsigned long long* bar, unsigned parity) {
  for (int it = 0; it < (1 << 22); ++it) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Per-CTA state of the tensor-memory products, kept across tasks: the accumulator
// address, one MMA-completion barrier per stage buffer, their parities and which of
// them still has a commit outstanding.
struct UmmaState {
  unsigned long long bar[2];
  unsigned tmem;
  unsigned parity;    // bit st: parity of the next completion of bar[st]
  unsigned pending;   // bit st: a commit on bar[st] not yet waited for
};

// All threads: barriers, accumulator allocation (warp 0).  Contains __syncthreads().
__device__ __forceinline__ void umma_init(UmmaState* us) {
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&us->bar[0])) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&us->bar[1])) : "memory");
    us->parity = 0;
    us->pending = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (threadIdx.x < 32) tmem_alloc(&us->tmem);
  tmem_fence_before();
  __syncthreads();
  tmem_fence_after();
}

// Thread 0: wait (bounded) for the outstanding commit of stage st, if any.
__device__ __forceinline__ bool umma_drain_stage(UmmaState* us, int st) {
  if (!((us->pending >> st) & 1u)) return true;
  const bool ok = mbar_wait_parity(&us->bar[st], (us->parity >> st) & 1u);
  us->parity ^= 1u << st;
  us->pending &= ~(1u << st);
  return ok;
}

// All threads, at the end of the kernel: wait for the outstanding MMAs, then free the
// accumulators (warp 0).  Contains __syncthreads().
__device__ __forceinline__ void umma_release(UmmaState* us) {
  if (threadIdx.x == 0) {
    umma_drain_stage(us, 0);
    umma_drain_stage(us, 1);
  }
  tmem_fence_before();
  __syncthreads();
  tmem_fence_after();
  if (threadIdx.x < 32) tmem_dealloc(us->tmem);
}

// Thread 0: issue one tile step from stage buffer `stage` (the left tile at plane 0,
// the right tile at UMMA_RIGHT_PLANE, zero planes around it; 512-byte aligned) and
// commit it to bar[st].  q: plane shift of the left tile (>= OZ_S: nothing to add);
// trans: the left planes are stored [k][m]; fresh: groups whose next MMA starts a new
// sum (cleared here for the groups written).
__device__ __forceinline__ void umma_oz_step(UmmaState* us, int st, const __half* stage, int q, bool trans,
                                             unsigned& fresh) {
  const unsigned lbase = smem_u32(stage), rbase = lbase + UMMA_RIGHT_PLANE * OZ_PLANE * 2;
  const unsigned idesc = umma_idesc(trans);
  tmem_fence_after();
#pragma unroll
  for (int gi = 0; gi < UMMA_GROUPS; ++gi) {
    const int d0 = umma_group_d0(gi), smax = umma_group_smax(gi);
    const unsigned dt = us->tmem + (unsigned)(gi * 32);
    for (int s = q; s <= smax; ++s) {
      const unsigned a0 = rbase + (unsigned)((d0 - s) * OZ_PLANE * 2);
      const unsigned b0 = lbase + (unsigned)((s - q) * OZ_PLANE * 2);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const unsigned acc = ((fresh >> gi) & 1u) ? 0u : 1u;
        umma_f16(dt, umma_sdesc(a0 + h * 32), umma_sdesc(b0 + (trans ? h * 1024 : h * 32)), idesc, acc);
        fresh &= ~(1u << gi);
      }
    }
  }
  umma_commit(&us->bar[st]);
  us->pending |= 1u << st;
}

// Output element ownership of the folded accumulator: thread (warp w, lane n) holds
// elements (m = 8 w + e, n), e = 0 .. 7.
__device__ __forceinline__ int umma_row(int e) { return 8 * (threadIdx.x >> 5) + e; }
__device__ __forceinline__ int umma_col() { return threadIdx.x & 31; }

// All threads: v[e] -= sum_d P_d(m, n) 2^(esum - 12 - 7 d) for the thread's elements,
// from the accumulator groups in `written` (the others count as zero).  The caller
// has made the last step's MMAs complete (bar wait by thread 0, then a barrier) and
// passes xch: 9 KB of shared scratch.  Contains __syncthreads().
__device__ __forceinline__ void umma_fold_sub(const UmmaState* us, unsigned written, int esum, double (&v)[8],
                                              float* xch) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const unsigned tl = us->tmem + ((unsigned)(32 * w) << 16);
  tmem_fence_after();
  // rounds r: elements m = 8 r .. 8 r + 7 (accumulator columns) go to warp r through
  // xch[d][e][n]
#pragma unroll 1
  for (int r = 0; r < 4; ++r) {
    float pv[8];
    if (w == 0 && (written & 1u)) {
      tmem_ld8(tl + 8 * r, pv);
#pragma unroll
      for (int e = 0; e < 8; ++e) xch[(0 * 8 + e) * 32 + lane] = pv[e];
    }
    if (written & 2u) {
      tmem_ld8(tl + 32 + 8 * r, pv);
#pragma unroll
      for (int e = 0; e < 8; ++e) xch[((1 + w) * 8 + e) * 32 + lane] = pv[e];
    }
    if (written & 4u) {
      tmem_ld8(tl + 64 + 8 * r, pv);
#pragma unroll
      for (int e = 0; e < 8; ++e) xch[((5 + w) * 8 + e) * 32 + lane] = pv[e];
    }
    if (r == 3) tmem_fence_before();
    __syncthreads();
    if (w == r) {
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        int I[OZ_ND];
#pragma unroll
        for (int d = 0; d < OZ_ND; ++d) {
          const unsigned gbit = d == 0 ? 1u : (d <= 4 ? 2u : 4u);
          I[d] = (written & gbit) ? __float2int_rn(xch[(d * 8 + e) * 32 + lane]) : 0;
        }
        const long long hi = (((long long)I[0] * 128 + I[1]) * 128 + I[2]) * 128 + I[3];
        const long long lo = ((((long long)I[4] * 128 + I[5]) * 128 + I[6]) * 128 + I[7]) * 128 + I[8];
        const double vv = fma((double)lo, 0x1p-35, (double)hi);
        const double sc = __longlong_as_double((long long)(1023 + esum - 33) << 52);
        v[e] = fma(-vv, sc, v[e]);
      }
    }
    __syncthreads();
  }
}

// Dynamic shared memory rounded up to the 512-byte boundary of the swizzled operands
// (the launch adds 512 bytes).
__device__ __forceinline__ unsigned char* smem_align512(unsigned char* p) {
  return p + ((512u - (smem_u32(p) & 511u)) & 511u);
}

// All threads: zero the zero planes of `nstages` stage buffers of UMMA_STAGE_PLANES
// planes each, visible to the tensor core.  Contains __syncthreads().
__device__ __forceinline__ void umma_zero_planes(__half* stages, int nstages) {
  constexpr int PER_PLANE = OZ_PLANE / 8;   // uint4 per plane
  constexpr int NZ = UMMA_ZLEAD + 1;
  for (int idx = threadIdx.x; idx < nstages * NZ * PER_PLANE; idx += NT) {
    const int st = idx / (NZ * PER_PLANE), z = (idx / PER_PLANE) % NZ, k = idx % PER_PLANE;
    const int plane = z < UMMA_ZLEAD ? OZ_S + z : UMMA_STAGE_PLANES - 1;
    reinterpret_cast<uint4*>(stages + ((size_t)st * UMMA_STAGE_PLANES + plane) * OZ_PLANE)[k] =
        make_uint4(0u, 0u, 0u, 0u);
  }
  fence_async_smem();
  __syncthreads();
}

}  // namespace gbta
