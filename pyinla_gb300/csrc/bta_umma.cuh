// Digit-plane products on the 5th-generation tensor cores (tcgen05.mma, kind::f16,
// fp32 accumulators in tensor memory).
//
// One tile step adds the pair products P_st(m, n) = sum_k X_s(m, k) Y_t(n, k) of the
// 43 pairs s + t <= 8 of the digit planes X_s of the left tile and Y_t of the right
// tile (32 x 32 x 32 integer products; bta_ozaki.cuh has the digit scheme) to fp32
// accumulators that a fold later combines per diagonal d = s + t.
//
// An MMA of 128 x N x 16 costs about the same for every N up to 128 and reaches the
// tensor core's rate only near N = 256, so the pairs are grouped into wide MMAs.  The
// A operand (M = 128) stacks four right planes (row 32 j + n = row n of plane t0 + j),
// the B operand stacks left planes along N (column 32 i + m), and the accumulator
// cell (lane block j, column block i) collects the pairs with s + t = i + j:
//   * right planes 0..3 x left planes 0..7 (N = 256): pair (s, t) into cell (t, s);
//   * right planes 4..7 x left planes 0..3 (N = 128, columns 128..255): pair (s, t)
//     into cell (t - 4, s + 4);
//   * the remaining pair (4, 4) runs on mma.sync (oz_pair44) into registers.
// Two K-halves each: 4 MMAs, 256 accumulator columns (two CTAs per SM fit in tensor
// memory), 48 pairs computed of which 42 are kept (the fold skips cells with
// i + j > 8).  A cell holds at most two pairs, so UMMA_CHUNK steps keep every cell,
// and the (4, 4) sums, below 2^24: fp32 accumulation stays exact.
//
// A left tile in the frame of a larger exponent is staged shifted down by q planes
// (global plane s - q in plane s, zeros below).  A transposed left tile (stored
// [k][m]) is read as an MN-major operand.
//
// Layouts: every plane is 32 rows of 64 bytes with the 16-byte chunks of row r
// permuted by (r >> 1) & 3 (oz_swz), which is the 64-byte swizzle of the tensor core
// when the plane starts on a 512-byte boundary.  A stage buffer holds the left tile's
// planes followed by the right tile's.
#pragma once

#include "bta_ozaki.cuh"

namespace gbta {

constexpr int UMMA_TMEM_COLS = 256;   // accumulator columns per CTA
constexpr int UMMA_CHUNK = 48;        // tile steps per exact fp32 accumulation
constexpr int UMMA_NSTAGE = 3;        // stage buffers of a product loop
constexpr int UMMA_RIGHT_PLANE = OZ_S;
constexpr int UMMA_ISSUER = 32;       // the thread that issues, commits and awaits the MMAs
constexpr int UMMA_STAGE_PLANES = 2 * OZ_S;
static_assert(2 * TS * 64 * 64 * UMMA_CHUNK < (1 << 24), "accumulator cells must stay below 2^24");
static_assert(8ll * 64 * 64 * TS * UMMA_CHUNK < (1ll << 31), "diagonal sums must fit in 32 bits");

// Shared-memory matrix descriptor, 64-byte swizzle: lbo / sbo are the byte offsets of
// the leading / stride dimension (for a K-major operand the 8-row groups are sbo
// apart; for an MN-major one the 32-element column blocks are lbo apart and the
// 8-row K groups sbo apart).
__device__ __forceinline__ unsigned long long umma_sdesc(unsigned saddr, unsigned lbo = 512, unsigned sbo = 512) {
  return (unsigned long long)((saddr >> 4) & 0x3fffu) | ((unsigned long long)((lbo >> 4) & 0x3fffu) << 16) |
         ((unsigned long long)((sbo >> 4) & 0x3fffu) << 32) | (1ull << 46) | (4ull << 61);
}
// Instruction descriptor: fp32 accumulator, fp16 A and B, A K-major, B K-major or
// MN-major, M = 128, N = n (a multiple of 16 up to 256).
__device__ __forceinline__ unsigned umma_idesc(bool b_mn_major, unsigned n = 32) {
  return (1u << 4) | ((b_mn_major ? 1u : 0u) << 16) | ((n >> 3) << 17) | ((128u >> 4) << 24);
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

// Warp-wide: allocate / free ncols columns (a power of two >= 32; the address goes to
// *s_addr).
__device__ __forceinline__ void tmem_alloc(unsigned* s_addr, unsigned ncols = UMMA_TMEM_COLS) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(s_addr)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(unsigned taddr, unsigned ncols = UMMA_TMEM_COLS) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
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
  unsigned long long bar[UMMA_NSTAGE];
  unsigned tmem;
  unsigned parity;    // bit st: parity of the next completion of bar[st]
  unsigned pending;   // bit st: a commit on bar[st] not yet waited for
};

// All threads: barriers, accumulator allocation (warp 0).  Contains __syncthreads().
__device__ __forceinline__ void umma_init(UmmaState* us, unsigned ncols = UMMA_TMEM_COLS) {
  if (threadIdx.x == 0) {
    for (int k = 0; k < UMMA_NSTAGE; ++k)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&us->bar[k])) : "memory");
    us->parity = 0;
    us->pending = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();   // the allocation is warp-wide
  if (threadIdx.x < 32) tmem_alloc(&us->tmem, ncols);
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
__device__ __forceinline__ void umma_release(UmmaState* us, unsigned ncols = UMMA_TMEM_COLS) {
  __syncthreads();
  if (threadIdx.x == UMMA_ISSUER)
    for (int k = 0; k < UMMA_NSTAGE; ++k) umma_drain_stage(us, k);
  tmem_fence_before();
  __syncthreads();
  tmem_fence_after();
  __syncwarp();
  if (threadIdx.x < 32) tmem_dealloc(us->tmem, ncols);
}

// Thread 0: issue one tile step from stage buffer `stage` (layout above, 512-byte
// aligned) and commit it to bar[st].  trans: the left planes are stored [k][m]
// (MN-major: 32-column blocks one plane apart, 8-row K groups 512 bytes apart; with
// mn_swap the two offsets trade descriptor fields); fresh: the accumulators start a
// new sum (cleared here).
__device__ __forceinline__ void umma_oz_step(UmmaState* us, int st, const __half* stage, bool trans, bool& fresh,
                                             bool mn_swap = false) {
  constexpr unsigned PB = OZ_PLANE * 2;   // bytes per plane
  const unsigned base = smem_u32(stage), rbase = base + UMMA_RIGHT_PLANE * PB;
  const unsigned lbo = trans ? (mn_swap ? 512u : PB) : 512u, sbo = trans ? (mn_swap ? PB : 512u) : 512u;
  tmem_fence_after();
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const unsigned ka = h * 32, kb = trans ? h * 1024 : h * 32;
    umma_f16(us->tmem, umma_sdesc(rbase + ka), umma_sdesc(base + kb, lbo, sbo), umma_idesc(trans, 256),
             (fresh && h == 0) ? 0u : 1u);
  }
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const unsigned ka = h * 32, kb = trans ? h * 1024 : h * 32;
    umma_f16(us->tmem + 128, umma_sdesc(rbase + 4 * PB + ka), umma_sdesc(base + kb, lbo, sbo),
             umma_idesc(trans, 128), 1u);
  }
  fresh = false;
  umma_commit(&us->bar[st]);
  us->pending |= 1u << st;
}

// Output element ownership of the folded accumulator: thread (warp w, lane n) holds
// elements (m, n) with m = 8 r + 2 w + k, e = 2 r + k (r = 0..3, k = 0..1).
__device__ __forceinline__ int umma_row(int e) { return 8 * (e >> 1) + 2 * (threadIdx.x >> 5) + (e & 1); }
__device__ __forceinline__ int umma_col() { return threadIdx.x & 31; }

// All threads: the pair (4, 4) of one tile step, c += X_4 Y_4^T, on mma.sync (warp w:
// the 16 x 16 block at rows (w/2)*16, columns (w%2)*16; mma C layout, see oz_row /
// oz_col).  The left plane is read transposed when trans (stored [k][m]).
__device__ __forceinline__ void oz_pair44(float (&c)[2][4], const __half* stage, bool trans) {
  __syncwarp();   // ldmatrix and mma.sync need the whole warp (a lane may come from single-thread work)
  const __half* As = stage + 4 * OZ_PLANE;
  const __half* Bs = stage + (UMMA_RIGHT_PLANE + 4) * OZ_PLANE;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int m0 = (w >> 1) * 16, n0 = (w & 1) * 16;
  const int ar = m0 + (lane & 7) + ((lane >> 3) & 1) * 8, ac = (lane >> 4) * 8;
  const int tr = (lane >> 4) * 8 + (lane & 7), tc = m0 + ((lane >> 3) & 1) * 8;
  const int br = n0 + (lane & 7) + (lane >> 4) * 8, bc = ((lane >> 3) & 1) * 8;
#pragma unroll
  for (int kk = 0; kk < TS; kk += 16) {
    unsigned a[4], b[4];
    if (trans)
      ldsm_x4_trans(a, As + oz_swz(kk + tr, tc));
    else
      ldsm_x4(a, As + oz_swz(ar, kk + ac));
    ldsm_x4(b, Bs + oz_swz(br, kk + bc));
    mma16816(c[0], a, b[0], b[1]);
    mma16816(c[1], a, b[2], b[3]);
  }
}

// All threads: v[e] -= sum_d P_d(m, n) 2^(esum - 12 - 7 d) for the thread's elements,
// from the accumulator cells and the (4, 4) sums p44 (cleared here).  The caller has
// made the last step's MMAs complete (bar wait by thread 0, then a barrier) and passes
// xch (32 KB) and x44 (4 KB) of shared scratch that no copy is filling.  Warp w reads
// lane block w, where cell (w, i) of element (m, n) holds diagonal w + i.  Round r
// covers the columns m = 8 r .. 8 r + 7: every warp stores its raw cells of those
// columns, and each element's owner adds the cells of each diagonal as integers,
// combines the nine diagonals exactly into two 64-bit words (diagonals 0..3 and 4..8,
// as the mma.sync fold does) and folds them into FP64.  Contains __syncthreads().
__device__ __forceinline__ void umma_fold_sub(const UmmaState* us, int esum, double (&v)[8], float (&p44)[2][4],
                                              float* xch, float* x44) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const unsigned tl = us->tmem + ((unsigned)(32 * w) << 16);
  const double sc = __longlong_as_double((long long)(1023 + esum - 33) << 52);
  __syncwarp();
#pragma unroll
  for (int n = 0; n < 2; ++n)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      x44[oz_row(n, j) * TS + oz_col(n, j)] = p44[n][j];
      p44[n][j] = 0.f;
    }
  tmem_fence_after();
#pragma unroll 1
  for (int r = 0; r < 4; ++r) {
    // columns 32 i + 8 r + e, i = 0..7, into xch[w][i][e][lane]
    unsigned cv[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
      asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                   : "=r"(cv[i][0]), "=r"(cv[i][1]), "=r"(cv[i][2]), "=r"(cv[i][3]), "=r"(cv[i][4]), "=r"(cv[i][5]),
                     "=r"(cv[i][6]), "=r"(cv[i][7])
                   : "r"(tl + 32 * i + 8 * r)
                   : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    if (r == 3) tmem_fence_before();
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int e = 0; e < 8; ++e) xch[((w * 8 + i) * 8 + e) * 32 + lane] = __uint_as_float(cv[i][e]);
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const int e = 2 * w + k;   // column 8 r + e
      int I[OZ_ND];
#pragma unroll
      for (int d = 0; d < OZ_ND; ++d) I[d] = 0;
#pragma unroll
      for (int ww = 0; ww < 4; ++ww)
#pragma unroll
        for (int i = 0; i < 8; ++i)
          if (ww + i < OZ_ND) I[ww + i] += __float2int_rn(xch[((ww * 8 + i) * 8 + e) * 32 + lane]);
      I[8] += __float2int_rn(x44[(8 * r + e) * TS + lane]);
      const long long hi = (((long long)I[0] * 128 + I[1]) * 128 + I[2]) * 128 + I[3];
      const long long lo = ((((long long)I[4] * 128 + I[5]) * 128 + I[6]) * 128 + I[7]) * 128 + I[8];
      const double vv = fma((double)lo, 0x1p-35, (double)hi);
      double& acc = r == 0 ? v[k] : (r == 1 ? v[2 + k] : (r == 2 ? v[4 + k] : v[6 + k]));
      acc = fma(-vv, sc, acc);
    }
    if (r == 3) fence_async_smem();   // xch, x44 lie in stage buffers that bulk copies refill
    __syncthreads();
  }
}

// Dynamic shared memory rounded up to the 512-byte boundary of the swizzled operands
// (the launch adds 512 bytes).
__device__ __forceinline__ unsigned char* smem_align512(unsigned char* p) {
  return p + ((512u - (smem_u32(p) & 511u)) & 511u);
}

}  // namespace gbta
