// FP64 tile products on the tensor cores (Ozaki scheme with exact integer slices).
//
// GB300 executes FP64 FMAs at 1.2 TFLOP/s but fp16 mma.sync (f32 accumulate) at ~600
// TFLOP/s.  A product acc -= X Y^T of FP64 tiles is therefore computed as follows
// (Ozaki, Ogita, Oishi, Rump, "Error-free transformations of matrix multiplication
// by using fast routines of matrix multiplication and its applications", Numer.
// Algorithms 59 (2012); integer-slice variant as in Ootomo, Ozaki, Yokota, "DGEMM on
// integer matrix multiplication unit", IJHPCA 2024):
//
//  * every element x of row g is written in fixed point relative to a per-row
//    exponent E_g with |x| < 2^E_g: N = round(x 2^(55 - E_g)) (|N| <= 2^55, error
//    <= 2^(E_g - 56)) in balanced base 128, x ~ sum_{s=0..7} d_s 2^(E_g - 6 - 7 s)
//    with d_1..d_7 in [-64, 63] and d_0 in [-64, 64].  The digits are exact in fp16
//    and are stored once per tile, as 8 "digit planes";
//  * sum_k x_ik y_jk = sum_{s,t} 2^(E_i + E_j - 12 - 7(s+t)) sum_k d_s,ik g_t,jk.  Each
//    inner sum is an integer matrix product computed by mma.sync; the 43 pairs with
//    s + t <= 8 are kept (the dropped ones weigh below 2^(E_i+E_j-55) in total for a
//    32-term tile product, under FP64 rounding of the result) and pairs of equal
//    s + t share one fp32 accumulator;
//  * every partial sum is an integer of magnitude below 8 * 64^2 * 32 * OZ_CHUNK < 2^24,
//    so the fp32 accumulation is exact; every OZ_CHUNK tile steps the nine diagonals
//    are combined exactly in 64-bit integers and folded into the FP64 accumulator.
//
// Balanced digits (rather than magnitude digits with the sign applied) carry 7 bits
// each at the same product magnitude (|d| <= 64), so 8 planes and 43 pairs give what
// 9 planes and 53 pairs of 6-bit magnitude digits gave, with a smaller error.
//
// For the Cholesky factor the per-row exponents come from the matrix itself: a row of
// L satisfies sum_j L_gj^2 = Q_gg, so E_g = ilogb(sqrt(Q_gg)) + 2 bounds every element
// of row g in every tile, and the same digits serve as left and right operand.
#pragma once

#include <cuda_fp16.h>

#include "bta_common.cuh"

namespace gbta {

constexpr int OZ_S = 8;                       // digit planes per tile
constexpr int OZ_W = 7;                       // bits per digit
constexpr int OZ_ND = 9;                      // diagonals s + t = 0 .. 8
constexpr int OZ_CHUNK = 15;                  // tile steps per exact fp32 accumulation
constexpr int OZ_ZERO = 64;                   // biased field of the digit 0 (field = d + 64)
constexpr int OZ_PLANE = TS * TS;            // halves per plane (global and shared memory alike)
constexpr int OZ_OPER = OZ_S * OZ_PLANE;      // halves per operand tile in shared memory
constexpr int OZ_TILE = OZ_S * TS * TS;       // halves per tile in the global digit buffer
constexpr int OZ_CHUNKS16 = OZ_S * TS * 4;    // 16-byte pieces per tile (8 * 32 rows * 64 B)

// Half index of element (row, col) of a digit plane.  Planes are stored as 32 rows of
// 64 bytes in global and shared memory alike (a tile's planes are one contiguous 16 KB
// block, copied as is); the four 16-byte chunks of row r are permuted by (r >> 1) & 3,
// so that the eight rows one ldmatrix reads land in distinct shared-memory banks.
__host__ __device__ constexpr int oz_swz(int row, int col) {
  return row * TS + ((((col >> 3) ^ (row >> 1)) & 3) << 3) + (col & 7);
}

// At most 8 pairs share a diagonal; |d| <= 64.
static_assert(8 * 64 * 64 * TS * OZ_CHUNK < (1 << 24), "fp32 accumulation must stay exact");

// Row exponent: E = ilogb(sqrt(q)) + 2 (q > 0), so |x| <= sqrt(q) < 2^(E-1).
__device__ __forceinline__ int oz_row_exponent(double q) {
  if (!(q > 0.0) || !isfinite(q)) return 0;
  return ilogb(sqrt(q)) + 2;
}

// The fixed-point value N = round(x 2^(55 - E)) (ties away from zero, |N| <= 2^55) of
// x relative to 2^E, from the bits of x with integer instructions only and no branch
// (lanes whose values sit in different binades take the same path): the 53-bit
// significand m is shifted left by sh in [0, 2] or right, with rounding, by -sh; sh > 2
// saturates (only reachable for x beyond the bound 2^(E-1)); zero, infinities and NaN
// give 0.
__device__ __forceinline__ long long oz_fixed(double x, int E) {
  const long long bits = __double_as_longlong(x);
  const int ex = (int)((bits >> 52) & 0x7ff);
  const unsigned long long mag = (unsigned long long)bits & 0x7fffffffffffffffull;
  const unsigned long long m = (bits & 0xfffffffffffffull) | (ex ? (1ull << 52) : 0ull);
  const int sh = (ex ? ex : 1) - 1075 + 55 - E;   // |x| 2^(55 - E) = m 2^sh
  const int ls = sh > 0 ? (sh < 2 ? sh : 2) : 0;
  const int rs = sh >= 0 ? 0 : (sh > -63 ? -sh : 63);   // (a shift of 54 or more gives 0)
  const unsigned long long half = rs > 0 ? (1ull << (rs - 1)) : 0ull;
  unsigned long long F = ((m << ls) + half) >> rs;
  F = sh > 2 ? (1ull << 55) : F;
  F = F > (1ull << 55) ? (1ull << 55) : F;
  F = (ex == 0x7ff || mag == 0) ? 0ull : F;
  const long long sg = bits >> 63;   // 0 or -1
  return ((long long)F ^ sg) - sg;
}

// The eight digit planes of two elements (fixed-point values N0, N1) as fp16 pairs, one
// 32-bit word per plane (N0's digit in the low half).  The balanced base-128 digits are
// the 7-bit fields of P = N + sum_s 64 * 128^s (non-negative, so no carries: each field
// is d_s + 64; the top field d_0 + 64 is in [0, 128]).  P is split into two 28-bit
// words holding planes 0-3 and 4-7, so that each plane of both elements comes from
// 32-bit shifts and masks; the fp16 bit pattern 0x6400 + f is the integer 1024 + f, so
// one half2 subtraction of 1088 turns both fields into their digits exactly.  Returns
// the number of leading planes in which both digits are zero.
__device__ __forceinline__ int oz_pair_planes(long long N0, long long N1, unsigned (&w)[OZ_S]) {
  constexpr unsigned long long BIAS = 0x0081020408102040ull;   // sum_{s=0..7} 64 * 128^s
  const unsigned long long P0 = (unsigned long long)N0 + BIAS, P1 = (unsigned long long)N1 + BIAS;
  const unsigned h0 = (unsigned)(P0 >> 28), l0 = (unsigned)P0 & 0xfffffffu;
  const unsigned h1 = (unsigned)(P1 >> 28), l1 = (unsigned)P1 & 0xfffffffu;
  const __half h1088 = __ushort_as_half((unsigned short)0x6440);
  const __half2 off = __halves2half2(h1088, h1088);
  int lz = 0;
#pragma unroll
  for (int s = 0; s < OZ_S; ++s) {
    const unsigned a = s < 4 ? h0 : l0, b = s < 4 ? h1 : l1;
    const int k = OZ_W * (3 - (s & 3));   // 21, 14, 7, 0 within the 28-bit word
    const unsigned mk = s == 0 ? 0xffu : 0x7fu;
    const unsigned lo = (a >> k) & mk;
    const unsigned hi = (k <= 16 ? (b << (16 - k)) : (b >> (k - 16))) & (mk << 16);
    const unsigned f = lo | hi | 0x64006400u;
    if (lz == s && f == 0x64406440u) lz = s + 1;   // both fields 64: both digits 0
    const __half2 hv = __hsub2(*reinterpret_cast<const __half2*>(&f), off);
    w[s] = *reinterpret_cast<const unsigned*>(&hv);
  }
  return lz;
}

// Minimum of v over the CTA (every thread gets it); red: NT / 32 ints of shared memory.
// Contains barriers.
__device__ __forceinline__ int cta_min_int(int v, int* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  int m = red[0];
#pragma unroll
  for (int w = 1; w < NT / 32; ++w) m = min(m, red[w]);
  __syncthreads();
  return m;
}

// Two tiles whose digit planes below z_A, z_B are zero (z = OZ_S: the tile is zero)
// multiply only through the pairs (s, t) with z_A <= s < OZ_S, z_B <= t < OZ_S and
// s + t <= OZ_ND - 1: there are none when this returns true, and the step is skipped.
__device__ __forceinline__ bool oz_pairs_vanish(int za, int zb) {
  return za >= OZ_S || zb >= OZ_S || za + zb > OZ_ND - 1;
}


// Write the digit planes of the valid part of a shared FP64 tile X (rows x cols)
// to dst ([plane][row][col] halves), row r relative to 2^Eof(r).  Each thread converts
// pairs of adjacent columns and stores them as one 32-bit word; the rest is zero.
template <class EOf>
__device__ __forceinline__ void oz_store_digits_e(__half* dst, const double* X, int rows, int cols, EOf Eof) {
#pragma unroll
  for (int q = 0; q < PER_THREAD / 2; ++q) {
    const int p = threadIdx.x + q * NT;
    const int r = p / (TS / 2), c = 2 * (p % (TS / 2));
    const long long n0 = (r < rows && c < cols) ? oz_fixed(X[r * LDS + c], Eof(r)) : 0ll;
    const long long n1 = (r < rows && c + 1 < cols) ? oz_fixed(X[r * LDS + c + 1], Eof(r)) : 0ll;
    unsigned wv[OZ_S];
    oz_pair_planes(n0, n1, wv);
    unsigned* w = reinterpret_cast<unsigned*>(dst + oz_swz(r, c));
#pragma unroll
    for (int s = 0; s < OZ_S; ++s) w[s * (OZ_PLANE / 2)] = wv[s];
  }
}

// Digit planes of rows row0 .. row0 + FEED_ROWS - 1 of a shared tile (valid part rows x
// cols, row r relative to 2^E[r]); one column pair per thread.
__device__ __forceinline__ void oz_store_digits_rows(__half* dst, const double* X, int row0, int rows, int cols,
                                                     const int* E) {
  static_assert(FEED_ROWS * TS / 2 == NT, "one column pair of the row group per thread");
  const int r = row0 + threadIdx.x / (TS / 2), c = 2 * (threadIdx.x % (TS / 2));
  const long long n0 = (r < rows && c < cols) ? oz_fixed(X[r * LDS + c], E[r]) : 0ll;
  const long long n1 = (r < rows && c + 1 < cols) ? oz_fixed(X[r * LDS + c + 1], E[r]) : 0ll;
  unsigned wv[OZ_S];
  oz_pair_planes(n0, n1, wv);
  unsigned* w = reinterpret_cast<unsigned*>(dst + oz_swz(r, c));
#pragma unroll
  for (int s = 0; s < OZ_S; ++s) w[s * (OZ_PLANE / 2)] = wv[s];
}

// Rows relative to per-row exponents E[row].
__device__ __forceinline__ void oz_store_digits(__half* dst, const double* X, int rows, int cols, const int* E) {
  oz_store_digits_e(dst, X, rows, cols, [E](int r) { return E[r]; });
}
// All rows relative to one exponent E.
__device__ __forceinline__ void oz_store_digits_uniform(__half* dst, const double* X, int rows, int cols, int E) {
  oz_store_digits_e(dst, X, rows, cols, [E](int) { return E; });
}

// ilogb of a finite nonzero double given by its magnitude bits (integer instructions
// only; subnormals through the leading-zero count).
__device__ __forceinline__ int ilogb_bits(unsigned long long a) {
  const int e = (int)(a >> 52);
  return e ? e - 1023 : -1011 - __clzll((long long)a);
}

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void cp_async16(void* sdst, const void* gsrc) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(sdst)), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async4(void* sdst, const void* gsrc) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(sdst)), "l"(gsrc) : "memory");
}
// Order this thread's generic shared-memory writes before later bulk (async-proxy)
// copies into the same bytes.
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Stage one tile's digit planes (global, compact rows) into shared memory (padded rows).
__device__ __forceinline__ void oz_load_async(__half* sdst, const __half* gsrc) {
  for (int q = threadIdx.x; q < OZ_CHUNKS16; q += NT) cp_async16(sdst + q * 8, gsrc + q * 8);
}

// ---- bulk staging of digit planes -------------------------------------------------
// A product loop stages each step's operands (one contiguous 16 KB block per tile, or
// its leading planes) with cp.async.bulk copies issued by one thread; the copies
// signal one mbarrier per stage buffer.  OzPipe is the per-CTA state: the two
// barriers and the parity of the next completion of each (kept across tasks).
struct OzPipe {
  unsigned long long bar[2];
  unsigned phase;   // bit st: parity of the next completion of stage st
};

__device__ __forceinline__ void oz_pipe_init(OzPipe* pp) {
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&pp->bar[0])) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&pp->bar[1])) : "memory");
    pp->phase = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
}

// Thread 0: expect `bytes` on stage st's barrier (one arrival), then the copies.
__device__ __forceinline__ void oz_bulk_expect(OzPipe* pp, int st, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&pp->bar[st])), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void oz_bulk_copy(OzPipe* pp, int st, __half* sdst, const __half* gsrc, unsigned bytes) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(sdst)),
               "l"(gsrc), "r"(bytes), "r"(smem_u32(&pp->bar[st]))
               : "memory");
}

// Every thread: wait (bounded) for stage st's next completion; flips the parity bit
// in `ph`.  False if the limit ran out (the copies of a healthy GPU take microseconds).
__device__ __forceinline__ bool oz_stage_wait(OzPipe* pp, int st, unsigned& ph) {
  const unsigned parity = (ph >> st) & 1u;
  for (int it = 0; it < (1 << 22); ++it) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smem_u32(&pp->bar[st])), "r"(parity)
        : "memory");
    if (done) {
      ph ^= 1u << st;
      return true;
    }
  }
  return false;
}

// Stage a tile's digit planes shifted down by q planes: shared plane s holds global
// plane s - q (zero for s < q; global planes past the last are dropped).  Reading a
// tile sliced against 2^E_t in the frame of a larger exponent E = E_t + 7q.
__device__ __forceinline__ void oz_load_async_shift(__half* sdst, const __half* gsrc, int q) {
  for (int idx = threadIdx.x; idx < OZ_CHUNKS16; idx += NT) {
    const int s = idx / (TS * 4);
    __half* d = sdst + idx * 8;
    if (s < q)
      *reinterpret_cast<uint4*>(d) = make_uint4(0u, 0u, 0u, 0u);
    else
      cp_async16(d, gsrc + idx * 8 - q * OZ_PLANE);
  }
}

__device__ __forceinline__ void ldsm_x4(unsigned (&r)[4], const __half* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x4_trans(unsigned (&r)[4], const __half* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}
__device__ __forceinline__ void mma16816(float (&c)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Per-thread state of an Ozaki K-loop: warp w owns the 16 x 16 output block at rows
// (w/2)*16, cols (w%2)*16; each thread holds 2 n8-tiles x 4 elements (mma C layout).
struct OzAcc {
  float p[OZ_ND][2][4];   // exact integer partial sums per diagonal
  double v[2][4];         // FP64 accumulator (same layout)
};

__device__ __forceinline__ int oz_row(int nt_, int j) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  return (w >> 1) * 16 + (lane >> 2) + (j >> 1) * 8;
}
__device__ __forceinline__ int oz_col(int nt_, int j) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  return (w & 1) * 16 + nt_ * 8 + 2 * (lane & 3) + (j & 1);
}

__device__ __forceinline__ void oz_clear_partials(OzAcc& a) {
#pragma unroll
  for (int d = 0; d < OZ_ND; ++d)
#pragma unroll
    for (int n = 0; n < 2; ++n)
#pragma unroll
      for (int j = 0; j < 4; ++j) a.p[d][n][j] = 0.f;
}

// One tile step: p[s+t] += d_s(A) * d_t(B)^T for the 43 pairs s + t <= 8, or only for
// s >= SA, t >= SB when the A planes below SA and the B planes below SB are known to be
// zero (a left tile staged SA or more planes down, a right tile whose leading digits
// vanish): neither their loads nor their products are issued (the products left out
// are exact zeros, so the result is the full step's).  The A planes hold A(m, k) at
// [m][k], or, with TA, at [k][m] (read with ldmatrix.trans).
template <bool TA, int SA = 0, int SB = 0>
__device__ __forceinline__ void oz_step_t(OzAcc& acc, const __half* As, const __half* Bs) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int m0 = (w >> 1) * 16, n0 = (w & 1) * 16;
  const int ar = m0 + (lane & 7) + ((lane >> 3) & 1) * 8, ac = (lane >> 4) * 8;
  // transposed A: lane supplies row k = (lane >> 4) * 8 + (lane & 7) at column m
  const int tr = (lane >> 4) * 8 + (lane & 7), tc = m0 + ((lane >> 3) & 1) * 8;
  const int br = n0 + (lane & 7) + (lane >> 4) * 8, bc = ((lane >> 3) & 1) * 8;
#pragma unroll
  for (int kk = 0; kk < TS; kk += 16) {
    unsigned a[OZ_S][4], b[OZ_S][4];
    if (TA) {
#pragma unroll
      for (int s = SA; s < OZ_S; ++s)
        if (s + SB <= OZ_ND - 1) ldsm_x4_trans(a[s], As + s * OZ_PLANE + oz_swz(kk + tr, tc));
    } else {
#pragma unroll
      for (int s = SA; s < OZ_S; ++s)
        if (s + SB <= OZ_ND - 1) ldsm_x4(a[s], As + s * OZ_PLANE + oz_swz(ar, kk + ac));
    }
#pragma unroll
    for (int t = SB; t < OZ_S; ++t)
      if (t + SA <= OZ_ND - 1) ldsm_x4(b[t], Bs + t * OZ_PLANE + oz_swz(br, kk + bc));
#pragma unroll
    for (int s = SA; s < OZ_S; ++s)
#pragma unroll
      for (int t = SB; t + s < OZ_ND && t < OZ_S; ++t) {
        mma16816(acc.p[s + t][0], a[s], b[t][0], b[t][1]);
        mma16816(acc.p[s + t][1], a[s], b[t][2], b[t][3]);
      }
  }
}

__device__ __forceinline__ void oz_step(OzAcc& acc, const __half* As, const __half* Bs) {
  oz_step_t<false>(acc, As, Bs);
}

// Plane pairs (s, t) that oz_step_t<TA, SA, SB> multiplies.
__host__ __device__ constexpr int oz_pairs_from(int SA, int SB) {
  int n = 0;
  for (int s = SA; s < OZ_S; ++s)
    for (int t = SB; t < OZ_S && s + t < OZ_ND; ++t) ++n;
  return n;
}
static_assert(oz_pairs_from(0, 0) == 43, "the 43 pairs s + t <= 8");
// Leading zero planes that oz_step_z leaves out at most (A, B).
constexpr int OZ_SA_MAX = 2, OZ_SB_MAX = 3;
// ... and the pairs oz_step_z multiplies for runtime counts (0 when oz_pairs_vanish).
__device__ __forceinline__ int oz_pairs_issued(int za, int zb) {
  return oz_pairs_vanish(za, zb) ? 0
                                 : oz_pairs_from(za < OZ_SA_MAX ? za : OZ_SA_MAX, zb < OZ_SB_MAX ? zb : OZ_SB_MAX);
}

// The tile step for runtime counts of zero leading planes za (A) and zb (B): the
// variant that leaves out min(za, OZ_SA_MAX) A planes and min(zb, OZ_SB_MAX) B planes
// (compile-time plane ranges keep the operands in registers); the B planes it does not
// read need not hold anything.  Requires !oz_pairs_vanish(za, zb).
template <bool TA>
__device__ __forceinline__ void oz_step_z(OzAcc& acc, const __half* As, const __half* Bs, int za, int zb) {
  static_assert(OZ_SA_MAX == 2 && OZ_SB_MAX == 3, "the variants below");
  switch ((za < OZ_SA_MAX ? za : OZ_SA_MAX) * 4 + (zb < OZ_SB_MAX ? zb : OZ_SB_MAX)) {
    case 0: oz_step_t<TA, 0, 0>(acc, As, Bs); break;
    case 1: oz_step_t<TA, 0, 1>(acc, As, Bs); break;
    case 2: oz_step_t<TA, 0, 2>(acc, As, Bs); break;
    case 3: oz_step_t<TA, 0, 3>(acc, As, Bs); break;
    case 4: oz_step_t<TA, 1, 0>(acc, As, Bs); break;
    case 5: oz_step_t<TA, 1, 1>(acc, As, Bs); break;
    case 6: oz_step_t<TA, 1, 2>(acc, As, Bs); break;
    case 7: oz_step_t<TA, 1, 3>(acc, As, Bs); break;
    case 8: oz_step_t<TA, 2, 0>(acc, As, Bs); break;
    case 9: oz_step_t<TA, 2, 1>(acc, As, Bs); break;
    case 10: oz_step_t<TA, 2, 2>(acc, As, Bs); break;
    default: oz_step_t<TA, 2, 3>(acc, As, Bs); break;
  }
}

// Fold the exact partial sums into the FP64 accumulator:
// v -= sum_D p_D 2^(Ei+Ej-12-7D) (D = 0..8).
// `esum[n][j]` = E_i + E_j of the thread's elements.  Clears the partials.
__device__ __forceinline__ void oz_fold_sub(OzAcc& acc, const int (&esum)[2][4]) {
#pragma unroll
  for (int n = 0; n < 2; ++n)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int I[OZ_ND];
#pragma unroll
      for (int d = 0; d < OZ_ND; ++d) {
        I[d] = __float2int_rn(acc.p[d][n][j]);
        acc.p[d][n][j] = 0.f;
      }
      // diagonals 0..3 and 4..8 in two exact 64-bit integers (|I| < 2^24, so the high
      // word stays below 2^46 and the low one below 2^53: both convert exactly), then
      // two conversions and one FMA; diagonal 3 has weight 2^(Ei+Ej-33)
      const long long hi = (((long long)I[0] * 128 + I[1]) * 128 + I[2]) * 128 + I[3];
      const long long lo = ((((long long)I[4] * 128 + I[5]) * 128 + I[6]) * 128 + I[7]) * 128 + I[8];
      const double vv = fma((double)lo, 0x1p-35, (double)hi);
      const double sc = __longlong_as_double((long long)(1023 + esum[n][j] - 33) << 52);
      acc.v[n][j] = fma(-vv, sc, acc.v[n][j]);
    }
}

// The same fold for partial sums of at most OZ_SHORT tile steps since the last fold.
// Diagonal d then holds at most pairs(d) <= 8 products of digits of magnitude <= 64
// over 32 terms per step, |I_d| <= pairs(d) 2^17 OZ_SHORT, so both words stay below 2^51
// (bound below) and convert exactly by adding them to the bits of 1.5 * 2^52; the two
// conversions become one subtraction folded into the combining FMA:
// fma(L, 2^-35, H - (1.5 * 2^52 + 1.5 * 2^17)) with L = 1.5 * 2^52 + lo and
// H = 1.5 * 2^52 + hi is hi + lo 2^-35 with the one rounding of the fold above
// (H - ... is exact: both operands lie within a factor of two of each other), so the
// result is the same in every bit, for three FP64-pipe instructions per element
// instead of four.
constexpr int OZ_SHORT = 12;
static_assert((double)(1 << 17) * OZ_SHORT * (5.0 * (1 << 28) + 6.0 * (1 << 21) + 7.0 * (1 << 14) + 8.0 * 128 + 7.0) <
                  2251799813685248.0,
              "the low word of a short fold stays below 2^51");
__device__ __forceinline__ void oz_fold_sub_short(OzAcc& acc, const int (&esum)[2][4]) {
#pragma unroll
  for (int n = 0; n < 2; ++n)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int I[OZ_ND];
#pragma unroll
      for (int d = 0; d < OZ_ND; ++d) {
        I[d] = __float2int_rn(acc.p[d][n][j]);
        acc.p[d][n][j] = 0.f;
      }
      const long long hi = (((long long)I[0] * 128 + I[1]) * 128 + I[2]) * 128 + I[3];
      const long long lo = ((((long long)I[4] * 128 + I[5]) * 128 + I[6]) * 128 + I[7]) * 128 + I[8];
      const double L = __longlong_as_double(lo + 0x4338000000000000ll);
      const double H = __longlong_as_double(hi + 0x4338000000000000ll);
      const double vv = fma(L, 0x1p-35, H - (0x1.8p52 + 0x1.8p17));
      const double sc = __longlong_as_double((long long)(1023 + esum[n][j] - 33) << 52);
      acc.v[n][j] = fma(-vv, sc, acc.v[n][j]);
    }
}

// The fold of partial sums of `steps` tile steps (uniform over the CTA).
__device__ __forceinline__ void oz_fold_sub_steps(OzAcc& acc, const int (&esum)[2][4], int steps) {
  if (steps <= OZ_SHORT)
    oz_fold_sub_short(acc, esum);
  else
    oz_fold_sub(acc, esum);
}

}  // namespace gbta
