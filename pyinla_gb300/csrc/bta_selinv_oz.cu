// Single-instance BTA selected-inversion kernel with tensor-core (Ozaki digit-plane)
// products (the task body is selinv_oz_task in bta_selinv_task.cuh), and the two
// pre-passes over the factor that prepare its right operands.
#include "../../include/pyinla_gb300.h"
#include "bta_selinv_task.cuh"

namespace gbta {

// ---- pre-passes over the factor ---------------------------------------------------
// One CTA per (block i, column tile c): ecol[i*b + c*TS + j] = exponent of
// max |F(m, j)| over the rows m of the column's pattern (D_i below tile c, block i's
// coupling slot, R_i).
__global__ void __launch_bounds__(NT) k_fac_col_exponents(const double* D, const double* L, const double* R, Geom g,
                                                          int use_arrow, int* ecol) {
  // the maximum magnitude as the integer maximum of the magnitude bits (the order of
  // non-negative doubles; no FP64 instruction), NaN and infinity giving exponent 0
  __shared__ unsigned long long red[NT];
  const int ic = blockIdx.x;
  const int i = ic / g.B, c = ic % g.B;
  const size_t bb = (size_t)g.b * g.b, ab = (size_t)g.a * g.b;
  const int j = threadIdx.x % TS, r0 = threadIdx.x / TS;   // 4 row groups
  const int col = c * TS + j;
  auto mag = [](double x) {
    return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
  };
  unsigned long long m = 0;
  if (col < g.b) {
    for (int row = (c + 1) * TS + r0; row < g.b; row += NT / TS) m = max(m, mag(D[i * bb + (size_t)row * g.b + col]));
    if (g.nxt(i) >= 0) {
      const size_t ls = (size_t)g.lslot(i);
      for (int row = r0; row < g.b; row += NT / TS) m = max(m, mag(L[ls * bb + (size_t)row * g.b + col]));
    }
    if (use_arrow)
      for (int row = r0; row < g.a; row += NT / TS) m = max(m, mag(R[i * ab + (size_t)row * g.b + col]));
  }
  red[threadIdx.x] = m;
  __syncthreads();
  if (threadIdx.x < TS) {
    const unsigned long long mm =
        max(max(red[threadIdx.x], red[threadIdx.x + TS]), max(red[threadIdx.x + 2 * TS], red[threadIdx.x + 3 * TS]));
    const bool finite = mm < 0x7ff0000000000000ull;
    if (col < g.b) ecol[(size_t)i * g.b + col] = (mm != 0 && finite) ? ilogb_bits(mm) + 1 : 0;
  }
}

// One CTA per flag slot that is a factor tile of some column pattern: digits relative
// to the column exponents, stored transposed: dst[s][j][m] = digit s of F[m][j]; and
// dz[slot] = the number of leading digit planes that are zero over the whole tile (8:
// the tile is zero -- the coupling blocks of banded couplings have many), which lets
// the inversion leave out the products those planes would contribute.
__global__ void __launch_bounds__(NT) k_fac_digits_t(const double* D, const double* L, const double* R, Geom g,
                                                     int use_arrow, const int* ecol, __half* dig, int* dz) {
  __shared__ int red[NT / 32];
  __shared__ __align__(16) __half planes[OZ_TILE];   // the tile's planes, written out in 16-byte pieces
  const int slot = blockIdx.x;
  const int B = g.B;
  const size_t bb = (size_t)g.b * g.b, ab = (size_t)g.a * g.b;
  int i, r, c;
  Tile t;
  if (slot < g.nt * B * B) {
    i = slot / (B * B);
    r = (slot / B) % B;
    c = slot % B;
    if (r <= c) return;
    t = make_tile(D + i * bb, g.b, r * TS, c * TS, g.b, g.b);
  } else if (slot < (2 * g.nt - 1) * B * B) {
    const int s2 = slot - g.nt * B * B;
    const int j = s2 / (B * B);   // L slot j: columns of block lcol(j)
    r = (s2 / B) % B;
    c = s2 % B;
    i = g.lcol(j);
    t = make_tile(L + j * bb, g.b, r * TS, c * TS, g.b, g.b);
  } else if (slot < (2 * g.nt - 1) * B * B + g.nt * B) {
    if (!use_arrow) return;
    const int s3 = slot - (2 * g.nt - 1) * B * B;
    i = s3 / B;
    c = s3 % B;
    t = make_tile(R + i * ab, g.b, 0, c * TS, g.a, g.b);
  } else {
    return;
  }
  __half* dst = dig + (size_t)slot * OZ_TILE;
  int lz = OZ_S;
  // pairs of rows (m, m+1) of one column jj: adjacent in the transposed layout
  double x0[PER_THREAD / 2], x1[PER_THREAD / 2];
  bool nz = false;
#pragma unroll
  for (int q = 0; q < PER_THREAD / 2; ++q) {
    const int p = threadIdx.x + q * NT;
    const int jj = p % TS, m = 2 * (p / TS);
    x0[q] = (m < t.rows && jj < t.cols) ? t.p[(size_t)m * t.ld + jj] : 0.0;
    x1[q] = (m + 1 < t.rows && jj < t.cols) ? t.p[(size_t)(m + 1) * t.ld + jj] : 0.0;
    nz |= x0[q] != 0.0 || x1[q] != 0.0;
  }
  // a zero tile: the inversion drops the products of a tile whose count is OZ_S and
  // never reads its planes, so only the count is written
  if (dz && !__syncthreads_or(nz)) {
    if (threadIdx.x == 0) dz[slot] = OZ_S;
    return;
  }
#pragma unroll
  for (int q = 0; q < PER_THREAD / 2; ++q) {
    const int p = threadIdx.x + q * NT;
    const int jj = p % TS, m = 2 * (p / TS);
    const int e = (jj < t.cols) ? ecol[(size_t)i * g.b + c * TS + jj] : 0;
    const long long n0 = (m < t.rows && jj < t.cols) ? oz_fixed(x0[q], e) : 0ll;
    const long long n1 = (m + 1 < t.rows && jj < t.cols) ? oz_fixed(x1[q], e) : 0ll;
    unsigned wv[OZ_S];
    lz = min(lz, oz_pair_planes(n0, n1, wv));
    unsigned* w = reinterpret_cast<unsigned*>(planes + oz_swz(jj, m));
#pragma unroll
    for (int s = 0; s < OZ_S; ++s) w[s * (OZ_PLANE / 2)] = wv[s];
  }
  lz = cta_min_int(lz, red);   // (contains the barriers that complete the planes)
  // with the counts, the inversion reads no plane below min(lz, OZ_SB_MAX) (oz_step_z)
  const int first = dz ? min(lz, OZ_SB_MAX) : 0;
  for (int k = first * (OZ_PLANE / 8) + threadIdx.x; k < OZ_CHUNKS16; k += NT)
    reinterpret_cast<uint4*>(dst)[k] = reinterpret_cast<const uint4*>(planes)[k];
  if (dz && threadIdx.x == 0) dz[slot] = lz;
}

// Column exponents and transposed digit planes of the factor (before a selected
// inversion with tensor-core products).
void launch_selinv_oz_prepare(const Geom& g, const double* D, const double* L, const double* R, int use_arrow,
                              __half* fdig, int* ecol, int* fdz, cudaStream_t stream) {
  static bool attr_set = false;   // the largest shared-memory carveout (see launch_solve)
  if (!attr_set) {
    cudaFuncSetAttribute(k_fac_col_exponents, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    cudaFuncSetAttribute(k_fac_digits_t, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    attr_set = true;
  }
  k_fac_col_exponents<<<g.nt * g.B, NT, 0, stream>>>(D, L, R, g, use_arrow, ecol);
  k_fac_digits_t<<<g.nflags(), NT, 0, stream>>>(D, L, R, g, use_arrow, ecol, fdig, fdz);
  count_launches(2);
}

__global__ void __launch_bounds__(NT, OZS_CTAS_PER_SM) k_selinv_oz(SelinvArgs p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_ok, s_t, s_ready;
  __shared__ OzPipe pipe;
  oz_pipe_init(&pipe);
  while (true) {
    const int t = cta_ticket(p.c, &s_t);
    if (t < 0 || t >= p.ntasks) break;
    if (!selinv_oz_task(p, t, smem_raw, &s_ok, &s_ready, &pipe)) break;
  }
}

size_t selinv_oz_digit_bytes(const Geom& g) { return (size_t)g.nflags() * OZ_TILE * sizeof(__half); }

void launch_selinv_oz(const Geom& g, const double* D, const double* L, const double* R, const double* T, double* SD,
                      double* SL, double* SR, double* ST, int use_arrow, const int4* tasks, int ntasks, __half* fdig,
                      int* ecol, const double* cinv, __half* sdig, double* part, int* part_flag,
                      const LaunchCtl& lc, int* fdz) {
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(k_selinv_oz, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)OZS_SMEM);
    // the largest shared-memory carveout, so that two CTAs fit on an SM
    cudaFuncSetAttribute(k_selinv_oz, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    attr_set = true;
  }
  launch_selinv_oz_prepare(g, D, L, R, use_arrow, fdig, ecol, fdz, lc.stream);
  SelinvArgs p;
  p.D = D;
  p.L = L;
  p.R = R;
  p.T = T;
  p.SD = SD;
  p.SL = SL;
  p.SR = SR;
  p.ST = ST;
  p.g = g;
  p.use_arrow = use_arrow;
  p.method = GBTA_METHOD_OZAKI;
  p.tasks = tasks;
  p.ntasks = ntasks;
  p.fdig = fdig;
  p.fdz = fdz;
  p.ecol = ecol;
  p.cinv = cinv;
  p.sdig = sdig;
  p.part = part;
  p.part_flag = part_flag;
  p.merged = 1;
  p.c.ctrl = lc.ctrl;
  p.c.flags = lc.flags;
  p.c.epoch = lc.epoch;
  p.c.wait_ns = lc.wait_ns;
  p.c.trace = lc.trace;
  k_selinv_oz<<<launch_grid((const void*)k_selinv_oz, NT, OZS_SMEM, lc), NT, OZS_SMEM, lc.stream>>>(p);
  count_launches(1);
}

}  // namespace gbta
