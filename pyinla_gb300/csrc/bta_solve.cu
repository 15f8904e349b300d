// BTA triangular sweeps (Serinv pobtas / pobts) as one persistent dataflow kernel.
//
// Replaces the block forward / backward substitutions the reference runs through
// Serinv (src/pyinla/solvers/structured_solver.py:112-140): trans = 0 solves
// L y = b, trans = 1 solves L^T x = y, in place on the right-hand side.  One task
// produces one TS-row tile of the solution: it subtracts the tile-vector products
// of the solution tiles it depends on (waiting on their flags), then solves with
// its diagonal factor tile (warp-level substitution).  The forward sweep also
// leaves the arrow contribution R_i(:,r) y(i,r) of each tile in a partial buffer
// that the arrow task sums in a fixed order.
#include "bta_common.cuh"

namespace gbta {

constexpr int NC = SOLVE_NC;   // right-hand-side columns per launch (thread t: row t/NC, column t%NC)
static_assert(TS * NC == NT, "one solution element per thread");

struct SolveArgs {
  const double* D;
  const double* L;
  const double* R;
  const double* T;
  double* B;        // right-hand sides (row-major, row stride ldb), columns [0, nc)
  int ldb;
  int nc;
  Geom g;
  int use_arrow;
  int trans;
  double* part;     // [nt*B][TS*NC] arrow partials
  Ctl c;
};

__device__ __forceinline__ int vflag(const Geom& g, int i, int r) { return i * g.B + r; }

// s(TS x NC, one element per thread) -= M * v, M staged in shared memory (Ms), v in Vs.
__device__ __forceinline__ double tile_gemv(double s, const double* Ms, const double* Vs) {
  const int row = threadIdx.x / NC, col = threadIdx.x % NC;
#pragma unroll 8
  for (int m = 0; m < TS; ++m) s = fma(-Ms[row * LDS + m], Vs[m * NC + col], s);
  return s;
}

// Load the solution tile starting at global row `row0` (rows valid) into Vs.
__device__ __forceinline__ void vec_load(double* Vs, const SolveArgs& p, int row0, int rows) {
  const int row = threadIdx.x / NC, col = threadIdx.x % NC;
  Vs[row * NC + col] = (row < rows && col < p.nc) ? __ldcg(p.B + (size_t)(row0 + row) * p.ldb + col) : 0.0;
}

// Substitution of the NC columns of Ss (TS x NC, row-major) with the TS x TS lower
// factor tile F (identity padded): forward (L y = s) or backward (L^T x = s).  Warp q
// handles column q; rd = 1/diag(F), so each step is one multiply and one FMA.
__device__ void warp_trsv(double* Ss, const double* F, const double* rd, bool upper, int ncols) {
  const int q = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (q >= ncols) return;
  double s = Ss[lane * NC + q];
  if (!upper) {
    for (int j = 0; j < TS; ++j) {
      const double yj = __shfl_sync(0xffffffffu, s, j) * rd[j];
      if (lane == j) s = yj;
      else if (lane > j) s = fma(-F[lane * LDS + j], yj, s);
    }
  } else {
    for (int j = TS - 1; j >= 0; --j) {
      const double xj = __shfl_sync(0xffffffffu, s, j) * rd[j];
      if (lane == j) s = xj;
      else if (lane < j) s = fma(-F[j * LDS + lane], xj, s);
    }
  }
  Ss[lane * NC + q] = s;
}

__global__ void __launch_bounds__(NT, 1) k_solve(SolveArgs p) {
  __shared__ double Ms[TILE_SMEM];
  __shared__ double Fs[TILE_SMEM];
  __shared__ double Vs[TS * NC];
  __shared__ double Ss[TS * NC];
  __shared__ double rd[TS];
  __shared__ int s_ok, s_t;
  const Geom& g = p.g;
  const Ctl& c = p.c;
  const int row = threadIdx.x / NC, col = threadIdx.x % NC;
  const int ntile = g.nt * g.B;
  const int ntasks = ntile + (p.use_arrow ? 1 : 0);
  const size_t bb = (size_t)g.b * g.b, ab = (size_t)g.a * g.b;
  const int arrow_row0 = g.nt * g.b;

  while (true) {
    const int t = cta_ticket(c, &s_t);
    if (t < 0 || t >= ntasks) break;
    // Forward order: tiles ascending, arrow last.  Backward: arrow first, then descending.
    bool is_arrow;
    int gi;
    if (p.trans == 0) {
      is_arrow = t == ntile;
      gi = t;
    } else {
      is_arrow = p.use_arrow && t == 0;
      gi = ntile - 1 - (t - (p.use_arrow ? 1 : 0));
    }

    if (is_arrow) {
      double s = (row < g.a && col < p.nc) ? __ldcg(p.B + (size_t)(arrow_row0 + row) * p.ldb + col) : 0.0;
      if (p.trans == 0) {
        bool ok = true;
        for (int k = 0; k < ntile; ++k) {
          if (!(ok = cta_wait(c, c.flags + k, nullptr, &s_ok))) break;
          s -= __ldcg(p.part + (size_t)k * TS * NC + threadIdx.x);
        }
        if (!ok) break;
      }
      Ss[threadIdx.x] = s;
      tile_load(Fs, make_tile(p.T, g.a, 0, 0, g.a, g.a));
      __syncthreads();
      tile_pad_identity(Fs, g.a);
      __syncthreads();
      tile_diag_recip(Fs, rd);
      __syncthreads();
      warp_trsv(Ss, Fs, rd, p.trans != 0, p.nc);
      __syncthreads();
      if (row < g.a && col < p.nc) p.B[(size_t)(arrow_row0 + row) * p.ldb + col] = Ss[threadIdx.x];
      cta_publish(c, c.flags + ntile);
      continue;
    }

    const int i = gi / g.B, r = gi % g.B;
    const int rows = g.vrows(r);
    const int row0 = i * g.b + r * TS;
    double s = (row < rows && col < p.nc) ? __ldcg(p.B + (size_t)(row0 + row) * p.ldb + col) : 0.0;
    // The diagonal factor tile and its reciprocals do not depend on other tasks:
    // stage them before waiting on any dependency.
    tile_load(Fs, make_tile(p.D + i * bb, g.b, r * TS, r * TS, g.b, g.b));
    __syncthreads();
    tile_pad_identity(Fs, rows);
    __syncthreads();
    tile_diag_recip(Fs, rd);
    bool ok = true;
    if (p.trans == 0) {
      // s -= L_{i-1}(r,k) y(i-1,k) for all k; s -= D_i(r,k) y(i,k) for k < r
      const int nprev = i > 0 ? g.B : 0;
      for (int st = 0; st < nprev + r; ++st) {
        const bool pv = st < nprev;
        const int k = pv ? st : st - nprev;
        const int bi = pv ? i - 1 : i;
        if (!(ok = cta_wait(c, c.flags + vflag(g, bi, k), nullptr, &s_ok))) break;
        const Tile M = pv ? make_tile(p.L + (i - 1) * bb, g.b, r * TS, k * TS, g.b, g.b)
                          : make_tile(p.D + i * bb, g.b, r * TS, k * TS, g.b, g.b);
        tile_load(Ms, M);
        vec_load(Vs, p, bi * g.b + k * TS, g.vrows(k));
        __syncthreads();
        s = tile_gemv(s, Ms, Vs);
        __syncthreads();
      }
    } else {
      // s -= D_i(k,r)^T x(i,k) (k > r); L_i(k,r)^T x(i+1,k); R_i(:,r)^T x_a
      const int nd = g.B - 1 - r;
      const int nl = i < g.nt - 1 ? g.B : 0;
      const int na = p.use_arrow ? 1 : 0;
      for (int st = 0; st < na + nl + nd; ++st) {
        double v[PER_THREAD];
        int vrow0, vrows;
        const int* f;
        if (st < na) {
          tile_ldg(v, make_tile(p.R + i * ab, g.b, 0, r * TS, g.a, g.b));
          vrow0 = arrow_row0;
          vrows = g.a;
          f = c.flags + ntile;
        } else if (st < na + nl) {
          const int k = g.B - 1 - (st - na);
          tile_ldg(v, make_tile(p.L + i * bb, g.b, k * TS, r * TS, g.b, g.b));
          vrow0 = (i + 1) * g.b + k * TS;
          vrows = g.vrows(k);
          f = c.flags + vflag(g, i + 1, k);
        } else {
          const int k = g.B - 1 - (st - na - nl);
          tile_ldg(v, make_tile(p.D + i * bb, g.b, k * TS, r * TS, g.b, g.b));
          vrow0 = i * g.b + k * TS;
          vrows = g.vrows(k);
          f = c.flags + vflag(g, i, k);
        }
        tile_sts_t(Ms, v);   // stage the transposed tile
        if (!(ok = cta_wait(c, f, nullptr, &s_ok))) break;
        vec_load(Vs, p, vrow0, vrows);
        __syncthreads();
        s = tile_gemv(s, Ms, Vs);
        __syncthreads();
      }
    }
    if (!ok) break;
    Ss[threadIdx.x] = s;
    __syncthreads();
    warp_trsv(Ss, Fs, rd, p.trans != 0, p.nc);
    __syncthreads();
    if (row < rows && col < p.nc) p.B[(size_t)(row0 + row) * p.ldb + col] = Ss[threadIdx.x];
    if (p.trans == 0 && p.use_arrow) {
      // arrow partial R_i(:, r) y(i, r)
      tile_load(Ms, make_tile(p.R + i * ab, g.b, 0, r * TS, g.a, g.b));
      __syncthreads();
      const double pa = -tile_gemv(0.0, Ms, Ss);
      p.part[(size_t)gi * TS * NC + threadIdx.x] = pa;
    }
    cta_publish(c, c.flags + vflag(g, i, r));
  }
}

void launch_solve(const Geom& g, const double* D, const double* L, const double* R, const double* T, double* Bv,
                  int ldb, int nc, int trans, int use_arrow, double* arrow_part, const LaunchCtl& lc) {
  // One launch covers nc <= NC right-hand-side columns starting at Bv (row stride ldb).
  SolveArgs p;
  p.D = D;
  p.L = L;
  p.R = R;
  p.T = T;
  p.B = Bv;
  p.ldb = ldb;
  p.nc = nc;
  p.g = g;
  p.use_arrow = use_arrow;
  p.trans = trans;
  p.part = arrow_part;
  p.c.ctrl = lc.ctrl;
  p.c.flags = lc.flags;
  p.c.epoch = lc.epoch;
  p.c.wait_ns = lc.wait_ns;
  k_solve<<<lc.grid, NT, 0, lc.stream>>>(p);
  count_launches(1);
}

}  // namespace gbta
