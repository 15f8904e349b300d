// Per-task body of the BTA triangular sweeps, shared by the single-instance kernel
// (bta_solve.cu) and the multi-instance kernel (bta_batch.cu).  The tiles are solved in
// the elimination order of the factor (Geom: top-down, or both chains towards the
// separator block and then the separator; the backward sweep in reverse).
//
// Replaces the block forward / backward substitutions the reference runs through
// Serinv (src/pyinla/solvers/structured_solver.py:112-140): trans = 0 solves
// L y = b, trans = 1 solves L^T x = y, in place on the right-hand side.  One task
// produces one 32-row tile g of the solution.  The tiles form a chain (tile g needs
// tile g-1 in the forward sweep, g+1 in the backward sweep), so each task does all
// of its work that does not depend on that neighbour before waiting for it:
//   * invert its diagonal factor tile, Linv = F^{-1}, and form M = Linv P
//     (backward: Linv^T P^T) with P the block coupling it to the neighbour tile;
//   * subtract the products of every other solution tile it depends on, then
//     u = Linv s (backward: Linv^T s);
// leaving only  y_g = u - M y_neighbour  (one 32 x 32 matrix-vector product spread
// over the whole CTA) between the neighbour's publication and its own.  The forward
// sweep also leaves the arrow contribution R_i(:,r) y(i,r) of each tile in a partial
// buffer, after publishing the tile and under a flag of its own (off the chain), and
// the arrow task sums the partials in a fixed order.
#pragma once

#include "bta_common.cuh"

namespace gbta {

constexpr int NC = SOLVE_NC;   // right-hand-side columns per launch

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
  int ntasks;       // nt*B (+1 with the arrow); both sweeps: twice that
  int both;         // one launch for the forward sweep and then the backward sweep
  int bflag0;       // (both) offset of the backward sweep's tile and arrow flags
  Ctl c;
};

static __device__ __forceinline__ int vflag(const Geom& g, int i, int r) { return i * g.B + r; }
// Flag of the forward sweep's arrow partial of tile gi (published after the tile).
static __device__ __forceinline__ int pflag(const Geom& g, int gi) { return g.nt * g.B + 1 + gi; }

// Vectors are TS x NC, stored [row][col] in shared memory (V[row*NC + col]).
// res[q] = sum_m M[row][m] v[m][q] for q < nc, with M[row][m] = Ms[row*LDS + m]
// (MT = false) or Ms[m*LDS + row] (MT = true).  Thread t owns row t/4 and the
// k-range [8*(t%4), +8); the four partial sums of a row are combined with shuffles,
// so every thread of the row returns the full dot products.
template <bool MT>
static __device__ __forceinline__ void cta_gemv(const double* Ms, const double* V, int nc, double (&res)[NC]) {
  const int row = threadIdx.x >> 2, part = threadIdx.x & 3;
#pragma unroll
  for (int q = 0; q < NC; ++q) {
    double s = 0.0;
    if (q < nc) {
#pragma unroll
      for (int k = 0; k < TS / 4; ++k) {
        const int m = part * (TS / 4) + k;
        const double mv = MT ? Ms[m * LDS + row] : Ms[row * LDS + m];
        s = fma(mv, V[m * NC + q], s);
      }
    }
    s += __shfl_xor_sync(0xffffffffu, s, 1);
    s += __shfl_xor_sync(0xffffffffu, s, 2);
    res[q] = s;
  }
}

// Load the solution tile starting at global row `row0` (rows valid) into V.
static __device__ __forceinline__ void vec_load(double* V, const SolveArgs& p, int row0, int rows) {
  const int row = threadIdx.x / NC, col = threadIdx.x % NC;
  V[row * NC + col] = (row < rows && col < p.nc) ? __ldcg(p.B + (size_t)(row0 + row) * p.ldb + col) : 0.0;
}

// Dependency of a sweep step: the matrix tile (row-major; used as is in the forward
// sweep, transposed in the backward sweep), the solution rows it multiplies, its flag.
struct DepTile {
  Tile t;
  int vrow0, vrows;
  const int* flag;
};

// Shared memory of a solve task: the diagonal factor tile Fs, Linv = F^{-1} (Ws),
// M = Linv P (forward) or Linv^T P^T (backward) (Ms), a staged dependency tile (Ts),
// the staged solution tile (Vs), the accumulated right-hand side (Ss) and the
// reciprocals of the diagonal (rd).
constexpr size_t SOLVE_SMEM = (4 * TILE_SMEM + 2 * TS * NC + TS) * sizeof(double);

// Task t of a solve instance.  `raw` is SOLVE_SMEM bytes of shared memory.  Returns
// false when the launch is aborted.
static __device__ __forceinline__ bool solve_task(const SolveArgs& p, int t, unsigned char* raw, int* s_okp) {
  double* Fs = reinterpret_cast<double*>(raw);
  double* Ws = Fs + TILE_SMEM;
  double* Ms = Ws + TILE_SMEM;
  double* Ts = Ms + TILE_SMEM;
  double* Vs = Ts + TILE_SMEM;
  double* Ss = Vs + TS * NC;
  double* rd = Ss + TS * NC;
  int& s_ok = *s_okp;
  const Geom& g = p.g;
  const Ctl& c = p.c;
  const int ntile = g.nt * g.B;
  const size_t bb = (size_t)g.b * g.b, ab = (size_t)g.a * g.b;
  const int arrow_row0 = g.nt * g.b;
  // With p.both the tickets of the forward sweep come first and those of the backward
  // sweep follow (its tasks also wait for the forward sweep's tile they start from); the
  // backward sweep's flags sit at p.bflag0.
  const int nsweep = ntile + (p.use_arrow ? 1 : 0);
  const bool fwd = p.both ? t < nsweep : p.trans == 0;
  const int fo = (p.both && !fwd) ? p.bflag0 : 0;   // offset of this sweep's flags
  const int tt = t;                                  // the ticket (trace record)
  if (p.both && !fwd) t -= nsweep;
  {
    const unsigned long long t_task0 = c.trace ? gtimer() : 0ull;
    // ticket -> tile in the elimination order of the blocks (Geom): forward, the tiles of
    // the two chains interleaved one for one, then the separator's, then the arrow;
    // backward, the arrow, the separator's tiles from the last, then both chains outwards
    bool is_arrow;
    int i = 0, r = 0;
    {
      const int sp = g.sep(), n1 = sp * g.B, n2 = (g.nt - 1 - sp) * g.B;
      if (fwd) {
        is_arrow = t == ntile;
        if (!is_arrow) {
          if (t < n1 + n2) {
            int k;
            const int ch = Geom::interleave(n1, n2, t, &k);
            i = ch == 0 ? k / g.B : g.nt - 1 - k / g.B;
            r = k % g.B;
          } else {
            i = sp;
            r = t - (n1 + n2);
          }
        }
      } else {
        is_arrow = p.use_arrow && t == 0;
        const int u = t - (p.use_arrow ? 1 : 0);
        if (!is_arrow) {
          if (u < g.B) {
            i = sp;
            r = g.B - 1 - u;
          } else {
            int k;
            const int ch = Geom::interleave(n1, n2, u - g.B, &k);
            i = ch == 0 ? sp - 1 - k / g.B : sp + 1 + k / g.B;
            r = g.B - 1 - k % g.B;
          }
        }
      }
    }
    const int gi = i * g.B + r;
    const int srow = threadIdx.x / NC, scol = threadIdx.x % NC;

    if (is_arrow) {
      // forward: s = b_a - ordered sum of the partials, y_a = T^{-1} s;
      // backward: x_a = T^{-T} y_a
      tile_load(Fs, make_tile(p.T, g.a, 0, 0, g.a, g.a));
      __syncthreads();
      tile_pad_identity(Fs, g.a);
      for (int idx = threadIdx.x; idx < TS * TS; idx += NT) Ws[(idx / TS) * LDS + idx % TS] = (idx / TS == idx % TS);
      __syncthreads();
      tile_diag_recip(Fs, rd);
      smem_trsm_rln(Ws, Fs, rd);   // Ws = T^{-1}
      if (p.both && !fwd && !cta_wait(c, c.flags + ntile, nullptr, &s_ok)) return false;   // the forward y_a
      double s = (srow < g.a && scol < p.nc) ? __ldcg(p.B + (size_t)(arrow_row0 + srow) * p.ldb + scol) : 0.0;
      if (fwd) {
        // every tile's partial: the flags are polled by all threads at once; thread t then
        // sums the partials k = t (mod NT), RE entries per round, and the NT sums of an
        // entry are combined in a fixed binary tree (a fixed order: reproducible)
        bool ok = true;
        for (int k = threadIdx.x; k < ntile && ok; k += NT) ok = spin_ready(c, c.flags + pflag(g, k));
        if (!__syncthreads_and(ok)) return false;
        constexpr int RE = 8;
        double* red = Ts;                // NT x RE doubles (free in the arrow task)
        const int ne = g.a * NC;         // entries row * NC + q of the partials with row < a
        for (int e0 = 0; e0 < ne; e0 += RE) {
          double acc[RE];
#pragma unroll
          for (int e = 0; e < RE; ++e) acc[e] = 0.0;
          for (int k = threadIdx.x; k < ntile; k += NT) {
            const double* P = p.part + (size_t)k * TS * NC + e0;
#pragma unroll
            for (int e = 0; e < RE; ++e)
              if (e0 + e < ne) acc[e] += __ldcg(P + e);
          }
#pragma unroll
          for (int e = 0; e < RE; ++e) red[threadIdx.x * RE + e] = acc[e];
          for (int st = NT / 2; st > 0; st >>= 1) {
            __syncthreads();
            if (threadIdx.x < st)
#pragma unroll
              for (int e = 0; e < RE; ++e) red[threadIdx.x * RE + e] += red[(threadIdx.x + st) * RE + e];
          }
          __syncthreads();
          // entry row * NC + q is thread (row, q)'s right-hand side element
          if (threadIdx.x >= e0 && threadIdx.x < e0 + RE && threadIdx.x < ne) s -= red[threadIdx.x - e0];
          __syncthreads();
        }
      }
      Ss[threadIdx.x] = s;
      __syncthreads();
      double res[NC];
      if (fwd)
        cta_gemv<false>(Ws, Ss, p.nc, res);
      else
        cta_gemv<true>(Ws, Ss, p.nc, res);
      if ((threadIdx.x & 3) == 0) {
        const int row = threadIdx.x >> 2;
        for (int q = 0; q < p.nc; ++q)
          if (row < g.a) p.B[(size_t)(arrow_row0 + row) * p.ldb + q] = res[q];
      }
      cta_publish(c, c.flags + fo + ntile);
      trace_task(c, tt, 1, t_task0);
      return true;
    }

    const int rows = g.vrows(r);
    const int row0 = i * g.b + r * TS;
    // ---- independent of other tasks: Linv of the diagonal tile and M
    tile_load(Fs, make_tile(p.D + i * bb, g.b, r * TS, r * TS, g.b, g.b));
    __syncthreads();
    tile_pad_identity(Fs, rows);
    for (int idx = threadIdx.x; idx < TS * TS; idx += NT) Ws[(idx / TS) * LDS + idx % TS] = (idx / TS == idx % TS);
    __syncthreads();
    tile_diag_recip(Fs, rd);
    smem_trsm_rln(Ws, Fs, rd);   // Ws = F^{-1}
    bool has_nb = false;
    DepTile nb;
    // the neighbour tile: forward, the tile eliminated just before (i, r-1), or for r = 0
    // the last tile of the first neighbour block eliminated before i, through its coupling
    // slot; backward, the tile eliminated just after: (i, r+1), or for r = B-1 the first
    // tile of nxt(i), through block i's coupling slot
    const int np = g.nprev(i), nx = g.nxt(i), lsi = g.lslot(i);
    if (fwd) {
      if (r > 0) {
        has_nb = true;
        nb.t = make_tile(p.D + i * bb, g.b, r * TS, (r - 1) * TS, g.b, g.b);
        nb.vrow0 = i * g.b + (r - 1) * TS;
        nb.vrows = g.vrows(r - 1);
        nb.flag = c.flags + fo + vflag(g, i, r - 1);
      } else if (np > 0) {
        const int p0 = g.prev(i, 0);
        has_nb = true;
        nb.t = make_tile(p.L + g.lslot(p0) * bb, g.b, 0, (g.B - 1) * TS, g.b, g.b);
        nb.vrow0 = p0 * g.b + (g.B - 1) * TS;
        nb.vrows = g.vrows(g.B - 1);
        nb.flag = c.flags + fo + vflag(g, p0, g.B - 1);
      }
    } else {
      if (r < g.B - 1) {
        has_nb = true;
        nb.t = make_tile(p.D + i * bb, g.b, (r + 1) * TS, r * TS, g.b, g.b);
        nb.vrow0 = i * g.b + (r + 1) * TS;
        nb.vrows = g.vrows(r + 1);
        nb.flag = c.flags + fo + vflag(g, i, r + 1);
      } else if (nx >= 0) {
        has_nb = true;
        nb.t = make_tile(p.L + lsi * bb, g.b, 0, r * TS, g.b, g.b);
        nb.vrow0 = nx * g.b;
        nb.vrows = g.vrows(0);
        nb.flag = c.flags + fo + vflag(g, nx, 0);
      }
    }
    if (has_nb) {
      // forward M = F^{-1} P, backward M = F^{-T} P^T: M[row][m] multiplies the
      // neighbour's solution element m.
      tile_load(Ts, nb.t);
      __syncthreads();
      for (int idx = threadIdx.x; idx < TS * TS; idx += NT) {
        const int rr = idx / TS, cc = idx % TS;
        double sacc = 0.0;
        if (fwd) {
#pragma unroll 8
          for (int m = 0; m < TS; ++m) sacc = fma(Ws[rr * LDS + m], Ts[m * LDS + cc], sacc);
        } else {
#pragma unroll 8
          for (int m = 0; m < TS; ++m) sacc = fma(Ws[m * LDS + rr], Ts[cc * LDS + m], sacc);
        }
        Ms[rr * LDS + cc] = sacc;
      }
    }
    // ---- the other dependencies (all solved before the neighbour): s -= A_k v_k
    if (p.both && !fwd && !cta_wait(c, c.flags + vflag(g, i, r), nullptr, &s_ok)) return false;   // the forward y
    Ss[threadIdx.x] = (srow < rows && scol < p.nc) ? __ldcg(p.B + (size_t)(row0 + srow) * p.ldb + scol) : 0.0;
    __syncthreads();
    int ndep, nfirst, n0 = 0;
    if (fwd) {
      // for each neighbour block p eliminated before i: S_p(r, k) y(p, k) for k < B (S_p
      // its coupling slot), then D_i(r, k) y(i, k) for k < r, minus the neighbour tile
      n0 = np > 0 ? ((r == 0) ? g.B - 1 : g.B) : 0;
      nfirst = n0 + (np > 1 ? g.B : 0);
      ndep = nfirst + (r > 0 ? r - 1 : 0);
    } else {
      // arrow, S_i(k, r)^T x(nxt(i), k) for k < B, D_i(k, r)^T x(i, k) for k > r, minus the
      // neighbour tile
      nfirst = (nx >= 0) ? ((r == g.B - 1) ? g.B - 1 : g.B) : 0;
      ndep = (p.use_arrow ? 1 : 0) + nfirst + (r < g.B - 1 ? g.B - 2 - r : 0);
    }
    bool ok = true;
    for (int st = 0; st < ndep && ok; ++st) {
      DepTile d;
      if (fwd) {
        if (st < nfirst) {
          const int pb = g.prev(i, st < n0 ? 0 : 1), k = st < n0 ? st : st - n0;
          d.t = make_tile(p.L + g.lslot(pb) * bb, g.b, r * TS, k * TS, g.b, g.b);
          d.vrow0 = pb * g.b + k * TS;
          d.vrows = g.vrows(k);
          d.flag = c.flags + fo + vflag(g, pb, k);
        } else {
          const int k = st - nfirst;   // k < r - 1
          d.t = make_tile(p.D + i * bb, g.b, r * TS, k * TS, g.b, g.b);
          d.vrow0 = i * g.b + k * TS;
          d.vrows = g.vrows(k);
          d.flag = c.flags + fo + vflag(g, i, k);
        }
      } else {
        int s2 = st;
        if (p.use_arrow && s2 == 0) {
          d.t = make_tile(p.R + i * ab, g.b, 0, r * TS, g.a, g.b);
          d.vrow0 = arrow_row0;
          d.vrows = g.a;
          d.flag = c.flags + fo + ntile;
        } else {
          if (p.use_arrow) --s2;
          if (s2 < nfirst) {
            const int k = g.B - 1 - s2;   // coupling slot rows B-1 down to (r == B-1 ? 1 : 0)
            d.t = make_tile(p.L + lsi * bb, g.b, k * TS, r * TS, g.b, g.b);
            d.vrow0 = nx * g.b + k * TS;
            d.vrows = g.vrows(k);
            d.flag = c.flags + fo + vflag(g, nx, k);
          } else {
            const int k = g.B - 1 - (s2 - nfirst);   // D_i rows B-1 down to r+2
            d.t = make_tile(p.D + i * bb, g.b, k * TS, r * TS, g.b, g.b);
            d.vrow0 = i * g.b + k * TS;
            d.vrows = g.vrows(k);
            d.flag = c.flags + fo + vflag(g, i, k);
          }
        }
      }
      tile_load(Ts, d.t);   // the matrix tile does not depend on other tasks
      if (!(ok = cta_wait(c, d.flag, nullptr, &s_ok))) break;
      vec_load(Vs, p, d.vrow0, d.vrows);
      __syncthreads();
      double res[NC];
      if (fwd)
        cta_gemv<false>(Ts, Vs, p.nc, res);
      else
        cta_gemv<true>(Ts, Vs, p.nc, res);
      if ((threadIdx.x & 3) == 0)
        for (int q = 0; q < p.nc; ++q) Ss[(threadIdx.x >> 2) * NC + q] -= res[q];
      __syncthreads();
    }
    if (!ok) return false;
    trace_clear_marks(c, tt);
    trace_mark(c, tt, 0);   // every dependency but the neighbour done
    // u = Linv s (forward) or Linv^T s (backward)
    double u[NC];
    if (fwd)
      cta_gemv<false>(Ws, Ss, p.nc, u);
    else
      cta_gemv<true>(Ws, Ss, p.nc, u);
    // ---- the neighbour: y = u - M v_nb
    if (has_nb) {
      if (!cta_wait(c, nb.flag, nullptr, &s_ok)) return false;
      trace_mark(c, tt, 1);   // neighbour published
      vec_load(Vs, p, nb.vrow0, nb.vrows);
      __syncthreads();
      double res[NC];
      cta_gemv<false>(Ms, Vs, p.nc, res);
#pragma unroll
      for (int q = 0; q < NC; ++q) u[q] -= res[q];
    }
    __syncthreads();
    if ((threadIdx.x & 3) == 0) {
      const int row = threadIdx.x >> 2;
      for (int q = 0; q < NC; ++q) {
        Ss[row * NC + q] = (q < p.nc && row < rows) ? u[q] : 0.0;
        if (q < p.nc && row < rows) p.B[(size_t)(row0 + row) * p.ldb + q] = u[q];
      }
    }
    trace_mark(c, tt, 2);   // solution tile computed and stored
    cta_publish(c, c.flags + fo + vflag(g, i, r));   // the next tile's wait ends here
    trace_mark(c, tt, 3);   // published
    if (fwd && p.use_arrow) {
      // arrow partial R_i(:, r) y(i, r) (rows >= a of the staged tile are zero), off
      // the chain, under its own flag
      tile_load(Ts, make_tile(p.R + i * ab, g.b, 0, r * TS, g.a, g.b));
      __syncthreads();
      double res[NC];
      cta_gemv<false>(Ts, Ss, p.nc, res);
      if ((threadIdx.x & 3) == 0) {
        const int row = threadIdx.x >> 2;
        for (int q = 0; q < NC; ++q) p.part[(size_t)gi * TS * NC + row * NC + q] = (q < p.nc) ? res[q] : 0.0;
      }
      cta_publish(c, c.flags + pflag(g, gi));
    }
    trace_task(c, tt, 0, t_task0);
  }
  return true;
}

}  // namespace gbta
