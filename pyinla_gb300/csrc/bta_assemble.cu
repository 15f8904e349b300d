// On-device assembly of BTA precisions and the trace contractions of the adjoint.
//
// Assembly replaces, for the Gaussian spatio-temporal models, the chain the reference
// runs on every objective evaluation:
//   Q_prior: sum of Kronecker products of temporal and spatial sparse matrices
//            (src/pyinla/submodels/spatio_temporal.py:114-149, coregional mixing in
//            src/pyinla/models/coregional_model.py:274-555),
//   Q_cond = Q_prior - A^T D A with D = -tau_y I (src/pyinla/core/model.py:384-423,
//            src/pyinla/likelihoods/gaussian.py:127-129),
//   then the sparse-to-BTA scatter (src/pyinla/solvers/structured_solver.py:192-468).
// Here the BTA blocks are written directly: every block row is zero-filled and the
// spatial terms, scaled by their temporal/theta coefficients, are added row by row
// (one warp per block row; one lane per union-pattern entry, so every sum is taken
// in a fixed order and the result is deterministic), followed by the tau_y A^T A
// rows.  The theta-independent A^T A is precomputed once (the reference rebuilds the
// product on every call).
//
// The contraction kernel evaluates <Sigma_tt, S_k>, <Sigma_{t+1,t}, S_k>,
// mu_t^T S_k mu_t and mu_{t+1}^T S_k mu_t per term and time block, plus the same
// quantities for A^T A -- everything tr(Q^{-1} dQ/dtheta) and mu^T dQ/dtheta mu need.
#include <cuda_runtime.h>

#include "../../include/pyinla_gb300.h"
#include "bta_internal.h"

namespace gbta {

struct KronDesc {
  int ns, nv, nterms;
  const int* upat_rowptr;   // [ns+1]
  const int* upat_col;      // [nu]
  const double* uval;       // [nu * nterms]
  const int* term_vw;       // [2 * nterms]
};

struct LikDesc {
  const long long* rowptr;  // [nt*b + 1] or null
  const int* col;           // block-local columns
  const double* val;
  const double* Rdense;     // [nt*a*b] or null
  const double* Tdense;     // [a*a] or null
  const double* scale;      // [nv] noise precision of each variate (device)
  const int* arrow_var;     // [a] variate of each fixed effect, or null (all variate 0)
};

// Variate of fixed effect i (out-of-range labels count as "no variate": -1).
__device__ __forceinline__ int arrow_variate(const LikDesc& ld, int i, int nv) {
  const int v = ld.arrow_var ? ld.arrow_var[i] : 0;
  return (v >= 0 && v < nv) ? v : -1;
}

constexpr int AS_WARPS = 8;

__global__ void __launch_bounds__(AS_WARPS * 32) k_assemble_rows(Geom g, KronDesc kd, LikDesc ld, const double* alpha,
                                                                 const double* beta, double* D, double* L) {
  const int lane = threadIdx.x & 31;
  const long long wid = (long long)blockIdx.x * AS_WARPS + (threadIdx.x >> 5);
  const long long nrows = (long long)g.nt * g.b;
  if (wid >= nrows) return;
  const int t = (int)(wid / g.b), rho = (int)(wid % g.b);
  double* drow = D + ((size_t)t * g.b + rho) * g.b;
  double* lrow = (t < g.nt - 1) ? L + ((size_t)t * g.b + rho) * g.b : nullptr;
  for (int c = lane; c < g.b; c += 32) {
    drow[c] = 0.0;
    if (lrow) lrow[c] = 0.0;
  }
  __syncwarp();
  const int v = rho / kd.ns, r = rho % kd.ns;
  const int e0 = kd.upat_rowptr[r], e1 = kd.upat_rowptr[r + 1];
  for (int e = e0 + lane; e < e1; e += 32) {
    const int col = kd.upat_col[e];
    for (int k = 0; k < kd.nterms; ++k) {
      if (kd.term_vw[2 * k] != v) continue;
      const double val = kd.uval[(size_t)e * kd.nterms + k];
      if (val == 0.0) continue;
      const int cc = kd.term_vw[2 * k + 1] * kd.ns + col;
      drow[cc] += alpha[(size_t)k * g.nt + t] * val;
      if (lrow) lrow[cc] += beta[(size_t)k * (g.nt - 1) + t] * val;
    }
  }
  if (ld.rowptr) {
    __syncwarp();
    const long long l0 = ld.rowptr[wid], l1 = ld.rowptr[wid + 1];
    const double sc = ld.scale[v];   // observations of variate v touch only its own nodes
    for (long long e = l0 + lane; e < l1; e += 32) drow[ld.col[e]] += sc * ld.val[e];
  }
}

// Arrow blocks: R entries take the scale of their column's variate, T entries that of
// their row's fixed effect (A^T A couples a fixed effect only with its own variate).
__global__ void k_assemble_arrow(Geom g, int ns, int nv, LikDesc ld, double tip_diag, double* R, double* T) {
  const size_t nR = (size_t)g.nt * g.a * g.b, nT = (size_t)g.a * g.a;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < nR + nT; e += (size_t)gridDim.x * blockDim.x) {
    if (e < nR) {
      R[e] = ld.Rdense ? ld.scale[(int)(e % g.b) / ns] * ld.Rdense[e] : 0.0;
    } else {
      const size_t q = e - nR;
      const int i = (int)(q / g.a), j = (int)(q % g.a);
      const int v = arrow_variate(ld, i, nv);
      T[q] = ((ld.Tdense && v >= 0) ? ld.scale[v] * ld.Tdense[q] : 0.0) + (i == j ? tip_diag : 0.0);
    }
  }
}

// ---------------------------------------------------------------------------
// Contractions.  One CTA per time block t (plus CTA nt for the tip), fixed-order
// reductions.  Output layout (K = nterms):
//   out[0*K*nt + k*nt + t]  <Sigma_tt, S_k>              (Sigma_tt = SD[t])
//   out[1*K*nt + k*nt + t]  <Sigma_{t+1,t}, S_k>         (SL[t]; 0 for t = nt-1)
//   out[2*K*nt + k*nt + t]  mu_t^T S_k mu_t
//   out[3*K*nt + k*nt + t]  mu_{t+1}^T S_k mu_t
//   out[4*K*nt + v*2*(nt+1) + t]           <Sigma, A_v^T A_v> restricted to block t
//                                           (D part + 2 * R part); index nt: the tip part
//   out[4*K*nt + v*2*(nt+1) + (nt+1) + t]  the same with mu mu^T
// where A_v^T A_v is the part of A^T A of variate v's observations (its rows and
// columns lie in variate v's nodes and fixed effects).
// ---------------------------------------------------------------------------
constexpr int CT_THREADS = 256;
constexpr int CT_CHUNK = 8;   // terms accumulated per pass

__device__ double block_sum(double v, double* red) {
  red[threadIdx.x] = v;
  __syncthreads();
  for (int w = CT_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  const double s = red[0];
  __syncthreads();
  return s;
}

__global__ void __launch_bounds__(CT_THREADS) k_contract(Geom g, KronDesc kd, LikDesc ld, const double* SD,
                                                         const double* SL, const double* SR, const double* ST,
                                                         const double* mu, double* out) {
  __shared__ double red[CT_THREADS];
  const int t = blockIdx.x;
  const int K = kd.nterms;
  const size_t KN = (size_t)K * g.nt;
  const size_t bb = (size_t)g.b * g.b;
  const size_t LS = 2 * (size_t)(g.nt + 1);   // per-variate stride of the A^T A sums
  if (t == g.nt) {   // tip block of A^T A
    for (int v = 0; v < kd.nv; ++v) {
      double sc = 0.0, sq = 0.0;
      if (ld.Tdense && g.a > 0) {
        const double* mua = mu ? mu + (size_t)g.nt * g.b : nullptr;
        for (int q = threadIdx.x; q < g.a * g.a; q += CT_THREADS) {
          const int i = q / g.a, j = q % g.a;
          if (arrow_variate(ld, i, kd.nv) != v) continue;
          if (ST) sc += ST[q] * ld.Tdense[q];
          if (mua) sq += mua[i] * ld.Tdense[q] * mua[j];
        }
      }
      sc = block_sum(sc, red);
      sq = block_sum(sq, red);
      if (threadIdx.x == 0) {
        out[4 * KN + v * LS + g.nt] = sc;
        out[4 * KN + v * LS + (g.nt + 1) + g.nt] = sq;
      }
    }
    return;
  }
  const double* Dt = SD ? SD + t * bb : nullptr;
  const double* Lt = (SL && t < g.nt - 1) ? SL + t * bb : nullptr;
  const double* mut = mu ? mu + (size_t)t * g.b : nullptr;
  const double* mun = (mu && t < g.nt - 1) ? mu + (size_t)(t + 1) * g.b : nullptr;
  for (int k0 = 0; k0 < K; k0 += CT_CHUNK) {
    double c[CT_CHUNK], d[CT_CHUNK], qc[CT_CHUNK], qd[CT_CHUNK];
#pragma unroll
    for (int j = 0; j < CT_CHUNK; ++j) c[j] = d[j] = qc[j] = qd[j] = 0.0;
    for (int rho = threadIdx.x; rho < g.b; rho += CT_THREADS) {
      const int v = rho / kd.ns, r = rho % kd.ns;
      for (int e = kd.upat_rowptr[r]; e < kd.upat_rowptr[r + 1]; ++e) {
        const int col = kd.upat_col[e];
#pragma unroll
        for (int j = 0; j < CT_CHUNK; ++j) {
          const int k = k0 + j;
          if (k >= K || kd.term_vw[2 * k] != v) continue;
          const double val = kd.uval[(size_t)e * K + k];
          const int cc = kd.term_vw[2 * k + 1] * kd.ns + col;
          if (Dt) c[j] += Dt[(size_t)rho * g.b + cc] * val;
          if (Lt) d[j] += Lt[(size_t)rho * g.b + cc] * val;
          if (mut) qc[j] += mut[rho] * val * mut[cc];
          if (mun) qd[j] += mun[rho] * val * mut[cc];
        }
      }
    }
#pragma unroll
    for (int j = 0; j < CT_CHUNK; ++j) {
      const double sc = block_sum(c[j], red), sd = block_sum(d[j], red);
      const double sqc = block_sum(qc[j], red), sqd = block_sum(qd[j], red);
      const int k = k0 + j;
      if (threadIdx.x == 0 && k < K) {
        out[0 * KN + (size_t)k * g.nt + t] = sc;
        out[1 * KN + (size_t)k * g.nt + t] = sd;
        out[2 * KN + (size_t)k * g.nt + t] = sqc;
        out[3 * KN + (size_t)k * g.nt + t] = sqd;
      }
    }
  }
  // A^T A on block t, per variate: D part (CSR rows of the variate's nodes) and arrow
  // part (dense R columns of the variate's nodes, counted twice).
  for (int v = 0; v < kd.nv; ++v) {
    double lc = 0.0, lq = 0.0;
    if (ld.rowptr) {
      for (int rho = v * kd.ns + threadIdx.x; rho < (v + 1) * kd.ns; rho += CT_THREADS) {
        const long long row = (long long)t * g.b + rho;
        for (long long e = ld.rowptr[row]; e < ld.rowptr[row + 1]; ++e) {
          const int cc = ld.col[e];
          if (Dt) lc += Dt[(size_t)rho * g.b + cc] * ld.val[e];
          if (mut) lq += mut[rho] * ld.val[e] * mut[cc];
        }
      }
    }
    if (ld.Rdense && g.a > 0) {
      const double* Rt = ld.Rdense + (size_t)t * g.a * g.b;
      const double* SRt = SR ? SR + (size_t)t * g.a * g.b : nullptr;
      const double* mua = mu ? mu + (size_t)g.nt * g.b : nullptr;
      for (int q = threadIdx.x; q < g.a * kd.ns; q += CT_THREADS) {
        const int r = q / kd.ns, col = v * kd.ns + q % kd.ns;
        const size_t e = (size_t)r * g.b + col;
        if (SRt) lc += 2.0 * SRt[e] * Rt[e];
        if (mua) lq += 2.0 * mua[r] * Rt[e] * mut[col];
      }
    }
    lc = block_sum(lc, red);
    lq = block_sum(lq, red);
    if (threadIdx.x == 0) {
      out[4 * KN + v * LS + t] = lc;
      out[4 * KN + v * LS + (g.nt + 1) + t] = lq;
    }
  }
}

}  // namespace gbta

extern "C" int gbta_set_error(int code, const char* msg);

static int kron_args_ok(int b, int ns, int nv, int nterms, const int* rp, const int* col, const double* uval,
                        const int* vw) {
  if (ns < 1 || nv < 1 || nv * ns != b) return gbta_set_error(GBTA_ERR_ARG, "kron: need nv * ns == b");
  if (nv > GBTA_MAX_VARIATES) return gbta_set_error(GBTA_ERR_ARG, "kron: too many variates");
  if (nterms < 0 || (nterms > 0 && (!rp || !col || !uval || !vw)))
    return gbta_set_error(GBTA_ERR_ARG, "kron: null term pointer");
  return GBTA_OK;
}

extern "C" int gbta_assemble_kron(gbta_solver* s, int ns, int nv, int nterms, const int* upat_rowptr,
                                  const int* upat_col, const double* uval, const int* term_vw, const double* alpha,
                                  const double* beta, const long long* lik_rowptr, const int* lik_col,
                                  const double* lik_val, const double* lik_R, const double* lik_T,
                                  const double* lik_scale, const int* arrow_variate, double tip_diag, double* D,
                                  double* L, double* R, double* T) {
  int b, nt, a;
  void* st;
  if (int r = gbta_geometry(s, &b, &nt, &a, &st)) return r;
  if (int r = kron_args_ok(b, ns, nv, nterms, upat_rowptr, upat_col, uval, term_vw)) return r;
  if (!D || (nt > 1 && !L) || (nterms > 0 && !alpha) || (nterms > 0 && nt > 1 && !beta))
    return gbta_set_error(GBTA_ERR_ARG, "assemble: null block or coefficient pointer");
  if (lik_rowptr && (!lik_col || !lik_val)) return gbta_set_error(GBTA_ERR_ARG, "assemble: incomplete A^T A CSR");
  if ((lik_rowptr || lik_R || lik_T) && !lik_scale)
    return gbta_set_error(GBTA_ERR_ARG, "assemble: A^T A given without lik_scale");
  if (a > 0 && (!R || !T)) return gbta_set_error(GBTA_ERR_ARG, "assemble: R/T required when a > 0");
  gbta::Geom g{b, nt, a, (b + gbta::TS - 1) / gbta::TS};
  gbta::KronDesc kd{ns, nv, nterms, upat_rowptr, upat_col, uval, term_vw};
  gbta::LikDesc ld{lik_rowptr, lik_col, lik_val, lik_R, lik_T, lik_scale, arrow_variate};
  cudaStream_t stream = (cudaStream_t)st;
  const long long rows = (long long)nt * b;
  const long long blocks = (rows + gbta::AS_WARPS - 1) / gbta::AS_WARPS;
  gbta::k_assemble_rows<<<(unsigned)blocks, gbta::AS_WARPS * 32, 0, stream>>>(g, kd, ld, alpha, beta, D, L);
  if (a > 0) gbta::k_assemble_arrow<<<256, 256, 0, stream>>>(g, ns, nv, ld, tip_diag, R, T);
  gbta::count_launches(1 + (a > 0));
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return gbta_set_error(GBTA_ERR_CUDA, cudaGetErrorString(e));
  return GBTA_OK;
}

extern "C" int gbta_contract_kron(gbta_solver* s, int ns, int nv, int nterms, const int* upat_rowptr,
                                  const int* upat_col, const double* uval, const int* term_vw,
                                  const long long* lik_rowptr, const int* lik_col, const double* lik_val,
                                  const double* lik_R, const double* lik_T, const int* arrow_variate,
                                  const double* SD, const double* SL, const double* SR, const double* ST,
                                  const double* mu, double* out) {
  int b, nt, a;
  void* st;
  if (int r = gbta_geometry(s, &b, &nt, &a, &st)) return r;
  if (int r = kron_args_ok(b, ns, nv, nterms, upat_rowptr, upat_col, uval, term_vw)) return r;
  if (!out) return gbta_set_error(GBTA_ERR_ARG, "contract: out is null");
  if (lik_rowptr && (!lik_col || !lik_val)) return gbta_set_error(GBTA_ERR_ARG, "contract: incomplete A^T A CSR");
  gbta::Geom g{b, nt, a, (b + gbta::TS - 1) / gbta::TS};
  gbta::KronDesc kd{ns, nv, nterms, upat_rowptr, upat_col, uval, term_vw};
  gbta::LikDesc ld{lik_rowptr, lik_col, lik_val, lik_R, lik_T, nullptr, arrow_variate};
  gbta::k_contract<<<nt + 1, gbta::CT_THREADS, 0, (cudaStream_t)st>>>(g, kd, ld, SD, SL, SR, ST, mu, out);
  gbta::count_launches(1);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return gbta_set_error(GBTA_ERR_CUDA, cudaGetErrorString(e));
  return GBTA_OK;
}
