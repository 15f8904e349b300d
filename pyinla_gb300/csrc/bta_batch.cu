// Many independent BTA instances (a gradient's, Hessian's or theta grid's Q(theta),
// possibly of different sizes) solved together: each phase -- factorization, solves,
// selected inversion -- of ALL instances runs as ONE persistent launch whose ticket
// dispenser hands out the tasks of every instance, merged into one list.  The
// reference evaluates such sets one Q(theta) at a time (src/pyinla/core/pyinla.py:
// 512-600 for the gradient's 2d+1 points, :747-910 for the Hessian); here the
// instances fill the GPU together: one instance's dataflow chain is latency-bound
// (a tile column waits on the previous one), many chains side by side are not.
//
// The merged list keeps every instance's own topological order, so a task still only
// waits for tasks with smaller tickets and the launch cannot deadlock.  Each instance
// has its own ready flags, workspace and pivot-failure slot; the ticket counter and
// the abort flag are shared.  The host sequence of one run contains no host
// synchronisation, so it can be captured once into a CUDA graph and replayed
// (gbta_batch_graph_launch): one graph launch then runs factor, logdet, solves and
// selected inversion of every instance.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <string>
#include <vector>

#include "../../include/pyinla_gb300.h"
#include "bta_factor_task.cuh"
#include "bta_selinv_task.cuh"
#include "bta_solve_task.cuh"

namespace gbta {

constexpr size_t BATCH_FACTOR_SMEM = OZF_SMEM > FP64F_SMEM ? OZF_SMEM : FP64F_SMEM;
constexpr size_t BATCH_SELINV_SMEM = OZS_SMEM > FP64S_SMEM ? OZS_SMEM : FP64S_SMEM;

// Ticket k runs task order[k].y of instance order[k].x, with that instance's method.
__global__ void __launch_bounds__(NT, 1) k_factor_batch(const FactorArgs* __restrict__ inst,
                                                        const int2* __restrict__ order, int ntotal, Ctl c) {
  extern __shared__ __align__(16) unsigned char raw[];
  __shared__ int s_ok, s_t, s_ready;
  __shared__ OzPipe pipe;
  oz_pipe_init(&pipe);
  const OzFactorSmem sm = oz_factor_smem(raw, &s_ok, &s_ready, &pipe);
  while (true) {
    const int t = cta_ticket(c, &s_t);
    if (t < 0 || t >= ntotal) break;
    const int2 o = order[t];
    const FactorArgs& p = inst[o.x];
    const bool ok = (p.method == GBTA_METHOD_OZAKI) ? factor_oz_task(p, o.y, sm) : factor_fp64_task(p, o.y, raw, &s_ok);
    if (!ok) break;
  }
}

__global__ void __launch_bounds__(NT, 1) k_selinv_batch(const SelinvArgs* __restrict__ inst,
                                                        const int2* __restrict__ order, int ntotal, Ctl c) {
  extern __shared__ __align__(16) unsigned char raw[];
  __shared__ int s_ok, s_t, s_ready;
  __shared__ OzPipe pipe;
  oz_pipe_init(&pipe);
  while (true) {
    const int t = cta_ticket(c, &s_t);
    if (t < 0 || t >= ntotal) break;
    const int2 o = order[t];
    const SelinvArgs& p = inst[o.x];
    const bool ok = (p.method == GBTA_METHOD_OZAKI) ? selinv_oz_task(p, o.y, raw, &s_ok, &s_ready, &pipe)
                                                    : selinv_fp64_task(p, o.y, raw, &s_ok);
    if (!ok) break;
  }
}

__global__ void __launch_bounds__(NT, 1) k_solve_batch(const SolveArgs* __restrict__ inst,
                                                       const int2* __restrict__ order, int ntotal, Ctl c) {
  __shared__ __align__(16) unsigned char raw[SOLVE_SMEM];
  __shared__ int s_ok, s_t;
  while (true) {
    const int t = cta_ticket(c, &s_t);
    if (t < 0 || t >= ntotal) break;
    const int2 o = order[t];
    if (!solve_task(inst[o.x], o.y, raw, &s_ok)) break;
  }
}

// Merge per-instance task lists (sizes n[k]) into one ticket order.
static std::vector<int2> merge_order(const std::vector<int>& n, int policy) {
  std::vector<int2> out;
  size_t total = 0;
  for (int v : n) total += (size_t)v;
  out.reserve(total);
  const int m = (int)n.size();
  if (policy == GBTA_BATCH_ORDER_SEQUENTIAL) {
    for (int k = 0; k < m; ++k)
      for (int j = 0; j < n[k]; ++j) out.push_back(make_int2(k, j));
  } else if (policy == GBTA_BATCH_ORDER_ROUND_ROBIN) {
    int maxn = 0;
    for (int v : n) maxn = std::max(maxn, v);
    for (int j = 0; j < maxn; ++j)
      for (int k = 0; k < m; ++k)
        if (j < n[k]) out.push_back(make_int2(k, j));
  } else {   // proportional: every instance advances at the same fraction of its list
    struct Key {
      double f;
      int k, j;
    };
    std::vector<Key> keys;
    keys.reserve(total);
    for (int k = 0; k < m; ++k)
      for (int j = 0; j < n[k]; ++j) keys.push_back({(j + 0.5) / n[k], k, j});
    std::stable_sort(keys.begin(), keys.end(), [](const Key& a, const Key& b) { return a.f < b.f; });
    for (const Key& q : keys) out.push_back(make_int2(q.k, q.j));
  }
  return out;
}

}  // namespace gbta

namespace {

constexpr int CTRL_INTS = 8;

int bfail(int code, const std::string& msg) { return gbta_set_error(code, msg.c_str()); }

#define BATCH_CUDA(call)                                                                   \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) return bfail(GBTA_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

struct BatchInst {
  gbta::Geom g;
  int method = GBTA_METHOD_OZAKI;
  size_t flags_off = 0;     // in ints, into the flag pool
  size_t faux_off = 0;      // in ints, into the feeder pool (flags [nt*B])
  int n_ftasks = 0, n_stasks = 0, n_vtasks = 0;
  // device workspace (inside the pool)
  int4* ftasks = nullptr;
  int4* stasks = nullptr;
  double* tip_part = nullptr;
  double* arrow_part = nullptr;
  double* ld = nullptr;       // logdet partials [nt + 1]
  double* sig = nullptr;      // Sigma workspace
  double* selws = nullptr;    // selected-inversion pre-pass (diagonal inverses)
  __half* digits = nullptr;   // Ozaki only
  int* erow = nullptr;        // Ozaki only
  __half* sdig = nullptr;     // Ozaki only: digit planes of the Sigma tiles
  int* tz = nullptr;          // Ozaki only: leading zero digit planes per tile slot
  // bound caller buffers
  double *D = nullptr, *L = nullptr, *R = nullptr, *T = nullptr, *rhs = nullptr;
};

size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

struct gbta_batch {
  int n = 0;
  int device = 0;
  int nsm = 0;
  std::vector<BatchInst> inst;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  unsigned long long wait_ns = 20ull * 1000 * 1000 * 1000;
  int policy = GBTA_BATCH_ORDER_PROPORTIONAL;
  int ctas_per_sm = 0;   // persistent CTAs per SM (0: as many as fit)
  int* d_ctrl = nullptr;
  int* d_info = nullptr;
  int* d_flags = nullptr;
  size_t nflags_total = 0;
  int* d_faux = nullptr;    // feeder "products done" flags of every instance
  size_t nfaux_total = 0;
  void* pool = nullptr;
  size_t pool_bytes = 0;
  int* h_ctrl = nullptr;   // pinned
  int* h_info = nullptr;   // pinned
  // per-phase argument arrays and ticket orders (device)
  gbta::FactorArgs* d_fargs = nullptr;
  gbta::SelinvArgs* d_sargs = nullptr;
  gbta::SolveArgs* d_vargs = nullptr;   // [2n]: forward sweeps, then backward sweeps
  int2* d_forder = nullptr;
  int2* d_sorder = nullptr;
  int2* d_vorder = nullptr;
  int n_forder = 0, n_sorder = 0, n_vorder = 0;
  bool bound = false;
  // captured run
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int graph_phases = -1;
  double* graph_logdet = nullptr;
  long long graph_launches = 0;
};

namespace {

int check_batch(const gbta_batch* bt) {
  if (!bt) return bfail(GBTA_ERR_ARG, "null batch");
  return GBTA_OK;
}

void drop_graph(gbta_batch* bt) {
  if (bt->gexec) cudaGraphExecDestroy(bt->gexec);
  if (bt->graph) cudaGraphDestroy(bt->graph);
  bt->gexec = nullptr;
  bt->graph = nullptr;
  bt->graph_phases = -1;
}

int upload_orders(gbta_batch* bt) {
  std::vector<int> nf, ns, nv;
  for (const BatchInst& q : bt->inst) {
    nf.push_back(q.n_ftasks);
    ns.push_back(q.n_stasks);
    nv.push_back(q.n_vtasks);
  }
  const std::vector<int2> fo = gbta::merge_order(nf, bt->policy), so = gbta::merge_order(ns, bt->policy),
                          vo = gbta::merge_order(nv, bt->policy);
  cudaFree(bt->d_forder);
  cudaFree(bt->d_sorder);
  cudaFree(bt->d_vorder);
  bt->d_forder = bt->d_sorder = bt->d_vorder = nullptr;
  BATCH_CUDA(cudaMalloc(&bt->d_forder, std::max<size_t>(fo.size(), 1) * sizeof(int2)));
  BATCH_CUDA(cudaMalloc(&bt->d_sorder, std::max<size_t>(so.size(), 1) * sizeof(int2)));
  BATCH_CUDA(cudaMalloc(&bt->d_vorder, std::max<size_t>(vo.size(), 1) * sizeof(int2)));
  BATCH_CUDA(cudaMemcpy(bt->d_forder, fo.data(), fo.size() * sizeof(int2), cudaMemcpyHostToDevice));
  BATCH_CUDA(cudaMemcpy(bt->d_sorder, so.data(), so.size() * sizeof(int2), cudaMemcpyHostToDevice));
  BATCH_CUDA(cudaMemcpy(bt->d_vorder, vo.data(), vo.size() * sizeof(int2), cudaMemcpyHostToDevice));
  bt->n_forder = (int)fo.size();
  bt->n_sorder = (int)so.size();
  bt->n_vorder = (int)vo.size();
  return GBTA_OK;
}

gbta::Ctl batch_ctl(const gbta_batch* bt, int* flags, int epoch) {
  gbta::Ctl c;
  c.ctrl = bt->d_ctrl;
  c.flags = flags;
  c.epoch = epoch << gbta::EPOCH_SHIFT;
  c.wait_ns = bt->wait_ns;
  c.trace = nullptr;
  return c;
}

// Phase epochs of one run (the flag pool is cleared at the start of every run).
constexpr int EP_FACTOR = 1, EP_SOLVE_N = 2, EP_SOLVE_C = 3, EP_SELINV = 4;

int build_args(gbta_batch* bt) {
  const int n = bt->n;
  std::vector<gbta::FactorArgs> fa(n);
  std::vector<gbta::SelinvArgs> sa(n);
  std::vector<gbta::SolveArgs> va(2 * n);
  for (int k = 0; k < n; ++k) {
    BatchInst& q = bt->inst[k];
    const gbta::Geom& g = q.g;
    int* flags = bt->d_flags + q.flags_off;
    const int use_arrow = g.a > 0;
    gbta::FactorArgs& f = fa[k];
    f.D = q.D;
    f.L = q.L;
    f.R = q.R;
    f.T = q.T;
    f.g = g;
    f.use_arrow = use_arrow;
    f.method = q.method;
    f.tasks = q.ftasks;
    f.ntasks = q.n_ftasks;
    f.tip_part = q.tip_part;
    f.digits = q.digits;
    f.erow = q.erow;
    f.info = bt->d_info + k;
    f.feed_pre = bt->d_faux + q.faux_off;
    f.diag_pre = bt->d_faux + q.faux_off + (size_t)g.nt * g.B;
    f.kf = g.nt > 1 ? bt->d_faux + q.faux_off + 3 * (size_t)g.nt * g.B : nullptr;
    f.c = batch_ctl(bt, flags, EP_FACTOR);
    gbta::SelinvArgs& s = sa[k];
    const size_t bb = (size_t)g.b * g.b;
    s.D = q.D;
    s.L = q.L;
    s.R = q.R;
    s.T = q.T;
    if (q.method == GBTA_METHOD_OZAKI) {   // Sigma over the factor (gbta_pobtasi does the same)
      s.SD = q.D;
      s.SL = q.L;
      s.SR = q.R;
      s.ST = q.T;
    } else {
      s.SD = q.sig;
      s.SL = q.sig + (size_t)g.nt * bb;
      s.SR = s.SL + (size_t)(g.nt - 1) * bb;
      s.ST = s.SR + (size_t)g.nt * g.a * g.b;
    }
    s.g = g;
    s.use_arrow = use_arrow;
    s.method = q.method;
    s.tasks = q.stasks;
    s.ntasks = q.n_stasks;
    s.fdig = q.digits;
    s.fdz = q.g.nflags() < (1 << 24) ? q.tz : nullptr;
    s.ecol = q.erow;
    s.sdig = q.sdig;
    s.merged = q.method == GBTA_METHOD_OZAKI;
    s.part = q.tip_part;                  // the factorization's tip partials are dead here
    s.part_flag = bt->d_faux + q.faux_off;
    s.cinv = q.selws + (size_t)g.nt * g.B * gbta::TS * gbta::TS;
    s.c = batch_ctl(bt, flags, EP_SELINV);
    for (int dir = 0; dir < 2; ++dir) {
      gbta::SolveArgs& v = va[dir * n + k];
      v.D = q.D;
      v.L = q.L;
      v.R = q.R;
      v.T = q.T;
      v.B = q.rhs;
      v.ldb = 1;
      v.nc = 1;
      v.g = g;
      v.use_arrow = use_arrow;
      v.trans = dir;
      v.part = q.arrow_part;
      v.ntasks = q.n_vtasks;
      v.both = 0;
      v.bflag0 = 0;
      v.c = batch_ctl(bt, flags, dir == 0 ? EP_SOLVE_N : EP_SOLVE_C);
    }
  }
  BATCH_CUDA(cudaMemcpy(bt->d_fargs, fa.data(), n * sizeof(gbta::FactorArgs), cudaMemcpyHostToDevice));
  BATCH_CUDA(cudaMemcpy(bt->d_sargs, sa.data(), n * sizeof(gbta::SelinvArgs), cudaMemcpyHostToDevice));
  BATCH_CUDA(cudaMemcpy(bt->d_vargs, va.data(), 2 * n * sizeof(gbta::SolveArgs), cudaMemcpyHostToDevice));
  return GBTA_OK;
}

int reset_ticket(gbta_batch* bt) {
  BATCH_CUDA(cudaMemsetAsync(bt->d_ctrl, 0, sizeof(int), bt->stream));
  return GBTA_OK;
}

int grid_of(const gbta_batch* bt, const void* kernel, size_t smem, int ntasks) {
  gbta::LaunchCtl lc;
  lc.grid = 1;
  lc.nsm = bt->nsm;
  lc.ctas_per_sm = bt->ctas_per_sm;
  lc.ntasks = ntasks;
  return gbta::launch_grid(kernel, gbta::NT, smem, lc);
}

int run_async(gbta_batch* bt, int phases, double* logdet_out) {
  if (!bt->bound) return bfail(GBTA_ERR_ARG, "batch: gbta_batch_bind must come first");
  if (phases & ~(GBTA_PHASE_FACTOR | GBTA_PHASE_LOGDET | GBTA_PHASE_SOLVE | GBTA_PHASE_SELINV))
    return bfail(GBTA_ERR_ARG, "batch: unknown phase bits");
  if ((phases & GBTA_PHASE_LOGDET) && !logdet_out) return bfail(GBTA_ERR_ARG, "batch: logdet output required");
  if (phases & GBTA_PHASE_SOLVE)
    for (const BatchInst& q : bt->inst)
      if (!q.rhs) return bfail(GBTA_ERR_ARG, "batch: solve phase needs every instance's rhs");
  cudaStream_t st = bt->stream;
  BATCH_CUDA(cudaMemsetAsync(bt->d_ctrl, 0, CTRL_INTS * sizeof(int), st));
  BATCH_CUDA(cudaMemsetAsync(bt->d_info, 0, bt->n * sizeof(int), st));
  BATCH_CUDA(cudaMemsetAsync(bt->d_flags, 0, bt->nflags_total * sizeof(int), st));
  BATCH_CUDA(cudaMemsetAsync(bt->d_faux, 0, bt->nfaux_total * sizeof(int), st));
  const gbta::Ctl c = batch_ctl(bt, nullptr, 0);
  if (phases & GBTA_PHASE_FACTOR) {
    for (const BatchInst& q : bt->inst)
      if (q.g.nt > 1) {
        gbta::launch_transpose_lslots(q.g, q.L, st);
        gbta::launch_coupling_kfirst(q.g, q.L, bt->d_faux + q.faux_off + 3 * (size_t)q.g.nt * q.g.B, st);
      }
    for (const BatchInst& q : bt->inst)
      if (q.method == GBTA_METHOD_OZAKI) gbta::launch_row_exponents(q.g, q.D, q.T, q.g.a > 0, q.erow, st);
    gbta::k_factor_batch<<<grid_of(bt, (const void*)gbta::k_factor_batch, gbta::BATCH_FACTOR_SMEM, bt->n_forder), gbta::NT,
                            gbta::BATCH_FACTOR_SMEM, st>>>(
        bt->d_fargs, bt->d_forder, bt->n_forder, c);
    gbta::count_launches(1);
    BATCH_CUDA(cudaGetLastError());
  }
  if (phases & GBTA_PHASE_LOGDET) {
    for (int k = 0; k < bt->n; ++k) {
      const BatchInst& q = bt->inst[k];
      gbta::launch_logdet(q.g, q.D, q.T, q.g.a > 0, q.ld, logdet_out + k, st);
    }
    BATCH_CUDA(cudaGetLastError());
  }
  if (phases & GBTA_PHASE_SOLVE) {
    for (int dir = 0; dir < 2; ++dir) {
      if (int r = reset_ticket(bt)) return r;
      gbta::k_solve_batch<<<grid_of(bt, (const void*)gbta::k_solve_batch, 0, bt->n_vorder), gbta::NT, 0, st>>>(bt->d_vargs + dir * bt->n, bt->d_vorder,
                                                                            bt->n_vorder, c);
      gbta::count_launches(1);
      BATCH_CUDA(cudaGetLastError());
    }
  }
  if (phases & GBTA_PHASE_SELINV) {
    // tensor-core G tiles from the digit planes this run's factorization left
    for (const BatchInst& q : bt->inst) {
      const bool tc_g = q.method == GBTA_METHOD_OZAKI && (phases & GBTA_PHASE_FACTOR);
      const int* kf = q.g.nt > 1 ? bt->d_faux + q.faux_off + 3 * (size_t)q.g.nt * q.g.B : nullptr;
      gbta::launch_selinv_prepare(q.g, q.D, q.L, q.R, q.g.a > 0, q.selws, st, tc_g ? q.digits : nullptr, q.erow, kf);
    }
    for (const BatchInst& q : bt->inst)
      if (q.method == GBTA_METHOD_OZAKI)
        gbta::launch_selinv_oz_prepare(q.g, q.D, q.L, q.R, q.g.a > 0, q.digits, q.erow,
                                       q.g.nflags() < (1 << 24) ? q.tz : nullptr, st);
    if (int r = reset_ticket(bt)) return r;
    gbta::k_selinv_batch<<<grid_of(bt, (const void*)gbta::k_selinv_batch, gbta::BATCH_SELINV_SMEM, bt->n_sorder), gbta::NT,
                            gbta::BATCH_SELINV_SMEM, st>>>(
        bt->d_sargs, bt->d_sorder, bt->n_sorder, c);
    gbta::count_launches(1);
    for (const BatchInst& q : bt->inst) {
      const gbta::Geom& g = q.g;
      if (q.method == GBTA_METHOD_OZAKI) {
        gbta::launch_selinv_finish_inplace(g, q.D, q.L, st);
        continue;
      }
      const size_t bb = (size_t)g.b * g.b;
      double* SD = q.sig;
      double* SL = SD + (size_t)g.nt * bb;
      double* SR = SL + (size_t)(g.nt - 1) * bb;
      double* ST = SR + (size_t)g.nt * g.a * g.b;
      gbta::launch_selinv_writeback(g, SD, SL, SR, ST, q.D, q.L, q.R, q.T, g.a > 0, st);
    }
    BATCH_CUDA(cudaGetLastError());
  }
  return GBTA_OK;
}

}  // namespace

extern "C" {

int gbta_batch_create(int n, const int* b, const int* nt, const int* a, const int* methods, gbta_batch** out) {
  if (!out) return bfail(GBTA_ERR_ARG, "batch: out is null");
  *out = nullptr;
  if (n < 1 || !b || !nt || !a) return bfail(GBTA_ERR_ARG, "batch: need n >= 1 and b, nt, a arrays");
  for (int k = 0; k < n; ++k) {
    if (b[k] < 1 || nt[k] < 1 || a[k] < 0 || a[k] > gbta::TS)
      return bfail(GBTA_ERR_ARG, "batch: instance " + std::to_string(k) + " needs b >= 1, nt >= 1, 0 <= a <= 32");
    if (methods && methods[k] != GBTA_METHOD_FP64 && methods[k] != GBTA_METHOD_OZAKI)
      return bfail(GBTA_ERR_ARG, "batch: unknown method for instance " + std::to_string(k));
    const gbta::Geom g{b[k], nt[k], a[k], (b[k] + gbta::TS - 1) / gbta::TS};
    if ((long long)(2 * g.nt - 1) * g.B * g.B + (long long)g.nt * g.B + 1 > 0x7fffffffll)
      return bfail(GBTA_ERR_ARG, "batch: instance " + std::to_string(k) + " is too large");
  }
  gbta_batch* bt = new gbta_batch();
  bt->n = n;
  bt->inst.resize(n);
#define CREATE_CUDA(call)                                                                     \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess) {                                                                  \
      const int r_ = bfail(GBTA_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
      gbta_batch_destroy(bt);                                                                 \
      return r_;                                                                              \
    }                                                                                         \
  } while (0)
  CREATE_CUDA(cudaGetDevice(&bt->device));
  CREATE_CUDA(cudaDeviceGetAttribute(&bt->nsm, cudaDevAttrMultiProcessorCount, bt->device));
  if (const char* v = std::getenv("GBTA_WAIT_LIMIT_MS")) {
    const double ms = std::atof(v);
    if (ms > 0.0) bt->wait_ns = (unsigned long long)(ms * 1e6);
  }
  CREATE_CUDA(cudaStreamCreateWithFlags(&bt->own_stream, cudaStreamNonBlocking));
  bt->stream = bt->own_stream;
  // ---- plan the pool
  size_t off = 0, flags_total = 0;
  std::vector<std::vector<int4>> ft(n), st(n);
  std::vector<size_t> o_ft(n), o_st(n), o_tip(n), o_arw(n), o_ld(n), o_sig(n), o_sel(n), o_dig(n), o_erow(n),
      o_sdig(n), o_tz(n);
  for (int k = 0; k < n; ++k) {
    BatchInst& q = bt->inst[k];
    q.g = gbta::Geom{b[k], nt[k], a[k], (b[k] + gbta::TS - 1) / gbta::TS};
    q.g.m = gbta::default_sep(nt[k]);   // the single-instance solver's elimination order
    q.method = methods ? methods[k] : GBTA_METHOD_OZAKI;
    const gbta::Geom& g = q.g;
    ft[k] = gbta::factor_task_list(g);
    st[k] = gbta::selinv_task_list(g, q.method == GBTA_METHOD_OZAKI);
    q.n_ftasks = (int)ft[k].size();
    q.n_stasks = (int)st[k].size();
    q.n_vtasks = g.nt * g.B + (g.a > 0 ? 1 : 0);
    q.flags_off = flags_total;
    q.faux_off = bt->nfaux_total;
    // feeder flags, diagonal- and feeder-partial flags, then the coupling slots' kfirst
    bt->nfaux_total += 3 * (size_t)g.nt * g.B + (size_t)(g.nt - 1) * g.B;
    flags_total += (size_t)g.nflags();
    const size_t ntile = (size_t)g.nt * g.B, bb = (size_t)g.b * g.b;
    o_ft[k] = off;
    off = align_up(off + ft[k].size() * sizeof(int4));
    o_st[k] = off;
    off = align_up(off + st[k].size() * sizeof(int4));
    o_tip[k] = off;
    off = align_up(off + ntile * gbta::TS * gbta::TS * sizeof(double));
    o_arw[k] = off;
    off = align_up(off + ntile * gbta::TS * gbta::SOLVE_NC * sizeof(double));
    o_ld[k] = off;
    off = align_up(off + (g.nt + 2) * sizeof(double));
    o_sig[k] = off;   // Sigma workspace: FP64 method only (the tensor-core method writes in place)
    if (q.method != GBTA_METHOD_OZAKI)
      off = align_up(off + (g.nt * bb + (g.nt - 1) * bb + (size_t)g.nt * g.a * g.b + (size_t)g.a * g.a) *
                               sizeof(double));
    o_sel[k] = off;
    off = align_up(off + gbta::selinv_prepare_bytes(g));
    o_dig[k] = o_erow[k] = o_sdig[k] = o_tz[k] = 0;
    if (q.method == GBTA_METHOD_OZAKI) {
      o_dig[k] = off;
      off = align_up(off + gbta::factor_oz_digit_bytes(g));
      o_erow[k] = off;
      off = align_up(off + ((size_t)g.nt * g.b + g.a) * sizeof(int));
      o_sdig[k] = off;
      off = align_up(off + gbta::selinv_oz_digit_bytes(g));
      o_tz[k] = off;
      off = align_up(off + (size_t)g.nflags() * sizeof(int));
    }
  }
  bt->pool_bytes = off;
  bt->nflags_total = flags_total;
  CREATE_CUDA(cudaMalloc(&bt->pool, off));
  CREATE_CUDA(cudaMalloc(&bt->d_flags, flags_total * sizeof(int)));
  CREATE_CUDA(cudaMalloc(&bt->d_faux, bt->nfaux_total * sizeof(int)));
  CREATE_CUDA(cudaMalloc(&bt->d_ctrl, CTRL_INTS * sizeof(int)));
  CREATE_CUDA(cudaMalloc(&bt->d_info, n * sizeof(int)));
  CREATE_CUDA(cudaMallocHost(&bt->h_ctrl, CTRL_INTS * sizeof(int)));
  CREATE_CUDA(cudaMallocHost(&bt->h_info, n * sizeof(int)));
  CREATE_CUDA(cudaMalloc(&bt->d_fargs, n * sizeof(gbta::FactorArgs)));
  CREATE_CUDA(cudaMalloc(&bt->d_sargs, n * sizeof(gbta::SelinvArgs)));
  CREATE_CUDA(cudaMalloc(&bt->d_vargs, 2 * n * sizeof(gbta::SolveArgs)));
  char* base = static_cast<char*>(bt->pool);
  for (int k = 0; k < n; ++k) {
    BatchInst& q = bt->inst[k];
    q.ftasks = reinterpret_cast<int4*>(base + o_ft[k]);
    q.stasks = reinterpret_cast<int4*>(base + o_st[k]);
    q.tip_part = reinterpret_cast<double*>(base + o_tip[k]);
    q.arrow_part = reinterpret_cast<double*>(base + o_arw[k]);
    q.ld = reinterpret_cast<double*>(base + o_ld[k]);
    q.sig = reinterpret_cast<double*>(base + o_sig[k]);
    q.selws = reinterpret_cast<double*>(base + o_sel[k]);
    if (q.method == GBTA_METHOD_OZAKI) {
      q.digits = reinterpret_cast<__half*>(base + o_dig[k]);
      q.erow = reinterpret_cast<int*>(base + o_erow[k]);
      q.sdig = reinterpret_cast<__half*>(base + o_sdig[k]);
      q.tz = reinterpret_cast<int*>(base + o_tz[k]);
    }
    CREATE_CUDA(cudaMemcpy(q.ftasks, ft[k].data(), ft[k].size() * sizeof(int4), cudaMemcpyHostToDevice));
    CREATE_CUDA(cudaMemcpy(q.stasks, st[k].data(), st[k].size() * sizeof(int4), cudaMemcpyHostToDevice));
  }
  if (upload_orders(bt) != GBTA_OK) {
    gbta_batch_destroy(bt);
    return GBTA_ERR_CUDA;
  }
  CREATE_CUDA(cudaFuncSetAttribute(gbta::k_factor_batch, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)gbta::BATCH_FACTOR_SMEM));
  CREATE_CUDA(cudaFuncSetAttribute(gbta::k_selinv_batch, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)gbta::BATCH_SELINV_SMEM));
  // the largest shared-memory carveout, so that two CTAs fit on an SM
  CREATE_CUDA(cudaFuncSetAttribute(gbta::k_factor_batch, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  CREATE_CUDA(cudaFuncSetAttribute(gbta::k_solve_batch, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  CREATE_CUDA(cudaFuncSetAttribute(gbta::k_selinv_batch, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
#undef CREATE_CUDA
  *out = bt;
  return GBTA_OK;
}

int gbta_batch_destroy(gbta_batch* bt) {
  if (!bt) return GBTA_OK;
  if (bt->stream) cudaStreamSynchronize(bt->stream);
  drop_graph(bt);
  cudaFree(bt->pool);
  cudaFree(bt->d_flags);
  cudaFree(bt->d_faux);
  cudaFree(bt->d_ctrl);
  cudaFree(bt->d_info);
  cudaFree(bt->d_fargs);
  cudaFree(bt->d_sargs);
  cudaFree(bt->d_vargs);
  cudaFree(bt->d_forder);
  cudaFree(bt->d_sorder);
  cudaFree(bt->d_vorder);
  if (bt->h_ctrl) cudaFreeHost(bt->h_ctrl);
  if (bt->h_info) cudaFreeHost(bt->h_info);
  if (bt->own_stream) cudaStreamDestroy(bt->own_stream);
  delete bt;
  return GBTA_OK;
}

size_t gbta_batch_workspace_bytes(const gbta_batch* bt) {
  return bt ? bt->pool_bytes + (bt->nflags_total + bt->nfaux_total) * sizeof(int) : 0;
}

int gbta_batch_set_stream(gbta_batch* bt, void* stream) {
  if (int r = check_batch(bt)) return r;
  if ((cudaStream_t)stream != bt->stream) drop_graph(bt);
  bt->stream = (cudaStream_t)stream;
  return GBTA_OK;
}

int gbta_batch_set_order(gbta_batch* bt, int policy) {
  if (int r = check_batch(bt)) return r;
  if (policy != GBTA_BATCH_ORDER_PROPORTIONAL && policy != GBTA_BATCH_ORDER_ROUND_ROBIN &&
      policy != GBTA_BATCH_ORDER_SEQUENTIAL)
    return bfail(GBTA_ERR_ARG, "batch: unknown order policy");
  if (policy == bt->policy) return GBTA_OK;
  BATCH_CUDA(cudaStreamSynchronize(bt->stream));
  drop_graph(bt);
  bt->policy = policy;
  return upload_orders(bt);
}

int gbta_batch_set_ctas_per_sm(gbta_batch* bt, int n) {
  if (int r = check_batch(bt)) return r;
  if (n < 0 || n > 8) return bfail(GBTA_ERR_ARG, "batch: ctas_per_sm must be in [0, 8]");
  if (n != bt->ctas_per_sm) drop_graph(bt);
  bt->ctas_per_sm = n;
  return GBTA_OK;
}

int gbta_batch_set_wait_limit_ms(gbta_batch* bt, double ms) {
  if (int r = check_batch(bt)) return r;
  if (!(ms > 0)) return bfail(GBTA_ERR_ARG, "wait limit must be positive");
  bt->wait_ns = (unsigned long long)(ms * 1e6);
  if (bt->bound) {
    BATCH_CUDA(cudaStreamSynchronize(bt->stream));
    drop_graph(bt);
    return build_args(bt);
  }
  return GBTA_OK;
}

int gbta_batch_bind(gbta_batch* bt, double* const* D, double* const* L, double* const* R, double* const* T,
                    double* const* rhs) {
  if (int r = check_batch(bt)) return r;
  if (!D || !L) return bfail(GBTA_ERR_ARG, "batch: D and L pointer arrays are required");
  for (int k = 0; k < bt->n; ++k) {
    const gbta::Geom& g = bt->inst[k].g;
    if (!D[k] || (g.nt > 1 && !L[k])) return bfail(GBTA_ERR_ARG, "batch: null D/L for instance " + std::to_string(k));
    if (g.a > 0 && (!R || !T || !R[k] || !T[k]))
      return bfail(GBTA_ERR_ARG, "batch: R/T required for instance " + std::to_string(k));
  }
  BATCH_CUDA(cudaStreamSynchronize(bt->stream));
  drop_graph(bt);
  for (int k = 0; k < bt->n; ++k) {
    BatchInst& q = bt->inst[k];
    q.D = D[k];
    q.L = L[k];
    q.R = (q.g.a > 0) ? R[k] : nullptr;
    q.T = (q.g.a > 0) ? T[k] : nullptr;
    q.rhs = rhs ? rhs[k] : nullptr;
  }
  if (int r = build_args(bt)) return r;
  bt->bound = true;
  return GBTA_OK;
}

int gbta_batch_run_async(gbta_batch* bt, int phases, double* logdet_out) {
  if (int r = check_batch(bt)) return r;
  return run_async(bt, phases, logdet_out);
}

int gbta_batch_graph_launch(gbta_batch* bt, int phases, double* logdet_out) {
  if (int r = check_batch(bt)) return r;
  if (!bt->stream) return bfail(GBTA_ERR_ARG, "batch: graph launches need a non-default stream");
  if (!bt->gexec || bt->graph_phases != phases || bt->graph_logdet != logdet_out) {
    drop_graph(bt);
    const long long l0 = gbta_kernel_launches();
    BATCH_CUDA(cudaStreamBeginCapture(bt->stream, cudaStreamCaptureModeThreadLocal));
    const int r = run_async(bt, phases, logdet_out);
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(bt->stream, &graph);
    const long long captured = gbta_kernel_launches() - l0;
    gbta::count_launches(-(int)captured);   // nothing ran yet
    if (r != GBTA_OK) {
      if (graph) cudaGraphDestroy(graph);
      return r;
    }
    if (e != cudaSuccess) return bfail(GBTA_ERR_CUDA, std::string("stream capture: ") + cudaGetErrorString(e));
    bt->graph = graph;
    BATCH_CUDA(cudaGraphInstantiate(&bt->gexec, graph, 0));
    bt->graph_phases = phases;
    bt->graph_logdet = logdet_out;
    bt->graph_launches = captured;
  }
  BATCH_CUDA(cudaGraphLaunch(bt->gexec, bt->stream));
  gbta::count_launches((int)bt->graph_launches);
  return GBTA_OK;
}

long long gbta_batch_graph_kernels(const gbta_batch* bt) { return bt ? bt->graph_launches : 0; }

int gbta_batch_status(gbta_batch* bt, int* info) {
  if (int r = check_batch(bt)) return r;
  BATCH_CUDA(cudaStreamSynchronize(bt->stream));
  BATCH_CUDA(cudaGetLastError());
  BATCH_CUDA(cudaMemcpy(bt->h_ctrl, bt->d_ctrl, CTRL_INTS * sizeof(int), cudaMemcpyDeviceToHost));
  BATCH_CUDA(cudaMemcpy(bt->h_info, bt->d_info, bt->n * sizeof(int), cudaMemcpyDeviceToHost));
  if (info)
    for (int k = 0; k < bt->n; ++k) info[k] = bt->h_info[k];
  if (bt->h_ctrl[gbta::CTRL_ERR] == gbta::ERR_TIMEOUT)
    return bfail(GBTA_ERR_TIMEOUT, "batch: a kernel wait exceeded the wait limit; the launch was abandoned");
  for (int k = 0; k < bt->n; ++k)
    if (bt->h_info[k] > 0)
      return bfail(bt->h_info[k], "batch: instance " + std::to_string(k) +
                                      " is not positive definite (non-positive pivot at row " +
                                      std::to_string(bt->h_info[k]) + ")");
  return GBTA_OK;
}

}  // extern "C"
