// C ABI of the GB300 BTA solver (declared in include/pyinla_gb300.h).
//
// A gbta_solver plays the role of the reference's SerinvSolver object
// (src/pyinla/solvers/structured_solver.py:19-70) without the block buffers, which
// the caller owns: it holds the geometry, the device workspace of the dataflow
// kernels (tile flags, task lists, partial buffers, the selected-inversion output
// blocks) and the stream the work is enqueued on.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pyinla_gb300.h"
#include "bta_internal.h"

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

#define GBTA_CUDA(call)                                                                   \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return fail(GBTA_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));   \
  } while (0)

constexpr int CTRL_INTS = 8;
constexpr int CTRL_INFO = 2, CTRL_ERR = 3;   // sticky status words of the control block
constexpr int CTRL_MMA = 4;                  // words 4-5: the launch's tile-pair product count

}  // namespace

struct gbta_solver {
  gbta::Geom g;
  int device = 0;
  int nsm = 0;
  int ctas_per_sm = 0;   // persistent CTAs per SM (0: as many as fit)
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  unsigned long long wait_ns = 20ull * 1000 * 1000 * 1000;
  int epoch = 0;

  int* d_ctrl = nullptr;
  int* d_flags = nullptr;
  int4* d_ftasks = nullptr;
  int n_ftasks = 0;
  int4* d_stasks = nullptr;    // selected-inversion tasks (FP64 method)
  int4* d_stasks_m = nullptr;  // merged list of the tensor-core method (same count)
  int n_stasks = 0;
  double* d_tip_part = nullptr;
  double* d_arrow_part = nullptr;
  int* d_faux = nullptr;      // feeder "products done" flags [nt*B]
  int* d_dpre = nullptr;      // diagonal and feeder tiles' "partial stored" flags [2*nt*B]
  int* d_kf = nullptr;        // first nonzero column tile per coupling-slot row tile [(nt-1)*B]
  bool fac_digits = false;    // d_digits holds the digit planes of the current factor
  // Overlapped selected inversion (gbta_set_selinv_overlap): the inversion runs on a
  // second stream from the factorization's completion, next to the sweeps enqueued after
  // it, with its own control block and flags, into the Sigma workspace; the write-back
  // into the caller's blocks comes on the solver's stream after both.
  bool overlap = false;
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fac = nullptr;   // the last factorization's completion (solver's stream)
  cudaEvent_t ev_sel = nullptr;   // the overlapped inversion's completion (side stream)
  cudaEvent_t ev_swp = nullptr;   // the last sweeps' completion (solver's stream)
  bool fac_evt = false;           // ev_fac belongs to the factor the blocks hold
  bool swept = false;             // sweeps were enqueued since that factorization
  int* d_ctrl2 = nullptr;         // control block of the side stream's launches
  int* d_flags2 = nullptr;        // their ready flags
  double* d_ld = nullptr;   // logdet partials [nt + 1] + result [1]
  double* d_sig = nullptr;  // selected-inversion output blocks (lazy)
  double* d_selws = nullptr;  // selected-inversion pre-pass: diagonal inverses (lazy)
  size_t sig_elems = 0;
  int* h_ctrl = nullptr;    // pinned
  size_t ws_bytes = 0;
  int method = GBTA_METHOD_OZAKI;  // how tile products are computed in the factorization
  void* d_digits = nullptr;         // Ozaki digit planes (lazy)
  void* d_sdig = nullptr;           // Ozaki digit planes of the Sigma tiles (lazy)
  int* d_erow = nullptr;            // Ozaki row exponents (lazy)
  int* d_tz = nullptr;              // Ozaki: leading zero digit planes per tile slot (lazy)
  size_t digit_bytes = 0;
  long long* d_trace = nullptr;   // task trace of the last launch (when enabled)
  long long trace_cap = 0;        // records
  long long trace_n = 0;          // records of the last traced launch
  // Kernel timing (off by default): CUDA events around the dataflow launch of the last
  // factorization [0, 1], selected inversion [2, 3] and solve call [4, 5].
  bool timing = false;
  cudaEvent_t tev[6] = {};
  bool timed[3] = {false, false, false};
  long long* h_pairs = nullptr;   // pinned: tile-pair products of the last timed factor, selinv
};

namespace gbta {

// Task lists in a topological order of the dataflow DAGs (each task only waits for
// tasks earlier in the list, so the ticket dispenser cannot deadlock).
// Per block column (i, c): the feeder's products (they do not need the diagonal tile,
// so they come first), the diagonal tile, the feeder's row groups (triangular solves
// split over FEED_ROWS-row tasks, so that the solve on the critical path of the
// factorization runs on several SMs), the other tiles of the column.  The columns of
// the two chains of the elimination order (Geom) are interleaved one for one, so that
// the CTAs holding the earliest tickets serve both chains; then the separator's
// columns, then the tip.
// With diag_split, the products of diagonal tile (i, c) and of the feeder of column c,
// except their last step(s), form FT_PART tasks at the end of column c-2's group (their
// last operands before the last step are OFFD tasks of that group); column 1's, which
// have only the neighbour blocks' terms, open column 0's group; a block's first column's
// close column B-2's group of the block before it in the chain (the separator, with two
// neighbours, opens its own first group).  The diagonal and feeder tasks themselves
// become FT_TAIL tasks.
static void column_partials(const Geom& g, int i, int c, std::vector<int4>& t) {
  if (diag_has_partial(g, i, c)) t.push_back(make_int4(FT_DIAG | FT_PART, i, c, c));
  const int fk = g.feeder_kind(i, c);
  if (feeder_has_partial(g, i, c)) {
    if (fk == 1) t.push_back(make_int4(FT_OFFD | FT_PRE | FT_PART, i, c + 1, c));
    else t.push_back(make_int4(FT_LOW | FT_PRE | FT_PART, i, 0, c));
  }
}

static void factor_column_tasks(const Geom& g, int i, int c, bool split, std::vector<int4>& t) {
  const int fk = g.feeder_kind(i, c);
  if (split && c == 0 && g.nprev(i) > 1) column_partials(g, i, 0, t);
  if (split && c == 0 && g.B >= 2) column_partials(g, i, 1, t);
  const int ftail = (split && feeder_has_partial(g, i, c)) ? FT_TAIL : 0;
  if (fk == 1) t.push_back(make_int4(FT_OFFD | FT_PRE | ftail, i, c + 1, c));
  if (fk == 2) t.push_back(make_int4(FT_LOW | FT_PRE | ftail, i, 0, c));
  t.push_back(make_int4(FT_DIAG | (split && diag_has_partial(g, i, c) ? FT_TAIL : 0), i, c, c));
  for (int q = 0; q < g.feeder_quarters(i, c); ++q) t.push_back(make_int4(FT_FEEDQ, i, q, c));
  for (int r = c + 1 + (fk == 1 ? 1 : 0); r < g.B; ++r) t.push_back(make_int4(FT_OFFD, i, r, c));
  if (g.nxt(i) >= 0)
    for (int r = (fk == 2 ? 1 : 0); r < g.B; ++r) t.push_back(make_int4(FT_LOW, i, r, c));
  if (g.a > 0) t.push_back(make_int4(FT_ARW, i, 0, c));
  if (split && c + 2 < g.B) column_partials(g, i, c + 2, t);
  // the next block of the chain (the one whose only earlier neighbour is i)
  const int n = g.nxt(i);
  if (split && n >= 0 && g.nprev(n) == 1 && c == (g.B >= 2 ? g.B - 2 : 0)) column_partials(g, n, 0, t);
}

std::vector<int4> factor_task_list(const Geom& g, bool diag_split) {
  std::vector<int4> t;
  const int s = g.sep(), n1 = s * g.B, n2 = (g.nt - 1 - s) * g.B;
  for (int u = 0; u < n1 + n2; ++u) {
    int k;
    const int i = Geom::interleave(n1, n2, u, &k) == 0 ? k / g.B : g.nt - 1 - k / g.B;
    factor_column_tasks(g, i, k % g.B, diag_split, t);
  }
  for (int c = 0; c < g.B; ++c) factor_column_tasks(g, s, c, diag_split, t);
  if (g.a > 0) t.push_back(make_int4(FT_TIP, 0, 0, 0));
  return t;
}

// Merged form (tensor-core method): the column chain of the inversion runs diagonal
// tile -> sub-diagonal tile of the next column -> its diagonal tile -> ...; the
// sub-diagonal tile's last product needs the diagonal tile just finished, so the
// diagonal task finishes it itself, from the partial sum of its other products that
// an ST_PART task (placed before that diagonal task) leaves.  The next column after
// (i, 0) is (prev(i, 0), B-1); the separator has two such columns (one per chain), and
// their sub-diagonal tiles are computed by ordinary tasks.
// Order: the tip, the separator's columns from the last, then the columns of the two
// chains outwards from the separator, interleaved one for one.
static void selinv_column_tasks(const Geom& g, int i, int c, bool merged, std::vector<int4>& t) {
  const int B = g.B;
  auto sub_code = [&](int bi, int bc) {
    if (bc + 1 < B) return bc + 1;
    const int n = g.nxt(bi);
    return (n >= 0 && g.nprev(n) == 1) ? B : -1;
  };
  const int sub = merged ? sub_code(i, c) : -1;
  if (g.a > 0) t.push_back(make_int4(ST_OFF, i, 2 * B, c));
  if (g.nxt(i) >= 0)
    for (int r = 0; r < B; ++r)
      if (B + r != sub) t.push_back(make_int4(ST_OFF, i, B + r, c));
  for (int r = c + 1; r < B; ++r)
    if (r != sub) t.push_back(make_int4(ST_OFF, i, r, c));
  if (merged) {   // the partial of the next column's sub-diagonal tile
    if (c > 0) t.push_back(make_int4(ST_PART, i, c, c - 1));
    else if (g.nprev(i) == 1) t.push_back(make_int4(ST_PART, g.prev(i, 0), B, B - 1));
  }
  t.push_back(make_int4(ST_DIAG, i, c, c));
}

std::vector<int4> selinv_task_list(const Geom& g, bool merged) {
  std::vector<int4> t;
  const int B = g.B, s = g.sep(), n1 = s * B, n2 = (g.nt - 1 - s) * B;
  if (g.a > 0) t.push_back(make_int4(ST_TIP, 0, 0, 0));
  for (int c = B - 1; c >= 0; --c) selinv_column_tasks(g, s, c, merged, t);
  for (int u = 0; u < n1 + n2; ++u) {
    int k;
    const int i = Geom::interleave(n1, n2, u, &k) == 0 ? s - 1 - k / B : s + 1 + k / B;
    selinv_column_tasks(g, i, B - 1 - k % B, merged, t);
  }
  return t;
}

}  // namespace gbta

namespace {

gbta::LaunchCtl next_launch(gbta_solver* s, int ntasks) {
  gbta::LaunchCtl lc;
  s->epoch += 1;
  if (s->epoch >= (1 << (31 - gbta::EPOCH_SHIFT)) - 1) {   // wrap: clear every epoch-stamped word
    cudaMemsetAsync(s->d_flags, 0, (size_t)s->g.nflags() * sizeof(int), s->stream);
    cudaMemsetAsync(s->d_faux, 0, (size_t)s->g.nt * s->g.B * sizeof(int), s->stream);
    cudaMemsetAsync(s->d_dpre, 0, 2 * (size_t)s->g.nt * s->g.B * sizeof(int), s->stream);
    s->epoch = 1;
  }
  lc.ctrl = s->d_ctrl;
  lc.flags = s->d_flags;
  lc.epoch = s->epoch << gbta::EPOCH_SHIFT;
  lc.wait_ns = s->wait_ns;
  lc.grid = 0;
  lc.nsm = s->nsm;
  lc.ctas_per_sm = s->ctas_per_sm;
  lc.ntasks = ntasks;
  lc.stream = s->stream;
  if (s->d_trace && ntasks <= s->trace_cap) {
    lc.trace = s->d_trace;
    s->trace_n = ntasks;
  }
  return lc;
}

// The same for a launch on the side stream (overlapped inversion).
gbta::LaunchCtl next_side_launch(gbta_solver* s, int ntasks) {
  const int e0 = s->epoch;
  gbta::LaunchCtl lc = next_launch(s, ntasks);
  if (s->epoch < e0)   // the epoch counter wrapped: the side flags start over too
    cudaMemsetAsync(s->d_flags2, 0, (size_t)s->g.nflags() * sizeof(int), s->side);
  lc.ctrl = s->d_ctrl2;
  lc.flags = s->d_flags2;
  lc.stream = s->side;
  return lc;
}

// Reset the ticket counter and the abort flag of the next launch (not the sticky
// status words).
int reset_ticket(gbta_solver* s) {
  GBTA_CUDA(cudaMemsetAsync(s->d_ctrl, 0, 2 * sizeof(int), s->stream));
  if (s->timing) GBTA_CUDA(cudaMemsetAsync(s->d_ctrl + CTRL_MMA, 0, sizeof(long long), s->stream));
  return GBTA_OK;
}
int reset_side_ticket(gbta_solver* s) {
  GBTA_CUDA(cudaMemsetAsync(s->d_ctrl2, 0, 2 * sizeof(int), s->side));
  if (s->timing) GBTA_CUDA(cudaMemsetAsync(s->d_ctrl2 + CTRL_MMA, 0, sizeof(long long), s->side));
  return GBTA_OK;
}

int check_solver(const gbta_solver* s) {
  if (!s) return fail(GBTA_ERR_ARG, "null solver");
  return GBTA_OK;
}

}  // namespace

extern "C" {

int gbta_version(void) { return 100; }

int gbta_set_error(int code, const char* msg) { return fail(code, msg ? msg : ""); }

int gbta_geometry(const gbta_solver* s, int* b, int* nt, int* a, void** stream) {
  if (!s) return fail(GBTA_ERR_ARG, "null solver");
  if (b) *b = s->g.b;
  if (nt) *nt = s->g.nt;
  if (a) *a = s->g.a;
  if (stream) *stream = (void*)s->stream;
  return GBTA_OK;
}

const char* gbta_last_error(void) { return g_last_error.c_str(); }

int gbta_create(int b, int nt, int a, gbta_solver** out) {
  if (!out) return fail(GBTA_ERR_ARG, "out is null");
  *out = nullptr;
  if (b < 1 || nt < 1 || a < 0) return fail(GBTA_ERR_ARG, "require b >= 1, nt >= 1, a >= 0");
  if (a > gbta::TS)
    return fail(GBTA_ERR_ARG, "arrowhead block size above " + std::to_string(gbta::TS) + " is not supported");
  auto* s = new gbta_solver();
  s->g.b = b;
  s->g.nt = nt;
  s->g.a = a;
  s->g.B = (b + gbta::TS - 1) / gbta::TS;
  s->g.m = gbta::default_sep(nt);
  const long long nflags = (long long)(2 * nt - 1) * s->g.B * s->g.B + (long long)nt * s->g.B + 1;
  if (nflags > (1ll << 31) - 1) {
    delete s;
    return fail(GBTA_ERR_ARG, "problem too large for 32-bit tile indices");
  }
  auto cleanup = [&](int code) {
    gbta_destroy(s);
    return code;
  };
  cudaError_t e;
#define CREATE_CUDA(call)                                                                     \
  if ((e = (call)) != cudaSuccess) {                                                           \
    const std::string m = std::string(#call) + ": " + cudaGetErrorString(e);                   \
    cleanup(0);                                                                                \
    return fail(GBTA_ERR_CUDA, m);                                                             \
  }
  CREATE_CUDA(cudaGetDevice(&s->device));
  CREATE_CUDA(cudaDeviceGetAttribute(&s->nsm, cudaDevAttrMultiProcessorCount, s->device));
  if (const char* v = std::getenv("GBTA_CTAS_PER_SM")) {
    const int k = std::atoi(v);
    if (k >= 0 && k <= 8) s->ctas_per_sm = k;
  }
  if (const char* v = std::getenv("GBTA_WAIT_LIMIT_MS")) {
    const double ms = std::atof(v);
    if (ms > 0.0) s->wait_ns = (unsigned long long)(ms * 1e6);
  }
  CREATE_CUDA(cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking));
  s->stream = s->own_stream;
  CREATE_CUDA(cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking));
  CREATE_CUDA(cudaEventCreateWithFlags(&s->ev_fac, cudaEventDisableTiming));
  CREATE_CUDA(cudaEventCreateWithFlags(&s->ev_sel, cudaEventDisableTiming));
  CREATE_CUDA(cudaEventCreateWithFlags(&s->ev_swp, cudaEventDisableTiming));

  const std::vector<int4> ft = gbta::factor_task_list(s->g), st = gbta::selinv_task_list(s->g),
                          stm = gbta::selinv_task_list(s->g, true);
  s->n_ftasks = (int)ft.size();
  s->n_stasks = (int)st.size();
  const size_t ntile = (size_t)nt * s->g.B;
  CREATE_CUDA(cudaMalloc(&s->d_ctrl, CTRL_INTS * sizeof(int)));
  CREATE_CUDA(cudaMalloc(&s->d_flags, (size_t)nflags * sizeof(int)));
  CREATE_CUDA(cudaMalloc(&s->d_ctrl2, CTRL_INTS * sizeof(int)));
  CREATE_CUDA(cudaMalloc(&s->d_flags2, (size_t)nflags * sizeof(int)));
  CREATE_CUDA(cudaMemsetAsync(s->d_ctrl2, 0, CTRL_INTS * sizeof(int), s->stream));
  CREATE_CUDA(cudaMemsetAsync(s->d_flags2, 0, (size_t)nflags * sizeof(int), s->stream));
  CREATE_CUDA(cudaMalloc(&s->d_ftasks, ft.size() * sizeof(int4)));
  CREATE_CUDA(cudaMalloc(&s->d_stasks, st.size() * sizeof(int4)));
  CREATE_CUDA(cudaMalloc(&s->d_stasks_m, stm.size() * sizeof(int4)));
  CREATE_CUDA(cudaMalloc(&s->d_tip_part, ntile * gbta::TS * gbta::TS * sizeof(double)));
  CREATE_CUDA(cudaMalloc(&s->d_arrow_part, ntile * gbta::TS * gbta::SOLVE_NC * sizeof(double)));
  CREATE_CUDA(cudaMalloc(&s->d_faux, ntile * sizeof(int)));
  CREATE_CUDA(cudaMemsetAsync(s->d_faux, 0, ntile * sizeof(int), s->stream));
  CREATE_CUDA(cudaMalloc(&s->d_dpre, 2 * ntile * sizeof(int)));
  CREATE_CUDA(cudaMemsetAsync(s->d_dpre, 0, 2 * ntile * sizeof(int), s->stream));
  if (nt > 1) CREATE_CUDA(cudaMalloc(&s->d_kf, (size_t)(nt - 1) * s->g.B * sizeof(int)));
  CREATE_CUDA(cudaMalloc(&s->d_ld, (nt + 2) * sizeof(double)));
  CREATE_CUDA(cudaMallocHost(&s->h_ctrl, CTRL_INTS * sizeof(int)));
  CREATE_CUDA(cudaMemsetAsync(s->d_ctrl, 0, CTRL_INTS * sizeof(int), s->stream));
  CREATE_CUDA(cudaMemsetAsync(s->d_flags, 0, (size_t)nflags * sizeof(int), s->stream));
  CREATE_CUDA(cudaMemcpyAsync(s->d_ftasks, ft.data(), ft.size() * sizeof(int4), cudaMemcpyHostToDevice, s->stream));
  CREATE_CUDA(cudaMemcpyAsync(s->d_stasks, st.data(), st.size() * sizeof(int4), cudaMemcpyHostToDevice, s->stream));
  CREATE_CUDA(cudaMemcpyAsync(s->d_stasks_m, stm.data(), stm.size() * sizeof(int4), cudaMemcpyHostToDevice, s->stream));
  CREATE_CUDA(cudaStreamSynchronize(s->stream));
#undef CREATE_CUDA
  s->ws_bytes = 2 * (CTRL_INTS * sizeof(int) + (size_t)nflags * sizeof(int)) + (ft.size() + st.size()) * sizeof(int4) +
                ntile * gbta::TS * (gbta::TS + gbta::SOLVE_NC) * sizeof(double) + (nt + 2) * sizeof(double) +
                3 * ntile * sizeof(int) + (size_t)(nt - 1) * s->g.B * sizeof(int);
  *out = s;
  g_last_error.clear();
  return GBTA_OK;
}

int gbta_destroy(gbta_solver* s) {
  if (!s) return GBTA_OK;
  if (s->stream) cudaStreamSynchronize(s->stream);
  if (s->side) cudaStreamSynchronize(s->side);
  cudaFree(s->d_ctrl);
  cudaFree(s->d_flags);
  cudaFree(s->d_ftasks);
  cudaFree(s->d_stasks);
  cudaFree(s->d_stasks_m);
  cudaFree(s->d_tip_part);
  cudaFree(s->d_arrow_part);
  cudaFree(s->d_faux);
  cudaFree(s->d_dpre);
  cudaFree(s->d_kf);
  cudaFree(s->d_ld);
  cudaFree(s->d_sig);
  cudaFree(s->d_selws);
  cudaFree(s->d_trace);
  cudaFree(s->d_digits);
  cudaFree(s->d_sdig);
  cudaFree(s->d_erow);
  cudaFree(s->d_tz);
  if (s->h_ctrl) cudaFreeHost(s->h_ctrl);
  if (s->h_pairs) cudaFreeHost(s->h_pairs);
  for (cudaEvent_t ev : s->tev)
    if (ev) cudaEventDestroy(ev);
  cudaFree(s->d_ctrl2);
  cudaFree(s->d_flags2);
  if (s->ev_fac) cudaEventDestroy(s->ev_fac);
  if (s->ev_sel) cudaEventDestroy(s->ev_sel);
  if (s->ev_swp) cudaEventDestroy(s->ev_swp);
  if (s->side) cudaStreamDestroy(s->side);
  if (s->own_stream) cudaStreamDestroy(s->own_stream);
  delete s;
  return GBTA_OK;
}

int gbta_set_twist(gbta_solver* s, int enable) {
  if (int r = check_solver(s)) return r;
  const int m = enable ? gbta::default_sep(s->g.nt) : s->g.nt - 1;
  if (m == s->g.sep()) return GBTA_OK;
  GBTA_CUDA(cudaStreamSynchronize(s->stream));
  s->g.m = m;
  // the inversion's lists keep their lengths (every block but the separator has a
  // coupling slot); the factorization's depends on which diagonal tiles get a partial
  const std::vector<int4> ft = gbta::factor_task_list(s->g), st = gbta::selinv_task_list(s->g),
                          stm = gbta::selinv_task_list(s->g, true);
  if ((int)st.size() != s->n_stasks || stm.size() != st.size())
    return fail(GBTA_ERR_ARG, "internal: selected-inversion task list length changed with the elimination order");
  if ((int)ft.size() != s->n_ftasks) {
    int4* d = nullptr;
    GBTA_CUDA(cudaMalloc(&d, ft.size() * sizeof(int4)));
    cudaFree(s->d_ftasks);
    s->d_ftasks = d;
    s->ws_bytes = s->ws_bytes - (size_t)s->n_ftasks * sizeof(int4) + ft.size() * sizeof(int4);
    s->n_ftasks = (int)ft.size();
  }
  GBTA_CUDA(cudaMemcpy(s->d_ftasks, ft.data(), ft.size() * sizeof(int4), cudaMemcpyHostToDevice));
  GBTA_CUDA(cudaMemcpy(s->d_stasks, st.data(), st.size() * sizeof(int4), cudaMemcpyHostToDevice));
  GBTA_CUDA(cudaMemcpy(s->d_stasks_m, stm.data(), stm.size() * sizeof(int4), cudaMemcpyHostToDevice));
  return GBTA_OK;
}

int gbta_get_twist(const gbta_solver* s) { return s ? (s->g.twisted() ? 1 : 0) : -1; }

int gbta_set_kernel_timing(gbta_solver* s, int enable) {
  if (int r = check_solver(s)) return r;
  if (enable) {
    for (cudaEvent_t& ev : s->tev)
      if (!ev) GBTA_CUDA(cudaEventCreate(&ev));
    if (!s->h_pairs) GBTA_CUDA(cudaMallocHost(&s->h_pairs, 2 * sizeof(long long)));
    s->h_pairs[0] = s->h_pairs[1] = -1;
  }
  s->timing = enable != 0;
  for (bool& t : s->timed) t = false;
  return GBTA_OK;
}

int gbta_kernel_pairs(gbta_solver* s, long long* pairs) {
  if (int r = check_solver(s)) return r;
  if (!pairs) return fail(GBTA_ERR_ARG, "pairs is null");
  pairs[0] = pairs[1] = -1;
  if (!s->timing || !s->h_pairs) return GBTA_OK;
  GBTA_CUDA(cudaStreamSynchronize(s->stream));
  for (int k = 0; k < 2; ++k) pairs[k] = s->timed[k] ? s->h_pairs[k] : -1;
  return GBTA_OK;
}

int gbta_kernel_ms(gbta_solver* s, double* ms) {
  if (int r = check_solver(s)) return r;
  if (!ms) return fail(GBTA_ERR_ARG, "ms is null");
  for (int k = 0; k < 3; ++k) {
    ms[k] = -1.0;
    if (!s->timed[k]) continue;
    GBTA_CUDA(cudaEventSynchronize(s->tev[2 * k + 1]));
    float v = 0.f;
    GBTA_CUDA(cudaEventElapsedTime(&v, s->tev[2 * k], s->tev[2 * k + 1]));
    ms[k] = v;
  }
  return GBTA_OK;
}

int gbta_set_stream(gbta_solver* s, void* stream) {
  if (int r = check_solver(s)) return r;
  s->stream = (cudaStream_t)stream;   // NULL is the CUDA default stream
  return GBTA_OK;
}

int gbta_set_method(gbta_solver* s, int method) {
  if (int r = check_solver(s)) return r;
  if (method != GBTA_METHOD_FP64 && method != GBTA_METHOD_OZAKI) return fail(GBTA_ERR_ARG, "unknown method");
  s->method = method;
  return GBTA_OK;
}

int gbta_get_method(const gbta_solver* s) { return s ? s->method : -1; }

int gbta_set_selinv_overlap(gbta_solver* s, int enable) {
  if (int r = check_solver(s)) return r;
  s->overlap = enable != 0;
  return GBTA_OK;
}

int gbta_set_ctas_per_sm(gbta_solver* s, int n) {
  if (int r = check_solver(s)) return r;
  if (n < 0 || n > 8) return fail(GBTA_ERR_ARG, "ctas_per_sm must be in [0, 8]");
  s->ctas_per_sm = n;
  return GBTA_OK;
}

int gbta_set_trace(gbta_solver* s, int enable) {
  if (int r = check_solver(s)) return r;
  GBTA_CUDA(cudaStreamSynchronize(s->stream));
  cudaFree(s->d_trace);
  s->d_trace = nullptr;
  s->trace_cap = s->trace_n = 0;
  if (enable) {
    const long long cap = s->n_ftasks > s->n_stasks ? s->n_ftasks : s->n_stasks;
    GBTA_CUDA(cudaMalloc(&s->d_trace, (size_t)cap * 8 * sizeof(long long)));
    GBTA_CUDA(cudaMemset(s->d_trace, 0, (size_t)cap * 8 * sizeof(long long)));
    s->trace_cap = cap;
  }
  return GBTA_OK;
}

long long gbta_get_trace(gbta_solver* s, long long* out, long long max_records) {
  if (!s || !s->d_trace || !out) return 0;
  const long long n = s->trace_n < max_records ? s->trace_n : max_records;
  if (cudaStreamSynchronize(s->stream) != cudaSuccess) return 0;
  if (cudaMemcpy(out, s->d_trace, (size_t)n * 8 * sizeof(long long), cudaMemcpyDeviceToHost) != cudaSuccess) return 0;
  return n;
}

long long gbta_get_task_list(gbta_solver* s, int which, int* out, long long max_tasks) {
  if (!s || !out || (which != 0 && which != 1)) return 0;
  const int4* d = which == 0 ? s->d_ftasks : (s->method == GBTA_METHOD_OZAKI ? s->d_stasks_m : s->d_stasks);
  const long long n0 = which == 0 ? s->n_ftasks : s->n_stasks;
  const long long n = n0 < max_tasks ? n0 : max_tasks;
  if (cudaStreamSynchronize(s->stream) != cudaSuccess) return 0;
  if (cudaMemcpy(out, d, (size_t)n * sizeof(int4), cudaMemcpyDeviceToHost) != cudaSuccess) return 0;
  return n;
}

int gbta_set_wait_limit_ms(gbta_solver* s, double ms) {
  if (int r = check_solver(s)) return r;
  if (!(ms > 0)) return fail(GBTA_ERR_ARG, "wait limit must be positive");
  s->wait_ns = (unsigned long long)(ms * 1e6);
  return GBTA_OK;
}

size_t gbta_workspace_bytes(const gbta_solver* s) {
  return s ? s->ws_bytes + s->sig_elems * sizeof(double) + s->digit_bytes +
                 (s->d_selws ? gbta::selinv_prepare_bytes(s->g) : 0)
           : 0;
}

int gbta_status(gbta_solver* s) {
  if (int r = check_solver(s)) return r;
  GBTA_CUDA(cudaStreamSynchronize(s->stream));
  GBTA_CUDA(cudaStreamSynchronize(s->side));
  GBTA_CUDA(cudaGetLastError());
  // the sticky words of both control blocks (the side stream's: an overlapped inversion)
  int info = 0, err = 0;
  for (int* ctrl : {s->d_ctrl, s->d_ctrl2}) {
    GBTA_CUDA(cudaMemcpy(s->h_ctrl, ctrl, CTRL_INTS * sizeof(int), cudaMemcpyDeviceToHost));
    if (s->h_ctrl[CTRL_ERR] != 0) err = s->h_ctrl[CTRL_ERR];
    if (s->h_ctrl[CTRL_INFO] != 0 && info == 0) info = s->h_ctrl[CTRL_INFO];
  }
  if (info != 0 || err != 0) {
    GBTA_CUDA(cudaMemsetAsync(s->d_ctrl, 0, CTRL_INTS * sizeof(int), s->stream));
    GBTA_CUDA(cudaMemsetAsync(s->d_ctrl2, 0, CTRL_INTS * sizeof(int), s->stream));
    GBTA_CUDA(cudaStreamSynchronize(s->stream));
  }
  if (err == 1) return fail(GBTA_ERR_TIMEOUT, "a kernel wait exceeded the wait limit; the launch was abandoned");
  if (info > 0)
    return fail(info, "matrix is not positive definite (non-positive pivot at global row " + std::to_string(info) + ")");
  return GBTA_OK;
}

// ---------------------------------------------------------------- Ozaki workspace
// Digit planes (one 9 x 32 x 32 fp16 block per tile slot) and per-row / per-column
// exponents, shared by the factorization and the selected inversion.
static int ensure_digits(gbta_solver* s) {
  if (s->d_digits) return GBTA_OK;
  GBTA_CUDA(cudaStreamSynchronize(s->stream));
  const size_t bytes = gbta::factor_oz_digit_bytes(s->g);
  const size_t ebytes = ((size_t)s->g.nt * s->g.b + s->g.a) * sizeof(int);
  const size_t zbytes = (size_t)s->g.nflags() * sizeof(int);
  GBTA_CUDA(cudaMalloc(&s->d_digits, bytes));
  GBTA_CUDA(cudaMalloc(&s->d_erow, ebytes));
  GBTA_CUDA(cudaMalloc(&s->d_tz, zbytes));
  s->digit_bytes = bytes + ebytes + zbytes;
  return GBTA_OK;
}

// ---------------------------------------------------------------- factorization
static int factor_async(gbta_solver* s, double* D, double* L, double* R, double* T, int use_arrow) {
  if (int r = check_solver(s)) return r;
  if (!D || (s->g.nt > 1 && !L)) return fail(GBTA_ERR_ARG, "D/L must be device pointers");
  if (use_arrow && (!R || !T)) return fail(GBTA_ERR_ARG, "R/T must be device pointers for the bta factorization");
  if (s->method == GBTA_METHOD_OZAKI)
    if (int r = ensure_digits(s)) return r;
  if (int r = reset_ticket(s)) return r;
  if (s->g.nt > 1) {
    gbta::launch_transpose_lslots(s->g, L, s->stream);
    gbta::launch_coupling_kfirst(s->g, L, s->d_kf, s->stream);
  }
  gbta::launch_clear_feeders(s->g, s->d_flags, s->stream);
  const gbta::LaunchCtl lc = next_launch(s, s->n_ftasks);
  if (s->timing) GBTA_CUDA(cudaEventRecord(s->tev[0], s->stream));
  s->fac_digits = s->method == GBTA_METHOD_OZAKI;
  if (s->method == GBTA_METHOD_OZAKI)
    gbta::launch_factor_oz(s->g, D, L, R, T, use_arrow, s->d_ftasks, s->n_ftasks, s->d_tip_part,
                           (__half*)s->d_digits, s->d_erow, lc, s->d_faux, s->d_dpre, s->d_kf);
  else
    gbta::launch_factor(s->g, D, L, R, T, use_arrow, s->d_ftasks, s->n_ftasks, s->d_tip_part, lc, s->d_faux,
                        s->d_dpre, s->d_kf);
  GBTA_CUDA(cudaGetLastError());
  GBTA_CUDA(cudaEventRecord(s->ev_fac, s->stream));
  s->fac_evt = true;
  s->swept = false;
  if (s->timing) {
    GBTA_CUDA(cudaEventRecord(s->tev[1], s->stream));
    s->timed[0] = true;
    GBTA_CUDA(cudaMemcpyAsync(s->h_pairs, s->d_ctrl + CTRL_MMA, sizeof(long long), cudaMemcpyDeviceToHost,
                              s->stream));
  }
  return GBTA_OK;
}

int gbta_pobtaf_async(gbta_solver* s, double* D, double* L, double* R, double* T) {
  return factor_async(s, D, L, R, T, s && s->g.a > 0);
}
int gbta_pobtf_async(gbta_solver* s, double* D, double* L) { return factor_async(s, D, L, nullptr, nullptr, 0); }
int gbta_pobtaf(gbta_solver* s, double* D, double* L, double* R, double* T) {
  if (int r = gbta_pobtaf_async(s, D, L, R, T)) return r;
  return gbta_status(s);
}
int gbta_pobtf(gbta_solver* s, double* D, double* L) {
  if (int r = gbta_pobtf_async(s, D, L)) return r;
  return gbta_status(s);
}

// ---------------------------------------------------------------- solves
static int solve_async(gbta_solver* s, const double* D, const double* L, const double* R, const double* T, double* B,
                       int nrhs, int trans, int use_arrow) {
  if (int r = check_solver(s)) return r;
  if (!D || !B || (s->g.nt > 1 && !L)) return fail(GBTA_ERR_ARG, "D/L/B must be device pointers");
  if (use_arrow && (!R || !T)) return fail(GBTA_ERR_ARG, "R/T must be device pointers for the bta solve");
  if (nrhs < 1) return fail(GBTA_ERR_ARG, "nrhs must be >= 1");
  if (trans != 0 && trans != 1 && trans != 2) return fail(GBTA_ERR_ARG, "trans must be 0 (N), 1 (C) or 2 (both)");
  // both sweeps in one launch where the flag array has room for the second sweep's flags
  // (every geometry but b <= 32), else one after the other
  const bool both = trans == 2 && gbta::solve_both_fits(s->g);
  const int ntasks = (s->g.nt * s->g.B + (use_arrow ? 1 : 0)) * (both ? 2 : 1);
  if (s->timing) GBTA_CUDA(cudaEventRecord(s->tev[4], s->stream));
  for (int c0 = 0; c0 < nrhs; c0 += gbta::SOLVE_NC) {
    const int nc = nrhs - c0 < gbta::SOLVE_NC ? nrhs - c0 : gbta::SOLVE_NC;
    if (int r = reset_ticket(s)) return r;
    gbta::LaunchCtl lc = next_launch(s, ntasks);
    // the sweeps run one CTA per SM unless set otherwise: their chain needs few, and
    // more spend the SMs' issue slots and memory traffic on waiting tasks (alone at
    // nt = 128, b = 1024: 9.7 ms against 12.4 ms with as many as fit), and next to an
    // overlapped inversion its CTAs take the rest of each SM
    if (s->ctas_per_sm == 0) lc.ctas_per_sm = 1;
    if (both) {
      gbta::launch_solve(s->g, D, L, R, T, B + c0, nrhs, nc, 0, use_arrow, s->d_arrow_part, lc, 1);
    } else {
      for (int tr = (trans == 1 ? 1 : 0); tr <= (trans == 0 ? 0 : 1); ++tr) {
        if (tr == 1 && trans == 2) {   // the second sweep of trans = 2: its own launch
          if (int r = reset_ticket(s)) return r;
          lc = next_launch(s, ntasks);
          if (s->ctas_per_sm == 0) lc.ctas_per_sm = 1;
        }
        gbta::launch_solve(s->g, D, L, R, T, B + c0, nrhs, nc, tr, use_arrow, s->d_arrow_part, lc);
      }
    }
    GBTA_CUDA(cudaGetLastError());
  }
  s->swept = true;
  GBTA_CUDA(cudaEventRecord(s->ev_swp, s->stream));
  if (s->timing) {
    GBTA_CUDA(cudaEventRecord(s->tev[5], s->stream));
    s->timed[2] = true;
  }
  return GBTA_OK;
}

int gbta_pobtas_async(gbta_solver* s, const double* D, const double* L, const double* R, const double* T, double* B,
                      int nrhs, int trans) {
  return solve_async(s, D, L, R, T, B, nrhs, trans, s && s->g.a > 0);
}
int gbta_pobtas(gbta_solver* s, const double* D, const double* L, const double* R, const double* T, double* B,
                int nrhs, int trans) {
  if (int r = gbta_pobtas_async(s, D, L, R, T, B, nrhs, trans)) return r;
  return gbta_status(s);
}
int gbta_pobts(gbta_solver* s, const double* D, const double* L, double* B, int nrhs, int trans) {
  if (int r = solve_async(s, D, L, nullptr, nullptr, B, nrhs, trans, 0)) return r;
  return gbta_status(s);
}

// ---------------------------------------------------------------- logdet
int gbta_logdet(gbta_solver* s, const double* D, const double* T, int with_tip, double* out) {
  if (int r = check_solver(s)) return r;
  if (!D || !out) return fail(GBTA_ERR_ARG, "D and out are required");
  const int tip = with_tip && s->g.a > 0;
  if (tip && !T) return fail(GBTA_ERR_ARG, "T is required for the bta logdet");
  gbta::launch_logdet(s->g, D, T, tip, s->d_ld, s->d_ld + s->g.nt + 1, s->stream);
  GBTA_CUDA(cudaGetLastError());
  double v = 0.0;
  GBTA_CUDA(cudaMemcpyAsync(&v, s->d_ld + s->g.nt + 1, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  GBTA_CUDA(cudaStreamSynchronize(s->stream));
  *out = v;
  if (std::isnan(v)) return fail(GBTA_ERR_ARG, "Logdet is NaN. Check the input matrix.");
  return GBTA_OK;
}

// ---------------------------------------------------------------- selected inversion
static int selinv_async(gbta_solver* s, double* D, double* L, double* R, double* T, int use_arrow) {
  if (int r = check_solver(s)) return r;
  if (!D || (s->g.nt > 1 && !L)) return fail(GBTA_ERR_ARG, "D/L must be device pointers");
  if (use_arrow && (!R || !T)) return fail(GBTA_ERR_ARG, "R/T must be device pointers for the bta selected inversion");
  const gbta::Geom& g = s->g;
  const size_t bb = (size_t)g.b * g.b;
  const bool ozaki = s->method == GBTA_METHOD_OZAKI;
  // with a tensor-core factorization's digit planes (until the inversion's own pre-pass
  // overwrites them) the G tiles go through the tensor cores too
  const bool tc_g = ozaki && s->fac_digits;
  // Overlapped: the whole inversion reads the factor's blocks only (the G tiles go to the
  // Sigma workspace), so it runs on the side stream from the factorization's completion,
  // next to whatever the solver's stream runs meanwhile (the sweeps), and the write-back
  // follows on the solver's stream after both.  Only when sweeps were enqueued since the
  // factorization and have not finished yet (with nothing to overlap, the write-back is
  // pure cost), and not while tracing (one trace buffer).
  bool sweeping = false;
  if (s->overlap && s->swept) {
    const cudaError_t q = cudaEventQuery(s->ev_swp);
    if (q != cudaSuccess && q != cudaErrorNotReady)
      return fail(GBTA_ERR_CUDA, std::string("cudaEventQuery: ") + cudaGetErrorString(q));
    sweeping = q == cudaErrorNotReady;
  }
  const bool over = s->overlap && tc_g && s->fac_evt && sweeping && !s->d_trace;
  // The tensor-core method reads the factor only through its digit planes, sliced by the
  // pre-pass, and the tip task reads T before it writes Sigma_T: without the overlap Sigma
  // goes straight into the caller's buffers.  The FP64 method reads the factor tiles
  // during the inversion, so Sigma goes to a workspace and is copied back.
  const bool inplace = ozaki && !over;
  const size_t need = g.nt * bb + (g.nt - 1) * bb + (size_t)g.nt * g.a * g.b + (size_t)g.a * g.a;
  if (!inplace && s->sig_elems < need) {
    GBTA_CUDA(cudaStreamSynchronize(s->stream));
    GBTA_CUDA(cudaStreamSynchronize(s->side));
    cudaFree(s->d_sig);
    s->d_sig = nullptr;
    s->sig_elems = 0;
    GBTA_CUDA(cudaMalloc(&s->d_sig, need * sizeof(double)));
    s->sig_elems = need;
  }
  if (!s->d_selws) {
    GBTA_CUDA(cudaStreamSynchronize(s->stream));
    GBTA_CUDA(cudaMalloc(&s->d_selws, gbta::selinv_prepare_bytes(g)));
  }
  const double* cinv = s->d_selws + (size_t)g.nt * g.B * gbta::TS * gbta::TS;
  double* SD = inplace ? D : s->d_sig;
  double* SL = inplace ? L : SD + g.nt * bb;
  double* SR = inplace ? R : SL + (g.nt - 1) * bb;
  double* ST = inplace ? T : SR + (size_t)g.nt * g.a * g.b;
  if (ozaki) {
    if (int r = ensure_digits(s)) return r;
    if (!s->d_sdig) {
      GBTA_CUDA(cudaStreamSynchronize(s->stream));
      const size_t bytes = gbta::selinv_oz_digit_bytes(g);
      GBTA_CUDA(cudaMalloc(&s->d_sdig, bytes));
      s->digit_bytes += bytes;
    }
  }
  cudaStream_t st = over ? s->side : s->stream;
  if (over) GBTA_CUDA(cudaStreamWaitEvent(s->side, s->ev_fac, 0));
  gbta::launch_selinv_prepare(g, D, L, R, use_arrow, s->d_selws, st, tc_g ? (__half*)s->d_digits : nullptr,
                              s->d_erow, s->d_kf, over ? SD : nullptr, over ? SL : nullptr, over ? SR : nullptr);
  if (ozaki) s->fac_digits = false;
  s->fac_evt = false;
  if (int r = over ? reset_side_ticket(s) : reset_ticket(s)) return r;
  gbta::LaunchCtl lc = over ? next_side_launch(s, s->n_stasks) : next_launch(s, s->n_stasks);
  // (its grid is the full one: the CTAs that find no slot next to the sweeps' CTAs,
  // which were launched first and keep one per SM, start when those exit)
  if (s->timing) GBTA_CUDA(cudaEventRecord(s->tev[2], st));
  if (ozaki)   // (its pre-pass reads the G tiles: from the workspace when overlapped)
    gbta::launch_selinv_oz(g, over ? SD : D, over ? SL : L, over ? SR : R, T, SD, SL, SR, ST, use_arrow,
                           s->d_stasks_m, s->n_stasks, (__half*)s->d_digits, s->d_erow, cinv, (__half*)s->d_sdig,
                           s->d_tip_part, s->d_faux, lc, g.nflags() < (1 << 24) ? s->d_tz : nullptr);
  else
    gbta::launch_selinv(g, D, L, R, T, SD, SL, SR, ST, use_arrow, s->d_stasks, s->n_stasks, cinv, lc);
  GBTA_CUDA(cudaGetLastError());
  if (s->timing) {
    GBTA_CUDA(cudaEventRecord(s->tev[3], st));
    s->timed[1] = true;
    GBTA_CUDA(cudaMemcpyAsync(s->h_pairs + 1, (over ? s->d_ctrl2 : s->d_ctrl) + CTRL_MMA, sizeof(long long),
                              cudaMemcpyDeviceToHost, st));
  }
  if (over) {
    GBTA_CUDA(cudaEventRecord(s->ev_sel, s->side));
    GBTA_CUDA(cudaStreamWaitEvent(s->stream, s->ev_sel, 0));
  }
  if (inplace)
    gbta::launch_selinv_finish_inplace(g, D, L, s->stream);
  else
    gbta::launch_selinv_writeback(g, SD, SL, SR, ST, D, L, R, T, use_arrow, s->stream);
  GBTA_CUDA(cudaGetLastError());
  return GBTA_OK;
}

int gbta_pobtasi_async(gbta_solver* s, double* D, double* L, double* R, double* T) {
  return selinv_async(s, D, L, R, T, s && s->g.a > 0);
}
int gbta_pobtasi(gbta_solver* s, double* D, double* L, double* R, double* T) {
  if (int r = gbta_pobtasi_async(s, D, L, R, T)) return r;
  return gbta_status(s);
}
int gbta_pobtsi(gbta_solver* s, double* D, double* L) {
  if (int r = selinv_async(s, D, L, nullptr, nullptr, 0)) return r;
  return gbta_status(s);
}

}  // extern "C"
