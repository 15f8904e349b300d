// Internal launch interface between the C ABI (bta_api.cu) and the kernels.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

namespace gbta {

constexpr int TS = 32;  // tile edge (FP64 elements)

// Launch epochs are multiples of 2^EPOCH_SHIFT: a ready flag holds epoch + payload,
// payload < 2^EPOCH_SHIFT (the selected inversion stores each Sigma tile's exponent
// there), and "ready" is flag >= epoch.  Epoch-stamped words are cleared before the
// epoch counter would pass 2^(31 - EPOCH_SHIFT).
constexpr int EPOCH_SHIFT = 9;

// Task codes of the factorization DAG.  FT_PRE is a flag on an FT_OFFD / FT_LOW task:
// the task only forms the tile's products and leaves the triangular solve to the
// FT_FEEDQ tasks of its rows (the feeder tile of a diagonal tile, see Geom).
enum FactorTask { FT_DIAG = 0, FT_OFFD = 1, FT_LOW = 2, FT_ARW = 3, FT_TIP = 4, FT_FEEDQ = 5 };
constexpr int FT_PRE = 8;
// Split product loops.  A diagonal tile (i, c) and the feeder tile of column c share the
// same left-looking loop, whose last step -- the product with the previous column's
// feeder tile (k = c - 1), or with each neighbour block's last column when c = 0 -- is
// the only one that waits on the factorization's column chain.  FT_PART on an FT_DIAG
// task or on a feeder's FT_PRE task: every step but that last one, stored in the tile
// and flagged (diag_pre / feed_part); FT_TAIL: the tile from that partial, the last
// step(s) and the rest of the task.  Placed two columns ahead, the partials take both
// long product loops off the chain.
constexpr int FT_TAIL = 16;
constexpr int FT_PART = 32;
constexpr int FEED_ROWS = 8;   // rows of a feeder tile solved by one FT_FEEDQ task
// Task codes of the selected-inversion DAG.
// ST_PART: the products of the sub-diagonal tile of a column except its last (tensor-
// core method; the diagonal task of the previous column finishes that tile).
enum SelinvTask { ST_TIP = 0, ST_OFF = 1, ST_DIAG = 2, ST_PART = 3 };

// Geometry of one BTA matrix and the flag layout shared by all kernels.
//
// Elimination order.  With the separator block m = sep() < nt - 1 the blocks are
// eliminated from both ends towards m (a "twisted" block Cholesky): the top chain
// 0, 1, ..., m-1 downwards, the bottom chain nt-1, nt-2, ..., m+1 upwards, side by side,
// then m, then the arrow tip.  Both chains are ordinary block-tridiagonal recurrences,
// so nothing fills in and the flop count is the sequential one, while the longest chain
// of dependent tile columns is about half as long.  m = nt - 1 (the default m = -1) is
// the plain top-down order of the reference's Serinv recurrence.
//
// Block i is coupled to nxt(i), the neighbour eliminated after it (i + 1 above the
// separator, i - 1 below it, none for m), through the b x b slot lslot(i) of the L
// buffer, whose rows are those of block nxt(i) and whose columns those of block i.
// Above the separator that is the caller's L_i = Q(i+1, i) itself; below it the slot
// L_{i-1} holds Q(i-1, i), i.e. the caller's block transposed (launch_transpose_lslots
// transposes those slots before a factorization; the selected inversion's write-back
// transposes them back).  prev(i, k) lists the (one or two) neighbours eliminated
// before i, whose Schur updates block i receives.
struct Geom {
  int b, nt, a, B;   // block size, number of diagonal blocks, arrow size, tiles per block edge
  int m = -1;        // separator block (-1: nt - 1, the top-down order)
  __host__ __device__ int fD(int i, int r, int c) const { return (i * B + r) * B + c; }
  __host__ __device__ int fL(int i, int r, int c) const { return nt * B * B + (i * B + r) * B + c; }
  __host__ __device__ int fR(int i, int c) const { return (2 * nt - 1) * B * B + i * B + c; }
  __host__ __device__ int fT() const { return (2 * nt - 1) * B * B + nt * B; }
  __host__ __device__ int nflags() const { return (2 * nt - 1) * B * B + nt * B + 1; }
  __host__ __device__ int vrows(int r) const {   // valid rows of block-tile r
    const int v = b - r * TS;
    return v < TS ? v : TS;
  }
  __host__ __device__ int sep() const { return m < 0 ? nt - 1 : m; }
  __host__ __device__ bool twisted() const { return sep() < nt - 1; }
  __host__ __device__ int nxt(int i) const {
    const int s = sep();
    return i < s ? i + 1 : (i > s ? i - 1 : -1);
  }
  __host__ __device__ int lslot(int i) const {
    const int s = sep();
    return i < s ? i : (i > s ? i - 1 : -1);
  }
  // row block and column block of L slot j
  __host__ __device__ int lrow(int j) const { return j < sep() ? j + 1 : j; }
  __host__ __device__ int lcol(int j) const { return j < sep() ? j : j + 1; }
  // neighbours eliminated before block i (the top one first)
  __host__ __device__ int nprev(int i) const {
    const int s = sep();
    if (i < s) return i > 0 ? 1 : 0;
    if (i > s) return i < nt - 1 ? 1 : 0;
    return (s > 0 ? 1 : 0) + (s < nt - 1 ? 1 : 0);
  }
  __host__ __device__ int prev(int i, int k) const {
    const int s = sep();
    if (i < s) return i - 1;
    if (i > s) return i + 1;
    return (k == 0 && s > 0) ? s - 1 : s + 1;
  }
  // Position u of a sequence that interleaves the top chain's n1 units with the bottom
  // chain's n2 units (top, bottom, top, ... while both last, then the rest of the longer
  // one): returns 0 (top) or 1 (bottom) and the unit index within that chain.
  __host__ __device__ static int interleave(int n1, int n2, int u, int* k) {
    const int mn = n1 < n2 ? n1 : n2;
    if (u < 2 * mn) {
      *k = u >> 1;
      return u & 1;
    }
    *k = mn + (u - 2 * mn);
    return n1 > mn ? 0 : 1;
  }
  // Blocks in elimination order: position q < nt -> block (interleaved chains, then m).
  __host__ __device__ int elim_block(int q) const {
    const int s = sep(), n1 = s, n2 = nt - 1 - s;
    if (q >= n1 + n2) return s;
    int k;
    return interleave(n1, n2, q, &k) == 0 ? k : nt - 1 - k;
  }
  // The feeder of diagonal tile (i, c): the tile right below it in the next global tile
  // row of the elimination, whose solve against (i, c) and product with itself are the
  // last steps before the next diagonal tile can be factored.  0: none (last tile column
  // of the separator), 1: D_i(c + 1, c), 2: tile (0, c) of slot lslot(i).
  __host__ __device__ int feeder_kind(int i, int c) const { return c + 1 < B ? 1 : (nxt(i) >= 0 ? 2 : 0); }
  __host__ __device__ int feeder_rows(int i, int c) const { return feeder_kind(i, c) == 1 ? vrows(c + 1) : vrows(0); }
  __host__ __device__ int feeder_quarters(int i, int c) const {
    return feeder_kind(i, c) ? (feeder_rows(i, c) + FEED_ROWS - 1) / FEED_ROWS : 0;
  }
};

// Separator block of the elimination order the solvers use: the middle block once there
// are three or more blocks (two chains of about nt/2 blocks), else the plain order.
inline int default_sep(int nt) { return nt >= 3 ? nt / 2 : nt - 1; }

struct LaunchCtl {
  int* ctrl;
  int* flags;
  int epoch;
  unsigned long long wait_ns;
  int grid;                     // persistent CTAs when nsm == 0
  cudaStream_t stream;
  long long* trace = nullptr;   // per-task trace records, or null
  int nsm = 0;                  // > 0: size the grid from the kernel's occupancy (launch_grid)
  int ctas_per_sm = 0;          // CTAs per SM (0: as many as fit)
  int ntasks = 0;               // never more CTAs than tasks
};

// Persistent grid of a kernel with `threads` threads and `smem` bytes of dynamic
// shared memory: lc.grid when lc.nsm == 0, else nsm x (ctas_per_sm, capped by the
// kernel's occupancy; all that fit when 0), at most ntasks.
int launch_grid(const void* kernel, int threads, size_t smem, const LaunchCtl& lc);
// CTAs per SM that fit a kernel's registers, shared memory and threads, and, with
// tmem_cols > 0, the SM's 512 tensor-memory columns.  This is the occupancy rule for
// a kernel that allocates tensor memory: the CUDA occupancy calculator reports one
// CTA per SM for every such kernel, whatever it allocates.
int resident_ctas(const void* kernel, int threads, size_t smem, int tmem_cols);

// Task lists of the factorization and selected-inversion DAGs (bta_api.cu).
// diag_split: split the diagonal and feeder tiles' loops into FT_PART and FT_TAIL tasks
// (the kernel then needs the diag_pre flags).
std::vector<int4> factor_task_list(const Geom& g, bool diag_split = true);
// Whether diagonal tile (i, c) has products besides its last step(s) (the condition for
// its FT_DIAG|FT_PART task).
inline bool diag_has_partial(const Geom& g, int i, int c) {
  if (c >= 1) return g.nprev(i) * g.B + c - 1 > 0;
  return g.nprev(i) > 0 && g.B >= 2;
}
// The same for the feeder of diagonal tile (i, c): an OFFD feeder (c + 1, c) has the
// diagonal tile's loop, an L-slot feeder (0, B - 1) only its own block's B - 1 steps.
inline bool feeder_has_partial(const Geom& g, int i, int c) {
  const int fk = g.feeder_kind(i, c);
  if (fk == 1) return diag_has_partial(g, i, c);
  return fk == 2 && g.B >= 3;
}
// merged: the list of the tensor-core method, where each diagonal task also finishes
// the sub-diagonal tile of the next column (ST_PART tasks form its other products).
std::vector<int4> selinv_task_list(const Geom& g, bool merged = false);

// Host-side count of kernel launches issued by this library (see gbta_kernel_launches).
void count_launches(int n);

// feed_aux: nt * B ints (feeder "products done" flags), or null when the task list has
// no FT_PRE / FT_FEEDQ tasks.  With FT_FEEDQ tasks the feeder tiles' own ready flags
// must be zero at launch (launch_clear_feeders, or a cleared flag array).
// diag_pre: 2 * nt * B ints -- flags of the diagonal tiles' partial products, then of
// the feeder tiles' partial products -- or null when the task list has no FT_PART /
// FT_TAIL tasks.
// kf: (nt - 1) * B ints from launch_coupling_kfirst (the products of structurally zero
// coupling tiles are left out), or null (every product is formed).
void launch_factor(const Geom& g, double* D, double* L, double* R, double* T, int use_arrow,
                   const int4* tasks, int ntasks, double* tip_part, const LaunchCtl& lc, int* feed_aux = nullptr,
                   int* diag_pre = nullptr, const int* kf = nullptr);

// Transpose, in place, the L slots below the separator (slots sep() .. nt-2): before a
// factorization they hold the caller's Q(j+1, j), afterwards the factor needs Q(j, j+1).
// No launch when the order is top-down.
void launch_transpose_lslots(const Geom& g, double* L, cudaStream_t stream);

// Structurally zero tiles of the factor's coupling slots.  The factor's slot is
// L_j = Q_j F^{-T} with F the (lower triangular) factor of the diagonal block it
// couples from, so its tile (r, k) is zero when the input's row tile r is zero in every
// column tile <= k.  kf[j * B + r] = the first column tile of slot j's row tile r that
// holds a nonzero (B: none), read from the L slots as the factorization sees them
// (after launch_transpose_lslots).  Every product with a tile k < kf is exactly zero.
void launch_coupling_kfirst(const Geom& g, const double* L, int* kf, cudaStream_t stream);

// Zero the ready flags of the feeder tiles (Geom::feeder_kind): the FT_FEEDQ tasks of
// a factorization add shares of the epoch to them.
void launch_clear_feeders(const Geom& g, int* flags, cudaStream_t stream);

constexpr int SOLVE_NC = 4;   // right-hand-side columns per solve launch

// Tensor-core (Ozaki) factorization: digit-plane workspace bytes, and the launcher.
size_t factor_oz_digit_bytes(const Geom& g);
void launch_factor_oz(const Geom& g, double* D, double* L, double* R, double* T, int use_arrow,
                      const int4* tasks, int ntasks, double* tip_part, __half* digits, int* erow,
                      const LaunchCtl& lc, int* feed_aux = nullptr, int* diag_pre = nullptr,
                      const int* kf = nullptr);

// Row exponents of the input matrix (before a tensor-core factorization).
void launch_row_exponents(const Geom& g, const double* D, const double* T, int use_arrow, int* erow,
                          cudaStream_t stream);

size_t selinv_oz_digit_bytes(const Geom& g);
// Column exponents and transposed digit planes of the factor (before a tensor-core
// selected inversion).
// fdz (flag-slot count of ints, or null): the leading zero digit planes of every G tile.
void launch_selinv_oz_prepare(const Geom& g, const double* D, const double* L, const double* R, int use_arrow,
                              __half* fdig, int* ecol, int* fdz, cudaStream_t stream);
// sdig: digit planes (selinv_oz_digit_bytes) of the Sigma tiles, written by the tasks
// that produce them (their exponents travel in the tiles' flag words).  tasks: the
// merged list (selinv_task_list(g, true)); part: nt*B FP64 tiles and part_flag: nt*B
// epoch-stamped flags for the partial sums of the sub-diagonal tiles.
void launch_selinv_oz(const Geom& g, const double* D, const double* L, const double* R, const double* T,
                      double* SD, double* SL, double* SR, double* ST, int use_arrow, const int4* tasks,
                      int ntasks, __half* fdig, int* ecol, const double* cinv, __half* sdig, double* part,
                      int* part_flag, const LaunchCtl& lc, int* fdz = nullptr);

// both: the forward and then the backward sweep in one launch (needs 3 nt B + 2 flags,
// solve_both_fits); trans is then ignored.
void launch_solve(const Geom& g, const double* D, const double* L, const double* R, const double* T,
                  double* Bv, int ldb, int nc, int trans, int use_arrow, double* arrow_part,
                  const LaunchCtl& lc, int both = 0);
inline bool solve_both_fits(const Geom& g) { return 3LL * g.nt * g.B + 2 <= g.nflags(); }

void launch_selinv(const Geom& g, const double* D, const double* L, const double* R, const double* T,
                   double* SD, double* SL, double* SR, double* ST, int use_arrow, const int4* tasks,
                   int ntasks, const double* cinv, const LaunchCtl& lc);

// Selected-inversion pre-pass over the factor (both product methods): replaces every
// off-diagonal pattern tile F(l,c) by G = F(l,c) F(c,c)^{-1} (in place) and writes
// C_c = F(c,c)^{-T} F(c,c)^{-1} per diagonal tile into `ws` (selinv_prepare_bytes).
// With fdig (the digit planes a tensor-core factorization left for every final tile,
// rows relative to erow) the G tiles are formed on the tensor cores, skipping the
// structurally zero coupling tiles of kf (or none: null); without, in FP64.  With GD
// (and GL, GR; tensor-core path only) the G tiles go to those blocks instead and the
// factor's blocks are only read, so the pre-pass can run next to kernels that read them.
size_t selinv_prepare_bytes(const Geom& g);
void launch_selinv_prepare(const Geom& g, const double* D, double* L, double* R, int use_arrow, double* ws,
                           cudaStream_t stream, const __half* fdig = nullptr, const int* erow = nullptr,
                           const int* kf = nullptr, double* GD = nullptr, double* GL = nullptr,
                           double* GR = nullptr);

// Finish of a selected inversion with tensor-core products written in place over the
// factor (its product loops read only digit planes, so Sigma can overwrite the factor
// tiles): mirror each D block's lower tiles into its upper tiles and transpose the
// coupling slots below the separator back to the caller's orientation.
void launch_selinv_finish_inplace(const Geom& g, double* D, double* L, cudaStream_t stream);

void launch_selinv_writeback(const Geom& g, const double* SD, const double* SL, const double* SR,
                             const double* ST, double* D, double* L, double* R, double* T, int use_arrow,
                             cudaStream_t stream);

void launch_logdet(const Geom& g, const double* D, const double* T, int with_tip, double* partial,
                   double* out, cudaStream_t stream);

}  // namespace gbta
