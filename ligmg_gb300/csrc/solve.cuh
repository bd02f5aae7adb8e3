// solve.cuh — solve-phase kernels (SpMM with fused epilogues, transfers,
// column reductions, Krylov updates).  T = float (FP32 hierarchy) or double.
#pragma once
#include "common.cuh"

namespace lg {

// Matrix view used by the solve kernels.  Rows longer than hub_thresh are
// split into chunks processed by separate warps (power-law hub rows); the
// last chunk to finish sums the partials in chunk order and runs the
// epilogue, so results do not depend on scheduling.
template <typename T>
struct MatView {
  i64 n = 0;
  const i64 *rp = nullptr;
  const i32 *ci = nullptr;
  const T *v = nullptr;
  // hub rows
  i64 hub_thresh = 0;      // 0: no hub handling
  i64 nchunks = 0;
  const i64 *ch_row = nullptr, *ch_beg = nullptr, *ch_end = nullptr;
  const i32 *ch_hub = nullptr, *ch_first = nullptr, *ch_cnt = nullptr;
  int *hub_counter = nullptr;  // one per hub row, zero between launches
  T *partial = nullptr;        // nchunks x K
  int lanes_per_row = 32;      // 4, 8, 16 or 32 (single-RHS layout)
  int krow_lanes = 32;         // k = 8 .. 32, a warp per row: 32, or 16 (two rows per warp)
  int tb = 256;                // threads per block of the launch (64, 128 or 256)
  // single right-hand side, tile layout (0 tiles: row layout).  Tile t:
  // tdesc[t] = {first row, rows, e, abase / 4}: its entries are [abase + s,
  // abase + e) with abase the first entry rounded down to a multiple of four,
  // s < 4 and e <= kTilePos.  tbits[t * kTilePos / 32 + w] bit b: entry
  // abase + 32 w + b starts a row of the tile.  Hub rows (longer than a
  // tile holds) are never in a tile.
  i64 ntiles = 0;
  const int4 *tdesc = nullptr;
  const u32 *tbits = nullptr;
  int tile_pipe = 0;  // 1: a resident grid, the next tile fetched during this one's gathers
  // Epi::Split only: the second gathered operand and the first column taken from it
  const T *x2 = nullptr;
  i64 xsplit = 0;
  // k > 1, row streams (0 streams: a warp per row).  Stream w is the rows
  // [srow[w], srow[w + 1]); hub rows in it are left to their chunks.
  // stream_blocks: resident 256-thread blocks per SM of the launch's register
  // budget (5 or 6).
  i64 nstream = 0;
  const i32 *srow = nullptr;
  int stream_blocks = 5;
};

// Hub-row schedule owned by a level (built once at setup).
// A row is split when it holds more than 64 units of U nonzeros, into at most
// 256 chunks of at least 32 units (U from split_unit).
template <typename T>
struct HubPlan {
  i64 thresh = 0, nchunks = 0, nhubs = 0;
  DBuf<i64> row, beg, end;
  DBuf<i32> hub, first, cnt;
  DBuf<int> counter;
  DBuf<T> partial;
  int kcap = 0;
  bool built = false;
  // k = 1 tile layout (MatView::tdesc, tbits); ntiles = 0 when not built
  DBuf<int4> tdesc;
  DBuf<u32> tbits;
  i64 ntiles = 0;
  int tile_pipe = 0;
  // k > 1 row streams (MatView::srow); nstream = 0 when not built
  DBuf<i32> srow;
  i64 nstream = 0;
  int stream_blocks = 5;
  // launch shape kept with the plan (picked by the autotuner or defaults)
  int tb = 256;    // threads per block
  int lanes = 0;   // lanes per row for k = 1 (0: the level's default)
  int krow_lanes = 32;  // lanes per row for k = 8 .. 32 (32 or 16)
  i64 split = 0;   // target entries per chunk: rows longer than 2 x split are
                   // cut into chunks of about split entries (at most 256 chunks)
  // rows longer than `over` entries (default 2 x split_len) are split
  void build(const i64 *rp_host, i64 n, i64 split_len, int kmax, cudaStream_t s, i64 over = 0);
  // k = 1 tile layout: rows longer than a tile holds are hub rows (the split
  // is set so); the other rows are packed into tiles in order
  void build_tiles(const i64 *rp_host, i64 n, cudaStream_t s, int kmax = 1);
  // k > 1 row streams over the rows of this plan (hub rows, already set by
  // build, count as empty): consecutive rows until a stream holds about
  // `per_stream` entries (a row costs its entries plus 16).  Not built
  // (nstream = 0) when the matrix has 2^31 entries or more.
  void build_stream(const i64 *rp_host, i64 n, i64 per_stream, int blocks, cudaStream_t s);
  void fill(MatView<T> &m) const;
};
// Row streams: the first row of every run of consecutive rows holding about
// per_stream entries (a row costs its entries plus 16; rows longer than
// hub_thresh count as empty), then n; empty when the matrix has 2^31 entries
// or rows or more.
std::vector<i32> row_stream_starts(const i64 *rp_host, i64 n, i64 hub_thresh, i64 per_stream);

// Single right-hand side tile layout: at most kTilePos entries (counted from
// the tile's first entry rounded down to a multiple of four) and kTileRows
// rows per tile; a warp takes a tile, a lane 8 consecutive entries.
#ifndef LG_TILE_POS
#define LG_TILE_POS 256
#endif
constexpr int kTilePos = LG_TILE_POS;      // a multiple of 128 (4 entries per lane at least)
constexpr int kTileRows = kTilePos / 8;
// worthwhile from this many nonzeros per row on average
constexpr double kTileMinMeanRow = 6.0;
// Hub split unit U for k right-hand sides: the nonzeros a 32-lane group
// advances per step (E = 32 / (k / VW) entry slots).  The default chunk is
// 32 U entries (eight unrolled steps of four).
int split_unit(int value_bytes, int k);

enum class Epi {
  Store,       // y = A x
  Resid,       // y = b - A x
  ChebA,       // r = b - A x; d = invd r / theta; xo = x + d
  ChebB,       // r' = r - A d; d' = c1 d + c2 invd r'; xo = xi + d'
  ElimInterp,  // y = A x + q .* b   (A = P, x = xc)
  Jacobi,      // y = xi + w invd (b - A x)   (weighted Jacobi sweep, w = c1)
  Split,       // y = A [X; x2]: columns < xsplit gather X, the others x2 (row j - xsplit)
  ChebZ,       // first two Chebyshev steps from x = 0 with A D^-1 values, X = b:
               // d0 = invd b / theta; r = b - (A D^-1 b) / theta;
               // d = c1 d0 + c2 invd r; xo = d0 + d
  FcgDir,      // FCG direction and its product in one pass, X = z:
               // p = (z - mu) - beta pp;  y = A z - mu rowsum(A) - beta qp
               // (= A p, as qp = A pp); pp, qp null on the first iteration
};

struct EpiArgs {
  // generic pointers (type-erased, T*)
  void *y = nullptr;         // Store/Resid/ElimInterp output
  const void *b = nullptr;   // Resid/ChebA/ElimInterp rhs
  const void *invd = nullptr;
  const void *xin = nullptr; // ChebA: x (own row); ChebB: x_{k+1}
  void *xout = nullptr;
  const void *rin = nullptr; // ChebB: r_k (may equal b)
  void *rout = nullptr;      // ChebA/ChebB (nullable in ChebB)
  const void *din = nullptr; // ChebB: d_k (own row)
  void *dout = nullptr;      // ChebA/ChebB (nullable in ChebB)
  const void *q = nullptr;   // ElimInterp diagonal; FcgDir row sums of A
  const void *cmu = nullptr, *cbeta = nullptr;  // FcgDir: per-column mu, beta (k values)
  double ith = 1, c1 = 0, c2 = 0;  // ith = 1 / theta: a product, never an FP64 division
  // float copies of ith, c1, c2 for FP32 epilogues (set by mirror())
  float fith = 1, fc1 = 0, fc2 = 0;
  void mirror() {
    fith = (float)ith;
    fc1 = (float)c1;
    fc2 = (float)c2;
  }
};

// y-epilogue SpMM over k columns (X and all vectors are n x k row-major).
template <typename T>
void spmm(const MatView<T> &A, const T *X, int k, Epi epi, const EpiArgs &a, cudaStream_t s);

// Double-float SpMM for the outer FP64 Krylov product y = A x.  GB300's FP64
// rate makes a k-column FP64 SpMM compute-bound; here every FP64 value is held
// as an unevaluated float pair (hi + lo, 48-bit significand) and products are
// accumulated with error-free transformations (Dekker/Knuth TwoProd/TwoSum via
// FMA) at FP32 throughput.  vdf: nnz (hi, lo) pairs of A's values; X: n x k
// (hi, lo) pairs; Y: n x k doubles.  Hub rows use A's FP64 plan for k.
void spmm_df(const MatView<double> &A, const float2 *vdf, const float2 *X, int k, double *Y,
             cudaStream_t s);
void split_df(i64 count, const double *v, float2 *out, cudaStream_t s);

// elementwise / transfer kernels (n x k row-major)
// d = scale D^-1 b: the first smoothing step from a zero guess
template <typename T>
void cheb_init_zero(i64 n, int k, const T *b, const T *invd, double scale, T *d, cudaStream_t s);
template <typename T>
void fill_value(i64 cnt, T *x, T v, cudaStream_t s);
template <typename T>
void prolong_agg(i64 n, int k, const i32 *agg, const T *xc, T *x, cudaStream_t s);
template <typename T>
void coarse_apply(i64 n, int k, const T *pinv, const T *b, T *x, cudaStream_t s);
template <typename T>
void scale_vec(i64 n, int k, T *x, double f, cudaStream_t s);
template <typename S, typename D>
void convert(i64 count, const S *src, D *dst, cudaStream_t s);

// Column reductions with FP64 accumulation, deterministic (fixed blocks,
// fixed tree, block partials summed in order).  out[c] for c < k.
enum class Red { Sum, Dot, Sum2Dot };  // Sum2Dot: out = [sum(x), x.y] (2k)
template <typename T>
void col_reduce(i64 n, int k, Red op, const T *x, const T *y, double *out, double *scratch,
                i64 scratch_len, cudaStream_t s);
i64 col_reduce_scratch(i64 n, int k);

// Krylov helpers on device scalars (length k arrays of double)
template <typename T>
void sub_mean(i64 n, int k, T *x, const double *colsum, cudaStream_t s);   // x -= sum/n
template <typename T>
void axpby_cols(i64 n, int k, T *y, const T *x, const double *alpha, double sa, double sb,
                cudaStream_t s);  // y = sb*y + sa*alpha[c]*x
// y = coef[c] x (y and x may not overlap)
template <typename T>
void scale_cols(i64 n, int k, T *y, const T *x, const double *coef, cudaStream_t s);
// out[c] = 1 / sqrt(sq[c]), 0 where sq[c] <= 0 (k <= 64 per launch block)
void rsqrt_cols(int k, const double *sq, double *out, cudaStream_t s);
// Inner FGMRES least squares for k columns: H(i, j) at Hb[(i m + j) k + c]
// (i <= j: Arnoldi dot products; i = j + 1: the squared norm), b2 = |b|^2;
// y (m x k) minimises |b| e1 - H y.  m <= kGmresInnerMax.
constexpr int kGmresInnerMax = 16;
void gmres_small(int k, int m, const double *Hb, const double *b2, double *y, cudaStream_t s);
template <typename T>
void fcg_direction(i64 n, int k, T *p, const T *z, const T *pprev, const double *beta,
                   cudaStream_t s);  // p = z - beta p_prev (pprev null: p = z)
template <typename T>
void fcg_update(i64 n, int k, T *x, T *r, const T *p, const T *q, const double *alpha,
                bool update_r, cudaStream_t s, const float *alpha_f = nullptr,
                bool x_zero = false);  // x += a p (x_zero: x = a p); r -= a q (a: alpha_f if set)
template <typename T>
void cg_direction(i64 n, int k, T *p, const T *z, const double *beta, cudaStream_t s);  // p = z + beta p

// Fused FCG steps with one-launch reductions.  A reduction writes one
// partial per block into `scratch`; the last block to finish (ticket counter
// at scratch[0], reset by that block) sums the partials in block order and
// computes the step's scalars, so no second launch and no host round trip.
struct FcgScalars {
  double *mu;        // k: mean of z
  double *beta;      // k
  double *eta;       // k: p.(A p) of this iteration
  double *eta_prev;  // k
  double *alpha;     // k
  const int *frozen; // k or null: alpha forced to 0
  // float copies of mu, beta (written by fcg_beta) and alpha (fcg_alpha) for
  // the elementwise kernels of an FP32 solve, which then convert no FP64
  // scalar per element (GB300's FP64 pipe is narrow); null: none
  float *mu_f = nullptr, *beta_f = nullptr, *alpha_f = nullptr;
};
i64 fused_scratch_len(i64 n, int k);
// mu = sum(z)/n; beta = (z.qp - mu sum(qp)) / eta_prev (beta = 0 if qp null)
template <typename T>
void fcg_beta(i64 n, int k, const T *z, const T *qp, FcgScalars sc, double *scratch,
              cudaStream_t s);
// p = (z - mu) - beta pp   (pp null: p = z - mu); pdf (optional, FP64 only):
// the same p as (hi, lo) float pairs for spmm_df
template <typename T>
void fcg_dir(i64 n, int k, T *p, const T *z, const T *pp, FcgScalars sc, cudaStream_t s,
             float2 *pdf = nullptr);
// eta = p.q; alpha = (p.r)/eta (0 when frozen or eta == 0)
template <typename T>
void fcg_alpha(i64 n, int k, const T *p, const T *q, const T *r, FcgScalars sc,
               double *scratch, cudaStream_t s);
// out = sum(x.y) per column, one launch
template <typename T>
void col_dot1(i64 n, int k, const T *x, const T *y, double *out, double *scratch, cudaStream_t s);

// ---- segment mode (a batch of graphs stored as one block-diagonal matrix) --
// Rows of segment s are [ptr[s], ptr[s+1]); every level keeps segments
// contiguous.  Krylov scalars are per segment (one right-hand side column).
struct SegInfo {
  i64 nseg = 0;
  const i64 *ptr = nullptr;    // nseg + 1 row offsets
  const i32 *rowseg = nullptr; // segment id of every row
};
// One block per segment; the block also computes the step's scalars.
template <typename T>
void seg_fcg_beta(const SegInfo &S, const T *z, const T *qp, FcgScalars sc, cudaStream_t s);
template <typename T>
void seg_fcg_alpha(const SegInfo &S, const T *p, const T *q, const T *r, FcgScalars sc,
                   cudaStream_t s);
template <typename T>
void seg_dot(const SegInfo &S, const T *x, const T *y, double *out, cudaStream_t s);
// out[g] = mean of x over graph g's rows
template <typename T>
void seg_mean(const SegInfo &S, const T *x, double *out, cudaStream_t s);
// x_i -= means[rowseg[i]]
template <typename T>
void seg_sub_mean(const SegInfo &S, i64 n, T *x, const double *means, cudaStream_t s);
template <typename T>
void seg_fcg_dir(const SegInfo &S, i64 n, T *p, const T *z, const T *pp, FcgScalars sc,
                 cudaStream_t s, float2 *pdf = nullptr);
template <typename T>
void seg_fcg_update(const SegInfo &S, i64 n, T *x, T *r, const T *p, const T *q,
                    const double *alpha, bool update_r, cudaStream_t s);
// device-side convergence: frozen[s] |= rn2[s] <= tol^2 rn0sq[s]; iters[s] set
// to `it` + 1 for segments still active after this iteration
void seg_converge(i64 nseg, const double *rn2, const double *rn0sq, double tol, int it,
                  int *frozen, int *iters, cudaStream_t s);

// scalar kernels on device (k columns)
void scal_div(int k, const double *num, const double *den, double *out, const int *frozen,
              cudaStream_t s);  // out = frozen ? 0 : num/den (0 when den == 0)
void scal_beta(int k, const double *zq, const double *eta_prev, double *beta, cudaStream_t s);

}  // namespace lg
