// api.cu — host driver of the GB300 LigMG solver and its C ABI.
//
//   ligmg_create  : make_hierarchy (include/ligmg/multigrid.hpp:162-263) on the
//                   GPU: elimination, aggregation, Galerkin products, Chebyshev
//                   eigenvalue estimates and the coarse pseudo-inverse.
//   ligmg_solve*  : solve (multigrid.hpp:316-370): top elimination, outer
//                   FP64 CG/FCG (cg.hpp:18-116) preconditioned by a V- or
//                   K-cycle (multigrid.hpp:87-130) in FP64 or FP32.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <type_traits>
#include <memory>
#include <new>

#include "prims.cuh"
#include "setup.cuh"
#include "solve.cuh"
#include "prep.cuh"
#include "tail.cuh"
#include "queue.cuh"
#include "peaks.cuh"

namespace lg {
namespace {

// glibc rand() (TYPE_3 additive feedback generator), restated from its
// published description: r[0] = seed (1 if 0); r[i] = 16807 r[i-1] mod
// (2^31 - 1) (Schrage) for i < 31; r[i] = r[i-31] for i = 31..33;
// r[i] = r[i-3] + r[i-31] mod 2^32; output k is r[k + 344] >> 1.
// The reference draws its test vectors with rand() (combblas_extra.hpp:186-192).
struct GlibcRand {
  uint32_t ring[32];
  i64 i = 0;
  explicit GlibcRand(uint32_t seed) {
    int32_t r[34];
    r[0] = (int32_t)(seed == 0 ? 1u : seed);
    for (int k = 1; k < 31; k++) {
      int32_t hi = r[k - 1] / 127773, lo = r[k - 1] % 127773;
      int32_t word = 16807 * lo - 2836 * hi;
      if (word < 0) word += 2147483647;
      r[k] = word;
    }
    for (int k = 31; k < 34; k++) r[k] = r[k - 31];
    for (int k = 0; k < 34; k++) ring[k & 31] = (uint32_t)r[k];
    i = 34;
    for (int k = 34; k < 344; k++) raw();
  }
  uint32_t raw() {
    uint32_t v = ring[(i - 31) & 31] + ring[(i - 3) & 31];
    ring[i & 31] = v;
    i++;
    return v;
  }
  int32_t next() { return (int32_t)(raw() >> 1); }
};

// right-hand side of the eigenvalue estimate (hash of the row index)
inline double est_rhs(i64 i) {
  uint32_t x = (uint32_t)i * 2654435761u + 0x9E3779B9u;
  x ^= x >> 16;
  x *= 0x85EBCA6Bu;
  x ^= x >> 13;
  x *= 0xC2B2AE35u;
  x ^= x >> 16;
  return (double)x * (1.0 / 4294967296.0) - 0.5;
}

double tridiag_lmax(const std::vector<double> &d, const std::vector<double> &e) {
  int m = (int)d.size();
  if (m == 0) return 0.0;
  double lo = d[0], hi = d[0];
  for (int i = 0; i < m; i++) {
    double r = 0;
    if (i > 0) r += std::fabs(e[i - 1]);
    if (i + 1 < m) r += std::fabs(e[i]);
    lo = std::min(lo, d[i] - r);
    hi = std::max(hi, d[i] + r);
  }
  for (int it = 0; it < 200; it++) {
    double mid = 0.5 * (lo + hi);
    if (mid <= lo || mid >= hi) break;
    int cnt = 0;
    double q = 1.0;
    for (int i = 0; i < m; i++) {
      double off = (i > 0) ? e[i - 1] * e[i - 1] : 0.0;
      q = d[i] - mid - ((i > 0) ? off / q : 0.0);
      if (q == 0.0) q = -1e-300;
      if (q < 0) cnt++;
    }
    if (cnt == m) hi = mid; else lo = mid;
  }
  return hi;
}

__global__ void k_ad_values(i64 nnz, const i32 *ci, const double *v, const double *invd,
                            double *ad) {
  const i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nnz) ad[t] = v[t] * invd[ci[t]];
}

// rs_i = sum of row i's stored values (in column order, accumulated in FP64)
template <typename V>
__global__ void k_rowsum(const i64 *rp, const V *v, i64 n, V *rs) {
  i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double t = 0;
  for (i64 k = rp[i]; k < rp[i + 1]; k++) t += (double)v[k];
  rs[i] = (V)t;
}

__global__ void k_invdiag(const i64 *rp, const i32 *ci, const double *v, i64 n, double *invd) {
  i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  i64 lo = rp[i], hi = rp[i + 1];
  while (lo < hi) {
    i64 mid = (lo + hi) >> 1;
    if (ci[mid] < i) lo = mid + 1; else hi = mid;
  }
  double d = v[lo];
  invd[i] = d > 0 ? 1.0 / d : 0.0;  // a one-vertex component of a batch has d = 0
}

// dloss/dw_ij = -(x_i - x_j)(lambda_i - lambda_j) for each stored off-diagonal
// entry; one warp per row
__global__ void k_edge_grad(const i64 *rp, const i32 *ci, i64 n, const double *x,
                            const double *lam, double *dw) {
  i64 i = ((i64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= n) return;
  double xi = x[i], li = lam[i];
  for (i64 e = rp[i] + (threadIdx.x & 31); e < rp[i + 1]; e += 32) {
    i32 j = ci[e];
    dw[e] = (j == i) ? 0.0 : -(xi - x[j]) * (li - lam[j]);
  }
}

// segment offsets of the next level: the first new id inside each segment.
// A graph of the batch can vanish from a level (a lone vertex eliminated),
// so trailing segments may be empty and start at n, past the scan's end:
// they start at nc on the next level.
__global__ void k_gather_offsets(const i32 *scan, const i64 *seg_in, i64 nseg, i64 n, i64 nc,
                                 i64 *seg_out) {
  i64 sg = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (sg > nseg) return;
  seg_out[sg] = (sg == nseg || seg_in[sg] >= n) ? nc : (i64)scan[seg_in[sg]];
}

__global__ void k_fill_rowseg(const i64 *segptr, i64 nseg, i64 n, i32 *rowseg) {
  i64 r = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  i64 lo = 0, hi = nseg - 1;  // largest sg with segptr[sg] <= r
  while (lo < hi) {
    i64 mid = (lo + hi + 1) >> 1;
    if (segptr[mid] <= r) lo = mid; else hi = mid - 1;
  }
  rowseg[r] = (i32)lo;
}

// every row's columns must stay inside its segment (block-diagonal batch)
__global__ void k_check_blockdiag(const i64 *rp, const i32 *ci, i64 n, const i32 *rowseg,
                                  const i64 *segptr, int *bad) {
  i64 r = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  i32 sg = rowseg[r];
  i64 lo = segptr[sg], hi = segptr[sg + 1];
  for (i64 e = rp[r]; e < rp[r + 1]; e++)
    if (ci[e] < lo || ci[e] >= hi) {
      *bad = 1;
      return;
    }
}

__global__ void k_mul_diag(i64 n, const double *d, const double *x, double *y) {
  i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = d[i] * x[i];
}

}  // namespace

// ---------------------------------------------------------------------------
struct Level {
  int type = LIGMG_LEVEL_AGG;
  DCsr<double> A;
  i64 nc = 0;
  double lmax = 0;
  DBuf<double> invd;
  ElimResult elim;
  AggResult agg;
  DBuf<double> pinv;
  // FP32 copies for the FP32 hierarchy
  bool has32 = false;
  DBuf<float> Av32, invd32, Pv32, Rv32, Q32, pinv32;
  DBuf<float2> Adf;  // (hi, lo) float pairs of A's FP64 values (outer product)
  // aggregation levels: unit values of the member matrix R (nc x n, rows
  // agg.mrp / agg.members), so restriction runs through the hub-split SpMM
  DBuf<double> ones64;
  DBuf<float> ones32;
  // aggregation levels: C = [R | -R A] (nc x 2n), the residual and its
  // restriction in one SpMM: bc = C [b; x]
  DCsr<double> Cr;
  DBuf<float> Cr32;
  // A D^-1 values (a_ij / a_jj): the first Chebyshev step from a zero guess
  // gathers b itself (A d0 = A D^-1 b / theta)
  DBuf<double> ADv;
  DBuf<float> AD32;
  // row sums of A's stored values (zero up to rounding for a Laplacian): the
  // fused FCG direction product uses A (z - mu 1) = A z - mu rs
  DBuf<double> rs64;
  DBuf<float> rs32;
  // hub-row plans: hubA64 (FP64, k = 1) is built at setup; the others are
  // built on first use per (precision, k) from the cached host row pointers
  HubPlan<double> hubA64;
  mutable std::map<int, HubPlan<double>> hA64k, hR64k, hC64k;
  mutable std::map<int, HubPlan<float>> hA32k, hR32k, hC32k;
  std::vector<i64> rp_host, rrp_host, crp_host;
  int lanesA = 32, lanesR = 32, lanesP = 4, lanesC = 32;
  bool autotune = true;  // options.autotune at creation
  int tiles = 1;         // options.spmv_tiles at creation
  int streams = 1;       // options.spmm_streams at creation
  // row streams of A for the double-float outer product (built on first use;
  // -1: not yet, 0: none)
  DBuf<i32> dfsrow;
  i64 dfnstream = -1;
  int ktiles = 1;        // options.spmm_tiles at creation
  // Chebyshev coefficients
  double theta = 1, delta = 1;
  std::vector<double> c1, c2;

  // batch mode: rows of segment (graph) s are [seg_host[s], seg_host[s+1])
  std::vector<i64> seg_host;
  DBuf<i64> segptr;
  DBuf<i32> rowseg;
  SegInfo seginfo() const {
    SegInfo S;
    S.nseg = seg_host.empty() ? 0 : (i64)seg_host.size() - 1;
    S.ptr = segptr.p;
    S.rowseg = rowseg.p;
    return S;
  }

  bool is_exact() const { return type == LIGMG_LEVEL_ELIM; }
  i64 work(const ligmg_options &o) const {
    if (type == LIGMG_LEVEL_AGG)
      return (i64)(o.pre_smooth + o.post_smooth + 1) * A.nnz + 3 * A.n;
    if (type == LIGMG_LEVEL_ELIM) return elim.P.nnz + elim.R.nnz + (A.n - elim.nc);
    return A.nnz;
  }
};

int lanes_for(i64 nnz, i64 n) {
  double m = n ? (double)nnz / (double)n : 0;
  if (m <= 4.5) return 4;
  if (m <= 9) return 8;
  if (m <= 18) return 16;
  return 32;
}


// matrices of a level that have hub plans
enum Mat : int { MAT_A = 0, MAT_R = 1, MAT_C = 2 };

template <typename T>
std::map<int, HubPlan<T>> &plans(const Level &L, int which);
template <>
std::map<int, HubPlan<double>> &plans<double>(const Level &L, int which) {
  return which == MAT_C ? L.hC64k : which == MAT_R ? L.hR64k : L.hA64k;
}
template <>
std::map<int, HubPlan<float>> &plans<float>(const Level &L, int which) {
  return which == MAT_C ? L.hC32k : which == MAT_R ? L.hR32k : L.hA32k;
}
inline const std::vector<i64> &plan_rows(const Level &L, int which) {
  return which == MAT_C ? L.crp_host : which == MAT_R ? L.rrp_host : L.rp_host;
}

template <typename T>
const T *valsA(const Level &L);
template <typename T>
const T *valsR(const Level &L);
template <typename T>
const T *valsC(const Level &L) {
  if constexpr (sizeof(T) == 8) return (const T *)L.Cr.v.p;
  else return (const T *)L.Cr32.p;
}

// The level's matrix A, its restriction R or its fused residual restriction
// C (x2 unset), without a hub plan.
template <typename T>
MatView<T> bare_view(const Level &L, int which) {
  MatView<T> m;
  if (which == MAT_C) {
    m.n = L.Cr.n; m.rp = L.Cr.rp.p; m.ci = L.Cr.ci.p; m.v = valsC<T>(L);
    m.lanes_per_row = L.lanesC;
    m.xsplit = L.A.n;
  } else if (which == MAT_A) {
    m.n = L.A.n; m.rp = L.A.rp.p; m.ci = L.A.ci.p; m.v = valsA<T>(L); m.lanes_per_row = L.lanesA;
  } else if (L.type == LIGMG_LEVEL_AGG) {
    m.n = L.nc; m.rp = L.agg.mrp.p; m.ci = L.agg.members.p; m.v = valsR<T>(L);
    m.lanes_per_row = L.lanesR;
  } else {
    m.n = L.elim.R.n; m.rp = L.elim.R.rp.p; m.ci = L.elim.R.ci.p; m.v = valsR<T>(L);
    m.lanes_per_row = L.lanesR;
  }
  return m;
}

// SpMM launch-shape autotuner.  On first use of a (level, matrix, precision,
// k), every candidate shape is timed on this level's own matrix (y = A x,
// x = 0, one warm-up and three timed launches on the handle's stream) and the
// fastest is kept with the plan:
//   chunk size       split unit U x {8, 16, 32, 64, 128} entries (rows over
//                    twice that are cut): long rows stay whole on levels
//                    with many rows; on levels of at most 2^17 rows, where a
//                    launch has too few warps to hide the gather latency,
//                    rows of a few dozen entries are cut into several
//                    warps' chunks (8 U and 16 U are tried there only)
//   threads/block    {64, 128, 256}: small blocks free their slot as soon as
//                    their rows finish (rows differ widely in length)
//   lanes per row    {4, 8, 16, 32} for k = 1 on levels without hub rows;
//                    32 or 16 (two rows per warp) for k = 8 .. 32
//   k-column tiles   rows of at most 128 bytes: tiles of whole rows in steps
//                    of consecutive entries (k_spmm_ktile)
//   row streams      k >= 8: the row-stream kernel (a warp per run of
//                    consecutive rows; 1, 2, 4 or 8 runs per resident warp;
//                    five or six resident blocks per SM) against a warp per
//                    row
// The choice only changes launch shapes and, on hub rows, how a row's sum is
// split into chunk partials (its rounding); autotune = 0 uses the defaults
// (chunks of 32 U, 64 threads for k > 1, 256 for k = 1, the level's lanes).
template <typename T>
void build_plan(const Level &L, int which, int k, HubPlan<T> &best, bool autotune,
                cudaStream_t s) {
  const std::vector<i64> &rp = plan_rows(L, which);
  const i64 n = (i64)rp.size() - 1;
  const int unit = split_unit(sizeof(T), k);
  // the single right-hand side tile layout, for matrices whose rows fill a
  // lane's run of entries on average
  const bool tile_ok = k == 1 && L.tiles && n > 0 &&
                       (double)(rp[n] - rp[0]) >= kTileMinMeanRow * (double)n;
  // k columns: tiles of whole rows for rows of at most 128 bytes
  const bool ktile_ok = k >= 2 && k * (int)sizeof(T) <= 128 && L.ktiles != 0 && n > 0;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  LG_CUDA(cudaStreamIsCapturing(s, &cs));
  if (!autotune || cs != cudaStreamCaptureStatusNone || n <= 0) {
    if (tile_ok) {
      best.build_tiles(rp.data(), n, s);
      best.tile_pipe = L.tiles == 2;
    } else {
      best.build(rp.data(), n, 32 * (i64)unit, k, s);
    }
    best.tb = k > 1 ? 64 : 256;
    if (k >= 8 && L.streams == 2 && n > 0) best.build_stream(rp.data(), n, 2048, 5, s);
    if (ktile_ok && L.ktiles == 2) {
      HubPlan<T> cand;
      cand.build_tiles(rp.data(), n, s, k);
      if (cand.ntiles > 0) best = std::move(cand);
    }
    return;
  }
  MatView<T> base = bare_view<T>(L, which);
  DBuf<T> X(L.A.n * k, s), Y(n * k, s);
  X.zero();
  // the yardstick: A's k-column plans are timed on the smoother's most
  // frequent product (a later Chebyshev step: r, d, x and D^-1 read, x
  // written), whose epilogue traffic separates the layouts; the others on
  // their own epilogue (C: the residual restriction) or y = A x
  const bool cheb = which == MAT_A && k > 1;
  const Epi epi = which == MAT_C ? Epi::Split : (cheb ? Epi::ChebB : Epi::Store);
  if (which == MAT_C) base.x2 = X.p;  // both halves of the operand
  DBuf<T> Rv, Xv, invd;
  if (cheb) {
    Rv.alloc(n * k, s);
    Rv.zero();
    Xv.alloc(n * k, s);
    Xv.zero();
    invd.alloc(n, s);
    invd.zero();
  }
  auto bench_args = [&] {
    EpiArgs a;
    a.y = Y.p;
    if (cheb) {
      a.rin = Rv.p;
      a.din = X.p;
      a.xin = Xv.p;
      a.xout = Y.p;
      a.invd = invd.p;
    }
    return a;
  };
  cudaEvent_t e0, e1;
  LG_CUDA(cudaEventCreate(&e0));
  LG_CUDA(cudaEventCreate(&e1));
  float best_ms = 1e30f;
  bool have = false;
  bool chunks_seen = true;
  for (int f : {8, 16, 32, 64, 128}) {
    if (!chunks_seen) break;  // no long rows at a smaller split: none at larger ones
    // the finer cuts only pay where a launch has few warps for its rows
    if (f < 32 && n > (i64)131072) continue;
    HubPlan<T> cand;
    cand.build(rp.data(), n, (i64)unit * f, k, s);
    chunks_seen = cand.nchunks > 0;
    std::vector<int> lane_opts{0};
    if (k == 1 && cand.nchunks == 0) lane_opts = {4, 8, 16, 32};
    // k = 8 .. 32 without hub rows: also two rows per warp (16 lanes each)
    const bool half = k >= 8 && k <= 32 && cand.nchunks == 0;
    if (half) lane_opts = {0, 16};
    float cand_ms = 1e30f;
    int cand_tb = 256, cand_lanes = 0;
    for (int lanes : lane_opts)
      for (int tb : {64, 128, 256}) {
        MatView<T> m = base;
        cand.fill(m);
        m.tb = tb;
        if (half) m.krow_lanes = lanes ? lanes : 32;
        else if (lanes) m.lanes_per_row = lanes;
        EpiArgs a = bench_args();
        spmm<T>(m, X.p, k, epi, a, s);
        LG_CUDA(cudaEventRecord(e0, s));
        for (int r = 0; r < 3; r++) spmm<T>(m, X.p, k, epi, a, s);
        LG_CUDA(cudaEventRecord(e1, s));
        LG_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        LG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < cand_ms) {
          cand_ms = ms;
          cand_tb = tb;
          cand_lanes = lanes;
        }
      }
    // k >= 8: the row-stream kernel at five or six resident blocks per SM,
    // with 1, 2, 4 or 8 streams per resident warp of the five-block launch
    // (stream lengths from the level's own cost: entries plus 16 per row)
    i64 cand_ps = 0;
    int cand_sb = 0;
    if (k >= 8 && L.streams != 0) {
      const i64 cost = (rp[n] - rp[0]) + 16 * n;
      const i64 resident = (i64)kSMs * 5 * 8;
      std::vector<i64> lens;
      for (int c : {1, 2, 4, 8}) {
        const i64 ps = std::max<i64>(64, cdiv(cost, resident * c));
        if (lens.empty() || ps != lens.back()) lens.push_back(ps);
      }
      for (i64 ps : lens) {
        cand.build_stream(rp.data(), n, ps, 5, s);
        if (cand.nstream == 0) break;
        for (int sb : {5, 6}) {
          MatView<T> m = base;
          cand.fill(m);
          m.stream_blocks = sb;
          EpiArgs a = bench_args();
          spmm<T>(m, X.p, k, epi, a, s);
          LG_CUDA(cudaEventRecord(e0, s));
          for (int r = 0; r < 3; r++) spmm<T>(m, X.p, k, epi, a, s);
          LG_CUDA(cudaEventRecord(e1, s));
          LG_CUDA(cudaEventSynchronize(e1));
          float ms = 0;
          LG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
          if (ms < cand_ms) {
            cand_ms = ms;
            cand_ps = ps;
            cand_sb = sb;
          }
        }
      }
      if (cand_ps > 0) cand.build_stream(rp.data(), n, cand_ps, cand_sb, s);
      else cand.nstream = 0;
    }
    if (!have || cand_ms < best_ms) {
      best = std::move(cand);
      best.tb = cand_tb;
      best.lanes = half ? 0 : cand_lanes;
      best.krow_lanes = half && cand_lanes ? cand_lanes : 32;
      best_ms = cand_ms;
      have = true;
    }
  }
  if (k >= 8 && L.streams == 2 && best.nstream == 0) best.build_stream(rp.data(), n, 2048, 5, s);
  if (ktile_ok) {
    HubPlan<T> cand;
    cand.build_tiles(rp.data(), n, s, k);
    if (cand.ntiles > 0) {
      MatView<T> m = base;
      cand.fill(m);
      EpiArgs a = bench_args();
      spmm<T>(m, X.p, k, epi, a, s);
      LG_CUDA(cudaEventRecord(e0, s));
      for (int r = 0; r < 3; r++) spmm<T>(m, X.p, k, epi, a, s);
      LG_CUDA(cudaEventRecord(e1, s));
      LG_CUDA(cudaEventSynchronize(e1));
      float ms = 0;
      LG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      if (!have || ms < best_ms || L.ktiles == 2) {
        best = std::move(cand);
        best.tb = 256;
        best_ms = ms;
        have = true;
      }
    }
  }
  if (tile_ok) {
    HubPlan<T> cand;
    cand.build_tiles(rp.data(), n, s);
    if (cand.ntiles > 0) {
      // a warp per tile, or the pipelined resident grid
      float tms = 1e30f;
      int tpipe = 0;
      for (int pipe : {0, 1}) {
        if (L.tiles == 2 && pipe == 0) continue;  // pipelined tiles only
        MatView<T> m = base;
        cand.fill(m);
        m.tile_pipe = pipe;
        EpiArgs a = bench_args();
        spmm<T>(m, X.p, k, epi, a, s);
        LG_CUDA(cudaEventRecord(e0, s));
        for (int r = 0; r < 3; r++) spmm<T>(m, X.p, k, epi, a, s);
        LG_CUDA(cudaEventRecord(e1, s));
        LG_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        LG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < tms) {
          tms = ms;
          tpipe = pipe;
        }
      }
      if (!have || tms < best_ms || L.tiles == 2) {
        best = std::move(cand);
        best.tb = 256;
        best.tile_pipe = tpipe;
        best_ms = tms;
        have = true;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  LG_CUDA(cudaStreamSynchronize(s));
}

template <typename T>
const HubPlan<T> &plan_for(const Level &L, int which, int k, cudaStream_t s) {
  if constexpr (sizeof(T) == 8) {
    if (which == MAT_A && k == 1) return L.hubA64;
  }
  HubPlan<T> &p = plans<T>(L, which)[k];
  if (!p.built) build_plan<T>(L, which, k, p, L.autotune, s);
  return p;
}

// The view of A for the double-float outer product with k columns: A's
// hub-row chunks (from the FP64 plan for k) and, for k >= 8, row streams of
// its other rows, one run per four resident warps' worth of entries (built
// on first use, outside graph capture).
MatView<double> df_view(Level &L, MatView<double> A, int k, cudaStream_t s) {
  if (k < 8 || L.streams == 0) return A;
  if (L.dfnstream < 0) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    LG_CUDA(cudaStreamIsCapturing(s, &cs));
    if (cs != cudaStreamCaptureStatusNone) return A;
    const i64 n = A.n;
    const i64 cost = (L.rp_host[n] - L.rp_host[0]) + 16 * n;
    const i64 per = std::max<i64>(64, cdiv(cost, (i64)kSMs * 4 * 8 * 4));
    std::vector<i32> st = row_stream_starts(L.rp_host.data(), n, A.hub_thresh, per);
    L.dfnstream = st.size() >= 2 ? (i64)st.size() - 1 : 0;
    if (L.dfnstream > 0) {
      L.dfsrow.alloc((i64)st.size(), s);
      L.dfsrow.upload(st.data(), (i64)st.size());
      LG_CUDA(cudaStreamSynchronize(s));
    }
  }
  A.nstream = L.dfnstream;
  A.srow = L.dfsrow.p;
  return A;
}

template <typename T>
const T *valsA(const Level &L) {
  if constexpr (sizeof(T) == 8) return (const T *)L.A.v.p;
  else return (const T *)L.Av32.p;
}
template <typename T>
const T *valsR(const Level &L) {
  if (L.type == LIGMG_LEVEL_AGG) {
    if constexpr (sizeof(T) == 8) return (const T *)L.ones64.p;
    else return (const T *)L.ones32.p;
  }
  if constexpr (sizeof(T) == 8) return (const T *)L.elim.R.v.p;
  else return (const T *)L.Rv32.p;
}

template <typename T>
MatView<T> viewA(const Level &L, int k, cudaStream_t s) {
  MatView<T> m = bare_view<T>(L, false);
  plan_for<T>(L, false, k, s).fill(m);
  return m;
}
template <typename T>
MatView<T> viewAD(const Level &L, int k, cudaStream_t s) {
  MatView<T> m = bare_view<T>(L, MAT_A);
  plan_for<T>(L, MAT_A, k, s).fill(m);
  if constexpr (sizeof(T) == 8) m.v = (const T *)L.ADv.p;
  else m.v = (const T *)L.AD32.p;
  return m;
}
template <typename T>
MatView<T> viewR(const Level &L, int k, cudaStream_t s) {
  MatView<T> m = bare_view<T>(L, MAT_R);
  plan_for<T>(L, MAT_R, k, s).fill(m);
  return m;
}
// C with its second operand: bc = C [b; x] = R (b - A x)
template <typename T>
MatView<T> viewC(const Level &L, int k, const T *x, cudaStream_t s) {
  MatView<T> m = bare_view<T>(L, MAT_C);
  plan_for<T>(L, MAT_C, k, s).fill(m);
  m.x2 = x;
  return m;
}
template <typename T>
MatView<T> viewP(const Level &L) {
  MatView<T> m;
  m.n = L.elim.P.n; m.rp = L.elim.P.rp.p; m.ci = L.elim.P.ci.p;
  if constexpr (sizeof(T) == 8) m.v = (const T *)L.elim.P.v.p;
  else m.v = (const T *)L.Pv32.p;
  m.lanes_per_row = L.lanesP;
  return m;
}
template <typename T>
const T *invdT(const Level &L) {
  if constexpr (sizeof(T) == 8) return (const T *)L.invd.p;
  else return (const T *)L.invd32.p;
}
template <typename T>
const T *rowsumT(const Level &L) {
  if constexpr (sizeof(T) == 8) return (const T *)L.rs64.p;
  else return (const T *)L.rs32.p;
}
template <typename T>
const T *QT(const Level &L) {
  if constexpr (sizeof(T) == 8) return (const T *)L.elim.Q.p;
  else return (const T *)L.Q32.p;
}
template <typename T>
const T *pinvT(const Level &L) {
  if constexpr (sizeof(T) == 8) return (const T *)L.pinv.p;
  else return (const T *)L.pinv32.p;
}

// per-level scalar slots (k doubles each)
// S_F32: float copies of mu, beta and alpha (3 k floats) for FP32 levels
enum Slot { S_SUM = 0, S_ZQ, S_BETA, S_ETA0, S_ETA1, S_RHO, S_ALPHA, S_PQR, S_F32, S_NSLOT };

template <typename T>
struct LevelWork {
  i64 n = 0;
  DBuf<T> in, out, r, d0, d1, xt;           // cycle buffers
  DBuf<T> fz, fp0, fp1, fq0, fq1;           // K-cycle FCG buffers (fr = in, fx = out)
  DBuf<T> gV, gZ, gW;                       // K-cycle FGMRES: basis, preconditioned basis, A z
  DBuf<double> gH;                          // K-cycle FGMRES scalars
  DBuf<double> sc, scratch, fscratch;
  DBuf<double> segsc;  // batch mode: S_NSLOT x nseg scalars
  i64 scratch_len = 0, nseg = 0;
  double *slot(int s, int k) { return sc.p + (i64)s * k * 2; }
  double *sslot(int s) { return segsc.p + (i64)s * nseg; }
};

// The recorded coarse-tail program of one Work (k columns).
template <typename T>
struct TailState {
  bool planned = false; // start level decided
  bool tried = false;   // program built and timed
  bool decided = false; // autotune: kept or dropped against the launched levels
  bool on = false;
  float best_ms = 0;    // autotune: time of one launch in the chosen shape
  int start = 0;        // first level of the tail (0: none)
  bool smem_mode = false;
  bool cluster = false; // shared-memory mode in clusters (sl.cluster CTAs per slice)
  int G = 0;            // grid mode: CTAs of the cooperative launch
  int nops = 0;
  double bytes = 0;     // compulsory bytes of a visit: its input and output
                        // vectors and one read of every tail level's matrix
  TailSmemLaunch sl;    // shared-memory mode launch (image in `image`)
  DBuf<unsigned char> image;
  DBuf<TOp<T>> ops;
  DBuf<double> partial;
  DBuf<TailSync> sync;
};

template <typename T>
struct Work {
  int k = 0;
  std::vector<LevelWork<T>> lw;
  TailState<T> tail;
};

// batch-mode outer scalars (one per graph)
struct SegOuter {
  DBuf<double> sc, rn2, rn0sq;
  DBuf<int> frozen, iters;
  DBuf<float2> Pdf;
};

struct OuterWork {
  SegOuter so;
  int k = 0;
  i64 n = 0;
  DBuf<double> X, R, Z, P0, P1, Q0, Q1, B, Bfull, Xfull, Res, sc, scratch, fscratch;
  DBuf<float2> Pdf;
  DBuf<int> frozen;
  i64 scratch_len = 0;
  // FGMRES: Arnoldi basis V (m+1 blocks of n x k), preconditioned basis Z
  // (m blocks), the new direction, dot products and per-column coefficients
  DBuf<double> fgV, fgZ, fgW, fgH, fgC;
  double *slot(int s) { return sc.p + (i64)s * k * 2; }
};

// Batch solves on the persistent work-queue kernel: the recorded programs
// (outer iterations 0..15, and 16..31 for every later launch) and the state
// of a launch.
struct QueueProgram {
  DBuf<QOp> ops;
  DBuf<unsigned long long> items;
  unsigned long long nitems = 0;
  cudaGraphExec_t exec = nullptr;  // state reset + the launch, captured once
  ~QueueProgram() {
    if (exec) cudaGraphExecDestroy(exec);
  }
};
struct QueueRun {
  size_t base = 0;
  int prec = -1;
  QueueProgram first, more;
  DBuf<const i64 *> segs;
  DBuf<int> prog, blk;
  DBuf<double> part;
  DBuf<QueueState> st;
};

// per-kernel event timing (ligmg_profile_enable / ligmg_kernel_stats)
struct ProfRec {
  int level, kind, k, fp64;
  cudaEvent_t a, b;
  double bytes;
  bool graph_owned;  // events belong to a captured graph (re-recorded per replay)
};
struct Profiler {
  bool on = false;
  bool capturing = false;
  bool suspended = false;  // no records while capturing a whole batch solve
  std::vector<ProfRec> capture_tmpl;
  std::vector<cudaEvent_t> pool;
  std::vector<ProfRec> pending;
  std::map<std::tuple<int, int, int, int>, ligmg_kernel_stat> stats;
  cudaEvent_t get() {
    if (!pool.empty()) {
      cudaEvent_t e = pool.back();
      pool.pop_back();
      return e;
    }
    cudaEvent_t e;
    LG_CUDA(cudaEventCreate(&e));
    return e;
  }
  void collect() {
    if (pending.empty()) return;
    LG_CUDA(cudaEventSynchronize(pending.back().b));
    for (auto &r : pending) {
      float ms = 0;
      LG_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
      auto key = std::make_tuple(r.level, r.kind, r.k, r.fp64);
      auto it = stats.find(key);
      if (it == stats.end()) {
        ligmg_kernel_stat z{};
        z.level = r.level; z.kind = r.kind; z.k = r.k; z.fp64 = r.fp64;
        it = stats.emplace(key, z).first;
      }
      it->second.launches += 1;
      it->second.seconds += ms * 1e-3;
      it->second.bytes += r.bytes;
      if (!r.graph_owned) {
        pool.push_back(r.a);
        pool.push_back(r.b);
      }
    }
    pending.clear();
  }
  ~Profiler() {
    for (auto &r : pending)
      if (!r.graph_owned) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
    for (auto e : pool) cudaEventDestroy(e);
  }
};

// A preconditioner application captured as a CUDA graph (one per k,
// precision, base level and profiling state).
struct PrecGraph {
  cudaGraphExec_t exec = nullptr;
  const double *r = nullptr;
  double *z = nullptr;
  bool prof = false;
  int64_t kernels = 0;  // library kernels recorded in the graph
  std::vector<ProfRec> tmpl;
  void reset() {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
    for (auto &t : tmpl) {
      cudaEventDestroy(t.a);
      cudaEventDestroy(t.b);
    }
    tmpl.clear();
  }
};

}  // namespace lg

struct ligmg_handle_s {
  std::map<std::tuple<int, int, int>, lg::PrecGraph> pgraphs;
  // batch mode: vertex offsets of the graphs in the block-diagonal input
  std::vector<lg::i64> seg0;
  cudaGraphExec_t batch_first = nullptr, batch_more = nullptr;  // whole-solve graphs
  int64_t batch_first_kernels = 0, batch_more_kernels = 0;
  size_t batch_base = 0;
  lg::DBuf<double> fwd_x;  // forward solution kept for ligmg_backward
  bool has_fwd = false;
  lg::Profiler prof;
  ligmg_options opts;
  int device = 0;
  cudaStream_t s = nullptr;
  bool own_stream = true;
  std::vector<cudaStream_t> old_streams;
  std::vector<std::unique_ptr<lg::Level>> h;
  lg::i64 nnz0 = 0;
  double setup_s = 0;
  double setup_phase[LIGMG_SETUP_NPHASES] = {0};  // seconds per setup phase
  std::map<int, std::unique_ptr<lg::Work<float>>> w32;
  std::map<int, std::unique_ptr<lg::Work<double>>> w64;
  std::map<int, std::unique_ptr<lg::OuterWork>> ow;
  std::unique_ptr<lg::QueueRun> queue;  // batch solves on the work-queue kernel
  ~ligmg_handle_s() {
    // Buffers keep the stream they were allocated on, which may be a stream
    // that is destroyed below or a caller's stream that no longer exists.
    // After the handle's streams are idle, every buffer is therefore freed
    // with a synchronous cudaFree, and all of them (fwd_x included) before
    // any stream is destroyed.
    if (s) cudaStreamSynchronize(s);
    for (auto o : old_streams) cudaStreamSynchronize(o);
    lg::SyncFreeScope sync_free;
    for (auto &g : pgraphs) g.second.reset();
    pgraphs.clear();
    if (batch_first) cudaGraphExecDestroy(batch_first);
    if (batch_more) cudaGraphExecDestroy(batch_more);
    queue.reset();
    w32.clear();
    w64.clear();
    ow.clear();
    h.clear();
    fwd_x.release();
    for (auto o : old_streams) cudaStreamDestroy(o);
    if (s && own_stream) cudaStreamDestroy(s);
  }
};

namespace lg {
namespace {

using Handle = ligmg_handle_s;

template <typename F>
void timed(Handle &H, int level, int kind, int k, int fp64, double bytes, F &&f) {
  if (!H.prof.on || H.prof.suspended) {
    f();
    return;
  }
  if (H.prof.capturing) {  // event-record nodes owned by the graph
    cudaEvent_t a, b;
    LG_CUDA(cudaEventCreate(&a));
    LG_CUDA(cudaEventCreate(&b));
    // inside a capture a plain record is only a dependency marker; External
    // makes it an event-record node that every replay re-records
    LG_CUDA(cudaEventRecordWithFlags(a, H.s, cudaEventRecordExternal));
    f();
    LG_CUDA(cudaEventRecordWithFlags(b, H.s, cudaEventRecordExternal));
    H.prof.capture_tmpl.push_back({level, kind, k, fp64, a, b, bytes, true});
    return;
  }
  cudaEvent_t a = H.prof.get(), b = H.prof.get();
  LG_CUDA(cudaEventRecord(a, H.s));
  f();
  LG_CUDA(cudaEventRecord(b, H.s));
  H.prof.pending.push_back({level, kind, k, fp64, a, b, bytes, false});
}

// algorithmic (compulsory) bytes: every array element read or written once
inline double core_bytes(i64 rows, i64 nnz, i64 xrows, int k, int sv) {
  return 8.0 * (rows + 1) + (double)nnz * (4 + sv) + (double)xrows * k * sv;
}

void ensure_fp32(Handle &H) {
  cudaStream_t s = H.s;
  for (auto &Lp : H.h) {
    Level &L = *Lp;
    if (L.has32) continue;
    L.Av32.alloc(L.A.nnz, s);
    convert<double, float>(L.A.nnz, L.A.v.p, L.Av32.p, s);
    L.rs32.alloc(L.A.n, s);
    k_rowsum<float><<<grid_for(L.A.n, 256), 256, 0, s>>>(L.A.rp.p, L.Av32.p, L.A.n, L.rs32.p);
    LG_LAUNCH();
    if (L.invd.n) {
      L.invd32.alloc(L.invd.n, s);
      convert<double, float>(L.invd.n, L.invd.p, L.invd32.p, s);
    }
    if (L.type == LIGMG_LEVEL_ELIM) {
      L.Pv32.alloc(L.elim.P.nnz, s);
      convert<double, float>(L.elim.P.nnz, L.elim.P.v.p, L.Pv32.p, s);
      L.Rv32.alloc(L.elim.R.nnz, s);
      convert<double, float>(L.elim.R.nnz, L.elim.R.v.p, L.Rv32.p, s);
      L.Q32.alloc(L.A.n, s);
      convert<double, float>(L.A.n, L.elim.Q.p, L.Q32.p, s);
    }
    if (L.type == LIGMG_LEVEL_COARSE) {
      L.pinv32.alloc(L.pinv.n, s);
      convert<double, float>(L.pinv.n, L.pinv.p, L.pinv32.p, s);
    }
    if (L.type == LIGMG_LEVEL_AGG && L.Cr.nnz) {
      L.Cr32.alloc(L.Cr.nnz, s);
      convert<double, float>(L.Cr.nnz, L.Cr.v.p, L.Cr32.p, s);
    }
    if (L.ADv.n) {
      L.AD32.alloc(L.ADv.n, s);
      convert<double, float>(L.ADv.n, L.ADv.p, L.AD32.p, s);
    }
    L.has32 = true;
  }
  LG_CUDA(cudaStreamSynchronize(s));
}

template <typename T>
Work<T> &get_work(Handle &H, int k);
template <>
Work<float> &get_work<float>(Handle &H, int k) {
  auto &slot = H.w32[k];
  if (!slot) slot.reset(new Work<float>());
  return *slot;
}
template <>
Work<double> &get_work<double>(Handle &H, int k) {
  auto &slot = H.w64[k];
  if (!slot) slot.reset(new Work<double>());
  return *slot;
}

template <typename T>
Work<T> &work_for(Handle &H, int k) {
  Work<T> &W = get_work<T>(H, k);
  if (W.k == k) return W;
  cudaStream_t s = H.s;
  W.k = k;
  W.lw.resize(H.h.size());
  for (size_t l = 0; l < H.h.size(); l++) {
    Level &L = *H.h[l];
    LevelWork<T> &w = W.lw[l];
    i64 n = L.A.n;
    w.n = n;
    w.in.alloc(n * k, s);
    w.out.alloc(n * k, s);
    if (L.type == LIGMG_LEVEL_AGG) {
      w.r.alloc(n * k, s);
      w.d0.alloc(n * k, s);
      w.d1.alloc(n * k, s);
      w.xt.alloc(n * k, s);
      w.fz.alloc(n * k, s);
      w.fp0.alloc(n * k, s);
      w.fp1.alloc(n * k, s);
      w.fq0.alloc(n * k, s);
      w.fq1.alloc(n * k, s);
    }
    w.sc.alloc((i64)S_NSLOT * k * 2, s);
    w.sc.zero();
    w.scratch_len = col_reduce_scratch(n, k);
    w.scratch.alloc(w.scratch_len, s);
    w.fscratch.alloc(fused_scratch_len(n, k), s);
    w.fscratch.zero();  // reduction ticket starts at zero
    w.nseg = L.seginfo().nseg;
    if (w.nseg > 0) {
      w.segsc.alloc((i64)S_NSLOT * w.nseg, s);
      w.segsc.zero();
    }
  }
  return W;
}

// Zeroed barrier state carrying the handle's wait limit (options.wait_spins).
inline void tail_sync_reset(Handle &H, DBuf<TailSync> &sync) {
  TailSync z{};
  z.limit = H.opts.wait_spins;
  LG_CUDA(cudaMemcpyAsync(sync.p, &z, sizeof(TailSync), cudaMemcpyHostToDevice, H.s));
  LG_CUDA(cudaStreamSynchronize(H.s));
}

// ---------------------------------------------------------------------------
// Coarse-tail program: the operations Engine below issues for one visit of
// the levels from `start` down, recorded (same order, buffers and scalars)
// instead of launched.  Mirrors Engine::smooth / cycle / recurse / fcg_fixed.
template <typename T>
struct TailBuilder {
  Handle &H;
  Work<T> &W;
  int k;
  cudaStream_t s;
  std::vector<TOp<T>> ops;
  bool whole_rows = false;  // no hub-row chunks: one warp takes each row
  TailBuilder(Handle &h, Work<T> &w) : H(h), W(w), k(w.k), s(h.s) {}
  const ligmg_options &o() const { return H.opts; }

  void spmm(const MatView<T> &A, const T *X, Epi e, const EpiArgs &a) {
    TOp<T> op;
    op.kind = TOpKind::Spmm;
    op.epi = e;
    op.n = A.n;
    op.A = A;
    if (whole_rows) {
      op.A.hub_thresh = 0;
      op.A.nchunks = 0;
    }
    op.x0 = X;
    op.a = a;
    op.a.mirror();
    ops.push_back(op);
  }
  void elem(TOpKind kind, i64 n, const T *x0, const T *x1, T *y0, double f = 1) {
    TOp<T> op;
    op.kind = kind;
    op.n = n;
    op.x0 = x0;
    op.x1 = x1;
    op.y0 = y0;
    op.f = f;
    ops.push_back(op);
  }

  void smooth(size_t l, T *x, const T *b, int iters, bool x_zero) {
    Level &L = *H.h[l];
    LevelWork<T> &w = W.lw[l];
    i64 n = L.A.n;
    MatView<T> A = viewA<T>(L, k, s);
    const T *invd = invdT<T>(L);
    if (o().smoother_type == LIGMG_SMOOTHER_JACOBI) {
      const double omega = 2.0 / 3.0;
      if (x_zero) {
        elem(TOpKind::Cheb0, n, b, invd, x, omega);
        return;
      }
      EpiArgs a;
      a.b = b; a.invd = invd; a.xin = x; a.y = w.xt.p; a.c1 = omega;
      spmm(A, x, Epi::Jacobi, a);
      elem(TOpKind::Copy, n, w.xt.p, nullptr, x);
      return;
    }
    if (iters <= 0) return;
    const T *r_cur;
    const T *x_cur;
    T *d_cur;
    T *d_other = w.d1.p;
    int first = 1;
    if (x_zero && iters == 1) {
      elem(TOpKind::Cheb0, n, b, invd, x, 1.0 / L.theta);
      return;
    }
    if (x_zero) {
      const bool last = iters == 2;
      EpiArgs a;
      a.b = b; a.invd = invd; a.ith = 1.0 / L.theta; a.c1 = L.c1[0]; a.c2 = L.c2[0];
      a.rout = last ? nullptr : w.r.p;
      a.dout = last ? nullptr : w.d1.p;
      a.xout = last ? x : w.xt.p;
      spmm(viewAD<T>(L, k, s), b, Epi::ChebZ, a);
      if (last) return;
      r_cur = w.r.p;
      d_cur = w.d1.p;
      d_other = w.d0.p;
      x_cur = w.xt.p;
      first = 2;
    } else {
      EpiArgs a;
      a.b = b; a.invd = invd; a.xin = x; a.rout = w.r.p; a.dout = w.d0.p; a.xout = w.xt.p;
      a.ith = 1.0 / L.theta;
      spmm(A, x, Epi::ChebA, a);
      d_cur = w.d0.p;
      x_cur = w.xt.p;
      r_cur = w.r.p;
      if (iters == 1) {
        elem(TOpKind::Copy, n, w.xt.p, nullptr, x);
        return;
      }
    }
    for (int it = first; it < iters; it++) {
      bool last = it == iters - 1;
      EpiArgs a;
      a.invd = invd;
      a.rin = r_cur;
      a.din = d_cur;
      a.xin = x_cur;
      a.c1 = L.c1[it - 1];
      a.c2 = L.c2[it - 1];
      a.rout = last ? nullptr : w.r.p;
      a.dout = last ? nullptr : d_other;
      a.xout = last ? x : w.xt.p;
      spmm(A, d_cur, Epi::ChebB, a);
      if (!last) {
        r_cur = w.r.p;
        std::swap(d_cur, d_other);
        x_cur = w.xt.p;
      }
    }
  }

  void cycle(size_t l, const T *b, T *x) {
    Level &L = *H.h[l];
    i64 n = L.A.n;
    if (L.type == LIGMG_LEVEL_COARSE) {
      elem(TOpKind::Coarse, n, b, pinvT<T>(L), x);
      return;
    }
    LevelWork<T> &nw = W.lw[l + 1];
    if (L.type == LIGMG_LEVEL_ELIM) {
      EpiArgs a;
      a.y = nw.in.p;
      spmm(viewR<T>(L, k, s), b, Epi::Store, a);
      recurse(l, nw.in.p, nw.out.p);
      EpiArgs c;
      c.y = x; c.b = b; c.q = QT<T>(L);
      spmm(viewP<T>(L), nw.out.p, Epi::ElimInterp, c);
      return;
    }
    smooth(l, x, b, o().pre_smooth, true);
    EpiArgs rs;
    rs.y = nw.in.p;
    spmm(viewC<T>(L, k, x, s), b, Epi::Split, rs);
    recurse(l, nw.in.p, nw.out.p);
    TOp<T> pr;
    pr.kind = TOpKind::Prolong;
    pr.n = n;
    pr.x0 = nw.out.p;
    pr.y0 = x;
    pr.idx = L.agg.agg.p;
    ops.push_back(pr);
    smooth(l, x, b, o().post_smooth, false);
    if (o().constant_correction) elem(TOpKind::Scale, n, nullptr, nullptr, x, 4.0 / 3.0);
  }

  void recurse(size_t l, T *bc, T *xc) {
    const Level &N = *H.h[l + 1];
    if (!o().kcycle || N.is_exact() || N.type == LIGMG_LEVEL_COARSE) {
      cycle(l + 1, bc, xc);
      return;
    }
    fcg_fixed(l + 1, bc, xc, o().kcycle_iters);
  }

  void fcg_fixed(size_t l, T *b, T *x, int iters) {
    Level &L = *H.h[l];
    LevelWork<T> &w = W.lw[l];
    i64 n = L.A.n;
    MatView<T> A = viewA<T>(L, k, s);
    elem(TOpKind::Zero, n, nullptr, nullptr, x);
    T *r = b;
    T *p = w.fp0.p, *pp = w.fp1.p, *q = w.fq0.p, *qp = w.fq1.p;
    FcgScalars sc{w.slot(S_SUM, k), w.slot(S_BETA, k), w.slot(S_ETA0, k), w.slot(S_ETA1, k),
                  w.slot(S_ALPHA, k), nullptr};
    for (int it = 0; it < iters; it++) {
      cycle(l, r, w.fz.p);
      TOp<T> rb;
      rb.kind = TOpKind::RedBeta;
      rb.n = n;
      rb.x0 = w.fz.p;
      rb.x1 = it > 0 ? qp : nullptr;
      rb.flag = it > 0;
      ops.push_back(rb);
      TOp<T> d;
      d.kind = TOpKind::Dir;
      d.n = n;
      d.x0 = w.fz.p;
      d.x1 = it > 0 ? pp : nullptr;
      d.y0 = p;
      d.flag = it > 0;
      d.sc = sc;
      ops.push_back(d);
      EpiArgs a;
      a.y = q;
      spmm(A, p, Epi::Store, a);
      TOp<T> ra;
      ra.kind = TOpKind::RedAlpha;
      ra.n = n;
      ra.x0 = p;
      ra.x1 = q;
      ra.x2 = r;
      ops.push_back(ra);
      TOp<T> u;
      u.kind = TOpKind::Update;
      u.n = n;
      u.x0 = p;
      u.x1 = q;
      u.y0 = x;
      u.y1 = r;
      u.flag = it + 1 < iters;
      u.sc = sc;
      ops.push_back(u);
      std::swap(p, pp);
      std::swap(q, qp);
      std::swap(sc.eta, sc.eta_prev);
    }
  }
};

// First level of the grid-mode tail (tail_rows > 0): every level from it
// down has at most tail_rows rows; at least level 1, since the tail is
// entered from Engine::recurse of the level above (0: none).
inline size_t tail_start_level(const Handle &H) {
  const i64 lim = H.opts.tail_rows;
  if (lim <= 0 || H.h.size() < 2) return 0;
  // a top elimination level is applied once outside the cycle
  // (multigrid.hpp:322), so the cycle starts at level 1 and the tail is
  // entered at level 2 at the earliest
  const size_t first = (H.opts.top_elim && H.h[0]->type == LIGMG_LEVEL_ELIM) ? 2 : 1;
  size_t t = H.h.size();
  while (t > first && H.h[t - 1]->A.n <= lim) t--;
  return t < H.h.size() ? t : 0;
}

// Record the tail program entered as recurse(start - 1).  With smem_avail >
// 0 it is laid out for the shared-memory launch with kl columns per CTA:
//   [program | read-only arrays the program reads | work vector slices]
// where the work vectors are every buffer of the levels from `start` down
// (the start level's input and output included: staged in and out); each
// CTA holds an n x kl slice of each (the Krylov scalar slots whole).  The
// program's pointers into them are rewritten as kSmemTag | offset.
// `consts` lists the read-only arrays to copy into the image; every row of
// the tail's SpMMs is taken whole by one warp (no hub chunks, whose partials
// are global and would be shared by the CTAs).  Returns false when the layout
// needs more than smem_avail bytes.
struct TailCopy {
  const void *src;
  size_t off, bytes;
};
template <typename T>
// spill (cluster mode): read-only arrays go to shared memory level by level,
// deepest first, while they fit after the program and the work vectors; the
// other levels' arrays stay in global memory (their products are divided
// among a cluster's CTAs).  Otherwise everything must fit.
bool tail_record(Handle &H, Work<T> &W, size_t start, int smem_avail, int kl,
                 std::vector<TOp<T>> &ops, TailSmemLaunch &sl, std::vector<TailCopy> &consts,
                 bool spill = false) {
  TailBuilder<T> B(H, W);
  B.whole_rows = smem_avail > 0;  // a CTA of its own: the chunk partials are global
  LevelWork<T> &top = W.lw[start];
  B.recurse(start - 1, top.in.p, top.out.p);
  ops = std::move(B.ops);
  sl = TailSmemLaunch{};
  consts.clear();
  if (smem_avail <= 0) return true;
  const int k = W.k;
  // regions: global extent [base, base + gbytes), `bytes` of shared memory
  struct Reg {
    const char *base;
    size_t gbytes, bytes;
    long long off;
    size_t lev = 0;     // read-only arrays: their level
    bool keep = true;   // read-only arrays: placed in shared memory
    bool used = false;  // read-only arrays: read by the program
    bool inside(const void *p) const {
      const char *c = (const char *)p;
      return c >= base && c < base + gbytes;
    }
  };
  std::vector<Reg> vecs, scs, cons;  // n x k vectors (sliced), scalar slots, read-only arrays
  for (size_t l = start; l < W.lw.size(); l++) {
    LevelWork<T> &w = W.lw[l];
    for (DBuf<T> *b : {&w.in, &w.out, &w.r, &w.d0, &w.d1, &w.xt, &w.fz, &w.fp0, &w.fp1, &w.fq0,
                       &w.fq1})
      if (b->p && b->n)
        vecs.push_back({(const char *)b->p, sizeof(T) * (size_t)b->n,
                        sizeof(T) * (size_t)(b->n / k * kl), -1});
    if (w.sc.p && w.sc.n) {
      const size_t nb = sizeof(double) * (size_t)w.sc.n;
      scs.push_back({(const char *)w.sc.p, nb, nb, -1});
    }
    const Level &L = *H.h[l];
    auto add = [&](const void *p, size_t bytes) {
      if (p && bytes) cons.push_back({(const char *)p, bytes, bytes, -1, l});
    };
    const size_t n = (size_t)L.A.n, sv = sizeof(T);
    add(L.A.rp.p, 8 * (n + 1));
    add(L.A.ci.p, 4 * (size_t)L.A.nnz);
    add(valsA<T>(L), sv * (size_t)L.A.nnz);
    add(invdT<T>(L), sv * n);
    if (L.type == LIGMG_LEVEL_AGG) {
      add(L.agg.agg.p, 4 * n);
      add(L.agg.mrp.p, 8 * ((size_t)L.nc + 1));
      add(L.agg.members.p, 4 * n);
      add(valsR<T>(L), sv * n);
      if constexpr (sizeof(T) == 8) add(L.ADv.p, sv * (size_t)L.A.nnz);
      else add(L.AD32.p, sv * (size_t)L.A.nnz);
      add(L.Cr.rp.p, 8 * ((size_t)L.Cr.n + 1));
      add(L.Cr.ci.p, 4 * (size_t)L.Cr.nnz);
      add(valsC<T>(L), sv * (size_t)L.Cr.nnz);
    } else if (L.type == LIGMG_LEVEL_ELIM) {
      const DCsr<double> &R = L.elim.R, &P = L.elim.P;
      add(R.rp.p, 8 * ((size_t)R.n + 1));
      add(R.ci.p, 4 * (size_t)R.nnz);
      add(valsR<T>(L), sv * (size_t)R.nnz);
      add(P.rp.p, 8 * ((size_t)P.n + 1));
      add(P.ci.p, 4 * (size_t)P.nnz);
      if constexpr (sizeof(T) == 8) add(P.v.p, sv * (size_t)P.nnz);
      else add(L.Pv32.p, sv * (size_t)P.nnz);
      add(QT<T>(L), sv * n);
    } else {
      add(pinvT<T>(L), sv * n * n);
    }
  }
  auto owner = [](std::vector<Reg> &regs, const void *p) -> Reg * {
    if (!p) return nullptr;
    for (Reg &r : regs)
      if (r.inside(p)) return &r;
    return nullptr;
  };
  auto up16 = [](size_t x) { return (x + 15) & ~(size_t)15; };
  size_t total = up16(sizeof(TOp<T>) * ops.size());
  auto claim = [&](Reg *r) {
    if (r && r->off < 0) {
      r->off = (long long)total;
      total += up16(r->bytes);
    }
  };
  auto vec_fields = [](TOp<T> &op, auto &&f) {
    f(op.x0); f(op.x1); f(op.x2); f(op.y0); f(op.y1); f(op.A.x2);
    f(op.a.y); f(op.a.b); f(op.a.xin); f(op.a.xout); f(op.a.rin); f(op.a.rout);
    f(op.a.din); f(op.a.dout);
  };
  auto sc_fields = [](TOp<T> &op, auto &&f) {
    f(op.sc.mu); f(op.sc.beta); f(op.sc.eta); f(op.sc.eta_prev); f(op.sc.alpha);
  };
  auto con_fields = [](TOp<T> &op, auto &&f) {
    f(op.A.rp); f(op.A.ci); f(op.A.v); f(op.a.invd); f(op.a.q); f(op.x1); f(op.idx);
  };
  for (TOp<T> &op : ops)
    con_fields(op, [&](auto &p) {
      if (owner(vecs, p)) return;
      if (Reg *r = owner(cons, p)) r->used = true;
    });
  if (spill) {
    // the work vectors and scalar slots the program touches
    size_t wbytes = 0;
    std::vector<const Reg *> seen;
    auto count = [&](const Reg *r) {
      if (!r || std::find(seen.begin(), seen.end(), r) != seen.end()) return;
      seen.push_back(r);
      wbytes += up16(r->bytes);
    };
    for (TOp<T> &op : ops) {
      vec_fields(op, [&](auto &p) {
        if (p && !owner(cons, p)) count(owner(vecs, p));
      });
      sc_fields(op, [&](auto &p) {
        if (p) count(owner(scs, p));
      });
    }
    count(owner(vecs, top.in.p));
    count(owner(vecs, top.out.p));
    long long budget = (long long)smem_avail - (long long)total - (long long)wbytes;
    for (Reg &r : cons) r.keep = false;
    for (size_t l = W.lw.size(); l-- > start;) {
      size_t lb = 0;
      for (const Reg &r : cons)
        if (r.lev == l && r.used) lb += up16(r.bytes);
      if ((long long)lb > budget) break;  // this level and the shallower ones stay global
      budget -= (long long)lb;
      for (Reg &r : cons)
        if (r.lev == l) r.keep = true;
    }
  }
  // image first (program, then read-only arrays), then the writable regions
  for (TOp<T> &op : ops)
    con_fields(op, [&](auto &p) {
      if (owner(vecs, p)) return;
      Reg *r = owner(cons, p);
      if (r && r->keep) claim(r);
    });
  sl.image_bytes = (int)total;
  bool ok = true;
  for (TOp<T> &op : ops) {
    vec_fields(op, [&](auto &p) {
      if (!p || owner(cons, p)) return;
      Reg *r = owner(vecs, p);
      if (!r) {
        ok = false;  // a vector outside the tail's buffers
        return;
      }
      if ((const char *)p != r->base) ok = false;  // slices need buffer bases
      claim(r);
    });
    sc_fields(op, [&](auto &p) {
      if (p) claim(owner(scs, p));
    });
  }
  claim(owner(vecs, top.in.p));
  claim(owner(vecs, top.out.p));
  if (!ok || total > (size_t)smem_avail) return false;
  auto tag = [](auto &p, long long off) {
    p = reinterpret_cast<std::remove_reference_t<decltype(p)>>(kSmemTag | (unsigned long long)off);
  };
  for (TOp<T> &op : ops) {
    con_fields(op, [&](auto &p) {
      if (owner(vecs, p)) return;
      Reg *r = owner(cons, p);
      if (r && r->off >= 0) tag(p, r->off + ((const char *)p - r->base));
    });
    vec_fields(op, [&](auto &p) {
      Reg *r = owner(vecs, p);
      if (r) tag(p, r->off);
    });
    sc_fields(op, [&](auto &p) {
      Reg *r = owner(scs, p);
      if (r) tag(p, r->off + ((const char *)p - r->base));
    });
  }
  for (const Reg &r : cons)
    if (r.off >= 0) consts.push_back({r.base, (size_t)r.off, r.bytes});
  sl.kl = kl;
  sl.nops = (int)ops.size();
  sl.smem = (int)std::max<size_t>(total, 16);
  sl.gin = top.in.p;
  sl.gout = top.out.p;
  sl.n = H.h[start]->A.n;
  sl.in_off = (unsigned)owner(vecs, top.in.p)->off;
  sl.out_off = (unsigned)owner(vecs, top.out.p)->off;
  return true;
}

// Columns per CTA tried by the shared-memory mode for k columns.
inline std::vector<int> tail_slices(int k) {
  std::vector<int> v;
  for (int kl : {1, 4, 8})
    if (kl <= k && k % kl == 0) v.push_back(kl);
  return v;
}

// Decide the tail's start level (planning only; no program is kept).
//   tail_rows > 0: grid-mode program from tail_start_level;
//   tail_rows = 0: shared-memory program from the shallowest level whose
//                  program, read-only arrays and one-column work-vector
//                  slices fit in one CTA's shared memory;
//   tail_rows < 0: none.
template <typename T>
void tail_plan(Handle &H, Work<T> &W) {
  TailState<T> &ts = W.tail;
  ts.planned = true;
  ts.start = 0;
  const i64 lim = H.opts.tail_rows;
  if (lim < 0 || H.h.size() < 2) return;
  if (H.opts.kcycle && H.opts.kcycle_ksp_type != LIGMG_KSP_FCG) return;  // programs record FCG
  if (H.h[0]->seginfo().nseg > 0) return;  // batch mode keeps per-graph kernels
  if (lim > 0) {
    if (tail_max_ctas<T>(W.k) <= 0) return;
    ts.start = (int)tail_start_level(H);
    return;
  }
  if (tail_slices(W.k).empty()) return;
  const int avail = tail_smem_prepare<T>(1, 0);
  std::vector<TOp<T>> ops;
  std::vector<TailCopy> consts;
  TailSmemLaunch sl;
  size_t plain = 0;  // shallowest start of the plain shared-memory mode
  for (size_t t = 1; t < H.h.size(); t++) {
    if (tail_record<T>(H, W, t, avail, 1, ops, sl, consts)) {
      plain = t;
      break;
    }
  }
  // cluster mode: the shallowest start whose work vectors fit (the larger
  // levels' matrices stay in global memory), when shallower than `plain`
  if (H.opts.tail_cluster && tail_cluster_ok<T>(1, 2, 0)) {
    const size_t lim_t = plain ? plain : H.h.size();
    for (size_t t = 1; t < lim_t; t++) {
      if (H.h[t]->type == LIGMG_LEVEL_COARSE) break;
      if (tail_record<T>(H, W, t, avail, 1, ops, sl, consts, true)) {
        ts.start = (int)t;
        ts.smem_mode = true;
        ts.cluster = true;
        return;
      }
    }
  }
  if (plain) {
    ts.start = (int)plain;
    ts.smem_mode = true;
  }
}

// One launch of the current shape.
template <typename T>
void tail_launch(Handle &H, Work<T> &W, int G) {
  TailState<T> &ts = W.tail;
  if (ts.smem_mode) {
    ts.sl.image = ts.image.p;
    launch_tail_smem<T>(ts.sl, W.k, ts.sync.p, H.s);
  } else {
    launch_tail_grid<T>(ts.ops.p, ts.nops, W.k, G, ts.partial.p, ts.sync.p, H.s);
  }
}

// Upload the shared-memory image of `kl` columns per CTA (program followed by
// the read-only arrays).
template <typename T>
bool tail_build_smem(Handle &H, Work<T> &W, int kl, int cluster = 1) {
  TailState<T> &ts = W.tail;
  const int avail = tail_smem_prepare<T>(kl, 0);
  std::vector<TOp<T>> ops;
  std::vector<TailCopy> consts;
  TailSmemLaunch sl;
  if (!tail_record<T>(H, W, (size_t)ts.start, avail, kl, ops, sl, consts, ts.cluster))
    return false;
  tail_smem_prepare<T>(kl, sl.smem);
  if (ts.cluster && !tail_cluster_ok<T>(kl, cluster, sl.smem)) return false;
  sl.cluster = ts.cluster ? cluster : 1;
  ts.image.alloc(sl.image_bytes, H.s);
  LG_CUDA(cudaMemcpyAsync(ts.image.p, ops.data(), sizeof(TOp<T>) * ops.size(),
                          cudaMemcpyHostToDevice, H.s));
  for (const TailCopy &c : consts)
    LG_CUDA(cudaMemcpyAsync(ts.image.p + c.off, c.src, c.bytes, cudaMemcpyDeviceToDevice, H.s));
  LG_CUDA(cudaStreamSynchronize(H.s));  // `ops` is pageable host memory
  ts.sl = sl;
  ts.nops = sl.nops;
  return true;
}

// Build the program of the planned start level and pick its launch shape by
// timing (grid mode: CTA count; shared-memory mode: columns per CTA).  The
// restriction input bc is saved and restored around each timing run (the
// program updates it).  best_ms: the chosen shape's time, for the autotune
// choice against the launched levels.
template <typename T>
void tail_prepare(Handle &H, Work<T> &W) {
  TailState<T> &ts = W.tail;
  ts.tried = true;
  const int k = W.k;
  cudaStream_t s = H.s;
  const size_t start = (size_t)ts.start;
  LevelWork<T> &top = W.lw[start];
  const i64 nin = H.h[start]->A.n * k;
  DBuf<T> save(nin, s);
  LG_CUDA(cudaMemcpyAsync(save.p, top.in.p, sizeof(T) * nin, cudaMemcpyDeviceToDevice, s));
  ts.sync.alloc(1, s);
  tail_sync_reset(H, ts.sync);
  ts.bytes = 2.0 * H.h[start]->A.n * k * sizeof(T);
  for (size_t l = start; l < H.h.size(); l++)
    ts.bytes += 8.0 * (H.h[l]->A.n + 1) + (double)H.h[l]->A.nnz * (4 + sizeof(T));
  cudaEvent_t e0, e1;
  LG_CUDA(cudaEventCreate(&e0));
  LG_CUDA(cudaEventCreate(&e1));
  auto time_once = [&](int G) {
    float tot = 0;
    for (int rep = 0; rep < 3; rep++) {
      LG_CUDA(cudaMemcpyAsync(top.in.p, save.p, sizeof(T) * nin, cudaMemcpyDeviceToDevice, s));
      LG_CUDA(cudaEventRecord(e0, s));
      tail_launch<T>(H, W, G);
      LG_CUDA(cudaEventRecord(e1, s));
      LG_CUDA(cudaEventSynchronize(e1));
      float ms = 0;
      LG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      if (rep > 0) tot += ms;
    }
    return tot / 2;
  };
  float best = 1e30f;
  if (ts.smem_mode) {
    int best_kl = 0, best_cl = 1;
    std::vector<int> kls = tail_slices(k);
    // without autotune: the widest slice that fits (fewest CTAs)
    if (!H.opts.autotune) std::reverse(kls.begin(), kls.end());
    std::vector<int> cls{1};
    if (ts.cluster) cls = H.opts.autotune ? std::vector<int>{2, 4, 8, 16} : std::vector<int>{4};
    for (int kl : kls) {
      for (int cl : cls) {
        if (!tail_build_smem<T>(H, W, kl, cl)) continue;
        const float ms = time_once(0);
        if (ms < best) {
          best = ms;
          best_kl = kl;
          best_cl = cl;
        }
      }
      if (!H.opts.autotune && best_kl) break;
    }
    if (best_kl == 0) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return;
    }
    if (best_kl != ts.sl.kl || best_cl != ts.sl.cluster) tail_build_smem<T>(H, W, best_kl, best_cl);
  } else {
    std::vector<TOp<T>> ops;
    std::vector<TailCopy> consts;
    TailSmemLaunch unused;
    tail_record<T>(H, W, start, 0, 0, ops, unused, consts);
    ts.nops = (int)ops.size();
    ts.ops.alloc(ts.nops, s);
    ts.ops.upload(ops.data(), ts.nops);
    LG_CUDA(cudaStreamSynchronize(s));
    const int G0 = std::min(tail_max_ctas<T>(k), kSMs);
    ts.partial.alloc((i64)G0 * 3 * k, s);
    ts.G = G0;
    std::vector<int> cands{G0};
    if (H.opts.autotune) cands = {1, 4, 16, G0 / 4, G0};
    for (int G : cands) {
      if (G < 1 || G > G0) continue;
      const float ms = time_once(G);
      if (ms < best) {
        best = ms;
        ts.G = G;
      }
    }
  }
  ts.best_ms = best;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  LG_CUDA(cudaMemcpyAsync(top.in.p, save.p, sizeof(T) * nin, cudaMemcpyDeviceToDevice, s));
  LG_CUDA(cudaStreamSynchronize(s));
  // a barrier wait that ran out during the timing runs fails the call like
  // one in a solve (the tail stays off; the state is reset for a retry)
  TailSync h{};
  LG_CUDA(cudaMemcpy(&h, ts.sync.p, sizeof(TailSync), cudaMemcpyDeviceToHost));
  if (h.err) {
    tail_sync_reset(H, ts.sync);
    ts.tried = false;
    throw Error(LIGMG_ERR_INTERNAL, "coarse-tail kernel: a grid barrier wait ran out");
  }
  ts.on = true;
}

// Error raised by a persistent tail launch (a grid barrier that gave up).
template <typename T>
void tail_check(Handle &H, Work<T> &W, cudaStream_t s) {
  if (!W.tail.on) return;
  TailSync h{};
  LG_CUDA(cudaMemcpyAsync(&h, W.tail.sync.p, sizeof(TailSync), cudaMemcpyDeviceToHost, s));
  LG_CUDA(cudaStreamSynchronize(s));
  if (h.err) {
    // an abandoned barrier leaves the arrival counter mid-way: start clean
    tail_sync_reset(H, W.tail.sync);
    throw Error(LIGMG_ERR_INTERNAL, "coarse-tail kernel: a grid barrier wait ran out");
  }
}

// ---------------------------------------------------------------------------
template <typename T>
struct Engine {
  Handle &H;
  Work<T> &W;
  int k;
  cudaStream_t s;
  Engine(Handle &h, Work<T> &w) : H(h), W(w), k(w.k), s(h.s) {}

  const ligmg_options &o() const { return H.opts; }

  void smooth(size_t l, T *x, const T *b, int iters, bool x_zero) {
    Level &L = *H.h[l];
    LevelWork<T> &w = W.lw[l];
    i64 n = L.A.n;
    MatView<T> A = viewA<T>(L, k, s);
    const T *invd = invdT<T>(L);
    if (o().smoother_type == LIGMG_SMOOTHER_JACOBI) {
      // create_smoother (smoothing.hpp:206-211): one weighted-Jacobi sweep
      // (omega = 2/3) per smoother call, whatever the iteration count
      const double omega = 2.0 / 3.0;
      if (x_zero) {
        timed(H, (int)l, LIGMG_KERNEL_VECTOR, k, sizeof(T) == 8, (2.0 * n * k + n) * sizeof(T),
              [&] { cheb_init_zero<T>(n, k, b, invd, omega, x, s); });
        return;
      }
      EpiArgs a;
      a.b = b; a.invd = invd; a.xin = x; a.y = w.xt.p; a.c1 = omega;
      timed(H, (int)l, LIGMG_KERNEL_RESID, k, sizeof(T) == 8,
            core_bytes(n, L.A.nnz, n, k, sizeof(T)) + (3.0 * n * k + n) * sizeof(T),
            [&] { spmm<T>(A, x, k, Epi::Jacobi, a, s); });
      timed(H, (int)l, LIGMG_KERNEL_VECTOR, k, sizeof(T) == 8, 2.0 * n * k * sizeof(T), [&] {
        LG_CUDA(cudaMemcpyAsync(x, w.xt.p, sizeof(T) * n * k, cudaMemcpyDeviceToDevice, s));
      });
      return;
    }
    if (iters <= 0) return;
    const T *r_cur;
    const T *x_cur;
    T *d_cur;
    T *d_other = w.d1.p;
    int first = 1;  // next Chebyshev step of the loop below
    if (x_zero && iters == 1) {
      timed(H, (int)l, LIGMG_KERNEL_VECTOR, k, sizeof(T) == 8, (2.0 * n * k + n) * sizeof(T),
            [&] { cheb_init_zero<T>(n, k, b, invd, 1.0 / L.theta, x, s); });
      return;
    }
    if (x_zero) {
      // steps 0 and 1 in one SpMM gathering b with the A D^-1 values
      const bool last = iters == 2;
      EpiArgs a;
      a.b = b; a.invd = invd; a.ith = 1.0 / L.theta; a.c1 = L.c1[0]; a.c2 = L.c2[0];
      a.rout = last ? nullptr : w.r.p;
      a.dout = last ? nullptr : w.d1.p;
      a.xout = last ? x : w.xt.p;
      timed(H, (int)l, LIGMG_KERNEL_CHEB_B, k, sizeof(T) == 8,
            core_bytes(n, L.A.nnz, n, k, sizeof(T)) + ((last ? 1.0 : 3.0) * n * k + n) * sizeof(T),
            [&] { spmm<T>(viewAD<T>(L, k, s), b, k, Epi::ChebZ, a, s); });
      if (last) return;
      r_cur = w.r.p;
      d_cur = w.d1.p;
      d_other = w.d0.p;
      x_cur = w.xt.p;
      first = 2;
    } else {
      EpiArgs a;
      a.b = b; a.invd = invd; a.xin = x; a.rout = w.r.p; a.dout = w.d0.p; a.xout = w.xt.p;
      a.ith = 1.0 / L.theta;
      timed(H, (int)l, LIGMG_KERNEL_CHEB_A, k, sizeof(T) == 8,
            core_bytes(n, L.A.nnz, n, k, sizeof(T)) + (5.0 * n * k + n) * sizeof(T),
            [&] { spmm<T>(A, x, k, Epi::ChebA, a, s); });
      d_cur = w.d0.p;
      x_cur = w.xt.p;
      r_cur = w.r.p;
      if (iters == 1) {
        timed(H, (int)l, LIGMG_KERNEL_VECTOR, k, sizeof(T) == 8, 2.0 * n * k * sizeof(T), [&] {
          LG_CUDA(cudaMemcpyAsync(x, w.xt.p, sizeof(T) * n * k, cudaMemcpyDeviceToDevice, s));
        });
        return;
      }
    }
    for (int it = first; it < iters; it++) {
      bool last = it == iters - 1;
      EpiArgs a;
      a.invd = invd;
      a.rin = r_cur;
      a.din = d_cur;
      a.xin = x_cur;
      a.c1 = L.c1[it - 1];
      a.c2 = L.c2[it - 1];
      a.rout = last ? nullptr : w.r.p;
      a.dout = last ? nullptr : d_other;
      T *xo = last ? x : w.xt.p;
      a.xout = xo;
      timed(H, (int)l, LIGMG_KERNEL_CHEB_B, k, sizeof(T) == 8,
            core_bytes(n, L.A.nnz, n, k, sizeof(T)) + ((last ? 4.0 : 6.0) * n * k + n) * sizeof(T),
            [&] { spmm<T>(A, d_cur, k, Epi::ChebB, a, s); });
      if (!last) {
        r_cur = w.r.p;
        std::swap(d_cur, d_other);
        x_cur = w.xt.p;
      }
    }
  }

  // x = M_l(b) with zero initial guess
  void cycle(size_t l, const T *b, T *x) {
    Level &L = *H.h[l];
    i64 n = L.A.n;
    if (L.type == LIGMG_LEVEL_COARSE) {
      timed(H, (int)l, LIGMG_KERNEL_COARSE, k, sizeof(T) == 8,
            ((double)n * n + 2.0 * n * k) * sizeof(T),
            [&] { coarse_apply<T>(n, k, pinvT<T>(L), b, x, s); });
      return;
    }
    LevelWork<T> &nw = W.lw[l + 1];
    if (L.type == LIGMG_LEVEL_ELIM) {  // elimination.hpp:33-52
      EpiArgs a;
      a.y = nw.in.p;
      timed(H, (int)l, LIGMG_KERNEL_ELIM_RESTRICT, k, sizeof(T) == 8,
            core_bytes(L.elim.R.n, L.elim.R.nnz, n, k, sizeof(T)) + (double)L.elim.R.n * k * sizeof(T),
            [&] { spmm<T>(viewR<T>(L, k, s), b, k, Epi::Store, a, s); });
      recurse(l, nw.in.p, nw.out.p);
      EpiArgs c;
      c.y = x; c.b = b; c.q = QT<T>(L);
      timed(H, (int)l, LIGMG_KERNEL_ELIM_INTERP, k, sizeof(T) == 8,
            core_bytes(n, L.elim.P.nnz, L.nc, k, sizeof(T)) + (2.0 * n * k + n) * sizeof(T),
            [&] { spmm<T>(viewP<T>(L), nw.out.p, k, Epi::ElimInterp, c, s); });
      return;
    }
    // aggregation.hpp:209-241
    smooth(l, x, b, o().pre_smooth, true);
    // residual and restriction in one SpMM: bc = R (b - A x) = C [b; x]
    EpiArgs rs;
    rs.y = nw.in.p;
    timed(H, (int)l, LIGMG_KERNEL_AGG_RESTRICT, k, sizeof(T) == 8,
          core_bytes(L.nc, L.Cr.nnz, 2 * n, k, sizeof(T)) + (double)L.nc * k * sizeof(T),
          [&] { spmm<T>(viewC<T>(L, k, x, s), b, k, Epi::Split, rs, s); });
    recurse(l, nw.in.p, nw.out.p);
    timed(H, (int)l, LIGMG_KERNEL_AGG_PROLONG, k, sizeof(T) == 8,
          4.0 * n + (2.0 * n + L.nc) * k * sizeof(T),
          [&] { prolong_agg<T>(n, k, L.agg.agg.p, nw.out.p, x, s); });
    smooth(l, x, b, o().post_smooth, false);
    if (o().constant_correction)
      timed(H, (int)l, LIGMG_KERNEL_VECTOR, k, sizeof(T) == 8, 2.0 * n * k * sizeof(T),
            [&] { scale_vec<T>(n, k, x, 4.0 / 3.0, s); });
  }

  void recurse(size_t l, T *bc, T *xc) {
    if (try_tail(l + 1, bc, xc)) return;
    recurse_launched(l, bc, xc);
  }
  void recurse_launched(size_t l, T *bc, T *xc) {
    const Level &N = *H.h[l + 1];
    if (!o().kcycle || N.is_exact() || N.type == LIGMG_LEVEL_COARSE) {
      cycle(l + 1, bc, xc);
      return;
    }
    if (o().kcycle_ksp_type == LIGMG_KSP_FGMRES) fgmres_fixed(l + 1, bc, xc, o().kcycle_iters);
    else fcg_fixed(l + 1, bc, xc, o().kcycle_iters);
  }

  // K-cycle inner FGMRES (kcycle_ksp_type = fgmres, parse_options.hpp:399-400):
  // exactly m Arnoldi steps from x = 0 (PETSc's restart length, 30, exceeds the
  // K-cycle's iteration count), the outer FGMRES's arithmetic otherwise: b's
  // constant projected out, right preconditioning with the cycle of level l
  // (its constant projected out), classical Gram-Schmidt, Givens rotations and
  // back substitution.  The Hessenberg least squares runs on the device (one
  // thread per column), so the inner solve stays inside the preconditioner's
  // CUDA graph; b (the level's restriction buffer) is overwritten.
  void fgmres_fixed(size_t l, T *b, T *x, int m) {
    Level &L = *H.h[l];
    LevelWork<T> &w = W.lw[l];
    const i64 n = L.A.n, nk = n * k;
    if (w.gW.n != nk || w.gV.n != (i64)(m + 1) * nk) {
      w.gV.alloc((i64)(m + 1) * nk, s);
      w.gZ.alloc((i64)m * nk, s);
      w.gW.alloc(nk, s);
      w.gH.alloc((i64)((m + 1) * m + m + 3) * k, s);
    }
    auto V = [&](int i) { return w.gV.p + (i64)i * nk; };
    auto Z = [&](int i) { return w.gZ.p + (i64)i * nk; };
    double *Hb = w.gH.p;  // H(i, j) at Hb[(i m + j) k + c]
    auto Hs = [&](int i, int j) { return Hb + ((i64)i * m + j) * k; };
    double *b2 = Hb + (i64)(m + 1) * m * k, *rcp = b2 + k, *sum = rcp + k, *y = sum + k;
    const bool f64 = sizeof(T) == 8;
    const double vb = (double)nk * sizeof(T);
    MatView<T> A = viewA<T>(L, k, s);
    auto project = [&](T *v) {  // v -= mean(v), per column
      col_reduce<T>(n, k, Red::Sum, v, nullptr, sum, w.scratch.p, w.scratch_len, s);
      sub_mean<T>(n, k, v, sum, s);
    };
    timed(H, (int)l, LIGMG_KERNEL_KRYLOV, k, f64, 5.0 * vb, [&] {
      project(b);
      col_reduce<T>(n, k, Red::Dot, b, b, b2, w.scratch.p, w.scratch_len, s);
      rsqrt_cols(k, b2, rcp, s);
      scale_cols<T>(n, k, V(0), b, rcp, s);
    });
    for (int j = 0; j < m; j++) {
      cycle(l, V(j), Z(j));
      timed(H, (int)l, LIGMG_KERNEL_KRYLOV, k, f64, 3.0 * vb, [&] { project(Z(j)); });
      EpiArgs a;
      a.y = w.gW.p;
      timed(H, (int)l, LIGMG_KERNEL_SPMV, k, f64,
            core_bytes(n, L.A.nnz, n, k, sizeof(T)) + vb,
            [&] { spmm<T>(A, Z(j), k, Epi::Store, a, s); });
      timed(H, (int)l, LIGMG_KERNEL_KRYLOV, k, f64, (5.0 * (j + 1) + 3) * vb, [&] {
        for (int i = 0; i <= j; i++)
          col_reduce<T>(n, k, Red::Dot, V(i), w.gW.p, Hs(i, j), w.scratch.p, w.scratch_len, s);
        for (int i = 0; i <= j; i++) axpby_cols<T>(n, k, w.gW.p, V(i), Hs(i, j), -1.0, 1.0, s);
        col_reduce<T>(n, k, Red::Dot, w.gW.p, w.gW.p, Hs(j + 1, j), w.scratch.p, w.scratch_len,
                      s);
        if (j + 1 < m) {
          rsqrt_cols(k, Hs(j + 1, j), rcp, s);
          scale_cols<T>(n, k, V(j + 1), w.gW.p, rcp, s);
        }
      });
    }
    timed(H, (int)l, LIGMG_KERNEL_KRYLOV, k, f64, (2.0 * m + 1) * vb, [&] {
      gmres_small(k, m, Hb, b2, y, s);
      LG_CUDA(cudaMemsetAsync(x, 0, sizeof(T) * nk, s));
      for (int i = 0; i < m; i++) axpby_cols<T>(n, k, x, Z(i), y + (i64)i * k, 1.0, 1.0, s);
    });
  }

  // The levels from `start` down as one persistent launch when that level
  // starts the tail (planned and built on first use, outside graph capture;
  // with autotune, apply_prec keeps it only where a whole preconditioner
  // application runs faster with it).
  bool try_tail(size_t start, T *bc, T *xc) {
    TailState<T> &ts = W.tail;
    if (!ts.planned || !ts.tried) {
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      LG_CUDA(cudaStreamIsCapturing(s, &cs));
      if (cs != cudaStreamCaptureStatusNone) return false;
    }
    if (!ts.planned) tail_plan<T>(H, W);
    if (ts.start <= 0 || (size_t)ts.start != start) return false;
    if (bc != W.lw[start].in.p || xc != W.lw[start].out.p) return false;
    if (!ts.tried) {
      tail_prepare<T>(H, W);
      if (ts.on && o().verbose)
        fprintf(stderr, "[ligmg] tail k=%d from level %zu (%s, %d ops, %d CTAs, %d B shared): "
                        "%.1f us per visit alone\n",
                k, start, ts.smem_mode ? (ts.cluster ? "shared, clusters" : "shared") : "grid",
                ts.nops, ts.smem_mode ? k / ts.sl.kl * ts.sl.cluster : ts.G,
                ts.smem_mode ? ts.sl.smem : 0, 1e3 * ts.best_ms);
    }
    if (!ts.on) return false;
    timed(H, (int)start, LIGMG_KERNEL_TAIL, k, sizeof(T) == 8, ts.bytes,
          [&] { tail_launch<T>(H, W, ts.G); });
    return true;
  }

  // K-cycle inner FCG with a fixed number of iterations, x0 = 0; r = b is
  // updated in place (b is the level's restriction buffer).  Four launches
  // per iteration besides the cycle: beta (fused reduction), direction and
  // its product in one SpMM (Epi::FcgDir), alpha (fused reduction), update.
  // The product of the direction p = (z - mu) - beta pp is formed as
  // A z - mu rowsum(A) - beta qp: equal to A p up to rounding, since qp is
  // the previous direction's product (batch mode: direction, then SpMM).
  void fcg_fixed(size_t l, T *b, T *x, int iters) {
    Level &L = *H.h[l];
    LevelWork<T> &w = W.lw[l];
    i64 n = L.A.n;
    MatView<T> A = viewA<T>(L, k, s);
    T *r = b;
    T *p = w.fp0.p, *pp = w.fp1.p, *q = w.fq0.p, *qp = w.fq1.p;
    const SegInfo S = L.seginfo();
    const bool seg = S.nseg > 0;
    if (seg)  // x = 0 (otherwise the first update writes x = alpha p)
      timed(H, (int)l, LIGMG_KERNEL_VECTOR, k, sizeof(T) == 8, 1.0 * n * k * sizeof(T),
            [&] { LG_CUDA(cudaMemsetAsync(x, 0, sizeof(T) * n * k, s)); });
    FcgScalars sc{w.slot(S_SUM, k), w.slot(S_BETA, k), w.slot(S_ETA0, k), w.slot(S_ETA1, k),
                  w.slot(S_ALPHA, k), nullptr};
    if constexpr (sizeof(T) == 4) {
      float *f = reinterpret_cast<float *>(w.slot(S_F32, k));
      sc.mu_f = f;
      sc.beta_f = f + k;
      sc.alpha_f = f + 2 * k;
    }
    if (seg)  // one set of Krylov scalars per graph of the batch
      sc = FcgScalars{w.sslot(S_SUM), w.sslot(S_BETA), w.sslot(S_ETA0), w.sslot(S_ETA1),
                      w.sslot(S_ALPHA), nullptr};
    for (int it = 0; it < iters; it++) {
      cycle(l, r, w.fz.p);
      const double nk = (double)n * k * sizeof(T);
      if (seg) {  // per-graph scalars: direction, then its product
        timed(H, (int)l, LIGMG_KERNEL_KRYLOV, k, sizeof(T) == 8, (it > 0 ? 5.0 : 3.0) * nk, [&] {
          seg_fcg_beta<T>(S, w.fz.p, it > 0 ? qp : nullptr, sc, s);
          seg_fcg_dir<T>(S, n, p, w.fz.p, it > 0 ? pp : nullptr, sc, s);
        });
        EpiArgs a;
        a.y = q;
        timed(H, (int)l, LIGMG_KERNEL_SPMV, k, sizeof(T) == 8,
              core_bytes(n, L.A.nnz, n, k, sizeof(T)) + 1.0 * n * k * sizeof(T),
              [&] { spmm<T>(A, p, k, Epi::Store, a, s); });
      } else {
        // beta (reduction), then p and q = A p in one SpMM gathering z
        timed(H, (int)l, LIGMG_KERNEL_KRYLOV, k, sizeof(T) == 8, (it > 0 ? 2.0 : 1.0) * nk,
              [&] { fcg_beta<T>(n, k, w.fz.p, it > 0 ? qp : nullptr, sc, w.fscratch.p, s); });
        EpiArgs a;
        a.xin = w.fz.p;
        a.q = rowsumT<T>(L);
        if constexpr (sizeof(T) == 4) {
          a.cmu = sc.mu_f;
          a.cbeta = sc.beta_f;
        } else {
          a.cmu = sc.mu;
          a.cbeta = sc.beta;
        }
        if (it > 0) {
          a.din = pp;
          a.rin = qp;
        }
        a.dout = p;
        a.y = q;
        timed(H, (int)l, LIGMG_KERNEL_SPMV, k, sizeof(T) == 8,
              core_bytes(n, L.A.nnz, n, k, sizeof(T)) + (it > 0 ? 5.0 : 3.0) * nk + n * sizeof(T),
              [&] { spmm<T>(A, w.fz.p, k, Epi::FcgDir, a, s); });
      }
      timed(H, (int)l, LIGMG_KERNEL_KRYLOV, k, sizeof(T) == 8, (it + 1 < iters ? 9.0 : 6.0) * nk,
            [&] {
              if (seg) {
                seg_fcg_alpha<T>(S, p, q, r, sc, s);
                seg_fcg_update<T>(S, n, x, r, p, q, sc.alpha, it + 1 < iters, s);
              } else {
                fcg_alpha<T>(n, k, p, q, r, sc, w.fscratch.p, s);
                fcg_update<T>(n, k, x, r, p, q, sc.alpha, it + 1 < iters, s, sc.alpha_f, it == 0);
              }
            });
      std::swap(p, pp);
      std::swap(q, qp);
      std::swap(sc.eta, sc.eta_prev);
    }
  }
};

// ---------------------------------------------------------------------------
// setup
void estimate_lmax(Handle &H, Level &L) {
  cudaStream_t s = H.s;
  i64 n = L.A.n;
  std::vector<double> rh(n);
  for (i64 i = 0; i < n; i++) rh[i] = est_rhs(i);
  DBuf<double> r(n, s), z(n, s), p(n, s), q(n, s), sc(8, s);
  i64 slen = col_reduce_scratch(n, 1);
  DBuf<double> scratch(slen, s);
  r.upload(rh.data(), n);
  col_reduce<double>(n, 1, Red::Sum, r.p, nullptr, sc.p, scratch.p, slen, s);
  sub_mean<double>(n, 1, r.p, sc.p, s);
  k_mul_diag<<<grid_for(n, 256), 256, 0, s>>>(n, L.invd.p, r.p, z.p);
  LG_LAUNCH();
  LG_CUDA(cudaMemcpyAsync(p.p, z.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  col_reduce<double>(n, 1, Red::Dot, r.p, z.p, sc.p, scratch.p, slen, s);
  double rz = read_scalar(sc.p, s);
  MatView<double> A = viewA<double>(L, 1, s);
  std::vector<double> alphas, betas;
  for (int it = 0; it < 5; it++) {
    if (!(rz > 0)) break;
    EpiArgs a;
    a.y = q.p;
    spmm<double>(A, p.p, 1, Epi::Store, a, s);
    col_reduce<double>(n, 1, Red::Dot, p.p, q.p, sc.p, scratch.p, slen, s);
    double pq = read_scalar(sc.p, s);
    if (!(pq > 0)) break;
    double alpha = rz / pq;
    LG_CUDA(cudaMemcpyAsync(sc.p + 1, &alpha, sizeof(double), cudaMemcpyHostToDevice, s));
    axpby_cols<double>(n, 1, r.p, q.p, sc.p + 1, -1.0, 1.0, s);
    k_mul_diag<<<grid_for(n, 256), 256, 0, s>>>(n, L.invd.p, r.p, z.p);
    LG_LAUNCH();
    col_reduce<double>(n, 1, Red::Dot, r.p, z.p, sc.p, scratch.p, slen, s);
    double rz_new = read_scalar(sc.p, s);
    double beta = rz_new / rz;
    rz = rz_new;
    LG_CUDA(cudaMemcpyAsync(sc.p + 2, &beta, sizeof(double), cudaMemcpyHostToDevice, s));
    cg_direction<double>(n, 1, p.p, z.p, sc.p + 2, s);
    alphas.push_back(alpha);
    betas.push_back(beta);
    LG_CUDA(cudaStreamSynchronize(s));
  }
  int m = (int)alphas.size();
  if (m == 0) {
    L.lmax = 2.0;
  } else {
    std::vector<double> d(m), e(m > 1 ? m - 1 : 0);
    for (int kk = 0; kk < m; kk++) {
      d[kk] = 1.0 / alphas[kk] + (kk > 0 ? betas[kk - 1] / alphas[kk - 1] : 0.0);
      if (kk + 1 < m) e[kk] = std::sqrt(betas[kk]) / alphas[kk];
    }
    L.lmax = tridiag_lmax(d, e);
  }
}

void setup_smoother_params(const ligmg_options &o, Level &L) {
  double a = o.cheby_lower * L.lmax, bb = o.cheby_upper * L.lmax;
  double theta = (bb + a) / 2, delta = (bb - a) / 2;
  double sigma = theta / delta, rho = 1 / sigma;
  L.theta = theta;
  L.delta = delta;
  int m = std::max(o.pre_smooth, o.post_smooth);
  L.c1.assign(std::max(m, 1), 0.0);
  L.c2.assign(std::max(m, 1), 0.0);
  for (int kk = 0; kk + 1 < m; kk++) {
    double rho_new = 1 / (2 * sigma - rho);
    L.c1[kk] = rho_new * rho;
    L.c2[kk] = 2 * rho_new / delta;
    rho = rho_new;
  }
}

void finish_level(Handle &H, Level &L) {
  cudaStream_t s = H.s;
  L.invd.alloc(L.A.n, s);
  k_invdiag<<<grid_for(L.A.n, 256), 256, 0, s>>>(L.A.rp.p, L.A.ci.p, L.A.v.p, L.A.n, L.invd.p);
  LG_LAUNCH();
  L.rs64.alloc(L.A.n, s);
  k_rowsum<double><<<grid_for(L.A.n, 256), 256, 0, s>>>(L.A.rp.p, L.A.v.p, L.A.n, L.rs64.p);
  LG_LAUNCH();
  L.lanesA = lanes_for(L.A.nnz, L.A.n);
  L.autotune = H.opts.autotune != 0;
  L.tiles = H.opts.spmv_tiles;
  L.streams = H.opts.spmm_streams;
  L.ktiles = H.opts.spmm_tiles;
  L.rp_host = L.A.rp.to_host();
  // the FP64 single right-hand-side plan of A is built (and, with autotune,
  // its layout and launch shape timed) at setup: ligmg_spmv_device_noalloc
  // and every FP64 solve use it without building anything later
  build_plan<double>(L, MAT_A, 1, L.hubA64, L.autotune, s);
  if (L.type == LIGMG_LEVEL_ELIM) {
    L.rrp_host = L.elim.R.rp.to_host();
    L.lanesR = lanes_for(L.elim.R.nnz, L.elim.R.n);
    L.lanesP = lanes_for(L.elim.P.nnz, L.elim.P.n);
  }
  if (L.type == LIGMG_LEVEL_AGG) {
    L.ADv.alloc(L.A.nnz, s);
    k_ad_values<<<grid_for(L.A.nnz, 256), 256, 0, s>>>(L.A.nnz, L.A.ci.p, L.A.v.p, L.invd.p,
                                                       L.ADv.p);
    LG_LAUNCH();
    gpu_restrict_residual_matrix(L.A, L.agg.agg.p, L.agg.mrp.p, L.agg.members.p, L.nc, L.Cr, s);
    L.crp_host = L.Cr.rp.to_host();
    L.lanesC = lanes_for(L.Cr.nnz, L.Cr.n);
    L.rrp_host = L.agg.mrp.to_host();
    L.lanesR = lanes_for(L.A.n, L.nc);
    L.ones64.alloc(L.A.n, s);
    L.ones32.alloc(L.A.n, s);
    fill_value<double>(L.A.n, L.ones64.p, 1.0, s);
    fill_value<float>(L.A.n, L.ones32.p, 1.0f, s);
  }
}

void make_hierarchy(Handle &H, i64 n, const i64 *rowptr, const i32 *col, const double *val) {
  const ligmg_options &o = H.opts;
  cudaStream_t s = H.s;
  auto t0 = std::chrono::steady_clock::now();
  i64 nnz = rowptr[n];
  DCsr<double> cur;
  cur.n = cur.m = n;
  cur.nnz = nnz;
  cur.rp.alloc(n + 1, s);
  cur.ci.alloc(nnz, s);
  cur.v.alloc(nnz, s);
  cur.rp.upload(rowptr, n + 1);
  cur.ci.upload(col, nnz);
  cur.v.upload(val, nnz);
  ligmg_status st = gpu_validate(cur, s);
  if (st != LIGMG_OK) throw Error(st, "input validation");
  H.nnz0 = nnz;
  // batch mode: segment offsets of the current matrix, carried level to level
  const i64 nseg = H.seg0.empty() ? 0 : (i64)H.seg0.size() - 1;
  std::vector<i64> cur_seg = H.seg0;
  auto attach = [&](Level &L) {
    if (!nseg) return;
    L.seg_host = cur_seg;
    L.segptr.alloc(nseg + 1, s);
    L.segptr.upload(cur_seg.data(), nseg + 1);
    L.rowseg.alloc(L.A.n, s);
    k_fill_rowseg<<<grid_for(L.A.n, 256), 256, 0, s>>>(L.segptr.p, nseg, L.A.n, L.rowseg.p);
    LG_LAUNCH();
    LG_CUDA(cudaStreamSynchronize(s));
  };
  auto next_offsets = [&](const Level &L, const i32 *scan, i64 nc) {
    if (!nseg) return;
    DBuf<i64> out(nseg + 1, s);
    k_gather_offsets<<<grid_for(nseg + 1, 128), 128, 0, s>>>(scan, L.segptr.p, nseg, L.A.n, nc,
                                                             out.p);
    LG_LAUNCH();
    cur_seg = out.to_host();
  };
  if (nseg) {  // the input must be block-diagonal along the given offsets
    DBuf<i64> sp(nseg + 1, s);
    DBuf<i32> rs(n, s);
    DBuf<int> bad(1, s);
    bad.zero();
    sp.upload(cur_seg.data(), nseg + 1);
    k_fill_rowseg<<<grid_for(n, 256), 256, 0, s>>>(sp.p, nseg, n, rs.p);
    k_check_blockdiag<<<grid_for(n, 256), 256, 0, s>>>(cur.rp.p, cur.ci.p, n, rs.p, sp.p, bad.p);
    LG_LAUNCH();
    if (read_scalar(bad.p, s)) throw Error(LIGMG_ERR_INVALID_ARGUMENT, "batch not block-diagonal");
  }
  GlibcRand rng(o.seed);
  for (i64 i = 0; i < o.rng_skip; i++) rng.next();
  AggParams ap;
  ap.num_tvs = o.num_tvs;
  ap.tvs_smooth = o.tvs_smooth;
  ap.agg_iters = o.agg_iters;
  ap.strength_metric = o.strength_metric;
  ap.aff_scaling = o.aff_scaling;
  ap.neighbor_of_neighbor = o.neighbor_of_neighbor != 0;
  ap.thresh = o.thresh;
  ap.agg_init_factor = o.agg_init_factor;
  ap.agg_iter_factor = o.agg_iter_factor;
  ap.votes_to_seed = (double)o.votes_to_seed;
  ap.max_agg_size = (double)o.max_agg_size;
  ap.rejection_ratio = o.rejection_ratio;
  ap.rejection_to_seed = o.rejection_to_seed != 0;
  auto &h = H.h;
  // per-phase wall time (the stream is drained at each phase boundary)
  auto tp = std::chrono::steady_clock::now();
  auto phase = [&](int ph) {
    LG_CUDA(cudaStreamSynchronize(s));
    auto t = std::chrono::steady_clock::now();
    H.setup_phase[ph] += std::chrono::duration<double>(t - tp).count();
    tp = t;
  };
  phase(LIGMG_SETUP_VALIDATE);
  while ((int)h.size() < o.max_levels && (h.empty() || h.back()->A.nnz > o.min_size)) {
    if (o.always_elim && o.elim_iters >= 1) {
      auto E = std::make_unique<Level>();
      E->type = LIGMG_LEVEL_ELIM;
      gpu_elimination(cur, o.elim_degree, o.elim_factor, E->elim, s);
      phase(LIGMG_SETUP_ELIMINATION);
      if (E->elim.accepted) {
        DCsr<double> next;
        gpu_galerkin(cur, E->elim.P, next, s);
        phase(LIGMG_SETUP_GALERKIN);
        E->A = std::move(cur);
        E->nc = E->elim.nc;
        finish_level(H, *E);
        phase(LIGMG_SETUP_SOLVE_DATA);
        attach(*E);
        next_offsets(*E, E->elim.pos.p, E->nc);
        h.push_back(std::move(E));
        cur = std::move(next);
      }
    }
    auto G = std::make_unique<Level>();
    G->type = LIGMG_LEVEL_AGG;
    i64 cn = cur.n;
    std::vector<double> tvs;
    bool need_tvs = o.strength_metric == LIGMG_STRENGTH_AFFINITY ||
                    o.strength_metric == LIGMG_STRENGTH_ALGEBRAIC_DISTANCE;
    if (need_tvs) {  // create_tvs (aggregation.hpp:24-36)
      tvs.resize((size_t)o.num_tvs * cn);
      for (int t = 0; t < o.num_tvs; t++) {
        double *x = tvs.data() + (size_t)t * cn;
        for (i64 i = 0; i < cn; i++) x[i] = double(rng.next()) / 2147483647;
        double sm = 0.0;
        for (i64 i = 0; i < cn; i++) sm += x[i];
        sm = sm / (double)cn;
        for (i64 i = 0; i < cn; i++) x[i] = x[i] - sm;
      }
    }
    phase(LIGMG_SETUP_AGGREGATION);  // the host's test vectors count here
    gpu_aggregation(cur, ap, tvs.data(), G->agg, s);
    G->nc = G->agg.nc;
    phase(LIGMG_SETUP_AGGREGATION);
    DCsr<double> next;
    gpu_galerkin_agg(cur, G->agg.agg.p, G->nc, next, s);
    phase(LIGMG_SETUP_GALERKIN);
    G->A = std::move(cur);
    finish_level(H, *G);
    attach(*G);
    next_offsets(*G, G->agg.rank.p, G->nc);
    phase(LIGMG_SETUP_SOLVE_DATA);
    estimate_lmax(H, *G);
    setup_smoother_params(o, *G);
    phase(LIGMG_SETUP_SMOOTHER);
    h.push_back(std::move(G));
    cur = std::move(next);
  }
  auto C = std::make_unique<Level>();
  C->type = LIGMG_LEVEL_COARSE;
  C->A = std::move(cur);
  attach(*C);
  st = gpu_coarse_pinv(C->A, C->pinv, s, nseg ? C->rowseg.p : nullptr,
                       nseg ? C->segptr.p : nullptr);
  if (st != LIGMG_OK) throw Error(st, "coarse pseudo-inverse");
  phase(LIGMG_SETUP_COARSE);
  finish_level(H, *C);
  h.push_back(std::move(C));
  LG_CUDA(cudaStreamSynchronize(s));
  H.setup_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

double cycle_complexity(Handle &H, int start) {  // multigrid.hpp:372-387
  double sm = 0;
  i64 iters = 1;
  for (size_t i = start; i < H.h.size(); i++) {
    sm += (double)(iters * H.h[i]->work(H.opts));
    if (!H.h[i]->is_exact() && H.opts.kcycle) iters *= H.opts.kcycle_iters;
  }
  return sm / (double)H.nnz0;
}

// ---------------------------------------------------------------------------
// outer solve on device arrays B (n0 x k, FP64) -> X (n0 x k)
OuterWork &outer_work(Handle &H, int k, i64 nb, i64 n0) {
  auto &slot = H.ow[k];
  if (!slot) slot.reset(new OuterWork());
  OuterWork &w = *slot;
  if (w.k == k && w.n == nb) return w;
  cudaStream_t s = H.s;
  w.k = k;
  w.n = nb;
  for (DBuf<double> *b : {&w.X, &w.R, &w.Z, &w.P0, &w.P1, &w.Q0, &w.Q1, &w.B})
    b->alloc(nb * k, s);
  w.Bfull.alloc(n0 * k, s);
  w.Xfull.alloc(n0 * k, s);
  w.Res.alloc(n0 * k, s);
  w.sc.alloc((i64)(S_NSLOT + 4) * k * 2, s);
  w.sc.zero();
  w.scratch_len = std::max(col_reduce_scratch(nb, k), col_reduce_scratch(n0, k));
  w.scratch.alloc(w.scratch_len, s);
  w.fscratch.alloc(std::max(fused_scratch_len(nb, k), fused_scratch_len(n0, k)), s);
  w.fscratch.zero();
  w.frozen.alloc(k, s);
  w.Pdf.alloc(nb * k, s);
  return w;
}

// z = M(r) with the constant projected out of z.  `sum`, `scratch` are the
// outer workspace's reduction slots.
template <typename T>
void apply_prec_body(Handle &H, int k, size_t base, const double *r, double *z, double *sum,
                     double *scratch, i64 scratch_len) {
  Level &L = *H.h[base];
  i64 n = L.A.n;
  Work<T> &W = work_for<T>(H, k);
  Engine<T> E(H, W);
  if constexpr (sizeof(T) == 8) {
    E.cycle(base, r, z);
  } else {
    LevelWork<T> &w = W.lw[base];
    timed(H, (int)base, LIGMG_KERNEL_VECTOR, k, 0, 12.0 * n * k,
          [&] { convert<double, float>(n * k, r, w.in.p, H.s); });
    E.cycle(base, w.in.p, w.out.p);
    timed(H, (int)base, LIGMG_KERNEL_VECTOR, k, 0, 12.0 * n * k,
          [&] { convert<float, double>(n * k, w.out.p, z, H.s); });
  }
  const SegInfo S = L.seginfo();
  timed(H, (int)base, LIGMG_KERNEL_OUTER, k, 1, 24.0 * n * k, [&] {
    if (S.nseg > 0) {  // one constant per graph of the batch
      seg_mean<double>(S, z, sum, H.s);
      seg_sub_mean<double>(S, n, z, sum, H.s);
      return;
    }
    col_reduce<double>(n, k, Red::Sum, z, nullptr, sum, scratch, scratch_len, H.s);
    sub_mean<double>(n, k, z, sum, H.s);
  });
}

// The K-cycle issues thousands of small kernels per application; after one
// direct run (which also creates every lazily built plan and buffer) the
// sequence is captured once into a CUDA graph and replayed.
template <typename T>
void apply_prec(Handle &H, int k, size_t base, const double *r, double *z, double *sum,
                double *scratch, i64 scratch_len) {
  auto body = [&] { apply_prec_body<T>(H, k, base, r, z, sum, scratch, scratch_len); };
  TailState<T> &ts = work_for<T>(H, k).tail;
  // autotune: the persistent tail stays only if a whole application is
  // faster with it (z is recomputed from r each time, so runs repeat)
  auto decide_tail = [&](auto &&run_on, auto &&run_off) {
    ts.decided = true;
    cudaEvent_t e0, e1;
    LG_CUDA(cudaEventCreate(&e0));
    LG_CUDA(cudaEventCreate(&e1));
    auto time3 = [&](auto &&run) {
      run();
      LG_CUDA(cudaEventRecord(e0, H.s));
      run();
      run();
      LG_CUDA(cudaEventRecord(e1, H.s));
      LG_CUDA(cudaEventSynchronize(e1));
      float ms = 0;
      LG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      return ms / 2;
    };
    const float t_on = time3(run_on);
    const float t_off = time3(run_off);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (H.opts.verbose)
      fprintf(stderr, "[ligmg] preconditioner k=%d: %.1f us with the tail, %.1f us without\n",
              k, 1e3 * t_on, 1e3 * t_off);
    return t_on < t_off;
  };
  auto decide = [&] { return H.opts.autotune && ts.on && !ts.decided && !H.prof.on; };
  if (!H.opts.use_graphs) {
    body();
    if (decide()) {
      auto on = [&] { ts.on = true; body(); };
      auto off = [&] { ts.on = false; body(); };
      ts.on = decide_tail(on, off);
      body();
    }
    return;
  }
  PrecGraph &g = H.pgraphs[std::make_tuple(k, (int)sizeof(T), (int)base)];
  if (g.exec && g.r == r && g.z == z && g.prof == H.prof.on) {
    LG_CUDA(cudaGraphLaunch(g.exec, H.s));
    add_launches(g.kernels);
    if (H.prof.on)
      for (const ProfRec &t : g.tmpl) H.prof.pending.push_back(t);
    return;
  }
  g.reset();
  body();  // direct run: produces this application's result
  auto capture = [&](int64_t &kernels) {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    H.prof.capture_tmpl.clear();
    H.prof.capturing = H.prof.on;
    const int64_t c0 = launches_now();
    LG_CUDA(cudaStreamBeginCapture(H.s, cudaStreamCaptureModeThreadLocal));
    try {
      body();
    } catch (...) {
      cudaStreamEndCapture(H.s, &graph);
      if (graph) cudaGraphDestroy(graph);
      H.prof.capturing = false;
      add_launches(c0 - launches_now());
      throw;
    }
    H.prof.capturing = false;
    kernels = launches_now() - c0;
    add_launches(-kernels);
    LG_CUDA(cudaStreamEndCapture(H.s, &graph));
    cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    LG_CUDA(e);
    return exec;
  };
  const bool dec = decide();  // after the direct run, which prepares the tail
  g.exec = capture(g.kernels);
  if (dec) {
    int64_t k_off = 0;
    ts.on = false;
    cudaGraphExec_t off = capture(k_off);
    auto run_on = [&] {
      LG_CUDA(cudaGraphLaunch(g.exec, H.s));
      add_launches(g.kernels);
    };
    auto run_off = [&] {
      LG_CUDA(cudaGraphLaunch(off, H.s));
      add_launches(k_off);
    };
    if (decide_tail(run_on, run_off)) {
      cudaGraphExecDestroy(off);
      ts.on = true;
    } else {
      cudaGraphExecDestroy(g.exec);
      g.exec = off;
      g.kernels = k_off;
    }
    // this application's result from the path that is kept, like every later one
    LG_CUDA(cudaGraphLaunch(g.exec, H.s));
    add_launches(g.kernels);
  }
  g.r = r;
  g.z = z;
  g.prof = H.prof.on;
  g.tmpl = H.prof.capture_tmpl;
  H.prof.capture_tmpl.clear();
}

struct SolveResult {
  int iters = 0;
  bool converged = false;
  std::vector<double> hist0;
  std::vector<int> col_iters;
  std::vector<double> rel;  // last/first per column
};

// Outer Krylov (petsc_fcg, cg.hpp:18-116) with k columns; r0 = b (x0 = 0).
template <typename T>
SolveResult outer_solve(Handle &H, size_t base, OuterWork &w, int k) {
  const ligmg_options &o = H.opts;
  cudaStream_t s = H.s;
  Level &L = *H.h[base];
  i64 n = L.A.n;
  MatView<double> A = viewA<double>(L, k, s);
  SolveResult res;
  res.col_iters.assign(k, 0);
  res.rel.assign(k, 1.0);
  double *sum = w.slot(S_SUM), *tmp = w.slot(S_ZQ), *beta = w.slot(S_BETA);
  double *eta = w.slot(S_ETA0), *eta_prev = w.slot(S_ETA1), *rho = w.slot(S_RHO);
  double *alpha = w.slot(S_ALPHA), *rn2 = w.slot(S_PQR), *bcg = w.slot(S_NSLOT),
         *bcg_old = w.slot(S_NSLOT + 1);
  // project the constant out of the right-hand side
  col_reduce<double>(n, k, Red::Sum, w.B.p, nullptr, sum, w.scratch.p, w.scratch_len, s);
  sub_mean<double>(n, k, w.B.p, sum, s);
  LG_CUDA(cudaMemsetAsync(w.X.p, 0, sizeof(double) * n * k, s));
  LG_CUDA(cudaMemcpyAsync(w.R.p, w.B.p, sizeof(double) * n * k, cudaMemcpyDeviceToDevice, s));
  LG_CUDA(cudaMemsetAsync(w.frozen.p, 0, sizeof(int) * k, s));
  col_reduce<double>(n, k, Red::Dot, w.R.p, w.R.p, rn2, w.scratch.p, w.scratch_len, s);
  std::vector<double> h_rn2(k), rn0(k);
  LG_CUDA(cudaMemcpyAsync(h_rn2.data(), rn2, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
  LG_CUDA(cudaStreamSynchronize(s));
  std::vector<int> frozen(k, 0);
  int active = 0;
  for (int c = 0; c < k; c++) {
    rn0[c] = std::sqrt(h_rn2[c]);
    if (!std::isfinite(rn0[c]))  // NaN or Inf in the right-hand side
      throw Error(LIGMG_ERR_NONFINITE, "right-hand side holds a NaN or Inf");
    if (rn0[c] == 0) frozen[c] = 1; else active++;
  }
  res.hist0.push_back(rn0[0]);
  LG_CUDA(cudaMemcpyAsync(w.frozen.p, frozen.data(), sizeof(int) * k, cudaMemcpyHostToDevice, s));
  bool cg = o.outer_ksp_type == LIGMG_KSP_CG;
  // FP32 hierarchy: the outer product A p runs in double-float (48-bit
  // significand at FP32 throughput); the FP64 hierarchy keeps native FP64
  bool dfprod = sizeof(T) == 4;
  if (dfprod && L.Adf.n != L.A.nnz) {
    L.Adf.alloc(L.A.nnz, s);
    split_df(L.A.nnz, L.A.v.p, L.Adf.p, s);
  }
  double *P = w.P0.p, *PP = w.P1.p, *Q = w.Q0.p, *QP = w.Q1.p;
  auto precondition = [&]() {
    apply_prec<T>(H, k, base, w.R.p, w.Z.p, sum, w.scratch.p, w.scratch_len);
  };
  if (cg && active) {
    precondition();
    col_reduce<double>(n, k, Red::Dot, w.Z.p, w.R.p, bcg, w.scratch.p, w.scratch_len, s);
  }
  int it = 0;
  for (; it < o.iters && active > 0; it++) {
    if (cg) {  // KSPCG
      if (it == 0) {
        LG_CUDA(cudaMemcpyAsync(P, w.Z.p, sizeof(double) * n * k, cudaMemcpyDeviceToDevice, s));
      } else {
        scal_div(k, bcg, bcg_old, beta, nullptr, s);
        cg_direction<double>(n, k, P, w.Z.p, beta, s);
      }
      EpiArgs a;
      a.y = Q;
      timed(H, (int)base, LIGMG_KERNEL_SPMV, k, 1, core_bytes(n, L.A.nnz, n, k, 8) + 8.0 * n * k,
            [&] { spmm<double>(A, P, k, Epi::Store, a, s); });
      col_reduce<double>(n, k, Red::Dot, P, Q, eta, w.scratch.p, w.scratch_len, s);
      scal_div(k, bcg, eta, alpha, w.frozen.p, s);
      fcg_update<double>(n, k, w.X.p, w.R.p, P, Q, alpha, true, s);
    } else {  // FCG (Notay), one stored direction; fused scalar reductions
      precondition();
      FcgScalars sc{tmp, beta, eta, eta_prev, alpha, w.frozen.p};
      const double nk = 8.0 * n * k;
      timed(H, (int)base, LIGMG_KERNEL_OUTER, k, 1, (it > 0 ? 5.0 : 3.0) * nk, [&] {
        fcg_beta<double>(n, k, w.Z.p, it > 0 ? QP : nullptr, sc, w.fscratch.p, s);
        fcg_dir<double>(n, k, P, w.Z.p, it > 0 ? PP : nullptr, sc, s, dfprod ? w.Pdf.p : nullptr);
      });
      EpiArgs a;
      a.y = Q;
      timed(H, (int)base, LIGMG_KERNEL_SPMV, k, 1, core_bytes(n, L.A.nnz, n, k, 8) + 8.0 * n * k,
            [&] {
              if (dfprod) spmm_df(df_view(L, A, k, s), L.Adf.p, w.Pdf.p, k, Q, s);
              else spmm<double>(A, P, k, Epi::Store, a, s);
            });
      timed(H, (int)base, LIGMG_KERNEL_OUTER, k, 1, 9.0 * nk, [&] {
        fcg_alpha<double>(n, k, P, Q, w.R.p, sc, w.fscratch.p, s);
        fcg_update<double>(n, k, w.X.p, w.R.p, P, Q, alpha, true, s);
      });
      std::swap(P, PP);
      std::swap(Q, QP);
      std::swap(eta, eta_prev);
    }
    timed(H, (int)base, LIGMG_KERNEL_OUTER, k, 1, 8.0 * n * k,
          [&] { col_dot1<double>(n, k, w.R.p, w.R.p, rn2, w.fscratch.p, s); });
    LG_CUDA(cudaMemcpyAsync(h_rn2.data(), rn2, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
    LG_CUDA(cudaStreamSynchronize(s));
    if (H.prof.on) H.prof.collect();  // graph replays re-record the same events
    bool changed = false;
    for (int c = 0; c < k; c++) {
      if (frozen[c]) continue;
      double rn = std::sqrt(h_rn2[c]);
      res.col_iters[c] = it + 1;
      res.rel[c] = rn / rn0[c];
      if (c == 0) res.hist0.push_back(rn);
      if (!std::isfinite(rn)) throw Error(LIGMG_ERR_BREAKDOWN, "non-finite residual");
      if (rn <= std::max(o.tol * rn0[c], 1e-60)) {
        frozen[c] = 1;
        active--;
        changed = true;
      }
    }
    if (changed)
      LG_CUDA(cudaMemcpyAsync(w.frozen.p, frozen.data(), sizeof(int) * k, cudaMemcpyHostToDevice, s));
    if (cg && active > 0) {
      precondition();
      LG_CUDA(cudaMemcpyAsync(bcg_old, bcg, sizeof(double) * k, cudaMemcpyDeviceToDevice, s));
      col_reduce<double>(n, k, Red::Dot, w.Z.p, w.R.p, bcg, w.scratch.p, w.scratch_len, s);
    }
  }
  res.iters = it;
  res.converged = active == 0;
  return res;
}

// FGMRES(m) outer solve on k columns (PETSc KSPFGMRES semantics, selectable
// as the reference's outer KSP type, parse_options.hpp:383-384): right
// preconditioning with the cycle (constant projected out), classical
// Gram-Schmidt, Givens rotations, the Arnoldi residual estimate as the
// convergence test, restart after m steps from the true residual.  Every
// column keeps its own basis; the small Hessenberg arithmetic runs on the host
// from the device dot products (one synchronisation per step).
template <typename T>
SolveResult outer_solve_fgmres(Handle &H, size_t base, OuterWork &w, int k) {
  const ligmg_options &o = H.opts;
  cudaStream_t s = H.s;
  Level &L = *H.h[base];
  const i64 n = L.A.n, nk = n * k;
  const int m = std::max(1, o.gmres_restart);
  MatView<double> A = viewA<double>(L, k, s);
  SolveResult res;
  res.col_iters.assign(k, 0);
  res.rel.assign(k, 1.0);
  double *sum = w.slot(S_SUM), *rn2 = w.slot(S_PQR);
  if (w.fgV.n != (i64)(m + 1) * nk) {
    w.fgV.alloc((i64)(m + 1) * nk, s);
    w.fgZ.alloc((i64)m * nk, s);
    w.fgW.alloc(nk, s);
    w.fgH.alloc((i64)(m + 1) * k, s);
    w.fgC.alloc((i64)m * k, s);
  }
  auto V = [&](int i) { return w.fgV.p + (i64)i * nk; };
  auto Z = [&](int i) { return w.fgZ.p + (i64)i * nk; };
  col_reduce<double>(n, k, Red::Sum, w.B.p, nullptr, sum, w.scratch.p, w.scratch_len, s);
  sub_mean<double>(n, k, w.B.p, sum, s);
  LG_CUDA(cudaMemsetAsync(w.X.p, 0, sizeof(double) * nk, s));
  LG_CUDA(cudaMemcpyAsync(w.R.p, w.B.p, sizeof(double) * nk, cudaMemcpyDeviceToDevice, s));
  auto col_norms = [&](const double *x, std::vector<double> &out) {
    col_reduce<double>(n, k, Red::Dot, x, x, rn2, w.scratch.p, w.scratch_len, s);
    out.resize(k);
    LG_CUDA(cudaMemcpyAsync(out.data(), rn2, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
    LG_CUDA(cudaStreamSynchronize(s));
    for (double &v : out) v = std::sqrt(v);
  };
  std::vector<double> beta, rn0, ttol(k);
  col_norms(w.R.p, beta);
  rn0 = beta;
  std::vector<char> done(k, 0);
  int active = 0;
  for (int c = 0; c < k; c++) {
    if (!std::isfinite(rn0[c]))
      throw Error(LIGMG_ERR_NONFINITE, "right-hand side holds a NaN or Inf");
    ttol[c] = std::max(o.tol * rn0[c], 1e-60);
    if (rn0[c] == 0) done[c] = 1;
    else active++;
  }
  res.hist0.push_back(rn0[0]);
  std::vector<double> Hm((size_t)k * (m + 1) * m), cs((size_t)k * m), sn((size_t)k * m),
      g((size_t)k * (m + 1)), coef(k), hv, ycoef((size_t)m * k);
  std::vector<int> jc(k);
  std::vector<char> conv(k);
  auto Hij = [&](int c, int i, int j) -> double & { return Hm[((size_t)c * (m + 1) + i) * m + j]; };
  auto scale_into = [&](double *dst, const double *src) {  // dst = coef[c] * src
    LG_CUDA(cudaMemcpyAsync(w.fgC.p, coef.data(), sizeof(double) * k, cudaMemcpyHostToDevice, s));
    LG_CUDA(cudaMemsetAsync(dst, 0, sizeof(double) * nk, s));
    axpby_cols<double>(n, k, dst, src, w.fgC.p, 1.0, 0.0, s);
  };
  int it = 0;
  while (active > 0 && it < o.iters) {
    for (int c = 0; c < k; c++) {
      coef[c] = (!done[c] && beta[c] > 0) ? 1.0 / beta[c] : 0.0;
      std::fill(g.begin() + (size_t)c * (m + 1), g.begin() + (size_t)(c + 1) * (m + 1), 0.0);
      g[(size_t)c * (m + 1)] = done[c] ? 0.0 : beta[c];
      jc[c] = 0;
      conv[c] = 0;
    }
    scale_into(V(0), w.R.p);
    int j = 0;
    int open = active;  // columns still iterating in this cycle
    while (j < m && it < o.iters && open > 0) {
      LG_CUDA(cudaMemcpyAsync(w.R.p, V(j), sizeof(double) * nk, cudaMemcpyDeviceToDevice, s));
      apply_prec<T>(H, k, base, w.R.p, w.Z.p, sum, w.scratch.p, w.scratch_len);
      LG_CUDA(cudaMemcpyAsync(Z(j), w.Z.p, sizeof(double) * nk, cudaMemcpyDeviceToDevice, s));
      EpiArgs a;
      a.y = w.fgW.p;
      timed(H, (int)base, LIGMG_KERNEL_SPMV, k, 1, core_bytes(n, L.A.nnz, n, k, 8) + 8.0 * nk,
            [&] { spmm<double>(A, Z(j), k, Epi::Store, a, s); });
      timed(H, (int)base, LIGMG_KERNEL_OUTER, k, 1, (4.0 * (j + 1) + 1) * 8.0 * nk, [&] {
        for (int i = 0; i <= j; i++)
          col_reduce<double>(n, k, Red::Dot, V(i), w.fgW.p, w.fgH.p + (i64)i * k, w.scratch.p,
                             w.scratch_len, s);
        for (int i = 0; i <= j; i++)
          axpby_cols<double>(n, k, w.fgW.p, V(i), w.fgH.p + (i64)i * k, -1.0, 1.0, s);
        col_reduce<double>(n, k, Red::Dot, w.fgW.p, w.fgW.p, w.fgH.p + (i64)(j + 1) * k,
                           w.scratch.p, w.scratch_len, s);
      });
      hv.resize((size_t)(j + 2) * k);
      LG_CUDA(cudaMemcpyAsync(hv.data(), w.fgH.p, sizeof(double) * hv.size(),
                              cudaMemcpyDeviceToHost, s));
      LG_CUDA(cudaStreamSynchronize(s));
      if (H.prof.on) H.prof.collect();
      for (int c = 0; c < k; c++) {
        coef[c] = 0.0;
        if (done[c] || conv[c]) continue;
        for (int i = 0; i <= j; i++) Hij(c, i, j) = hv[(size_t)i * k + c];
        const double hn = std::sqrt(std::max(hv[(size_t)(j + 1) * k + c], 0.0));
        Hij(c, j + 1, j) = hn;
        coef[c] = hn > 0 ? 1.0 / hn : 0.0;
        double *csc = &cs[(size_t)c * m], *snc = &sn[(size_t)c * m], *gc = &g[(size_t)c * (m + 1)];
        for (int i = 0; i < j; i++) {
          const double x = Hij(c, i, j), y = Hij(c, i + 1, j);
          Hij(c, i, j) = csc[i] * x + snc[i] * y;
          Hij(c, i + 1, j) = -snc[i] * x + csc[i] * y;
        }
        const double x = Hij(c, j, j), y = Hij(c, j + 1, j);
        const double rho = std::sqrt(x * x + y * y);
        csc[j] = rho > 0 ? x / rho : 1.0;
        snc[j] = rho > 0 ? y / rho : 0.0;
        Hij(c, j, j) = rho;
        Hij(c, j + 1, j) = 0.0;
        gc[j + 1] = -snc[j] * gc[j];
        gc[j] = csc[j] * gc[j];
        const double rn = std::fabs(gc[j + 1]);
        jc[c] = j + 1;
        res.col_iters[c] = it + 1;
        if (!std::isfinite(rn)) throw Error(LIGMG_ERR_BREAKDOWN, "non-finite residual");
        if (c == 0) res.hist0.push_back(rn);
        if (rn <= ttol[c]) {
          conv[c] = 1;
          open--;
          coef[c] = 0.0;
        }
      }
      scale_into(V(j + 1), w.fgW.p);
      it++;
      j++;
    }
    // x += sum_i y_i Z_i, y from each column's triangular system
    std::fill(ycoef.begin(), ycoef.end(), 0.0);
    for (int c = 0; c < k; c++) {
      if (done[c]) continue;
      const int jj = jc[c];
      const double *gc = &g[(size_t)c * (m + 1)];
      for (int i = jj - 1; i >= 0; i--) {
        double acc = gc[i];
        for (int l = i + 1; l < jj; l++) acc -= Hij(c, i, l) * ycoef[(size_t)l * k + c];
        ycoef[(size_t)i * k + c] = Hij(c, i, i) != 0 ? acc / Hij(c, i, i) : 0.0;
      }
    }
    LG_CUDA(cudaMemcpyAsync(w.fgC.p, ycoef.data(), sizeof(double) * (size_t)j * k,
                            cudaMemcpyHostToDevice, s));
    for (int i = 0; i < j; i++)
      axpby_cols<double>(n, k, w.X.p, Z(i), w.fgC.p + (i64)i * k, 1.0, 1.0, s);
    EpiArgs a;
    a.y = w.R.p;
    a.b = w.B.p;
    spmm<double>(A, w.X.p, k, Epi::Resid, a, s);  // true residual for the restart
    col_norms(w.R.p, beta);
    for (int c = 0; c < k; c++) {
      if (done[c]) continue;
      res.rel[c] = beta[c] / rn0[c];
      if (conv[c] || beta[c] <= ttol[c]) {
        done[c] = 1;
        active--;
      } else if (!std::isfinite(beta[c])) {
        throw Error(LIGMG_ERR_BREAKDOWN, "non-finite residual");
      }
    }
  }
  res.iters = it;
  res.converged = active == 0;
  return res;
}

// Batch mode outer FCG: every graph has its own Krylov scalars and its own
// convergence test, evaluated on the device, so a whole solve needs no host
// round trip.  kGraphIters iterations are captured into one CUDA graph (the
// first from x0 = 0, later blocks continue); a batch that converges within
// the first block is solved by one graph launch.
constexpr int kGraphIters = 16;  // even: the continuation block repeats the buffer parity

template <typename T>
void seg_outer_iteration(Handle &H, size_t base, OuterWork &w, SegOuter &so, int it,
                         bool dfprod) {
  cudaStream_t s = H.s;
  Level &L = *H.h[base];
  i64 n = L.A.n, ns = L.seginfo().nseg;
  SegInfo S = L.seginfo();
  auto slot = [&](int q) { return so.sc.p + (i64)q * ns; };
  bool odd = it & 1;
  double *P = odd ? w.P1.p : w.P0.p, *PP = odd ? w.P0.p : w.P1.p;
  double *Q = odd ? w.Q1.p : w.Q0.p, *QP = odd ? w.Q0.p : w.Q1.p;
  double *eta = odd ? slot(S_ETA1) : slot(S_ETA0), *eta_prev = odd ? slot(S_ETA0) : slot(S_ETA1);
  apply_prec_body<T>(H, 1, base, w.R.p, w.Z.p, slot(S_SUM), w.scratch.p, w.scratch_len);
  FcgScalars sc{slot(S_ZQ), slot(S_BETA), eta, eta_prev, slot(S_ALPHA), so.frozen.p};
  seg_fcg_beta<double>(S, w.Z.p, it > 0 ? QP : nullptr, sc, s);
  seg_fcg_dir<double>(S, n, P, w.Z.p, it > 0 ? PP : nullptr, sc, s, dfprod ? so.Pdf.p : nullptr);
  MatView<double> A = viewA<double>(L, 1, s);
  EpiArgs a;
  a.y = Q;
  if (dfprod) spmm_df(A, L.Adf.p, so.Pdf.p, 1, Q, s);
  else spmm<double>(A, P, 1, Epi::Store, a, s);
  seg_fcg_alpha<double>(S, P, Q, w.R.p, sc, s);
  seg_fcg_update<double>(S, n, w.X.p, w.R.p, P, Q, slot(S_ALPHA), true, s);
  seg_dot<double>(S, w.R.p, w.R.p, so.rn2.p, s);
  seg_converge(ns, so.rn2.p, so.rn0sq.p, H.opts.tol, it, so.frozen.p, so.iters.p, s);
}

// ---------------------------------------------------------------------------
// Batch program for the persistent work-queue kernel (queue.cuh): the
// operations of kQueueIters outer iterations, in the order the launched
// segment path issues them (seg_outer_iteration, Engine in segment mode:
// smooth / cycle / recurse / fcg_fixed), each tagged with the level whose
// graph row ranges split it.  Matrices are read by whole rows.
template <typename T>
struct QueueBuilder {
  Handle &H;
  Work<T> &W;
  OuterWork &w;
  cudaStream_t s;
  std::vector<QOp> ops;
  static constexpr int DT = sizeof(T) == 8;
  QueueBuilder(Handle &h, Work<T> &wk, OuterWork &ow) : H(h), W(wk), w(ow), s(h.s) {}
  const ligmg_options &o() const { return H.opts; }

  static int lanes_of(i64 nnz, i64 n) { return (n > 0 && nnz >= 32 * n) ? 32 : 8; }
  template <typename V>
  static MatView<V> whole(MatView<V> m) {
    m.hub_thresh = 0;
    m.nchunks = 0;
    m.ntiles = 0;
    return m;
  }
  void spmm(int lev, const MatView<T> &A, i64 nnz, const T *X, Epi e, const EpiArgs &a) {
    QOp op;
    op.kind = QKind::Spmm;
    op.dbl = DT;
    op.epi = e;
    op.seglev = lev;
    op.n = A.n;
    op.lanes = lanes_of(nnz, A.n);
    if constexpr (DT) op.Ad = whole(A);
    else op.Af = whole(A);
    op.x0 = X;
    op.a = a;
    op.a.mirror();
    ops.push_back(op);
  }
  QOp &elem(QKind kind, int lev, i64 n, const void *x0, const void *x1, void *y0, double f = 1,
            int dbl = DT) {
    QOp op;
    op.kind = kind;
    op.dbl = dbl;
    op.seglev = lev;
    op.n = n;
    op.x0 = x0;
    op.x1 = x1;
    op.y0 = y0;
    op.f = f;
    ops.push_back(op);
    return ops.back();
  }

  void smooth(size_t l, T *x, const T *b, int iters, bool x_zero) {
    Level &L = *H.h[l];
    LevelWork<T> &lw = W.lw[l];
    const int lv = (int)l;
    i64 n = L.A.n;
    MatView<T> A = viewA<T>(L, 1, s);
    const T *invd = invdT<T>(L);
    if (o().smoother_type == LIGMG_SMOOTHER_JACOBI) {
      const double omega = 2.0 / 3.0;
      if (x_zero) {
        elem(QKind::Cheb0, lv, n, b, invd, x, omega);
        return;
      }
      EpiArgs a;
      a.b = b; a.invd = invd; a.xin = x; a.y = lw.xt.p; a.c1 = omega;
      spmm(lv, A, L.A.nnz, x, Epi::Jacobi, a);
      elem(QKind::Copy, lv, n, lw.xt.p, nullptr, x);
      return;
    }
    if (iters <= 0) return;
    const T *r_cur;
    const T *x_cur;
    T *d_cur;
    T *d_other = lw.d1.p;
    int first = 1;
    if (x_zero && iters == 1) {
      elem(QKind::Cheb0, lv, n, b, invd, x, 1.0 / L.theta);
      return;
    }
    if (x_zero) {
      const bool last = iters == 2;
      EpiArgs a;
      a.b = b; a.invd = invd; a.ith = 1.0 / L.theta; a.c1 = L.c1[0]; a.c2 = L.c2[0];
      a.rout = last ? nullptr : lw.r.p;
      a.dout = last ? nullptr : lw.d1.p;
      a.xout = last ? x : lw.xt.p;
      spmm(lv, viewAD<T>(L, 1, s), L.A.nnz, b, Epi::ChebZ, a);
      if (last) return;
      r_cur = lw.r.p;
      d_cur = lw.d1.p;
      d_other = lw.d0.p;
      x_cur = lw.xt.p;
      first = 2;
    } else {
      EpiArgs a;
      a.b = b; a.invd = invd; a.xin = x; a.rout = lw.r.p; a.dout = lw.d0.p; a.xout = lw.xt.p;
      a.ith = 1.0 / L.theta;
      spmm(lv, A, L.A.nnz, x, Epi::ChebA, a);
      d_cur = lw.d0.p;
      x_cur = lw.xt.p;
      r_cur = lw.r.p;
      if (iters == 1) {
        elem(QKind::Copy, lv, n, lw.xt.p, nullptr, x);
        return;
      }
    }
    for (int it = first; it < iters; it++) {
      bool last = it == iters - 1;
      EpiArgs a;
      a.invd = invd;
      a.rin = r_cur;
      a.din = d_cur;
      a.xin = x_cur;
      a.c1 = L.c1[it - 1];
      a.c2 = L.c2[it - 1];
      a.rout = last ? nullptr : lw.r.p;
      a.dout = last ? nullptr : d_other;
      a.xout = last ? x : lw.xt.p;
      spmm(lv, A, L.A.nnz, d_cur, Epi::ChebB, a);
      if (!last) {
        r_cur = lw.r.p;
        std::swap(d_cur, d_other);
        x_cur = lw.xt.p;
      }
    }
  }

  void cycle(size_t l, const T *b, T *x) {
    Level &L = *H.h[l];
    const int lv = (int)l;
    i64 n = L.A.n;
    if (L.type == LIGMG_LEVEL_COARSE) {
      elem(QKind::Coarse, lv, n, b, pinvT<T>(L), x);
      return;
    }
    LevelWork<T> &nw = W.lw[l + 1];
    if (L.type == LIGMG_LEVEL_ELIM) {
      EpiArgs a;
      a.y = nw.in.p;
      spmm(lv + 1, viewR<T>(L, 1, s), L.elim.R.nnz, b, Epi::Store, a);
      recurse(l, nw.in.p, nw.out.p);
      EpiArgs c;
      c.y = x; c.b = b; c.q = QT<T>(L);
      spmm(lv, viewP<T>(L), L.elim.P.nnz, nw.out.p, Epi::ElimInterp, c);
      return;
    }
    smooth(l, x, b, o().pre_smooth, true);
    EpiArgs rs;
    rs.y = nw.in.p;
    spmm(lv + 1, viewC<T>(L, 1, x, s), L.Cr.nnz, b, Epi::Split, rs);
    recurse(l, nw.in.p, nw.out.p);
    QOp &pr = elem(QKind::Prolong, lv, n, nw.out.p, nullptr, x);
    pr.idx = L.agg.agg.p;
    smooth(l, x, b, o().post_smooth, false);
    if (o().constant_correction) elem(QKind::Scale, lv, n, nullptr, nullptr, x, 4.0 / 3.0);
  }

  void recurse(size_t l, T *bc, T *xc) {
    const Level &N = *H.h[l + 1];
    if (!o().kcycle || N.is_exact() || N.type == LIGMG_LEVEL_COARSE) {
      cycle(l + 1, bc, xc);
      return;
    }
    fcg_fixed(l + 1, bc, xc, o().kcycle_iters);
  }

  // K-cycle inner FCG in segment mode: per-graph scalars, x = 0 first
  void fcg_fixed(size_t l, T *b, T *x, int iters) {
    Level &L = *H.h[l];
    LevelWork<T> &lw = W.lw[l];
    const int lv = (int)l;
    i64 n = L.A.n;
    MatView<T> A = viewA<T>(L, 1, s);
    elem(QKind::Zero, lv, n, nullptr, nullptr, x);
    T *r = b;
    T *p = lw.fp0.p, *pp = lw.fp1.p, *q = lw.fq0.p, *qp = lw.fq1.p;
    FcgScalars sc{lw.sslot(S_SUM), lw.sslot(S_BETA), lw.sslot(S_ETA0), lw.sslot(S_ETA1),
                  lw.sslot(S_ALPHA), nullptr};
    for (int it = 0; it < iters; it++) {
      cycle(l, r, lw.fz.p);
      QOp &rb = elem(QKind::RedBeta, lv, n, lw.fz.p, it > 0 ? qp : nullptr, nullptr);
      rb.flag = it > 0;
      rb.sc = sc;
      QOp &d = elem(QKind::Dir, lv, n, lw.fz.p, it > 0 ? pp : nullptr, p);
      d.flag = it > 0;
      d.sc = sc;
      EpiArgs a;
      a.y = q;
      spmm(lv, A, L.A.nnz, p, Epi::Store, a);
      QOp &ra = elem(QKind::RedAlpha, lv, n, p, q, nullptr);
      ra.x2 = r;
      ra.sc = sc;
      QOp &u = elem(QKind::Update, lv, n, p, q, x);
      u.y1 = r;
      u.flag = it + 1 < iters;
      u.sc = sc;
      std::swap(p, pp);
      std::swap(q, qp);
      std::swap(sc.eta, sc.eta_prev);
    }
  }

  // one outer FCG iteration (seg_outer_iteration with a native FP64 product)
  void outer(size_t base, int it) {
    Level &L = *H.h[base];
    const int lv = (int)base;
    const i64 n = L.A.n, ns = L.seginfo().nseg;
    SegOuter &so = w.so;
    auto slot = [&](int q) { return so.sc.p + (i64)q * ns; };
    const bool odd = it & 1;
    double *P = odd ? w.P1.p : w.P0.p, *PP = odd ? w.P0.p : w.P1.p;
    double *Q = odd ? w.Q1.p : w.Q0.p, *QP = odd ? w.Q0.p : w.Q1.p;
    double *eta = odd ? slot(S_ETA1) : slot(S_ETA0), *eta_prev = odd ? slot(S_ETA0) : slot(S_ETA1);
    if constexpr (DT) {
      cycle(base, w.R.p, w.Z.p);
    } else {
      LevelWork<T> &lw = W.lw[base];
      elem(QKind::ToFloat, lv, n, w.R.p, nullptr, lw.in.p, 1, 0);
      cycle(base, lw.in.p, lw.out.p);
      elem(QKind::ToDouble, lv, n, lw.out.p, nullptr, w.Z.p, 1, 0);
    }
    QOp &rs = elem(QKind::RedSum, lv, n, w.Z.p, nullptr, nullptr, 1, 1);
    rs.out = slot(S_SUM);
    elem(QKind::SubMean, lv, n, nullptr, slot(S_SUM), w.Z.p, 1, 1);
    FcgScalars sc{slot(S_ZQ), slot(S_BETA), eta, eta_prev, slot(S_ALPHA), so.frozen.p};
    QOp &rb = elem(QKind::RedBeta, lv, n, w.Z.p, it > 0 ? QP : nullptr, nullptr, 1, 1);
    rb.flag = it > 0;
    rb.sc = sc;
    QOp &d = elem(QKind::Dir, lv, n, w.Z.p, it > 0 ? PP : nullptr, P, 1, 1);
    d.flag = it > 0;
    d.sc = sc;
    QOp sp;
    sp.kind = QKind::Spmm;
    sp.dbl = 1;
    sp.epi = Epi::Store;
    sp.seglev = lv;
    sp.n = n;
    sp.lanes = lanes_of(L.A.nnz, n);
    sp.Ad = whole(viewA<double>(L, 1, s));
    sp.x0 = P;
    sp.a.y = Q;
    ops.push_back(sp);
    QOp &ra = elem(QKind::RedAlpha, lv, n, P, Q, nullptr, 1, 1);
    ra.x2 = w.R.p;
    ra.sc = sc;
    QOp &u = elem(QKind::Update, lv, n, P, Q, w.X.p, 1, 1);
    u.y1 = w.R.p;
    u.flag = 1;
    u.sc = sc;
    QOp &rn = elem(QKind::RedNorm, lv, n, w.R.p, nullptr, nullptr, 1, 1);
    rn.out = so.rn2.p;
    rn.rn0sq = so.rn0sq.p;
    rn.tol2 = H.opts.tol * H.opts.tol;
    rn.frozen = so.frozen.p;
    rn.iters = so.iters.p;
    rn.it = it;
  }
};

// Record kQueueIters outer iterations from it0 as a program: the operations
// and their (graph, row block) items.
template <typename T>
void queue_record(Handle &H, Work<T> &W, OuterWork &w, size_t base, int it0, QueueProgram &P) {
  QueueBuilder<T> B(H, W, w);
  for (int it = it0; it < it0 + kQueueIters; it++) B.outer(base, it);
  const i64 ns = H.h[base]->seginfo().nseg;
  const size_t nops = B.ops.size();
  // Items per graph: a block item per row block of an operation where the
  // graph has more than kQueueRows rows, and one chain item for every run of
  // consecutive operations where it has fewer.  Sorted (first operation,
  // graph, block), every item depends only on items with smaller tickets.
  std::vector<unsigned long long> items;
  for (i64 g = 0; g < ns; g++) {
    auto rows = [&](size_t i) {
      const std::vector<i64> &sg = H.h[B.ops[i].seglev]->seg_host;
      return sg[g + 1] - sg[g];
    };
    size_t i = 0;
    while (i < nops) {
      const i64 r = rows(i);
      if (r > kQueueRows) {
        const i64 nb = cdiv(r, kQueueRows);
        if (nb > kQueueMaxBlocks)
          throw Error(LIGMG_ERR_UNSUPPORTED, "a graph of the batch is too large for the work queue");
        for (i64 b = 0; b < nb; b++)
          items.push_back(((unsigned long long)i << 40) | ((unsigned long long)g << 20) |
                          (unsigned long long)b);
        i++;
        continue;
      }
      const size_t i0 = i;
      while (i < nops && rows(i) <= kQueueRows && i - i0 < (size_t)kQueueChain - 1) i++;
      items.push_back(((unsigned long long)i0 << 40) | ((unsigned long long)g << 20) |
                      kQueueChain | (unsigned long long)(i - i0));
    }
  }
  std::sort(items.begin(), items.end());
  if (B.ops.size() >= ((size_t)1 << 23) || ns >= ((i64)1 << 20))
    throw Error(LIGMG_ERR_UNSUPPORTED, "batch program too large for the work queue");
  P.ops.alloc((i64)B.ops.size(), H.s);
  P.ops.upload(B.ops.data(), (i64)B.ops.size());
  P.items.alloc((i64)items.size(), H.s);
  P.items.upload(items.data(), (i64)items.size());
  P.nitems = items.size();
  LG_CUDA(cudaStreamSynchronize(H.s));
}

// Batch outer solve on the work-queue kernel: one launch per kQueueIters
// outer iterations of every graph (captured with its state reset in a CUDA
// graph), relaunched until all graphs have converged or the limit is reached.
template <typename T>
SolveResult outer_solve_queue(Handle &H, size_t base, OuterWork &w) {
  cudaStream_t s = H.s;
  Level &L = *H.h[base];
  const i64 n = L.A.n;
  const SegInfo S = L.seginfo();
  const i64 ns = S.nseg;
  SegOuter &so = w.so;
  if (so.frozen.n != ns) {
    so.sc.alloc((i64)S_NSLOT * ns, s);
    so.sc.zero();
    so.rn2.alloc(ns, s);
    so.rn0sq.alloc(ns, s);
    so.frozen.alloc(ns, s);
    so.iters.alloc(ns, s);
  }
  LG_CUDA(cudaMemsetAsync(w.X.p, 0, sizeof(double) * n, s));
  LG_CUDA(cudaMemcpyAsync(w.R.p, w.B.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  LG_CUDA(cudaMemsetAsync(so.frozen.p, 0, sizeof(int) * ns, s));
  seg_dot<double>(S, w.R.p, w.R.p, so.rn0sq.p, s);
  seg_converge(ns, so.rn0sq.p, so.rn0sq.p, 0.0, -1, so.frozen.p, so.iters.p, s);  // b = 0
  Work<T> &W = work_for<T>(H, 1);
  const int prec = (int)sizeof(T);
  if (!H.queue || H.queue->base != base || H.queue->prec != prec) {
    H.queue.reset(new QueueRun());
    QueueRun &Q = *H.queue;
    Q.base = base;
    Q.prec = prec;
    std::vector<const i64 *> segs;
    for (auto &lv : H.h) segs.push_back(lv->segptr.p);
    Q.segs.alloc((i64)segs.size(), s);
    Q.segs.upload(segs.data(), (i64)segs.size());
    Q.prog.alloc(ns, s);
    Q.blk.alloc(ns, s);
    Q.part.alloc(ns * kQueueMaxBlocks * 3, s);
    Q.st.alloc(1, s);
    Q.st.zero();
    queue_record<T>(H, W, w, base, 0, Q.first);
    queue_record<T>(H, W, w, base, kQueueIters, Q.more);
  }
  QueueRun &Q = *H.queue;
  auto args = [&](QueueProgram &P) {
    QueueArgs a;
    a.ops = P.ops.p;
    a.items = P.items.p;
    a.nitems = P.nitems;
    a.segs = Q.segs.p;
    a.nseg = (int)ns;
    a.prog = Q.prog.p;
    a.blk = Q.blk.p;
    a.part = Q.part.p;
    a.frozen = so.frozen.p;
    a.st = Q.st.p;
    a.wait_limit = H.opts.wait_spins > 0 ? H.opts.wait_spins : (1ll << 23);
    return a;
  };
  // the launch and its state reset (ticket, error, progress counters) as one
  // captured graph per program
  auto graph_of = [&](QueueProgram &P) {
    if (P.exec) return P.exec;
    cudaGraph_t g = nullptr;
    LG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    try {
      LG_CUDA(cudaMemsetAsync(Q.st.p, 0, offsetof(QueueState, it_offset), s));
      LG_CUDA(cudaMemsetAsync(Q.prog.p, 0, sizeof(int) * ns, s));
      LG_CUDA(cudaMemsetAsync(Q.blk.p, 0, sizeof(int) * ns, s));
      launch_queue(args(P), s);
    } catch (...) {
      cudaStreamEndCapture(s, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    LG_CUDA(cudaStreamEndCapture(s, &g));
    cudaError_t e = cudaGraphInstantiate(&P.exec, g, 0);
    cudaGraphDestroy(g);
    LG_CUDA(e);
    add_launches(-1);  // the capture counted the launch; replays count it below
    return P.exec;
  };
  SolveResult res;
  std::vector<int> fz(ns), its(ns);
  int done = 0;
  for (int launch = 0; done < H.opts.iters; launch++) {
    QueueProgram &P = launch == 0 ? Q.first : Q.more;
    cudaGraphExec_t ex = graph_of(P);
    const int offset = launch == 0 ? 0 : done - kQueueIters;
    LG_CUDA(cudaMemcpyAsync(&Q.st.p->it_offset, &offset, sizeof(int), cudaMemcpyHostToDevice, s));
    LG_CUDA(cudaGraphLaunch(ex, s));
    add_launches(1);
    done += kQueueIters;
    QueueState hs{};
    LG_CUDA(cudaMemcpyAsync(&hs, Q.st.p, sizeof(QueueState), cudaMemcpyDeviceToHost, s));
    LG_CUDA(cudaMemcpyAsync(fz.data(), so.frozen.p, sizeof(int) * ns, cudaMemcpyDeviceToHost, s));
    LG_CUDA(cudaStreamSynchronize(s));
    if (hs.err) throw Error(LIGMG_ERR_INTERNAL, "batch work queue: a wait ran out");
    bool all = true;
    for (int v : fz) all = all && v;
    if (all) break;
  }
  std::vector<double> r2(ns), r0(ns);
  LG_CUDA(cudaMemcpyAsync(its.data(), so.iters.p, sizeof(int) * ns, cudaMemcpyDeviceToHost, s));
  LG_CUDA(cudaMemcpyAsync(r2.data(), so.rn2.p, sizeof(double) * ns, cudaMemcpyDeviceToHost, s));
  LG_CUDA(cudaMemcpyAsync(r0.data(), so.rn0sq.p, sizeof(double) * ns, cudaMemcpyDeviceToHost, s));
  LG_CUDA(cudaStreamSynchronize(s));
  res.converged = true;
  res.col_iters = its;
  res.rel.assign(ns, 0.0);
  for (i64 g = 0; g < ns; g++) {
    if (!std::isfinite(r0[g]))
      throw Error(LIGMG_ERR_NONFINITE, "right-hand side holds a NaN or Inf");
    if (!std::isfinite(r2[g]) && !fz[g]) throw Error(LIGMG_ERR_BREAKDOWN, "non-finite residual");
    res.converged = res.converged && fz[g];
    res.iters = std::max(res.iters, its[g]);
    res.rel[g] = r0[g] > 0 ? std::sqrt(r2[g] / r0[g]) : 0.0;
  }
  res.hist0 = {std::sqrt(r0[0]), std::sqrt(r2[0])};
  return res;
}

template <typename T>
SolveResult outer_solve_seg(Handle &H, size_t base, OuterWork &w) {
  cudaStream_t s = H.s;
  Level &L = *H.h[base];
  i64 n = L.A.n;
  const SegInfo S = L.seginfo();
  i64 ns = S.nseg;
  bool dfprod = sizeof(T) == 4;
  if (dfprod && L.Adf.n != L.A.nnz) {
    L.Adf.alloc(L.A.nnz, s);
    split_df(L.A.nnz, L.A.v.p, L.Adf.p, s);
  }
  SegOuter &so = w.so;
  if (so.frozen.n != ns || so.Pdf.n != n) {
    so.sc.alloc((i64)S_NSLOT * ns, s);
    so.sc.zero();
    so.rn2.alloc(ns, s);
    so.rn0sq.alloc(ns, s);
    so.frozen.alloc(ns, s);
    so.iters.alloc(ns, s);
    so.Pdf.alloc(n, s);
  }
  // x0 = 0, r0 = b (b's constant per graph already removed by the caller)
  LG_CUDA(cudaMemsetAsync(w.X.p, 0, sizeof(double) * n, s));
  LG_CUDA(cudaMemcpyAsync(w.R.p, w.B.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  LG_CUDA(cudaMemsetAsync(so.frozen.p, 0, sizeof(int) * ns, s));
  seg_dot<double>(S, w.R.p, w.R.p, so.rn0sq.p, s);
  seg_converge(ns, so.rn0sq.p, so.rn0sq.p, 0.0, -1, so.frozen.p, so.iters.p, s);  // b = 0
  // direct run of one cycle: creates every lazily built plan and buffer
  apply_prec_body<T>(H, 1, base, w.R.p, w.Z.p, so.sc.p, w.scratch.p, w.scratch_len);
  auto capture = [&](int it0, int64_t &kernels) {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t e = nullptr;
    const int64_t c0 = launches_now();
    LG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    H.prof.suspended = true;
    try {
      for (int it = it0; it < it0 + kGraphIters; it++)
        seg_outer_iteration<T>(H, base, w, so, it, dfprod);
    } catch (...) {
      H.prof.suspended = false;
      cudaStreamEndCapture(s, &g);
      if (g) cudaGraphDestroy(g);
      add_launches(c0 - launches_now());
      throw;
    }
    H.prof.suspended = false;
    kernels = launches_now() - c0;
    add_launches(-kernels);
    LG_CUDA(cudaStreamEndCapture(s, &g));
    cudaError_t err = cudaGraphInstantiate(&e, g, 0);
    cudaGraphDestroy(g);
    LG_CUDA(err);
    return e;
  };
  if (!H.batch_first || H.batch_base != base) {
    if (H.batch_first) cudaGraphExecDestroy(H.batch_first);
    if (H.batch_more) cudaGraphExecDestroy(H.batch_more);
    H.batch_first = capture(0, H.batch_first_kernels);
    H.batch_more = capture(kGraphIters, H.batch_more_kernels);
    H.batch_base = base;
  }
  SolveResult res;
  std::vector<int> fz(ns), its(ns);
  int done = 0;
  for (int launch = 0; done < H.opts.iters; launch++) {
    LG_CUDA(cudaGraphLaunch(launch == 0 ? H.batch_first : H.batch_more, s));
    add_launches(launch == 0 ? H.batch_first_kernels : H.batch_more_kernels);
    done += kGraphIters;
    LG_CUDA(cudaMemcpyAsync(fz.data(), so.frozen.p, sizeof(int) * ns, cudaMemcpyDeviceToHost, s));
    LG_CUDA(cudaStreamSynchronize(s));
    bool all = true;
    for (int v : fz) all = all && v;
    if (all) break;
  }
  std::vector<double> r2(ns), r0(ns);
  LG_CUDA(cudaMemcpyAsync(its.data(), so.iters.p, sizeof(int) * ns, cudaMemcpyDeviceToHost, s));
  LG_CUDA(cudaMemcpyAsync(r2.data(), so.rn2.p, sizeof(double) * ns, cudaMemcpyDeviceToHost, s));
  LG_CUDA(cudaMemcpyAsync(r0.data(), so.rn0sq.p, sizeof(double) * ns, cudaMemcpyDeviceToHost, s));
  LG_CUDA(cudaStreamSynchronize(s));
  res.converged = true;
  res.col_iters = its;
  res.rel.assign(ns, 0.0);
  for (i64 g = 0; g < ns; g++) {
    if (!std::isfinite(r0[g]))
      throw Error(LIGMG_ERR_NONFINITE, "right-hand side holds a NaN or Inf");
    if (!std::isfinite(r2[g])) throw Error(LIGMG_ERR_BREAKDOWN, "non-finite residual");
    res.converged = res.converged && fz[g];
    res.iters = std::max(res.iters, its[g]);
    res.rel[g] = r0[g] > 0 ? std::sqrt(r2[g] / r0[g]) : 0.0;
  }
  res.hist0 = {std::sqrt(r0[0]), std::sqrt(r2[0])};
  return res;
}

// full solve: B (n0 x k) in w.Bfull -> w.Xfull; fills info
// Raise the error of any persistent tail launch of this handle.
void check_tails(Handle &H) {
  for (auto &w : H.w32) tail_check<float>(H, *w.second, H.s);
  for (auto &w : H.w64) tail_check<double>(H, *w.second, H.s);
}

ligmg_status solve_device(Handle &H, int k, int from, const double *dB, double *dX,
                          ligmg_info *info) {
  auto t0 = std::chrono::steady_clock::now();
  DepLaunchScope dep(H.opts.pdl != 0);
  cudaStream_t s = H.s;
  if (from < 0 || from >= (int)H.h.size()) throw Error(LIGMG_ERR_INVALID_ARGUMENT, "from");
  Level &F = *H.h[from];
  i64 n0 = F.A.n;
  bool do_once = H.opts.top_elim && F.type == LIGMG_LEVEL_ELIM;  // multigrid.hpp:322
  size_t base = do_once ? from + 1 : from;
  i64 nb = H.h[base]->A.n;
  if (H.h[base]->type == LIGMG_LEVEL_COARSE && H.h.size() == 1)
    ;  // single coarse level: the pseudo-inverse is the preconditioner
  OuterWork &w = outer_work(H, k, nb, n0);
  const SegInfo SF = F.seginfo();
  const bool seg = SF.nseg > 0;
  if (seg && k != 1) throw Error(LIGMG_ERR_UNSUPPORTED, "batch mode solves one RHS per graph");
  DBuf<double> segbuf;
  if (seg) segbuf.alloc(2 * SF.nseg, s);
  LG_CUDA(cudaMemcpyAsync(w.Bfull.p, dB, sizeof(double) * n0 * k, cudaMemcpyDeviceToDevice, s));
  // remove the constant from b first (the reference expects a mean-free b
  // from its caller, main.cpp:138-139; R 1 is not constant)
  if (seg) {
    seg_mean<double>(SF, w.Bfull.p, segbuf.p, s);
    seg_sub_mean<double>(SF, n0, w.Bfull.p, segbuf.p, s);
  } else {
    col_reduce<double>(n0, k, Red::Sum, w.Bfull.p, nullptr, w.slot(S_SUM), w.scratch.p,
                       w.scratch_len, s);
    sub_mean<double>(n0, k, w.Bfull.p, w.slot(S_SUM), s);
  }
  if (do_once) {
    EpiArgs a;
    a.y = w.B.p;
    timed(H, from, LIGMG_KERNEL_ELIM_RESTRICT, k, 1,
          core_bytes(F.elim.R.n, F.elim.R.nnz, n0, k, 8) + 8.0 * F.elim.R.n * k,
          [&] { spmm<double>(viewR<double>(F, k, s), w.Bfull.p, k, Epi::Store, a, s); });
  } else {
    LG_CUDA(cudaMemcpyAsync(w.B.p, w.Bfull.p, sizeof(double) * n0 * k, cudaMemcpyDeviceToDevice, s));
  }
  SolveResult res;
  if (seg && H.opts.outer_ksp_type == LIGMG_KSP_FGMRES)
    throw Error(LIGMG_ERR_UNSUPPORTED, "batch mode runs FCG or CG outer iterations");
  if (seg)
    if (H.opts.batch_queue)
      res = (H.opts.precision == LIGMG_PREC_FP32) ? outer_solve_queue<float>(H, base, w)
                                                  : outer_solve_queue<double>(H, base, w);
    else
      res = (H.opts.precision == LIGMG_PREC_FP32) ? outer_solve_seg<float>(H, base, w)
                                                  : outer_solve_seg<double>(H, base, w);
  else if (H.opts.outer_ksp_type == LIGMG_KSP_FGMRES)
    res = (H.opts.precision == LIGMG_PREC_FP32) ? outer_solve_fgmres<float>(H, base, w, k)
                                                : outer_solve_fgmres<double>(H, base, w, k);
  else
    res = (H.opts.precision == LIGMG_PREC_FP32) ? outer_solve<float>(H, base, w, k)
                                                : outer_solve<double>(H, base, w, k);
  if (do_once) {  // x = P x + Q b (:349-354)
    EpiArgs c;
    c.y = w.Xfull.p; c.b = w.Bfull.p; c.q = F.elim.Q.p;
    timed(H, from, LIGMG_KERNEL_ELIM_INTERP, k, 1,
          core_bytes(n0, F.elim.P.nnz, nb, k, 8) + (2.0 * n0 * k + n0) * 8,
          [&] { spmm<double>(viewP<double>(F), w.X.p, k, Epi::ElimInterp, c, s); });
  } else {
    LG_CUDA(cudaMemcpyAsync(w.Xfull.p, w.X.p, sizeof(double) * n0 * k, cudaMemcpyDeviceToDevice, s));
  }
  LG_CUDA(cudaMemcpyAsync(dX, w.Xfull.p, sizeof(double) * n0 * k, cudaMemcpyDeviceToDevice, s));
  // true residual ||b - L x|| / ||b|| with b's constant projected out
  double *d1 = w.slot(S_ZQ), *d2 = w.slot(S_BETA);
  EpiArgs a;
  a.y = w.Res.p;
  a.b = w.Bfull.p;
  timed(H, from, LIGMG_KERNEL_RESID, k, 1, core_bytes(n0, F.A.nnz, n0, k, 8) + 16.0 * n0 * k,
        [&] { spmm<double>(viewA<double>(F, k, s), w.Xfull.p, k, Epi::Resid, a, s); });
  int kc = seg ? (int)SF.nseg : k;  // reported columns: RHS columns or graphs
  std::vector<double> h1(kc), h2(kc);
  if (seg) {
    seg_dot<double>(SF, w.Res.p, w.Res.p, segbuf.p, s);
    seg_dot<double>(SF, w.Bfull.p, w.Bfull.p, segbuf.p + SF.nseg, s);
    LG_CUDA(cudaMemcpyAsync(h1.data(), segbuf.p, sizeof(double) * kc, cudaMemcpyDeviceToHost, s));
    LG_CUDA(cudaMemcpyAsync(h2.data(), segbuf.p + SF.nseg, sizeof(double) * kc,
                            cudaMemcpyDeviceToHost, s));
  } else {
    col_reduce<double>(n0, k, Red::Dot, w.Res.p, w.Res.p, d1, w.scratch.p, w.scratch_len, s);
    col_reduce<double>(n0, k, Red::Dot, w.Bfull.p, w.Bfull.p, d2, w.scratch.p, w.scratch_len, s);
    LG_CUDA(cudaMemcpyAsync(h1.data(), d1, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
    LG_CUDA(cudaMemcpyAsync(h2.data(), d2, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
  }
  LG_CUDA(cudaStreamSynchronize(s));
  double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  H.prof.collect();
  if (info) {
    double worst_true = 0, worst_rel = 0;
    for (int c = 0; c < kc; c++) {
      double tr = h2[c] > 0 ? std::sqrt(h1[c]) / std::sqrt(h2[c]) : 0.0;
      worst_true = std::max(worst_true, tr);
      worst_rel = std::max(worst_rel, res.rel[c]);
      if (info->col_iters) info->col_iters[c] = res.col_iters[c];
      if (info->col_true_rel_residual) info->col_true_rel_residual[c] = tr;
    }
    info->iters = res.iters;
    info->converged = res.converged ? 1 : 0;
    info->rel_residual = worst_rel;
    info->true_rel_residual = worst_true;
    info->cycle_complexity = cycle_complexity(H, (int)base);
    info->work = res.iters * (1 + info->cycle_complexity);
    info->solve_seconds = secs;
    info->setup_seconds = H.setup_s;
    info->history_len = 0;
    if (info->residual_history && info->history_capacity > 0) {
      int m = std::min((int)res.hist0.size(), info->history_capacity);
      std::copy(res.hist0.begin(), res.hist0.begin() + m, info->residual_history);
      info->history_len = m;
    }
  }
  check_tails(H);
  return res.converged ? LIGMG_OK : LIGMG_NOT_CONVERGED;
}

bool k_supported(int k) {
  return k == 1 || k == 2 || k == 4 || k == 8 || k == 16 || k == 32 || k == 64;
}

// the message of the last failed call in this thread (ligmg_last_error)
thread_local std::string g_last_error;

template <typename F>
ligmg_status guard_impl(F &&f) {
  try {
    (void)cudaGetLastError();  // a failed earlier call must not leak into this one
    return f();
  } catch (const Error &e) {
    g_last_error = e.what();
    return e.status;
  } catch (const std::bad_alloc &) {
    g_last_error = "host allocation failed";
    return LIGMG_ERR_OUT_OF_MEMORY;
  } catch (const std::exception &e) {
    g_last_error = e.what();
    return LIGMG_ERR_INTERNAL;
  } catch (...) {
    g_last_error = "unknown error";
    return LIGMG_ERR_INTERNAL;
  }
}
template <typename F>
ligmg_status guard(F &&f) {
  return guard_impl(std::forward<F>(f));
}

}  // namespace
}  // namespace lg

using namespace lg;

extern "C" {

void ligmg_default_options(ligmg_options *o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->max_levels = 50;
  o->always_elim = 1;
  o->min_size = 4000;
  o->top_elim = 1;
  o->elim_degree = 4;
  o->elim_factor = 0.9;
  o->elim_iters = 1;
  o->iters = 500;
  o->tol = 1e-8;
  o->thresh = 1e-8;
  o->agg_iters = 10;
  o->num_tvs = 10;
  o->agg_init_factor = 0.5;
  o->agg_iter_factor = 0.5;
  o->votes_to_seed = 1;
  o->max_agg_size = -1;
  o->rejection_ratio = -1;
  o->rejection_to_seed = 0;
  o->neighbor_of_neighbor = 0;
  o->tvs_smooth = 4;
  o->strength_metric = LIGMG_STRENGTH_AFFINITY;
  o->aff_scaling = LIGMG_AFF_MAX;
  o->pre_smooth = 2;
  o->post_smooth = 2;
  o->smoother_type = LIGMG_SMOOTHER_CHEBYSHEV;
  o->cheby_lower = 0.3;
  o->cheby_upper = 1.1;
  o->constant_correction = 0;
  o->kcycle = 0;
  o->kcycle_iters = 2;
  o->outer_ksp_type = LIGMG_KSP_CG;
  o->kcycle_ksp_type = LIGMG_KSP_FCG;
  o->precision = LIGMG_PREC_FP64;
  o->seed = 0;
  o->fcg_mmax = 1;
  o->rng_skip = 0;
  o->verbose = 0;
  o->device = 0;
  o->use_graphs = 1;
  o->autotune = 1;
  o->tail_rows = 0;
  o->gmres_restart = 30;
  o->spmv_tiles = 1;
  o->wait_spins = 0;
  o->batch_queue = 1;
  o->spmm_streams = 1;
  o->tail_cluster = 0;
  o->spmm_tiles = 1;
  o->pdl = 0;
}

const char *ligmg_status_string(ligmg_status s) {
  switch (s) {
    case LIGMG_OK: return "ok";
    case LIGMG_NOT_CONVERGED: return "not converged (iteration limit reached)";
    case LIGMG_ERR_INVALID_ARGUMENT: return "invalid argument";
    case LIGMG_ERR_NOT_SYMMETRIC: return "matrix not symmetric";
    case LIGMG_ERR_BAD_DIAGONAL: return "missing or non-positive diagonal";
    case LIGMG_ERR_POSITIVE_OFFDIAG: return "positive off-diagonal entry";
    case LIGMG_ERR_NONFINITE: return "non-finite value";
    case LIGMG_ERR_DISCONNECTED: return "graph is disconnected";
    case LIGMG_ERR_CUDA: return "CUDA error";
    case LIGMG_ERR_OUT_OF_MEMORY: return "out of device memory";
    case LIGMG_ERR_BREAKDOWN: return "Krylov breakdown";
    case LIGMG_ERR_UNSUPPORTED: return "unsupported option combination";
    case LIGMG_ERR_INTERNAL: return "internal error";
    case LIGMG_ERR_NOT_SORTED: return "CSR columns not sorted";
    default: return "unknown status";
  }
}

ligmg_status ligmg_create(int64_t n, const int64_t *rowptr, const int32_t *col,
                          const double *val, const ligmg_options *opts, ligmg_handle *out) {
  if (!out) return LIGMG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (n <= 0 || n >= INT32_MAX || !rowptr || !col || !val) return LIGMG_ERR_INVALID_ARGUMENT;
  if (rowptr[0] != 0 || rowptr[n] < n) return LIGMG_ERR_INVALID_ARGUMENT;
  return guard([&]() -> ligmg_status {
    std::unique_ptr<Handle> H(new Handle());
    if (opts) H->opts = *opts; else ligmg_default_options(&H->opts);
    const ligmg_options &o = H->opts;
    if (o.kcycle_iters < 1 || o.num_tvs < 0 || o.max_levels < 1 || o.iters < 0 ||
        (o.precision != LIGMG_PREC_FP64 && o.precision != LIGMG_PREC_FP32))
      return LIGMG_ERR_INVALID_ARGUMENT;
    if (o.outer_ksp_type == LIGMG_KSP_FGMRES && o.gmres_restart < 1)
      return LIGMG_ERR_INVALID_ARGUMENT;
    if (o.spmm_streams < 0 || o.spmm_streams > 2 || o.spmv_tiles < 0 || o.spmv_tiles > 2 ||
        o.pdl < 0 || o.pdl > 1 || o.spmm_tiles < 0 || o.spmm_tiles > 2)
      return LIGMG_ERR_INVALID_ARGUMENT;
    if (o.smoother_type > LIGMG_SMOOTHER_CHEBYSHEV || o.outer_ksp_type > LIGMG_KSP_FGMRES ||
        (o.kcycle_ksp_type != LIGMG_KSP_FCG && o.kcycle_ksp_type != LIGMG_KSP_FGMRES) ||
        o.elim_iters > 1 || o.aff_scaling < LIGMG_AFF_NONE || o.aff_scaling > LIGMG_AFF_MAX)
      return LIGMG_ERR_UNSUPPORTED;
    if (o.kcycle_ksp_type == LIGMG_KSP_FGMRES && o.kcycle_iters > kGmresInnerMax)
      return LIGMG_ERR_UNSUPPORTED;
    H->device = o.device;
    LG_CUDA(cudaSetDevice(H->device));
    LG_CUDA(cudaStreamCreateWithFlags(&H->s, cudaStreamNonBlocking));
    make_hierarchy(*H, n, rowptr, col, val);
    *out = H.release();
    return LIGMG_OK;
  });
}

ligmg_status ligmg_destroy(ligmg_handle h) {
  if (!h) return LIGMG_ERR_INVALID_ARGUMENT;
  return guard([&]() -> ligmg_status {
    cudaSetDevice(h->device);
    delete h;
    return LIGMG_OK;
  });
}

ligmg_status ligmg_solve_batched_device(ligmg_handle h, const double *dB, int32_t k, double *dX,
                                        ligmg_info *info) {
  if (!h || !dB || !dX || !k_supported(k)) return LIGMG_ERR_INVALID_ARGUMENT;
  return guard([&]() -> ligmg_status {
    LG_CUDA(cudaSetDevice(h->device));
    if (h->opts.precision == LIGMG_PREC_FP32) ensure_fp32(*h);
    return solve_device(*h, k, 0, dB, dX, info);
  });
}

static ligmg_status solve_host(ligmg_handle h, const double *B, int32_t k, double *X, int from,
                               ligmg_info *info) {
  if (!h || !B || !X || !k_supported(k)) return LIGMG_ERR_INVALID_ARGUMENT;
  return guard([&]() -> ligmg_status {
    LG_CUDA(cudaSetDevice(h->device));
    if (from < 0 || from >= (int)h->h.size()) return LIGMG_ERR_INVALID_ARGUMENT;
    if (h->opts.precision == LIGMG_PREC_FP32) ensure_fp32(*h);
    i64 n = h->h[from]->A.n;
    DBuf<double> dB(n * k, h->s), dX(n * k, h->s);
    dB.upload(B, n * k);
    ligmg_status st = solve_device(*h, k, from, dB.p, dX.p, info);
    dX.download(X, n * k);
    LG_CUDA(cudaStreamSynchronize(h->s));
    return st;
  });
}

ligmg_status ligmg_solve(ligmg_handle h, const double *b, double *x, ligmg_info *info) {
  return solve_host(h, b, 1, x, 0, info);
}
ligmg_status ligmg_solve_from(ligmg_handle h, const double *b, double *x, int32_t from,
                              ligmg_info *info) {
  return solve_host(h, b, 1, x, from, info);
}
ligmg_status ligmg_solve_batched(ligmg_handle h, const double *B, int32_t k, double *X,
                                 ligmg_info *info) {
  return solve_host(h, B, k, X, 0, info);
}

ligmg_status ligmg_forward(ligmg_handle h, const double *b, double *x, ligmg_info *info) {
  if (!h || !b || !x) return LIGMG_ERR_INVALID_ARGUMENT;
  return guard([&]() -> ligmg_status {
    LG_CUDA(cudaSetDevice(h->device));
    if (h->opts.precision == LIGMG_PREC_FP32) ensure_fp32(*h);
    i64 n = h->h[0]->A.n;
    DBuf<double> dB(n, h->s);
    if (h->fwd_x.n != n) h->fwd_x.alloc(n, h->s);
    dB.upload(b, n);
    ligmg_status st = solve_device(*h, 1, 0, dB.p, h->fwd_x.p, info);
    h->fwd_x.download(x, n);
    LG_CUDA(cudaStreamSynchronize(h->s));
    h->has_fwd = true;
    return st;
  });
}

ligmg_status ligmg_backward(ligmg_handle h, const double *g, double *dw, double *db,
                            ligmg_info *info) {
  if (!h || !g) return LIGMG_ERR_INVALID_ARGUMENT;
  if (!h->has_fwd) return LIGMG_ERR_INVALID_ARGUMENT;  // no kept forward solution
  return guard([&]() -> ligmg_status {
    LG_CUDA(cudaSetDevice(h->device));
    const Level &L0 = *h->h[0];
    i64 n = L0.A.n;
    DBuf<double> dG(n, h->s), lam(n, h->s);
    dG.upload(g, n);
    // adjoint solve: L is symmetric, so lambda = L^+ g uses the same hierarchy
    ligmg_status st = solve_device(*h, 1, 0, dG.p, lam.p, info);
    // db = lambda with its mean removed (x depends on b only through its
    // mean-free part)
    OuterWork &w = *h->ow[1];
    col_reduce<double>(n, 1, Red::Sum, lam.p, nullptr, w.slot(S_SUM), w.scratch.p,
                       w.scratch_len, h->s);
    sub_mean<double>(n, 1, lam.p, w.slot(S_SUM), h->s);
    if (dw) {
      DBuf<double> ddw(L0.A.nnz, h->s);
      k_edge_grad<<<grid_for(n * 32, 256), 256, 0, h->s>>>(L0.A.rp.p, L0.A.ci.p, n,
                                                           h->fwd_x.p, lam.p, ddw.p);
      LG_LAUNCH();
      ddw.download(dw, L0.A.nnz);
      LG_CUDA(cudaStreamSynchronize(h->s));
    }
    if (db) lam.download(db, n);
    LG_CUDA(cudaStreamSynchronize(h->s));
    return st;
  });
}

ligmg_status ligmg_prepare_graph(int64_t n, const int64_t *rowptr, const int32_t *col,
                                 const double *val, int32_t flags, int32_t device,
                                 int64_t *n_out, int64_t *nnz_out, int64_t *rowptr_out,
                                 int32_t *col_out, double *val_out, int64_t *orig_out) {
  if (n <= 0 || !rowptr || !col || !val || !n_out || !nnz_out ||
      (flags & ~(LIGMG_PREP_LCC | LIGMG_PREP_LAPLACIAN)))
    return LIGMG_ERR_INVALID_ARGUMENT;
  const bool arrays = rowptr_out || col_out || val_out;
  if (arrays && !(rowptr_out && col_out && val_out)) return LIGMG_ERR_INVALID_ARGUMENT;
  return guard([&]() -> ligmg_status {
    LG_CUDA(cudaSetDevice(device));
    cudaStream_t s = nullptr;
    LG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    PrepResult r;
    try {
      prepare_graph(n, rowptr, col, val, (flags & LIGMG_PREP_LCC) != 0,
                    (flags & LIGMG_PREP_LAPLACIAN) != 0, arrays || orig_out, r, s);
    } catch (...) {
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
      throw;
    }
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    *n_out = r.n;
    *nnz_out = r.nnz;
    if (arrays) {
      std::copy(r.rowptr.begin(), r.rowptr.end(), rowptr_out);
      std::copy(r.col.begin(), r.col.end(), col_out);
      std::copy(r.val.begin(), r.val.end(), val_out);
    }
    if (orig_out) std::copy(r.orig.begin(), r.orig.end(), orig_out);
    return LIGMG_OK;
  });
}

ligmg_status ligmg_solve_pcg_jacobi(ligmg_handle h, const double *b, double *x,
                                    ligmg_info *info) {
  if (!h || !b || !x) return LIGMG_ERR_INVALID_ARGUMENT;
  return guard([&]() -> ligmg_status {
    LG_CUDA(cudaSetDevice(h->device));
    auto t0 = std::chrono::steady_clock::now();
    cudaStream_t s = h->s;
    const Level &L = *h->h[0];
    i64 n = L.A.n;
    MatView<double> A = viewA<double>(L, 1, s);
    DBuf<double> X(n, s), R(n, s), Z(n, s), P(n, s), Q(n, s), sc(8, s), red(fused_scratch_len(n, 1), s);
    red.zero();
    R.upload(b, n);
    i64 slen = col_reduce_scratch(n, 1);
    DBuf<double> scratch(slen, s);
    col_reduce<double>(n, 1, Red::Sum, R.p, nullptr, sc.p, scratch.p, slen, s);
    sub_mean<double>(n, 1, R.p, sc.p, s);
    X.zero();
    auto prec = [&]() {  // z = D^-1 r, constant removed (null space on the Mat)
      k_mul_diag<<<grid_for(n, 256), 256, 0, s>>>(n, L.invd.p, R.p, Z.p);
      LG_LAUNCH();
      col_reduce<double>(n, 1, Red::Sum, Z.p, nullptr, sc.p, scratch.p, slen, s);
      sub_mean<double>(n, 1, Z.p, sc.p, s);
    };
    double *rz = sc.p + 1, *rz_old = sc.p + 2, *beta = sc.p + 3, *pq = sc.p + 4,
           *alpha = sc.p + 5, *rn2 = sc.p + 6;
    col_dot1<double>(n, 1, R.p, R.p, rn2, red.p, s);
    double rn0 = std::sqrt(read_scalar(rn2, s));
    if (!std::isfinite(rn0)) throw Error(LIGMG_ERR_NONFINITE, "right-hand side holds a NaN or Inf");
    std::vector<double> hist{rn0};
    int it = 0;
    bool conv = rn0 == 0;
    if (!conv) {
      prec();
      col_dot1<double>(n, 1, Z.p, R.p, rz, red.p, s);
      LG_CUDA(cudaMemcpyAsync(P.p, Z.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    }
    for (; !conv && it < h->opts.iters; it++) {
      EpiArgs a;
      a.y = Q.p;
      spmm<double>(A, P.p, 1, Epi::Store, a, s);
      col_dot1<double>(n, 1, P.p, Q.p, pq, red.p, s);
      scal_div(1, rz, pq, alpha, nullptr, s);
      fcg_update<double>(n, 1, X.p, R.p, P.p, Q.p, alpha, true, s);
      col_dot1<double>(n, 1, R.p, R.p, rn2, red.p, s);
      double rn = std::sqrt(read_scalar(rn2, s));
      hist.push_back(rn);
      if (!std::isfinite(rn)) throw Error(LIGMG_ERR_BREAKDOWN, "non-finite residual");
      if (rn <= std::max(h->opts.tol * rn0, 1e-60)) {
        conv = true;
        it++;
        break;
      }
      prec();
      LG_CUDA(cudaMemcpyAsync(rz_old, rz, sizeof(double), cudaMemcpyDeviceToDevice, s));
      col_dot1<double>(n, 1, Z.p, R.p, rz, red.p, s);
      scal_div(1, rz, rz_old, beta, nullptr, s);
      cg_direction<double>(n, 1, P.p, Z.p, beta, s);
    }
    X.download(x, n);
    LG_CUDA(cudaStreamSynchronize(s));
    if (info) {
      info->iters = it;
      info->converged = conv;
      info->rel_residual = rn0 > 0 ? hist.back() / rn0 : 0.0;
      info->true_rel_residual = info->rel_residual;
      info->cycle_complexity = (double)n / (double)L.A.nnz;  // main.cpp:177
      info->work = it * (1 + info->cycle_complexity);
      info->solve_seconds =
          std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      info->setup_seconds = 0;
      info->history_len = 0;
      if (info->residual_history && info->history_capacity > 0) {
        int m = std::min((int)hist.size(), info->history_capacity);
        std::copy(hist.begin(), hist.begin() + m, info->residual_history);
        info->history_len = m;
      }
    }
    return conv ? LIGMG_OK : LIGMG_NOT_CONVERGED;
  });
}

ligmg_status ligmg_batch_create(int32_t num_graphs, const int64_t *vertex_offsets,
                                const int64_t *rowptr, const int32_t *col, const double *val,
                                const ligmg_options *opts, ligmg_handle *out) {
  if (!out) return LIGMG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (num_graphs < 1 || !vertex_offsets || !rowptr || !col || !val)
    return LIGMG_ERR_INVALID_ARGUMENT;
  i64 n = vertex_offsets[num_graphs];
  if (vertex_offsets[0] != 0 || n <= 0 || n >= INT32_MAX || rowptr[0] != 0)
    return LIGMG_ERR_INVALID_ARGUMENT;
  for (int32_t g = 0; g < num_graphs; g++)
    if (vertex_offsets[g + 1] <= vertex_offsets[g]) return LIGMG_ERR_INVALID_ARGUMENT;
  return guard([&]() -> ligmg_status {
    std::unique_ptr<Handle> H(new Handle());
    if (opts) H->opts = *opts; else ligmg_default_options(&H->opts);
    const ligmg_options &o = H->opts;
    if (o.outer_ksp_type != LIGMG_KSP_FCG || o.smoother_type > LIGMG_SMOOTHER_CHEBYSHEV ||
        o.elim_iters > 1 || o.kcycle_ksp_type != LIGMG_KSP_FCG ||
        (o.precision != LIGMG_PREC_FP64 && o.precision != LIGMG_PREC_FP32))
      return LIGMG_ERR_UNSUPPORTED;
    H->seg0.assign(vertex_offsets, vertex_offsets + num_graphs + 1);
    H->device = o.device;
    LG_CUDA(cudaSetDevice(H->device));
    LG_CUDA(cudaStreamCreateWithFlags(&H->s, cudaStreamNonBlocking));
    make_hierarchy(*H, n, rowptr, col, val);
    *out = H.release();
    return LIGMG_OK;
  });
}

ligmg_status ligmg_batch_solve(ligmg_handle h, const double *b, double *x, int32_t *iters,
                               double *true_rel_residual, ligmg_info *info) {
  if (!h || !b || !x || h->seg0.empty()) return LIGMG_ERR_INVALID_ARGUMENT;
  return guard([&]() -> ligmg_status {
    LG_CUDA(cudaSetDevice(h->device));
    if (h->opts.precision == LIGMG_PREC_FP32) ensure_fp32(*h);
    i64 n = h->h[0]->A.n;
    ligmg_info local{};
    ligmg_info *inf = info ? info : &local;
    inf->col_iters = iters;
    inf->col_true_rel_residual = true_rel_residual;
    DBuf<double> dB(n, h->s), dX(n, h->s);
    dB.upload(b, n);
    ligmg_status st = solve_device(*h, 1, 0, dB.p, dX.p, inf);
    dX.download(x, n);
    LG_CUDA(cudaStreamSynchronize(h->s));
    return st;
  });
}

ligmg_status ligmg_level_prolongation(ligmg_handle h, int32_t level, int64_t *nnz,
                                      int64_t *rowptr, int32_t *col, double *val, double *q) {
  if (!h || !nnz || level < 0 || level >= (int)h->h.size()) return LIGMG_ERR_INVALID_ARGUMENT;
  const Level &L = *h->h[level];
  if (L.type == LIGMG_LEVEL_COARSE) return LIGMG_ERR_INVALID_ARGUMENT;
  return guard([&]() -> ligmg_status {
    LG_CUDA(cudaSetDevice(h->device));
    i64 n = L.A.n;
    if (L.type == LIGMG_LEVEL_AGG) {
      *nnz = n;
      if (rowptr)
        for (i64 i = 0; i <= n; i++) rowptr[i] = i;
      if (col) L.agg.agg.download(col, n);
      if (val)
        for (i64 i = 0; i < n; i++) val[i] = 1.0;
      if (q)
        for (i64 i = 0; i < n; i++) q[i] = 0.0;
    } else {
      *nnz = L.elim.P.nnz;
      if (rowptr) L.elim.P.rp.download(rowptr, n + 1);
      if (col) L.elim.P.ci.download(col, L.elim.P.nnz);
      if (val) L.elim.P.v.download(val, L.elim.P.nnz);
      if (q) L.elim.Q.download(q, n);
    }
    LG_CUDA(cudaStreamSynchronize(h->s));
    return LIGMG_OK;
  });
}

ligmg_status ligmg_import_hierarchy(int32_t num_levels, const ligmg_level_desc *levels,
                                    const ligmg_options *opts, ligmg_handle *out) {
  if (!out) return LIGMG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (num_levels < 1 || !levels) return LIGMG_ERR_INVALID_ARGUMENT;
  for (int32_t l = 0; l < num_levels; l++) {
    const ligmg_level_desc &d = levels[l];
    bool last = l == num_levels - 1;
    if (d.n <= 0 || !d.rowptr || !d.col || !d.val || d.rowptr[d.n] != d.nnz)
      return LIGMG_ERR_INVALID_ARGUMENT;
    if (last != (d.type == LIGMG_LEVEL_COARSE)) return LIGMG_ERR_INVALID_ARGUMENT;
    if (d.type == LIGMG_LEVEL_AGG && (!d.ids || d.nc <= 0)) return LIGMG_ERR_INVALID_ARGUMENT;
    if (d.type == LIGMG_LEVEL_ELIM && (!d.prow || !d.pcol || !d.pval || !d.q || d.nc <= 0))
      return LIGMG_ERR_INVALID_ARGUMENT;
    if (!last && levels[l + 1].n != d.nc) return LIGMG_ERR_INVALID_ARGUMENT;
  }
  return guard([&]() -> ligmg_status {
    std::unique_ptr<Handle> H(new Handle());
    if (opts) H->opts = *opts; else ligmg_default_options(&H->opts);
    H->device = H->opts.device;
    LG_CUDA(cudaSetDevice(H->device));
    LG_CUDA(cudaStreamCreateWithFlags(&H->s, cudaStreamNonBlocking));
    cudaStream_t s = H->s;
    auto t0 = std::chrono::steady_clock::now();
    H->nnz0 = levels[0].nnz;
    for (int32_t l = 0; l < num_levels; l++) {
      const ligmg_level_desc &d = levels[l];
      auto L = std::make_unique<Level>();
      L->type = d.type;
      L->A.n = L->A.m = d.n;
      L->A.nnz = d.nnz;
      L->A.rp.alloc(d.n + 1, s);
      L->A.ci.alloc(d.nnz, s);
      L->A.v.alloc(d.nnz, s);
      L->A.rp.upload(d.rowptr, d.n + 1);
      L->A.ci.upload(d.col, d.nnz);
      L->A.v.upload(d.val, d.nnz);
      if (l == 0) {
        ligmg_status st = gpu_validate(L->A, s);
        if (st != LIGMG_OK) return st;
      }
      L->nc = d.type == LIGMG_LEVEL_COARSE ? 0 : d.nc;
      if (d.type == LIGMG_LEVEL_AGG) {
        L->agg.nc = d.nc;
        L->agg.agg.alloc(d.n, s);
        L->agg.agg.upload(d.ids, d.n);
        gpu_members(L->agg.agg.p, d.n, d.nc, L->agg.mrp, L->agg.members, s);
      } else if (d.type == LIGMG_LEVEL_ELIM) {
        ElimResult &E = L->elim;
        E.accepted = true;
        E.nc = d.nc;
        E.P.n = d.n;
        E.P.m = d.nc;
        E.P.nnz = d.pnnz;
        E.P.rp.alloc(d.n + 1, s);
        E.P.ci.alloc(d.pnnz, s);
        E.P.v.alloc(d.pnnz, s);
        E.P.rp.upload(d.prow, d.n + 1);
        E.P.ci.upload(d.pcol, d.pnnz);
        E.P.v.upload(d.pval, d.pnnz);
        E.Q.alloc(d.n, s);
        E.Q.upload(d.q, d.n);
        gpu_transpose(E.P, E.R, s);
        std::vector<i32> nid(d.n, -1);  // coarse id of kept vertices (P entry 1 on a kept row)
        for (i64 i = 0; i < d.n; i++)
          if (d.q[i] == 0.0 && d.prow[i + 1] - d.prow[i] == 1) nid[i] = d.pcol[d.prow[i]];
        E.new_id.alloc(d.n, s);
        E.new_id.upload(nid.data(), d.n);
      } else {
        ligmg_status st = gpu_coarse_pinv(L->A, L->pinv, s);
        if (st != LIGMG_OK) return st;
      }
      finish_level(*H, *L);
      if (d.type == LIGMG_LEVEL_AGG) {
        estimate_lmax(*H, *L);
        setup_smoother_params(H->opts, *L);
      }
      LG_CUDA(cudaStreamSynchronize(s));
      H->h.push_back(std::move(L));
    }
    H->setup_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    *out = H.release();
    return LIGMG_OK;
  });
}

ligmg_status ligmg_hierarchy_levels(ligmg_handle h, int32_t *num_levels) {
  if (!h || !num_levels) return LIGMG_ERR_INVALID_ARGUMENT;
  *num_levels = (int32_t)h->h.size();
  return LIGMG_OK;
}

ligmg_status ligmg_level_info(ligmg_handle h, int32_t level, int32_t *type, int64_t *n,
                              int64_t *nnz, int64_t *nc) {
  if (!h || level < 0 || level >= (int)h->h.size()) return LIGMG_ERR_INVALID_ARGUMENT;
  const Level &L = *h->h[level];
  if (type) *type = L.type;
  if (n) *n = L.A.n;
  if (nnz) *nnz = L.A.nnz;
  if (nc) *nc = L.nc;
  return LIGMG_OK;
}

ligmg_status ligmg_level_matrix(ligmg_handle h, int32_t level, int64_t *rowptr, int32_t *col,
                                double *val) {
  if (!h || level < 0 || level >= (int)h->h.size() || !rowptr || !col || !val)
    return LIGMG_ERR_INVALID_ARGUMENT;
  return guard([&]() -> ligmg_status {
    LG_CUDA(cudaSetDevice(h->device));
    const Level &L = *h->h[level];
    L.A.rp.download(rowptr, L.A.n + 1);
    L.A.ci.download(col, L.A.nnz);
    L.A.v.download(val, L.A.nnz);
    LG_CUDA(cudaStreamSynchronize(h->s));
    return LIGMG_OK;
  });
}

ligmg_status ligmg_level_ids(ligmg_handle h, int32_t level, int32_t *ids) {
  if (!h || level < 0 || level >= (int)h->h.size() || !ids) return LIGMG_ERR_INVALID_ARGUMENT;
  return guard([&]() -> ligmg_status {
    LG_CUDA(cudaSetDevice(h->device));
    const Level &L = *h->h[level];
    if (L.type == LIGMG_LEVEL_ELIM) L.elim.new_id.download(ids, L.A.n);
    else if (L.type == LIGMG_LEVEL_AGG) L.agg.agg.download(ids, L.A.n);
    else return LIGMG_ERR_INVALID_ARGUMENT;
    LG_CUDA(cudaStreamSynchronize(h->s));
    return LIGMG_OK;
  });
}

ligmg_status ligmg_setup_times(ligmg_handle h, double *seconds) {
  if (!h || !seconds) return LIGMG_ERR_INVALID_ARGUMENT;
  for (int i = 0; i < LIGMG_SETUP_NPHASES; i++) seconds[i] = h->setup_phase[i];
  return LIGMG_OK;
}

ligmg_status ligmg_level_lmax(ligmg_handle h, int32_t level, double *lmax) {
  if (!h || level < 0 || level >= (int)h->h.size() || !lmax) return LIGMG_ERR_INVALID_ARGUMENT;
  *lmax = h->h[level]->lmax;
  return LIGMG_OK;
}

ligmg_status ligmg_cycle(ligmg_handle h, int32_t level, const double *b, double *x) {
  if (!h || level < 0 || level >= (int)h->h.size() || !b || !x) return LIGMG_ERR_INVALID_ARGUMENT;
  return guard([&]() -> ligmg_status {
    LG_CUDA(cudaSetDevice(h->device));
    if (h->opts.precision == LIGMG_PREC_FP32) ensure_fp32(*h);
    i64 n = h->h[level]->A.n;
    DBuf<double> db(n, h->s), dx(n, h->s);
    db.upload(b, n);
    if (h->opts.precision == LIGMG_PREC_FP32) {
      Work<float> &W = work_for<float>(*h, 1);
      Engine<float> E(*h, W);
      LevelWork<float> &w = W.lw[level];
      convert<double, float>(n, db.p, w.in.p, h->s);
      E.cycle(level, w.in.p, w.out.p);
      convert<float, double>(n, w.out.p, dx.p, h->s);
    } else {
      Work<double> &W = work_for<double>(*h, 1);
      Engine<double> E(*h, W);
      E.cycle(level, db.p, dx.p);
    }
    dx.download(x, n);
    LG_CUDA(cudaStreamSynchronize(h->s));
    check_tails(*h);
    return LIGMG_OK;
  });
}

ligmg_status ligmg_spmv(ligmg_handle h, int32_t level, const double *x, double *y) {
  if (!h || level < 0 || level >= (int)h->h.size() || !x || !y) return LIGMG_ERR_INVALID_ARGUMENT;
  return guard([&]() -> ligmg_status {
    LG_CUDA(cudaSetDevice(h->device));
    const Level &L = *h->h[level];
    i64 n = L.A.n;
    DBuf<double> dx(n, h->s), dy(n, h->s);
    dx.upload(x, n);
    EpiArgs a;
    a.y = dy.p;
    spmm<double>(viewA<double>(L, 1, h->s), dx.p, 1, Epi::Store, a, h->s);
    dy.download(y, n);
    LG_CUDA(cudaStreamSynchronize(h->s));
    return LIGMG_OK;
  });
}

ligmg_status ligmg_set_stream(ligmg_handle h, void *stream) {
  if (!h || !stream) return LIGMG_ERR_INVALID_ARGUMENT;
  return guard([&]() -> ligmg_status {
    LG_CUDA(cudaSetDevice(h->device));
    LG_CUDA(cudaStreamSynchronize(h->s));
    if (h->own_stream) {
      // buffers were allocated stream-ordered on the old stream; keep it alive
      h->old_streams.push_back(h->s);
      h->own_stream = false;
    }
    h->s = (cudaStream_t)stream;
    return LIGMG_OK;
  });
}

ligmg_status ligmg_get_stream(ligmg_handle h, void **stream) {
  if (!h || !stream) return LIGMG_ERR_INVALID_ARGUMENT;
  *stream = (void *)h->s;
  return LIGMG_OK;
}

const char *ligmg_last_error(void) { return g_last_error.c_str(); }

ligmg_status ligmg_measure_gather_peak(int64_t rows, int32_t width, int64_t count,
                                       int32_t blocks_per_sm, double *rows_per_s) {
  if (!rows_per_s || rows <= 0 || rows > (int64_t)INT32_MAX || count <= 0 ||
      count > ((int64_t)1 << 31) || blocks_per_sm < 0 || blocks_per_sm > 8 ||
      (width != 4 && width != 8 && width != 128))
    return LIGMG_ERR_INVALID_ARGUMENT;
  return guard([&]() -> ligmg_status {
    *rows_per_s = gather_peak(rows, width, count, blocks_per_sm);
    return LIGMG_OK;
  });
}

ligmg_status ligmg_launch_count(int64_t *count) {
  if (!count) return LIGMG_ERR_INVALID_ARGUMENT;
  *count = __atomic_load_n(&lg::g_launches, __ATOMIC_RELAXED);
  return LIGMG_OK;
}

ligmg_status ligmg_profile_enable(ligmg_handle h, int32_t enable) {
  if (!h) return LIGMG_ERR_INVALID_ARGUMENT;
  return guard([&]() -> ligmg_status {
    LG_CUDA(cudaSetDevice(h->device));
    h->prof.collect();
    h->prof.on = enable != 0;
    if (enable) h->prof.stats.clear();
    return LIGMG_OK;
  });
}

ligmg_status ligmg_kernel_stats(ligmg_handle h, ligmg_kernel_stat *out, int32_t cap,
                                int32_t *count) {
  if (!h || !count || (cap > 0 && !out)) return LIGMG_ERR_INVALID_ARGUMENT;
  return guard([&]() -> ligmg_status {
    LG_CUDA(cudaSetDevice(h->device));
    h->prof.collect();
    std::vector<ligmg_kernel_stat> v;
    for (auto &kv : h->prof.stats) v.push_back(kv.second);
    std::sort(v.begin(), v.end(), [](const ligmg_kernel_stat &a, const ligmg_kernel_stat &b) {
      return a.seconds > b.seconds;
    });
    *count = (int32_t)v.size();
    for (int i = 0; i < cap && i < (int)v.size(); i++) out[i] = v[i];
    return LIGMG_OK;
  });
}

}  // extern "C"

// ---------------------------------------------------------------------------
// ligmg_spmv_device_noalloc: the level SpMV without any allocation.  Its only
// scratch (split hub-row partial sums and their completion counters) lives in
// this fixed device array instead of buffers owned by the handle.
namespace {
constexpr i64 kNoallocMaxChunks = 262144;
constexpr i64 kNoallocMaxHubs = 131072;
constexpr size_t kNoallocCounterOffset = sizeof(double) * kNoallocMaxChunks;
static __device__ __align__(256) unsigned char
    g_spmv_scratch[sizeof(double) * kNoallocMaxChunks + sizeof(int) * kNoallocMaxHubs];

// device address of g_spmv_scratch, looked up once per device with that
// device current (the host-side symbol is only a stand-in)
std::mutex g_noalloc_mu;
void *g_noalloc_addr[128] = {nullptr};

void *noalloc_scratch(int device) {
  if (device < 0 || device >= 128) throw Error(LIGMG_ERR_INVALID_ARGUMENT, "device ordinal");
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_addr[device]) {
    void *p = nullptr;
    LG_CUDA(cudaGetSymbolAddress(&p, g_spmv_scratch));
    g_noalloc_addr[device] = p;
  }
  return g_noalloc_addr[device];
}
}  // namespace

extern "C" ligmg_status ligmg_spmv_device_noalloc(ligmg_handle h, int32_t level,
                                                  const double *dx, double *dy) {
  if (!h || !dx || !dy || level < 0 || level >= (int)h->h.size())
    return LIGMG_ERR_INVALID_ARGUMENT;
  return guard([&]() -> ligmg_status {
    LG_CUDA(cudaSetDevice(h->device));
    const Level &L = *h->h[level];
    if (L.hubA64.nchunks > kNoallocMaxChunks || L.hubA64.nhubs > kNoallocMaxHubs)
      throw Error(LIGMG_ERR_UNSUPPORTED,
                  "level has more split hub rows than the no-allocation scratch holds");
    unsigned char *base = (unsigned char *)noalloc_scratch(h->device);
    MatView<double> A = viewA<double>(L, 1, h->s);
    A.partial = (double *)base;
    A.hub_counter = (int *)(base + kNoallocCounterOffset);
    // the split-row kernel resets each counter when a row completes; zeroing
    // them here only guards against a previous call that stopped part-way
    if (L.hubA64.nhubs > 0)
      LG_CUDA(cudaMemsetAsync(A.hub_counter, 0, sizeof(int) * L.hubA64.nhubs, h->s));
    EpiArgs a;
    a.y = dy;
    spmm<double>(A, dx, 1, Epi::Store, a, h->s);
    return LIGMG_OK;
  });
}
