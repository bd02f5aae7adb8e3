// solve.cu — solve-phase kernels for sm_103a.
//
// SpMM layout: X is n x k row-major.  A row is processed by a group of G lanes
// (G = 32 for k > 1).  Inside a group, L = k / VW lanes cover the k columns of
// one matrix entry with 16-byte vector loads (VW = 4 floats or 2 doubles) and
// E = G / L entries are in flight per step; partial sums of the E entry slots
// are combined with warp shuffles and the first L lanes run the fused
// epilogue on their VW columns.  The matrix is read once per k vectors.
#include <algorithm>

#include "spmm_dev.cuh"

namespace lg {

// ---------------------------------------------------------------------------
int split_unit(int value_bytes, int k) {
  int W = value_bytes == 4 ? 4 : 2;
  int VW = (k % W == 0) ? W : 1;
  int L = std::max(1, k / VW);
  return std::max(1, 32 / L);
}

template <typename T>
void HubPlan<T>::build(const i64 *rp_host, i64 n, i64 split_len, int kmax, cudaStream_t s,
                       i64 over) {
  built = true;
  kcap = kmax;
  split = split_len;
  thresh = over > 0 ? over : 2 * split_len;
  i64 thr = thresh;
  std::vector<i64> row, beg, end;
  std::vector<i32> hub, first, cnt;
  nhubs = 0;
  for (i64 r = 0; r < n; r++) {
    i64 len = rp_host[r + 1] - rp_host[r];
    if (len <= thr) continue;
    i64 want = std::min<i64>(std::max<i64>(cdiv(len, split_len), 2), 256);
    i64 chunk = cdiv(len, want);
    i32 nc = (i32)cdiv(len, chunk);
    i32 f = (i32)row.size();
    for (i32 c = 0; c < nc; c++) {
      row.push_back(r);
      beg.push_back(rp_host[r] + c * chunk);
      end.push_back(std::min(rp_host[r + 1], rp_host[r] + (c + 1) * chunk));
      hub.push_back((i32)nhubs);
      first.push_back(f);
      cnt.push_back(nc);
    }
    nhubs++;
  }
  nchunks = (i64)row.size();
  if (nchunks == 0) {
    thresh = 0;
    return;
  }
  auto up64 = [&](DBuf<i64> &d, const std::vector<i64> &h) { d.alloc((i64)h.size(), s); d.upload(h.data(), (i64)h.size()); };
  auto up32 = [&](DBuf<i32> &d, const std::vector<i32> &h) { d.alloc((i64)h.size(), s); d.upload(h.data(), (i64)h.size()); };
  up64(this->row, row);
  up64(this->beg, beg);
  up64(this->end, end);
  up32(this->hub, hub);
  up32(this->first, first);
  up32(this->cnt, cnt);
  counter.alloc(nhubs, s);
  counter.zero();
  partial.alloc(nchunks * kmax, s);
  LG_CUDA(cudaStreamSynchronize(s));
}

template <typename T>
void HubPlan<T>::build_tiles(const i64 *rp_host, i64 n, cudaStream_t s, int kmax) {
  // rows of up to kTilePos - 4 entries always fit a tile (after rounding the
  // start down by at most three); longer ones become hub rows, cut into
  // chunks of about 1024 entries (at least two)
  build(rp_host, n, 1024, kmax, s, kTilePos - 4);
  const i64 nnz = rp_host[n];
  std::vector<int4> desc;
  std::vector<u32> bits;
  bool ok = nnz < ((i64)1 << 33);
  i64 r = 0;
  while (ok && r < n) {
    const i64 len = rp_host[r + 1] - rp_host[r];
    if (len <= 0) {  // empty rows are not supported by the tile layout
      ok = false;
      break;
    }
    if (thresh > 0 && len > thresh) {
      r++;
      continue;
    }
    const i64 r0 = r, ab = rp_host[r0] & ~(i64)3;
    while (r < n && r - r0 < kTileRows) {
      const i64 l = rp_host[r + 1] - rp_host[r];
      if (l <= 0 || (thresh > 0 && l > thresh) || rp_host[r + 1] - ab > kTilePos) break;
      r++;
    }
    if (r == r0) {  // cannot happen for rows of at most thresh entries
      ok = false;
      break;
    }
    desc.push_back(make_int4((int)r0, (int)(r - r0), (int)(rp_host[r] - ab), (int)(ab >> 2)));
    u32 w[kTilePos / 32] = {0};
    for (i64 q = r0; q < r; q++) {
      const i64 rel = rp_host[q] - ab;
      w[rel >> 5] |= 1u << (rel & 31);
    }
    bits.insert(bits.end(), w, w + kTilePos / 32);
  }
  ntiles = ok ? (i64)desc.size() : 0;
  if (ntiles) {
    tdesc.alloc(ntiles, s);
    tdesc.upload(desc.data(), ntiles);
    tbits.alloc((i64)bits.size(), s);
    tbits.upload(bits.data(), (i64)bits.size());
    LG_CUDA(cudaStreamSynchronize(s));
  }
}

std::vector<i32> row_stream_starts(const i64 *rp_host, i64 n, i64 hub_thresh, i64 per_stream) {
  std::vector<i32> st;
  if (n <= 0 || rp_host[n] >= ((i64)1 << 31) - 1 || n >= ((i64)1 << 31) - 1) return st;
  st.push_back(0);
  i64 acc = 0;
  for (i64 r = 0; r < n; r++) {
    const i64 len = rp_host[r + 1] - rp_host[r];
    acc += (hub_thresh > 0 && len > hub_thresh ? 0 : len) + 16;
    if (acc >= per_stream) {
      st.push_back((i32)(r + 1));
      acc = 0;
    }
  }
  if (st.back() != (i32)n) st.push_back((i32)n);
  return st;
}

template <typename T>
void HubPlan<T>::build_stream(const i64 *rp_host, i64 n, i64 per_stream, int blocks,
                              cudaStream_t s) {
  nstream = 0;
  stream_blocks = blocks;
  std::vector<i32> st = row_stream_starts(rp_host, n, thresh, per_stream);
  if (st.size() < 2) return;
  nstream = (i64)st.size() - 1;
  srow.alloc((i64)st.size(), s);
  srow.upload(st.data(), (i64)st.size());
  LG_CUDA(cudaStreamSynchronize(s));
}

template <typename T>
void HubPlan<T>::fill(MatView<T> &m) const {
  m.hub_thresh = thresh;
  m.nchunks = nchunks;
  m.ch_row = row.p;
  m.ch_beg = beg.p;
  m.ch_end = end.p;
  m.ch_hub = hub.p;
  m.ch_first = first.p;
  m.ch_cnt = cnt.p;
  m.hub_counter = counter.p;
  m.partial = partial.p;
  m.tb = tb;
  if (lanes > 0) m.lanes_per_row = lanes;
  m.ntiles = ntiles;
  m.tdesc = tdesc.p;
  m.tbits = tbits.p;
  m.tile_pipe = tile_pipe;
  m.krow_lanes = krow_lanes;
  m.nstream = nstream;
  m.srow = srow.p;
  m.stream_blocks = stream_blocks;
}
template struct HubPlan<float>;
template struct HubPlan<double>;

// ---------------------------------------------------------------------------
namespace {

using namespace dev;

template <typename T, int K, int G, Epi EP>
__global__ void __launch_bounds__(256, 6) k_spmm(const MatView<T> A, const T *__restrict__ X,
                                              const EpiArgs a) {
  dep_prologue();
  const i64 warp = ((i64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  dev::spmm_unit<T, K, G, EP>(A, X, a, warp, threadIdx.x & 31);
}

// ---- single right-hand side, nonzero-balanced tiles -------------------------
// GB300 issues about two FP64 lane operations per SM clock, so a warp-wide
// FP64 instruction holds the SM's FP64 pipe for ~16 clocks whatever its
// active mask; a warp per row spends a five-step shuffle reduction and a
// lane-0 epilogue (a dozen such instructions) on every row.  Here a warp
// takes a tile of whole rows (at most kTilePos entries), a lane kTilePos / 32
// consecutive entries accumulated with one FMA each; rows crossing lanes are
// combined by one segmented scan over the warp (five FP64 adds per tile),
// complete row sums go to shared memory and the epilogue runs one row per
// lane.  Every load of a tile (descriptor aside) is independent of the
// others: one round trip brings the column indices, values and row-start
// bits (16-byte vector loads that do not allocate in L1, so L1 keeps the
// gathered vector), a second one all the gathers of a lane, and the
// epilogue's inputs are prefetched into L1 before the gathers.  Summation
// order: within a lane in entry order, across lanes by the scan's fixed tree.
constexpr int kTileLane = kTilePos / 32;  // entries per lane
constexpr int kTileWarps = 8;             // warps per block
#ifndef LG_TILE_MIN_BLOCKS
#define LG_TILE_MIN_BLOCKS 6  // resident blocks per SM the register budget is set for
#endif

__device__ __forceinline__ int4 ld_stream_i4(const i32 *p) {
  int4 r;
  asm volatile("ld.global.nc.L1::no_allocate.v4.s32 {%0, %1, %2, %3}, [%4];"
               : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
               : "l"(p));
  return r;
}
__device__ __forceinline__ void ld_stream_v(const double *p, double (&o)[2]) {
  asm volatile("ld.global.nc.L1::no_allocate.v2.f64 {%0, %1}, [%2];"
               : "=d"(o[0]), "=d"(o[1])
               : "l"(p));
}
__device__ __forceinline__ void ld_stream_v(const float *p, float (&o)[4]) {
  asm volatile("ld.global.nc.L1::no_allocate.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(o[0]), "=f"(o[1]), "=f"(o[2]), "=f"(o[3])
               : "l"(p));
}
__device__ __forceinline__ void prefetch_l1(const void *p) {
  asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}
// L1 prefetch of the vectors an epilogue reads for row r (1 right-hand side)
template <typename T, Epi EP>
__device__ __forceinline__ void epilogue_prefetch(const EpiArgs &a, i64 r) {
  const T *b = (const T *)a.b, *xin = (const T *)a.xin, *rin = (const T *)a.rin,
          *din = (const T *)a.din, *invd = (const T *)a.invd, *q = (const T *)a.q;
  if constexpr (EP == Epi::Resid || EP == Epi::ElimInterp) prefetch_l1(b + r);
  if constexpr (EP == Epi::ChebA || EP == Epi::Jacobi) {
    prefetch_l1(b + r);
    prefetch_l1(xin + r);
    prefetch_l1(invd + r);
  }
  if constexpr (EP == Epi::ChebB) {
    prefetch_l1(rin + r);
    prefetch_l1(din + r);
    prefetch_l1(xin + r);
    prefetch_l1(invd + r);
  }
  if constexpr (EP == Epi::ChebZ) {
    prefetch_l1(b + r);
    prefetch_l1(invd + r);
  }
  if constexpr (EP == Epi::ElimInterp) prefetch_l1(q + r);
  if constexpr (EP == Epi::FcgDir) {
    prefetch_l1(xin + r);
    prefetch_l1(q + r);
    if (din) {
      prefetch_l1(din + r);
      prefetch_l1(rin + r);
    }
  }
}

// A tile in registers: the descriptor, this lane's row-start bits and column
// indices (fetched one tile ahead by the pipelined kernel), and its values.
template <typename T>
struct TileIdx {
  int4 d;
  u32 word;
  i32 c[kTileLane];
};

// Row-start bits and column indices of tile t (descriptor d), and an L1
// prefetch of the rows its epilogue reads.
template <typename T, Epi EP>
__device__ __forceinline__ void tile_fetch(const MatView<T> &A, const EpiArgs &a, i64 t, int4 d,
                                           int lane, TileIdx<T> &I) {
  constexpr int U = kTileLane;
  static_assert(U == 32 || U == 16 || U == 8 || U == 4, "entries per lane");
  I.d = d;
  const int e_rel = d.z;
  const i64 ab = (i64)d.w << 2;
  const int lb = lane * U;
  const int wbit = lane * U;
  I.word = U == 32 ? __ldg(A.tbits + t * (kTilePos / 32) + lane)
                   : (__ldg(A.tbits + t * (kTilePos / 32) + (wbit >> 5)) >> (wbit & 31)) &
                         ((1u << (U & 31)) - 1u);
#pragma unroll
  for (int g = 0; g < U / 4; g++) {
    const int rel = lb + 4 * g;
    if (rel + 4 <= e_rel) {
      const int4 cc = ld_stream_i4(A.ci + ab + rel);
      I.c[4 * g] = cc.x;
      I.c[4 * g + 1] = cc.y;
      I.c[4 * g + 2] = cc.z;
      I.c[4 * g + 3] = cc.w;
    } else {
#pragma unroll
      for (int q = 0; q < 4; q++) I.c[4 * g + q] = rel + q < e_rel ? __ldg(A.ci + ab + rel + q) : 0;
    }
  }
  for (int i = lane; i < d.y; i += 32) epilogue_prefetch<T, EP>(a, (i64)d.x + i);
}

// This lane's entries of the tile (bit j: entry lane * U + j is in it)
template <typename T>
__device__ __forceinline__ u32 tile_mask(const TileIdx<T> &I, int lane) {
  constexpr int U = kTileLane;
  const int lb = lane * U;
  const int s_rel = __ffs(__shfl_sync(0xffffffffu, I.word, 0)) - 1;  // the tile's first entry
  const int lo = max(s_rel - lb, 0), hi = min(I.d.z - lb, U);
  u32 okm = 0;
  if (hi > lo) okm = (hi >= 32 ? 0xffffffffu : ((1u << hi) - 1u)) & ~((1u << lo) - 1u);
  return okm;
}

// The tile's values and gathered x entries (independent loads)
template <typename T, Epi EP>
__device__ __forceinline__ void tile_gather(const MatView<T> &A, const T *__restrict__ X,
                                            const TileIdx<T> &I, u32 okm, int lane,
                                            T (&v)[kTileLane], T (&xv)[kTileLane]) {
  constexpr bool SPLIT = EP == Epi::Split;
  constexpr int U = kTileLane, VWV = 16 / (int)sizeof(T);
  const int e_rel = I.d.z;
  const i64 ab = (i64)I.d.w << 2;
  const int lb = lane * U;
#pragma unroll
  for (int g = 0; g < U / 4; g++) {
    const int rel = lb + 4 * g;
    if (rel + 4 <= e_rel) {
#pragma unroll
      for (int h = 0; h < 4 / VWV; h++) {
        T tv[VWV];
        ld_stream_v(A.v + ab + rel + h * VWV, tv);
#pragma unroll
        for (int q = 0; q < VWV; q++) v[4 * g + h * VWV + q] = tv[q];
      }
    } else {
#pragma unroll
      for (int q = 0; q < 4; q++) v[4 * g + q] = rel + q < e_rel ? __ldg(A.v + ab + rel + q) : (T)0;
    }
  }
#pragma unroll
  for (int j = 0; j < U; j++)
    xv[j] = ((okm >> j) & 1u) ? __ldg(xsrc<T, 1, SPLIT>(A, X, I.c[j])) : (T)0;
}

// Row sums of the tile (lane sums in entry order, a segmented scan across
// lanes) and the epilogue, one row per lane.
template <typename T, Epi EP>
__device__ __forceinline__ void tile_finish(const EpiArgs &a, const TileIdx<T> &I, u32 okm,
                                            const T (&v)[kTileLane], const T (&xv)[kTileLane],
                                            int lane, T *ssum) {
  constexpr int U = kTileLane;
  const int r0 = I.d.x, nr = I.d.y, e_rel = I.d.z;
  const u32 word = I.word;
  // rows started before this lane: exclusive scan of the row-start counts
  const int cnt = __popc(word);
  int inc = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += u;
  }
  const int pre = inc - cnt;
  int ri = pre - 1;  // the row open at the lane's first entry
  bool cont = true, brk = false;
  T acc = (T)0, hs = (T)0;
#pragma unroll
  for (int j = 0; j < U; j++) {
    const T vj = ((okm >> j) & 1u) ? v[j] : (T)0;
    if ((word >> j) & 1u) {  // a row starts: close the open one
      if (cont) hs = acc;
      else ssum[ri] = acc;
      cont = false;
      brk = true;
      ri++;
      acc = (T)0;
    }
    acc = fma(vj, xv[j], acc);
  }
  // inclusive scan of the lanes' open sums, restarted at every lane where a
  // row starts: S = the lane's last row summed up to the lane's end
  T S = acc;
  int f = brk;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T su = __shfl_up_sync(0xffffffffu, S, o);
    const int fu = __shfl_up_sync(0xffffffffu, f, o);
    if (lane >= o) {
      if (!f) S += su;
      f |= fu;
    }
  }
  const T sprev = __shfl_up_sync(0xffffffffu, S, 1);
  if (lane > 0 && brk) ssum[pre - 1] = sprev + hs;  // the row open at this lane's start ends here
  if (lane == (e_rel - 1) / U) ssum[nr - 1] = S;     // the tile's last row
  __syncwarp();
  for (int i = lane; i < nr; i += 32) {
    T r1[1] = {ssum[i]};
    epilogue<T, 1, 1, EP>(a, (i64)r0 + i, 0, r1);
  }
  __syncwarp();
}

template <typename T, Epi EP>
__device__ __forceinline__ void tile_unit(const MatView<T> &A, const T *__restrict__ X,
                                          const EpiArgs &a, i64 t, int lane, T *ssum) {
  TileIdx<T> I;
  tile_fetch<T, EP>(A, a, t, __ldg(A.tdesc + t), lane, I);
  const u32 okm = tile_mask(I, lane);
  T v[kTileLane], xv[kTileLane];
  tile_gather<T, EP>(A, X, I, okm, lane, v, xv);
  tile_finish<T, EP>(a, I, okm, v, xv, lane, ssum);
}

template <typename T, Epi EP>
__global__ void __launch_bounds__(kTileWarps * 32, LG_TILE_MIN_BLOCKS)
    k_spmv_tile(const MatView<T> A, const T *__restrict__ X, const EpiArgs a) {
  dep_prologue();
  __shared__ T ssum[kTileWarps][kTileRows];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const i64 warp = (i64)blockIdx.x * kTileWarps + w;
  if (warp < A.ntiles) tile_unit<T, EP>(A, X, a, warp, lane, ssum[w]);
  else dev::hub_unit<T, 1, EP>(A, X, a, warp - A.ntiles, lane);
}

// Pipelined tiles: a resident grid whose warp w takes tiles w, w + W, w + 2W,
// ... (W warps in the grid).  The one-warp-per-tile kernel waits for three
// dependent round trips per tile (descriptor, column indices, gathers) of
// which one gathers; here the lanes fetch the warp's next 32 descriptors with
// one load, and the next tile's row-start bits and column indices are loaded
// while this tile's gathers are in flight, so a tile costs about one round
// trip.  Values are loaded with the gathers.  Same per-tile arithmetic, same
// results.  Hub chunks follow, strided the same way.
#ifndef LG_TILEP_MIN_BLOCKS
#define LG_TILEP_MIN_BLOCKS 3  // 80 registers
#endif
__device__ __forceinline__ int4 shfl_int4(int4 v, int src) {
  int4 r;
  r.x = __shfl_sync(0xffffffffu, v.x, src);
  r.y = __shfl_sync(0xffffffffu, v.y, src);
  r.z = __shfl_sync(0xffffffffu, v.z, src);
  r.w = __shfl_sync(0xffffffffu, v.w, src);
  return r;
}

template <typename T, Epi EP>
__global__ void __launch_bounds__(kTileWarps * 32, LG_TILEP_MIN_BLOCKS)
    k_spmv_tile_pipe(const MatView<T> A, const T *__restrict__ X, const EpiArgs a) {
  dep_prologue();
  __shared__ T ssum[kTileWarps][kTileRows];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // tile counts fit 32 bits (the pipelined launch is used below 2^31 tiles)
  const int gw = (int)blockIdx.x * kTileWarps + w;
  const int nw = (int)gridDim.x * kTileWarps;
  const int nt = (int)A.ntiles;
  const int mine = gw < nt ? (nt - 1 - gw) / nw + 1 : 0;  // this warp's tiles
  if (mine > 0) {
    // lane l: descriptor of the warp's tile (batch + l)
    int4 dl = lane < mine ? __ldg(A.tdesc + gw + (i64)lane * nw) : make_int4(0, 0, 0, 0);
    TileIdx<T> cur;
    tile_fetch<T, EP>(A, a, gw, shfl_int4(dl, 0), lane, cur);
    for (int i = 0; i < mine; i++) {
      const u32 okm = tile_mask(cur, lane);
      T v[kTileLane], xv[kTileLane];
      tile_gather<T, EP>(A, X, cur, okm, lane, v, xv);
      TileIdx<T> nxt;
      const int in = i + 1;
      if (in < mine) {
        if ((in & 31) == 0) {
          const int q = in + lane;
          dl = q < mine ? __ldg(A.tdesc + gw + (i64)q * nw) : make_int4(0, 0, 0, 0);
        }
        tile_fetch<T, EP>(A, a, gw + (i64)in * nw, shfl_int4(dl, in & 31), lane, nxt);
      }
      tile_finish<T, EP>(a, cur, okm, v, xv, lane, ssum[w]);
      if (in < mine) cur = nxt;
    }
  }
  for (i64 c = gw; c < A.nchunks; c += nw) dev::hub_unit<T, 1, EP>(A, X, a, c, lane);
}

// ---- k right-hand sides, row streams ---------------------------------------
// The warp-per-row kernel pays, on every row, dependent round trips that
// gather nothing: the row bounds, the first column indices and the
// epilogue's input rows (about a third of a row's time on the large R-MAT
// levels, whose rows take five or six gather steps).  Here warp w takes the
// consecutive rows [srow[w], srow[w + 1]) (balanced by entries at plan time):
// the next row's end is loaded while this row gathers, the last step of a
// row fetches the next row's first column indices, and the epilogue's input
// rows are prefetched into L1 in that step, one round trip before they are
// read.  Steps are warp-uniform, U entries per slot, masked past the row's
// end; every slot adds its entries in entry order, as the row kernel does,
// so the results are the same bits.

// L1 prefetch of the k-column rows (and per-row scalars) an epilogue reads
template <typename T, int K, Epi EP>
__device__ __forceinline__ void epilogue_prefetch_rows(const EpiArgs &a, i64 r, int lane) {
  constexpr int RB = K * (int)sizeof(T);  // bytes of a vector's row
  constexpr int LINES = (RB + 127) / 128;
  const void *v0 = nullptr, *v1 = nullptr, *v2 = nullptr, *sc = nullptr;
  if constexpr (EP == Epi::Resid || EP == Epi::ElimInterp) v0 = a.b;
  if constexpr (EP == Epi::ChebZ) {
    v0 = a.b;
    sc = a.invd;
  }
  if constexpr (EP == Epi::ChebA || EP == Epi::Jacobi) {
    v0 = a.b;
    v1 = a.xin;
    sc = a.invd;
  }
  if constexpr (EP == Epi::ChebB) {
    v0 = a.rin;
    v1 = a.din;
    v2 = a.xin;
    sc = a.invd;
  }
  if constexpr (EP == Epi::FcgDir) {
    v0 = a.xin;
    v1 = a.din;
    v2 = a.rin;
  }
  if constexpr (EP == Epi::ElimInterp || EP == Epi::FcgDir) sc = a.q;
  const int v = lane / LINES, l = lane % LINES;
  const void *p = v == 0 ? v0 : v == 1 ? v1 : v == 2 ? v2 : nullptr;
  if (p) prefetch_l1((const char *)p + r * RB + l * 128);
  if (lane == 31 && sc) prefetch_l1((const T *)sc + r);
}

template <typename T, int K, Epi EP, int U>
__device__ __forceinline__ void stream_unit(const MatView<T> &A, const T *__restrict__ X,
                                            const EpiArgs &a, i64 w, int lane) {
  constexpr bool SPLIT = EP == Epi::Split;
  constexpr int VW = (K % VT<T>::W == 0) ? VT<T>::W : 1;
  constexpr int L = K / VW;
  constexpr int E = 32 / L;
  constexpr int STEP = U * E;
  const int slot = lane / L, ch = lane % L;
  const T *__restrict__ av = A.v;
  const i32 *__restrict__ ac = A.ci;
  const i64 *__restrict__ rp = A.rp;
  const int hub = (int)A.hub_thresh;  // 0: no hub rows
  int r = __ldg(A.srow + w);
  const int r1 = __ldg(A.srow + w + 1);
  int b = (int)__ldg(rp + r), e = (int)__ldg(rp + r + 1);
  int ee = (hub > 0 && e - b > hub) ? b : e;  // a hub row's entries belong to its chunks
  i32 jn[U];
#pragma unroll
  for (int u = 0; u < U; u++) {
    const int q = b + slot + u * E;
    jn[u] = q < ee ? __ldg(ac + q) : -1;
  }
  while (true) {
    const bool last = r + 1 >= r1;
    const int en = last ? e : (int)__ldg(rp + r + 2);
    T acc[VW];
#pragma unroll
    for (int q = 0; q < VW; q++) acc[q] = (T)0;
    int kb = b;
    while (true) {
      i32 j[U];
#pragma unroll
      for (int u = 0; u < U; u++) j[u] = jn[u];
      const int kn = kb + STEP;
      const bool more = kn < ee;
      if (more) {
#pragma unroll
        for (int u = 0; u < U; u++) {
          const int q = kn + slot + u * E;
          jn[u] = q < ee ? __ldg(ac + q) : -1;
        }
      } else {  // the next row's first step, and this row's epilogue inputs
        const int nee = (last || (hub > 0 && en - e > hub)) ? e : en;
#pragma unroll
        for (int u = 0; u < U; u++) {
          const int q = e + slot + u * E;
          jn[u] = q < nee ? __ldg(ac + q) : -1;
        }
        if (ee > b || e == b) epilogue_prefetch_rows<T, K, EP>(a, r, lane);
      }
      T va[U], x[U][VW];
#pragma unroll
      for (int u = 0; u < U; u++) {
        if (j[u] >= 0) {
          va[u] = __ldg(av + kb + slot + u * E);
          xload<T, VW, true>(xsrc<T, K, SPLIT>(A, X, j[u]) + ch * VW, x[u]);
        } else {
          va[u] = (T)0;
#pragma unroll
          for (int q = 0; q < VW; q++) x[u][q] = (T)0;
        }
      }
#pragma unroll
      for (int u = 0; u < U; u++)
#pragma unroll
        for (int q = 0; q < VW; q++) acc[q] += va[u] * x[u][q];
      if (!more) break;
      kb = kn;
    }
    reduce_slots<T, VW, L, 32>(acc);
    if ((ee > b || e == b) && slot == 0) epilogue<T, K, VW, EP>(a, r, ch * VW, acc);
    if (last) break;
    r++;
    b = e;
    e = en;
    ee = (hub > 0 && e - b > hub) ? b : e;
  }
}

template <typename T, int K, Epi EP, int MINB>
__global__ void __launch_bounds__(256, MINB)
    k_spmm_rs(const MatView<T> A, const T *__restrict__ X, const EpiArgs a) {
  dep_prologue();
  const i64 warp = ((i64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp < A.nstream) stream_unit<T, K, EP, 4>(A, X, a, warp, lane);
  else dev::hub_unit<T, K, EP>(A, X, a, warp - A.nstream, lane);
}

// stream_blocks: the resident 256-thread blocks per SM the register budget is
// set for (5: 48 registers; 6: 40)
template <typename T, int K, Epi EP>
void launch_spmm_rs(const MatView<T> &A, const T *X, const EpiArgs &a, cudaStream_t s) {
  const i64 warps = A.nstream + A.nchunks;
  if (A.stream_blocks == 6)
    launch_dep(k_spmm_rs<T, K, EP, 6>, grid_for(warps * 32, 256), 256, 0, s, A, X, a);
  else
    launch_dep(k_spmm_rs<T, K, EP, 5>, grid_for(warps * 32, 256), 256, 0, s, A, X, a);
  LG_LAUNCH();
}

// ---- k right-hand sides, tiles of whole rows --------------------------------
// On levels with short rows a warp per row (or per run of rows) spends most
// 16-entry steps partly masked: a 33-entry row takes three.  Here a warp
// takes a tile of whole rows (the single right-hand side layout: at most
// kTilePos entries from a 4-aligned start, row-start bitmap) and walks its
// entries in steps of U E consecutive entries whatever the rows: slot s (L
// lanes, VW columns each) takes U contiguous entries, adds them in order,
// closes the rows that start and end inside them into shared memory, and a
// segmented scan across the slots (restarted at a slot holding a row start)
// completes the rows that cross slots; the row still open at a step's end is
// carried into the next step's first slot.  The next step's column indices
// and values are loaded during this step's gathers.  Summation order is
// fixed (entry order in a slot, the scan's tree across slots, step order).
constexpr int kKTileWarps = 8;
// row sums of a warp's tile live in static shared memory: rows of at most 128
// bytes (FP32 k <= 32, FP64 k <= 16)
template <typename T, int K>
constexpr bool ktile_fits() {
  return K >= 2 && K * (int)sizeof(T) <= 128;
}

template <typename T, int K, Epi EP>
__device__ __forceinline__ void ktile_load(const MatView<T> &A, i64 ab, int p0, int e_rel,
                                           i32 (&c)[4], T (&v)[4]) {
  constexpr int VWV = 16 / (int)sizeof(T);
  if (p0 + 4 <= e_rel) {
    const int4 cc = ld_stream_i4(A.ci + ab + p0);
    c[0] = cc.x;
    c[1] = cc.y;
    c[2] = cc.z;
    c[3] = cc.w;
#pragma unroll
    for (int h = 0; h < 4 / VWV; h++) {
      T tv[VWV];
      ld_stream_v(A.v + ab + p0 + h * VWV, tv);
#pragma unroll
      for (int q = 0; q < VWV; q++) v[h * VWV + q] = tv[q];
    }
  } else {
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const bool in = p0 + u < e_rel;
      c[u] = in ? __ldg(A.ci + ab + p0 + u) : 0;
      v[u] = in ? __ldg(A.v + ab + p0 + u) : (T)0;
    }
  }
}

template <typename T, int K, Epi EP>
__device__ __forceinline__ void ktile_unit(const MatView<T> &A, const T *__restrict__ X,
                                           const EpiArgs &a, i64 t, int lane, T *ssum) {
  constexpr bool SPLIT = EP == Epi::Split;
  constexpr int VW = (K % VT<T>::W == 0) ? VT<T>::W : 1;
  constexpr int L = K / VW;  // lanes per entry
  constexpr int E = 32 / L;  // slots
  constexpr int U = 4;       // contiguous entries per slot and step
  constexpr int STEP = U * E;
  constexpr int NW = kTilePos / 32;  // bitmap words
  static_assert(NW <= 32 && STEP % 4 == 0, "tile layout");
  const int slot = lane / L, ch = lane % L;
  const int4 d = __ldg(A.tdesc + t);
  const int r0 = d.x, nr = d.y, e_rel = d.z;
  const i64 ab = (i64)d.w << 2;
  // lane w < NW: bitmap word w and the row starts in the words before it
  const u32 wl = lane < NW ? __ldg(A.tbits + t * NW + lane) : 0u;
  int pw = __popc(wl);
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, pw, o);
    if (lane >= o) pw += y;
  }
  pw -= __popc(wl);  // exclusive
  const int nsteps = (e_rel + STEP - 1) / STEP;
  for (int i = 0; i < nr; i++) epilogue_prefetch_rows<T, K, EP>(a, (i64)r0 + i, lane);
  T carry[VW];
#pragma unroll
  for (int q = 0; q < VW; q++) carry[q] = (T)0;
  i32 cn[4];
  T vn[4];
  ktile_load<T, K, EP>(A, ab, slot * U, e_rel, cn, vn);
  for (int j = 0; j < nsteps; j++) {
    const int p0 = j * STEP + slot * U;  // this slot's first entry (from ab)
    i32 c[4];
    T va[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      c[u] = cn[u];
      va[u] = vn[u];
    }
    if (j + 1 < nsteps) ktile_load<T, K, EP>(A, ab, p0 + STEP, e_rel, cn, vn);
    // this slot's entries of the tile: [s_rel, e_rel) (s_rel < 4: the first
    // row start, in word 0)
    const u32 w0 = __shfl_sync(0xffffffffu, wl, 0);
    const int s_rel = __ffs(w0) - 1;
    T x[4][VW];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const bool ok = p0 + u >= s_rel && p0 + u < e_rel;
      if (ok) {
        xload<T, VW, true>(xsrc<T, K, SPLIT>(A, X, c[u]) + ch * VW, x[u]);
      } else {
        va[u] = (T)0;
#pragma unroll
        for (int q = 0; q < VW; q++) x[u][q] = (T)0;
      }
    }
    const int wi = p0 >> 5;
    const u32 wd = __shfl_sync(0xffffffffu, wl, wi < NW ? wi : 0);
    const u32 b4 = wi < NW ? (wd >> (p0 & 31)) & 0xFu : 0u;
    const int pre = __shfl_sync(0xffffffffu, pw, wi < NW ? wi : 0) +
                    (wi < NW ? __popc(wd & ((1u << (p0 & 31)) - 1u)) : 0);
    T run[VW], hs[VW];
#pragma unroll
    for (int q = 0; q < VW; q++) {
      run[q] = slot == 0 ? carry[q] : (T)0;
      hs[q] = (T)0;
    }
    bool cont = true, brk = false;
    int ri = pre - 1;  // the row open at this slot's first entry
#pragma unroll
    for (int u = 0; u < 4; u++) {
      if ((b4 >> u) & 1u) {  // a row starts: close the open one
        if (cont) {
#pragma unroll
          for (int q = 0; q < VW; q++) hs[q] = run[q];
        } else {
#pragma unroll
          for (int q = 0; q < VW; q++) ssum[ri * K + ch * VW + q] = run[q];
        }
        cont = false;
        brk = true;
        ri++;
#pragma unroll
        for (int q = 0; q < VW; q++) run[q] = (T)0;
      }
#pragma unroll
      for (int q = 0; q < VW; q++) run[q] += va[u] * x[u][q];
    }
    // inclusive scan of the slots' open sums, restarted at a slot with a row start
    T S[VW];
#pragma unroll
    for (int q = 0; q < VW; q++) S[q] = run[q];
    int f = brk;
#pragma unroll
    for (int o = 1; o < E; o <<= 1) {
      T su[VW];
#pragma unroll
      for (int q = 0; q < VW; q++) su[q] = __shfl_up_sync(0xffffffffu, S[q], o * L);
      const int fu = __shfl_up_sync(0xffffffffu, f, o * L);
      if (slot >= o) {
        if (!f)
#pragma unroll
          for (int q = 0; q < VW; q++) S[q] += su[q];
        f |= fu;
      }
    }
    T sp[VW];
#pragma unroll
    for (int q = 0; q < VW; q++) sp[q] = __shfl_up_sync(0xffffffffu, S[q], L);
    // the row open at this slot's start ends inside it: previous slots' open
    // sum (the carry is in slot 0's own head) plus this slot's head
    if (brk && pre > 0)
#pragma unroll
      for (int q = 0; q < VW; q++) ssum[(pre - 1) * K + ch * VW + q] = (slot > 0 ? sp[q] : (T)0) + hs[q];
#pragma unroll
    for (int q = 0; q < VW; q++) carry[q] = __shfl_sync(0xffffffffu, S[q], (E - 1) * L + ch);
  }
  if (slot == 0)  // the tile's last row ends with the tile
#pragma unroll
    for (int q = 0; q < VW; q++) ssum[(nr - 1) * K + ch * VW + q] = carry[q];
  __syncwarp();
  for (int i = slot; i < nr; i += E) {
    T acc[VW];
#pragma unroll
    for (int q = 0; q < VW; q++) acc[q] = ssum[i * K + ch * VW + q];
    epilogue<T, K, VW, EP>(a, (i64)r0 + i, ch * VW, acc);
  }
  __syncwarp();
}

template <typename T, int K, Epi EP>
__global__ void __launch_bounds__(kKTileWarps * 32, 4)
    k_spmm_ktile(const MatView<T> A, const T *__restrict__ X, const EpiArgs a) {
  dep_prologue();
  __shared__ T ssum[kKTileWarps][kTileRows * K];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const i64 warp = (i64)blockIdx.x * kKTileWarps + w;
  if (warp < A.ntiles) ktile_unit<T, K, EP>(A, X, a, warp, lane, ssum[w]);
  else dev::hub_unit<T, K, EP>(A, X, a, warp - A.ntiles, lane);
}

template <typename T, int K, int G, Epi EP>
void launch_spmm(const MatView<T> &A, const T *X, const EpiArgs &a, cudaStream_t s) {
  constexpr int RPW = 32 / G;
  i64 warps = cdiv(A.n, RPW) + ((G == 32) ? A.nchunks : 0);
  if (warps == 0) return;
  const int tb = (A.tb == 64 || A.tb == 128) ? A.tb : 256;
  launch_dep(k_spmm<T, K, G, EP>, grid_for(warps * 32, tb), tb, 0, s, A, X, a);
  LG_LAUNCH();
}

template <typename T, int K, Epi EP>
void dispatch_g(const MatView<T> &A, const T *X, const EpiArgs &a, cudaStream_t s) {
  if constexpr (K == 1) {
    // the tile layout reads 16-byte aligned column and value arrays
    if (A.ntiles > 0 && (((uintptr_t)A.ci | (uintptr_t)A.v) & 15) == 0) {
      if (A.tile_pipe && A.ntiles < ((i64)1 << 31) - ((i64)kSMs << 8)) {
        static int per_sm = 0;  // resident blocks of this instantiation
        if (per_sm == 0)
          LG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_spmv_tile_pipe<T, EP>,
                                                                kTileWarps * 32, 0));
        const i64 g = std::min<i64>((i64)std::max(per_sm, 1) * kSMs,
                                    cdiv(A.ntiles + A.nchunks, kTileWarps));
        launch_dep(k_spmv_tile_pipe<T, EP>, (unsigned)g, kTileWarps * 32, 0, s, A, X, a);
      } else {
        launch_dep(k_spmv_tile<T, EP>, grid_for(A.ntiles + A.nchunks, kTileWarps), kTileWarps * 32, 0, s, 
            A, X, a);
      }
      LG_LAUNCH();
      return;
    }
    int g = A.nchunks > 0 ? 32 : A.lanes_per_row;
    switch (g) {
      case 4: return launch_spmm<T, 1, 4, EP>(A, X, a, s);
      case 8: return launch_spmm<T, 1, 8, EP>(A, X, a, s);
      case 16: return launch_spmm<T, 1, 16, EP>(A, X, a, s);
      default: return launch_spmm<T, 1, 32, EP>(A, X, a, s);
    }
  } else {
    if constexpr (ktile_fits<T, K>()) {
      if (A.ntiles > 0 && (((uintptr_t)A.ci | (uintptr_t)A.v) & 15) == 0) {
        launch_dep(k_spmm_ktile<T, K, EP>, grid_for(A.ntiles + A.nchunks, kKTileWarps),
                   kKTileWarps * 32, 0, s, A, X, a);
        LG_LAUNCH();
        return;
      }
    }
    if constexpr (K >= 8) {
      if (A.nstream > 0) return launch_spmm_rs<T, K, EP>(A, X, a, s);
      // short rows: two rows per warp, half the lanes each (no hub chunks)
      if constexpr (K <= 32)
        if (A.krow_lanes == 16 && A.nchunks == 0) return launch_spmm<T, K, 16, EP>(A, X, a, s);
    }
    launch_spmm<T, K, 32, EP>(A, X, a, s);
  }
}

template <typename T, Epi EP>
void dispatch_k(const MatView<T> &A, const T *X, int k, const EpiArgs &a, cudaStream_t s) {
  switch (k) {
    case 1: return dispatch_g<T, 1, EP>(A, X, a, s);
    case 2: return dispatch_g<T, 2, EP>(A, X, a, s);
    case 4: return dispatch_g<T, 4, EP>(A, X, a, s);
    case 8: return dispatch_g<T, 8, EP>(A, X, a, s);
    case 16: return dispatch_g<T, 16, EP>(A, X, a, s);
    case 32: return dispatch_g<T, 32, EP>(A, X, a, s);
    case 64: return dispatch_g<T, 64, EP>(A, X, a, s);
    default: throw Error(LIGMG_ERR_UNSUPPORTED, "k must be 1,2,4,8,16,32,64");
  }
}

}  // namespace

template <typename T>
void spmm(const MatView<T> &A, const T *X, int k, Epi epi, const EpiArgs &args, cudaStream_t s) {
  EpiArgs a = args;
  a.mirror();
  switch (epi) {
    case Epi::Store: return dispatch_k<T, Epi::Store>(A, X, k, a, s);
    case Epi::Resid: return dispatch_k<T, Epi::Resid>(A, X, k, a, s);
    case Epi::ChebA: return dispatch_k<T, Epi::ChebA>(A, X, k, a, s);
    case Epi::ChebB: return dispatch_k<T, Epi::ChebB>(A, X, k, a, s);
    case Epi::ElimInterp: return dispatch_k<T, Epi::ElimInterp>(A, X, k, a, s);
    case Epi::Jacobi: return dispatch_k<T, Epi::Jacobi>(A, X, k, a, s);
    case Epi::Split: return dispatch_k<T, Epi::Split>(A, X, k, a, s);
    case Epi::ChebZ: return dispatch_k<T, Epi::ChebZ>(A, X, k, a, s);
    case Epi::FcgDir: return dispatch_k<T, Epi::FcgDir>(A, X, k, a, s);
  }
}
template void spmm<float>(const MatView<float> &, const float *, int, Epi, const EpiArgs &,
                          cudaStream_t);
template void spmm<double>(const MatView<double> &, const double *, int, Epi, const EpiArgs &,
                           cudaStream_t);

// ---------------------------------------------------------------------------
namespace {

template <typename T>
__global__ void k_cheb_init_zero(i64 n, int k, const T *b, const T *invd, T scale, T *d) {
  dep_prologue();
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n * k) d[t] = (invd[t / k] * scale) * b[t];
}

template <typename T>
__global__ void k_fill(i64 cnt, T *x, T v) {
  dep_prologue();
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < cnt) x[t] = v;
}

template <typename T>
__global__ void k_prolong_agg(i64 n, int k, const i32 *agg, const T *xc, T *x) {
  dep_prologue();
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * k) return;
  i64 i = t / k;
  x[t] += xc[(i64)agg[i] * k + (t % k)];
}

template <typename T>
__global__ void k_coarse_apply(i64 n, int k, const T *pinv, const T *b, T *x) {
  dep_prologue();
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * k) return;
  i64 i = t / k;
  int c = (int)(t % k);
  T s = 0;
  for (i64 j = 0; j < n; j++) s += pinv[i * n + j] * b[j * k + c];
  x[t] = s;
}

template <typename T>
__global__ void k_scale(i64 nk, T *x, T f) {
  dep_prologue();
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nk) x[t] = x[t] * f;
}

template <typename S, typename D>
__global__ void k_convert(i64 cnt, const S *src, D *dst) {
  dep_prologue();
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < cnt) dst[t] = (D)src[t];
}

// column reductions.  Thread t of a BS-thread block takes column t % k and
// rows t / k, t / k + BS / k, ... (four rows per pass, loads issued first).
// Inputs of 2^17 elements or more: one 1024-thread block per SM at most, so
// few block partials remain for the ticketed last block (with 256-thread
// blocks a 561k-element reduction left it 34 partials per thread); smaller
// inputs: 256-thread blocks (shorter trees, more blocks).
constexpr int kRedBS = 1024;
constexpr i64 kRedBig = i64(1) << 17;
template <typename T, int OP, int BS>
__global__ void __launch_bounds__(BS) k_colred(i64 n, int k, const T *x, const T *y,
                                                i64 rows_per_block, double *part) {
  dep_prologue();
  __shared__ double sh0[BS], sh1[BS];
  const int tid = threadIdx.x;
  const int c = tid % k, rsub = tid / k, rstride = BS / k;
  const i64 r0 = (i64)blockIdx.x * rows_per_block;
  const i64 r1 = min(n, r0 + rows_per_block);
  double a0 = 0, a1 = 0;
  for (i64 r = r0 + rsub; r < r1; r += 4 * (i64)rstride) {
    T xv[4], yv[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const i64 rr = r + (i64)u * rstride;
      const bool ok = rr < r1;
      xv[u] = ok ? x[rr * k + c] : (T)0;
      if constexpr (OP != 0) yv[u] = ok ? y[rr * k + c] : (T)0;
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const double xd = (double)xv[u];
      if constexpr (OP == 0) {
        a0 += xd;
      } else if constexpr (OP == 1) {
        a0 += xd * (double)yv[u];
      } else {
        a0 += xd;
        a1 += xd * (double)yv[u];
      }
    }
  }
  sh0[tid] = a0;
  sh1[tid] = a1;
  __syncthreads();
  for (int s = BS / 2; s >= k; s >>= 1) {
    if (tid < s) {
      sh0[tid] += sh0[tid + s];
      sh1[tid] += sh1[tid + s];
    }
    __syncthreads();
  }
  const int nv = (OP == 2) ? 2 : 1;
  if (tid < k) {
    part[(i64)blockIdx.x * nv * k + tid] = sh0[tid];
    if (OP == 2) part[(i64)blockIdx.x * nv * k + k + tid] = sh1[tid];
  }
}

// one block per output column: 128 threads take strided block partials, then
// a fixed shared-memory tree (deterministic order)
__global__ void __launch_bounds__(128) k_colred_final(int nb, int width, const double *part,
                                                      double *out) {
  dep_prologue();
  __shared__ double sh[128];
  const int j = blockIdx.x, tid = threadIdx.x;
  double s = 0;
#pragma unroll 4
  for (int b = tid; b < nb; b += 128) s += part[(i64)b * width + j];
  sh[tid] = s;
  __syncthreads();
  for (int st = 64; st >= 1; st >>= 1) {
    if (tid < st) sh[tid] += sh[tid + st];
    __syncthreads();
  }
  if (tid == 0) out[j] = sh[0];
}

int red_threads(i64 n, int k) { return n * k >= kRedBig ? kRedBS : 256; }
int colred_blocks(i64 n, int k) {
  if (n * k >= kRedBig)
    return (int)std::max<i64>(1, std::min<i64>(cdiv(n * k, (i64)kRedBS * 16), kSMs));
  return (int)std::max<i64>(1, std::min<i64>(cdiv(n * k, 256 * 8), 2 * kSMs));
}

template <typename T>
__global__ void k_sub_mean(i64 n, int k, T *x, const double *colsum, double inv_n) {
  dep_prologue();
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * k) return;
  double mu = colsum[t % k] * inv_n;  // a product: an FP64 division per element is slow here
  x[t] = (T)((double)x[t] - mu);
}

template <typename T>
__global__ void k_axpby(i64 n, int k, T *y, const T *x, const double *alpha, double sa, double sb) {
  dep_prologue();
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * k) return;
  double a = alpha ? alpha[t % k] : 1.0;
  y[t] = (T)(sb * (double)y[t] + sa * a * (double)x[t]);
}

template <typename T>
__global__ void k_scale_cols(i64 n, int k, T *y, const T *x, const double *coef) {
  dep_prologue();
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * k) return;
  y[t] = (T)((double)x[t] * coef[t % k]);
}

__global__ void k_rsqrt_cols(int k, const double *sq, double *out) {
  dep_prologue();
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= k) return;
  const double v = sq[c];
  out[c] = v > 0 ? 1.0 / sqrt(v) : 0.0;
}

// One thread per column: Givens rotations of the (m + 1) x m Hessenberg
// matrix column by column, then back substitution of the rotated triangle
// (the arithmetic of the outer FGMRES, all steps at once).
__global__ void k_gmres_small(int k, int m, const double *Hb, const double *b2, double *y) {
  dep_prologue();
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= k) return;
  double R[kGmresInnerMax + 1][kGmresInnerMax], cs[kGmresInnerMax], sn[kGmresInnerMax],
      g[kGmresInnerMax + 1], yv[kGmresInnerMax];
  for (int i = 0; i <= m; i++) g[i] = 0.0;
  g[0] = sqrt(fmax(b2[c], 0.0));
  for (int j = 0; j < m; j++) {
    for (int i = 0; i <= j; i++) R[i][j] = Hb[((i64)i * m + j) * k + c];
    R[j + 1][j] = sqrt(fmax(Hb[((i64)(j + 1) * m + j) * k + c], 0.0));
    for (int i = 0; i < j; i++) {
      const double a = R[i][j], b = R[i + 1][j];
      R[i][j] = cs[i] * a + sn[i] * b;
      R[i + 1][j] = -sn[i] * a + cs[i] * b;
    }
    const double a = R[j][j], b = R[j + 1][j];
    const double rho = sqrt(a * a + b * b);
    cs[j] = rho > 0 ? a / rho : 1.0;
    sn[j] = rho > 0 ? b / rho : 0.0;
    R[j][j] = rho;
    R[j + 1][j] = 0.0;
    g[j + 1] = -sn[j] * g[j];
    g[j] = cs[j] * g[j];
  }
  for (int i = m - 1; i >= 0; i--) {
    double t = g[i];
    for (int l = i + 1; l < m; l++) t -= R[i][l] * yv[l];
    yv[i] = R[i][i] != 0 ? t / R[i][i] : 0.0;
  }
  for (int i = 0; i < m; i++) y[(i64)i * k + c] = yv[i];
}

template <typename T>
__global__ void k_fcg_direction(i64 n, int k, T *p, const T *z, const T *pp, const double *beta) {
  dep_prologue();
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * k) return;
  if (pp) p[t] = z[t] - (T)beta[t % k] * pp[t];
  else p[t] = z[t];
}

// column scalar c in the data's type: the float copy when there is one (no
// per-element FP64 conversion), else the FP64 value
template <typename T>
__device__ __forceinline__ T col_scalar(const double *d, const float *f, int c) {
  if constexpr (sizeof(T) == 4) {
    if (f) return f[c];
  }
  return (T)d[c];
}

template <typename T>
__global__ void k_fcg_update(i64 n, int k, T *x, T *r, const T *p, const T *q, const double *alpha,
                             const float *alpha_f, int upd_r, int x_zero) {
  dep_prologue();
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * k) return;
  const T a = col_scalar<T>(alpha, alpha_f, (int)(t % k));
  x[t] = x_zero ? a * p[t] : x[t] + a * p[t];
  if (upd_r) r[t] = r[t] - a * q[t];
}

template <typename T>
__global__ void k_cg_direction(i64 n, int k, T *p, const T *z, const double *beta) {
  dep_prologue();
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * k) return;
  p[t] = z[t] + (T)beta[t % k] * p[t];
}

__global__ void k_scal_div(int k, const double *num, const double *den, double *out,
                           const int *frozen) {
  dep_prologue();
  int c = threadIdx.x + blockIdx.x * blockDim.x;
  if (c >= k) return;
  double d = den[c];
  out[c] = (frozen && frozen[c]) || d == 0.0 ? 0.0 : num[c] / d;
}

__global__ void k_scal_beta(int k, const double *zq, const double *eta_prev, double *beta) {
  dep_prologue();
  int c = threadIdx.x + blockIdx.x * blockDim.x;
  if (c >= k) return;
  double e = eta_prev[c];
  beta[c] = e == 0.0 ? 0.0 : zq[c] / e;
}

// ---- fused reductions ------------------------------------------------------
// FP32 data: the four rows of a group are combined in FP32 (a sum of four
// values or products, fixed order) and only the group's partial is widened
// and added in FP64: one FP64 add per four elements instead of up to five
// FP64-pipe operations (two widenings and three adds) per element, which
// bound these reductions on GB300.  Rows past the end contribute zeros.
template <int OP, int NV>
__device__ __forceinline__ void group4_add(const float (&x)[4], const float (&y)[4],
                                           const float (&w)[4], bool use_y, double (&a)[NV]) {
  if constexpr (OP == 0) {
    a[0] += (double)dev::sum4(x);
  } else if constexpr (OP == 1) {
    a[0] += (double)dev::dot4(x, y);
  } else if constexpr (OP == 2) {
    a[0] += (double)dev::sum4(x);
    if (use_y) {
      a[1] += (double)dev::dot4(x, y);
      a[2] += (double)dev::sum4(y);
    }
  } else {
    a[0] += (double)dev::dot4(x, y);
    a[1] += (double)dev::dot4(x, w);
  }
}
template <int OP, int NV>
__device__ __forceinline__ void group4_add(const double (&)[4], const double (&)[4],
                                           const double (&)[4], bool, double (&)[NV]) {}

// OP 0: [sum x]            OP 1: [sum x.y]
// OP 2: [sum x, sum x.y, sum y]   (FCG beta)     OP 3: [sum x.y, sum x.w]  (alpha)
template <typename T, int OP, int BS>
__global__ void __launch_bounds__(BS)
    k_fused_red(i64 n, int k, const T *x, const T *y, const T *w, i64 rows_per_block,
                double *scratch, FcgScalars sc, double *out) {
  dep_prologue();
  constexpr int NV = (OP == 2) ? 3 : (OP == 3 ? 2 : 1);
  __shared__ double sh[NV][BS];
  __shared__ int last;
  const int tid = threadIdx.x;
  const int c = tid % k, rsub = tid / k, rstride = BS / k;
  const i64 r0 = (i64)blockIdx.x * rows_per_block;
  const i64 r1 = min(n, r0 + rows_per_block);
  double a[NV];
#pragma unroll
  for (int v = 0; v < NV; v++) a[v] = 0;
  // four rows per pass, all loads issued before the (row-ordered) adds
  constexpr bool HAS_Y = OP != 0;
  constexpr bool HAS_W = OP == 3;
  const bool use_y = HAS_Y && y != nullptr;
  for (i64 r = r0 + rsub; r < r1; r += 4 * (i64)rstride) {
    T xv[4], yv[4], wv[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const i64 rr = r + (i64)u * rstride;
      const bool ok = rr < r1;
      const i64 o = rr * k + c;
      xv[u] = ok ? x[o] : (T)0;
      yv[u] = (ok && use_y) ? y[o] : (T)0;
      wv[u] = (HAS_W && ok) ? w[o] : (T)0;
    }
    if constexpr (sizeof(T) == 4) {
      group4_add<OP>(xv, yv, wv, use_y, a);
    } else {
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const double xd = (double)xv[u];
        if constexpr (OP == 0) {
          a[0] += xd;
        } else if constexpr (OP == 1) {
          a[0] += xd * (double)yv[u];
        } else if constexpr (OP == 2) {
          a[0] += xd;
          if (use_y) {
            const double yd = (double)yv[u];
            a[1] += xd * yd;
            a[2] += yd;
          }
        } else {
          a[0] += xd * (double)yv[u];
          a[1] += xd * (double)wv[u];
        }
      }
    }
  }
#pragma unroll
  for (int v = 0; v < NV; v++) sh[v][tid] = a[v];
  __syncthreads();
  for (int st = BS / 2; st >= k; st >>= 1) {
    if (tid < st)
#pragma unroll
      for (int v = 0; v < NV; v++) sh[v][tid] += sh[v][tid + st];
    __syncthreads();
  }
  double *part = scratch + 2;  // scratch[0]: ticket
  if (tid < k)
#pragma unroll
    for (int v = 0; v < NV; v++) part[((i64)blockIdx.x * NV + v) * k + tid] = sh[v][tid];
  __threadfence();
  __syncthreads();
  if (tid == 0) {
    unsigned t = atomicAdd((unsigned *)scratch, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  {
    // all threads: column c, block partials rsub, rsub + rstride, ...; then
    // the same fixed tree over the slots (deterministic order)
    double tb[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) tb[v] = 0;
#pragma unroll 4
    for (unsigned b = rsub; b < gridDim.x; b += rstride)
#pragma unroll
      for (int v = 0; v < NV; v++) tb[v] += __ldcg(part + ((i64)b * NV + v) * k + c);
    __syncthreads();
#pragma unroll
    for (int v = 0; v < NV; v++) sh[v][tid] = tb[v];
    __syncthreads();
    for (int st = BS / 2; st >= k; st >>= 1) {
      if (tid < st)
#pragma unroll
        for (int v = 0; v < NV; v++) sh[v][tid] += sh[v][tid + st];
      __syncthreads();
    }
  }
  if (tid < k) {
    double tot[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) tot[v] = sh[v][tid];
    if constexpr (OP == 0 || OP == 1) {
      out[tid] = tot[0];
    } else if constexpr (OP == 2) {
      double mu = tot[0] / (double)n;
      double beta = 0.0;
      if (y) {
        double e = sc.eta_prev[tid];
        beta = e == 0.0 ? 0.0 : (tot[1] - mu * tot[2]) / e;
      }
      sc.mu[tid] = mu;
      sc.beta[tid] = beta;
      if (sc.mu_f) {
        sc.mu_f[tid] = (float)mu;
        sc.beta_f[tid] = (float)beta;
      }
    } else {
      double eta = tot[0];
      sc.eta[tid] = eta;
      bool fz = sc.frozen && sc.frozen[tid];
      const double alpha = (fz || eta == 0.0) ? 0.0 : tot[1] / eta;
      sc.alpha[tid] = alpha;
      if (sc.alpha_f) sc.alpha_f[tid] = (float)alpha;
    }
  }
  if (tid == 0) *(unsigned *)scratch = 0u;
}

template <typename T>
__global__ void k_fcg_dir(i64 n, int k, T *p, const T *z, const T *pp, FcgScalars sc,
                          float2 *pdf) {
  dep_prologue();
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * k) return;
  int c = (int)(t % k);
  T v = z[t] - col_scalar<T>(sc.mu, sc.mu_f, c);
  if (pp) v = v - col_scalar<T>(sc.beta, sc.beta_f, c) * pp[t];
  p[t] = v;
  if (pdf) {
    float h = (float)v;
    pdf[t] = make_float2(h, (float)((double)v - (double)h));
  }
}

// ---- double-float SpMM ------------------------------------------------------
__device__ __forceinline__ void df_fma(float ah, float al, float xh, float xl, float &sh,
                                       float &sl) {
  float ph = __fmul_rn(ah, xh);
  float pl = __fmaf_rn(ah, xh, -ph);  // exact error of ah*xh
  pl = __fmaf_rn(ah, xl, pl);
  pl = __fmaf_rn(al, xh, pl);
  float s = __fadd_rn(sh, ph);        // TwoSum(sh, ph)
  float v = __fsub_rn(s, sh);
  float e = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, v)), __fsub_rn(ph, v));
  sl = __fadd_rn(sl, __fadd_rn(e, pl));
  sh = s;
}
__device__ __forceinline__ void df_add(float &sh, float &sl, float oh, float ol) {
  float s = __fadd_rn(sh, oh);
  float v = __fsub_rn(s, sh);
  float e = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, v)), __fsub_rn(oh, v));
  sl = __fadd_rn(__fadd_rn(sl, ol), e);
  sh = s;
}
template <int VW>
__device__ __forceinline__ void df_ldg(const float2 *p, float (&h)[VW], float (&l)[VW]) {
  if constexpr (VW == 2) {
    float4 t = __ldg(reinterpret_cast<const float4 *>(p));
    h[0] = t.x; l[0] = t.y; h[1] = t.z; l[1] = t.w;
  } else {
    float2 t = __ldg(p);
    h[0] = t.x; l[0] = t.y;
  }
}

// Entries k, k + E, ... of [k, e), four per step; the next step's column
// indices load before this step's gathers (one dependent latency per step),
// the last entries go one at a time.
template <int K, int VW, int E>
__device__ __forceinline__ void df_row(const MatView<double> &A, const float2 *__restrict__ vdf,
                                       const float2 *__restrict__ X, i64 k, i64 e, int ch,
                                       float (&sh)[VW], float (&sl)[VW]) {
  const i32 *__restrict__ ac = A.ci;
  if (k + 3 * E < e) {
    i32 jn[4];
#pragma unroll
    for (int u = 0; u < 4; u++) jn[u] = __ldg(ac + k + u * E);
    while (true) {
      i32 j[4];
#pragma unroll
      for (int u = 0; u < 4; u++) j[u] = jn[u];
      const i64 kn = k + 4 * E;
      const bool more = kn + 3 * E < e;
      if (more) {
#pragma unroll
        for (int u = 0; u < 4; u++) jn[u] = __ldg(ac + kn + u * E);
      }
      float2 a[4];
      float h[4][VW], l[4][VW];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        a[u] = __ldg(vdf + k + u * E);
        df_ldg<VW>(X + (i64)j[u] * K + ch * VW, h[u], l[u]);
      }
#pragma unroll
      for (int q = 0; q < VW; q++)
#pragma unroll
        for (int u = 0; u < 4; u++) df_fma(a[u].x, a[u].y, h[u][q], l[u][q], sh[q], sl[q]);
      k = kn;
      if (!more) break;
    }
  }
  for (; k < e; k += E) {
    float2 a0 = __ldg(vdf + k);
    i32 j0 = __ldg(ac + k);
    float h0[VW], l0[VW];
    df_ldg<VW>(X + (i64)j0 * K + ch * VW, h0, l0);
#pragma unroll
    for (int q = 0; q < VW; q++) df_fma(a0.x, a0.y, h0[q], l0[q], sh[q], sl[q]);
  }
}

template <int VW, int L, int G>
__device__ __forceinline__ void df_reduce_slots(float (&sh)[VW], float (&sl)[VW]) {
#pragma unroll
  for (int o = L; o < G; o <<= 1)
#pragma unroll
    for (int q = 0; q < VW; q++) {
      float oh = __shfl_xor_sync(0xffffffffu, sh[q], o);
      float ol = __shfl_xor_sync(0xffffffffu, sl[q], o);
      df_add(sh[q], sl[q], oh, ol);
    }
}

// Hub chunk c of the double-float product (32 lanes): chunk partials in
// FP64, the last chunk of a row sums them in chunk order.
template <int K>
__device__ __forceinline__ void df_hub_unit(const MatView<double> &A,
                                            const float2 *__restrict__ vdf,
                                            const float2 *__restrict__ X, double *Y, i64 c,
                                            int lane) {
  constexpr int VW = (K % 2 == 0) ? 2 : 1;
  constexpr int L = K / VW;
  constexpr int E = 32 / L;
  const int slot = lane / L, ch = lane % L;
  if (c >= A.nchunks) return;
  float sh[VW], sl[VW];
#pragma unroll
  for (int q = 0; q < VW; q++) sh[q] = sl[q] = 0.f;
  df_row<K, VW, E>(A, vdf, X, A.ch_beg[c] + slot, A.ch_end[c], ch, sh, sl);
  df_reduce_slots<VW, L, 32>(sh, sl);
  double *part = A.partial;
  if (slot == 0)
#pragma unroll
    for (int q = 0; q < VW; q++) part[c * K + ch * VW + q] = (double)sh[q] + (double)sl[q];
  __threadfence();
  __syncwarp();
  int last = 0;
  if (lane == 0) last = atomicAdd(&A.hub_counter[A.ch_hub[c]], 1) == A.ch_cnt[c] - 1;
  last = __shfl_sync(0xffffffffu, last, 0);
  if (!last) return;
  __threadfence();
  const i64 first = A.ch_first[c];
  const int cnt = A.ch_cnt[c];
  double t[VW];
#pragma unroll
  for (int q = 0; q < VW; q++) t[q] = 0.0;
  for (int u = slot; u < cnt; u += E)
#pragma unroll
    for (int q = 0; q < VW; q++) t[q] += __ldcg(part + (first + u) * K + ch * VW + q);
#pragma unroll
  for (int o = L; o < 32; o <<= 1)
#pragma unroll
    for (int q = 0; q < VW; q++) t[q] += __shfl_xor_sync(0xffffffffu, t[q], o);
  if (slot == 0)
#pragma unroll
    for (int q = 0; q < VW; q++) Y[A.ch_row[c] * K + ch * VW + q] = t[q];
  if (lane == 0) A.hub_counter[A.ch_hub[c]] = 0;
}

// Row streams of the double-float product (the k >= 8 row-stream layout of
// k_spmm_rs): warp w takes rows [srow[w], srow[w + 1]); the next row's end
// and first column indices are loaded during this row's gathers; steps are
// warp-uniform and masked past a row's end; every slot adds its entries in
// entry order as df_row does, so the sums are the same.
template <int K>
__device__ __forceinline__ void df_stream_unit(const MatView<double> &A,
                                               const float2 *__restrict__ vdf,
                                               const float2 *__restrict__ X, double *Y, i64 w,
                                               int lane) {
  constexpr int VW = (K % 2 == 0) ? 2 : 1;
  constexpr int L = K / VW;
  constexpr int E = 32 / L;
  constexpr int STEP = 4 * E;
  const int slot = lane / L, ch = lane % L;
  const i32 *__restrict__ ac = A.ci;
  const i64 *__restrict__ rp = A.rp;
  const int hub = (int)A.hub_thresh;
  int r = __ldg(A.srow + w);
  const int r1 = __ldg(A.srow + w + 1);
  int b = (int)__ldg(rp + r), e = (int)__ldg(rp + r + 1);
  int ee = (hub > 0 && e - b > hub) ? b : e;
  i32 jn[4];
#pragma unroll
  for (int u = 0; u < 4; u++) {
    const int q = b + slot + u * E;
    jn[u] = q < ee ? __ldg(ac + q) : -1;
  }
  while (true) {
    const bool last = r + 1 >= r1;
    const int en = last ? e : (int)__ldg(rp + r + 2);
    float sh[VW], sl[VW];
#pragma unroll
    for (int q = 0; q < VW; q++) sh[q] = sl[q] = 0.f;
    int kb = b;
    while (true) {
      i32 j[4];
#pragma unroll
      for (int u = 0; u < 4; u++) j[u] = jn[u];
      const int kn = kb + STEP;
      const bool more = kn < ee;
      if (more) {
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int q = kn + slot + u * E;
          jn[u] = q < ee ? __ldg(ac + q) : -1;
        }
      } else {
        const int nee = (last || (hub > 0 && en - e > hub)) ? e : en;
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int q = e + slot + u * E;
          jn[u] = q < nee ? __ldg(ac + q) : -1;
        }
      }
      float2 a[4];
      float h[4][VW], l[4][VW];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        if (j[u] >= 0) {
          a[u] = __ldg(vdf + kb + slot + u * E);
          df_ldg<VW>(X + (i64)j[u] * K + ch * VW, h[u], l[u]);
        } else {
          a[u] = make_float2(0.f, 0.f);
#pragma unroll
          for (int q = 0; q < VW; q++) h[u][q] = l[u][q] = 0.f;
        }
      }
#pragma unroll
      for (int q = 0; q < VW; q++)
#pragma unroll
        for (int u = 0; u < 4; u++)
          if (j[u] >= 0) df_fma(a[u].x, a[u].y, h[u][q], l[u][q], sh[q], sl[q]);
      if (!more) break;
      kb = kn;
    }
    df_reduce_slots<VW, L, 32>(sh, sl);
    if ((ee > b || e == b) && slot == 0)
#pragma unroll
      for (int q = 0; q < VW; q++) Y[(i64)r * K + ch * VW + q] = (double)sh[q] + (double)sl[q];
    if (last) break;
    r++;
    b = e;
    e = en;
    ee = (hub > 0 && e - b > hub) ? b : e;
  }
}

template <int K>
__global__ void __launch_bounds__(256, 4) k_spmm_df_rs(const MatView<double> A,
                                                       const float2 *__restrict__ vdf,
                                                       const float2 *__restrict__ X, double *Y) {
  dep_prologue();
  const i64 warp = ((i64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp < A.nstream) df_stream_unit<K>(A, vdf, X, Y, warp, lane);
  else df_hub_unit<K>(A, vdf, X, Y, warp - A.nstream, lane);
}

template <int K, int G>
__global__ void __launch_bounds__(256) k_spmm_df(const MatView<double> A,
                                                 const float2 *__restrict__ vdf,
                                                 const float2 *__restrict__ X, double *Y) {
  dep_prologue();
  constexpr int VW = (K % 2 == 0) ? 2 : 1;
  constexpr int L = K / VW;
  static_assert(L <= G && G <= 32 && (G % L) == 0, "bad layout");
  constexpr int E = G / L;
  constexpr int RPW = 32 / G;
  const int lane = threadIdx.x & 31;
  const int g = lane % G, slot = g / L, ch = g % L;
  const i64 warp = ((i64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const i64 nregw = (A.n + RPW - 1) / RPW;
  float sh[VW], sl[VW];
#pragma unroll
  for (int q = 0; q < VW; q++) sh[q] = sl[q] = 0.f;
  if (warp < nregw) {
    const i64 r = warp * RPW + lane / G;
    bool act = r < A.n;
    i64 b = 0, e = 0;
    if (act) {
      b = A.rp[r];
      e = A.rp[r + 1];
      if (A.hub_thresh > 0 && e - b > A.hub_thresh) act = false;
    }
    if (act) df_row<K, VW, E>(A, vdf, X, b + slot, e, ch, sh, sl);
    df_reduce_slots<VW, L, G>(sh, sl);
    if (act && slot == 0)
#pragma unroll
      for (int q = 0; q < VW; q++) Y[r * K + ch * VW + q] = (double)sh[q] + (double)sl[q];
    return;
  }
  if constexpr (G == 32) df_hub_unit<K>(A, vdf, X, Y, warp - nregw, lane);
}

template <int K, int G>
void launch_df(const MatView<double> &A, const float2 *vdf, const float2 *X, double *Y,
               cudaStream_t s) {
  constexpr int RPW = 32 / G;
  i64 warps = cdiv(A.n, RPW) + ((G == 32) ? A.nchunks : 0);
  if (warps == 0) return;
  launch_dep(k_spmm_df<K, G>, grid_for(warps * 32, 256), 256, 0, s, A, vdf, X, Y);
  LG_LAUNCH();
}

__global__ void k_split_df(i64 cnt, const double *v, float2 *o) {
  dep_prologue();
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= cnt) return;
  double x = v[t];
  float h = (float)x;
  o[t] = make_float2(h, (float)(x - (double)h));
}

int fused_blocks(i64 n, int k) {
  return colred_blocks(n, k);
}

}  // namespace

// ---- segment-mode kernels ---------------------------------------------------
namespace {
// OP 0: sum x; 1: x.y; 2: beta step (sum z, z.qp, sum qp); 3: alpha (p.q, p.r)
template <typename T, int OP>
__global__ void __launch_bounds__(256)
    k_seg_red(SegInfo S, const T *x, const T *y, const T *w, FcgScalars sc, double *out) {
  constexpr int NV = (OP == 2) ? 3 : (OP == 3 ? 2 : 1);
  __shared__ double sh[NV][256];
  const i64 sg = blockIdx.x;
  const i64 r0 = S.ptr[sg], r1 = S.ptr[sg + 1];
  double a[NV];
#pragma unroll
  for (int v = 0; v < NV; v++) a[v] = 0;
  for (i64 r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
    double xv = (double)x[r];
    if constexpr (OP == 0) {
      a[0] += xv;
    } else if constexpr (OP == 1) {
      a[0] += xv * (double)y[r];
    } else if constexpr (OP == 2) {
      a[0] += xv;
      if (y) {
        double yv = (double)y[r];
        a[1] += xv * yv;
        a[2] += yv;
      }
    } else {
      a[0] += xv * (double)y[r];
      a[1] += xv * (double)w[r];
    }
  }
#pragma unroll
  for (int v = 0; v < NV; v++) sh[v][threadIdx.x] = a[v];
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if ((int)threadIdx.x < st)
#pragma unroll
      for (int v = 0; v < NV; v++) sh[v][threadIdx.x] += sh[v][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x) return;
  if constexpr (OP == 0) {
    out[sg] = sh[0][0] / (double)(r1 - r0);  // the segment's mean
  } else if constexpr (OP == 1) {
    out[sg] = sh[0][0];
  } else if constexpr (OP == 2) {
    double mu = sh[0][0] / (double)(r1 - r0);
    sc.mu[sg] = mu;
    double e = sc.eta_prev[sg];
    sc.beta[sg] = (y && e != 0.0) ? (sh[1][0] - mu * sh[2][0]) / e : 0.0;
  } else {
    double eta = sh[0][0];
    sc.eta[sg] = eta;
    bool fz = sc.frozen && sc.frozen[sg];
    sc.alpha[sg] = (fz || eta == 0.0) ? 0.0 : sh[1][0] / eta;
  }
}

template <typename T>
__global__ void k_seg_sub_mean(SegInfo S, i64 n, T *x, const double *means) {
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  x[t] = (T)((double)x[t] - means[S.rowseg[t]]);
}

template <typename T>
__global__ void k_seg_fcg_dir(SegInfo S, i64 n, T *p, const T *z, const T *pp, FcgScalars sc,
                              float2 *pdf) {
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  i32 sg = S.rowseg[t];
  T v = z[t] - (T)sc.mu[sg];
  if (pp) v = v - (T)sc.beta[sg] * pp[t];
  p[t] = v;
  if (pdf) {
    float h = (float)v;
    pdf[t] = make_float2(h, (float)((double)v - (double)h));
  }
}

template <typename T>
__global__ void k_seg_fcg_update(SegInfo S, i64 n, T *x, T *r, const T *p, const T *q,
                                 const double *alpha, int upd) {
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  T a = (T)alpha[S.rowseg[t]];
  x[t] = x[t] + a * p[t];
  if (upd) r[t] = r[t] - a * q[t];
}

__global__ void k_seg_converge(i64 nseg, const double *rn2, const double *rn0sq, double tol2,
                               int it, int *frozen, int *iters) {
  i64 sg = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (sg >= nseg || frozen[sg]) return;
  iters[sg] = it + 1;
  if (rn2[sg] <= tol2 * rn0sq[sg]) frozen[sg] = 1;  // a NaN norm never freezes
}
}  // namespace

template <typename T>
void seg_fcg_beta(const SegInfo &S, const T *z, const T *qp, FcgScalars sc, cudaStream_t s) {
  k_seg_red<T, 2><<<(unsigned)S.nseg, 256, 0, s>>>(S, z, qp, nullptr, sc, nullptr);
  LG_LAUNCH();
}
template <typename T>
void seg_fcg_alpha(const SegInfo &S, const T *p, const T *q, const T *r, FcgScalars sc,
                   cudaStream_t s) {
  k_seg_red<T, 3><<<(unsigned)S.nseg, 256, 0, s>>>(S, p, q, r, sc, nullptr);
  LG_LAUNCH();
}
template <typename T>
void seg_dot(const SegInfo &S, const T *x, const T *y, double *out, cudaStream_t s) {
  FcgScalars none{};
  k_seg_red<T, 1><<<(unsigned)S.nseg, 256, 0, s>>>(S, x, y, nullptr, none, out);
  LG_LAUNCH();
}
template <typename T>
void seg_mean(const SegInfo &S, const T *x, double *out, cudaStream_t s) {
  FcgScalars none{};
  k_seg_red<T, 0><<<(unsigned)S.nseg, 256, 0, s>>>(S, x, nullptr, nullptr, none, out);
  LG_LAUNCH();
}
template <typename T>
void seg_sub_mean(const SegInfo &S, i64 n, T *x, const double *means, cudaStream_t s) {
  k_seg_sub_mean<T><<<grid_for(n, 256), 256, 0, s>>>(S, n, x, means);
  LG_LAUNCH();
}
template <typename T>
void seg_fcg_dir(const SegInfo &S, i64 n, T *p, const T *z, const T *pp, FcgScalars sc,
                 cudaStream_t s, float2 *pdf) {
  k_seg_fcg_dir<T><<<grid_for(n, 256), 256, 0, s>>>(S, n, p, z, pp, sc, pdf);
  LG_LAUNCH();
}
template <typename T>
void seg_fcg_update(const SegInfo &S, i64 n, T *x, T *r, const T *p, const T *q,
                    const double *alpha, bool update_r, cudaStream_t s) {
  k_seg_fcg_update<T><<<grid_for(n, 256), 256, 0, s>>>(S, n, x, r, p, q, alpha, update_r ? 1 : 0);
  LG_LAUNCH();
}
void seg_converge(i64 nseg, const double *rn2, const double *rn0sq, double tol, int it,
                  int *frozen, int *iters, cudaStream_t s) {
  k_seg_converge<<<grid_for(nseg, 128), 128, 0, s>>>(nseg, rn2, rn0sq, tol * tol, it, frozen,
                                                      iters);
  LG_LAUNCH();
}
#define LG_SEG_INST(T)                                                                      \
  template void seg_fcg_beta<T>(const SegInfo &, const T *, const T *, FcgScalars,          \
                                cudaStream_t);                                              \
  template void seg_fcg_alpha<T>(const SegInfo &, const T *, const T *, const T *,          \
                                 FcgScalars, cudaStream_t);                                 \
  template void seg_dot<T>(const SegInfo &, const T *, const T *, double *, cudaStream_t);  \
  template void seg_mean<T>(const SegInfo &, const T *, double *, cudaStream_t);            \
  template void seg_sub_mean<T>(const SegInfo &, i64, T *, const double *, cudaStream_t);   \
  template void seg_fcg_dir<T>(const SegInfo &, i64, T *, const T *, const T *, FcgScalars, \
                               cudaStream_t, float2 *);                                     \
  template void seg_fcg_update<T>(const SegInfo &, i64, T *, T *, const T *, const T *,     \
                                  const double *, bool, cudaStream_t);
LG_SEG_INST(float)
LG_SEG_INST(double)

i64 fused_scratch_len(i64 n, int k) { return 2 + (i64)fused_blocks(n, k) * 3 * k; }

template <typename T>
void fcg_beta(i64 n, int k, const T *z, const T *qp, FcgScalars sc, double *scratch,
              cudaStream_t s) {
  int nb = fused_blocks(n, k);
  if (red_threads(n, k) == kRedBS)
    launch_dep(k_fused_red<T, 2, kRedBS>, nb, kRedBS, 0, s, n, k, z, qp, nullptr, cdiv(n, nb), scratch, sc, nullptr);
  else
    launch_dep(k_fused_red<T, 2, 256>, nb, 256, 0, s, n, k, z, qp, nullptr, cdiv(n, nb), scratch, sc, nullptr);
  LG_LAUNCH();
}
template <typename T>
void fcg_dir(i64 n, int k, T *p, const T *z, const T *pp, FcgScalars sc, cudaStream_t s,
             float2 *pdf) {
  launch_dep(k_fcg_dir<T>, grid_for(n * k, 256), 256, 0, s, n, k, p, z, pp, sc, pdf);
  LG_LAUNCH();
}

void spmm_df(const MatView<double> &A, const float2 *vdf, const float2 *X, int k, double *Y,
             cudaStream_t s) {
  if (A.nstream > 0 && (k == 8 || k == 16 || k == 32 || k == 64)) {
    const unsigned g = grid_for((A.nstream + A.nchunks) * 32, 256);
    switch (k) {
      case 8: launch_dep(k_spmm_df_rs<8>, g, 256, 0, s, A, vdf, X, Y); break;
      case 16: launch_dep(k_spmm_df_rs<16>, g, 256, 0, s, A, vdf, X, Y); break;
      case 32: launch_dep(k_spmm_df_rs<32>, g, 256, 0, s, A, vdf, X, Y); break;
      default: launch_dep(k_spmm_df_rs<64>, g, 256, 0, s, A, vdf, X, Y); break;
    }
    LG_LAUNCH();
    return;
  }
  bool hub = A.nchunks > 0;
  int g = hub ? 32 : A.lanes_per_row;
  switch (k) {
    case 1:
      switch (g) {
        case 4: return launch_df<1, 4>(A, vdf, X, Y, s);
        case 8: return launch_df<1, 8>(A, vdf, X, Y, s);
        case 16: return launch_df<1, 16>(A, vdf, X, Y, s);
        default: return launch_df<1, 32>(A, vdf, X, Y, s);
      }
    case 2: return launch_df<2, 32>(A, vdf, X, Y, s);
    case 4: return launch_df<4, 32>(A, vdf, X, Y, s);
    case 8: return launch_df<8, 32>(A, vdf, X, Y, s);
    case 16: return launch_df<16, 32>(A, vdf, X, Y, s);
    case 32: return launch_df<32, 32>(A, vdf, X, Y, s);
    case 64: return launch_df<64, 32>(A, vdf, X, Y, s);
    default: throw Error(LIGMG_ERR_UNSUPPORTED, "k must be 1,2,4,8,16,32,64");
  }
}

void split_df(i64 count, const double *v, float2 *out, cudaStream_t s) {
  if (count <= 0) return;
  launch_dep(k_split_df, grid_for(count, 256), 256, 0, s, count, v, out);
  LG_LAUNCH();
}
template <typename T>
void fcg_alpha(i64 n, int k, const T *p, const T *q, const T *r, FcgScalars sc,
               double *scratch, cudaStream_t s) {
  int nb = fused_blocks(n, k);
  if (red_threads(n, k) == kRedBS)
    launch_dep(k_fused_red<T, 3, kRedBS>, nb, kRedBS, 0, s, n, k, p, q, r, cdiv(n, nb), scratch, sc, nullptr);
  else
    launch_dep(k_fused_red<T, 3, 256>, nb, 256, 0, s, n, k, p, q, r, cdiv(n, nb), scratch, sc, nullptr);
  LG_LAUNCH();
}
template <typename T>
void col_dot1(i64 n, int k, const T *x, const T *y, double *out, double *scratch, cudaStream_t s) {
  int nb = fused_blocks(n, k);
  FcgScalars none{};
  if (red_threads(n, k) == kRedBS)
    launch_dep(k_fused_red<T, 1, kRedBS>, nb, kRedBS, 0, s, n, k, x, y, nullptr, cdiv(n, nb), scratch, none, out);
  else
    launch_dep(k_fused_red<T, 1, 256>, nb, 256, 0, s, n, k, x, y, nullptr, cdiv(n, nb), scratch, none, out);
  LG_LAUNCH();
}

template <typename T>
void cheb_init_zero(i64 n, int k, const T *b, const T *invd, double scale, T *d, cudaStream_t s) {
  launch_dep(k_cheb_init_zero<T>, grid_for(n * k, 256), 256, 0, s, n, k, b, invd, (T)scale, d);
  LG_LAUNCH();
}
template <typename T>
void fill_value(i64 cnt, T *x, T v, cudaStream_t s) {
  if (cnt <= 0) return;
  launch_dep(k_fill<T>, grid_for(cnt, 256), 256, 0, s, cnt, x, v);
  LG_LAUNCH();
}
template <typename T>
void prolong_agg(i64 n, int k, const i32 *agg, const T *xc, T *x, cudaStream_t s) {
  launch_dep(k_prolong_agg<T>, grid_for(n * k, 256), 256, 0, s, n, k, agg, xc, x);
  LG_LAUNCH();
}
template <typename T>
void coarse_apply(i64 n, int k, const T *pinv, const T *b, T *x, cudaStream_t s) {
  launch_dep(k_coarse_apply<T>, grid_for(n * k, 128), 128, 0, s, n, k, pinv, b, x);
  LG_LAUNCH();
}
template <typename T>
void scale_vec(i64 n, int k, T *x, double f, cudaStream_t s) {
  launch_dep(k_scale<T>, grid_for(n * k, 256), 256, 0, s, n * k, x, (T)f);
  LG_LAUNCH();
}
template <typename S, typename D>
void convert(i64 count, const S *src, D *dst, cudaStream_t s) {
  if (count <= 0) return;
  launch_dep(k_convert<S, D>, grid_for(count, 256), 256, 0, s, count, src, dst);
  LG_LAUNCH();
}

i64 col_reduce_scratch(i64 n, int k) { return (i64)colred_blocks(n, k) * 2 * k; }

template <typename T>
void col_reduce(i64 n, int k, Red op, const T *x, const T *y, double *out, double *scratch,
                i64 scratch_len, cudaStream_t s) {
  if (256 % k != 0) throw Error(LIGMG_ERR_UNSUPPORTED, "reduction width");
  const bool big = red_threads(n, k) == kRedBS;
  int nb = colred_blocks(n, k);
  if ((i64)nb * 2 * k > scratch_len) throw Error(LIGMG_ERR_INTERNAL, "reduction scratch");
  i64 rpb = cdiv(n, nb);
  int width = k;
  switch (op) {
    case Red::Sum:
      if (big) launch_dep(k_colred<T, 0, kRedBS>, nb, kRedBS, 0, s, n, k, x, y, rpb, scratch);
      else launch_dep(k_colred<T, 0, 256>, nb, 256, 0, s, n, k, x, y, rpb, scratch);
      break;
    case Red::Dot:
      if (big) launch_dep(k_colred<T, 1, kRedBS>, nb, kRedBS, 0, s, n, k, x, y, rpb, scratch);
      else launch_dep(k_colred<T, 1, 256>, nb, 256, 0, s, n, k, x, y, rpb, scratch);
      break;
    case Red::Sum2Dot:
      if (big) launch_dep(k_colred<T, 2, kRedBS>, nb, kRedBS, 0, s, n, k, x, y, rpb, scratch);
      else launch_dep(k_colred<T, 2, 256>, nb, 256, 0, s, n, k, x, y, rpb, scratch);
      width = 2 * k;
      break;
  }
  LG_LAUNCH();
  launch_dep(k_colred_final, width, 128, 0, s, nb, width, scratch, out);
  LG_LAUNCH();
}

template <typename T>
void sub_mean(i64 n, int k, T *x, const double *colsum, cudaStream_t s) {
  launch_dep(k_sub_mean<T>, grid_for(n * k, 256), 256, 0, s, n, k, x, colsum, 1.0 / (double)n);
  LG_LAUNCH();
}
template <typename T>
void axpby_cols(i64 n, int k, T *y, const T *x, const double *alpha, double sa, double sb,
                cudaStream_t s) {
  launch_dep(k_axpby<T>, grid_for(n * k, 256), 256, 0, s, n, k, y, x, alpha, sa, sb);
  LG_LAUNCH();
}
template <typename T>
void scale_cols(i64 n, int k, T *y, const T *x, const double *coef, cudaStream_t s) {
  launch_dep(k_scale_cols<T>, grid_for(n * k, 256), 256, 0, s, n, k, y, x, coef);
  LG_LAUNCH();
}
void rsqrt_cols(int k, const double *sq, double *out, cudaStream_t s) {
  launch_dep(k_rsqrt_cols, 1, 64 * cdiv(k, 64), 0, s, k, sq, out);
  LG_LAUNCH();
}
void gmres_small(int k, int m, const double *Hb, const double *b2, double *y, cudaStream_t s) {
  if (m < 1 || m > kGmresInnerMax) throw Error(LIGMG_ERR_INVALID_ARGUMENT, "inner FGMRES steps");
  launch_dep(k_gmres_small, 1, 64 * cdiv(k, 64), 0, s, k, m, Hb, b2, y);
  LG_LAUNCH();
}
template <typename T>
void fcg_direction(i64 n, int k, T *p, const T *z, const T *pprev, const double *beta,
                   cudaStream_t s) {
  launch_dep(k_fcg_direction<T>, grid_for(n * k, 256), 256, 0, s, n, k, p, z, pprev, beta);
  LG_LAUNCH();
}
template <typename T>
void fcg_update(i64 n, int k, T *x, T *r, const T *p, const T *q, const double *alpha,
                bool update_r, cudaStream_t s, const float *alpha_f, bool x_zero) {
  launch_dep(k_fcg_update<T>, grid_for(n * k, 256), 256, 0, s, n, k, x, r, p, q, alpha, alpha_f,
                                                       update_r ? 1 : 0, x_zero ? 1 : 0);
  LG_LAUNCH();
}
template <typename T>
void cg_direction(i64 n, int k, T *p, const T *z, const double *beta, cudaStream_t s) {
  launch_dep(k_cg_direction<T>, grid_for(n * k, 256), 256, 0, s, n, k, p, z, beta);
  LG_LAUNCH();
}

void scal_div(int k, const double *num, const double *den, double *out, const int *frozen,
              cudaStream_t s) {
  launch_dep(k_scal_div, 1, 128, 0, s, k, num, den, out, frozen);
  LG_LAUNCH();
}
void scal_beta(int k, const double *zq, const double *eta_prev, double *beta, cudaStream_t s) {
  launch_dep(k_scal_beta, 1, 128, 0, s, k, zq, eta_prev, beta);
  LG_LAUNCH();
}

#define LG_INST(T)                                                                             \
  template void fcg_beta<T>(i64, int, const T *, const T *, FcgScalars, double *, cudaStream_t); \
  template void fcg_dir<T>(i64, int, T *, const T *, const T *, FcgScalars, cudaStream_t,     \
                           float2 *);                                                          \
  template void fcg_alpha<T>(i64, int, const T *, const T *, const T *, FcgScalars, double *,  \
                             cudaStream_t);                                                    \
  template void col_dot1<T>(i64, int, const T *, const T *, double *, double *, cudaStream_t); \
  template void cheb_init_zero<T>(i64, int, const T *, const T *, double, T *, cudaStream_t); \
  template void fill_value<T>(i64, T *, T, cudaStream_t);                                    \
  template void prolong_agg<T>(i64, int, const i32 *, const T *, T *, cudaStream_t);         \
  template void coarse_apply<T>(i64, int, const T *, const T *, T *, cudaStream_t);          \
  template void scale_vec<T>(i64, int, T *, double, cudaStream_t);                           \
  template void col_reduce<T>(i64, int, Red, const T *, const T *, double *, double *, i64,  \
                              cudaStream_t);                                                   \
  template void sub_mean<T>(i64, int, T *, const double *, cudaStream_t);                    \
  template void axpby_cols<T>(i64, int, T *, const T *, const double *, double, double,      \
                              cudaStream_t);                                                   \
  template void fcg_direction<T>(i64, int, T *, const T *, const T *, const double *,        \
                                 cudaStream_t);                                                \
  template void fcg_update<T>(i64, int, T *, T *, const T *, const T *, const double *, bool, \
                              cudaStream_t, const float *, bool);                              \
  template void cg_direction<T>(i64, int, T *, const T *, const double *, cudaStream_t);    \
  template void scale_cols<T>(i64, int, T *, const T *, const double *, cudaStream_t);
LG_INST(float)
LG_INST(double)
template void convert<double, float>(i64, const double *, float *, cudaStream_t);
template void convert<float, double>(i64, const float *, double *, cudaStream_t);
template void convert<double, double>(i64, const double *, double *, cudaStream_t);

}  // namespace lg
