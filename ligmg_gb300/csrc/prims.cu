// prims.cu — exclusive scan, stable radix sort and compaction on sm_103a.
#include "prims.cuh"

namespace lg {

int64_t g_launches = 0;
thread_local bool g_free_sync = false;
thread_local bool g_dep_launch = false;

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;

template <typename T>
__device__ T block_exclusive_scan(T v, T *warp_tot, T &block_total) {
  // inclusive warp scan
  unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (unsigned)o) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  if (warp == 0) {
    T t = (lane < (kScanThreads / 32)) ? warp_tot[lane] : T(0);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= (unsigned)o) t += y;
    }
    if (lane < (kScanThreads / 32)) warp_tot[lane] = t;  // inclusive per warp
  }
  __syncthreads();
  T warp_off = warp ? warp_tot[warp - 1] : T(0);
  block_total = warp_tot[kScanThreads / 32 - 1];
  return warp_off + x - v;  // exclusive
}

template <typename T>
__global__ void __launch_bounds__(kScanThreads) k_scan_sums(const T *in, i64 n, T *bsums) {
  i64 base = (i64)blockIdx.x * kScanTile;
  T s = 0;
  for (int k = 0; k < kScanItems; k++) {
    i64 i = base + (i64)k * kScanThreads + threadIdx.x;
    if (i < n) s += in[i];
  }
  __shared__ T red[kScanThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    T t = 0;
    for (int w = 0; w < kScanThreads / 32; w++) t += red[w];
    bsums[blockIdx.x] = t;
  }
}

template <typename T>
__global__ void __launch_bounds__(kScanThreads)
    k_scan_apply(const T *in, T *out, i64 n, const T *boffs, T *total) {
  __shared__ T tile[kScanTile];
  __shared__ T warp_tot[kScanThreads / 32];
  i64 base = (i64)blockIdx.x * kScanTile;
  for (int k = 0; k < kScanItems; k++) {
    int j = k * kScanThreads + threadIdx.x;
    i64 i = base + j;
    tile[j] = (i < n) ? in[i] : T(0);
  }
  __syncthreads();
  T loc[kScanItems];
  T s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    loc[k] = tile[threadIdx.x * kScanItems + k];
    s += loc[k];
  }
  T btot;
  T off = block_exclusive_scan<T>(s, warp_tot, btot);
  T boff = boffs ? boffs[blockIdx.x] : T(0);
  off += boff;
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    tile[threadIdx.x * kScanItems + k] = off;
    off += loc[k];
  }
  __syncthreads();
  for (int k = 0; k < kScanItems; k++) {
    int j = k * kScanThreads + threadIdx.x;
    i64 i = base + j;
    if (i < n) out[i] = tile[j];
  }
  if (total && blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) *total = boff + btot;
}

}  // namespace

template <typename T>
void exclusive_scan(const T *in, T *out, i64 n, cudaStream_t s, T *total) {
  if (n <= 0) {
    if (total) LG_CUDA(cudaMemsetAsync(total, 0, sizeof(T), s));
    return;
  }
  i64 nb = cdiv(n, kScanTile);
  if (nb == 1) {
    k_scan_apply<T><<<1, kScanThreads, 0, s>>>(in, out, n, nullptr, total);
    LG_LAUNCH();
    return;
  }
  DBuf<T> bs(nb, s), bo(nb, s);
  k_scan_sums<T><<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, bs.p);
  LG_LAUNCH();
  exclusive_scan<T>(bs.p, bo.p, nb, s, nullptr);
  k_scan_apply<T><<<(unsigned)nb, kScanThreads, 0, s>>>(in, out, n, bo.p, total);
  LG_LAUNCH();
}

template void exclusive_scan<i32>(const i32 *, i32 *, i64, cudaStream_t, i32 *);
template void exclusive_scan<i64>(const i64 *, i64 *, i64, cudaStream_t, i64 *);
template void exclusive_scan<u32>(const u32 *, u32 *, i64, cudaStream_t, u32 *);

// ---------------------------------------------------------------------------
// Stable LSD radix sort, 8-bit digits.  Each pass: per-tile digit histogram,
// exclusive scan over [digit][tile], then a stable scatter in which every
// tile ranks its items in input order (16 rounds of 256 items; inside a round
// a warp ranks equal digits with __match_any_sync, warps are ordered through
// shared-memory counts).
namespace {
constexpr int kRsThreads = 256;
constexpr int kRsRounds = 16;
constexpr int kRsTile = kRsThreads * kRsRounds;
constexpr int kRsWarps = kRsThreads / 32;

__global__ void __launch_bounds__(kRsThreads)
    k_radix_hist(const u64 *keys, i64 n, int shift, u32 *hist, i64 ntiles) {
  __shared__ u32 h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  i64 base = (i64)blockIdx.x * kRsTile;
  for (int r = 0; r < kRsRounds; r++) {
    i64 i = base + (i64)r * kRsThreads + threadIdx.x;
    if (i < n) atomicAdd(&h[(unsigned)(keys[i] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[(i64)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(kRsThreads)
    k_radix_scatter(const u64 *kin, const u32 *vin, u64 *kout, u32 *vout, i64 n, int shift,
                    const u32 *offs, i64 ntiles) {
  __shared__ u32 base_s[256];
  __shared__ u32 wcnt[kRsWarps][257];
  unsigned warp = threadIdx.x >> 5;
  base_s[threadIdx.x] = offs[(i64)threadIdx.x * ntiles + blockIdx.x];
  i64 tbase = (i64)blockIdx.x * kRsTile;
  unsigned ltmask = lanemask_lt();
  for (int r = 0; r < kRsRounds; r++) {
    for (int q = threadIdx.x; q < kRsWarps * 257; q += kRsThreads) (&wcnt[0][0])[q] = 0;
    __syncthreads();
    i64 i = tbase + (i64)r * kRsThreads + threadIdx.x;
    bool valid = i < n;
    u64 key = valid ? kin[i] : 0;
    u32 val = valid ? vin[i] : 0;
    unsigned d = valid ? ((unsigned)(key >> shift) & 255u) : 256u;
    unsigned mask = __match_any_sync(0xffffffffu, d);
    unsigned rank = __popc(mask & ltmask);
    if (rank == 0) wcnt[warp][d] = __popc(mask);
    __syncthreads();
    if (valid) {
      u32 off = base_s[d] + rank;
      for (unsigned w = 0; w < warp; w++) off += wcnt[w][d];
      kout[off] = key;
      vout[off] = val;
    }
    __syncthreads();
    u32 add = 0;
    for (int w = 0; w < kRsWarps; w++) add += wcnt[w][threadIdx.x];
    base_s[threadIdx.x] += add;
    __syncthreads();
  }
}
}  // namespace

void radix_sort_pairs(u64 *keys, u32 *vals, i64 n, int key_bits, cudaStream_t s) {
  if (n <= 1 || key_bits <= 0) return;
  if (n >= (i64)0xffffffffLL) throw Error(LIGMG_ERR_UNSUPPORTED, "radix sort size");
  i64 ntiles = cdiv(n, kRsTile);
  DBuf<u64> k2(n, s);
  DBuf<u32> v2(n, s);
  DBuf<u32> hist(256 * ntiles, s), offs(256 * ntiles, s);
  u64 *ka = keys, *kb = k2.p;
  u32 *va = vals, *vb = v2.p;
  int passes = (key_bits + 7) / 8;
  for (int p = 0; p < passes; p++) {
    int shift = 8 * p;
    k_radix_hist<<<(unsigned)ntiles, kRsThreads, 0, s>>>(ka, n, shift, hist.p, ntiles);
    LG_LAUNCH();
    exclusive_scan<u32>(hist.p, offs.p, 256 * ntiles, s);
    k_radix_scatter<<<(unsigned)ntiles, kRsThreads, 0, s>>>(ka, va, kb, vb, n, shift, offs.p,
                                                            ntiles);
    LG_LAUNCH();
    std::swap(ka, kb);
    std::swap(va, vb);
  }
  if (ka != keys) {
    LG_CUDA(cudaMemcpyAsync(keys, ka, sizeof(u64) * n, cudaMemcpyDeviceToDevice, s));
    LG_CUDA(cudaMemcpyAsync(vals, va, sizeof(u32) * n, cudaMemcpyDeviceToDevice, s));
  }
}

namespace {
__global__ void k_flags_to_i64(const uint8_t *f, i64 n, i64 *o) {
  i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) o[i] = f[i] ? 1 : 0;
}
__global__ void k_compact(const uint8_t *f, const i64 *pos, i64 n, i32 *out) {
  i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && f[i]) out[pos[i]] = (i32)i;
}
}  // namespace

i64 compact_indices(const uint8_t *flags, i64 n, i32 *out, cudaStream_t s) {
  if (n <= 0) return 0;
  DBuf<i64> t(n, s), pos(n, s), tot(1, s);
  k_flags_to_i64<<<grid_for(n, 256), 256, 0, s>>>(flags, n, t.p);
  LG_LAUNCH();
  exclusive_scan<i64>(t.p, pos.p, n, s, tot.p);
  k_compact<<<grid_for(n, 256), 256, 0, s>>>(flags, pos.p, n, out);
  LG_LAUNCH();
  return read_scalar(tot.p, s);
}

int bits_for(i64 maxval) {
  int b = 0;
  while (b < 63 && ((i64)1 << b) <= maxval) b++;
  return b;
}

}  // namespace lg
