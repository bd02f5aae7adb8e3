// peaks.cu — the gather ceiling that bounds the solve's sparse products.
//
// Every matrix entry of y = A X gathers one row of X (k values) from wherever
// its column points.  On the large levels X fits in L2 but not in L1, so the
// products are bound neither by HBM nor by arithmetic but by how many random
// rows per second the SMs can pull from L2: for 4- and 8-byte rows (k = 1)
// the L1's one distinct cache line per clock, for 128-byte rows (k = 32
// floats) the L2-to-SM return path.  This file measures that ceiling on the
// running GPU with the products' own access pattern stripped to the gathers:
// `count` rows of `width` bytes at pseudo-random positions (an index array
// read in order, as a product reads its column indices) of a table of `rows`
// rows, every SM full of warps with independent gathers in flight (or
// `blocks_per_sm` blocks of 256 threads per SM, to see how the rate depends
// on the gathers in flight).
#include "peaks.cuh"

namespace lg {
namespace {

constexpr int kPeakThreads = 256;
constexpr int kPeakBlocksPerSM = 8;

__device__ __forceinline__ u32 peak_hash(u32 x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

// Pseudo-random row positions, written once: the timed kernels read them
// like a sparse product reads its column indices (consecutive, coalesced).
__global__ void k_peak_index(i32 *idx, i64 len, u32 rows) {
  const i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < len) idx[t] = (i32)(peak_hash((u32)t) % rows);
}

// 4- or 8-byte rows: a thread gathers U independent rows per step.
template <typename T, int U>
__global__ void __launch_bounds__(kPeakThreads) k_peak_elems(const T *__restrict__ tab,
                                                            const i32 *__restrict__ idx,
                                                            i64 count, T *sink) {
  const i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  const i64 nt = (i64)gridDim.x * blockDim.x;
  T acc = 0;
  for (i64 base = t * U; base < count; base += nt * U) {
    i32 j[U];
#pragma unroll
    for (int u = 0; u < U; u++) j[u] = base + u < count ? __ldg(idx + base + u) : -1;
    T v[U];
#pragma unroll
    for (int u = 0; u < U; u++) v[u] = j[u] >= 0 ? __ldg(tab + j[u]) : (T)0;
#pragma unroll
    for (int u = 0; u < U; u++) acc += v[u];
  }
  if (acc == (T)-1) sink[0] = acc;  // never true for a zero table: keeps the loads
}

// 128-byte rows: eight lanes share a row (a 16-byte piece each), four rows
// per warp instruction, U instructions in flight per step.
template <int U>
__global__ void __launch_bounds__(kPeakThreads) k_peak_rows(const float4 *__restrict__ tab,
                                                           const i32 *__restrict__ idx,
                                                           i64 count, float *sink) {
  const int lane = threadIdx.x & 31, slot = lane >> 3, ch = lane & 7;
  const i64 w = ((i64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const i64 nw = ((i64)gridDim.x * blockDim.x) >> 5;
  float acc = 0.f;
  for (i64 base = w * 4 * U; base < count; base += nw * 4 * U) {
    i32 j[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const i64 e = base + 4 * u + slot;
      j[u] = e < count ? __ldg(idx + e) : -1;
    }
    float4 v[U];
#pragma unroll
    for (int u = 0; u < U; u++)
      v[u] = j[u] >= 0 ? __ldg(tab + (i64)j[u] * 8 + ch) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int u = 0; u < U; u++) acc += (v[u].x + v[u].y) + (v[u].z + v[u].w);
  }
  if (acc == -1.f) sink[0] = acc;
}

}  // namespace

double gather_peak(i64 rows, int width, i64 count, int blocks_per_sm) {
  cudaStream_t s;
  LG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  void *tab = nullptr, *sink = nullptr;
  i32 *idx = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  double rate = 0.0;
  bool failed = false;
  try {
    LG_CUDA(cudaMallocAsync(&tab, (size_t)rows * width, s));
    LG_CUDA(cudaMallocAsync(&sink, 64, s));
    LG_CUDA(cudaMallocAsync((void **)&idx, (size_t)count * sizeof(i32), s));
    LG_CUDA(cudaMemsetAsync(tab, 0, (size_t)rows * width, s));
    k_peak_index<<<grid_for(count, 256), 256, 0, s>>>(idx, count, (u32)rows);
    LG_LAUNCH();
    int dev = 0, sms = 0;
    LG_CUDA(cudaGetDevice(&dev));
    LG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const unsigned grid =
        (unsigned)(sms * (blocks_per_sm > 0 ? blocks_per_sm : kPeakBlocksPerSM));
    auto launch = [&] {
      if (width == 4)
        k_peak_elems<float, 8><<<grid, kPeakThreads, 0, s>>>((const float *)tab, idx, count,
                                                             (float *)sink);
      else if (width == 8)
        k_peak_elems<double, 8><<<grid, kPeakThreads, 0, s>>>((const double *)tab, idx, count,
                                                              (double *)sink);
      else
        k_peak_rows<4><<<grid, kPeakThreads, 0, s>>>((const float4 *)tab, idx, count,
                                                     (float *)sink);
      LG_LAUNCH();
    };
    LG_CUDA(cudaEventCreate(&e0));
    LG_CUDA(cudaEventCreate(&e1));
    for (int r = 0; r < 3; r++) launch();
    constexpr int kReps = 5;
    LG_CUDA(cudaEventRecord(e0, s));
    for (int r = 0; r < kReps; r++) launch();
    LG_CUDA(cudaEventRecord(e1, s));
    LG_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    LG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    rate = (double)count * kReps / ((double)ms * 1e-3);
  } catch (...) {
    failed = true;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (tab) cudaFreeAsync(tab, s);
  if (sink) cudaFreeAsync(sink, s);
  if (idx) cudaFreeAsync(idx, s);
  cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  if (failed) throw Error(LIGMG_ERR_CUDA, "gather peak measurement");
  return rate;
}

}  // namespace lg
