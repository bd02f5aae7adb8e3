// common.cuh — shared host/device helpers of the GB300 LigMG library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <stdexcept>
#include <utility>
#include <string>
#include <vector>

#include "../../include/ligmg_gpu.h"

namespace lg {

using i64 = int64_t;
using i32 = int32_t;
using u32 = uint32_t;
using u64 = uint64_t;

// Internal errors carry a ligmg_status and are converted at the C ABI.
struct Error : std::runtime_error {
  ligmg_status status;
  Error(ligmg_status s, const std::string &m) : std::runtime_error(m), status(s) {}
};

inline void cuda_check(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return;
  (void)cudaGetLastError();  // clear a non-sticky error so later calls start clean
  if (e == cudaErrorMemoryAllocation)
    throw Error(LIGMG_ERR_OUT_OF_MEMORY, std::string(what) + ": " + cudaGetErrorString(e));
  throw Error(LIGMG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
// kernels launched by the library (every launch site calls LG_LAUNCH once;
// a launch recorded into a CUDA graph is taken back out at capture and
// counted again on every replay of the graph)
extern int64_t g_launches;
inline int64_t launches_now() { return __atomic_load_n(&g_launches, __ATOMIC_RELAXED); }
inline void add_launches(int64_t d) { __atomic_fetch_add(&g_launches, d, __ATOMIC_RELAXED); }
#define LG_CUDA(x) ::lg::cuda_check((x), #x)
#define LG_LAUNCH()                                             \
  do {                                                          \
    __atomic_fetch_add(&::lg::g_launches, 1, __ATOMIC_RELAXED); \
    ::lg::cuda_check(cudaGetLastError(), "kernel launch");      \
  } while (0)

// While set (by SyncFreeScope, in this thread), DBuf::release frees with a
// synchronous cudaFree instead of a free ordered on the buffer's stream.
extern thread_local bool g_free_sync;
struct SyncFreeScope {
  bool prev;
  SyncFreeScope() : prev(g_free_sync) { g_free_sync = true; }
  ~SyncFreeScope() { g_free_sync = prev; }
};

constexpr int kSMs = 152;  // GB300: 2 dies x 76 SMs

// ---- programmatic dependent launch (the solve's kernels) -------------------
// A kernel launched with launch_dep may be scheduled while the kernel before
// it on the stream is still running; it first waits (griddepcontrol.wait)
// until that kernel has completed and its writes are visible, so only its
// launch latency overlaps.  A grid releases its dependents at its own start
// only when it is small (at most 1024 threads per SM): the dependents'
// waiting blocks are then resident beside it and never take the slots a
// later wave of a large grid would need.  Every kernel launched through
// launch_dep calls dep_prologue() before its first memory access.
constexpr long long kDepMaxThreads = (long long)kSMs * 1024;
__device__ __forceinline__ void dep_prologue() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  if ((long long)gridDim.x * gridDim.y * gridDim.z * blockDim.x * blockDim.y * blockDim.z <=
      kDepMaxThreads)
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
// Set (in this thread) while a handle with options.pdl solves.
extern thread_local bool g_dep_launch;
struct DepLaunchScope {
  bool prev;
  explicit DepLaunchScope(bool on) : prev(g_dep_launch) { g_dep_launch = on; }
  ~DepLaunchScope() { g_dep_launch = prev; }
};
template <typename... KArgs, typename... Args>
inline void launch_dep(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem,
                       cudaStream_t s, Args &&...args) {
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = g_dep_launch ? 1 : 0;
  const cudaError_t e = cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    throw Error(LIGMG_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  }
}

inline i64 cdiv(i64 a, i64 b) { return (a + b - 1) / b; }
inline unsigned grid_for(i64 work, int per_block) {
  i64 g = cdiv(work, per_block);
  if (g < 1) g = 1;
  if (g > 0x7fffffff) g = 0x7fffffff;
  return (unsigned)g;
}

// Stream-ordered device allocation.  Every buffer of a handle comes from
// here so that the handle's destructor releases exactly what it owns.
template <typename T>
struct DBuf {
  T *p = nullptr;
  i64 n = 0;
  cudaStream_t s = 0;
  DBuf() = default;
  DBuf(i64 count, cudaStream_t st) { alloc(count, st); }
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  DBuf(DBuf &&o) noexcept : p(o.p), n(o.n), s(o.s) { o.p = nullptr; o.n = 0; }
  DBuf &operator=(DBuf &&o) noexcept {
    if (this != &o) {
      release();
      p = o.p; n = o.n; s = o.s;
      o.p = nullptr; o.n = 0;
    }
    return *this;
  }
  ~DBuf() { release(); }
  void alloc(i64 count, cudaStream_t st) {
    release();
    s = st;
    n = count;
    if (count > 0) LG_CUDA(cudaMallocAsync((void **)&p, sizeof(T) * (size_t)count, st));
  }
  void release() {
    if (p) {
      if (g_free_sync) cudaFree(p);
      else cudaFreeAsync(p, s);
    }
    p = nullptr;
    n = 0;
  }
  void zero() {
    if (n) LG_CUDA(cudaMemsetAsync(p, 0, sizeof(T) * (size_t)n, s));
  }
  void upload(const T *h, i64 count) {
    LG_CUDA(cudaMemcpyAsync(p, h, sizeof(T) * (size_t)count, cudaMemcpyHostToDevice, s));
  }
  void download(T *h, i64 count) const {
    LG_CUDA(cudaMemcpyAsync(h, p, sizeof(T) * (size_t)count, cudaMemcpyDeviceToHost, s));
  }
  std::vector<T> to_host() const {
    std::vector<T> v((size_t)n);
    if (n) {
      download(v.data(), n);
      LG_CUDA(cudaStreamSynchronize(s));
    }
    return v;
  }
};

template <typename T>
inline T read_scalar(const T *dptr, cudaStream_t s) {
  T v;
  LG_CUDA(cudaMemcpyAsync(&v, dptr, sizeof(T), cudaMemcpyDeviceToHost, s));
  LG_CUDA(cudaStreamSynchronize(s));
  return v;
}

// Device CSR matrix (int64 row pointers, int32 columns ascending per row).
template <typename V>
struct DCsr {
  i64 n = 0, m = 0, nnz = 0;
  DBuf<i64> rp;
  DBuf<i32> ci;
  DBuf<V> v;
};

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31; }
__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

}  // namespace lg
