// spmm_dev.cuh — device side of the row-parallel SpMM with fused epilogues,
// shared by the launched kernels (solve.cu) and the persistent coarse-tail
// kernel (tail.cu).
//
// SpMM layout: X is n x k row-major.  A row is processed by a group of G lanes
// (G = 32 for k > 1).  Inside a group, L = k / VW lanes cover the k columns of
// one matrix entry with 16-byte vector loads (VW = 4 floats or 2 doubles) and
// E = G / L entries are in flight per step; partial sums of the E entry slots
// are combined with warp shuffles and the first L lanes run the fused
// epilogue on their VW columns.  The matrix is read once per k vectors.
#pragma once
#include "solve.cuh"

namespace lg {
namespace dev {

template <typename T>
struct VT;
template <>
struct VT<float> {
  static constexpr int W = 4;
};
template <>
struct VT<double> {
  static constexpr int W = 2;
};

template <typename T, int VW>
__device__ __forceinline__ void vload(const T *p, T (&o)[VW]) {
  if constexpr (VW == 4 && sizeof(T) == 4) {
    float4 t = *reinterpret_cast<const float4 *>(p);
    o[0] = t.x; o[1] = t.y; o[2] = t.z; o[3] = t.w;
  } else if constexpr (VW == 2 && sizeof(T) == 8) {
    double2 t = *reinterpret_cast<const double2 *>(p);
    o[0] = t.x; o[1] = t.y;
  } else {
#pragma unroll
    for (int q = 0; q < VW; q++) o[q] = p[q];
  }
}
template <typename T, int VW>
__device__ __forceinline__ void vldg(const T *p, T (&o)[VW]) {
  if constexpr (VW == 4 && sizeof(T) == 4) {
    float4 t = __ldg(reinterpret_cast<const float4 *>(p));
    o[0] = t.x; o[1] = t.y; o[2] = t.z; o[3] = t.w;
  } else if constexpr (VW == 2 && sizeof(T) == 8) {
    double2 t = __ldg(reinterpret_cast<const double2 *>(p));
    o[0] = t.x; o[1] = t.y;
  } else {
#pragma unroll
    for (int q = 0; q < VW; q++) o[q] = __ldg(p + q);
  }
}
template <typename T, int VW>
__device__ __forceinline__ void vstore(T *p, const T (&o)[VW]) {
  if constexpr (VW == 4 && sizeof(T) == 4) {
    *reinterpret_cast<float4 *>(p) = make_float4(o[0], o[1], o[2], o[3]);
  } else if constexpr (VW == 2 && sizeof(T) == 8) {
    *reinterpret_cast<double2 *>(p) = make_double2(o[0], o[1]);
  } else {
#pragma unroll
    for (int q = 0; q < VW; q++) p[q] = o[q];
  }
}

// Four FP32 values (rows of one reduction group) combined in a fixed order.
__device__ __forceinline__ float sum4(const float (&x)[4]) {
  return (x[0] + x[1]) + (x[2] + x[3]);
}
__device__ __forceinline__ float dot4(const float (&x)[4], const float (&y)[4]) {
  return __fmaf_rn(x[3], y[3], __fmaf_rn(x[2], y[2], __fmaf_rn(x[1], y[1], x[0] * y[0])));
}

// matrix arrays: read-only cache loads from global memory (GX) or generic loads
template <bool GX, typename V>
__device__ __forceinline__ V mld(const V *p) {
  if constexpr (GX) return __ldg(p);
  else return *p;
}
template <typename T, int VW, bool GX>
__device__ __forceinline__ void xload(const T *p, T (&o)[VW]) {
  if constexpr (GX) vldg<T, VW>(p, o);
  else vload<T, VW>(p, o);
}

// an epilogue scalar in the data's type: FP32 epilogues take the float copy
// (no FP64 conversion per thread)
template <typename T>
__device__ __forceinline__ T escal(double d, float f) {
  if constexpr (sizeof(T) == 4) return f;
  else return (T)d;
}

template <typename T, int K, int VW, Epi E>
__device__ __forceinline__ void epilogue(const EpiArgs &a, i64 r, int c0, T (&acc)[VW]) {
  const i64 off = r * K + c0;
  if constexpr (E == Epi::Store || E == Epi::Split) {
    vstore<T, VW>((T *)a.y + off, acc);
  } else if constexpr (E == Epi::Resid) {
    T b[VW];
    vload<T, VW>((const T *)a.b + off, b);
#pragma unroll
    for (int q = 0; q < VW; q++) b[q] = b[q] - acc[q];
    vstore<T, VW>((T *)a.y + off, b);
  } else if constexpr (E == Epi::ChebA) {
    T b[VW], x[VW], d[VW];
    vload<T, VW>((const T *)a.b + off, b);
    vload<T, VW>((const T *)a.xin + off, x);
    const T ivt = ((const T *)a.invd)[r] * escal<T>(a.ith, a.fith);
#pragma unroll
    for (int q = 0; q < VW; q++) {
      b[q] = b[q] - acc[q];
      d[q] = ivt * b[q];
      x[q] = x[q] + d[q];
    }
    vstore<T, VW>((T *)a.rout + off, b);
    vstore<T, VW>((T *)a.dout + off, d);
    vstore<T, VW>((T *)a.xout + off, x);
  } else if constexpr (E == Epi::ChebB) {
    T rr[VW], d[VW], x[VW];
    vload<T, VW>((const T *)a.rin + off, rr);
    vload<T, VW>((const T *)a.din + off, d);
    vload<T, VW>((const T *)a.xin + off, x);
    const T iv = ((const T *)a.invd)[r];
    const T c1 = escal<T>(a.c1, a.fc1), c2 = escal<T>(a.c2, a.fc2);
#pragma unroll
    for (int q = 0; q < VW; q++) {
      rr[q] = rr[q] - acc[q];
      d[q] = c1 * d[q] + c2 * (iv * rr[q]);
      x[q] = x[q] + d[q];
    }
    if (a.rout) vstore<T, VW>((T *)a.rout + off, rr);
    if (a.dout) vstore<T, VW>((T *)a.dout + off, d);
    vstore<T, VW>((T *)a.xout + off, x);
  } else if constexpr (E == Epi::ChebZ) {
    T b[VW], d0[VW], d[VW], x[VW];
    vload<T, VW>((const T *)a.b + off, b);
    const T iv = ((const T *)a.invd)[r];
    const T ith = escal<T>(a.ith, a.fith), ivt = iv * ith;
    const T c1 = escal<T>(a.c1, a.fc1), c2 = escal<T>(a.c2, a.fc2);
#pragma unroll
    for (int q = 0; q < VW; q++) {
      d0[q] = ivt * b[q];
      b[q] = b[q] - acc[q] * ith;  // the residual after the first step
      d[q] = c1 * d0[q] + c2 * (iv * b[q]);
      x[q] = d0[q] + d[q];
    }
    if (a.rout) vstore<T, VW>((T *)a.rout + off, b);
    if (a.dout) vstore<T, VW>((T *)a.dout + off, d);
    vstore<T, VW>((T *)a.xout + off, x);
  } else if constexpr (E == Epi::FcgDir) {
    T z[VW], mu[VW], pv[VW], qv[VW];
    vload<T, VW>((const T *)a.xin + off, z);
    vload<T, VW>((const T *)a.cmu + c0, mu);
    const T rs = ((const T *)a.q)[r];
#pragma unroll
    for (int q = 0; q < VW; q++) {
      pv[q] = z[q] - mu[q];
      qv[q] = acc[q] - mu[q] * rs;
    }
    if (a.din) {
      T be[VW], pp[VW], qp[VW];
      vload<T, VW>((const T *)a.cbeta + c0, be);
      vload<T, VW>((const T *)a.din + off, pp);
      vload<T, VW>((const T *)a.rin + off, qp);
#pragma unroll
      for (int q = 0; q < VW; q++) {
        pv[q] = pv[q] - be[q] * pp[q];
        qv[q] = qv[q] - be[q] * qp[q];
      }
    }
    vstore<T, VW>((T *)a.dout + off, pv);
    vstore<T, VW>((T *)a.y + off, qv);
  } else if constexpr (E == Epi::ElimInterp) {
    T b[VW];
    vload<T, VW>((const T *)a.b + off, b);
    const T qd = ((const T *)a.q)[r];
#pragma unroll
    for (int q = 0; q < VW; q++) b[q] = acc[q] + qd * b[q];
    vstore<T, VW>((T *)a.y + off, b);
  } else {  // Jacobi: for a Laplacian, sum over negative entries = (A x)_i - a_ii x_i
    T b[VW], x[VW];
    vload<T, VW>((const T *)a.b + off, b);
    vload<T, VW>((const T *)a.xin + off, x);
    const T wi = escal<T>(a.c1, a.fc1) * ((const T *)a.invd)[r];
#pragma unroll
    for (int q = 0; q < VW; q++) x[q] = x[q] + wi * (b[q] - acc[q]);
    vstore<T, VW>((T *)a.y + off, x);
  }
}

// Row j of the gathered operand: X, or with SPLIT (Epi::Split) X for j <
// xsplit and x2 row j - xsplit otherwise.
template <typename T, int K, bool SPLIT>
__device__ __forceinline__ const T *xsrc(const MatView<T> &A, const T *X, i32 j) {
  if constexpr (SPLIT) {
    const bool lo = j < A.xsplit;
    return (lo ? X : A.x2) + (lo ? (i64)j : (i64)j - A.xsplit) * K;
  } else {
    return X + (i64)j * K;
  }
}

// GX: matrix and X in global memory (read-only cache loads); otherwise they
// may be staged in shared memory and are read with generic loads.
//
// A lane takes entries k, k + E, k + 2E, ... of [k, e), four per step, and
// loads the column indices of the next step before gathering this step's X
// rows, so a step waits for one dependent latency (the gather) instead of two
// (index, then gather).  Products are added in entry order.
//   GX (global memory): full steps are branch-free; the last entries (fewer
//     than four) go one at a time.
//   otherwise (shared memory, coarse levels with short rows): the last step
//     is masked (no gather, zero product past e), so no row pays a second
//     loop.
template <typename T, int K, int VW, int E, bool GX = true, bool SPLIT = false>
__device__ __forceinline__ void row_accumulate(const MatView<T> &A, const T *__restrict__ X, i64 k,
                                               i64 e, int ch, T (&acc)[VW]) {
  const T *__restrict__ av = A.v;
  const i32 *__restrict__ ac = A.ci;
  if constexpr (GX) {
    if (k + 3 * E < e) {
      i32 jn[4];
#pragma unroll
      for (int u = 0; u < 4; u++) jn[u] = mld<GX>(ac + k + u * E);
      while (true) {
        i32 j[4];
#pragma unroll
        for (int u = 0; u < 4; u++) j[u] = jn[u];
        const i64 kn = k + 4 * E;
        const bool more = kn + 3 * E < e;
        if (more) {
#pragma unroll
          for (int u = 0; u < 4; u++) jn[u] = mld<GX>(ac + kn + u * E);
        }
        T a[4], x[4][VW];
#pragma unroll
        for (int u = 0; u < 4; u++) {
          a[u] = mld<GX>(av + k + u * E);
          xload<T, VW, GX>(xsrc<T, K, SPLIT>(A, X, j[u]) + ch * VW, x[u]);
        }
#pragma unroll
        for (int u = 0; u < 4; u++)
#pragma unroll
          for (int q = 0; q < VW; q++) acc[q] += a[u] * x[u][q];
        k = kn;
        if (!more) break;
      }
    }
    for (; k < e; k += E) {
      T a0 = mld<GX>(av + k);
      i32 j0 = mld<GX>(ac + k);
      T x0[VW];
      xload<T, VW, GX>(xsrc<T, K, SPLIT>(A, X, j0) + ch * VW, x0);
#pragma unroll
      for (int q = 0; q < VW; q++) acc[q] += a0 * x0[q];
    }
  } else {
    if (k >= e) return;
    i32 jn[4];
#pragma unroll
    for (int u = 0; u < 4; u++) jn[u] = (k + u * E < e) ? mld<GX>(ac + k + u * E) : -1;
    while (true) {
      i32 j[4];
#pragma unroll
      for (int u = 0; u < 4; u++) j[u] = jn[u];
      const i64 kn = k + 4 * E;
      const bool more = kn < e;
      if (more) {
#pragma unroll
        for (int u = 0; u < 4; u++) jn[u] = (kn + u * E < e) ? mld<GX>(ac + kn + u * E) : -1;
      }
      T a[4], x[4][VW];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        if (j[u] >= 0) {
          a[u] = mld<GX>(av + k + u * E);
          xload<T, VW, GX>(xsrc<T, K, SPLIT>(A, X, j[u]) + ch * VW, x[u]);
        } else {
          a[u] = (T)0;
#pragma unroll
          for (int q = 0; q < VW; q++) x[u][q] = (T)0;
        }
      }
#pragma unroll
      for (int u = 0; u < 4; u++)
#pragma unroll
        for (int q = 0; q < VW; q++) acc[q] += a[u] * x[u][q];
      if (!more) break;
      k = kn;
    }
  }
}

template <typename T, int VW, int L, int G>
__device__ __forceinline__ void reduce_slots(T (&acc)[VW]) {
#pragma unroll
  for (int o = L; o < G; o <<= 1)
#pragma unroll
    for (int q = 0; q < VW; q++) acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], o);
}

// Hub chunk c of y = A X: the warp sums its chunk into a partial; the warp
// that completes a hub row's last chunk sums the chunk partials in a fixed
// order and runs the epilogue, so results do not depend on scheduling.
template <typename T, int K, Epi EP, bool GX = true>
__device__ __forceinline__ void hub_unit(const MatView<T> &A, const T *__restrict__ X,
                                         const EpiArgs &a, i64 c, int lane) {
  constexpr int G = 32;
  constexpr int VW = (K % VT<T>::W == 0) ? VT<T>::W : 1;
  constexpr int L = K / VW;
  constexpr int E = G / L;
  const int slot = lane / L, ch = lane % L;
  if (c >= A.nchunks) return;
  T acc[VW];
#pragma unroll
  for (int q = 0; q < VW; q++) acc[q] = (T)0;
  row_accumulate<T, K, VW, E, GX, EP == Epi::Split>(A, X, A.ch_beg[c] + slot, A.ch_end[c], ch, acc);
  reduce_slots<T, VW, L, G>(acc);
  if (slot == 0) vstore<T, VW>(A.partial + c * K + ch * VW, acc);
  __threadfence();
  __syncwarp();
  int last = 0;
  if (lane == 0) last = atomicAdd(&A.hub_counter[A.ch_hub[c]], 1) == A.ch_cnt[c] - 1;
  last = __shfl_sync(0xffffffffu, last, 0);
  if (!last) return;
  __threadfence();
  {
    // every slot sums a strided subset of the chunk partials; the slot
    // partials are combined in a fixed shuffle tree (deterministic)
    const i64 first = A.ch_first[c];
    const int cnt = A.ch_cnt[c];
    T s[VW];
#pragma unroll
    for (int q = 0; q < VW; q++) s[q] = (T)0;
#pragma unroll 4
    for (int t = slot; t < cnt; t += E) {
#pragma unroll
      for (int q = 0; q < VW; q++) s[q] += __ldcg(A.partial + (first + t) * K + ch * VW + q);
    }
    reduce_slots<T, VW, L, G>(s);
    if (slot == 0) epilogue<T, K, VW, EP>(a, A.ch_row[c], ch * VW, s);
  }
  if (lane == 0) A.hub_counter[A.ch_hub[c]] = 0;
}

// One warp's share of y = A X with a fused epilogue: a regular row (or RPW
// rows) for warp < ceil(n / RPW), else hub chunk warp - ceil(n / RPW).
template <typename T, int K, int G, Epi EP, bool GX = true>
__device__ __forceinline__ void spmm_unit(const MatView<T> &A, const T *__restrict__ X,
                                          const EpiArgs &a, i64 warp, int lane) {
  constexpr int VW = (K % VT<T>::W == 0) ? VT<T>::W : 1;
  constexpr int L = K / VW;
  static_assert(L <= G && G <= 32 && (G % L) == 0, "bad SpMM layout");
  constexpr int E = G / L;
  constexpr int RPW = 32 / G;
  const int g = lane % G, slot = g / L, ch = g % L;
  const i64 nregw = (A.n + RPW - 1) / RPW;
  if (warp < nregw) {
    T acc[VW];
#pragma unroll
    for (int q = 0; q < VW; q++) acc[q] = (T)0;
    const i64 r = warp * RPW + lane / G;
    bool act = r < A.n;
    i64 b = 0, e = 0;
    if (act) {
      b = A.rp[r];
      e = A.rp[r + 1];
      if (A.hub_thresh > 0 && e - b > A.hub_thresh) act = false;
    }
    if (act) row_accumulate<T, K, VW, E, GX, EP == Epi::Split>(A, X, b + slot, e, ch, acc);
    reduce_slots<T, VW, L, G>(acc);
    if (act && slot == 0) epilogue<T, K, VW, EP>(a, r, ch * VW, acc);
    return;
  }
  if constexpr (G == 32) hub_unit<T, K, EP, GX>(A, X, a, warp - nregw, lane);
}

}  // namespace dev
}  // namespace lg
