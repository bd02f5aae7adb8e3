// tail.cu — persistent kernel executing the recorded coarse-tail program.
//
// Two modes.
// Grid mode: all G CTAs are resident (cooperative launch) and cooperate on
//   every operation; operations run in program order with a grid barrier
//   between two operations, so an operation sees all writes of the previous
//   ones.
// Shared-memory mode: the columns of the k right-hand sides are independent
//   through the whole cycle, so CTA g alone runs the program on columns
//   [g*KL, (g+1)*KL): its slice of every work vector, a copy of the program
//   and of every read-only array the program reads live in its shared memory;
//   only block barriers are needed.  The start level's input slice is staged
//   in at the beginning and its output slice written back at the end.
// Work inside an operation (cooperating CTAs c = 0..C-1):
//   Spmm        warp units (rows, then hub chunks) strided over the C*32
//               warps, the same per-warp code as the launched SpMM
//   elementwise n*KL elements strided over all C*NT threads
//   RedBeta/RedAlpha  CTA c reduces rows [c*rpc, (c+1)*rpc) into partial[c]
//   Dir/Update  every CTA sums the C partials in the same fixed order (so all
//               hold identical scalars), CTA 0 publishes them, and the
//               elementwise update follows without another barrier.
#include "spmm_dev.cuh"
#include "tail.cuh"

namespace lg {
namespace {

using namespace dev;

constexpr long long kBarrierSpins = 1ll << 23;  // default limit: ~0.3 s at 32 ns a spin

// Returns false when the barrier gave up (error recorded) or another CTA
// reported an error: the caller leaves the kernel.
__device__ __forceinline__ bool grid_barrier(TailSync *gs, int *sh_abort, int ncta) {
  __syncthreads();
  if (ncta == 1) return true;  // one cooperating CTA: the block barrier orders everything
  if (threadIdx.x == 0) {
    const unsigned add = blockIdx.x == 0 ? 0x80000000u - (gridDim.x - 1) : 1u;
    __threadfence();
    const unsigned old = atomicAdd(&gs->arrive, add);
    volatile unsigned *av = &gs->arrive;
    volatile int *ev = &gs->err;
    long long spins = 0;
    const long long limit = gs->limit > 0 ? gs->limit : kBarrierSpins;
    int abort = 0;
    while (((old ^ *av) & 0x80000000u) == 0) {
      if (*ev) { abort = 1; break; }
      if (++spins >= limit) {  // `limit` polls of an incomplete barrier
        atomicExch(&gs->err, 1);
        abort = 1;
        break;
      }
      __nanosleep(32);
    }
    __threadfence();
    if (!abort && *ev) abort = 1;
    *sh_abort = abort;
  }
  __syncthreads();
  return *sh_abort == 0;
}

// Shared-memory mode: the host tags pointers into the launch's dynamic shared
// memory as kSmemTag | byte offset.
extern __shared__ __align__(16) unsigned char tail_smem[];

template <bool SM, typename P>
__device__ __forceinline__ P *res(P *p) {
  if constexpr (SM) {
    const unsigned long long u = (unsigned long long)p;
    if ((u & ~kSmemOffMask) == kSmemTag) return (P *)(tail_smem + (u & kSmemOffMask));
  }
  return p;
}

// part / nparts (cluster mode): this CTA's share of the units, whose rows
// [*rbeg, *rend) it computes; otherwise part = 0, nparts = 1.
// ---- cluster mode (shared-memory mode launched as clusters of CTAs) --------
// A column slice is run by a cluster: every CTA holds the whole program and
// full copies of the slice's work vectors in its shared memory and runs every
// operation itself (identical inputs, identical order: identical results),
// except the products with a matrix left in global memory (the larger
// levels', too large for shared memory): their rows are divided among the
// cluster's CTAs; each CTA computes its rows into its own copies, the cluster
// meets at a hardware barrier (every CTA is past the earlier operations,
// which may read the old values), each CTA writes its rows into every peer's
// copies (distributed shared memory) and the cluster meets again.  CTAs run
// ahead of one another only between these products.
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\t"
               "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ unsigned cluster_size() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void st_peer(unsigned local, unsigned rank, float v) {
  unsigned ra;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(local), "r"(rank));
  asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(ra), "f"(v) : "memory");
}
__device__ __forceinline__ void st_peer(unsigned local, unsigned rank, double v) {
  unsigned ra;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(local), "r"(rank));
  asm volatile("st.shared::cluster.f64 [%0], %1;" ::"r"(ra), "d"(v) : "memory");
}
// rows [r0, r1) of a shared-memory vector (n x K) into every peer's copy
template <typename T, int K, int NT>
__device__ void cluster_push(const void *tagged, i64 r0, i64 r1, unsigned me, unsigned cs) {
  const unsigned long long u = (unsigned long long)tagged;
  if (!tagged || (u & ~kSmemOffMask) != kSmemTag) return;
  const T *v = reinterpret_cast<const T *>(tail_smem + (u & kSmemOffMask));
  const unsigned base = (unsigned)__cvta_generic_to_shared(v);
  for (i64 t = r0 * K + threadIdx.x; t < r1 * K; t += NT) {
    const T x = v[t];
    for (unsigned p = 0; p < cs; p++)
      if (p != me) st_peer(base + (unsigned)(t * (i64)sizeof(T)), p, x);
  }
}
template <typename P>
__device__ __forceinline__ bool is_global(const P *p) {
  return ((unsigned long long)p & ~kSmemOffMask) != kSmemTag;
}

template <typename T, int K, bool SM>
__device__ void run_spmm(const TOp<T> &op, i64 gwarp, i64 nwarps, int lane, int part = 0,
                         int nparts = 1, i64 *rbeg = nullptr, i64 *rend = nullptr) {
  const i64 units = op.A.n + op.A.nchunks;
  EpiArgs a = op.a;
  MatView<T> A = op.A;
  const T *X = res<SM>(op.x0);
  if constexpr (SM) {
    A.rp = res<SM>(A.rp);
    A.ci = res<SM>(A.ci);
    A.v = res<SM>(A.v);
    A.x2 = res<SM>(A.x2);
    a.invd = res<SM>(a.invd);
    a.q = res<SM>(a.q);
    a.y = res<SM>(a.y);
    a.b = res<SM>(a.b);
    a.xin = res<SM>(a.xin);
    a.xout = res<SM>(a.xout);
    a.rin = res<SM>(a.rin);
    a.rout = res<SM>(a.rout);
    a.din = res<SM>(a.din);
    a.dout = res<SM>(a.dout);
  }
  // Shared-memory mode (whole rows, no chunks): when a row averages at most
  // two unrolled steps of an 8-lane group, 8 lanes take each row and a warp
  // works on four rows at once; a warp of 32 lanes would walk the level's
  // short rows one by one, each ending in a five-level shuffle reduction.
  constexpr int VW = (K % VT<T>::W == 0) ? VT<T>::W : 1;
  constexpr int L = K / VW;
  bool narrow = false;
  if constexpr (SM && L <= 8) narrow = (A.rp[A.n] - A.rp[0]) * L <= (i64)64 * A.n;
  const i64 units8 = (A.n + 3) / 4;
  // this part's units: [u0, u1) of `units` (or of units8, four rows each)
  const i64 nu = narrow ? units8 : units;
  const i64 u0 = nu * part / nparts, u1 = nu * (part + 1) / nparts;
  if (rbeg) {
    *rbeg = narrow ? min(u0 * 4, A.n) : min(u0, A.n);
    *rend = narrow ? min(u1 * 4, A.n) : min(u1, A.n);
  }
  switch (op.epi) {
#define LG_TAIL_EPI(E)                                                        \
  case E:                                                                     \
    if constexpr (SM && L <= 8) {                                             \
      if (narrow) {                                                           \
        for (i64 u = u0 + gwarp; u < u1; u += nwarps)                         \
          spmm_unit<T, K, 8, E, !SM>(A, X, a, u, lane);                       \
        break;                                                                \
      }                                                                       \
    }                                                                         \
    for (i64 u = u0 + gwarp; u < u1; u += nwarps)                             \
      spmm_unit<T, K, 32, E, !SM>(A, X, a, u, lane);                          \
    break;
    LG_TAIL_EPI(Epi::Store)
    LG_TAIL_EPI(Epi::Resid)
    LG_TAIL_EPI(Epi::ChebA)
    LG_TAIL_EPI(Epi::ChebB)
    LG_TAIL_EPI(Epi::ElimInterp)
    LG_TAIL_EPI(Epi::Jacobi)
    LG_TAIL_EPI(Epi::Split)
    LG_TAIL_EPI(Epi::ChebZ)
#undef LG_TAIL_EPI
    default:  // Epi::FcgDir: the tail program keeps direction and product apart
      break;
  }
}

// Partial sums over cooperating CTA `cta`'s row range: NV values per column.
// One cooperating CTA: the totals stay in sh[v][c < K] for the next operation.
template <typename T, int K, int NV, int NT>
__device__ void block_partials(const T *x, const T *y, const T *w, bool use_y, i64 n, int cta,
                               int ncta, double *partial, double (*sh)[NT]) {
  const int tid = threadIdx.x;
  constexpr int RS = NT / K;
  const int c = tid % K, rsub = tid / K;
  const i64 rpc = (n + ncta - 1) / ncta;
  const i64 r0 = (i64)cta * rpc, r1 = min(n, r0 + rpc);
  double a[NV];
#pragma unroll
  for (int v = 0; v < NV; v++) a[v] = 0;
  if constexpr (sizeof(T) == 4) {
    // four rows per step combined in FP32, one FP64 add per group (as in the
    // launched reductions)
    for (i64 r = r0 + rsub; r < r1; r += 4 * (i64)RS) {
      float xv[4], yv[4], wv[4];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const i64 rr = r + (i64)u * RS;
        const bool ok = rr < r1;
        const i64 o = rr * K + c;
        xv[u] = ok ? x[o] : 0.f;
        yv[u] = (ok && use_y) ? y[o] : 0.f;
        wv[u] = (NV == 2 && ok) ? w[o] : 0.f;
      }
      if constexpr (NV == 3) {
        a[0] += (double)sum4(xv);
        if (use_y) {
          a[1] += (double)dot4(xv, yv);
          a[2] += (double)sum4(yv);
        }
      } else {
        a[0] += (double)dot4(xv, yv);
        a[1] += (double)dot4(xv, wv);
      }
    }
  } else {
    for (i64 r = r0 + rsub; r < r1; r += RS) {
      const i64 o = r * K + c;
      const double xv = (double)x[o];
      if constexpr (NV == 3) {  // sum z, z.qp, sum qp
        a[0] += xv;
        if (use_y) {
          const double yv = (double)y[o];
          a[1] += xv * yv;
          a[2] += yv;
        }
      } else {  // p.q, p.r
        a[0] += xv * (double)y[o];
        a[1] += xv * (double)w[o];
      }
    }
  }
#pragma unroll
  for (int v = 0; v < NV; v++) sh[v][tid] = a[v];
  __syncthreads();
  for (int st = NT / 2; st >= K; st >>= 1) {
    if (tid < st)
#pragma unroll
      for (int v = 0; v < NV; v++) sh[v][tid] += sh[v][tid + st];
    __syncthreads();
  }
  if (ncta > 1 && tid < K)
#pragma unroll
    for (int v = 0; v < NV; v++) partial[((i64)cta * 3 + v) * K + tid] = sh[v][tid];
}

// Sum of the cooperating CTAs' partials (fixed order, identical in every
// CTA) into sh[v][c] for c < K.
template <int K, int NV, int NT>
__device__ void finish_partials(const double *partial, int ncta, double (*sh)[NT]) {
  if (ncta == 1) return;  // totals left in sh by block_partials
  const int tid = threadIdx.x;
  constexpr int RS = NT / K;
  const int c = tid % K, rsub = tid / K;
  double a[NV];
#pragma unroll
  for (int v = 0; v < NV; v++) a[v] = 0;
  for (int b = rsub; b < ncta; b += RS)
#pragma unroll
    for (int v = 0; v < NV; v++) a[v] += __ldcg(partial + ((i64)b * 3 + v) * K + c);
  __syncthreads();
#pragma unroll
  for (int v = 0; v < NV; v++) sh[v][tid] = a[v];
  __syncthreads();
  for (int st = NT / 2; st >= K; st >>= 1) {
    if (tid < st)
#pragma unroll
      for (int v = 0; v < NV; v++) sh[v][tid] += sh[v][tid + st];
    __syncthreads();
  }
}

// Interface of a shared-memory launch: the start level's input and output
// (n x kg, global) and their slices' offsets in shared memory (n x K).
template <typename T>
struct TailIO {
  const T *gin;
  T *gout;
  i64 n;
  int kg;
  unsigned in_off, out_off;
};

// NT threads per CTA: 1024 in grid mode; 256 in shared-memory mode, where an
// operation has little work and every warp pays its preamble (reading the
// record, resolving its pointers).
template <typename T, int K, bool SM, int NT>
__global__ void __launch_bounds__(NT, 1)
    k_tail(const TOp<T> *__restrict__ ops, int nops, double *partial, TailSync *gs,
           const uint4 *__restrict__ image, int image_vec, TailIO<T> io) {
  static_assert(NT % K == 0 && NT >= 64, "tail block size");
  dep_prologue();
  __shared__ double sh[3][NT];
  __shared__ T scal[2][64];  // column scalars in the data's type (converted once)
  __shared__ int sh_abort;
  // cooperating CTAs: all of them (grid mode) or this one (shared-memory mode)
  const int cta = SM ? 0 : (int)blockIdx.x;
  const int ncta = SM ? 1 : (int)gridDim.x;
  // cluster mode: this CTA's rank in its cluster and the cluster's size (1:
  // a plain shared-memory launch); a cluster runs one column slice
  unsigned crank = 0, csize = 1;
  if constexpr (SM) {
    crank = cluster_rank();
    csize = cluster_size();
  }
  const int slice = (int)(blockIdx.x / csize);
  if constexpr (SM) {
    // stage the program, the read-only arrays and this CTA's column slice of
    // the start level's input
    uint4 *dst = reinterpret_cast<uint4 *>(tail_smem);
    for (int w = threadIdx.x; w < image_vec; w += NT) dst[w] = __ldg(image + w);
    T *sin = reinterpret_cast<T *>(tail_smem + io.in_off);
    const int c0 = slice * K;
    for (i64 t = threadIdx.x; t < io.n * K; t += NT)
      sin[t] = io.gin[(t / K) * io.kg + c0 + (t % K)];
    __syncthreads();
    ops = reinterpret_cast<const TOp<T> *>(tail_smem);
    if (csize > 1) cluster_sync_all();  // every peer started before any remote store
  }
  const int lane = threadIdx.x & 31;
  const i64 gwarp = ((i64)cta * NT + threadIdx.x) >> 5;
  const i64 nwarps = (i64)ncta * (NT / 32);
  const i64 gthr = (i64)cta * NT + threadIdx.x;
  const i64 nthr = (i64)ncta * NT;
  for (int i = 0; i < nops; i++) {
    const TOp<T> &op = ops[i];
    const i64 nk = op.n * K;
    const T *x0 = res<SM>(op.x0), *x1 = res<SM>(op.x1), *x2 = res<SM>(op.x2);
    T *y0 = res<SM>(op.y0), *y1 = res<SM>(op.y1);
    const i32 *idx = res<SM>(op.idx);
    FcgScalars sc = op.sc;
    if constexpr (SM) {
      sc.mu = res<SM>(sc.mu);
      sc.beta = res<SM>(sc.beta);
      sc.eta = res<SM>(sc.eta);
      sc.eta_prev = res<SM>(sc.eta_prev);
      sc.alpha = res<SM>(sc.alpha);
    }
    switch (op.kind) {
      case TOpKind::Spmm:
        if (SM && csize > 1 && is_global(op.A.rp)) {
          // own rows into this CTA's copies; then, once every peer has
          // finished the operations before this one (a peer may still read
          // the old values of these outputs there), into the peers' copies
          i64 r0 = 0, r1 = 0;
          run_spmm<T, K, SM>(op, gwarp, nwarps, lane, (int)crank, (int)csize, &r0, &r1);
          __syncthreads();
          cluster_sync_all();
          cluster_push<T, K, NT>(op.a.y, r0, r1, crank, csize);
          cluster_push<T, K, NT>(op.a.rout, r0, r1, crank, csize);
          cluster_push<T, K, NT>(op.a.dout, r0, r1, crank, csize);
          cluster_push<T, K, NT>(op.a.xout, r0, r1, crank, csize);
          cluster_sync_all();
        } else {
          run_spmm<T, K, SM>(op, gwarp, nwarps, lane);
        }
        break;
      case TOpKind::Cheb0: {
        const T f = (T)op.f;
        for (i64 t = gthr; t < nk; t += nthr) y0[t] = (x1[t / K] * f) * x0[t];
        break;
      }
      case TOpKind::Prolong:
        for (i64 t = gthr; t < nk; t += nthr) y0[t] += x0[(i64)idx[t / K] * K + (t % K)];
        break;
      case TOpKind::Coarse:
        for (i64 t = gthr; t < nk; t += nthr) {
          const i64 r = t / K;
          const int c = (int)(t % K);
          T s = 0;
          for (i64 j = 0; j < op.n; j++) s += x1[r * op.n + j] * x0[j * K + c];
          y0[t] = s;
        }
        break;
      case TOpKind::Scale: {
        const T f = (T)op.f;
        for (i64 t = gthr; t < nk; t += nthr) y0[t] = y0[t] * f;
        break;
      }
      case TOpKind::Zero:
        for (i64 t = gthr; t < nk; t += nthr) y0[t] = (T)0;
        break;
      case TOpKind::Copy:
        for (i64 t = gthr; t < nk; t += nthr) y0[t] = x0[t];
        break;
      case TOpKind::RedBeta:
        block_partials<T, K, 3, NT>(x0, x1, nullptr, op.flag != 0, op.n, cta, ncta, partial, sh);
        break;
      case TOpKind::RedAlpha:
        block_partials<T, K, 2, NT>(x0, x1, x2, true, op.n, cta, ncta, partial, sh);
        break;
      case TOpKind::Dir: {
        finish_partials<K, 3, NT>(partial, ncta, sh);
        if (threadIdx.x < K) {
          const int c = threadIdx.x;
          const double mu = sh[0][c] / (double)op.n;
          double beta = 0.0;
          if (op.flag) {
            const double e = sc.eta_prev[c];
            beta = e == 0.0 ? 0.0 : (sh[1][c] - mu * sh[2][c]) / e;
          }
          scal[0][c] = (T)mu;
          scal[1][c] = (T)beta;
          if (cta == 0) {
            sc.mu[c] = mu;
            sc.beta[c] = beta;
          }
        }
        __syncthreads();
        for (i64 t = gthr; t < nk; t += nthr) {
          const int c = (int)(t % K);
          T v = x0[t] - scal[0][c];
          if (op.flag) v = v - scal[1][c] * x1[t];
          y0[t] = v;
        }
        break;
      }
      case TOpKind::Update: {
        finish_partials<K, 2, NT>(partial, ncta, sh);
        if (threadIdx.x < K) {
          const int c = threadIdx.x;
          const double eta = sh[0][c];
          const double alpha = eta == 0.0 ? 0.0 : sh[1][c] / eta;
          scal[0][c] = (T)alpha;
          if (cta == 0) {
            sc.eta[c] = eta;
            sc.alpha[c] = alpha;
          }
        }
        __syncthreads();
        for (i64 t = gthr; t < nk; t += nthr) {
          const T a = scal[0][(int)(t % K)];
          y0[t] = y0[t] + a * x0[t];
          if (op.flag) y1[t] = y1[t] - a * x1[t];
        }
        break;
      }
    }
    if (!grid_barrier(gs, &sh_abort, ncta)) return;
  }
  if constexpr (SM) {  // write this CTA's column slice of the output back
    const T *sout = reinterpret_cast<const T *>(tail_smem + io.out_off);
    const int c0 = slice * K;
    if (crank == 0)
      for (i64 t = threadIdx.x; t < io.n * K; t += NT)
        io.gout[(t / K) * io.kg + c0 + (t % K)] = sout[t];
    if (csize > 1) cluster_sync_all();  // no peer leaves while stores may target it
  }
}

template <typename T, int K>
void launch_grid(const TOp<T> *ops, int nops, int G, double *partial, TailSync *sync,
                 cudaStream_t s) {
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)G);
  cfg.blockDim = dim3(kTailThreads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  TailIO<T> io{};
  LG_CUDA(cudaLaunchKernelEx(&cfg, k_tail<T, K, false, kTailThreads>, ops, nops, partial, sync,
                             (const uint4 *)nullptr, 0, io));
  LG_LAUNCH();
}

template <typename T, int KL>
void launch_smem(const TailSmemLaunch &L, int k, TailSync *sync, cudaStream_t s) {
  TailIO<T> io{(const T *)L.gin, (T *)L.gout, L.n, k, L.in_off, L.out_off};
  if (L.cluster > 1) {
    if (L.cluster > 8)
      LG_CUDA(cudaFuncSetAttribute(k_tail<T, KL, true, kTailSmemThreads>,
                                   cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)L.cluster;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(k / KL * L.cluster));
    cfg.blockDim = dim3(kTailSmemThreads);
    cfg.dynamicSmemBytes = (size_t)L.smem;
    cfg.stream = s;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    LG_CUDA(cudaLaunchKernelEx(&cfg, k_tail<T, KL, true, kTailSmemThreads>,
                               (const TOp<T> *)nullptr, L.nops, (double *)nullptr, sync,
                               (const uint4 *)L.image, L.image_bytes / 16, io));
  } else {
    launch_dep(k_tail<T, KL, true, kTailSmemThreads>, k / KL, kTailSmemThreads, (size_t)L.smem, s,
               (const TOp<T> *)nullptr, L.nops, (double *)nullptr, sync, (const uint4 *)L.image,
               L.image_bytes / 16, io);
  }
  LG_LAUNCH();
}

template <typename T, int KL>
bool cluster_ok_k(int cl, int smem) {
  if (cl > 8)
    LG_CUDA(cudaFuncSetAttribute(k_tail<T, KL, true, kTailSmemThreads>,
                                 cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)cl;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)cl);
  cfg.blockDim = dim3(kTailSmemThreads);
  cfg.dynamicSmemBytes = (size_t)smem;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, k_tail<T, KL, true, kTailSmemThreads>, &cfg) !=
      cudaSuccess) {
    cudaGetLastError();  // not launchable in this shape: clear the error
    return false;
  }
  return n > 0;
}

template <typename T, int K>
int max_ctas_k() {
  int dev = 0, sms = 0, per = 0;
  LG_CUDA(cudaGetDevice(&dev));
  LG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  LG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_tail<T, K, false, kTailThreads>,
                                                        kTailThreads, 0));
  return per * sms;
}

template <typename T, int KL>
int smem_limit_k(int want) {
  int dev = 0, optin = 0;
  LG_CUDA(cudaGetDevice(&dev));
  LG_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  cudaFuncAttributes fa{};
  LG_CUDA(cudaFuncGetAttributes(&fa, k_tail<T, KL, true, kTailSmemThreads>));
  const int avail = optin - (int)fa.sharedSizeBytes;
  // the opt-in is a property of the kernel, shared by every handle of the
  // process: it only grows, so a launch prepared by one handle stays valid
  // after another handle prepares a smaller one
  static int opted = 0;
  if (want > opted && want <= avail) {
    LG_CUDA(cudaFuncSetAttribute(k_tail<T, KL, true, kTailSmemThreads>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, want));
    opted = want;
  }
  return avail;
}

}  // namespace

template <typename T>
void launch_tail_grid(const TOp<T> *ops, int nops, int k, int G, double *partial,
                      TailSync *sync, cudaStream_t s) {
  switch (k) {
    case 1: return launch_grid<T, 1>(ops, nops, G, partial, sync, s);
    case 8: return launch_grid<T, 8>(ops, nops, G, partial, sync, s);
    case 16: return launch_grid<T, 16>(ops, nops, G, partial, sync, s);
    case 32: return launch_grid<T, 32>(ops, nops, G, partial, sync, s);
    default: throw Error(LIGMG_ERR_UNSUPPORTED, "tail program: k must be 1, 8, 16 or 32");
  }
}

template <typename T>
void launch_tail_smem(const TailSmemLaunch &L, int k, TailSync *sync, cudaStream_t s) {
  if (L.kl <= 0 || k % L.kl != 0) throw Error(LIGMG_ERR_INTERNAL, "tail column slice");
  switch (L.kl) {
    case 1: return launch_smem<T, 1>(L, k, sync, s);
    case 4: return launch_smem<T, 4>(L, k, sync, s);
    case 8: return launch_smem<T, 8>(L, k, sync, s);
    default: throw Error(LIGMG_ERR_UNSUPPORTED, "tail program: columns per CTA must be 1, 4 or 8");
  }
}

template <typename T>
bool tail_cluster_ok(int kl, int cl, int smem) {
  switch (kl) {
    case 1: return cluster_ok_k<T, 1>(cl, smem);
    case 4: return cluster_ok_k<T, 4>(cl, smem);
    case 8: return cluster_ok_k<T, 8>(cl, smem);
    default: return false;
  }
}

template <typename T>
int tail_max_ctas(int k) {
  switch (k) {
    case 1: return max_ctas_k<T, 1>();
    case 8: return max_ctas_k<T, 8>();
    case 16: return max_ctas_k<T, 16>();
    case 32: return max_ctas_k<T, 32>();
    default: return 0;
  }
}

template <typename T>
int tail_smem_prepare(int kl, int bytes) {
  switch (kl) {
    case 1: return smem_limit_k<T, 1>(bytes);
    case 4: return smem_limit_k<T, 4>(bytes);
    case 8: return smem_limit_k<T, 8>(bytes);
    default: return 0;
  }
}

template void launch_tail_grid<float>(const TOp<float> *, int, int, int, double *, TailSync *,
                                      cudaStream_t);
template void launch_tail_grid<double>(const TOp<double> *, int, int, int, double *,
                                       TailSync *, cudaStream_t);
template void launch_tail_smem<float>(const TailSmemLaunch &, int, TailSync *, cudaStream_t);
template void launch_tail_smem<double>(const TailSmemLaunch &, int, TailSync *, cudaStream_t);
template int tail_max_ctas<float>(int);
template int tail_max_ctas<double>(int);
template int tail_smem_prepare<float>(int, int);
template bool tail_cluster_ok<float>(int, int, int);
template bool tail_cluster_ok<double>(int, int, int);
template int tail_smem_prepare<double>(int, int);

}  // namespace lg
