// tail.cu — persistent kernel executing the recorded coarse-tail program.
//
// All G CTAs are resident (cooperative launch).  Operations run in program
// order; between two operations every CTA passes a grid barrier, so an
// operation sees all writes of the previous ones.  Work inside an operation:
//   Spmm       warp units (rows, then hub chunks) strided over the G*32 warps,
//              the same per-warp code as the launched SpMM (spmm_dev.cuh)
//   elementwise  n*k elements strided over all G*1024 threads
//   RedBeta/RedAlpha  CTA c reduces rows [c*rpc, (c+1)*rpc) into partial[c]
//   Dir/Update       every CTA sums the G partials in the same fixed order
//              (so all CTAs hold identical scalars), CTA 0 publishes them, and
//              the elementwise update follows without another barrier.
#include "spmm_dev.cuh"
#include "tail.cuh"

namespace lg {
namespace {

using namespace dev;

constexpr long long kBarrierSpins = 1ll << 23;  // ~0.3 s at 32 ns a spin

// Returns false when the barrier gave up (error recorded) or another CTA
// reported an error: the caller leaves the kernel.
__device__ __forceinline__ bool grid_barrier(TailSync *gs, int *sh_abort) {
  __syncthreads();
  if (gridDim.x == 1) return true;  // one CTA: the block barrier orders everything
  if (threadIdx.x == 0) {
    const unsigned add = blockIdx.x == 0 ? 0x80000000u - (gridDim.x - 1) : 1u;
    __threadfence();
    const unsigned old = atomicAdd(&gs->arrive, add);
    volatile unsigned *av = &gs->arrive;
    volatile int *ev = &gs->err;
    long long spins = 0;
    int abort = 0;
    while (((old ^ *av) & 0x80000000u) == 0) {
      if (*ev) { abort = 1; break; }
      if (++spins > kBarrierSpins) {
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

template <typename T, int K>
__device__ void run_spmm(const TOp<T> &op, i64 gwarp, i64 nwarps, int lane) {
  const i64 units = op.A.n + op.A.nchunks;
  switch (op.epi) {
#define LG_TAIL_EPI(E)                                                        \
  case E:                                                                     \
    for (i64 u = gwarp; u < units; u += nwarps)                               \
      spmm_unit<T, K, 32, E>(op.A, op.x0, op.a, u, lane);                     \
    break;
    LG_TAIL_EPI(Epi::Store)
    LG_TAIL_EPI(Epi::Resid)
    LG_TAIL_EPI(Epi::ChebA)
    LG_TAIL_EPI(Epi::ChebB)
    LG_TAIL_EPI(Epi::ElimInterp)
    LG_TAIL_EPI(Epi::Jacobi)
#undef LG_TAIL_EPI
  }
}

// CTA-level partial sums over this CTA's row range: NV values per column.
template <typename T, int K, int NV>
__device__ void block_partials(const T *x, const T *y, const T *w, bool use_y, i64 n,
                               double *partial, double (*sh)[kTailThreads]) {
  const int tid = threadIdx.x;
  constexpr int RS = kTailThreads / K;
  const int c = tid % K, rsub = tid / K;
  const i64 rpc = (n + gridDim.x - 1) / gridDim.x;
  const i64 r0 = (i64)blockIdx.x * rpc, r1 = min(n, r0 + rpc);
  double a[NV];
#pragma unroll
  for (int v = 0; v < NV; v++) a[v] = 0;
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
#pragma unroll
  for (int v = 0; v < NV; v++) sh[v][tid] = a[v];
  __syncthreads();
  for (int st = kTailThreads / 2; st >= K; st >>= 1) {
    if (tid < st)
#pragma unroll
      for (int v = 0; v < NV; v++) sh[v][tid] += sh[v][tid + st];
    __syncthreads();
  }
  if (tid < K)
#pragma unroll
    for (int v = 0; v < NV; v++) partial[((i64)blockIdx.x * 3 + v) * K + tid] = sh[v][tid];
}

// Sum of the G CTA partials (fixed order, identical in every CTA) into
// sh[v][c] for c < K.
template <int K, int NV>
__device__ void finish_partials(const double *partial, double (*sh)[kTailThreads]) {
  const int tid = threadIdx.x;
  constexpr int RS = kTailThreads / K;
  const int c = tid % K, rsub = tid / K;
  double a[NV];
#pragma unroll
  for (int v = 0; v < NV; v++) a[v] = 0;
  for (unsigned b = rsub; b < gridDim.x; b += RS)
#pragma unroll
    for (int v = 0; v < NV; v++) a[v] += __ldcg(partial + ((i64)b * 3 + v) * K + c);
  __syncthreads();
#pragma unroll
  for (int v = 0; v < NV; v++) sh[v][tid] = a[v];
  __syncthreads();
  for (int st = kTailThreads / 2; st >= K; st >>= 1) {
    if (tid < st)
#pragma unroll
      for (int v = 0; v < NV; v++) sh[v][tid] += sh[v][tid + st];
    __syncthreads();
  }
}

template <typename T, int K>
__global__ void __launch_bounds__(kTailThreads, 1)
    k_tail(const TOp<T> *__restrict__ ops, int nops, double *partial, TailSync *gs) {
  __shared__ double sh[3][kTailThreads];
  __shared__ double scal[2][64];
  __shared__ int sh_abort;
  const int lane = threadIdx.x & 31;
  const i64 gwarp = ((i64)blockIdx.x * kTailThreads + threadIdx.x) >> 5;
  const i64 nwarps = (i64)gridDim.x * (kTailThreads / 32);
  const i64 gthr = (i64)blockIdx.x * kTailThreads + threadIdx.x;
  const i64 nthr = (i64)gridDim.x * kTailThreads;
  for (int i = 0; i < nops; i++) {
    const TOp<T> &op = ops[i];
    const i64 nk = op.n * K;
    switch (op.kind) {
      case TOpKind::Spmm:
        run_spmm<T, K>(op, gwarp, nwarps, lane);
        break;
      case TOpKind::Cheb0: {
        const T th = (T)op.f;
        for (i64 t = gthr; t < nk; t += nthr) op.y0[t] = op.x1[t / K] * op.x0[t] / th;
        break;
      }
      case TOpKind::Prolong:
        for (i64 t = gthr; t < nk; t += nthr)
          op.y0[t] += op.x0[(i64)op.idx[t / K] * K + (t % K)];
        break;
      case TOpKind::Coarse:
        for (i64 t = gthr; t < nk; t += nthr) {
          const i64 r = t / K;
          const int c = (int)(t % K);
          T s = 0;
          for (i64 j = 0; j < op.n; j++) s += op.x1[r * op.n + j] * op.x0[j * K + c];
          op.y0[t] = s;
        }
        break;
      case TOpKind::Scale: {
        const T f = (T)op.f;
        for (i64 t = gthr; t < nk; t += nthr) op.y0[t] = op.y0[t] * f;
        break;
      }
      case TOpKind::Zero:
        for (i64 t = gthr; t < nk; t += nthr) op.y0[t] = (T)0;
        break;
      case TOpKind::Copy:
        for (i64 t = gthr; t < nk; t += nthr) op.y0[t] = op.x0[t];
        break;
      case TOpKind::RedBeta:
        block_partials<T, K, 3>(op.x0, op.x1, nullptr, op.flag != 0, op.n, partial, sh);
        break;
      case TOpKind::RedAlpha:
        block_partials<T, K, 2>(op.x0, op.x1, op.x2, true, op.n, partial, sh);
        break;
      case TOpKind::Dir: {
        finish_partials<K, 3>(partial, sh);
        if (threadIdx.x < K) {
          const int c = threadIdx.x;
          const double mu = sh[0][c] / (double)op.n;
          double beta = 0.0;
          if (op.flag) {
            const double e = op.sc.eta_prev[c];
            beta = e == 0.0 ? 0.0 : (sh[1][c] - mu * sh[2][c]) / e;
          }
          scal[0][c] = mu;
          scal[1][c] = beta;
          if (blockIdx.x == 0) {
            op.sc.mu[c] = mu;
            op.sc.beta[c] = beta;
          }
        }
        __syncthreads();
        for (i64 t = gthr; t < nk; t += nthr) {
          const int c = (int)(t % K);
          T v = op.x0[t] - (T)scal[0][c];
          if (op.flag) v = v - (T)scal[1][c] * op.x1[t];
          op.y0[t] = v;
        }
        break;
      }
      case TOpKind::Update: {
        finish_partials<K, 2>(partial, sh);
        if (threadIdx.x < K) {
          const int c = threadIdx.x;
          const double eta = sh[0][c];
          const double alpha = eta == 0.0 ? 0.0 : sh[1][c] / eta;
          scal[0][c] = alpha;
          if (blockIdx.x == 0) {
            op.sc.eta[c] = eta;
            op.sc.alpha[c] = alpha;
          }
        }
        __syncthreads();
        for (i64 t = gthr; t < nk; t += nthr) {
          const T a = (T)scal[0][(int)(t % K)];
          op.y0[t] = op.y0[t] + a * op.x0[t];
          if (op.flag) op.y1[t] = op.y1[t] - a * op.x1[t];
        }
        break;
      }
    }
    if (!grid_barrier(gs, &sh_abort)) return;
  }
}

template <typename T, int K>
void launch_k(const TOp<T> *ops, int nops, int G, double *partial, TailSync *sync,
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
  LG_CUDA(cudaLaunchKernelEx(&cfg, k_tail<T, K>, ops, nops, partial, sync));
  LG_LAUNCH();
}

template <typename T, int K>
int max_ctas_k() {
  int dev = 0, sms = 0, per = 0;
  LG_CUDA(cudaGetDevice(&dev));
  LG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  LG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_tail<T, K>, kTailThreads, 0));
  return per * sms;
}

}  // namespace

template <typename T>
void launch_tail(const TOp<T> *ops, int nops, int k, int G, double *partial, TailSync *sync,
                 cudaStream_t s) {
  switch (k) {
    case 1: return launch_k<T, 1>(ops, nops, G, partial, sync, s);
    case 8: return launch_k<T, 8>(ops, nops, G, partial, sync, s);
    case 16: return launch_k<T, 16>(ops, nops, G, partial, sync, s);
    case 32: return launch_k<T, 32>(ops, nops, G, partial, sync, s);
    default: throw Error(LIGMG_ERR_UNSUPPORTED, "tail program: k must be 1, 8, 16 or 32");
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

template void launch_tail<float>(const TOp<float> *, int, int, int, double *, TailSync *,
                                 cudaStream_t);
template void launch_tail<double>(const TOp<double> *, int, int, int, double *, TailSync *,
                                  cudaStream_t);
template int tail_max_ctas<float>(int);
template int tail_max_ctas<double>(int);

}  // namespace lg
