// queue.cu — the persistent work-queue kernel of batch solves (queue.cuh).
//
// One CTA works on one (operation, graph, row block) item at a time.  Thread
// 0 takes the next ticket, waits until the item's graph has finished every
// earlier operation (polls of its progress counter, bounded by wait_limit;
// on running out it records an error and every CTA leaves), and reads
// whether the graph has converged (then the item does no work).  After the
// block's work, the CTA that completes the graph's last block of the
// operation sums the reduction partials in block order, writes the graph's
// scalars and advances the graph's progress counter.
#include "queue.cuh"
#include "spmm_dev.cuh"

namespace lg {
namespace {

using namespace dev;

// rows [r0, r1) of y = A X with a fused epilogue, G lanes per row (k = 1)
template <typename T, int G, Epi EP>
__device__ void q_spmm_rows(const MatView<T> &A, const T *__restrict__ X, const EpiArgs &a,
                            i64 r0, i64 r1) {
  constexpr int RPW = 32 / G;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int grp = lane / G, slot = lane % G;
  for (i64 base = r0 + (i64)warp * RPW; base < r1; base += (kQueueThreads / 32) * RPW) {
    const i64 r = base + grp;
    const bool act = r < r1;
    T acc[1] = {(T)0};
    if (act) row_accumulate<T, 1, 1, G, true, EP == Epi::Split>(A, X, A.rp[r] + slot, A.rp[r + 1], 0, acc);
    reduce_slots<T, 1, 1, G>(acc);
    if (act && slot == 0) epilogue<T, 1, 1, EP>(a, r, 0, acc);
  }
}

template <typename T>
__device__ void q_spmm(const QOp &op, const MatView<T> &A, i64 r0, i64 r1) {
  const T *X = (const T *)op.x0;
  switch (op.epi) {
#define LG_Q_EPI(E)                                                               \
  case E:                                                                         \
    if (op.lanes == 8) q_spmm_rows<T, 8, E>(A, X, op.a, r0, r1);                  \
    else q_spmm_rows<T, 32, E>(A, X, op.a, r0, r1);                               \
    break;
    LG_Q_EPI(Epi::Store)
    LG_Q_EPI(Epi::Resid)
    LG_Q_EPI(Epi::ChebA)
    LG_Q_EPI(Epi::ChebB)
    LG_Q_EPI(Epi::ElimInterp)
    LG_Q_EPI(Epi::Jacobi)
    LG_Q_EPI(Epi::Split)
    LG_Q_EPI(Epi::ChebZ)
    LG_Q_EPI(Epi::FcgDir)
#undef LG_Q_EPI
  }
}

// block partial of a reduction: a fixed shared-memory tree over the
// threads' strided sums (deterministic), written by thread 0 to dst[0..2]
template <typename T>
__device__ void q_reduce(const QOp &op, i64 r0, i64 r1, double *dst,
                         double (*sh)[kQueueThreads]) {
  const T *x = (const T *)op.x0, *y = (const T *)op.x1, *w = (const T *)op.x2;
  double a0 = 0, a1 = 0, a2 = 0;
  for (i64 r = r0 + threadIdx.x; r < r1; r += kQueueThreads) {
    const double xv = (double)x[r];
    switch (op.kind) {
      case QKind::RedSum:
        a0 += xv;
        break;
      case QKind::RedBeta:
        a0 += xv;
        if (y) {
          const double yv = (double)y[r];
          a1 += xv * yv;
          a2 += yv;
        }
        break;
      case QKind::RedAlpha:
        a0 += xv * (double)y[r];
        a1 += xv * (double)w[r];
        break;
      default:  // RedNorm
        a0 += xv * xv;
        break;
    }
  }
  const int t = threadIdx.x;
  sh[0][t] = a0;
  sh[1][t] = a1;
  sh[2][t] = a2;
  __syncthreads();
  for (int st = kQueueThreads / 2; st > 0; st >>= 1) {
    if (t < st)
#pragma unroll
      for (int v = 0; v < 3; v++) sh[v][t] += sh[v][t + st];
    __syncthreads();
  }
  if (t == 0)
#pragma unroll
    for (int v = 0; v < 3; v++) dst[v] = sh[v][0];
}

template <typename T>
__device__ void q_elementwise(const QOp &op, int g, i64 r0, i64 r1, i64 g0, i64 g1) {
  T *y0 = (T *)op.y0;
  const T *x0 = (const T *)op.x0, *x1 = (const T *)op.x1;
  const int t0 = threadIdx.x;
  switch (op.kind) {
    case QKind::Cheb0: {
      const T f = (T)op.f;
      for (i64 r = r0 + t0; r < r1; r += kQueueThreads) y0[r] = (x1[r] * f) * x0[r];
      break;
    }
    case QKind::Prolong:
      for (i64 r = r0 + t0; r < r1; r += kQueueThreads) y0[r] += x0[op.idx[r]];
      break;
    case QKind::Coarse:  // the graph's diagonal block of the dense pseudo-inverse
      for (i64 r = r0 + t0; r < r1; r += kQueueThreads) {
        T s = 0;
        for (i64 j = g0; j < g1; j++) s += x1[r * op.n + j] * x0[j];
        y0[r] = s;
      }
      break;
    case QKind::Scale: {
      const T f = (T)op.f;
      for (i64 r = r0 + t0; r < r1; r += kQueueThreads) y0[r] = y0[r] * f;
      break;
    }
    case QKind::Zero:
      for (i64 r = r0 + t0; r < r1; r += kQueueThreads) y0[r] = (T)0;
      break;
    case QKind::Copy:
      for (i64 r = r0 + t0; r < r1; r += kQueueThreads) y0[r] = x0[r];
      break;
    case QKind::SubMean: {
      const double m = ((const double *)op.x1)[g];
      for (i64 r = r0 + t0; r < r1; r += kQueueThreads) y0[r] = (T)((double)y0[r] - m);
      break;
    }
    case QKind::Dir: {
      const T mu = (T)op.sc.mu[g], be = (T)op.sc.beta[g];
      for (i64 r = r0 + t0; r < r1; r += kQueueThreads) {
        T v = x0[r] - mu;
        if (x1) v = v - be * x1[r];
        y0[r] = v;
      }
      break;
    }
    case QKind::Update: {
      const T al = (T)op.sc.alpha[g];
      const T *q = x1;
      T *rr = (T *)op.y1;
      for (i64 r = r0 + t0; r < r1; r += kQueueThreads) {
        y0[r] = y0[r] + al * x0[r];
        if (op.flag) rr[r] = rr[r] - al * q[r];
      }
      break;
    }
    default:
      break;
  }
}

__device__ void q_item(const QOp &op, int g, int b, i64 r0, i64 r1, i64 g0, i64 g1,
                       double *part, double (*sh)[kQueueThreads]) {
  switch (op.kind) {
    case QKind::Spmm:
      if (op.dbl) q_spmm<double>(op, op.Ad, r0, r1);
      else q_spmm<float>(op, op.Af, r0, r1);
      break;
    case QKind::ToFloat:
      for (i64 r = r0 + threadIdx.x; r < r1; r += kQueueThreads)
        ((float *)op.y0)[r] = (float)((const double *)op.x0)[r];
      break;
    case QKind::ToDouble:
      for (i64 r = r0 + threadIdx.x; r < r1; r += kQueueThreads)
        ((double *)op.y0)[r] = (double)((const float *)op.x0)[r];
      break;
    case QKind::RedSum:
    case QKind::RedBeta:
    case QKind::RedAlpha:
    case QKind::RedNorm: {
      double *dst = part + ((i64)g * kQueueMaxBlocks + b) * 3;
      if (op.dbl) q_reduce<double>(op, r0, r1, dst, sh);
      else q_reduce<float>(op, r0, r1, dst, sh);
      break;
    }
    default:
      if (op.dbl) q_elementwise<double>(op, g, r0, r1, g0, g1);
      else q_elementwise<float>(op, g, r0, r1, g0, g1);
      break;
  }
}

__device__ bool q_is_reduction(QKind k) {
  return k == QKind::RedSum || k == QKind::RedBeta || k == QKind::RedAlpha || k == QKind::RedNorm;
}

// a graph's reduction totals t: its scalars (and the outer convergence test)
__device__ void q_scalars(const QOp &op, int g, const double (&t)[3], i64 ng, int it_offset) {
  switch (op.kind) {
    case QKind::RedSum:
      op.out[g] = t[0] / (double)ng;
      break;
    case QKind::RedBeta: {
      const double mu = t[0] / (double)ng;
      op.sc.mu[g] = mu;
      const double e = op.sc.eta_prev[g];
      op.sc.beta[g] = (op.flag && e != 0.0) ? (t[1] - mu * t[2]) / e : 0.0;
      break;
    }
    case QKind::RedAlpha: {
      const double eta = t[0];
      op.sc.eta[g] = eta;
      op.sc.alpha[g] = eta == 0.0 ? 0.0 : t[1] / eta;
      break;
    }
    default:  // RedNorm: the outer convergence test of this iteration
      op.out[g] = t[0];
      op.iters[g] = it_offset + op.it + 1;
      if (t[0] <= op.tol2 * op.rn0sq[g]) op.frozen[g] = 1;  // a NaN norm never freezes
      break;
  }
}

// the graph's operation is complete: sum the block partials in block order
__device__ void q_finalize(const QOp &op, int g, int nb, i64 ng, const double *part,
                           int it_offset) {
  if (!q_is_reduction(op.kind)) return;
  double t[3] = {0, 0, 0};
  for (int b = 0; b < nb; b++)
    for (int v = 0; v < 3; v++) t[v] += __ldcg(part + ((i64)g * kQueueMaxBlocks + b) * 3 + v);
  q_scalars(op, g, t, ng, it_offset);
}

__global__ void __launch_bounds__(kQueueThreads) k_queue(QueueArgs q) {
  __shared__ unsigned long long s_item;
  __shared__ int s_ctl, s_last;
  __shared__ double sh[3][kQueueThreads];
  const int tid = threadIdx.x;
  volatile int *ev = &q.st->err;
  while (true) {
    if (tid == 0) {
      const unsigned long long t = atomicAdd(&q.st->ticket, 1ull);
      s_ctl = t >= q.nitems ? 2 : 0;  // 2: leave
      if (t < q.nitems) s_item = q.items[t];
    }
    __syncthreads();
    if (s_ctl == 2) break;
    const unsigned long long it = s_item;
    const int opi = (int)(it >> 40), g = (int)((it >> 20) & 0xfffff);
    const unsigned low = (unsigned)(it & 0xfffff);
    const bool chain = (low & kQueueChain) != 0;
    const int cnt = chain ? (int)(low & (kQueueChain - 1)) : 1;
    // wait (bounded) until the graph has finished the earlier operations
    int bad = 0;
    if (tid == 0) {
      volatile int *pg = q.prog + g;
      long long polls = 0;
      while (*pg < opi) {
        if (*ev) {
          bad = 1;
          break;
        }
        if (++polls >= q.wait_limit) {
          atomicExch(&q.st->err, 1);
          bad = 1;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    if (__syncthreads_or(bad)) break;
    if (chain) {
      // one graph's consecutive single-block operations, back to back
      for (int i = opi; i < opi + cnt; i++) {
        const QOp &op = q.ops[i];
        const i64 *seg = q.segs[op.seglev];
        const i64 g0 = seg[g], g1 = seg[g + 1];
        const bool skip = ((volatile const int *)q.frozen)[g] != 0;
        if (!skip) q_item(op, g, 0, g0, g1, g0, g1, q.part, sh);
        __syncthreads();
        if (tid == 0 && !skip) q_finalize(op, g, 1, g1 - g0, q.part, q.st->it_offset);
        __syncthreads();
      }
      if (tid == 0) {
        __threadfence();
        atomicExch(q.prog + g, opi + cnt);
      }
      continue;
    }
    const QOp &op = q.ops[opi];
    const i64 *seg = q.segs[op.seglev];
    const int b = (int)low;
    const bool skip = ((volatile const int *)q.frozen)[g] != 0;
    const i64 g0 = seg[g], g1 = seg[g + 1];
    const i64 r0 = g0 + (i64)b * kQueueRows, r1 = min(g1, r0 + (i64)kQueueRows);
    const int nb = g1 > g0 ? (int)((g1 - g0 + kQueueRows - 1) / kQueueRows) : 1;
    if (!skip) q_item(op, g, b, r0, r1, g0, g1, q.part, sh);
    __syncthreads();
    if (tid == 0) {
      __threadfence();
      s_last = atomicAdd(q.blk + g, 1) + 1 == nb;
    }
    __syncthreads();
    if (tid == 0 && s_last) {
      __threadfence();
      if (!skip) q_finalize(op, g, nb, g1 - g0, q.part, q.st->it_offset);
      q.blk[g] = 0;
      __threadfence();
      atomicExch(q.prog + g, opi + 1);
    }
  }
}

int g_queue_blocks = 0;

}  // namespace

void launch_queue(const QueueArgs &q, cudaStream_t s) {
  if (g_queue_blocks <= 0) {
    int dev = 0, sms = 0, per = 0;
    LG_CUDA(cudaGetDevice(&dev));
    LG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    LG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_queue, kQueueThreads, 0));
    g_queue_blocks = std::max(1, per) * sms;
  }
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)g_queue_blocks);
  cfg.blockDim = dim3(kQueueThreads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  LG_CUDA(cudaLaunchKernelEx(&cfg, k_queue, q));
  LG_LAUNCH();
}

}  // namespace lg
