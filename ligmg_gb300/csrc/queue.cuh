// queue.cuh — a batch of graph solves as one persistent work-queue launch.
//
// The host records the exact operation sequence of kQueueIters outer FCG
// iterations of a batch solve (each preconditioner application with its
// K-/V-cycle, the per-graph constant projection, the outer Krylov steps and
// the convergence test) as a program of QOp records.  Every operation works
// on one level's rows, and the batch's graphs own disjoint, contiguous row
// ranges of every level (no aggregate, elimination or coarse block crosses
// graphs), so an operation splits into (graph, row-block) work items that
// depend only on the same graph's previous operation.  Where a graph's rows
// fit one block (its coarse levels, small graphs), its consecutive operations
// form one chain item run back to back by a single CTA.  The items, ordered
// by first operation, then graph, then block, form the queue; a cooperative
// launch of resident CTAs takes them from one atomic ticket.  Before working
// on an item a CTA waits (bounded) until its graph has finished the earlier
// operations; the CTA finishing a graph's last block of an operation sums
// that operation's block partials in block order (reductions) and advances
// the graph's progress counter.  Graphs therefore move through the program
// independently, each stopping work as soon as it has converged.
#pragma once
#include "solve.cuh"

namespace lg {

enum class QKind : int {
  Spmm,      // y = A X with epilogue `epi` (whole rows, `lanes` lanes per row)
  Cheb0,     // y0 = (x1 * f) * x0                (first smoothing step from 0)
  Prolong,   // y0 += x0[idx]
  Coarse,    // y0 = pinv(graph block) x0
  Scale,     // y0 *= f
  Zero,      // y0 = 0
  Copy,      // y0 = x0
  ToFloat,   // y0 (float) = x0 (double)
  ToDouble,  // y0 (double) = x0 (float)
  RedSum,    // out[g] = mean of x0 over the graph
  SubMean,   // y0 -= out[g]                      (x1: the mean array)
  RedBeta,   // FCG: mu = mean(z); beta = (z.qp - mu sum(qp)) / eta_prev (qp = x1, may be null)
  Dir,       // p (y0) = (z (x0) - mu) - beta pp (x1, may be null)
  RedAlpha,  // FCG: eta = p.q; alpha = (p.r) / eta   (x0 p, x1 q, x2 r)
  Update,    // x (y0) += alpha p (x0); r (y1) -= alpha q (x1) when flag
  RedNorm,   // outer test: rn2 = r.r; converged when rn2 <= tol2 rn0sq (sets frozen, iters)
};

struct QOp {
  QKind kind = QKind::Zero;
  int dbl = 0;        // 1: the operation's vectors are double, 0: float
  Epi epi = Epi::Store;
  int flag = 0;       // RedBeta/Dir: previous direction present; Update: update r
  int lanes = 32;     // Spmm: lanes per row (8 or 32)
  int seglev = 0;     // level whose graph row ranges split this operation's rows
  int it = 0;         // RedNorm: outer iteration number
  i64 n = 0;          // rows of the operation's row space (Coarse: the level size)
  MatView<float> Af;  // Spmm, dbl = 0
  MatView<double> Ad; // Spmm, dbl = 1
  EpiArgs a;
  const void *x0 = nullptr, *x1 = nullptr, *x2 = nullptr;
  void *y0 = nullptr, *y1 = nullptr;
  const i32 *idx = nullptr;
  double f = 1, tol2 = 0;
  FcgScalars sc{};    // per-graph scalar arrays (RedBeta/Dir/RedAlpha/Update)
  double *out = nullptr;          // RedSum: per-graph means; RedNorm: rn2
  const double *rn0sq = nullptr;  // RedNorm
  int *frozen = nullptr, *iters = nullptr;  // RedNorm (frozen also read by every item)
};

// Row blocks: a graph's rows of a level are cut into blocks of kQueueRows.
constexpr int kQueueRows = 2048;
constexpr int kQueueThreads = 256;
constexpr int kQueueIters = 16;       // outer iterations per recorded program
constexpr int kQueueMaxBlocks = 1024;  // blocks of one graph in one operation

// Device state of one launch (zeroed by the host before it): the ticket, per
// graph its progress (operations finished) and the finished blocks of its
// current operation, block partials of the current reduction, an error flag.
struct QueueState {
  unsigned long long ticket;
  int err;        // 1: a wait gave up (the call fails with LIGMG_ERR_INTERNAL)
  int it_offset;  // outer iterations done before this launch (set by the host)
};

// An item is op << 40 | graph << 20 | low.  low < kQueueChain: block `low`
// of operation `op` for a graph with more than kQueueRows rows there;
// low = kQueueChain | c: the c consecutive operations from `op` during which
// the graph's rows fit one block, run back to back by one CTA (the graph's
// coarse levels: thousands of small dependent operations with no hand-off
// between CTAs).
constexpr unsigned kQueueChain = 1u << 19;

struct QueueArgs {
  const QOp *ops = nullptr;
  const unsigned long long *items = nullptr;
  unsigned long long nitems = 0;
  const i64 *const *segs = nullptr;  // per level: nseg + 1 row offsets
  int nseg = 0;
  int *prog = nullptr;      // nseg
  int *blk = nullptr;       // nseg
  double *part = nullptr;   // nseg x kQueueMaxBlocks x 3
  const int *frozen = nullptr;
  QueueState *st = nullptr;
  long long wait_limit = 0;  // polls of a graph's progress before giving up
};

// Cooperative launch of all resident CTAs of k_queue.
void launch_queue(const QueueArgs &q, cudaStream_t s);

}  // namespace lg
