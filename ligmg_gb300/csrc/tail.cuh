// tail.cuh — the coarse end of the cycle as one persistent kernel.
//
// Below a size threshold every level visit of the K-/V-cycle is a handful of
// small, dependent kernels; in a CUDA graph each costs a few microseconds of
// launch and dependent memory latency whatever its size, and the coarse
// levels are visited exponentially often by the K-cycle.  The host records
// the exact operation sequence of one visit of the tail (the same operations,
// pointers and scalars the launched path would issue) as a program of TOp
// records; one launch of k_tail executes it, either by all CTAs with grid
// barriers, or column slice by column slice, each CTA alone with everything
// it touches in its shared memory.
#pragma once
#include "solve.cuh"

namespace lg {

enum class TOpKind : int {
  Spmm,      // y = A X with epilogue `epi` (hub chunks included)
  Cheb0,     // d = f D^-1 b (f = 1/theta; omega for Jacobi) (first smoothing step)
  Prolong,   // x += xc[agg]
  Coarse,    // x = pinv b (dense)
  Scale,     // x *= f
  Zero,      // x = 0
  Copy,      // y = X
  RedBeta,   // partial sums of z, z.qp, qp (FCG beta)
  Dir,       // finish beta; p = z - mu - beta pp
  RedAlpha,  // partial sums of p.q, p.r (FCG alpha)
  Update,    // finish alpha; x += alpha p; r -= alpha q
};

template <typename T>
struct TOp {
  TOpKind kind = TOpKind::Zero;
  Epi epi = Epi::Store;
  int flag = 0;             // RedBeta/Dir: previous direction present; Update: update r
  i64 n = 0;                // rows
  MatView<T> A;             // Spmm
  EpiArgs a;                // Spmm epilogue
  const T *x0 = nullptr;    // Spmm X; Cheb0 b; Prolong xc; Coarse b; Copy src;
                            // RedBeta z; Dir z; RedAlpha p; Update p
  const T *x1 = nullptr;    // Cheb0 invd; Coarse pinv; RedBeta qp; Dir pp; RedAlpha q; Update q
  const T *x2 = nullptr;    // RedAlpha r
  T *y0 = nullptr;          // Cheb0 d; Prolong/Coarse/Scale/Zero x; Copy dst; Dir p; Update x
  T *y1 = nullptr;          // Update r
  const i32 *idx = nullptr; // Prolong agg
  double f = 1;             // Cheb0 and Scale factor
  FcgScalars sc{};          // Dir/Update
};

// Grid barrier state (arrive and err zero-initialised).  Every completed
// barrier adds exactly 2^31 to `arrive` (CTA 0 adds 2^31 - (G - 1), the
// others 1), so its low 31 bits are zero at each barrier's start and bit 31
// flips exactly when the last CTA arrives.  err != 0: a wait ran out of its
// iteration limit; every CTA then leaves the kernel (the host resets the
// state).  limit: polls of an incomplete barrier before a CTA gives up
// (<= 0: 2^23).
struct TailSync {
  unsigned arrive;
  int err;
  long long limit;
};

constexpr int kTailThreads = 1024;      // grid mode
constexpr int kTailSmemThreads = 256;   // shared-memory mode

// Shared-memory mode: a pointer equal to kSmemTag | offset names byte
// `offset` of the launch's dynamic shared memory; any other pointer is global.
constexpr unsigned long long kSmemTag = 1ull << 62;
constexpr unsigned long long kSmemOffMask = (1ull << 32) - 1;

// Grid mode: cooperative launch of G CTAs of kTailThreads threads with grid
// barriers, running `ops` from global memory (k columns).  partial: G x 3 x k
// doubles of reduction scratch.
template <typename T>
void launch_tail_grid(const TOp<T> *ops, int nops, int k, int G, double *partial,
                      TailSync *sync, cudaStream_t s);

// Shared-memory mode: k / kl CTAs, CTA g on columns [g*kl, (g+1)*kl).  Each
// copies `image` (the program followed by every read-only array the program
// reads, image_bytes, a multiple of 16) to the start of its dynamic shared
// memory (smem bytes in all), stages its slice of gin (n x k) at in_off,
// runs the program and writes its slice of the result at out_off to gout.
struct TailSmemLaunch {
  int kl = 0, nops = 0, smem = 0, image_bytes = 0;
  int cluster = 1;  // CTAs per column slice (cluster mode when > 1)
  const void *image = nullptr;
  const void *gin = nullptr;
  void *gout = nullptr;
  i64 n = 0;
  unsigned in_off = 0, out_off = 0;
};
// Cluster mode (L.cluster > 1): k / kl clusters of L.cluster CTAs, the
// products with matrices outside shared memory divided among a cluster's
// CTAs (distributed shared memory, hardware cluster barriers).
template <typename T>
void launch_tail_smem(const TailSmemLaunch &L, int k, TailSync *sync, cudaStream_t s);
// Whether clusters of `cl` CTAs with `smem` bytes of dynamic shared memory
// each can be launched for kl columns per CTA (0 bytes: the opted-in size).
template <typename T>
bool tail_cluster_ok(int kl, int cl, int smem);

// CTAs of kTailThreads threads that can be resident at once for the
// k-column grid-mode kernel (0: unavailable for k).
template <typename T>
int tail_max_ctas(int k);
// Shared-memory mode with kl columns per CTA: the dynamic shared memory
// available to one CTA; when 0 < bytes <= that, the kernel is opted in to
// `bytes`.  0: kl not available.
template <typename T>
int tail_smem_prepare(int kl, int bytes);

}  // namespace lg
