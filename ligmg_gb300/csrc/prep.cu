// prep.cu — input preparation on the GPU (see prep.cuh).
//
// Largest connected component (cc.hpp:24-106): every vertex carries the
// largest vertex index of its component.  Starting from label[i] = i, a sweep
// raises each label to the maximum over its row's neighbours (the reference's
// MaxSRing SpMV) and a pointer jump raises label[i] to label[label[i]]; both
// only raise labels and keep them inside the component, so they reach the
// same fixed point (the component's maximum index) in fewer rounds than the
// SpMV alone.  Component sizes are counted per label; the largest wins, a tie
// going to the smaller label, as the reference's max_element over component
// ids does.  Kept vertices are renumbered in ascending order and only
// entries between kept vertices are kept, in the input's order.
//
// Laplacian (main.cpp:81-110): d_i = sum of row i's stored entries (the kept
// ones, in ascending column order, sequentially), L = D - A: off-diagonal
// entries negated, the diagonal d_i - a_ii (inserted in order when absent).
#include "prep.cuh"
#include "prims.cuh"

namespace lg {
namespace {

__global__ void k_prep_check(i64 n, const i64 *rp, const i32 *ci, int *err) {
  const i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const i64 b = rp[i], e = rp[i + 1];
  if (e < b) {
    atomicOr(err, 1);
    return;
  }
  for (i64 k = b; k < e; k++) {
    const i32 j = ci[k];
    if (j < 0 || j >= n) atomicOr(err, 1);
    else if (k > b && ci[k - 1] >= j) atomicOr(err, 2);
  }
}

__global__ void k_iota64(i64 n, i64 *x) {
  const i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = i;
}

// one warp per row: label[i] = max(label[i], label[j] for j in row i)
__global__ void k_label_sweep(i64 n, const i64 *rp, const i32 *ci, i64 *lab, int *changed) {
  const i64 i = ((i64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= n) return;
  i64 m = -1;
  for (i64 k = rp[i] + lane; k < rp[i + 1]; k += 32) m = max(m, lab[ci[k]]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, (i64)__shfl_xor_sync(0xffffffffu, m, o));
  if (lane == 0 && m > lab[i]) {
    atomicMax((unsigned long long *)&lab[i], (unsigned long long)m);
    *changed = 1;
  }
}

// label[i] = label[label[i]]: a label is a vertex of the same component whose
// own label is at least as large
__global__ void k_label_jump(i64 n, i64 *lab, int *changed) {
  const i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const i64 l = lab[i];
  const i64 ll = lab[l];
  if (ll > l) {
    atomicMax((unsigned long long *)&lab[i], (unsigned long long)ll);
    *changed = 1;
  }
}

__global__ void k_count_labels(i64 n, const i64 *lab, unsigned long long *cnt) {
  const i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) atomicAdd(&cnt[lab[i]], 1ull);
}

// key = count << 32 | (2^32 - 1 - label): the maximum key is the largest
// component, ties to the smaller label
__global__ void k_best_label(i64 n, const unsigned long long *cnt, unsigned long long *best) {
  const i64 v = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n || cnt[v] == 0) return;
  atomicMax(best, (cnt[v] << 32) | (0xffffffffull - (unsigned long long)v));
}

__global__ void k_keep(i64 n, const i64 *lab, const unsigned long long *best, i32 *keep) {
  const i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const i64 label = (i64)(0xffffffffull - (*best & 0xffffffffull));
  keep[i] = lab[i] == label ? 1 : 0;
}

__global__ void k_fill_one(i64 n, i32 *x) {
  const i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = 1;
}

// entries of kept row i in the output (and the diagonal's insertion)
__global__ void k_prep_count(i64 n, const i64 *rp, const i32 *ci, const i32 *keep,
                             const i32 *nid, int lap, i64 *cnt) {
  const i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !keep[i]) return;
  i64 c = 0;
  bool diag = false;
  for (i64 k = rp[i]; k < rp[i + 1]; k++) {
    const i32 j = ci[k];
    if (!keep[j]) continue;
    c++;
    if (j == i) diag = true;
  }
  if (lap && !diag) c++;
  cnt[nid[i]] = c;
}

__global__ void k_prep_fill(i64 n, const i64 *rp, const i32 *ci, const double *val,
                            const i32 *keep, const i32 *nid, int lap, const i64 *orp,
                            i32 *oci, double *oval, i64 *orig) {
  const i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !keep[i]) return;
  const i32 r = nid[i];
  orig[r] = i;
  double d = 0.0;
  if (lap)
    for (i64 k = rp[i]; k < rp[i + 1]; k++)
      if (keep[ci[k]]) d = __dadd_rn(d, val[k]);
  i64 p = orp[r];
  bool placed = false;
  for (i64 k = rp[i]; k < rp[i + 1]; k++) {
    const i32 j = ci[k];
    if (!keep[j]) continue;
    const i32 c = nid[j];
    if (lap && !placed && c > r) {  // absent diagonal, inserted in order
      oci[p] = r;
      oval[p++] = d;
      placed = true;
    }
    double v = val[k];
    if (lap) {
      if (c == r) {
        v = __dsub_rn(d, v);
        placed = true;
      } else {
        v = -v;
      }
    }
    oci[p] = c;
    oval[p++] = v;
  }
  if (lap && !placed) {
    oci[p] = r;
    oval[p] = d;
  }
}

}  // namespace

void prepare_graph(i64 n, const i64 *rowptr, const i32 *col, const double *val, bool lcc,
                   bool laplacian, bool want_arrays, PrepResult &out, cudaStream_t s) {
  if (n <= 0 || !rowptr || !col || !val) throw Error(LIGMG_ERR_INVALID_ARGUMENT, "graph");
  const i64 nnz = rowptr[n];
  if (rowptr[0] != 0 || nnz < 0) throw Error(LIGMG_ERR_INVALID_ARGUMENT, "row pointers");
  DBuf<i64> rp(n + 1, s);
  DBuf<i32> ci(std::max<i64>(nnz, 1), s);
  DBuf<double> v(std::max<i64>(nnz, 1), s);
  rp.upload(rowptr, n + 1);
  if (nnz) {
    ci.upload(col, nnz);
    v.upload(val, nnz);
  }
  DBuf<int> flag(1, s);
  flag.zero();
  k_prep_check<<<grid_for(n, 256), 256, 0, s>>>(n, rp.p, ci.p, flag.p);
  LG_LAUNCH();
  int err = 0;
  flag.download(&err, 1);
  LG_CUDA(cudaStreamSynchronize(s));
  if (err & 1) throw Error(LIGMG_ERR_INVALID_ARGUMENT, "column index out of range");
  if (err & 2) throw Error(LIGMG_ERR_NOT_SORTED, "columns not ascending within a row");

  DBuf<i32> keep(n, s), nid(n, s);
  if (lcc) {
    DBuf<i64> lab(n, s);
    k_iota64<<<grid_for(n, 256), 256, 0, s>>>(n, lab.p);
    LG_LAUNCH();
    for (i64 round = 0;; round++) {
      if (round > n + 1) throw Error(LIGMG_ERR_INTERNAL, "label propagation did not settle");
      flag.zero();
      k_label_sweep<<<grid_for(n * 32, 256), 256, 0, s>>>(n, rp.p, ci.p, lab.p, flag.p);
      LG_LAUNCH();
      k_label_jump<<<grid_for(n, 256), 256, 0, s>>>(n, lab.p, flag.p);
      LG_LAUNCH();
      int changed = 0;
      flag.download(&changed, 1);
      LG_CUDA(cudaStreamSynchronize(s));
      if (!changed) break;
    }
    DBuf<unsigned long long> cnt(n, s), best(1, s);
    cnt.zero();
    best.zero();
    k_count_labels<<<grid_for(n, 256), 256, 0, s>>>(n, lab.p, cnt.p);
    LG_LAUNCH();
    k_best_label<<<grid_for(n, 256), 256, 0, s>>>(n, cnt.p, best.p);
    LG_LAUNCH();
    k_keep<<<grid_for(n, 256), 256, 0, s>>>(n, lab.p, best.p, keep.p);
    LG_LAUNCH();
  } else {
    k_fill_one<<<grid_for(n, 256), 256, 0, s>>>(n, keep.p);
    LG_LAUNCH();
  }
  DBuf<i32> total(1, s);
  exclusive_scan<i32>(keep.p, nid.p, n, s, total.p);
  i32 nk = 0;
  total.download(&nk, 1);
  LG_CUDA(cudaStreamSynchronize(s));
  DBuf<i64> cnt(nk + 1, s), orp(nk + 1, s);
  cnt.zero();
  k_prep_count<<<grid_for(n, 256), 256, 0, s>>>(n, rp.p, ci.p, keep.p, nid.p, laplacian ? 1 : 0,
                                                cnt.p);
  LG_LAUNCH();
  DBuf<i64> onnz(1, s);
  exclusive_scan<i64>(cnt.p, orp.p, nk + 1, s, onnz.p);
  i64 m = 0;
  onnz.download(&m, 1);
  LG_CUDA(cudaStreamSynchronize(s));
  out.n = nk;
  out.nnz = m;
  if (!want_arrays) return;
  DBuf<i32> oci(std::max<i64>(m, 1), s);
  DBuf<double> oval(std::max<i64>(m, 1), s);
  DBuf<i64> orig(std::max<i64>(nk, 1), s);
  k_prep_fill<<<grid_for(n, 256), 256, 0, s>>>(n, rp.p, ci.p, v.p, keep.p, nid.p,
                                               laplacian ? 1 : 0, orp.p, oci.p, oval.p, orig.p);
  LG_LAUNCH();
  out.rowptr.resize(nk + 1);
  out.col.resize(m);
  out.val.resize(m);
  out.orig.resize(nk);
  orp.download(out.rowptr.data(), nk + 1);
  if (m) {
    oci.download(out.col.data(), m);
    oval.download(out.val.data(), m);
  }
  if (nk) orig.download(out.orig.data(), nk);
  LG_CUDA(cudaStreamSynchronize(s));
}

}  // namespace lg
