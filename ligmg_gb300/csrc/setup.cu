// setup.cu — GPU hierarchy construction (FP64, bit-exact).
//
// Compiled with --fmad=false: every FP64 product and sum is rounded on its
// own, in the order the CPU restatement uses, so that aggregate and
// elimination ids (which depend on FP64 comparisons) are identical.
// Orders that matter are fixed explicitly:
//   * per-row sums run sequentially in ascending column order;
//   * scatter-adds that the reference performs in ascending source order
//     (vote tally, Galerkin terms) become a stable sort by target followed by
//     a sequential per-segment sum.
#include "prims.cuh"
#include "setup.cuh"

namespace lg {
namespace {

constexpr int kWarpsPerBlock = 8;
constexpr int kBlock = 32 * kWarpsPerBlock;

__device__ __forceinline__ i64 warp_row() {
  return ((i64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
}

// ---------------------------------------------------------------------------
// generic helpers
__global__ void k_diag_pos(const i64 *rp, const i32 *ci, i64 n, i64 *dpos) {
  i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  i64 lo = rp[i], hi = rp[i + 1];
  while (lo < hi) {
    i64 mid = (lo + hi) >> 1;
    if (ci[mid] < i) lo = mid + 1; else hi = mid;
  }
  dpos[i] = (lo < rp[i + 1] && ci[lo] == i) ? lo : -1;
}

__global__ void k_expand_rows(const i64 *rp, i64 n, i32 *rows) {
  i64 w = warp_row();
  if (w >= n) return;
  for (i64 e = rp[w] + lane_id(); e < rp[w + 1]; e += 32) rows[e] = (i32)w;
}

__global__ void k_count_cols(const i32 *ci, i64 nnz, i64 *cnt) {
  i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < nnz) atomicAdd((unsigned long long *)&cnt[ci[e]], 1ull);
}

__global__ void k_iota_u32(u32 *x, i64 n) {
  i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = (u32)i;
}

__global__ void k_cols_to_keys(const i32 *ci, i64 nnz, u64 *keys) {
  i64 e = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < nnz) keys[e] = (u64)(u32)ci[e];
}

__global__ void k_transpose_fill(const u32 *perm, const i32 *rows, const double *v, i64 nnz,
                                 i32 *tci, double *tv) {
  i64 k = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nnz) return;
  u32 e = perm[k];
  tci[k] = rows[e];
  tv[k] = v[e];
}

// ---------------------------------------------------------------------------
// validation: sortedness, ranges, finiteness, signs, diagonal, symmetry
__global__ void k_validate(const i64 *rp, const i32 *ci, const double *v, i64 n, int *err) {
  i64 w = warp_row();
  if (w >= n) return;
  i64 b = rp[w], e = rp[w + 1];
  int code = 0;
  if (e < b) code = LIGMG_ERR_INVALID_ARGUMENT;
  int has_diag = 0;
  for (i64 k = b + lane_id(); k < e && code == 0; k += 32) {
    i32 j = ci[k];
    double a = v[k];
    if (j < 0 || j >= n) { code = LIGMG_ERR_INVALID_ARGUMENT; break; }
    if (k > b && ci[k - 1] >= j) { code = LIGMG_ERR_NOT_SORTED; break; }
    if (!isfinite(a)) { code = LIGMG_ERR_NONFINITE; break; }
    if (j == w) {
      has_diag = 1;
      if (!(a > 0)) { code = LIGMG_ERR_BAD_DIAGONAL; break; }
    } else if (a > 0) {
      code = LIGMG_ERR_POSITIVE_OFFDIAG;
      break;
    }
    // symmetric partner (w) in row j
    i64 lo = rp[j], hi = rp[j + 1];
    while (lo < hi) {
      i64 mid = (lo + hi) >> 1;
      if (ci[mid] < w) lo = mid + 1; else hi = mid;
    }
    if (lo >= rp[j + 1] || ci[lo] != w || v[lo] != a) { code = LIGMG_ERR_NOT_SYMMETRIC; break; }
  }
  has_diag = __any_sync(0xffffffffu, has_diag);
  if (code == 0 && !has_diag && lane_id() == 0) code = LIGMG_ERR_BAD_DIAGONAL;
  if (code) atomicMin(err, code);
}

// ---------------------------------------------------------------------------
// elimination.hpp:71-80 compute_degrees + :186-190 candidates
__global__ void k_elim_cand(const i64 *rp, const double *v, i64 n, int maxdeg, uint8_t *cand) {
  i64 w = warp_row();
  if (w >= n) return;
  i64 cnt = 0;
  for (i64 k = rp[w] + lane_id(); k < rp[w + 1]; k += 32) cnt += (v[k] == 0) ? 0 : 1;
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if (lane_id() == 0) cand[w] = (cnt - 1) <= maxdeg;
}

// IndxHashMin SpMV (elimination.hpp:122-154,201-202): the candidate of
// smallest index among nonzero entries of the row; eliminated iff that is i.
__global__ void k_elim_select(const i64 *rp, const i32 *ci, const double *v, i64 n,
                              const uint8_t *cand, i32 *keep) {
  i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int elim = 0;
  if (cand[i]) {
    for (i64 k = rp[i]; k < rp[i + 1]; k++) {
      i32 j = ci[k];
      if (v[k] != 0 && cand[j]) {
        elim = (j == i);
        break;
      }
    }
  }
  keep[i] = elim ? 0 : 1;
}

__global__ void k_new_ids(const i32 *keep, const i32 *pos, i64 n, i32 *new_id) {
  i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) new_id[i] = keep[i] ? pos[i] : -1;
}

// P row counts (elimination.hpp:295-331)
__global__ void k_elim_pcount(const i64 *rp, const i32 *ci, i64 n, const i32 *new_id,
                              i64 *pcnt) {
  i64 j = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  if (new_id[j] >= 0) { pcnt[j] = 1; return; }
  i64 c = 0;
  for (i64 k = rp[j]; k < rp[j + 1]; k++) {
    i32 i = ci[k];
    if (i != j && new_id[i] >= 0) c++;
  }
  pcnt[j] = c;
}

__global__ void k_elim_pfill(const i64 *rp, const i32 *ci, const double *v, i64 n,
                             const i32 *new_id, const i64 *dpos, const i64 *prp, i32 *pci,
                             double *pv, double *Q) {
  i64 j = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  i64 o = prp[j];
  if (new_id[j] >= 0) {
    pci[o] = new_id[j];
    pv[o] = 1.0;
    Q[j] = 0.0;
    return;
  }
  double inv = 1.0 / v[dpos[j]];  // 1 / diag_x.at(j)  (:323,:327)
  for (i64 k = rp[j]; k < rp[j + 1]; k++) {
    i32 i = ci[k];
    if (i == j || new_id[i] < 0) continue;
    pci[o] = new_id[i];
    pv[o] = __dmul_rn(inv, -v[k]);
    o++;
  }
  Q[j] = inv;
}

// ---------------------------------------------------------------------------
// Galerkin product
__global__ void k_gal_count(const i64 *rp, const i32 *ci, i64 n, const i64 *prp, const i32 *pci,
                            i64 *cnt) {
  i64 a = warp_row();
  if (a >= n) return;
  for (i64 e = rp[a] + lane_id(); e < rp[a + 1]; e += 32) {
    i32 b = ci[e];
    i64 c = 0;
    for (i64 x = prp[a]; x < prp[a + 1]; x++) {
      i32 I = pci[x];
      for (i64 y = prp[b]; y < prp[b + 1]; y++) c += (pci[y] >= I) ? 1 : 0;
    }
    cnt[e] = c;
  }
}

__global__ void k_gal_emit(const i64 *rp, const i32 *ci, const double *v, i64 n, const i64 *prp,
                           const i32 *pci, const double *pv, u64 nc, const i64 *off, u64 *keys,
                           u32 *idx, double *tv) {
  i64 a = warp_row();
  if (a >= n) return;
  for (i64 e = rp[a] + lane_id(); e < rp[a + 1]; e += 32) {
    i32 b = ci[e];
    double A_ab = v[e];
    i64 o = off[e];
    for (i64 x = prp[a]; x < prp[a + 1]; x++) {
      i32 I = pci[x];
      double t = __dmul_rn(pv[x], A_ab);
      for (i64 y = prp[b]; y < prp[b + 1]; y++) {
        i32 J = pci[y];
        if (J < I) continue;
        keys[o] = (u64)I * nc + (u64)J;
        idx[o] = (u32)o;
        tv[o] = __dmul_rn(t, pv[y]);
        o++;
      }
    }
  }
}

__global__ void k_seg_flags(const u64 *keys, i64 T, uint8_t *flag) {
  i64 k = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < T) flag[k] = (k == 0 || keys[k] != keys[k - 1]) ? 1 : 0;
}

__global__ void k_gal_segsum(const u64 *keys, const u32 *idx, const double *tv, const i32 *starts,
                             i64 nseg, i64 T, u64 nc, i32 *sI, i32 *sJ, double *sV) {
  i64 s = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  i64 b = starts[s], e = (s + 1 < nseg) ? starts[s + 1] : T;
  double acc = tv[idx[b]];
  for (i64 k = b + 1; k < e; k++) acc = __dadd_rn(acc, tv[idx[k]]);
  u64 key = keys[b];
  sI[s] = (i32)(key / nc);
  sJ[s] = (i32)(key % nc);
  sV[s] = acc;
}

__global__ void k_gal_rowcounts(const i32 *sI, const i32 *sJ, i64 nseg, i64 *uc, i64 *lc,
                                uint8_t *lflag) {
  i64 s = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  atomicAdd((unsigned long long *)&uc[sI[s]], 1ull);
  bool low = sJ[s] > sI[s];
  if (low) atomicAdd((unsigned long long *)&lc[sJ[s]], 1ull);
  lflag[s] = low ? 1 : 0;
}

__global__ void k_add_i64(const i64 *a, const i64 *b, i64 n, i64 *c) {
  i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) c[i] = a[i] + b[i];
}

__global__ void k_lower_keys(const i32 *lidx, const i32 *sJ, i64 nl, u64 *keys, u32 *vals) {
  i64 k = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nl) return;
  keys[k] = (u64)(u32)sJ[lidx[k]];
  vals[k] = (u32)lidx[k];
}

__global__ void k_gal_fill(i64 nc, const i64 *rp, const i64 *urp, const i64 *lrp, const i32 *sI,
                           const i32 *sJ, const double *sV, const u32 *lsorted, i32 *cci,
                           double *cv) {
  i64 r = warp_row();
  if (r >= nc) return;
  i64 base = rp[r];
  i64 l0 = lrp[r], l1 = lrp[r + 1];
  for (i64 k = l0 + lane_id(); k < l1; k += 32) {
    u32 s = lsorted[k];
    cci[base + (k - l0)] = sI[s];
    cv[base + (k - l0)] = sV[s];
  }
  base += l1 - l0;
  i64 u0 = urp[r], u1 = urp[r + 1];
  for (i64 k = u0 + lane_id(); k < u1; k += 32) {
    cci[base + (k - u0)] = sJ[k];
    cv[base + (k - u0)] = sV[k];
  }
}

__global__ void k_agg_prow(i64 n, const i32 *agg, i64 *prp, i32 *pci, double *pv) {
  i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    prp[i] = i;
    pci[i] = agg[i];
    pv[i] = 1.0;
  }
  if (i == n) prp[n] = n;
}

// ---------------------------------------------------------------------------
// aggregation: test vectors (AoS n x ntv), Jacobi with IgnoreDiagSR
// (smoothing.hpp:12-32,78-98); one warp per row, lane t owns test vector t.
__global__ void k_jacobi_tvs(const i64 *rp, const i32 *ci, const double *v, const i64 *dpos,
                             i64 n, int ntv, const double *xo, double *xn) {
  i64 i = warp_row();
  if (i >= n) return;
  int t = lane_id();
  if (t >= ntv) return;
  double y = 0;
  for (i64 k = rp[i]; k < rp[i + 1]; k++) {
    double a = v[k];
    if (a < 0) y = __dadd_rn(y, __dmul_rn(a, xo[(i64)ci[k] * ntv + t]));
  }
  const double w = 2.0 / 3.0;
  double d = v[dpos[i]];
  double x = xo[i * ntv + t];
  xn[i * ntv + t] = __dadd_rn(__ddiv_rn(__dmul_rn(w, __dsub_rn(0.0, y)), d),
                              __dmul_rn(__dsub_rn(1.0, w), x));
}

__global__ void k_tv_sq(const double *x, i64 n, int ntv, double *sq) {
  i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0;
  for (int t = 0; t < ntv; t++) s = __dadd_rn(s, __dmul_rn(x[i * ntv + t], x[i * ntv + t]));
  sq[i] = s;
}

// affinity values (aggregation.hpp:319-345) for entry (i, j) and for its
// transposed position (j, i); row and column maxima for Max scaling.
__global__ void k_aff_values(const i64 *rp, const i32 *ci, const double *v, i64 n, int ntv,
                             const double *x, const double *sq, int metric, double *aij,
                             double *aji, double *row_max, double *col_max) {
  i64 i = warp_row();
  if (i >= n) return;
  double rmax = 0.0, cmax = 0.0;
  for (i64 k = rp[i] + lane_id(); k < rp[i + 1]; k += 32) {
    i32 j = ci[k];
    double a1, a2;
    if (metric == LIGMG_STRENGTH_NONE) {
      a1 = a2 = (v[k] < 0) ? -v[k] : 0.0;
    } else if (j == i) {
      a1 = a2 = 0.0;
    } else if (metric == LIGMG_STRENGTH_AFFINITY) {
      double top = 0;
      for (int t = 0; t < ntv; t++)
        top = __dadd_rn(top, __dmul_rn(x[(i64)j * ntv + t], x[i * ntv + t]));
      double tt = __dmul_rn(top, top);
      double si = sq[i], sj = sq[j];
      a1 = __ddiv_rn(tt, __dmul_rn(__dmul_rn(__dmul_rn(sj, sj), si), si));
      a2 = __ddiv_rn(tt, __dmul_rn(__dmul_rn(__dmul_rn(si, si), sj), sj));
    } else {  // algebraic distance
      double mx = -1.0;
      for (int t = 0; t < ntv; t++) {
        double d = fabs(__dsub_rn(x[(i64)j * ntv + t], x[i * ntv + t]));
        if (t == 0 || d > mx) mx = d;
      }
      a1 = a2 = __ddiv_rn(1.0, mx);
    }
    aij[k] = a1;
    aji[k] = a2;
    rmax = fmax(rmax, a1);
    cmax = fmax(cmax, a2);
  }
  for (int o = 16; o > 0; o >>= 1) {
    rmax = fmax(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
    cmax = fmax(cmax, __shfl_xor_sync(0xffffffffu, cmax, o));
  }
  if (lane_id() == 0) {
    row_max[i] = rmax;
    col_max[i] = cmax;
  }
}

__device__ __forceinline__ double dmax_ref(double a, double b) { return (a < b) ? b : a; }

// Sequential per-row sums for the sum-based scalings (aggregation.hpp:352-367):
// mode 0: row sums of a(i,.) (entry order = ascending column);
// mode 1: column sums of a(.,i) = sums of the transposed values over row i;
// mode 2: column sums of the row-scaled matrix, a(j,i) / rowsum[j].
__global__ void k_aff_sums(const i64 *rp, const i32 *ci, i64 n, const double *aij,
                           const double *aji, const double *rowsum, int mode, double *out) {
  i64 i = warp_row();
  if (i >= n) return;
  unsigned lane = lane_id();
  double acc = 0.0;
  for (i64 base = rp[i]; base < rp[i + 1]; base += 32) {
    i64 k = base + lane;
    double v = 0.0;
    bool in = k < rp[i + 1];
    if (in) {
      if (mode == 0) v = aij[k];
      else if (mode == 1) v = aji[k];
      else v = __ddiv_rn(aji[k], rowsum[ci[k]]);
    }
    unsigned m = __ballot_sync(0xffffffffu, in);
    for (int q = 0; q < 32; q++) {
      double t = __shfl_sync(0xffffffffu, v, q);
      if (m & (1u << q)) acc = __dadd_rn(acc, t);
    }
  }
  if (lane == 0) out[i] = acc;
}

struct AffScale {
  int mode;
  const double *row_max, *col_max;  // MAX
  const double *rsum, *csum;        // ROW/SYM: rsum; COLUMN: csum; ROWCOLUMN: rsum + csum
};

// scaled value at (i, j) given the raw values a1 = a(i, j) and a2 = a(j, i)
__device__ __forceinline__ double aff_scaled(const AffScale &S, i64 i, i32 j, double a1,
                                             double a2) {
  switch (S.mode) {
    case LIGMG_AFF_MAX: return __ddiv_rn(a1, dmax_ref(S.row_max[i], S.col_max[j]));
    case LIGMG_AFF_ROW: return __ddiv_rn(a1, S.rsum[i]);
    case LIGMG_AFF_COLUMN: return __ddiv_rn(a1, S.csum[j]);
    case LIGMG_AFF_ROWCOLUMN: return __ddiv_rn(__ddiv_rn(a1, S.rsum[i]), S.csum[j]);
    case LIGMG_AFF_SYM: {  // (Aff^T + Aff) / 2 after row scaling (:361-367)
      double r1 = __ddiv_rn(a1, S.rsum[i]), r2 = __ddiv_rn(a2, S.rsum[j]);
      return __ddiv_rn(__dadd_rn(r2, r1), 2.0);
    }
    default: return a1;
  }
}

// Max scaling + prune (:368-401), kept counts per row, and column sums
// (:863-864) accumulated sequentially in ascending row order.
__global__ void k_aff_scale(const i64 *rp, const i32 *ci, i64 n, const double *aij,
                            const double *aji, AffScale S, double thresh, i64 *kcnt,
                            double *colsum) {
  i64 i = warp_row();
  if (i >= n) return;
  unsigned lane = lane_id();
  i64 cnt = 0;
  double cs = 0.0;
  for (i64 base = rp[i]; base < rp[i + 1]; base += 32) {
    i64 k = base + lane;
    bool in = k < rp[i + 1];
    double s1 = 0, s2 = 0;
    bool keep1 = false, keep2 = false;
    if (in) {
      i32 j = ci[k];
      s1 = aff_scaled(S, i, j, aij[k], aji[k]);  // entry (i, j)
      s2 = aff_scaled(S, j, (i32)i, aji[k], aij[k]);  // transposed entry (j, i)
      keep1 = !(s1 < thresh);
      keep2 = !(s2 < thresh);
    }
    cnt += __popc(__ballot_sync(0xffffffffu, keep1));
    unsigned m2 = __ballot_sync(0xffffffffu, keep2);
    for (int q = 0; q < 32; q++) {
      double val = __shfl_sync(0xffffffffu, s2, q);
      if (m2 & (1u << q)) cs = __dadd_rn(cs, val);
    }
  }
  if (lane == 0) {
    kcnt[i] = cnt;
    colsum[i] = cs;
  }
}

__global__ void k_aff_fill(const i64 *rp, const i32 *ci, i64 n, const double *aij,
                           const double *aji, AffScale S, double thresh, const i64 *arp,
                           i32 *aci, double *av) {
  i64 i = warp_row();
  if (i >= n) return;
  unsigned lane = lane_id();
  i64 o = arp[i];
  for (i64 base = rp[i]; base < rp[i + 1]; base += 32) {
    i64 k = base + lane;
    bool keep = false;
    double s1 = 0;
    i32 j = 0;
    if (k < rp[i + 1]) {
      j = ci[k];
      s1 = aff_scaled(S, i, j, aij[k], aji[k]);
      keep = !(s1 < thresh);
    }
    unsigned m = __ballot_sync(0xffffffffu, keep);
    if (keep) {
      i64 p = o + __popc(m & lanemask_lt());
      aci[p] = j;
      av[p] = s1;
    }
    o += __popc(m);
  }
}

// ---- voting (aggregation.hpp:408-561,702-750) ------------------------------
enum : int32_t { ST_Seed = 0, ST_SeedNeighbor = 1, ST_Decided = 2, ST_DecidedRoot = 3,
                 ST_Undecided = 4 };
enum : int32_t { VS_Seed = 0, VS_Undecided = 1, VS_Decided = 2 };

__device__ __forceinline__ int vs_prio(int s) { return s == VS_Seed ? 2 : (s == VS_Undecided ? 1 : 0); }

// AggSR add: with positions included, the left fold of the reference is the
// maximum of the key (state priority, weight, position).
struct VCand {
  int st;
  i32 ind;
  double w;
  i64 pos;
};
__device__ __forceinline__ bool vbetter(const VCand &b, const VCand &a) {  // b beats a?
  int pb = vs_prio(b.st), pa = vs_prio(a.st);
  if (pb != pa) return pb > pa;
  if (b.w != a.w) return b.w > a.w;
  return b.pos > a.pos;
}

__global__ void k_vote(const i64 *arp, const i32 *aci, const double *av, i64 n, const i32 *st,
                       const i32 *ind, double thr, int nn, i32 *va_st, i32 *va_ind,
                       double *va_w) {
  i64 i = warp_row();
  if (i >= n) return;
  VCand best{VS_Decided, -1, -1.0, -1};  // AggSR::id()
  for (i64 k = arp[i] + lane_id(); k < arp[i + 1]; k += 32) {
    i32 j = aci[k];
    double w = av[k];
    int s = st[j];
    VCand c;
    c.ind = ind[j];
    c.w = w;
    c.pos = k;
    if (s == ST_Seed || (nn && s == ST_SeedNeighbor)) c.st = (w > thr) ? VS_Seed : VS_Decided;
    else if (s == ST_Undecided) c.st = VS_Undecided;
    else c.st = VS_Decided;
    if (vbetter(c, best)) best = c;
  }
  for (int o = 16; o > 0; o >>= 1) {
    VCand oth;
    oth.st = __shfl_xor_sync(0xffffffffu, best.st, o);
    oth.ind = __shfl_xor_sync(0xffffffffu, best.ind, o);
    oth.w = __shfl_xor_sync(0xffffffffu, best.w, o);
    oth.pos = __shfl_xor_sync(0xffffffffu, best.pos, o);
    if (vbetter(oth, best)) best = oth;
  }
  if (lane_id() == 0) {
    va_st[i] = best.st;
    va_ind[i] = best.ind;
    va_w[i] = best.w;
  }
}

__global__ void k_tally_flags(i64 n, const i32 *st, const i32 *va_ind, const double *va_w,
                              double thr, i32 *voting_for, uint8_t *voter) {
  i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  i32 t = va_ind[i];
  bool v = st[i] == ST_Undecided && t >= 0 && va_w[i] >= thr && (i64)t != i;
  voting_for[i] = v ? t : -1;
  voter[i] = v ? 1 : 0;
}

__global__ void k_voter_keys(const i32 *voters, i64 nv, const i32 *va_ind, u64 *keys, u32 *vals) {
  i64 k = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nv) return;
  i32 i = voters[k];
  keys[k] = (u64)(u32)va_ind[i];
  vals[k] = (u32)i;
}

__global__ void k_tally_segsum(const u64 *keys, const u32 *vals, const i32 *starts, i64 nseg,
                               i64 T, const double *va_w, double *new_votes) {
  i64 s = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  i64 b = starts[s], e = (s + 1 < nseg) ? starts[s + 1] : T;
  double acc = 0.0;
  for (i64 k = b; k < e; k++) acc = __dadd_rn(acc, va_w[vals[k]]);
  new_votes[keys[b]] = acc;
}

__global__ void k_votes_add(i64 n, const double *nv, double *votes) {
  i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) votes[i] = __dadd_rn(nv[i], votes[i]);
}

__global__ void k_mark(i64 n, int first_iter, int nn, double max_agg_size, double votes_to_seed,
                       const i32 *voting_for, const double *votes, const double *colsum,
                       const i32 *va_st, const i32 *va_ind, i32 *st, i32 *ind) {
  i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int s = st[i];
  if (s == ST_Decided || s == ST_DecidedRoot || s == ST_SeedNeighbor) return;
  if (s == ST_Seed) {
    if (votes[i] > max_agg_size) st[i] = ST_DecidedRoot;
    return;
  }
  i32 vf = voting_for[i];
  if (vf >= 0 && first_iter && (i64)voting_for[vf] == i) {
    if (i < vf) {
      st[i] = ST_Seed;
      ind[i] = (i32)i;
    } else {
      st[i] = nn ? ST_SeedNeighbor : ST_Decided;
      ind[i] = vf;
    }
  } else if (va_st[i] == VS_Seed) {
    st[i] = nn ? ST_SeedNeighbor : ST_Decided;
    ind[i] = va_ind[i];
  } else if (votes[i] >= __dmul_rn(votes_to_seed, colsum[i])) {
    st[i] = ST_Seed;
    ind[i] = (i32)i;
  }
}

// ---- reject_aggregates (aggregation.hpp:630-685) --------------------------
__device__ __forceinline__ bool st_decided(int x) {
  return x == ST_Decided || x == ST_DecidedRoot || x == ST_Seed || x == ST_SeedNeighbor;
}
__global__ void k_rej_count(i64 n, const i32 *st, const i32 *ind, i64 *size, i64 *mcnt,
                            uint8_t *member) {
  i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int s = st[i];
  if (st_decided(s) && ind[i] >= 0) atomicAdd((unsigned long long *)&size[ind[i]], 1ull);
  bool m = (s == ST_Decided || s == ST_SeedNeighbor) && ind[i] >= 0;
  member[i] = m ? 1 : 0;
  if (m) atomicAdd((unsigned long long *)&mcnt[ind[i]], 1ull);
}
__global__ void k_rej_keys(const i32 *list, i64 m, const i32 *ind, u64 *keys, u32 *vals) {
  i64 k = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  keys[k] = (u64)(u32)ind[list[k]];
  vals[k] = (u32)list[k];
}
// members sorted by (root, index); reset the first csz^2/(size-1) of every
// root whose aggregate is larger than max_size; flag that root
__global__ void k_rej_apply(i64 m, const u64 *keys, const u32 *vals, const i64 *mstart,
                            const i64 *mcnt, const i64 *size, i64 max_size, i32 *st, i32 *ind,
                            uint8_t *rootflag) {
  i64 k = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  i64 root = (i64)keys[k];
  i64 sz = size[root];
  if (sz <= max_size) return;
  i64 csz = mcnt[root];
  i64 local = csz * csz / (sz - 1);
  if (k - mstart[root] < local) {
    st[vals[k]] = ST_Undecided;
    ind[vals[k]] = -1;
  }
  rootflag[root] = 1;
}
__global__ void k_rej_roots(i64 n, const uint8_t *rootflag, i32 *st) {
  i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && rootflag[i]) st[i] = ST_DecidedRoot;
}

// ---- conductance_rejection with ext_int_ratio (aggregation.hpp:563-628,752-778)
__global__ void k_ext_int_ratio(const i64 *rp, const i32 *ci, const double *v, i64 n,
                                const i32 *st, const i32 *ind, double *ratio) {
  i64 i = warp_row();
  if (i >= n) return;
  unsigned lane = lane_id();
  double ext = 0.0, inn = 0.0;
  bool me = st_decided(st[i]);
  if (me) {
    for (i64 base = rp[i]; base < rp[i + 1]; base += 32) {
      i64 k = base + lane;
      int kind = 0;  // 0: skip, 1: internal, 2: external
      double a = 0;
      if (k < rp[i + 1]) {
        i32 j = ci[k];
        if (j != i) {
          a = v[k];
          kind = (st_decided(st[j]) && ind[j] == ind[i]) ? 1 : 2;
        }
      }
      for (int q = 0; q < 32; q++) {
        int kq = __shfl_sync(0xffffffffu, kind, q);
        double aq = __shfl_sync(0xffffffffu, a, q);
        if (kq == 1) inn = __dsub_rn(inn, aq);
        else if (kq == 2) ext = __dsub_rn(ext, aq);
      }
    }
  }
  if (lane == 0) ratio[i] = __ddiv_rn(ext, inn);
}
__global__ void k_conductance(i64 n, const double *ratio, double thr, int to_seed, i32 *st,
                              i32 *ind) {
  i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int s = st[i];
  if (ratio[i] > thr && (s == ST_Decided || s == ST_SeedNeighbor)) {
    st[i] = to_seed ? ST_Seed : ST_Undecided;
    ind[i] = (i32)i;
  }
}

__global__ void k_init_states(i64 n, i32 *st, i32 *ind) {
  i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    st[i] = ST_Undecided;
    ind[i] = (i32)i;
  }
}

__global__ void k_root_flags(i64 n, i32 *ind, i32 *is_root) {
  i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  i32 r = ind[i];
  if (r < 0) {
    r = (i32)i;
    ind[i] = r;
  }
  is_root[r] = 1;  // idempotent
}

__global__ void k_agg_ids(i64 n, const i32 *ind, const i32 *rank, i32 *agg) {
  i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) agg[i] = rank[ind[i]];
}

__global__ void k_agg_keys(i64 n, const i32 *agg, u64 *keys, u32 *vals, i64 *cnt) {
  i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  keys[i] = (u64)(u32)agg[i];
  vals[i] = (u32)i;
  atomicAdd((unsigned long long *)&cnt[agg[i]], 1ull);
}

__global__ void k_u32_to_i32(const u32 *a, i64 n, i32 *b) {
  i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (i32)a[i];
}

// ---- coarse pseudo-inverse: Gauss-Jordan on M = A + 11'/n (SPD) -----------
// value of the constant projector 11'/n_s at (r, k): 1/n_s within a segment
__device__ __forceinline__ double proj_entry(i64 r, i64 k, i64 n, const i32 *rowseg,
                                             const i64 *segptr) {
  if (!rowseg) return 1.0 / (double)n;
  i32 a = rowseg[r];
  if (a != rowseg[k]) return 0.0;
  return 1.0 / (double)(segptr[a + 1] - segptr[a]);
}

__global__ void k_dense_init(const i64 *rp, const i32 *ci, const double *v, i64 n, double *M,
                             double *I, const i32 *rowseg, const i64 *segptr) {
  i64 r = warp_row();
  if (r >= n) return;
  for (i64 k = lane_id(); k < n; k += 32) {
    M[r * n + k] = proj_entry(r, k, n, rowseg, segptr);
    I[r * n + k] = (k == r) ? 1.0 : 0.0;
  }
  __syncwarp();
  for (i64 k = rp[r] + lane_id(); k < rp[r + 1]; k += 32) M[r * n + ci[k]] += v[k];
}

__global__ void k_gj_pivot(double *M, double *I, i64 n, i64 p, int *bad) {
  // scale pivot row
  double piv = M[p * n + p];
  if (!(piv > 0)) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *bad = 1;
    return;
  }
  double inv = 1.0 / piv;
  for (i64 k = (i64)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (i64)gridDim.x * blockDim.x) {
    I[p * n + k] *= inv;
    if (k != p) M[p * n + k] *= inv;
  }
}

__global__ void k_gj_finish_pivot(double *M, i64 n, i64 p) { M[p * n + p] = 1.0; }

__global__ void k_gj_eliminate(double *M, double *I, i64 n, i64 p, const double *fac) {
  i64 r = blockIdx.y;
  if (r == p) return;
  double f = fac[r];
  if (f == 0.0) return;
  for (i64 k = (i64)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (i64)gridDim.x * blockDim.x) {
    M[r * n + k] -= f * M[p * n + k];
    I[r * n + k] -= f * I[p * n + k];
  }
}

__global__ void k_gj_factors(const double *M, i64 n, i64 p, double *fac) {
  i64 r = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (r < n) fac[r] = M[r * n + p];
}

__global__ void k_sub_proj(double *I, i64 n, const i32 *rowseg, const i64 *segptr) {
  i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n * n) I[t] -= proj_entry(t / n, t % n, n, rowseg, segptr);
}

}  // namespace

// ===========================================================================
ligmg_status gpu_validate(const DCsr<double> &A, cudaStream_t s) {
  DBuf<int> err(1, s);
  int big = 1 << 30;
  err.upload(&big, 1);
  k_validate<<<grid_for(A.n * 32, kBlock), kBlock, 0, s>>>(A.rp.p, A.ci.p, A.v.p, A.n, err.p);
  LG_LAUNCH();
  int e = read_scalar(err.p, s);
  return e == big ? LIGMG_OK : e;
}

void gpu_transpose(const DCsr<double> &A, DCsr<double> &T, cudaStream_t s) {
  i64 nnz = A.nnz;
  T.n = A.m;
  T.m = A.n;
  T.nnz = nnz;
  T.rp.alloc(T.n + 1, s);
  T.ci.alloc(nnz, s);
  T.v.alloc(nnz, s);
  DBuf<i64> cnt(T.n + 1, s);
  cnt.zero();
  DBuf<i32> rows(nnz, s);
  DBuf<u64> keys(nnz, s);
  DBuf<u32> perm(nnz, s);
  if (nnz > 0) {
    k_expand_rows<<<grid_for(A.n * 32, kBlock), kBlock, 0, s>>>(A.rp.p, A.n, rows.p);
    k_count_cols<<<grid_for(nnz, 256), 256, 0, s>>>(A.ci.p, nnz, cnt.p);
    k_cols_to_keys<<<grid_for(nnz, 256), 256, 0, s>>>(A.ci.p, nnz, keys.p);
    k_iota_u32<<<grid_for(nnz, 256), 256, 0, s>>>(perm.p, nnz);
    LG_LAUNCH();
    radix_sort_pairs(keys.p, perm.p, nnz, bits_for(A.m - 1), s);
    k_transpose_fill<<<grid_for(nnz, 256), 256, 0, s>>>(perm.p, rows.p, A.v.p, nnz, T.ci.p,
                                                         T.v.p);
    LG_LAUNCH();
  }
  exclusive_scan<i64>(cnt.p, T.rp.p, T.n + 1, s);
}

void gpu_elimination(const DCsr<double> &A, int elim_degree, double elim_factor,
                     ElimResult &out, cudaStream_t s) {
  i64 n = A.n;
  DBuf<uint8_t> cand(n, s);
  DBuf<i32> keep(n, s), tot(1, s);
  out.pos.alloc(n, s);
  i32 *posp = out.pos.p;
  DBuf<i64> dpos(n, s);
  k_elim_cand<<<grid_for(n * 32, kBlock), kBlock, 0, s>>>(A.rp.p, A.v.p, n, elim_degree, cand.p);
  k_elim_select<<<grid_for(n, 256), 256, 0, s>>>(A.rp.p, A.ci.p, A.v.p, n, cand.p, keep.p);
  LG_LAUNCH();
  exclusive_scan<i32>(keep.p, posp, n, s, tot.p);
  i64 num_no_elim = read_scalar(tot.p, s);
  out.accepted = !((double)num_no_elim > (double)n * elim_factor);  // :226
  if (!out.accepted) return;
  i64 nc = num_no_elim;
  out.nc = nc;
  out.new_id.alloc(n, s);
  k_new_ids<<<grid_for(n, 256), 256, 0, s>>>(keep.p, posp, n, out.new_id.p);
  k_diag_pos<<<grid_for(n, 256), 256, 0, s>>>(A.rp.p, A.ci.p, n, dpos.p);
  DBuf<i64> pcnt(n + 1, s);
  pcnt.zero();
  k_elim_pcount<<<grid_for(n, 256), 256, 0, s>>>(A.rp.p, A.ci.p, n, out.new_id.p, pcnt.p);
  LG_LAUNCH();
  out.P.n = n;
  out.P.m = nc;
  out.P.rp.alloc(n + 1, s);
  DBuf<i64> ptot(1, s);
  exclusive_scan<i64>(pcnt.p, out.P.rp.p, n + 1, s, ptot.p);
  out.P.nnz = read_scalar(ptot.p, s);
  out.P.ci.alloc(out.P.nnz, s);
  out.P.v.alloc(out.P.nnz, s);
  out.Q.alloc(n, s);
  k_elim_pfill<<<grid_for(n, 256), 256, 0, s>>>(A.rp.p, A.ci.p, A.v.p, n, out.new_id.p, dpos.p,
                                                 out.P.rp.p, out.P.ci.p, out.P.v.p, out.Q.p);
  LG_LAUNCH();
  gpu_transpose(out.P, out.R, s);
}

void gpu_galerkin(const DCsr<double> &A, const DCsr<double> &P, DCsr<double> &C,
                  cudaStream_t s) {
  i64 n = A.n, nnz = A.nnz;
  u64 nc = (u64)P.m;
  DBuf<i64> cnt(nnz + 1, s), off(nnz + 1, s);
  cnt.zero();
  k_gal_count<<<grid_for(n * 32, kBlock), kBlock, 0, s>>>(A.rp.p, A.ci.p, n, P.rp.p, P.ci.p,
                                                           cnt.p);
  LG_LAUNCH();
  exclusive_scan<i64>(cnt.p, off.p, nnz + 1, s);
  i64 T = read_scalar(off.p + nnz, s);
  DBuf<u64> keys(T, s);
  DBuf<u32> idx(T, s);
  DBuf<double> tv(T, s);
  k_gal_emit<<<grid_for(n * 32, kBlock), kBlock, 0, s>>>(A.rp.p, A.ci.p, A.v.p, n, P.rp.p,
                                                          P.ci.p, P.v.p, nc, off.p, keys.p,
                                                          idx.p, tv.p);
  LG_LAUNCH();
  radix_sort_pairs(keys.p, idx.p, T, bits_for((i64)(nc * nc) - 1), s);
  DBuf<uint8_t> flag(T, s);
  DBuf<i32> starts(T, s);
  k_seg_flags<<<grid_for(T, 256), 256, 0, s>>>(keys.p, T, flag.p);
  LG_LAUNCH();
  i64 nseg = compact_indices(flag.p, T, starts.p, s);
  DBuf<i32> sI(nseg, s), sJ(nseg, s);
  DBuf<double> sV(nseg, s);
  k_gal_segsum<<<grid_for(nseg, 256), 256, 0, s>>>(keys.p, idx.p, tv.p, starts.p, nseg, T, nc,
                                                    sI.p, sJ.p, sV.p);
  LG_LAUNCH();
  // mirror into a full symmetric CSR
  DBuf<i64> uc(nc + 1, s), lc(nc + 1, s), tc(nc + 1, s);
  uc.zero();
  lc.zero();
  DBuf<uint8_t> lflag(nseg, s);
  k_gal_rowcounts<<<grid_for(nseg, 256), 256, 0, s>>>(sI.p, sJ.p, nseg, uc.p, lc.p, lflag.p);
  k_add_i64<<<grid_for(nc + 1, 256), 256, 0, s>>>(uc.p, lc.p, nc + 1, tc.p);
  LG_LAUNCH();
  DBuf<i64> urp(nc + 1, s), lrp(nc + 1, s);
  C.n = C.m = (i64)nc;
  C.rp.alloc(nc + 1, s);
  exclusive_scan<i64>(uc.p, urp.p, nc + 1, s);
  exclusive_scan<i64>(lc.p, lrp.p, nc + 1, s);
  exclusive_scan<i64>(tc.p, C.rp.p, nc + 1, s);
  DBuf<i32> lidx(nseg, s);
  i64 nl = compact_indices(lflag.p, nseg, lidx.p, s);
  DBuf<u64> lkeys(nl, s);
  DBuf<u32> lsorted(nl, s);
  if (nl > 0) {
    k_lower_keys<<<grid_for(nl, 256), 256, 0, s>>>(lidx.p, sJ.p, nl, lkeys.p, lsorted.p);
    LG_LAUNCH();
    radix_sort_pairs(lkeys.p, lsorted.p, nl, bits_for((i64)nc - 1), s);
  }
  C.nnz = nseg + nl;
  C.ci.alloc(C.nnz, s);
  C.v.alloc(C.nnz, s);
  k_gal_fill<<<grid_for((i64)nc * 32, kBlock), kBlock, 0, s>>>(
      (i64)nc, C.rp.p, urp.p, lrp.p, sI.p, sJ.p, sV.p, lsorted.p, C.ci.p, C.v.p);
  LG_LAUNCH();
}

namespace {
__global__ void k_ra_keys(const i64 *rp, const i32 *ci, i64 n, const i32 *agg, int cbits,
                          u64 *keys, u32 *idx) {
  const i64 i = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const u64 hi = (u64)agg[i] << cbits;
  for (i64 k = rp[i]; k < rp[i + 1]; k++) {
    keys[k] = hi | (u64)ci[k];
    idx[k] = (u32)k;
  }
}
__global__ void k_seg_heads(const u64 *keys, i64 m, uint8_t *head) {
  const i64 p = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (p < m) head[p] = (p == 0 || keys[p] != keys[p - 1]) ? 1 : 0;
}
// one thread per (aggregate, column) segment: the member entries summed in
// sorted (stable: ascending member row) order; row counts of R A
__global__ void k_ra_sum(const u64 *keys, const u32 *idx, const double *v, i64 m,
                         const i32 *starts, i64 nseg, int cbits, u64 cmask, i32 *racol,
                         double *raval, i64 *rcnt) {
  const i64 g = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= nseg) return;
  const i64 b = starts[g], e = g + 1 < nseg ? starts[g + 1] : m;
  double acc = 0.0;
  for (i64 p = b; p < e; p++) acc = __dadd_rn(acc, v[idx[p]]);
  racol[g] = (i32)(keys[b] & cmask);
  raval[g] = acc;
  atomicAdd((unsigned long long *)&rcnt[keys[b] >> cbits], 1ull);
}
__global__ void k_cr_count(i64 nc, const i64 *mrp, const i64 *rarp, i64 *cnt) {
  const i64 I = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (I < nc) cnt[I] = (mrp[I + 1] - mrp[I]) + (rarp[I + 1] - rarp[I]);
}
__global__ void k_cr_fill(i64 nc, i64 n, const i64 *mrp, const i32 *members, const i64 *rarp,
                          const i32 *racol, const double *raval, const i64 *crp, i32 *cci,
                          double *cv) {
  const i64 I = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= nc) return;
  i64 p = crp[I];
  for (i64 q = mrp[I]; q < mrp[I + 1]; q++) {
    cci[p] = members[q];
    cv[p++] = 1.0;
  }
  for (i64 q = rarp[I]; q < rarp[I + 1]; q++) {
    cci[p] = (i32)(n + racol[q]);
    cv[p++] = -raval[q];
  }
}
}  // namespace

void gpu_restrict_residual_matrix(const DCsr<double> &A, const i32 *agg, const i64 *mrp,
                                  const i32 *members, i64 nc, DCsr<double> &C, cudaStream_t s) {
  const i64 n = A.n, nnz = A.nnz;
  if (2 * n > (i64)INT32_MAX) throw Error(LIGMG_ERR_UNSUPPORTED, "level too large");
  const int cbits = bits_for(n - 1), abits = bits_for(nc - 1);
  DBuf<u64> keys(std::max<i64>(nnz, 1), s);
  DBuf<u32> idx(std::max<i64>(nnz, 1), s);
  k_ra_keys<<<grid_for(n, 256), 256, 0, s>>>(A.rp.p, A.ci.p, n, agg, cbits, keys.p, idx.p);
  LG_LAUNCH();
  radix_sort_pairs(keys.p, idx.p, nnz, cbits + abits, s);
  DBuf<uint8_t> head(std::max<i64>(nnz, 1), s);
  k_seg_heads<<<grid_for(nnz, 256), 256, 0, s>>>(keys.p, nnz, head.p);
  LG_LAUNCH();
  DBuf<i32> starts(std::max<i64>(nnz, 1), s);
  const i64 nseg = compact_indices(head.p, nnz, starts.p, s);
  DBuf<i32> racol(std::max<i64>(nseg, 1), s);
  DBuf<double> raval(std::max<i64>(nseg, 1), s);
  DBuf<i64> rcnt(nc + 1, s), rarp(nc + 1, s);
  rcnt.zero();
  k_ra_sum<<<grid_for(nseg, 256), 256, 0, s>>>(keys.p, idx.p, A.v.p, nnz, starts.p, nseg, cbits,
                                               (1ull << cbits) - 1, racol.p, raval.p, rcnt.p);
  LG_LAUNCH();
  exclusive_scan<i64>(rcnt.p, rarp.p, nc + 1, s);
  DBuf<i64> ccnt(nc + 1, s);
  ccnt.zero();
  k_cr_count<<<grid_for(nc, 256), 256, 0, s>>>(nc, mrp, rarp.p, ccnt.p);
  LG_LAUNCH();
  C.n = nc;
  C.m = 2 * n;
  C.rp.alloc(nc + 1, s);
  DBuf<i64> tot(1, s);
  exclusive_scan<i64>(ccnt.p, C.rp.p, nc + 1, s, tot.p);
  C.nnz = read_scalar(tot.p, s);
  C.ci.alloc(C.nnz, s);
  C.v.alloc(C.nnz, s);
  k_cr_fill<<<grid_for(nc, 256), 256, 0, s>>>(nc, n, mrp, members, rarp.p, racol.p, raval.p,
                                               C.rp.p, C.ci.p, C.v.p);
  LG_LAUNCH();
  LG_CUDA(cudaStreamSynchronize(s));
}

void gpu_galerkin_agg(const DCsr<double> &A, const i32 *agg, i64 nc, DCsr<double> &C,
                      cudaStream_t s) {
  DCsr<double> P;
  P.n = A.n;
  P.m = nc;
  P.nnz = A.n;
  P.rp.alloc(A.n + 1, s);
  P.ci.alloc(A.n, s);
  P.v.alloc(A.n, s);
  k_agg_prow<<<grid_for(A.n + 1, 256), 256, 0, s>>>(A.n, agg, P.rp.p, P.ci.p, P.v.p);
  LG_LAUNCH();
  gpu_galerkin(A, P, C, s);
}

void gpu_aggregation(const DCsr<double> &A, const AggParams &p, const double *tvs_host,
                     AggResult &out, cudaStream_t s) {
  i64 n = A.n, nnz = A.nnz;
  int ntv = p.num_tvs;
  bool need_tvs = p.strength_metric == LIGMG_STRENGTH_AFFINITY ||
                  p.strength_metric == LIGMG_STRENGTH_ALGEBRAIC_DISTANCE;
  if (need_tvs && (ntv < 1 || ntv > 32)) throw Error(LIGMG_ERR_UNSUPPORTED, "num_tvs");
  DBuf<i64> dpos(n, s);
  k_diag_pos<<<grid_for(n, 256), 256, 0, s>>>(A.rp.p, A.ci.p, n, dpos.p);
  LG_LAUNCH();
  DBuf<double> xa, xb, sq(n, s);
  if (need_tvs) {
    // tvs_host is num_tvs x n; the kernels use n x num_tvs (AoS)
    std::vector<double> aos((size_t)n * ntv);
    for (int t = 0; t < ntv; t++)
      for (i64 i = 0; i < n; i++) aos[(size_t)i * ntv + t] = tvs_host[(size_t)t * n + i];
    xa.alloc(n * ntv, s);
    xb.alloc(n * ntv, s);
    xa.upload(aos.data(), n * ntv);
    LG_CUDA(cudaStreamSynchronize(s));
    for (int it = 0; it < p.tvs_smooth; it++) {
      k_jacobi_tvs<<<grid_for(n * 32, kBlock), kBlock, 0, s>>>(A.rp.p, A.ci.p, A.v.p, dpos.p, n,
                                                               ntv, xa.p, xb.p);
      LG_LAUNCH();
      std::swap(xa, xb);
    }
    k_tv_sq<<<grid_for(n, 256), 256, 0, s>>>(xa.p, n, ntv, sq.p);
    LG_LAUNCH();
    out.tvs = std::move(xa);
  }
  DBuf<double> aij(nnz, s), aji(nnz, s), rmax(n, s), cmax(n, s);
  k_aff_values<<<grid_for(n * 32, kBlock), kBlock, 0, s>>>(
      A.rp.p, A.ci.p, A.v.p, n, ntv, out.tvs.p, sq.p, p.strength_metric, aij.p, aji.p, rmax.p,
      cmax.p);
  LG_LAUNCH();
  AffScale S{p.aff_scaling, rmax.p, cmax.p, nullptr, nullptr};
  DBuf<double> rsum, csum;
  int sm = p.aff_scaling;
  if (sm == LIGMG_AFF_ROW || sm == LIGMG_AFF_ROWCOLUMN || sm == LIGMG_AFF_SYM) {
    rsum.alloc(n, s);
    k_aff_sums<<<grid_for(n * 32, kBlock), kBlock, 0, s>>>(A.rp.p, A.ci.p, n, aij.p, aji.p,
                                                           nullptr, 0, rsum.p);
    LG_LAUNCH();
    S.rsum = rsum.p;
  }
  if (sm == LIGMG_AFF_COLUMN || sm == LIGMG_AFF_ROWCOLUMN) {
    csum.alloc(n, s);
    k_aff_sums<<<grid_for(n * 32, kBlock), kBlock, 0, s>>>(
        A.rp.p, A.ci.p, n, aij.p, aji.p, rsum.p, sm == LIGMG_AFF_ROWCOLUMN ? 2 : 1, csum.p);
    LG_LAUNCH();
    S.csum = csum.p;
  }
  DBuf<i64> kcnt(n + 1, s);
  kcnt.zero();
  out.colsum.alloc(n, s);
  k_aff_scale<<<grid_for(n * 32, kBlock), kBlock, 0, s>>>(A.rp.p, A.ci.p, n, aij.p, aji.p, S,
                                                           p.thresh, kcnt.p, out.colsum.p);
  LG_LAUNCH();
  DCsr<double> &F = out.aff;
  F.n = F.m = n;
  F.rp.alloc(n + 1, s);
  DBuf<i64> atot(1, s);
  exclusive_scan<i64>(kcnt.p, F.rp.p, n + 1, s, atot.p);
  F.nnz = read_scalar(atot.p, s);
  F.ci.alloc(F.nnz, s);
  F.v.alloc(F.nnz, s);
  k_aff_fill<<<grid_for(n * 32, kBlock), kBlock, 0, s>>>(A.rp.p, A.ci.p, n, aij.p, aji.p, S,
                                                          p.thresh, F.rp.p, F.ci.p, F.v.p);
  LG_LAUNCH();
  aij.release();
  aji.release();
  // voting iterations
  out.st.alloc(n, s);
  out.ind.alloc(n, s);
  out.votes.alloc(n, s);
  out.votes.zero();
  k_init_states<<<grid_for(n, 256), 256, 0, s>>>(n, out.st.p, out.ind.p);
  LG_LAUNCH();
  DBuf<i32> va_st(n, s), va_ind(n, s), vfor(n, s), voters(n, s), starts(n, s);
  DBuf<double> va_w(n, s), nv(n, s);
  DBuf<uint8_t> vflag(n, s), sflag(n, s);
  DBuf<u64> vkeys(n, s);
  DBuf<u32> vvals(n, s);
  int key_bits = bits_for(n - 1);
  for (int iter = 0; iter < p.agg_iters; iter++) {
    double thr = p.agg_init_factor * std::pow(p.agg_iter_factor, iter);  // :886
    k_vote<<<grid_for(n * 32, kBlock), kBlock, 0, s>>>(F.rp.p, F.ci.p, F.v.p, n, out.st.p,
                                                        out.ind.p, thr,
                                                        p.neighbor_of_neighbor ? 1 : 0, va_st.p,
                                                        va_ind.p, va_w.p);
    k_tally_flags<<<grid_for(n, 256), 256, 0, s>>>(n, out.st.p, va_ind.p, va_w.p, thr, vfor.p,
                                                    vflag.p);
    LG_LAUNCH();
    i64 nvot = compact_indices(vflag.p, n, voters.p, s);
    nv.zero();
    if (nvot > 0) {
      k_voter_keys<<<grid_for(nvot, 256), 256, 0, s>>>(voters.p, nvot, va_ind.p, vkeys.p, vvals.p);
      LG_LAUNCH();
      radix_sort_pairs(vkeys.p, vvals.p, nvot, key_bits, s);
      k_seg_flags<<<grid_for(nvot, 256), 256, 0, s>>>(vkeys.p, nvot, sflag.p);
      LG_LAUNCH();
      i64 nseg = compact_indices(sflag.p, nvot, starts.p, s);
      k_tally_segsum<<<grid_for(nseg, 256), 256, 0, s>>>(vkeys.p, vvals.p, starts.p, nseg, nvot,
                                                          va_w.p, nv.p);
      LG_LAUNCH();
    }
    k_votes_add<<<grid_for(n, 256), 256, 0, s>>>(n, nv.p, out.votes.p);
    k_mark<<<grid_for(n, 256), 256, 0, s>>>(n, iter == 0, p.neighbor_of_neighbor ? 1 : 0,
                                             p.max_agg_size, p.votes_to_seed, vfor.p,
                                             out.votes.p, out.colsum.p, va_st.p, va_ind.p,
                                             out.st.p, out.ind.p);
    LG_LAUNCH();
    if (p.max_agg_size > 0) {  // reject_aggregates
      DBuf<i64> size(n, s), mcnt(n + 1, s), mstart(n + 1, s);
      DBuf<uint8_t> member(n, s), rootflag(n, s);
      size.zero();
      mcnt.zero();
      rootflag.zero();
      k_rej_count<<<grid_for(n, 256), 256, 0, s>>>(n, out.st.p, out.ind.p, size.p, mcnt.p,
                                                   member.p);
      LG_LAUNCH();
      DBuf<i32> list(n, s);
      i64 m = compact_indices(member.p, n, list.p, s);
      if (m > 0) {
        exclusive_scan<i64>(mcnt.p, mstart.p, n + 1, s);
        DBuf<u64> keys(m, s);
        DBuf<u32> vals(m, s);
        k_rej_keys<<<grid_for(m, 256), 256, 0, s>>>(list.p, m, out.ind.p, keys.p, vals.p);
        LG_LAUNCH();
        radix_sort_pairs(keys.p, vals.p, m, key_bits, s);
        k_rej_apply<<<grid_for(m, 256), 256, 0, s>>>(m, keys.p, vals.p, mstart.p, mcnt.p, size.p,
                                                     (i64)p.max_agg_size, out.st.p, out.ind.p,
                                                     rootflag.p);
        k_rej_roots<<<grid_for(n, 256), 256, 0, s>>>(n, rootflag.p, out.st.p);
        LG_LAUNCH();
      }
    }
    if (iter >= p.agg_iters / 2 && p.rejection_ratio >= 0) {  // conductance_rejection
      DBuf<double> ratio(n, s);
      k_ext_int_ratio<<<grid_for(n * 32, kBlock), kBlock, 0, s>>>(A.rp.p, A.ci.p, A.v.p, n,
                                                                  out.st.p, out.ind.p, ratio.p);
      k_conductance<<<grid_for(n, 256), 256, 0, s>>>(n, ratio.p, p.rejection_ratio,
                                                     p.rejection_to_seed ? 1 : 0, out.st.p,
                                                     out.ind.p);
      LG_LAUNCH();
    }
  }
  // aggregate ids: rank of the root among roots (remove_zero_rows)
  DBuf<i32> is_root(n, s), ntot(1, s);
  out.rank.alloc(n, s);
  DBuf<i32> &rank = out.rank;
  is_root.zero();
  k_root_flags<<<grid_for(n, 256), 256, 0, s>>>(n, out.ind.p, is_root.p);
  LG_LAUNCH();
  exclusive_scan<i32>(is_root.p, rank.p, n, s, ntot.p);
  out.nc = read_scalar(ntot.p, s);
  out.agg.alloc(n, s);
  k_agg_ids<<<grid_for(n, 256), 256, 0, s>>>(n, out.ind.p, rank.p, out.agg.p);
  LG_LAUNCH();
  gpu_members(out.agg.p, n, out.nc, out.mrp, out.members, s);
}

void gpu_members(const i32 *agg, i64 n, i64 nc, DBuf<i64> &mrp, DBuf<i32> &members,
                 cudaStream_t s) {
  // members grouped by aggregate (R as CSR), ascending fine index
  DBuf<u64> mkeys(n, s);
  DBuf<u32> mvals(n, s);
  DBuf<i64> mcnt(nc + 1, s);
  mcnt.zero();
  k_agg_keys<<<grid_for(n, 256), 256, 0, s>>>(n, agg, mkeys.p, mvals.p, mcnt.p);
  LG_LAUNCH();
  radix_sort_pairs(mkeys.p, mvals.p, n, bits_for(nc - 1), s);
  members.alloc(n, s);
  k_u32_to_i32<<<grid_for(n, 256), 256, 0, s>>>(mvals.p, n, members.p);
  LG_LAUNCH();
  mrp.alloc(nc + 1, s);
  exclusive_scan<i64>(mcnt.p, mrp.p, nc + 1, s);
}

ligmg_status gpu_coarse_pinv(const DCsr<double> &A, DBuf<double> &out, cudaStream_t s,
                             const i32 *rowseg, const i64 *segptr) {
  i64 n = A.n;
  // dense n x n factor; the coarsening loop stops near nnz <= min_size, so a
  // coarse level this large means min_size was set far outside its range
  if (n > 16384) throw Error(LIGMG_ERR_UNSUPPORTED, "coarse level too large for a dense inverse");
  DBuf<double> M(n * n, s), fac(n, s);
  out.alloc(n * n, s);
  DBuf<int> bad(1, s);
  bad.zero();
  k_dense_init<<<grid_for(n * 32, kBlock), kBlock, 0, s>>>(A.rp.p, A.ci.p, A.v.p, n, M.p, out.p,
                                                            rowseg, segptr);
  LG_LAUNCH();
  unsigned gx = (unsigned)std::min<i64>(cdiv(n, 256), 64);
  for (i64 p = 0; p < n; p++) {
    k_gj_pivot<<<gx, 256, 0, s>>>(M.p, out.p, n, p, bad.p);
    k_gj_finish_pivot<<<1, 1, 0, s>>>(M.p, n, p);
    k_gj_factors<<<grid_for(n, 256), 256, 0, s>>>(M.p, n, p, fac.p);
    dim3 g(gx, (unsigned)n);
    k_gj_eliminate<<<g, 256, 0, s>>>(M.p, out.p, n, p, fac.p);
  }
  LG_LAUNCH();
  k_sub_proj<<<grid_for(n * n, 256), 256, 0, s>>>(out.p, n, rowseg, segptr);
  LG_LAUNCH();
  if (read_scalar(bad.p, s)) return LIGMG_ERR_DISCONNECTED;
  return LIGMG_OK;
}

}  // namespace lg
