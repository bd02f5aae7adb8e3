// ligmg_oracle.cpp — CPU restatement of LigMG's graph-Laplacian multigrid
// (setup + solve) at single-rank semantics.
//
// TEST INFRASTRUCTURE ONLY.  tests/, __graft_entry__.smoke() and bench.py's
// CPU-baseline leg use it to check or time against; the product library never
// does.
//
// Parity status: UNPINNED against the reference.  The reference (ligmg,
// header-only C++ over CombBLAS + PETSc + MPI) cannot be built here: MPI,
// PETSc, the CombBLAS fork and mxx are absent.  It also ships no golden
// vectors or tests.  Every function below follows the cited reference lines;
// where the reference delegates arithmetic to PETSc or CombBLAS (summation
// order of PSpGEMM, KSPCHEBYSHEV's recurrence and eigen estimate, KSPFCG's
// truncation, the CG+SOR coarse solve) the oracle DEFINES the semantics and
// the GPU library implements the same definition:
//   * Galerkin product: exactly symmetric; upper triangle (I <= J) summed
//     sequentially over fine entries (a, b) in row-major order, each term
//     (P(a,I) * A(a,b)) * P(b,J), then mirrored.
//   * Chebyshev: Saad, Iterative Methods for Sparse Linear Systems, 2nd ed.,
//     Alg. 12.1, on D^-1 A over [lower, upper] * lambda_max; lambda_max from
//     5 Jacobi-preconditioned CG steps (Lanczos tridiagonal) on a fixed
//     hashed right-hand side.
//   * Krylov: CG as PETSc KSPCG (Hestenes-Stiefel with beta = z'r ratio);
//     FCG as Notay's flexible CG with standard truncation (mmax directions);
//     the constant is projected out of the right-hand side and after every
//     preconditioner application (MatNullSpace semantics).
//   * Coarse level: dense pseudo-inverse L^+ = (L + 11'/n)^-1 - 11'/n.
// All FP64 arithmetic is compiled with -ffp-contract=off.
#include "ligmg_oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using i64 = int64_t;
using i32 = int32_t;

struct Csr {
  i64 n = 0;   // rows
  i64 m = 0;   // cols
  std::vector<i64> rp;
  std::vector<i32> ci;
  std::vector<double> v;
  i64 nnz() const { return (i64)ci.size(); }
};

// ---------------------------------------------------------------------------
// glibc rand() (TYPE_3 additive feedback generator, the default of srand()).
// Published algorithm: r[0] = seed (1 if seed == 0); r[i] = 16807 r[i-1]
// mod (2^31 - 1) by Schrage's method for i = 1..30; r[i] = r[i-31] for
// i = 31..33; r[i] = r[i-3] + r[i-31] mod 2^32 afterwards; the k-th output
// is r[k + 344] >> 1.  The reference draws its test vectors with rand()
// (combblas_extra.hpp:186-192).
struct GlibcRand {
  uint32_t ring[32];
  i64 i = 0;  // index of the next r[] to produce
  explicit GlibcRand(uint32_t seed) {
    int32_t r[34];
    int32_t s = (int32_t)(seed == 0 ? 1u : seed);
    r[0] = s;
    for (int k = 1; k < 31; k++) {
      int32_t hi = r[k - 1] / 127773;
      int32_t lo = r[k - 1] % 127773;
      int32_t word = 16807 * lo - 2836 * hi;
      if (word < 0) word += 2147483647;
      r[k] = word;
    }
    for (int k = 31; k < 34; k++) r[k] = r[k - 31];
    for (int k = 0; k < 34; k++) ring[k & 31] = (uint32_t)r[k];
    // note r[32], r[33] overwrite r[0], r[1] in the ring; both equal them
    i = 34;
    for (int k = 34; k < 344; k++) next_raw();
  }
  uint32_t next_raw() {
    uint32_t v = ring[(i - 31) & 31] + ring[(i - 3) & 31];
    ring[i & 31] = v;
    i++;
    return v;
  }
  int32_t next() { return (int32_t)(next_raw() >> 1); }
};

// ---------------------------------------------------------------------------
// Deterministic fixed-chunk reductions: identical results for any thread
// count (chunk partials summed in chunk order).
constexpr i64 kChunk = 16384;

double dot(const std::vector<double> &a, const std::vector<double> &b) {
  i64 n = (i64)a.size();
  i64 nch = (n + kChunk - 1) / kChunk;
  std::vector<double> part(nch, 0.0);
#pragma omp parallel for schedule(static)
  for (i64 c = 0; c < nch; c++) {
    double s = 0.0;
    i64 e = std::min(n, (c + 1) * kChunk);
    for (i64 i = c * kChunk; i < e; i++) s += a[i] * b[i];
    part[c] = s;
  }
  double s = 0.0;
  for (i64 c = 0; c < nch; c++) s += part[c];
  return s;
}

double sum(const std::vector<double> &a) {
  i64 n = (i64)a.size();
  i64 nch = (n + kChunk - 1) / kChunk;
  std::vector<double> part(nch, 0.0);
#pragma omp parallel for schedule(static)
  for (i64 c = 0; c < nch; c++) {
    double s = 0.0;
    i64 e = std::min(n, (c + 1) * kChunk);
    for (i64 i = c * kChunk; i < e; i++) s += a[i];
    part[c] = s;
  }
  double s = 0.0;
  for (i64 c = 0; c < nch; c++) s += part[c];
  return s;
}

// project the constant (MatNullSpaceRemove with has_cnst)
void remove_mean(std::vector<double> &x) {
  if (x.empty()) return;
  double mu = sum(x) / (double)x.size();
#pragma omp parallel for schedule(static)
  for (i64 i = 0; i < (i64)x.size(); i++) x[i] -= mu;
}

// y = A x, each row summed sequentially in ascending column order
// (PlusTimesSRing SpMV, util.hpp:467).
void spmv(const Csr &A, const std::vector<double> &x, std::vector<double> &y) {
  y.resize(A.n);
#pragma omp parallel for schedule(dynamic, 1024)
  for (i64 i = 0; i < A.n; i++) {
    double s = 0.0;
    for (i64 e = A.rp[i]; e < A.rp[i + 1]; e++) s += A.v[e] * x[A.ci[e]];
    y[i] = s;
  }
}

// r = b - A x   (residual, util.hpp:125-132)
void residual(const Csr &A, const std::vector<double> &x,
              const std::vector<double> &b, std::vector<double> &r) {
  spmv(A, x, r);
#pragma omp parallel for schedule(static)
  for (i64 i = 0; i < A.n; i++) r[i] = b[i] - r[i];
}

i64 diag_pos(const Csr &A, i64 i) {
  auto b = A.ci.begin() + A.rp[i], e = A.ci.begin() + A.rp[i + 1];
  auto it = std::lower_bound(b, e, (i32)i);
  if (it != e && *it == (i32)i) return it - A.ci.begin();
  return -1;
}

Csr transpose(const Csr &A) {
  Csr T;
  T.n = A.m;
  T.m = A.n;
  T.rp.assign(T.n + 1, 0);
  for (i64 e = 0; e < A.nnz(); e++) T.rp[A.ci[e] + 1]++;
  for (i64 i = 0; i < T.n; i++) T.rp[i + 1] += T.rp[i];
  T.ci.resize(A.nnz());
  T.v.resize(A.nnz());
  std::vector<i64> pos(T.rp.begin(), T.rp.end() - 1);
  for (i64 i = 0; i < A.n; i++)
    for (i64 e = A.rp[i]; e < A.rp[i + 1]; e++) {
      i64 p = pos[A.ci[e]]++;
      T.ci[p] = (i32)i;
      T.v[p] = A.v[e];
    }
  return T;
}

// ---------------------------------------------------------------------------
// Galerkin product Ac = P^T A P (triple_product, util.hpp:96-107; called at
// multigrid.hpp:142-143,156).  Exactly symmetric by construction: for I <= J
// the terms (P(a,I) * A(a,b)) * P(b,J) are summed sequentially in fine
// row-major (a, b) order; the lower triangle is the mirror image.  No
// numerical zeros are dropped (structural pattern kept).
Csr galerkin(const Csr &A, const Csr &P) {
  i64 nc = P.m;
  Csr PT = transpose(P);  // R = P^T: row I lists fine a ascending
  std::vector<std::vector<i32>> ucols(nc);
  std::vector<std::vector<double>> uvals(nc);
#pragma omp parallel
  {
    std::vector<double> acc(nc, 0.0);
    std::vector<char> mark(nc, 0);
    std::vector<i32> touched;
#pragma omp for schedule(dynamic, 64)
    for (i64 I = 0; I < nc; I++) {
      touched.clear();
      for (i64 ea = PT.rp[I]; ea < PT.rp[I + 1]; ea++) {
        i64 a = PT.ci[ea];
        double pa = PT.v[ea];
        for (i64 eb = A.rp[a]; eb < A.rp[a + 1]; eb++) {
          i64 b = A.ci[eb];
          double t = pa * A.v[eb];
          for (i64 ej = P.rp[b]; ej < P.rp[b + 1]; ej++) {
            i32 J = P.ci[ej];
            if (J < I) continue;
            double term = t * P.v[ej];
            if (!mark[J]) {
              mark[J] = 1;
              acc[J] = term;
              touched.push_back(J);
            } else {
              acc[J] = acc[J] + term;
            }
          }
        }
      }
      std::sort(touched.begin(), touched.end());
      ucols[I] = touched;
      uvals[I].resize(touched.size());
      for (size_t k = 0; k < touched.size(); k++) {
        uvals[I][k] = acc[touched[k]];
        mark[touched[k]] = 0;
      }
    }
  }
  // mirror: row r = lower entries (c, r) for c < r ascending, then upper
  Csr C;
  C.n = C.m = nc;
  C.rp.assign(nc + 1, 0);
  std::vector<i64> lower_cnt(nc, 0);
  for (i64 I = 0; I < nc; I++)
    for (i32 J : ucols[I])
      if (J > I) lower_cnt[J]++;
  for (i64 r = 0; r < nc; r++)
    C.rp[r + 1] = C.rp[r] + lower_cnt[r] + (i64)ucols[r].size();
  C.ci.resize(C.rp[nc]);
  C.v.resize(C.rp[nc]);
  std::vector<i64> fill(nc);
  for (i64 r = 0; r < nc; r++) fill[r] = C.rp[r];
  for (i64 I = 0; I < nc; I++)  // ascending I => lower parts come out sorted
    for (size_t k = 0; k < ucols[I].size(); k++) {
      i32 J = ucols[I][k];
      if (J > I) {
        i64 p = fill[J]++;
        C.ci[p] = (i32)I;
        C.v[p] = uvals[I][k];
      }
    }
  for (i64 r = 0; r < nc; r++) {
    i64 p = fill[r];
    for (size_t k = 0; k < ucols[r].size(); k++) {
      C.ci[p + k] = ucols[r][k];
      C.v[p + k] = uvals[r][k];
    }
  }
  return C;
}

// ---------------------------------------------------------------------------
// Input validation (the reference assumes a connected graph Laplacian,
// main.cpp:112-130 commented checks).
int validate(const Csr &A) {
  if (A.n <= 0 || A.n >= (i64)INT32_MAX) return LIGMG_ERR_INVALID_ARGUMENT;
  if (A.rp[0] != 0) return LIGMG_ERR_INVALID_ARGUMENT;
  for (i64 i = 0; i < A.n; i++) {
    if (A.rp[i + 1] < A.rp[i]) return LIGMG_ERR_INVALID_ARGUMENT;
    bool has_diag = false;
    for (i64 e = A.rp[i]; e < A.rp[i + 1]; e++) {
      i32 j = A.ci[e];
      if (j < 0 || j >= A.n) return LIGMG_ERR_INVALID_ARGUMENT;
      if (e > A.rp[i] && A.ci[e - 1] >= j) return LIGMG_ERR_NOT_SORTED;
      if (!std::isfinite(A.v[e])) return LIGMG_ERR_NONFINITE;
      if (j == i) {
        has_diag = true;
        if (!(A.v[e] > 0)) return LIGMG_ERR_BAD_DIAGONAL;
      } else if (A.v[e] > 0) {
        return LIGMG_ERR_POSITIVE_OFFDIAG;
      }
    }
    if (!has_diag) return LIGMG_ERR_BAD_DIAGONAL;
  }
  for (i64 i = 0; i < A.n; i++)
    for (i64 e = A.rp[i]; e < A.rp[i + 1]; e++) {
      i32 j = A.ci[e];
      auto b = A.ci.begin() + A.rp[j], en = A.ci.begin() + A.rp[j + 1];
      auto it = std::lower_bound(b, en, (i32)i);
      if (it == en || *it != (i32)i) return LIGMG_ERR_NOT_SYMMETRIC;
      if (A.v[it - A.ci.begin()] != A.v[e]) return LIGMG_ERR_NOT_SYMMETRIC;
    }
  return LIGMG_OK;
}

// ---------------------------------------------------------------------------
// Levels
enum class LT { Elim = 0, Agg = 1, Coarse = 2 };

// AggState / ST (aggregation.hpp:20,159-168); VoteAggState (:408)
enum ST : int32_t { Seed = 0, SeedNeighbor = 1, Decided = 2, DecidedRoot = 3, Undecided = 4 };
enum VS : int32_t { VSeed = 0, VUndecided = 1, VDecided = 2 };

struct Level {
  LT type;
  Csr A;                    // level input matrix (matrix(), levels.hpp:20)
  std::vector<double> invd; // 1 / A_ii
  double lmax = 0.0;        // Chebyshev eigenvalue estimate
  // elimination (elimination.hpp:20-68)
  Csr P, R;                 // P: n x nc, R = P^T
  std::vector<double> Q;    // diagonal of Q (0 on kept vertices)
  std::vector<i32> new_id;  // -1 when eliminated
  // aggregation (aggregation.hpp:176-274)
  std::vector<i32> agg;     // aggregate id per vertex
  i64 nc = 0;
  Csr aff;                  // pruned affinity (strength) matrix
  std::vector<double> dbg_tvs, dbg_colsum, dbg_votes;
  std::vector<i32> dbg_ind, dbg_st;
  // coarse (multigrid.hpp:41-84): dense pseudo-inverse
  std::vector<double> pinv;

  bool is_exact() const { return type == LT::Elim; }  // levels.hpp:18
  i64 work(const ligmg_options &o) const {
    if (type == LT::Agg)  // aggregation.hpp:247-250 (R and P have n entries)
      return (i64)(o.pre_smooth + o.post_smooth + 1) * A.nnz() + A.n + A.n + A.n;
    if (type == LT::Elim)  // elimination.hpp:58
      return P.nnz() + R.nnz() + (i64)std::count_if(Q.begin(), Q.end(),
                                                   [](double q) { return q != 0.0; });
    return A.nnz();  // multigrid.hpp:76
  }
};

// compute_degrees (elimination.hpp:71-80): nonzero values in the row minus one
std::vector<i64> compute_degrees(const Csr &A) {
  std::vector<i64> d(A.n);
  for (i64 i = 0; i < A.n; i++) {
    i64 c = 0;
    for (i64 e = A.rp[i]; e < A.rp[i + 1]; e++) c += (A.v[e] == 0) ? 0 : 1;
    d[i] = c - 1;
  }
  return d;
}

// single_elimination (elimination.hpp:157-345).  Returns false when the
// level is rejected (:226-228).
bool single_elimination(const Csr &A, const ligmg_options &o, Level &L) {
  i64 n = A.n;
  std::vector<i64> deg = compute_degrees(A);
  // candidates: degree <= max_degree (:186-190)
  std::vector<char> cand(n);
  for (i64 i = 0; i < n; i++) cand[i] = deg[i] <= o.elim_degree;
  // IndxHashMin SpMV (:82-154, :201-202): per row, the candidate with the
  // smallest index (std::hash<int> is the identity) among nonzero entries.
  // A candidate of degree < 0 (an empty row) can never be reached by the
  // multiply, so the "degree < 0" branches never fire.
  std::vector<char> elim(n, 0);
  i64 count = 0;
  for (i64 i = 0; i < n; i++) {
    i64 best = -1;
    for (i64 e = A.rp[i]; e < A.rp[i + 1]; e++) {
      i32 j = A.ci[e];
      if (A.v[e] != 0 && cand[j]) {
        best = j;  // columns ascend: the first hit is the minimum
        break;
      }
    }
    if (best == i) {
      elim[i] = 1;
      count++;
    }
  }
  i64 num_no_elim = n - count;  // :213
  if ((double)num_no_elim > (double)n * o.elim_factor) return false;  // :226
  // renumber kept vertices in index order (:236-261)
  L.new_id.assign(n, -1);
  i64 c = 0;
  for (i64 i = 0; i < n; i++)
    if (!elim[i]) L.new_id[i] = (i32)c++;
  i64 nc = c;
  // P, Q (:288-331)
  L.P.n = n;
  L.P.m = nc;
  L.P.rp.assign(n + 1, 0);
  L.Q.assign(n, 0.0);
  for (i64 j = 0; j < n; j++) {
    i64 dp = diag_pos(A, j);
    if (!elim[j]) {
      if (dp >= 0) {  // the diagonal entry carries P(j, new_j) = 1
        L.P.ci.push_back(L.new_id[j]);
        L.P.v.push_back(1.0);
      }
    } else {
      double dj = A.v[dp];
      for (i64 e = A.rp[j]; e < A.rp[j + 1]; e++) {
        i32 i = A.ci[e];
        if (i == j) continue;
        // an explicitly stored zero to another eliminated vertex has no
        // coarse id (the reference asserts here, :321); it is skipped
        if (L.new_id[i] < 0) continue;
        L.P.ci.push_back(L.new_id[i]);
        L.P.v.push_back(1 / dj * -A.v[e]);  // :323 (A symmetric: A(i,j) = A(j,i))
      }
      L.Q[j] = 1 / dj;  // :327
    }
    L.P.rp[j + 1] = (i64)L.P.ci.size();
  }
  L.R = transpose(L.P);  // :336-337
  L.type = LT::Elim;
  return true;
}

// rand_vec + orthagonalize (combblas_extra.hpp:186-192, util.hpp:19-24)
void rand_vec_ortho(GlibcRand &rng, std::vector<double> &x) {
  for (auto &y : x) y = double(rng.next()) / 2147483647;  // F(rand()) / RAND_MAX
  double s = 0.0;  // v.Reduce(std::plus<double>(), 0): sequential
  for (double y : x) s += y;
  s = s / (double)x.size();
  for (auto &y : x) y = y - s;
}

// jacobi with IgnoreDiagSR (smoothing.hpp:12-32,78-98): only negative
// entries contribute to R x; omega = 2/3.
void jacobi_sweep(const Csr &A, std::vector<double> &x, const std::vector<double> &b,
                  std::vector<double> &Rx) {
  const double weight = 2.0 / 3.0;
  Rx.resize(A.n);
#pragma omp parallel for schedule(dynamic, 1024)
  for (i64 i = 0; i < A.n; i++) {
    double y = 0;
    for (i64 e = A.rp[i]; e < A.rp[i + 1]; e++)
      if (A.v[e] < 0) y += A.v[e] * x[A.ci[e]];
    Rx[i] = y;
  }
#pragma omp parallel for schedule(static)
  for (i64 i = 0; i < A.n; i++) {
    i64 dp = diag_pos(A, i);
    if (dp < 0) continue;
    double k = A.v[dp];
    x[i] = weight * (b[i] - Rx[i]) / k + (1 - weight) * x[i];
  }
}

struct VoteAgg {
  int32_t st;
  i64 ind;
  double w;
};

inline bool gt(int32_t a, int32_t b) {  // aggregation.hpp:411-417
  if (a == VSeed) return true;
  if (b == VSeed) return false;
  if (a == VUndecided) return true;
  if (b == VUndecided) return false;
  return true;
}
inline VoteAgg agg_add(const VoteAgg &a1, const VoteAgg &a2) {  // :453-460
  if (a1.st == a2.st) return (a1.w > a2.w) ? a1 : a2;
  return gt(a1.st, a2.st) ? a1 : a2;
}
inline VoteAgg agg_mul(int32_t state, i64 ind, double w, double thr, bool nn) {  // :462-477
  if (state == Seed || (nn && state == SeedNeighbor)) {
    if (w > thr) return {VSeed, ind, w};
    return {VDecided, ind, w};
  } else if (state == Decided || state == DecidedRoot) {
    return {VDecided, ind, w};
  } else if (state == Undecided) {
    return {VUndecided, ind, w};
  }
  return {VDecided, ind, w};  // unreachable in the reference (:475-476)
}

// affinity_matrix (aggregation.hpp:276-404), pattern of A (symmetric).
Csr affinity_matrix(const Csr &A, const ligmg_options &o, GlibcRand &rng,
                    std::vector<double> &tvs_out) {
  i64 n = A.n;
  int ntv = o.num_tvs;
  Csr Aff = A;
  if (o.strength_metric == LIGMG_STRENGTH_AFFINITY ||
      o.strength_metric == LIGMG_STRENGTH_ALGEBRAIC_DISTANCE) {
    std::vector<std::vector<double>> tvs(ntv, std::vector<double>(n));
    for (int t = 0; t < ntv; t++) rand_vec_ortho(rng, tvs[t]);  // create_tvs :24-36
    std::vector<double> b(n, 0.0), Rx;
    for (int t = 0; t < ntv; t++)
      for (int s = 0; s < o.tvs_smooth; s++) jacobi_sweep(A, tvs[t], b, Rx);  // :299-303
    tvs_out.resize((size_t)ntv * n);
    for (int t = 0; t < ntv; t++)
      std::copy(tvs[t].begin(), tvs[t].end(), tvs_out.begin() + (size_t)t * n);
    std::vector<double> sq(n);
    for (i64 v = 0; v < n; v++) {
      double s = 0;
      for (int t = 0; t < ntv; t++) s += tvs[t][v] * tvs[t][v];
      sq[v] = s;
    }
#pragma omp parallel for schedule(dynamic, 1024)
    for (i64 r = 0; r < n; r++)
      for (i64 e = A.rp[r]; e < A.rp[r + 1]; e++) {
        i64 c = A.ci[e];
        double val;
        if (r != c) {
          if (o.strength_metric == LIGMG_STRENGTH_AFFINITY) {  // :321-331
            double top = 0;
            for (int t = 0; t < ntv; t++) top += tvs[t][c] * tvs[t][r];
            double bot1 = sq[c], bot2 = sq[r];
            val = top * top / (bot1 * bot1 * bot2 * bot2);
          } else {  // algebraic distance :333-338
            double mx = -1.0;
            for (int t = 0; t < ntv; t++) {
              double d = std::fabs(tvs[t][c] - tvs[t][r]);
              if (t == 0 || d > mx) mx = d;
            }
            val = 1 / mx;
          }
        } else {
          val = 0;
        }
        Aff.v[e] = val;
      }
  } else {  // :345
    for (auto &x : Aff.v) x = (x < 0) ? -x : 0;
  }
  // scaling (:348-398)
  std::vector<double> sums(n);
  if (o.aff_scaling == LIGMG_AFF_ROW || o.aff_scaling == LIGMG_AFF_ROWCOLUMN ||
      o.aff_scaling == LIGMG_AFF_SYM) {
    for (i64 r = 0; r < n; r++) {
      double s = 0.0;
      for (i64 e = Aff.rp[r]; e < Aff.rp[r + 1]; e++) s += Aff.v[e];
      sums[r] = s;
    }
    for (i64 r = 0; r < n; r++)
      for (i64 e = Aff.rp[r]; e < Aff.rp[r + 1]; e++) Aff.v[e] = Aff.v[e] / sums[r];
  }
  if (o.aff_scaling == LIGMG_AFF_COLUMN || o.aff_scaling == LIGMG_AFF_ROWCOLUMN) {
    std::fill(sums.begin(), sums.end(), 0.0);
    for (i64 r = 0; r < n; r++)  // ascending rows per column
      for (i64 e = Aff.rp[r]; e < Aff.rp[r + 1]; e++) sums[Aff.ci[e]] += Aff.v[e];
    for (i64 r = 0; r < n; r++)
      for (i64 e = Aff.rp[r]; e < Aff.rp[r + 1]; e++) Aff.v[e] = Aff.v[e] / sums[Aff.ci[e]];
  }
  if (o.aff_scaling == LIGMG_AFF_SYM) {  // Aff = (Aff^T + Aff) / 2 (:361-367)
    std::vector<double> sym(Aff.v.size());
    for (i64 r = 0; r < n; r++)
      for (i64 e = Aff.rp[r]; e < Aff.rp[r + 1]; e++) {
        i64 c = Aff.ci[e];
        auto b = Aff.ci.begin() + Aff.rp[c], en = Aff.ci.begin() + Aff.rp[c + 1];
        i64 t = std::lower_bound(b, en, (i32)r) - Aff.ci.begin();  // symmetric pattern
        sym[e] = (Aff.v[t] + Aff.v[e]) / 2;
      }
    Aff.v = sym;
  }
  if (o.aff_scaling == LIGMG_AFF_MAX) {
    std::vector<double> row_max(n, 0.0), col_max(n, 0.0);
    for (i64 r = 0; r < n; r++)
      for (i64 e = Aff.rp[r]; e < Aff.rp[r + 1]; e++) {
        double v = Aff.v[e];
        row_max[r] = std::max(row_max[r], v);
        col_max[Aff.ci[e]] = std::max(col_max[Aff.ci[e]], v);
      }
    for (i64 r = 0; r < n; r++)
      for (i64 e = Aff.rp[r]; e < Aff.rp[r + 1]; e++)
        Aff.v[e] = Aff.v[e] / std::max(row_max[r], col_max[Aff.ci[e]]);  // :395-397
  }
  // Prune v < thresh (:401); NaN survives like in the reference
  Csr P;
  P.n = P.m = n;
  P.rp.assign(n + 1, 0);
  for (i64 r = 0; r < n; r++) {
    for (i64 e = Aff.rp[r]; e < Aff.rp[r + 1]; e++)
      if (!(Aff.v[e] < o.thresh)) {
        P.ci.push_back(Aff.ci[e]);
        P.v.push_back(Aff.v[e]);
      }
    P.rp[r + 1] = (i64)P.ci.size();
  }
  return P;
}

// aggregation (aggregation.hpp:838-964) at single-rank semantics.
void aggregation(const Csr &A, const ligmg_options &o, GlibcRand &rng, Level &L) {
  i64 n = A.n;
  bool nn = o.neighbor_of_neighbor != 0;
  std::vector<i64> ind(n);
  std::vector<int32_t> st(n, Undecided);
  for (i64 i = 0; i < n; i++) ind[i] = i;  // :850-854
  L.aff = affinity_matrix(A, o, rng, L.dbg_tvs);
  const Csr &Aff = L.aff;
  // col_sum (:863-864): column sums, ascending row order
  std::vector<double> col_sum(n, 0.0);
  for (i64 r = 0; r < n; r++)
    for (i64 e = Aff.rp[r]; e < Aff.rp[r + 1]; e++) col_sum[Aff.ci[e]] += Aff.v[e];
  std::vector<double> votes(n, 0.0);
  std::vector<VoteAgg> va(n);
  std::vector<i64> voting_for(n);
  std::vector<double> new_votes(n);
  for (int iter = 0; iter < o.agg_iters; iter++) {
    double iter_thresh = o.agg_init_factor * std::pow(o.agg_iter_factor, iter);  // :886
    // vote: SpMV<AggSR> (:507-518); row entries visited in ascending column
#pragma omp parallel for schedule(dynamic, 1024)
    for (i64 i = 0; i < n; i++) {
      VoteAgg y{VDecided, -1, -1.0};  // AggSR::id()
      for (i64 e = Aff.rp[i]; e < Aff.rp[i + 1]; e++) {
        i64 j = Aff.ci[e];
        y = agg_add(y, agg_mul(st[j], ind[j], Aff.v[e], iter_thresh, nn));
      }
      va[i] = y;
    }
    // tally_votes (:522-561)
    std::fill(new_votes.begin(), new_votes.end(), 0.0);
    std::fill(voting_for.begin(), voting_for.end(), -1);
    for (i64 i = 0; i < n; i++) {
      i64 t = va[i].ind;
      if (st[i] == Undecided && t >= 0 && va[i].w >= iter_thresh && t != i) {
        new_votes[t] += va[i].w;
        voting_for[i] = t;
      }
    }
    for (i64 i = 0; i < n; i++) new_votes[i] += votes[i];
    votes.swap(new_votes);
    // mark_nodes (:702-750): every vertex reads only its own state
    for (i64 i = 0; i < n; i++) {
      int32_t s = st[i];
      if (s == Decided || s == DecidedRoot || s == SeedNeighbor) {
      } else if (s == Seed) {
        if (votes[i] > (double)o.max_agg_size) st[i] = DecidedRoot;
      } else if (voting_for[i] >= 0 && iter == 0 && voting_for[voting_for[i]] == i) {
        if (i < voting_for[i]) {
          st[i] = Seed;
          ind[i] = i;
        } else {
          st[i] = nn ? SeedNeighbor : Decided;
          ind[i] = voting_for[i];
        }
      } else if (va[i].st == VSeed) {
        st[i] = nn ? SeedNeighbor : Decided;
        ind[i] = va[i].ind;
      } else if (votes[i] >= (double)o.votes_to_seed * col_sum[i]) {
        st[i] = Seed;
        ind[i] = i;
      }
    }
    // reject_aggregates (:630-685), off by default (max_agg_size = -1)
    if (o.max_agg_size > 0) {
      std::vector<i64> sizes(n, 0);
      for (i64 i = 0; i < n; i++)
        if (st[i] != Undecided && ind[i] >= 0) sizes[ind[i]]++;
      std::vector<std::vector<i64>> members(n);
      for (i64 i = 0; i < n; i++)
        if ((st[i] == Decided || st[i] == SeedNeighbor) && ind[i] >= 0)
          members[ind[i]].push_back(i);
      for (i64 root = 0; root < n; root++) {
        if (members[root].empty()) continue;
        i64 size = sizes[root];
        if (size > o.max_agg_size) {
          i64 csz = (i64)members[root].size();
          i64 local_count = csz * csz / (size - 1);
          for (i64 k = 0; k < local_count && k < csz; k++) {
            st[members[root][k]] = Undecided;
            ind[members[root][k]] = -1;  // AggState() default
          }
          st[root] = DecidedRoot;
        }
      }
    }
    // conductance_rejection (:752-778) with ext_int_ratio (:563-628), from the
    // second half of the iterations; the ratio reads the states before any
    // vertex is rejected
    if (iter >= o.agg_iters / 2 && o.rejection_ratio >= 0) {
      auto decided = [](int32_t x) {
        return x == Decided || x == DecidedRoot || x == Seed || x == SeedNeighbor;
      };
      std::vector<double> ratio(n);
      for (i64 i = 0; i < n; i++) {
        double ext = 0, inn = 0;
        if (decided(st[i])) {
          for (i64 e = A.rp[i]; e < A.rp[i + 1]; e++) {
            i64 j = A.ci[e];
            if (j == i) continue;
            if (decided(st[j]) && ind[j] == ind[i]) inn -= A.v[e];
            else ext -= A.v[e];
          }
        }
        ratio[i] = ext / inn;
      }
      for (i64 i = 0; i < n; i++)
        if (ratio[i] > o.rejection_ratio && (st[i] == Decided || st[i] == SeedNeighbor)) {
          st[i] = o.rejection_to_seed ? Seed : Undecided;
          ind[i] = i;
        }
    }
  }
  L.dbg_colsum = col_sum;
  L.dbg_votes = votes;
  L.dbg_ind.assign(ind.begin(), ind.end());
  L.dbg_st.assign(st.begin(), st.end());
  // piecewise_constant_restriction + remove_zero_rows (:108-139,950-951;
  // util.hpp:623-632): aggregate id = rank of the root among roots.  A vertex
  // left with ind < 0 by reject_aggregates forms its own aggregate.
  std::vector<char> is_root(n, 0);
  for (i64 i = 0; i < n; i++) {
    if (ind[i] < 0) ind[i] = i;
    is_root[ind[i]] = 1;
  }
  std::vector<i64> rank(n, -1);
  i64 nc = 0;
  for (i64 v = 0; v < n; v++)
    if (is_root[v]) rank[v] = nc++;
  L.agg.resize(n);
  for (i64 i = 0; i < n; i++) L.agg[i] = (i32)rank[ind[i]];
  L.nc = nc;
  L.P.n = n;
  L.P.m = nc;
  L.P.rp.resize(n + 1);
  L.P.ci.resize(n);
  L.P.v.assign(n, 1.0);
  for (i64 i = 0; i <= n; i++) L.P.rp[i] = i;
  for (i64 i = 0; i < n; i++) L.P.ci[i] = L.agg[i];
  L.R = transpose(L.P);
  L.type = LT::Agg;
}

// Largest eigenvalue of a symmetric tridiagonal matrix (bisection on the
// Sturm sequence count).
double tridiag_lmax(const std::vector<double> &d, const std::vector<double> &e) {
  int m = (int)d.size();
  if (m == 0) return 0.0;
  double lo = d[0], hi = d[0];
  for (int i = 0; i < m; i++) {
    double r = 0;
    if (i > 0) r += std::fabs(e[i - 1]);
    if (i + 1 < m) r += std::fabs(e[i]);
    lo = std::min(lo, d[i] - r);
    hi = std::max(hi, d[i] + r);
  }
  for (int it = 0; it < 200; it++) {
    double mid = 0.5 * (lo + hi);
    if (mid <= lo || mid >= hi) break;
    int cnt = 0;  // eigenvalues < mid
    double q = 1.0;
    for (int i = 0; i < m; i++) {
      double off = (i > 0) ? e[i - 1] * e[i - 1] : 0.0;
      q = d[i] - mid - ((i > 0) ? off / q : 0.0);
      if (q == 0.0) q = -1e-300;
      if (q < 0) cnt++;
    }
    if (cnt == m) hi = mid; else lo = mid;
  }
  return hi;
}

// Deterministic right-hand side of the eigenvalue estimate: a 32-bit integer
// hash of the row index mapped to [-0.5, 0.5).
inline double est_rhs(i64 i) {
  uint32_t x = (uint32_t)i * 2654435761u + 0x9E3779B9u;
  x ^= x >> 16;
  x *= 0x85EBCA6Bu;
  x ^= x >> 13;
  x *= 0xC2B2AE35u;
  x ^= x >> 16;
  return (double)x * (1.0 / 4294967296.0) - 0.5;
}

// lambda_max of D^-1 A from 5 Jacobi-PCG steps (chebyshev_create,
// smoothing.hpp:161-165: KSPChebyshevEstEig with a 5-iteration CG).
double estimate_lmax(const Csr &A, const std::vector<double> &invd) {
  i64 n = A.n;
  std::vector<double> r(n), z(n), p(n), q(n);
  for (i64 i = 0; i < n; i++) r[i] = est_rhs(i);
  remove_mean(r);
  for (i64 i = 0; i < n; i++) z[i] = invd[i] * r[i];
  p = z;
  double rz = dot(r, z);
  std::vector<double> alphas, betas;
  for (int k = 0; k < 5; k++) {
    if (!(rz > 0)) break;
    spmv(A, p, q);
    double pq = dot(p, q);
    if (!(pq > 0)) break;
    double alpha = rz / pq;
    for (i64 i = 0; i < n; i++) r[i] -= alpha * q[i];
    for (i64 i = 0; i < n; i++) z[i] = invd[i] * r[i];
    double rz_new = dot(r, z);
    double beta = rz_new / rz;
    rz = rz_new;
    for (i64 i = 0; i < n; i++) p[i] = z[i] + beta * p[i];
    alphas.push_back(alpha);
    betas.push_back(beta);
  }
  int m = (int)alphas.size();
  if (m == 0) return 2.0;  // D^-1 L of a Laplacian is bounded by 2
  std::vector<double> d(m), e(m > 1 ? m - 1 : 0);
  for (int k = 0; k < m; k++) {
    d[k] = 1.0 / alphas[k] + (k > 0 ? betas[k - 1] / alphas[k - 1] : 0.0);
    if (k + 1 < m) e[k] = std::sqrt(betas[k]) / alphas[k];
  }
  return tridiag_lmax(d, e);
}

void setup_smoother(Level &L) {
  L.invd.resize(L.A.n);
  for (i64 i = 0; i < L.A.n; i++) L.invd[i] = 1.0 / L.A.v[diag_pos(L.A, i)];
  L.lmax = estimate_lmax(L.A, L.invd);
}

// Dense pseudo-inverse of a connected Laplacian, (L + 11'/n)^-1 - 11'/n,
// by Gauss-Jordan elimination without pivoting (the shifted matrix is SPD).
// The reference solves its coarse level with PETSc CG + SOR
// (multigrid.hpp:217-258); the dense pseudo-inverse replaces it.
int coarse_pinv(const Csr &A, std::vector<double> &pinv) {
  i64 n = A.n;
  std::vector<double> M((size_t)n * n, 1.0 / (double)n), fac(n);
  pinv.assign((size_t)n * n, 0.0);
  for (i64 i = 0; i < n; i++) {
    pinv[i * n + i] = 1.0;
    for (i64 e = A.rp[i]; e < A.rp[i + 1]; e++) M[i * n + A.ci[e]] += A.v[e];
  }
  for (i64 p = 0; p < n; p++) {
    double piv = M[p * n + p];
    if (!(piv > 0)) return LIGMG_ERR_DISCONNECTED;
    double inv = 1.0 / piv;
    for (i64 k = 0; k < n; k++) {
      pinv[p * n + k] *= inv;
      if (k != p) M[p * n + k] *= inv;
    }
    M[p * n + p] = 1.0;
    for (i64 r = 0; r < n; r++) fac[r] = M[r * n + p];
#pragma omp parallel for schedule(static)
    for (i64 r = 0; r < n; r++) {
      if (r == p) continue;
      double f = fac[r];
      if (f == 0.0) continue;
      for (i64 k = 0; k < n; k++) {
        M[r * n + k] -= f * M[p * n + k];
        pinv[r * n + k] -= f * pinv[p * n + k];
      }
    }
  }
  double c = 1.0 / (double)n;
  for (auto &x : pinv) x -= c;
  return LIGMG_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
struct orc_hier {
  ligmg_options opts;
  std::vector<Level> h;
  double setup_s = 0;
  i64 nnz0 = 0;

  // ---- solve phase -------------------------------------------------------
  void smooth(Level &L, std::vector<double> &x, const std::vector<double> &b, int iters,
              bool x_zero) {
    const ligmg_options &o = opts;
    i64 n = L.A.n;
    if (o.smoother_type == LIGMG_SMOOTHER_JACOBI) {  // smoothing.hpp:206-211: one sweep
      std::vector<double> Rx;
      jacobi_sweep(L.A, x, b, Rx);
      return;
    }
    if (iters <= 0) return;
    // Chebyshev, Saad Alg. 12.1 on D^-1 A, interval [lower, upper] * lmax
    double a = o.cheby_lower * L.lmax, bb = o.cheby_upper * L.lmax;
    double theta = (bb + a) / 2, delta = (bb - a) / 2;
    double sigma = theta / delta, rho = 1 / sigma;
    std::vector<double> r(n), d(n), Ad;
    if (x_zero) r = b; else residual(L.A, x, b, r);
    for (i64 i = 0; i < n; i++) d[i] = L.invd[i] * r[i] / theta;
    for (int k = 0; k < iters; k++) {
      for (i64 i = 0; i < n; i++) x[i] += d[i];
      if (k == iters - 1) break;
      spmv(L.A, d, Ad);
      for (i64 i = 0; i < n; i++) r[i] -= Ad[i];
      double rho_new = 1 / (2 * sigma - rho);
      double c1 = rho_new * rho, c2 = 2 * rho_new / delta;
      for (i64 i = 0; i < n; i++) d[i] = c1 * d[i] + c2 * (L.invd[i] * r[i]);
      rho = rho_new;
    }
  }

  // do_level with x = 0 on entry (all callers pass a zero guess)
  void cycle(size_t l, std::vector<double> &x, const std::vector<double> &b) {
    Level &L = h[l];
    i64 n = L.A.n;
    x.assign(n, 0.0);
    if (L.type == LT::Coarse) {  // multigrid.hpp:49-70 (dense pseudo-inverse)
#pragma omp parallel for schedule(static)
      for (i64 i = 0; i < n; i++) {
        double s = 0;
        for (i64 j = 0; j < n; j++) s += L.pinv[i * n + j] * b[j];
        x[i] = s;
      }
      return;
    }
    if (L.type == LT::Elim) {  // elimination.hpp:33-52
      std::vector<double> bc, xc;
      spmv(L.R, b, bc);
      recurse(l, xc, bc);
      spmv(L.P, xc, x);
      for (i64 i = 0; i < n; i++) x[i] += L.Q[i] * b[i];
      return;
    }
    // AggregationLevel::do_level (aggregation.hpp:209-241)
    smooth(L, x, b, opts.pre_smooth, true);
    std::vector<double> r, bc, xc;
    residual(L.A, x, b, r);
    bc.assign(L.nc, 0.0);
    for (i64 i = 0; i < n; i++) bc[L.agg[i]] += r[i];  // R r, ascending i
    recurse(l, xc, bc);
    for (i64 i = 0; i < n; i++) x[i] += xc[L.agg[i]];  // x += P xc
    smooth(L, x, b, opts.post_smooth, false);
    if (opts.constant_correction)
      for (auto &v : x) v = v * 4.0 / 3.0;
  }

  // the recurse lambda of vcycle / kcycle (multigrid.hpp:87-130)
  void recurse(size_t l, std::vector<double> &xc, const std::vector<double> &bc) {
    if (!opts.kcycle || h[l + 1].is_exact() || h[l + 1].type == LT::Coarse) {
      // V-cycle, or an exact next level.  A coarse next level is applied
      // directly: FCG preconditioned by the exact pseudo-inverse converges
      // in its first iteration (alpha = 1).
      cycle(l + 1, xc, bc);
      return;
    }
    // petsc_fcg with kcycle_iters iterations on h[l+1], x0 = 0 (:115-126)
    if (opts.kcycle_ksp_type == LIGMG_KSP_FGMRES) fgmres_fixed(l + 1, xc, bc, opts.kcycle_iters);
    else krylov_fixed(l + 1, xc, bc, opts.kcycle_iters);
  }

  // fixed-iteration FGMRES (K-cycle inner solve with kcycle_ksp_type fgmres,
  // parse_options.hpp:399-400): exactly m Arnoldi steps from x = 0 (PETSc's
  // restart length, 30, exceeds the K-cycle's iteration count), the outer
  // FGMRES's arithmetic otherwise: b's constant projected out, right
  // preconditioning with kcycle(l) (constant projected out), classical
  // Gram-Schmidt, Givens rotations, back substitution; normalisations multiply
  // by the reciprocal norm.
  void fgmres_fixed(size_t l, std::vector<double> &x, const std::vector<double> &b0, int m) {
    const Csr &A = h[l].A;
    const i64 n = A.n;
    x.assign(n, 0.0);
    std::vector<double> b = b0;
    remove_mean(b);
    const double b2 = dot(b, b);
    auto rsq = [](double v) { return v > 0 ? 1.0 / std::sqrt(v) : 0.0; };
    std::vector<std::vector<double>> V(m + 1, std::vector<double>(n)), Z(m);
    std::vector<double> w, H2((size_t)(m + 1) * m, 0.0);  // dots; (j + 1, j): squared norm
    auto Hij = [&](int i, int j) -> double & { return H2[(size_t)i * m + j]; };
    const double r0 = rsq(b2);
    for (i64 t = 0; t < n; t++) V[0][t] = b[t] * r0;
    for (int j = 0; j < m; j++) {
      cycle(l, Z[j], V[j]);
      remove_mean(Z[j]);
      spmv(A, Z[j], w);
      for (int i = 0; i <= j; i++) Hij(i, j) = dot(V[i], w);
      for (int i = 0; i <= j; i++)
        for (i64 t = 0; t < n; t++) w[t] -= Hij(i, j) * V[i][t];
      Hij(j + 1, j) = dot(w, w);
      if (j + 1 < m) {
        const double rj = rsq(Hij(j + 1, j));
        for (i64 t = 0; t < n; t++) V[j + 1][t] = w[t] * rj;
      }
    }
    // Hessenberg least squares: Givens column by column, then the triangle
    std::vector<double> R((size_t)(m + 1) * m, 0.0), cs(m), sn(m), g(m + 1, 0.0), y(m);
    auto Rij = [&](int i, int j) -> double & { return R[(size_t)i * m + j]; };
    g[0] = std::sqrt(std::max(b2, 0.0));
    for (int j = 0; j < m; j++) {
      for (int i = 0; i <= j; i++) Rij(i, j) = Hij(i, j);
      Rij(j + 1, j) = std::sqrt(std::max(Hij(j + 1, j), 0.0));
      for (int i = 0; i < j; i++) {
        const double a = Rij(i, j), c = Rij(i + 1, j);
        Rij(i, j) = cs[i] * a + sn[i] * c;
        Rij(i + 1, j) = -sn[i] * a + cs[i] * c;
      }
      const double a = Rij(j, j), c = Rij(j + 1, j);
      const double rho = std::sqrt(a * a + c * c);
      cs[j] = rho > 0 ? a / rho : 1.0;
      sn[j] = rho > 0 ? c / rho : 0.0;
      Rij(j, j) = rho;
      Rij(j + 1, j) = 0.0;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
    }
    for (int i = m - 1; i >= 0; i--) {
      double t = g[i];
      for (int q = i + 1; q < m; q++) t -= Rij(i, q) * y[q];
      y[i] = Rij(i, i) != 0 ? t / Rij(i, i) : 0.0;
    }
    for (int i = 0; i < m; i++)
      for (i64 t = 0; t < n; t++) x[t] += y[i] * Z[i][t];
  }

  // fixed-iteration FCG (K-cycle inner solve), preconditioner = kcycle(l)
  void krylov_fixed(size_t l, std::vector<double> &x, const std::vector<double> &b, int iters) {
    const Csr &A = h[l].A;
    i64 n = A.n;
    x.assign(n, 0.0);
    std::vector<double> r = b, z, p(n), q, pprev, qprev;
    double eta_prev = 0;
    for (int it = 0; it < iters; it++) {
      cycle(l, z, r);
      remove_mean(z);
      if (it > 0) {
        double beta = dot(z, qprev) / eta_prev;
        for (i64 i = 0; i < n; i++) p[i] = z[i] - beta * pprev[i];
      } else {
        p = z;
      }
      spmv(A, p, q);
      double eta = dot(p, q);
      if (!(eta > 0)) break;
      double alpha = dot(p, r) / eta;
      for (i64 i = 0; i < n; i++) x[i] += alpha * p[i];
      if (it + 1 < iters)
        for (i64 i = 0; i < n; i++) r[i] -= alpha * q[i];
      pprev = p;
      qprev = q;
      eta_prev = eta;
    }
  }

  double cycle_complexity(int start) {  // multigrid.hpp:372-387
    double s = 0;
    i64 iters = 1;
    for (size_t i = start; i < h.size(); i++) {
      s += (double)(iters * h[i].work(opts));
      if (!h[i].is_exact() && opts.kcycle) iters *= opts.kcycle_iters;
    }
    return s / (double)nnz0;
  }

  // FGMRES(m) (PETSc KSPFGMRES, selectable as the reference's outer KSP type,
  // parse_options.hpp:383-384): right preconditioning with the cycle (its
  // constant projected out), classical Gram-Schmidt, Givens rotations, the
  // Arnoldi residual estimate as convergence test, restart after m steps
  // from the true residual.  x = 0, r = b on entry.
  int fgmres(size_t base, std::vector<double> &x, const std::vector<double> &b,
             std::vector<double> r, double beta, double ttol, std::vector<double> &hist,
             int &iters_out) {
    const Csr &A = h[base].A;
    const i64 n = A.n;
    const int m = std::max(1, opts.gmres_restart);
    std::vector<std::vector<double>> V(m + 1, std::vector<double>(n)), Z(m);
    std::vector<double> w, Hm((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1);
    auto Hij = [&](int i, int j) -> double & { return Hm[(size_t)i * m + j]; };
    int it = 0;
    while (true) {
      for (i64 i = 0; i < n; i++) V[0][i] = r[i] / beta;
      std::fill(g.begin(), g.end(), 0.0);
      g[0] = beta;
      int j = 0;
      bool conv = false;
      while (j < m && it < opts.iters) {
        cycle(base, Z[j], V[j]);
        remove_mean(Z[j]);
        spmv(A, Z[j], w);
        for (int i = 0; i <= j; i++) Hij(i, j) = dot(V[i], w);
        for (int i = 0; i <= j; i++)
          for (i64 t = 0; t < n; t++) w[t] -= Hij(i, j) * V[i][t];
        const double hn = std::sqrt(dot(w, w));
        Hij(j + 1, j) = hn;
        for (i64 t = 0; t < n; t++) V[j + 1][t] = hn > 0 ? w[t] / hn : 0.0;
        for (int i = 0; i < j; i++) {
          const double a = Hij(i, j), c = Hij(i + 1, j);
          Hij(i, j) = cs[i] * a + sn[i] * c;
          Hij(i + 1, j) = -sn[i] * a + cs[i] * c;
        }
        const double a = Hij(j, j), c = Hij(j + 1, j);
        const double rho = std::sqrt(a * a + c * c);
        cs[j] = rho > 0 ? a / rho : 1.0;
        sn[j] = rho > 0 ? c / rho : 0.0;
        Hij(j, j) = rho;
        Hij(j + 1, j) = 0.0;
        g[j + 1] = -sn[j] * g[j];
        g[j] = cs[j] * g[j];
        const double rn = std::fabs(g[j + 1]);
        hist.push_back(rn);
        it++;
        j++;
        if (!std::isfinite(rn)) return LIGMG_ERR_BREAKDOWN;
        if (rn <= ttol) {
          conv = true;
          break;
        }
      }
      std::vector<double> y(j);
      for (int i = j - 1; i >= 0; i--) {
        double s = g[i];
        for (int l = i + 1; l < j; l++) s -= Hij(i, l) * y[l];
        y[i] = Hij(i, i) != 0 ? s / Hij(i, i) : 0.0;
      }
      for (int i = 0; i < j; i++)
        for (i64 t = 0; t < n; t++) x[t] += y[i] * Z[i][t];
      spmv(A, x, w);
      for (i64 t = 0; t < n; t++) r[t] = b[t] - w[t];
      beta = std::sqrt(dot(r, r));
      iters_out = it;
      if (conv || beta <= ttol) return LIGMG_OK;
      if (it >= opts.iters) return LIGMG_NOT_CONVERGED;
      if (!std::isfinite(beta) || beta == 0) return LIGMG_ERR_BREAKDOWN;
    }
  }

  // outer Krylov (petsc_fcg, cg.hpp:18-116) on h[base]
  int outer(size_t base, std::vector<double> &x, std::vector<double> b,
            std::vector<double> &hist, int &iters_out) {
    const Csr &A = h[base].A;
    i64 n = A.n;
    remove_mean(b);
    x.assign(n, 0.0);
    std::vector<double> r = b, z, p(n, 0.0), q;
    double rn0 = std::sqrt(dot(r, r));
    hist.assign(1, rn0);
    iters_out = 0;
    if (rn0 == 0) return LIGMG_OK;
    double ttol = std::max(opts.tol * rn0, 1e-60);  // KSPSetTolerances(tol, 1e-60)
    int mmax = std::max(1, opts.fcg_mmax);
    std::vector<std::vector<double>> P_hist, Q_hist;
    std::vector<double> eta_hist;
    if (opts.outer_ksp_type == LIGMG_KSP_FGMRES)
      return fgmres(base, x, b, r, rn0, ttol, hist, iters_out);
    double beta_cg = 0, beta_old = 0;
    bool cg = opts.outer_ksp_type == LIGMG_KSP_CG;
    if (cg) {
      cycle(base, z, r);
      remove_mean(z);
      beta_cg = dot(z, r);
    }
    for (int it = 0; it < opts.iters; it++) {
      if (cg) {  // KSPCG
        if (it == 0) p = z;
        else {
          double bcoef = beta_cg / beta_old;
          for (i64 i = 0; i < n; i++) p[i] = z[i] + bcoef * p[i];
        }
        spmv(A, p, q);
        double dpi = dot(p, q);
        if (!(dpi > 0) || !std::isfinite(dpi)) return LIGMG_ERR_BREAKDOWN;
        double a = beta_cg / dpi;
        for (i64 i = 0; i < n; i++) x[i] += a * p[i];
        for (i64 i = 0; i < n; i++) r[i] -= a * q[i];
      } else {  // FCG (Notay), standard truncation with mmax directions
        cycle(base, z, r);
        remove_mean(z);
        p = z;
        int nd = (int)P_hist.size();
        for (int k = 0; k < nd; k++) {
          double c = dot(z, Q_hist[k]) / eta_hist[k];
          for (i64 i = 0; i < n; i++) p[i] -= c * P_hist[k][i];
        }
        spmv(A, p, q);
        double eta = dot(p, q);
        if (!(eta > 0) || !std::isfinite(eta)) return LIGMG_ERR_BREAKDOWN;
        double alpha = dot(p, r) / eta;
        for (i64 i = 0; i < n; i++) x[i] += alpha * p[i];
        for (i64 i = 0; i < n; i++) r[i] -= alpha * q[i];
        P_hist.push_back(p);
        Q_hist.push_back(q);
        eta_hist.push_back(eta);
        if ((int)P_hist.size() > mmax) {
          P_hist.erase(P_hist.begin());
          Q_hist.erase(Q_hist.begin());
          eta_hist.erase(eta_hist.begin());
        }
      }
      double rn = std::sqrt(dot(r, r));
      hist.push_back(rn);
      iters_out = it + 1;
      if (!std::isfinite(rn)) return LIGMG_ERR_BREAKDOWN;
      if (rn <= ttol) return LIGMG_OK;
      if (cg) {
        cycle(base, z, r);
        remove_mean(z);
        beta_old = beta_cg;
        beta_cg = dot(z, r);
      }
    }
    return LIGMG_NOT_CONVERGED;
  }
};

extern "C" {

int orc_set_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_num_procs();
  omp_set_num_threads(nthreads);
  return nthreads;
#else
  (void)nthreads;
  return 1;
#endif
}

void orc_glibc_rand(uint32_t seed, int64_t skip, int64_t count, int32_t *out) {
  GlibcRand g(seed);
  for (int64_t i = 0; i < skip; i++) g.next();
  for (int64_t i = 0; i < count; i++) out[i] = g.next();
}

void orc_spmv(int64_t n, const int64_t *rowptr, const int32_t *col, const double *val,
              const double *x, double *y) {
  for (int64_t i = 0; i < n; i++) {
    double s = 0.0;
    for (int64_t e = rowptr[i]; e < rowptr[i + 1]; e++) s += val[e] * x[col[e]];
    y[i] = s;
  }
}

int orc_galerkin(int64_t n, const int64_t *rowptr, const int32_t *col, const double *val,
                 int64_t nc, const int64_t *prow, const int32_t *pcol, const double *pval,
                 int64_t *nnz_out, int64_t *crow, int32_t *ccol, double *cval) {
  Csr A, P;
  A.n = A.m = n;
  A.rp.assign(rowptr, rowptr + n + 1);
  A.ci.assign(col, col + rowptr[n]);
  A.v.assign(val, val + rowptr[n]);
  P.n = n;
  P.m = nc;
  P.rp.assign(prow, prow + n + 1);
  P.ci.assign(pcol, pcol + prow[n]);
  P.v.assign(pval, pval + prow[n]);
  Csr C = galerkin(A, P);
  *nnz_out = C.nnz();
  if (crow) std::copy(C.rp.begin(), C.rp.end(), crow);
  if (ccol) std::copy(C.ci.begin(), C.ci.end(), ccol);
  if (cval) std::copy(C.v.begin(), C.v.end(), cval);
  return LIGMG_OK;
}

// make_hierarchy (multigrid.hpp:162-263) at one rank: redistribution never
// triggers (should_redist needs more than one rank, redistribute.hpp:10-16).
int orc_create(int64_t n, const int64_t *rowptr, const int32_t *col, const double *val,
               const ligmg_options *opts, orc_handle *out) {
  if (!rowptr || !col || !val || !opts || !out || n <= 0) return LIGMG_ERR_INVALID_ARGUMENT;
  auto t0 = std::chrono::steady_clock::now();
  auto H = std::make_unique<orc_hier>();
  H->opts = *opts;
  Csr A;
  A.n = A.m = n;
  A.rp.assign(rowptr, rowptr + n + 1);
  i64 nnz = rowptr[n];
  A.ci.assign(col, col + nnz);
  A.v.assign(val, val + nnz);
  int st = validate(A);
  if (st != LIGMG_OK) return st;
  H->nnz0 = nnz;
  const ligmg_options &o = H->opts;
  GlibcRand rng(o.seed);
  for (int64_t i = 0; i < o.rng_skip; i++) rng.next();
  Csr cur = std::move(A);
  auto &h = H->h;
  while ((int)h.size() < o.max_levels &&
         (h.empty() || h.back().A.nnz() > o.min_size)) {  // :191-193
    if (o.always_elim) {  // add_elimination_level :133-149
      Level E;
      E.A = cur;
      if (o.elim_iters >= 1 && single_elimination(cur, o, E)) {
        Csr next = galerkin(cur, E.P);
        h.push_back(std::move(E));
        cur = std::move(next);
      }
    }
    // add_aggregation_level :151-159
    Level G;
    G.A = cur;
    aggregation(cur, o, rng, G);
    setup_smoother(G);
    Csr next = galerkin(cur, G.P);
    h.push_back(std::move(G));
    cur = std::move(next);
  }
  Level C;  // CoarseLevel (:217-258)
  C.type = LT::Coarse;
  C.A = std::move(cur);
  st = coarse_pinv(C.A, C.pinv);
  if (st != LIGMG_OK) return st;
  h.push_back(std::move(C));
  H->setup_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  *out = H.release();
  return LIGMG_OK;
}

void orc_destroy(orc_handle h) { delete h; }
int orc_num_levels(orc_handle h) { return (int)h->h.size(); }
double orc_setup_seconds(orc_handle h) { return h->setup_s; }
double orc_cycle_complexity(orc_handle h, int start) { return h->cycle_complexity(start); }

int orc_level_info(orc_handle h, int level, int32_t *type, int64_t *n, int64_t *nnz,
                   int64_t *nc) {
  if (level < 0 || level >= (int)h->h.size()) return LIGMG_ERR_INVALID_ARGUMENT;
  const Level &L = h->h[level];
  *type = (int32_t)L.type;
  *n = L.A.n;
  *nnz = L.A.nnz();
  *nc = L.type == LT::Elim ? L.P.m : (L.type == LT::Agg ? L.nc : 0);
  return LIGMG_OK;
}

int orc_level_matrix(orc_handle h, int level, int64_t *rowptr, int32_t *col, double *val) {
  if (level < 0 || level >= (int)h->h.size()) return LIGMG_ERR_INVALID_ARGUMENT;
  const Csr &A = h->h[level].A;
  std::copy(A.rp.begin(), A.rp.end(), rowptr);
  std::copy(A.ci.begin(), A.ci.end(), col);
  std::copy(A.v.begin(), A.v.end(), val);
  return LIGMG_OK;
}

int orc_level_ids(orc_handle h, int level, int32_t *ids) {
  if (level < 0 || level >= (int)h->h.size()) return LIGMG_ERR_INVALID_ARGUMENT;
  const Level &L = h->h[level];
  if (L.type == LT::Elim) std::copy(L.new_id.begin(), L.new_id.end(), ids);
  else if (L.type == LT::Agg) std::copy(L.agg.begin(), L.agg.end(), ids);
  else return LIGMG_ERR_INVALID_ARGUMENT;
  return LIGMG_OK;
}

int orc_level_lmax(orc_handle h, int level, double *lmax) {
  if (level < 0 || level >= (int)h->h.size()) return LIGMG_ERR_INVALID_ARGUMENT;
  *lmax = h->h[level].lmax;
  return LIGMG_OK;
}

int orc_level_prolongation(orc_handle h, int level, int64_t *nnz, int64_t *rowptr,
                           int32_t *col, double *val, double *q) {
  if (level < 0 || level >= (int)h->h.size() || h->h[level].type == LT::Coarse) return LIGMG_ERR_INVALID_ARGUMENT;
  const Level &L = h->h[level];
  *nnz = L.P.nnz();
  if (rowptr) std::copy(L.P.rp.begin(), L.P.rp.end(), rowptr);
  if (col) std::copy(L.P.ci.begin(), L.P.ci.end(), col);
  if (val) std::copy(L.P.v.begin(), L.P.v.end(), val);
  if (q) {
    if (L.type == LT::Elim) std::copy(L.Q.begin(), L.Q.end(), q);
    else std::fill(q, q + L.A.n, 0.0);
  }
  return LIGMG_OK;
}

int orc_level_aff_nnz(orc_handle h, int level, int64_t *nnz) {
  if (level < 0 || level >= (int)h->h.size() || h->h[level].type != LT::Agg)
    return LIGMG_ERR_INVALID_ARGUMENT;
  *nnz = h->h[level].aff.nnz();
  return LIGMG_OK;
}

int orc_level_aff(orc_handle h, int level, int64_t *rowptr, int32_t *col, double *val) {
  if (level < 0 || level >= (int)h->h.size() || h->h[level].type != LT::Agg)
    return LIGMG_ERR_INVALID_ARGUMENT;
  const Csr &A = h->h[level].aff;
  std::copy(A.rp.begin(), A.rp.end(), rowptr);
  std::copy(A.ci.begin(), A.ci.end(), col);
  std::copy(A.v.begin(), A.v.end(), val);
  return LIGMG_OK;
}

int orc_level_debug(orc_handle h, int level, int what, double *out) {
  if (level < 0 || level >= (int)h->h.size() || h->h[level].type != LT::Agg)
    return LIGMG_ERR_INVALID_ARGUMENT;
  const Level &L = h->h[level];
  switch (what) {
    case ORC_DBG_TVS: std::copy(L.dbg_tvs.begin(), L.dbg_tvs.end(), out); break;
    case ORC_DBG_COLSUM: std::copy(L.dbg_colsum.begin(), L.dbg_colsum.end(), out); break;
    case ORC_DBG_STATE_IND:
      for (size_t i = 0; i < L.dbg_ind.size(); i++) out[i] = L.dbg_ind[i];
      break;
    case ORC_DBG_STATE_ST:
      for (size_t i = 0; i < L.dbg_st.size(); i++) out[i] = L.dbg_st[i];
      break;
    case ORC_DBG_VOTES: std::copy(L.dbg_votes.begin(), L.dbg_votes.end(), out); break;
    case ORC_DBG_AFF_NNZ: out[0] = (double)L.aff.nnz(); break;
    default: return LIGMG_ERR_INVALID_ARGUMENT;
  }
  return LIGMG_OK;
}

int orc_cycle(orc_handle h, int level, const double *b, double *x) {
  if (level < 0 || level >= (int)h->h.size()) return LIGMG_ERR_INVALID_ARGUMENT;
  i64 n = h->h[level].A.n;
  std::vector<double> bb(b, b + n), xx;
  h->cycle(level, xx, bb);
  std::copy(xx.begin(), xx.end(), x);
  return LIGMG_OK;
}

// solve (multigrid.hpp:316-370)
int orc_solve(orc_handle H, const double *b, double *x, int from, ligmg_info *info) {
  auto &h = H->h;
  if (from < 0 || from >= (int)h.size()) return LIGMG_ERR_INVALID_ARGUMENT;
  auto t0 = std::chrono::steady_clock::now();
  i64 n = h[from].A.n;
  std::vector<double> bv(b, b + n), rhs;
  // the constant is removed from b before anything else: the reference leaves
  // this to its caller (main.cpp:138-139), and R 1 is not constant, so
  // projecting only the reduced right-hand side would change the answer
  remove_mean(bv);
  bool do_once = H->opts.top_elim && h[from].type == LT::Elim;  // :322
  size_t base = from;
  if (do_once) {
    spmv(h[from].R, bv, rhs);
    base = from + 1;
  } else {
    rhs = bv;
  }
  std::vector<double> xs, hist;
  int iters = 0;
  int st = H->outer(base, xs, rhs, hist, iters);
  std::vector<double> sol;
  if (do_once) {  // :349-354
    spmv(h[from].P, xs, sol);
    for (i64 i = 0; i < n; i++) sol[i] += h[from].Q[i] * bv[i];
  } else {
    sol = xs;
  }
  double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  std::copy(sol.begin(), sol.end(), x);
  if (info) {
    std::vector<double> r;
    const std::vector<double> &bp = bv;
    residual(h[from].A, sol, bp, r);
    double bn = std::sqrt(dot(bp, bp));
    info->iters = iters;
    info->converged = st == LIGMG_OK;
    info->rel_residual = hist.back() / hist.front();
    info->true_rel_residual = bn > 0 ? std::sqrt(dot(r, r)) / bn : 0.0;
    info->cycle_complexity = H->cycle_complexity((int)base);
    info->work = iters * (1 + info->cycle_complexity);
    info->solve_seconds = secs;
    info->setup_seconds = H->setup_s;
    info->history_len = 0;
    if (info->residual_history && info->history_capacity > 0) {
      int m = std::min((int)hist.size(), info->history_capacity);
      std::copy(hist.begin(), hist.begin() + m, info->residual_history);
      info->history_len = m;
    }
  }
  return st;
}

// Input preparation (the reference CLI's --cc then --adj, src/main.cpp:70-110).
// largest_cc (include/ligmg/cc.hpp:24-106): label = iota; repeat
// label' = max(label, max over the row's neighbours of label) (the MaxSRing
// SpMV of cc.hpp:40-50) until nothing changes; count vertices per label; the
// first label with the largest count (max_element, cc.hpp:67-68); renumber
// its vertices in ascending order and keep the entries between them
// (cc.hpp:74-100).  adjacency -> Laplacian (main.cpp:81-106): d_i = row sum
// (sequential, ascending columns), L = D - A (EWiseApply union with 0).
// Two-call protocol like ligmg_prepare_graph.
int orc_prepare_graph(int64_t n, const int64_t *rowptr, const int32_t *col, const double *val,
                      int32_t flags, int64_t *n_out, int64_t *nnz_out, int64_t *rowptr_out,
                      int32_t *col_out, double *val_out, int64_t *orig_out) {
  if (n <= 0) return LIGMG_ERR_INVALID_ARGUMENT;
  std::vector<int32_t> keep(n, 1);
  if (flags & LIGMG_PREP_LCC) {
    std::vector<int64_t> cc(n), old;
    for (int64_t i = 0; i < n; i++) cc[i] = i;
    while (true) {
      old = cc;
      bool same = true;
      for (int64_t i = 0; i < n; i++) {
        int64_t m = old[i];
        for (int64_t k = rowptr[i]; k < rowptr[i + 1]; k++) m = std::max(m, old[col[k]]);
        cc[i] = m;
        if (m != old[i]) same = false;
      }
      if (same) break;
    }
    std::vector<uint64_t> counts(n, 0);
    for (int64_t i = 0; i < n; i++) counts[cc[i]]++;
    const int64_t best = std::max_element(counts.begin(), counts.end()) - counts.begin();
    for (int64_t i = 0; i < n; i++) keep[i] = cc[i] == best;
  }
  std::vector<int64_t> nid(n, -1);
  int64_t nk = 0;
  for (int64_t i = 0; i < n; i++)
    if (keep[i]) nid[i] = nk++;
  const bool lap = (flags & LIGMG_PREP_LAPLACIAN) != 0;
  std::vector<int64_t> rp(1, 0);
  std::vector<int32_t> ci;
  std::vector<double> v;
  std::vector<int64_t> orig;
  for (int64_t i = 0; i < n; i++) {
    if (!keep[i]) continue;
    const int64_t r = nid[i];
    orig.push_back(i);
    double d = 0.0;
    if (lap)
      for (int64_t k = rowptr[i]; k < rowptr[i + 1]; k++)
        if (keep[col[k]]) d += val[k];
    bool placed = false;
    for (int64_t k = rowptr[i]; k < rowptr[i + 1]; k++) {
      const int32_t j = col[k];
      if (!keep[j]) continue;
      const int64_t c = nid[j];
      if (lap && !placed && c > r) {
        ci.push_back((int32_t)r);
        v.push_back(d);
        placed = true;
      }
      double x = val[k];
      if (lap) {
        if (c == r) {
          x = d - x;
          placed = true;
        } else {
          x = -x;
        }
      }
      ci.push_back((int32_t)c);
      v.push_back(x);
    }
    if (lap && !placed) {
      ci.push_back((int32_t)r);
      v.push_back(d);
    }
    rp.push_back((int64_t)ci.size());
  }
  *n_out = nk;
  *nnz_out = (int64_t)ci.size();
  if (rowptr_out) {
    std::copy(rp.begin(), rp.end(), rowptr_out);
    std::copy(ci.begin(), ci.end(), col_out);
    std::copy(v.begin(), v.end(), val_out);
  }
  if (orig_out) std::copy(orig.begin(), orig.end(), orig_out);
  return LIGMG_OK;
}

}  // extern "C"
