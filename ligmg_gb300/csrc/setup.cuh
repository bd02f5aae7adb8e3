// setup.cuh — GPU setup phase (hierarchy construction), FP64, bit-exact
// against the CPU restatement of the reference's setup.
#pragma once
#include "common.cuh"

namespace lg {

// Elimination level (single_elimination, elimination.hpp:157-345).
struct ElimResult {
  bool accepted = false;
  i64 nc = 0;
  DBuf<i32> new_id;   // n, -1 for eliminated
  DCsr<double> P;     // n x nc
  DCsr<double> R;     // nc x n  (P^T, rows ascending in fine index)
  DBuf<double> Q;     // n, 1/A_jj on eliminated vertices, 0 elsewhere
  DBuf<i32> pos;      // n, exclusive scan of the kept flags (new id of kept rows)
};
void gpu_elimination(const DCsr<double> &A, int elim_degree, double elim_factor,
                     ElimResult &out, cudaStream_t s);

// Aggregation level (aggregation(), aggregation.hpp:838-964).
struct AggResult {
  i64 nc = 0;
  DBuf<i32> agg;        // n aggregate ids
  DCsr<double> aff;     // pruned affinity matrix
  DBuf<i64> mrp;        // nc+1 member row pointers (R as CSR, values 1)
  DBuf<i32> members;    // n fine vertices grouped by aggregate, ascending
  DBuf<double> colsum, votes, tvs;
  DBuf<i32> ind, st;    // final AggState
  DBuf<i32> rank;       // n, number of aggregate roots with a smaller index
};
struct AggParams {
  int num_tvs, tvs_smooth, agg_iters, strength_metric, aff_scaling;
  bool neighbor_of_neighbor;
  double thresh, agg_init_factor, agg_iter_factor, votes_to_seed, max_agg_size;
  double rejection_ratio;
  bool rejection_to_seed;
};
// tvs_host: num_tvs x n test vectors already drawn and mean-projected on the
// host (row t = test vector t).
void gpu_aggregation(const DCsr<double> &A, const AggParams &p, const double *tvs_host,
                     AggResult &out, cudaStream_t s);

// Galerkin product Ac = P^T A P; exactly symmetric (upper triangle summed in
// fine row-major order, mirrored).  P given as CSR (n x nc).
void gpu_galerkin(const DCsr<double> &A, const DCsr<double> &P, DCsr<double> &C,
                  cudaStream_t s);
// Aggregation special case (P(i, agg[i]) = 1).
void gpu_galerkin_agg(const DCsr<double> &A, const i32 *agg, i64 nc, DCsr<double> &C,
                      cudaStream_t s);

// Fused residual restriction of an aggregation level: C = [R | -R A], nc x 2n,
// so that R (b - A x) = C [b; x] is one SpMM (columns < n gather b, columns
// >= n gather x).  Row I: its members (value 1, ascending), then the entries
// of R A (column n + j), each the sum of the members' a_mj in ascending member
// order.
void gpu_restrict_residual_matrix(const DCsr<double> &A, const i32 *agg, const i64 *mrp,
                                  const i32 *members, i64 nc, DCsr<double> &C, cudaStream_t s);

// Member CSR of an aggregation (R): fine vertices grouped by aggregate id,
// ascending inside each aggregate.
void gpu_members(const i32 *agg, i64 n, i64 nc, DBuf<i64> &mrp, DBuf<i32> &members,
                 cudaStream_t s);

// CSR transpose with rows of the result ascending (stable).
void gpu_transpose(const DCsr<double> &A, DCsr<double> &T, cudaStream_t s);

// Input validation on the GPU: returns a ligmg_status.
ligmg_status gpu_validate(const DCsr<double> &A, cudaStream_t s);

// Dense pseudo-inverse of a connected Laplacian (coarse level):
// out = (A + 11'/n)^-1 - 11'/n, row-major n x n.
// With rowseg/segptr (batch of graphs stored block-diagonally) the constant
// of every segment is handled separately.
ligmg_status gpu_coarse_pinv(const DCsr<double> &A, DBuf<double> &out, cudaStream_t s,
                             const i32 *rowseg = nullptr, const i64 *segptr = nullptr);

}  // namespace lg
