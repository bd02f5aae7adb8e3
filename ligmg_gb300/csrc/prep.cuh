// prep.cuh — input preparation on the GPU: the largest connected component
// and adjacency -> Laplacian assembly (the reference CLI's input pipeline,
// src/main.cpp:70-110; include/ligmg/cc.hpp:24-106).
#pragma once
#include "common.cuh"

namespace lg {

struct PrepResult {
  i64 n = 0, nnz = 0;
  std::vector<i64> rowptr;
  std::vector<i32> col;
  std::vector<double> val;
  std::vector<i64> orig;  // original index of every kept vertex
};

// Host CSR in (rows with ascending columns, symmetric pattern), host CSR out.
// lcc: keep the largest connected component (ties: the component whose
// largest vertex index is smallest), vertices renumbered in ascending order;
// laplacian: treat the (kept) matrix as weighted adjacency and return D - A
// with D the row sums.  want_arrays = false computes the sizes only.
void prepare_graph(i64 n, const i64 *rowptr, const i32 *col, const double *val, bool lcc,
                   bool laplacian, bool want_arrays, PrepResult &out, cudaStream_t s);

}  // namespace lg
