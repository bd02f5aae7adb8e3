/*
 * ligmg_oracle.h — C ABI of the CPU oracle (TEST INFRASTRUCTURE ONLY).
 *
 * The oracle is a plain C++ restatement of LigMG's hot path at single-rank
 * semantics.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg load it, and only to check or time against.  The product
 * library (ligmg_gb300/) never links or calls it.
 */
#ifndef LIGMG_ORACLE_H
#define LIGMG_ORACLE_H

#include <stdint.h>
#include "../include/ligmg_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_hier *orc_handle;

/* debug arrays kept per aggregation level (orc_level_debug `what`) */
#define ORC_DBG_TVS 0        /* num_tvs x n smoothed test vectors (row-major by tv) */
#define ORC_DBG_COLSUM 1     /* n column sums of the affinity matrix */
#define ORC_DBG_STATE_IND 2  /* n final AggState.ind */
#define ORC_DBG_STATE_ST 3   /* n final AggState.state */
#define ORC_DBG_VOTES 4      /* n cumulative votes */
#define ORC_DBG_AFF_NNZ 5    /* 1 value: nnz of the pruned affinity matrix */

int orc_create(int64_t n, const int64_t *rowptr, const int32_t *col,
               const double *val, const ligmg_options *opts, orc_handle *out);
void orc_destroy(orc_handle h);
int orc_num_levels(orc_handle h);
int orc_level_info(orc_handle h, int level, int32_t *type, int64_t *n,
                   int64_t *nnz, int64_t *nc);
int orc_level_matrix(orc_handle h, int level, int64_t *rowptr, int32_t *col,
                     double *val);
int orc_level_ids(orc_handle h, int level, int32_t *ids);
int orc_level_lmax(orc_handle h, int level, double *lmax);
/* prolongation (n x nc CSR) and Q diagonal of a non-coarse level; two-call
 * protocol (null arrays: only *nnz) */
int orc_level_prolongation(orc_handle h, int level, int64_t *nnz, int64_t *rowptr,
                           int32_t *col, double *val, double *q);
/* affinity matrix of an aggregation level: rowptr n+1, then col/val */
int orc_level_aff_nnz(orc_handle h, int level, int64_t *nnz);
int orc_level_aff(orc_handle h, int level, int64_t *rowptr, int32_t *col,
                  double *val);
int orc_level_debug(orc_handle h, int level, int what, double *out);
double orc_cycle_complexity(orc_handle h, int start);
double orc_setup_seconds(orc_handle h);

/* one cycle from `level` with zero initial guess */
int orc_cycle(orc_handle h, int level, const double *b, double *x);
/* full solve (Solver::solve(b, from)) */
int orc_solve(orc_handle h, const double *b, double *x, int from,
              ligmg_info *info);

/* y = A x for a host CSR matrix (sequential row sums) */
void orc_spmv(int64_t n, const int64_t *rowptr, const int32_t *col,
              const double *val, const double *x, double *y);
/* glibc TYPE_3 rand() restatement: srand(seed), skip `skip` draws, then
 * write `count` draws */
void orc_glibc_rand(uint32_t seed, int64_t skip, int64_t count, int32_t *out);
/* Galerkin product Ac = P^T A P (symmetric, upper triangle summed in fine
 * row-major order and mirrored).  Two-call protocol: first call with
 * out arrays null returns nnz in *nnz_out. */
int orc_galerkin(int64_t n, const int64_t *rowptr, const int32_t *col,
                 const double *val, int64_t nc, const int64_t *prow,
                 const int32_t *pcol, const double *pval, int64_t *nnz_out,
                 int64_t *crow, int32_t *ccol, double *cval);
/* --cc / --adj input preparation (largest connected component, adjacency ->
 * Laplacian); same arguments and two-call protocol as ligmg_prepare_graph. */
int orc_prepare_graph(int64_t n, const int64_t *rowptr, const int32_t *col, const double *val,
                      int32_t flags, int64_t *n_out, int64_t *nnz_out, int64_t *rowptr_out,
                      int32_t *col_out, double *val_out, int64_t *orig_out);
/* OpenMP threads used by the oracle (<=0: all cores). Returns the count. */
int orc_set_threads(int nthreads);

#ifdef __cplusplus
}
#endif
#endif
