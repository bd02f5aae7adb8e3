/*
 * ligmg_gpu.h — C ABI of the GB300 (sm_103a) LigMG graph-Laplacian multigrid
 * solver.  Everything here is plain C: pointers, sizes and int status codes.
 * No call throws or aborts across this boundary.
 *
 * The ABI replaces these reference interfaces (paths inside the ligmg project):
 *   ligmg_create           <- ligmg::Solver(A) / Solver(A, Options)
 *                             include/ligmg/ligmg.hpp:17-28, which calls
 *                             make_hierarchy (include/ligmg/multigrid.hpp:162-263)
 *   ligmg_solve            <- Solver::solve(b)            ligmg.hpp:31-33
 *   ligmg_solve_from       <- Solver::solve(b, from)      ligmg.hpp:36-38
 *   ligmg_default_options  <- ligmg::default_options()    options.hpp:136
 *   ligmg_options          <- struct ligmg::Options       options.hpp:80-134
 *   ligmg_info             <- ligmg::ConvergenceInfo      util.hpp:143-170
 *   ligmg_destroy          <- ~Solver / PCDestroy_LIGMG   petsc_shim.hpp:31-38
 *   ligmg_hierarchy_*      <- print_hierarchy / dump_hierarchy
 *                             multigrid.hpp:265-292, ligmg.hpp:47-52
 *   ligmg_cycle            <- vcycle / kcycle             multigrid.hpp:87-130
 *   ligmg_spmv             <- SpMV_inplace (MatShell MATOP_MULT)  util.hpp:451-476
 *   ligmg_status_string    <- PETSC_CHECK_ERROR message   util.hpp:653-660
 * The PETSc plugin PCCreate_LIGMG (petsc_shim.hpp:64-74) is a thin client of
 * ligmg_create / ligmg_solve.
 *
 * Rules:
 *   - status 0 (LIGMG_OK) is success; LIGMG_NOT_CONVERGED is a soft status
 *     (the solution is still written); everything else is an error.
 *   - matrices are CSR with int64 row pointers, int32 column indices sorted
 *     ascending inside each row, FP64 values; the graph Laplacian must be
 *     structurally and numerically symmetric, carry every diagonal entry,
 *     have non-positive off-diagonals and be connected.
 *   - functions without a _device suffix take HOST pointers; *_device
 *     variants take device pointers on the handle's device.
 *   - one CUDA stream per handle; a handle is not thread-safe, distinct
 *     handles are.
 */
#ifndef LIGMG_GPU_H
#define LIGMG_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int ligmg_status;

#define LIGMG_OK 0
#define LIGMG_NOT_CONVERGED 1          /* reached the iteration limit; x written */
#define LIGMG_ERR_INVALID_ARGUMENT 2   /* null pointer, bad size, bad option */
#define LIGMG_ERR_NOT_SYMMETRIC 3      /* pattern or values not symmetric */
#define LIGMG_ERR_BAD_DIAGONAL 4       /* missing or non-positive diagonal */
#define LIGMG_ERR_POSITIVE_OFFDIAG 5   /* off-diagonal entry > 0 */
#define LIGMG_ERR_NONFINITE 6          /* NaN or Inf in a matrix or vector */
#define LIGMG_ERR_DISCONNECTED 7       /* coarse operator singular beyond the constant */
#define LIGMG_ERR_CUDA 8               /* a CUDA runtime call failed */
#define LIGMG_ERR_OUT_OF_MEMORY 9      /* device allocation failed */
#define LIGMG_ERR_BREAKDOWN 10         /* Krylov breakdown / NaN residual */
#define LIGMG_ERR_UNSUPPORTED 11       /* option combination not built */
#define LIGMG_ERR_INTERNAL 12          /* a device-side check failed */
#define LIGMG_ERR_NOT_SORTED 13        /* CSR columns not strictly ascending */

/* enum values follow the reference enums (options.hpp:10-62) */
#define LIGMG_SMOOTHER_JACOBI 0
#define LIGMG_SMOOTHER_CHEBYSHEV 1
#define LIGMG_AFF_NONE 0
#define LIGMG_AFF_ROW 1
#define LIGMG_AFF_COLUMN 2
#define LIGMG_AFF_ROWCOLUMN 3
#define LIGMG_AFF_SYM 4
#define LIGMG_AFF_MAX 5
#define LIGMG_STRENGTH_AFFINITY 0
#define LIGMG_STRENGTH_ALGEBRAIC_DISTANCE 1
#define LIGMG_STRENGTH_NONE 2
#define LIGMG_KSP_CG 0
#define LIGMG_KSP_FCG 1
#define LIGMG_KSP_FGMRES 2  /* flexible GMRES(gmres_restart), right preconditioned */
#define LIGMG_KSP_PIPEFCG 3 /* the reference's pipelined FCG (parse_options.hpp:381-382):
                               not built; ligmg_create returns LIGMG_ERR_UNSUPPORTED */
#define LIGMG_PREC_FP64 0   /* hierarchy, smoothers and cycle in FP64 */
#define LIGMG_PREC_FP32 1   /* FP32 hierarchy/cycle inside the FP64 outer Krylov */

#define LIGMG_LEVEL_ELIM 0
#define LIGMG_LEVEL_AGG 1
#define LIGMG_LEVEL_COARSE 2

/* Hot-path fields of ligmg::Options (options.hpp:80-134) plus the GB300
 * additions at the end.  Fill with ligmg_default_options() first. */
typedef struct ligmg_options {
  int32_t max_levels;         /* 50   options.hpp:91 */
  int32_t always_elim;        /* 1    :84 */
  int64_t min_size;           /* 4000 (nnz) :92 */
  int32_t top_elim;           /* 1    :85 */
  int32_t elim_degree;        /* 4    :93 */
  double elim_factor;         /* 0.9  :121 */
  int32_t elim_iters;         /* 1    :123 */
  int32_t iters;              /* 500  :97 */
  double tol;                 /* 1e-8 :94 */
  double thresh;              /* 1e-8 :95 */
  int32_t agg_iters;          /* 10   :96 */
  int32_t num_tvs;            /* 10   :102 */
  double agg_init_factor;     /* 0.5  :115 */
  double agg_iter_factor;     /* 0.5  :114 */
  int64_t votes_to_seed;      /* 1    :112 */
  int64_t max_agg_size;       /* -1   :113 */
  double rejection_ratio;     /* -1   :124 */
  int32_t rejection_to_seed;  /* 0    :131 */
  int32_t neighbor_of_neighbor; /* 0  :130 */
  int32_t tvs_smooth;         /* 4    :103 */
  int32_t strength_metric;    /* AFFINITY :89 */
  int32_t aff_scaling;        /* MAX  :118 */
  int32_t pre_smooth;         /* 2    :100 */
  int32_t post_smooth;        /* 2    :101 */
  int32_t smoother_type;      /* CHEBYSHEV :105 */
  double cheby_lower;         /* 0.3  :116 */
  double cheby_upper;         /* 1.1  :117 */
  int32_t constant_correction;/* 0    :87 */
  int32_t kcycle;             /* 0    :107 */
  int32_t kcycle_iters;       /* 2    :111 */
  int32_t outer_ksp_type;     /* CG   :109 */
  int32_t kcycle_ksp_type;    /* FCG  :110 */
  /* ---- additions (no reference counterpart) ---- */
  int32_t precision;          /* LIGMG_PREC_FP64 */
  uint32_t seed;              /* srand() seed of the glibc rand() stream that
                                 feeds the aggregation test vectors */
  int32_t fcg_mmax;           /* stored directions of truncated FCG (1) */
  int64_t rng_skip;           /* rand() draws consumed before setup (0) */
  int32_t verbose;            /* 0 */
  int32_t device;             /* CUDA device ordinal (0) */
  int32_t use_graphs;         /* 1: replay each preconditioner application
                                 from a captured CUDA graph (default 1) */
  int32_t autotune;           /* 1: on first use of each (level, precision,
                                 k), time the SpMM launch shapes (block size,
                                 hub chunk size, lanes per row) on that
                                 level and keep the fastest; 0: fixed
                                 defaults, identical launch shapes on every
                                 run (default 1) */
  int64_t tail_rows;          /* the coarse end of the hierarchy as one
                                 persistent kernel per visit; with autotune
                                 it is kept only where it times faster than
                                 the launched levels.  0 (default): from the
                                 shallowest level whose program, matrices and
                                 work vectors fit in shared memory, each CTA
                                 alone on a slice of the k columns; > 0: all
                                 CTAs with grid barriers (k in 1, 8, 16, 32),
                                 from the first level below which every level
                                 has at most this many rows; < 0: every level
                                 launches its own kernels */
  int32_t gmres_restart;      /* FGMRES restart length (30, PETSc's default) */
  int32_t spmv_tiles;         /* 1 (default): single right-hand-side products
                                 of matrices averaging at least six entries
                                 per row use the nonzero-balanced tile layout
                                 (a warp per tile of whole rows, a lane per 8
                                 consecutive entries; with autotune, a warp
                                 per tile or a resident grid that fetches a
                                 warp's next tile during this tile's gathers,
                                 whichever is faster); 2: tiles, always the
                                 resident pipelined grid; 0: one group of
                                 lanes per row */
  int64_t wait_spins;         /* polls of an incomplete barrier before a
                                 device-side wait on other CTAs (the grid-mode
                                 tail kernel's barriers) gives up; the kernel
                                 then stops and the call returns
                                 LIGMG_ERR_INTERNAL.  0: the default (2^23) */
  int32_t batch_queue;        /* batch solves (ligmg_batch_solve): 1 (default):
                                 every 16 outer iterations of all graphs run as
                                 one persistent launch over a (graph,
                                 operation, row block) work queue, each graph
                                 advancing on its own and stopping when it
                                 converges; 0: level-by-level kernels over the
                                 union of the graphs replayed from a CUDA
                                 graph */
  int32_t spmm_streams;       /* products with 8 or more right-hand sides:
                                 1 (default): with autotune, the row-stream
                                 kernel (a warp per run of consecutive rows,
                                 the next row's first indices fetched while
                                 this row gathers) is timed against a warp per
                                 row and kept where faster; 0: a warp per row;
                                 2: row streams always (runs of ~2048
                                 entries).  Results are the same bits either
                                 way */
  int32_t tail_cluster;       /* shared-memory coarse tail (tail_rows = 0):
                                 0 (default): one CTA per column slice, from
                                 the first level whose matrices fit in shared
                                 memory; 1: when a shallower level's work
                                 vectors fit although its matrices do not, the
                                 tail starts there instead and runs a column
                                 slice on a cluster of CTAs that divide the
                                 products with matrices left in global memory
                                 (distributed shared memory, hardware cluster
                                 barriers); with autotune the cluster size is
                                 timed and the tail kept only where a whole
                                 preconditioner application is faster (on
                                 R-MAT 20 it is not: a CTA's eight warps walk
                                 their rows' L2 round trips one row after
                                 another) */
  int32_t spmm_tiles;         /* products with 2 or more right-hand sides and
                                 rows of at most 128 bytes (FP32 k <= 32, FP64
                                 k <= 16): 1 (default): with autotune, tiles
                                 of whole rows walked in steps of consecutive
                                 entries across row boundaries (no step half
                                 empty on short rows) are timed against the
                                 other layouts and kept where faster; 0:
                                 never; 2: always.  Sums are taken in a
                                 different fixed order than a warp per row */
  int32_t pdl;                /* 1: the solve's kernels are launched with
                                 programmatic dependent launch: a kernel may
                                 be scheduled while the one before it runs and
                                 waits on the device for its completion
                                 (launch latency overlapped; small grids only
                                 release their successors early); 0
                                 (default): ordinary stream order.  Same
                                 results either way; on R-MAT 20 the solves
                                 took the same time within run-to-run noise */
} ligmg_options;

/* ConvergenceInfo (util.hpp:143-170) of one solve.  For a batched solve the
 * scalar fields describe the worst column and the per-column arrays (when
 * non-null, length k) are filled. */
typedef struct ligmg_info {
  int32_t iters;              /* outer iterations (max over columns) */
  int32_t converged;          /* all columns reached tol */
  double rel_residual;        /* last / first outer residual (worst column) */
  double true_rel_residual;   /* ||b - L x||_2 / ||b||_2 on the input system, FP64 */
  double cycle_complexity;    /* multigrid.hpp:372-387 */
  double work;                /* iters * (1 + cycle_complexity)  cg.hpp:332 */
  double solve_seconds;       /* wall time of the solve */
  double setup_seconds;       /* wall time of ligmg_create */
  double *residual_history;   /* optional caller buffer (column 0) */
  int32_t history_capacity;   /* its capacity */
  int32_t history_len;        /* entries written */
  int32_t *col_iters;         /* optional, length k */
  double *col_true_rel_residual; /* optional, length k */
} ligmg_info;

typedef struct ligmg_handle_s *ligmg_handle;

void ligmg_default_options(ligmg_options *opts);
const char *ligmg_status_string(ligmg_status s);

/* Build the hierarchy on the GPU (setup).  rowptr[n+1], col[nnz], val[nnz]
 * are host arrays; they are copied and may be freed after the call. */
ligmg_status ligmg_create(int64_t n, const int64_t *rowptr, const int32_t *col,
                          const double *val, const ligmg_options *opts,
                          ligmg_handle *out);
ligmg_status ligmg_destroy(ligmg_handle h);

/* Solve L x = b (host arrays of length n). */
ligmg_status ligmg_solve(ligmg_handle h, const double *b, double *x,
                         ligmg_info *info);
/* Solve starting from hierarchy level `from` (ligmg.hpp:36-38). */
ligmg_status ligmg_solve_from(ligmg_handle h, const double *b, double *x,
                              int32_t from, ligmg_info *info);
/* Solve k right-hand sides at once: B and X are n x k row-major host arrays. */
ligmg_status ligmg_solve_batched(ligmg_handle h, const double *B, int32_t k,
                                 double *X, ligmg_info *info);
/* Same with device pointers (n x k row-major, FP64). */
ligmg_status ligmg_solve_batched_device(ligmg_handle h, const double *dB,
                                        int32_t k, double *dX,
                                        ligmg_info *info);

/* Hierarchy inspection (print_hierarchy / dump_hierarchy). */
ligmg_status ligmg_hierarchy_levels(ligmg_handle h, int32_t *num_levels);
/* type: LIGMG_LEVEL_*; n, nnz of the level's input matrix; nc = size of the
 * next level (0 for the coarse level). */
ligmg_status ligmg_level_info(ligmg_handle h, int32_t level, int32_t *type,
                              int64_t *n, int64_t *nnz, int64_t *nc);
/* Copy the level's input matrix to host CSR arrays (rowptr n+1, col/val nnz). */
ligmg_status ligmg_level_matrix(ligmg_handle h, int32_t level, int64_t *rowptr,
                                int32_t *col, double *val);
/* Level ids (length n): aggregate id per vertex for an aggregation level,
 * coarse id (or -1 when eliminated) for an elimination level. */
ligmg_status ligmg_level_ids(ligmg_handle h, int32_t level, int32_t *ids);
/* Prolongation of a level (n x nc CSR; P(i, agg[i]) = 1 for aggregation,
 * elimination.hpp:288-334 for elimination) and, for elimination levels, the
 * Q diagonal (length n; null to skip).  Two-call protocol: call with null
 * arrays to get *nnz.  Used by dump_hierarchy (ligmg.hpp:47-52). */
ligmg_status ligmg_level_prolongation(ligmg_handle h, int32_t level,
                                      int64_t *nnz, int64_t *rowptr,
                                      int32_t *col, double *val, double *q);

/* Build a handle from an existing hierarchy instead of running the setup:
 * the reverse of dump_hierarchy (ligmg.hpp:47-52, multigrid.hpp:295-313).
 * Every level gives its input matrix; aggregation levels give aggregate ids,
 * elimination levels give P (n x nc) and the Q diagonal; the last level is
 * the coarse level.  The handle estimates the Chebyshev bounds and forms the
 * coarse pseudo-inverse itself.  Arrays are host arrays, copied. */
typedef struct ligmg_level_desc {
  int32_t type;            /* LIGMG_LEVEL_* */
  int64_t n, nnz;          /* level matrix (CSR, same rules as ligmg_create) */
  const int64_t *rowptr;
  const int32_t *col;
  const double *val;
  int64_t nc;              /* size of the next level */
  const int32_t *ids;      /* aggregation: aggregate id per vertex */
  int64_t pnnz;            /* elimination: P (n x nc CSR) and Q diagonal */
  const int64_t *prow;
  const int32_t *pcol;
  const double *pval;
  const double *q;
} ligmg_level_desc;
ligmg_status ligmg_import_hierarchy(int32_t num_levels, const ligmg_level_desc *levels,
                                    const ligmg_options *opts, ligmg_handle *out);

/* Wall time of the setup phases (no reference counterpart; the reference
 * times the whole setup with MPI_Wtime, multigrid.hpp:183,260).  Each phase
 * ends with the handle's stream drained; seconds[LIGMG_SETUP_NPHASES]. */
#define LIGMG_SETUP_VALIDATE 0     /* upload and input checks */
#define LIGMG_SETUP_ELIMINATION 1  /* low-degree elimination selection and P/Q/R */
#define LIGMG_SETUP_AGGREGATION 2  /* test vectors, strength, voting, aggregate ids */
#define LIGMG_SETUP_GALERKIN 3     /* coarse matrices (RAP) */
#define LIGMG_SETUP_SOLVE_DATA 4   /* inverse diagonals, row sums, restriction
                                      matrices, single right-hand-side plans */
#define LIGMG_SETUP_SMOOTHER 5     /* Chebyshev eigenvalue estimates */
#define LIGMG_SETUP_COARSE 6       /* dense coarse pseudo-inverse */
#define LIGMG_SETUP_NPHASES 7
ligmg_status ligmg_setup_times(ligmg_handle h, double *seconds);

/* Largest eigenvalue estimate of D^-1 A used by the level's Chebyshev smoother. */
ligmg_status ligmg_level_lmax(ligmg_handle h, int32_t level, double *lmax);

/* One multigrid cycle x = M(b) starting at `level` with x = 0 on entry
 * (vcycle/kcycle per the handle's options), host arrays of the level's size. */
ligmg_status ligmg_cycle(ligmg_handle h, int32_t level, const double *b,
                         double *x);

/* y = A x with the level's matrix (host arrays).  Debug/measurement entry. */
ligmg_status ligmg_spmv(ligmg_handle h, int32_t level, const double *x,
                        double *y);

/* Per-kernel timing (no reference counterpart; the reference only times
 * setup and solve with MPI_Wtime, multigrid.hpp:183,260 and cg.hpp:23,331).
 * When enabled, every sparse kernel launch of a solve is bracketed by CUDA
 * events on the handle's stream and accumulated per (level, kind, k) with
 * its algorithmic (compulsory) byte count. */
#define LIGMG_KERNEL_SPMV 0        /* y = A x (outer Krylov / K-cycle) */
#define LIGMG_KERNEL_RESID 1       /* r = b - A x */
#define LIGMG_KERNEL_CHEB_A 2      /* first Chebyshev step, nonzero guess */
#define LIGMG_KERNEL_CHEB_B 3      /* later Chebyshev steps */
#define LIGMG_KERNEL_ELIM_INTERP 4 /* x = P xc + Q b */
#define LIGMG_KERNEL_ELIM_RESTRICT 5 /* bc = R b */
#define LIGMG_KERNEL_AGG_RESTRICT 6  /* bc = R r, R the 0/1 member matrix */
#define LIGMG_KERNEL_AGG_PROLONG 7   /* x += P xc */
#define LIGMG_KERNEL_COARSE 8        /* x = pinv b (dense coarse level) */
#define LIGMG_KERNEL_KRYLOV 9        /* K-cycle inner FCG reductions and updates */
#define LIGMG_KERNEL_VECTOR 10       /* smoother start, copies, scaling, conversions */
#define LIGMG_KERNEL_OUTER 11        /* outer Krylov reductions, updates, projection */
#define LIGMG_KERNEL_TAIL 12         /* the coarse tail as one persistent kernel */
typedef struct ligmg_kernel_stat {
  int32_t level;
  int32_t kind;      /* LIGMG_KERNEL_* */
  int32_t k;         /* right-hand sides per launch */
  int32_t fp64;      /* 1: FP64 values, 0: FP32 */
  int64_t launches;
  double seconds;    /* summed event time */
  double bytes;      /* summed algorithmic bytes */
} ligmg_kernel_stat;
ligmg_status ligmg_profile_enable(ligmg_handle h, int32_t enable);
/* Stream control (no reference counterpart): the handle's work is issued on
 * its stream (cudaStream_t passed as void*).  Setting a stream makes the
 * caller's events on that stream bracket the handle's kernels. */
ligmg_status ligmg_set_stream(ligmg_handle h, void *stream);
ligmg_status ligmg_get_stream(ligmg_handle h, void **stream);
/* Kernels launched by this library in this process so far (kernels run
 * from the library's CUDA graphs are counted on every replay). */
ligmg_status ligmg_launch_count(int64_t *count);

/* Message of the last call in this thread that returned an error status
 * (the failing CUDA call and its error string, or the check that failed);
 * valid until the next failing call in the thread. */
const char *ligmg_last_error(void);

/* The gather ceiling of the running GPU (no reference counterpart; a
 * measurement entry for roofline reports).  Every entry of a sparse product
 * gathers one row of the right-hand-side block; on the large levels that
 * block lies in L2, so the products are bound by the rate of random row
 * gathers from L2, not by HBM.  Times `count` gathers of `width`-byte rows
 * (4, 8 or 128) at pseudo-random positions (read from an index array in
 * order, as a product reads column indices) of a zeroed table of `rows` rows,
 * blocks_per_sm blocks of 256 threads per SM (1..8; 0: 8, every warp slot)
 * with independent gathers in flight, and returns rows per second.
 * count <= 2^31.  Allocates (rows * width + 4 count bytes) and frees on a
 * private stream. */
ligmg_status ligmg_measure_gather_peak(int64_t rows, int32_t width, int64_t count,
                                       int32_t blocks_per_sm, double *rows_per_s);

/* Input preparation on the GPU (the reference CLI's --cc / --adj steps,
 * src/main.cpp:70-110, with largest_cc of include/ligmg/cc.hpp:24-106).
 * Input: a host CSR with ascending columns and a symmetric pattern.
 * LIGMG_PREP_LCC keeps the largest connected component (a tie goes to the
 * component whose largest vertex index is smallest), vertices renumbered in
 * ascending order, entries between kept vertices kept in order;
 * LIGMG_PREP_LAPLACIAN then treats the matrix as weighted adjacency and
 * returns L = D - A, D the row sums (ascending column order).  Two-call
 * protocol: with rowptr_out/col_out/val_out null only *n_out and *nnz_out
 * are written; orig_out (nullable, n_out entries) receives each kept
 * vertex's input index.  Runs on `device` (its own stream); synchronous. */
#define LIGMG_PREP_LCC 1
#define LIGMG_PREP_LAPLACIAN 2
ligmg_status ligmg_prepare_graph(int64_t n, const int64_t *rowptr, const int32_t *col,
                                 const double *val, int32_t flags, int32_t device,
                                 int64_t *n_out, int64_t *nnz_out, int64_t *rowptr_out,
                                 int32_t *col_out, double *val_out, int64_t *orig_out);

/* Jacobi-preconditioned CG on the input matrix (the reference's own
 * comparison solver, --test-cg: src/main.cpp:168-180 with the InvDiagSR
 * preconditioner z = D^-1 r, smoothing.hpp:56-76), FP64, rtol opts.tol,
 * at most opts.iters iterations, constant projected out of b and of z. */
ligmg_status ligmg_solve_pcg_jacobi(ligmg_handle h, const double *b, double *x,
                                    ligmg_info *info);

/* A batch of independent graph Laplacians solved together (no reference
 * counterpart; the reference solves one graph per Solver).  The graphs are
 * given as one block-diagonal CSR matrix: graph g owns rows and columns
 * [vertex_offsets[g], vertex_offsets[g+1]) and no entry may leave its block.
 * One hierarchy is built for the union (no aggregate or elimination ever
 * crosses graphs); every graph keeps its own Krylov scalars, its own
 * null-space constant and its own convergence test, which runs on the GPU,
 * so ligmg_batch_solve replays the whole solve of all graphs from one
 * captured CUDA graph.  Requires outer_ksp_type = FCG.  b and x are the
 * concatenated right-hand sides and solutions (length vertex_offsets[G]);
 * iters and true_rel_residual (optional, length G) report per graph. */
ligmg_status ligmg_batch_create(int32_t num_graphs, const int64_t *vertex_offsets,
                                const int64_t *rowptr, const int32_t *col,
                                const double *val, const ligmg_options *opts,
                                ligmg_handle *out);
ligmg_status ligmg_batch_solve(ligmg_handle h, const double *b, double *x,
                               int32_t *iters, double *true_rel_residual,
                               ligmg_info *info);

/* Differentiation through the solve (no reference counterpart).
 * ligmg_forward solves L x = b like ligmg_solve and keeps x on the device.
 * ligmg_backward takes g = dloss/dx (host, length n), solves the adjoint
 * system lambda = L^+ g with the same hierarchy (L is symmetric), and writes
 *   dw[e] = -(x_i - x_j)(lambda_i - lambda_j)  for every stored off-diagonal
 *           entry e = (i, j) of the input CSR (the derivative with respect to
 *           the weight of edge {i, j}; both (i, j) and (j, i) carry it),
 *           0 on diagonal entries;                                (length nnz)
 *   db    = lambda with its mean removed                          (length n)
 * from the kept forward solution (no second forward solve).  Either output
 * may be null.  `info` (optional) describes the adjoint solve. */
ligmg_status ligmg_forward(ligmg_handle h, const double *b, double *x,
                           ligmg_info *info);
ligmg_status ligmg_backward(ligmg_handle h, const double *g, double *dw,
                            double *db, ligmg_info *info);

/* y = A x with the level's FP64 matrix, device pointers, allocating nothing.
 * This entry point has no counterpart in the reference.  It exists for
 * callers that cannot allocate device memory at the point of the call, such
 * as applications whose device memory is owned by their own pool allocator
 * or that run inside a region where a cudaMalloc would synchronise the
 * device.  ligmg_spmv allocates temporary buffers on every call; this
 * variant reads dx[n] and writes dy[n] (caller-owned) and keeps the
 * split-row partial sums of power-law hub rows in a fixed static device
 * array: at most 262144 row chunks and 131072 split rows per level (2 MiB +
 * 512 KiB, held by every GPU that loads the library until exit).  A level
 * beyond those limits returns LIGMG_ERR_UNSUPPORTED.  The work is queued on
 * the handle's stream and the call returns without synchronising.  The
 * first call on a device looks up the array's device address; make that
 * first call before any stream capture.  All calls share the one array, so
 * calls that overlap on the GPU (other streams or handles) race; serialise
 * them. */
ligmg_status ligmg_spmv_device_noalloc(ligmg_handle h, int32_t level,
                                       const double *dx, double *dy);
/* Writes up to cap records (sorted by descending time) and the total count;
 * enabling again clears the statistics. */
ligmg_status ligmg_kernel_stats(ligmg_handle h, ligmg_kernel_stat *out,
                                int32_t cap, int32_t *count);

#ifdef __cplusplus
}
#endif
#endif /* LIGMG_GPU_H */
