"""ctypes mirrors of the C structs in include/ligmg_gpu.h.

The field order and types must match the header exactly; tests check the
struct sizes against the compiled library.
"""
import ctypes as C

LIGMG_OK = 0
LIGMG_NOT_CONVERGED = 1

STATUS_NAMES = {
    0: "LIGMG_OK",
    1: "LIGMG_NOT_CONVERGED",
    2: "LIGMG_ERR_INVALID_ARGUMENT",
    3: "LIGMG_ERR_NOT_SYMMETRIC",
    4: "LIGMG_ERR_BAD_DIAGONAL",
    5: "LIGMG_ERR_POSITIVE_OFFDIAG",
    6: "LIGMG_ERR_NONFINITE",
    7: "LIGMG_ERR_DISCONNECTED",
    8: "LIGMG_ERR_CUDA",
    9: "LIGMG_ERR_OUT_OF_MEMORY",
    10: "LIGMG_ERR_BREAKDOWN",
    11: "LIGMG_ERR_UNSUPPORTED",
    12: "LIGMG_ERR_INTERNAL",
    13: "LIGMG_ERR_NOT_SORTED",
}

SMOOTHER = {"jacobi": 0, "chebyshev": 1}
AFF_SCALING = {"none": 0, "row": 1, "column": 2, "rowcolumn": 3, "sym": 4, "max": 5}
STRENGTH = {"affinity": 0, "algebraic-distance": 1, "none": 2}
KSP = {"cg": 0, "fcg": 1, "fgmres": 2, "pipefcg": 3}
PRECISION = {"fp64": 0, "fp32": 1}
LEVEL_TYPES = {0: "elim", 1: "agg", 2: "coarse"}


class Options(C.Structure):
    _fields_ = [
        ("max_levels", C.c_int32),
        ("always_elim", C.c_int32),
        ("min_size", C.c_int64),
        ("top_elim", C.c_int32),
        ("elim_degree", C.c_int32),
        ("elim_factor", C.c_double),
        ("elim_iters", C.c_int32),
        ("iters", C.c_int32),
        ("tol", C.c_double),
        ("thresh", C.c_double),
        ("agg_iters", C.c_int32),
        ("num_tvs", C.c_int32),
        ("agg_init_factor", C.c_double),
        ("agg_iter_factor", C.c_double),
        ("votes_to_seed", C.c_int64),
        ("max_agg_size", C.c_int64),
        ("rejection_ratio", C.c_double),
        ("rejection_to_seed", C.c_int32),
        ("neighbor_of_neighbor", C.c_int32),
        ("tvs_smooth", C.c_int32),
        ("strength_metric", C.c_int32),
        ("aff_scaling", C.c_int32),
        ("pre_smooth", C.c_int32),
        ("post_smooth", C.c_int32),
        ("smoother_type", C.c_int32),
        ("cheby_lower", C.c_double),
        ("cheby_upper", C.c_double),
        ("constant_correction", C.c_int32),
        ("kcycle", C.c_int32),
        ("kcycle_iters", C.c_int32),
        ("outer_ksp_type", C.c_int32),
        ("kcycle_ksp_type", C.c_int32),
        ("precision", C.c_int32),
        ("seed", C.c_uint32),
        ("fcg_mmax", C.c_int32),
        ("rng_skip", C.c_int64),
        ("verbose", C.c_int32),
        ("device", C.c_int32),
        ("use_graphs", C.c_int32),
        ("autotune", C.c_int32),
        ("tail_rows", C.c_int64),
        ("gmres_restart", C.c_int32),
        ("spmv_tiles", C.c_int32),
        ("wait_spins", C.c_int64),
        ("batch_queue", C.c_int32),
        ("spmm_streams", C.c_int32),
        ("tail_cluster", C.c_int32),
        ("spmm_tiles", C.c_int32),
        ("pdl", C.c_int32),
    ]


class Info(C.Structure):
    _fields_ = [
        ("iters", C.c_int32),
        ("converged", C.c_int32),
        ("rel_residual", C.c_double),
        ("true_rel_residual", C.c_double),
        ("cycle_complexity", C.c_double),
        ("work", C.c_double),
        ("solve_seconds", C.c_double),
        ("setup_seconds", C.c_double),
        ("residual_history", C.POINTER(C.c_double)),
        ("history_capacity", C.c_int32),
        ("history_len", C.c_int32),
        ("col_iters", C.POINTER(C.c_int32)),
        ("col_true_rel_residual", C.POINTER(C.c_double)),
    ]


def default_options(**overrides) -> Options:
    """ligmg::default_options() (options.hpp:80-136) plus GB300 additions."""
    o = Options()
    o.max_levels = 50
    o.always_elim = 1
    o.min_size = 4000
    o.top_elim = 1
    o.elim_degree = 4
    o.elim_factor = 0.9
    o.elim_iters = 1
    o.iters = 500
    o.tol = 1e-8
    o.thresh = 1e-8
    o.agg_iters = 10
    o.num_tvs = 10
    o.agg_init_factor = 0.5
    o.agg_iter_factor = 0.5
    o.votes_to_seed = 1
    o.max_agg_size = -1
    o.rejection_ratio = -1.0
    o.rejection_to_seed = 0
    o.neighbor_of_neighbor = 0
    o.tvs_smooth = 4
    o.strength_metric = STRENGTH["affinity"]
    o.aff_scaling = AFF_SCALING["max"]
    o.pre_smooth = 2
    o.post_smooth = 2
    o.smoother_type = SMOOTHER["chebyshev"]
    o.cheby_lower = 0.3
    o.cheby_upper = 1.1
    o.constant_correction = 0
    o.kcycle = 0
    o.kcycle_iters = 2
    o.outer_ksp_type = KSP["cg"]
    o.kcycle_ksp_type = KSP["fcg"]
    o.precision = PRECISION["fp64"]
    o.seed = 0
    o.fcg_mmax = 1
    o.rng_skip = 0
    o.verbose = 0
    o.device = 0
    o.use_graphs = 1
    o.autotune = 1
    o.tail_rows = 0
    o.gmres_restart = 30
    o.spmv_tiles = 1
    o.wait_spins = 0
    o.batch_queue = 1
    o.spmm_streams = 1
    o.tail_cluster = 0
    o.spmm_tiles = 1
    o.pdl = 0
    for k, v in overrides.items():
        if k in ("smoother_type",) and isinstance(v, str):
            v = SMOOTHER[v]
        elif k == "aff_scaling" and isinstance(v, str):
            v = AFF_SCALING[v]
        elif k == "strength_metric" and isinstance(v, str):
            v = STRENGTH[v]
        elif k in ("outer_ksp_type", "kcycle_ksp_type") and isinstance(v, str):
            v = KSP[v]
        elif k == "precision" and isinstance(v, str):
            v = PRECISION[v]
        if not hasattr(o, k):
            raise AttributeError(f"unknown option {k}")
        setattr(o, k, v)
    return o


KERNEL_KINDS = {0: "spmv", 1: "resid", 2: "cheb_a", 3: "cheb_b", 4: "elim_interp",
                5: "elim_restrict", 6: "agg_restrict", 7: "agg_prolong", 8: "coarse",
                9: "krylov", 10: "vector", 11: "outer", 12: "tail"}


class KernelStat(C.Structure):
    _fields_ = [
        ("level", C.c_int32),
        ("kind", C.c_int32),
        ("k", C.c_int32),
        ("fp64", C.c_int32),
        ("launches", C.c_int64),
        ("seconds", C.c_double),
        ("bytes", C.c_double),
    ]


class LevelDesc(C.Structure):
    _fields_ = [
        ("type", C.c_int32),
        ("n", C.c_int64),
        ("nnz", C.c_int64),
        ("rowptr", C.c_void_p),
        ("col", C.c_void_p),
        ("val", C.c_void_p),
        ("nc", C.c_int64),
        ("ids", C.c_void_p),
        ("pnnz", C.c_int64),
        ("prow", C.c_void_p),
        ("pcol", C.c_void_p),
        ("pval", C.c_void_p),
        ("q", C.c_void_p),
    ]
