"""CSV output in the reference's format: print_csv_header / print_csv
(util.hpp:187-205) after print_options_csv_header / operator<<(Options)
(options.hpp:139-167).

One row per solve: the options, then graph, solver, iters, rel_error,
cycle_complexity, wda, setup_time, solve_time, nnz, nodes.  Values are
written the way a C++ ostream writes them with default flags (doubles with six
significant digits as by %g, bools as 0/1, enums by their names).  Options this
build does not model (MPI redistribution, the random permutation, the
compatible-relaxation parameters) are written with the reference's default
values; `nodes` is the number of processes, 1.
"""
import math

from . import _abi

OPTIONS_HEADER = (
    "StrengthMetric,Redistribute,MaxLevels,MinSize,ElimDegree,AlwaysElim,TopElim,"
    "Tolerance,Threshold,AggregationIterations,MaxIterations,RedistributionFactor,"
    "RedistributionBound,PreSmoothing,PostSmoothing,ConstantCorrection,Smoother,NumberTVs,"
    "TVSmoothingIterations,KCycle,KCycleIterations,OuterKSPType,KCycleKSPType,VotesToSeed,"
    "MaxAggSize,AggIterFactor,ChebyLower,ChebyUpper,AffScaling,RandPerm,RejectionRatio,"
    "CRThreshold,CRTVs,CRIters,CRSmoothingIters,CRNorm")
RESULT_HEADER = ("graph,solver,iters,rel_error,cycle_complexity,wda,setup_time,solve_time,"
                 "nnz,nodes")
HEADER = OPTIONS_HEADER + "," + RESULT_HEADER

# enum names as the reference's operator<< prints them (options.hpp:16-77)
_STRENGTH = {0: "affinity", 1: "algebraic-distance", 2: "none"}
_SMOOTHER = {0: "jacobi", 1: "chebyshev"}
_AFF = {0: "None", 1: "combblas::Row", 2: "Column", 3: "RowColumn", 4: "Sym", 5: "Max"}
_KSP = {0: "cg", 1: "fcg", 2: "fgmres"}  # PETSc KSPType strings
# reference defaults of options without a counterpart here (options.hpp:83-129)
_REDIST, _REDIST_FACTOR, _REDIST_BOUND, _RAND_PERM = True, 10.0, 10000.0, True
_CR_THRESHOLD, _CR_TVS, _CR_ITERS, _CR_SMOOTHING, _CR_NORM = 0.1, 4, 2, 4, "inf"


def fmt(v):
    """A value as a default-formatted C++ ostream writes it."""
    if isinstance(v, bool):
        return "1" if v else "0"
    if isinstance(v, int):
        return str(v)
    if isinstance(v, float):
        if math.isnan(v):
            return "nan"
        if math.isinf(v):
            return "inf" if v > 0 else "-inf"
        return f"{v:g}"
    return str(v)


def options_row(o: _abi.Options) -> str:
    vals = [_STRENGTH[o.strength_metric], _REDIST, o.max_levels, o.min_size, o.elim_degree,
            bool(o.always_elim), bool(o.top_elim), float(o.tol), float(o.thresh), o.agg_iters,
            o.iters, _REDIST_FACTOR, _REDIST_BOUND, o.pre_smooth, o.post_smooth,
            bool(o.constant_correction), _SMOOTHER[o.smoother_type], o.num_tvs, o.tvs_smooth,
            bool(o.kcycle), o.kcycle_iters, _KSP[o.outer_ksp_type], _KSP[o.kcycle_ksp_type],
            o.votes_to_seed, o.max_agg_size, float(o.agg_iter_factor), float(o.cheby_lower),
            float(o.cheby_upper), _AFF[o.aff_scaling], _RAND_PERM, float(o.rejection_ratio),
            _CR_THRESHOLD, _CR_TVS, _CR_ITERS, _CR_SMOOTHING, _CR_NORM]
    return ",".join(fmt(v) for v in vals)


def result_row(graph, solver, info, setup_time, nnz, nodes=1) -> str:
    """graph .. nodes of print_csv (util.hpp:197-204) from a ConvergenceInfo."""
    vals = [graph, solver, int(info.iters()), float(info.rel_residual()),
            float(info.cycle_complexity()), float(info.wda()), float(setup_time),
            float(info.time()), int(nnz), int(nodes)]
    return ",".join(fmt(v) for v in vals)


def write(f, options, info, graph="graph", solver="ligmg", setup_time=0.0, nnz=0,
          header=True):
    """print_csv_header (when header) and print_csv to the text stream f."""
    if header:
        f.write(HEADER + "\n")
    f.write(options_row(options) + "," + result_row(graph, solver, info, setup_time, nnz) + "\n")
