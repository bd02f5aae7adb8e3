"""CSV output format (print_options_csv_header / print_csv_header /
print_csv, options.hpp:139-167 and util.hpp:187-205) on a synthetic
ConvergenceInfo; no GPU."""
import io
import math

from ligmg_gb300 import csvout
from ligmg_gb300._abi import default_options
from ligmg_gb300.solver import ConvergenceInfo

# the reference's column names, in order
REF_OPTION_COLUMNS = [
    "StrengthMetric", "Redistribute", "MaxLevels", "MinSize", "ElimDegree", "AlwaysElim",
    "TopElim", "Tolerance", "Threshold", "AggregationIterations", "MaxIterations",
    "RedistributionFactor", "RedistributionBound", "PreSmoothing", "PostSmoothing",
    "ConstantCorrection", "Smoother", "NumberTVs", "TVSmoothingIterations", "KCycle",
    "KCycleIterations", "OuterKSPType", "KCycleKSPType", "VotesToSeed", "MaxAggSize",
    "AggIterFactor", "ChebyLower", "ChebyUpper", "AffScaling", "RandPerm", "RejectionRatio",
    "CRThreshold", "CRTVs", "CRIters", "CRSmoothingIters", "CRNorm"]
REF_RESULT_COLUMNS = ["graph", "solver", "iters", "rel_error", "cycle_complexity", "wda",
                      "setup_time", "solve_time", "nnz", "nodes"]


def _info():
    # 5 iterations, residual 1 -> 1e-9, work = iters * (1 + 2.5) (cg.hpp:115)
    return ConvergenceInfo([1.0, 1e-3, 1e-9], 5, 0.25, 5 * 3.5, None, 1e-9, True)


def test_convergence_info_metrics_follow_the_reference_definitions():
    i = _info()  # util.hpp:150-167
    assert i.cycle_complexity() == 3.5                       # work / iters
    assert math.isclose(i.rel_residual(), 1e-9)             # last / first
    assert math.isclose(i.cf(), 1e-9 ** (1 / 5))             # per-cycle reduction
    assert math.isclose(i.ecf(), 1e-9 ** (1 / (5 * 3.5)))    # per unit of work
    assert math.isclose(i.wda(), -1 / math.log10(i.ecf()))   # work per digit


def test_csv_header_and_row():
    f = io.StringIO()
    o = default_options(kcycle=1, outer_ksp_type="fcg")
    csvout.write(f, o, _info(), graph="rmat20", setup_time=0.5, nnz=1234)
    head, row = f.getvalue().splitlines()
    assert head.split(",") == REF_OPTION_COLUMNS + REF_RESULT_COLUMNS
    cells = dict(zip(head.split(","), row.split(",")))
    assert len(row.split(",")) == len(head.split(","))
    assert cells["StrengthMetric"] == "affinity" and cells["Smoother"] == "chebyshev"
    assert cells["Tolerance"] == "1e-08" and cells["MinSize"] == "4000"
    assert cells["KCycle"] == "1" and cells["OuterKSPType"] == "fcg"
    assert cells["KCycleKSPType"] == "fcg" and cells["AffScaling"] == "Max"
    assert cells["ChebyLower"] == "0.3" and cells["MaxAggSize"] == "-1"
    assert cells["graph"] == "rmat20" and cells["solver"] == "ligmg"
    assert cells["iters"] == "5" and cells["rel_error"] == "1e-09"
    assert cells["cycle_complexity"] == "3.5" and cells["nnz"] == "1234"
    assert cells["nodes"] == "1" and cells["setup_time"] == "0.5"
    assert math.isclose(float(cells["wda"]), _info().wda(), rel_tol=1e-5)
