"""Solve metrics against the oracle: the cycle complexity of the hierarchy
(multigrid.hpp:372-387 with the per-level work of aggregation.hpp:247-250,
elimination.hpp:58 and the coarse level), the work of a solve
(iters * (1 + cycle complexity), cg.hpp:115), the reference's derived
metrics (cf, ecf, wda; util.hpp:150-167) and the CSV row (util.hpp:187-205)."""
import io
import math

import numpy as np
import pytest

from ligmg_gb300 import Solver
from ligmg_gb300 import graphs as G
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kw", [dict(), dict(kcycle=1, outer_ksp_type="fcg"),
                                dict(kcycle=1, kcycle_iters=3, outer_ksp_type="fcg"),
                                dict(pre_smooth=1, post_smooth=3)])
@pytest.mark.parametrize("name", ["rmat12", "grid48"])
def test_cycle_complexity_and_work_match_oracle(name, kw):
    L = G.rmat(12, seed=1) if name == "rmat12" else G.grid2d(48, weights="lognormal", seed=2)
    S, R = Solver(L, **kw), O.OracleSolver(L, **kw)
    b = G.rhs(L.n, seed=3)
    info = S.solve(b)
    _, ri = R.solve(b)
    # the solve reports the hierarchy's cycle complexity from its base level
    assert info._cc == ri["cycle_complexity"]
    base = 1 if R.level_info(0)["type"] == "elim" else 0
    assert ri["cycle_complexity"] == R.cycle_complexity(base)
    assert info.work() == info.iters() * (1 + info._cc)
    assert math.isclose(info.cycle_complexity(), 1 + info._cc, rel_tol=1e-15)  # work / iters
    rel = info.residuals[-1] / info.residuals[0]
    assert math.isclose(info.cf(), rel ** (1 / info.iters()))
    assert math.isclose(info.ecf(), rel ** (1 / (info.iters() * info.cycle_complexity())))
    assert math.isclose(info.wda(), -1 / math.log10(info.ecf()))


def test_dump_csv_row_of_a_solve():
    L = G.grid2d(32)
    S = Solver(L, kcycle=1, outer_ksp_type="fcg")
    info = S.solve(G.rhs(L.n, seed=1))
    f = io.StringIO()
    S.dump_csv(f, info, graph="grid32", setup_time=0.1)
    head, row = f.getvalue().splitlines()
    cells = dict(zip(head.split(","), row.split(",")))
    assert int(cells["iters"]) == info.iters() and int(cells["nnz"]) == L.nnz
    assert math.isclose(float(cells["cycle_complexity"]), info.cycle_complexity(), rel_tol=1e-5)
    assert cells["KCycle"] == "1" and cells["OuterKSPType"] == "fcg"


def test_pipefcg_is_reported_unsupported():
    from ligmg_gb300._lib import LigmgError
    with pytest.raises(LigmgError) as e:
        Solver(G.grid2d(8), outer_ksp_type="pipefcg")
    assert e.value.status == 11
    with pytest.raises(LigmgError) as e:
        Solver(G.grid2d(8), kcycle=1, kcycle_ksp_type="pipefcg")
    assert e.value.status == 11
