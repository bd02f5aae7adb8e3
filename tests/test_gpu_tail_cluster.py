"""Coarse tail in cluster mode (tail_cluster = 1): the tail starts at the
shallowest level whose work vectors fit in shared memory; the larger levels'
matrices stay in global memory and their products are divided among a
cluster's CTAs (distributed shared memory, cluster barriers).  With fixed
shapes (autotune = 0: clusters of four, the tail always kept) it must start
shallower than the one-CTA-per-slice tail and give the no-tail solve's
answer: same iterations (within one), solutions equal to 1e-6, FP64 true
residual at the tolerance."""
import numpy as np
import pytest

from ligmg_gb300 import Solver
from ligmg_gb300 import graphs as G

pytestmark = pytest.mark.gpu


def _tail_level(S, B):
    S.profile(True)
    S.solve_batched(B)
    st = S.kernel_stats()
    S.profile(False)
    lv = [r["level"] for r in st if r["kind"] == "tail"]
    return min(lv) if lv else None


def _proj(X):
    return X - X.mean(axis=0)


@pytest.mark.parametrize("prec,k", [("fp64", 1), ("fp32", 1), ("fp32", 32)])
def test_cluster_tail_matches_launched_levels(prec, k):
    L = G.rmat(16, seed=3)
    B = G.rhs(L.n, k=k, seed=5).reshape(L.n, k)
    kw = dict(precision=prec, kcycle=1, outer_ksp_type="fcg", autotune=0)
    C = Solver(L, tail_cluster=1, **kw)
    P = Solver(L, tail_cluster=0, **kw)
    N = Solver(L, tail_rows=-1, **kw)
    ic, ip, inn = C.solve_batched(B), P.solve_batched(B), N.solve_batched(B)
    assert ic.converged and ip.converged and inn.converged
    lc, lp = _tail_level(C, B), _tail_level(P, B)
    assert lc is not None and (lp is None or lc < lp), (lc, lp)
    assert abs(ic.iters() - inn.iters()) <= 1
    assert ic.true_rel_residual <= 2e-8
    x, y = _proj(ic.solution), _proj(inn.solution)
    assert np.linalg.norm(x - y) <= 1e-6 * np.linalg.norm(y)
    # a second solve replays the captured application with the cluster tail
    again = C.solve_batched(B)
    assert np.array_equal(again.solution, ic.solution)
