"""Batch of unevenly sized graphs solved together (ligmg_batch_*): every
graph's solution must match its own single-graph solve, and every graph must
reach the tolerance on its FP64 true residual."""
import numpy as np
import pytest

from conftest import my_matrix
from ligmg_gb300 import BatchSolver, Solver
from ligmg_gb300 import graphs as G
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _graphs():
    return [G.rgg(800, seed=1), G.grid2d(30, weights="lognormal", seed=2), G.rmat(10, seed=3),
            G.rgg(3000, seed=4), my_matrix(), G.grid3d(9, weights="lognormal", seed=5),
            G.rgg(1500, seed=6)]


def _rel(a, b):
    a = a - a.mean()
    b = b - b.mean()
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_batch_matches_single_graph_solves(prec):
    gs = _graphs()
    B = BatchSolver(gs, precision=prec, kcycle=1)
    bs = [G.rhs(g.n, seed=10 + i) for i, g in enumerate(gs)]
    xs, info = B.solve(bs)
    assert info.converged
    assert (info.col_true_rel_residual <= 2e-8).all(), info.col_true_rel_residual
    assert (info.col_iters > 0).all()
    for g, (L, b, x) in enumerate(zip(gs, bs, xs)):
        r = b - L.to_scipy() @ x
        assert np.linalg.norm(r) / np.linalg.norm(b) <= 2e-8, g
        xr, _ = O.OracleSolver(L, kcycle=1, outer_ksp_type="fcg").solve(b)
        assert _rel(x, xr) <= 1e-6, g
    # a second solve replays the captured whole-solve graph
    xs2, info2 = B.solve(bs)
    assert info2.converged
    for a, b2 in zip(xs, xs2):
        assert np.array_equal(a, b2)


def test_batch_rejects_off_block_entries():
    from ligmg_gb300._lib import LigmgError
    gs = [G.grid2d(4), G.grid2d(4)]
    offs, U = G.union(gs)
    bad = offs.copy()
    bad[1] = 10  # blocks no longer match the matrix
    import ctypes as C
    from ligmg_gb300._abi import default_options
    from ligmg_gb300._lib import lib
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    h = C.c_void_p()
    o = default_options(outer_ksp_type="fcg")
    st = lib().ligmg_batch_create(2, p(bad), p(U.rowptr), p(U.col), p(U.val), C.byref(o),
                                  C.byref(h))
    assert st == 2
