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


@pytest.mark.parametrize("kw", [dict(precision="fp64", kcycle=1), dict(precision="fp32", kcycle=1),
                                dict(precision="fp64", kcycle=0)])
def test_work_queue_matches_union_graph_mode(kw):
    # batch_queue = 1: one persistent launch over (graph, operation, row
    # block) items per 16 outer iterations; 0: level kernels over the union.
    # Same operations, reductions summed in a different fixed order.
    gs = _graphs()
    bs = [G.rhs(g.n, seed=30 + i) for i, g in enumerate(gs)]
    bs[2] = np.zeros(gs[2].n)  # a graph with nothing to solve
    xq, iq = BatchSolver(gs, batch_queue=1, **kw).solve(bs)
    xu, iu = BatchSolver(gs, batch_queue=0, **kw).solve(bs)
    assert iq.converged and iu.converged
    assert iq.col_iters[2] == 0 and not np.any(xq[2])
    assert (np.abs(iq.col_iters.astype(int) - iu.col_iters.astype(int)) <= 1).all(), \
        (iq.col_iters, iu.col_iters)
    for g, (a, b) in enumerate(zip(xq, xu)):
        if g != 2:
            assert _rel(a, b) <= 1e-6, g
            assert iq.col_true_rel_residual[g] <= 2e-8, g


def test_work_queue_relaunches_past_sixteen_iterations():
    # a slow configuration (V-cycle, one Jacobi sweep, tight tolerance) needs
    # more than one 16-iteration launch; iteration counts continue across
    # launches like the union-graph mode's on the same batch hierarchy (a
    # graph's own hierarchy differs: the union's level rules see all graphs),
    # and every graph matches its single-graph solve
    gs = _graphs()[:4]
    kw = dict(kcycle=0, smoother_type="jacobi", tol=1e-10)
    bs = [G.rhs(g.n, seed=40 + i) for i, g in enumerate(gs)]
    xs, info = BatchSolver(gs, batch_queue=1, **kw).solve(bs)
    _, iu = BatchSolver(gs, batch_queue=0, **kw).solve(bs)
    assert info.converged and info.col_iters.max() > 16
    assert (np.abs(info.col_iters.astype(int) - iu.col_iters.astype(int)) <= 1).all(), \
        (info.col_iters, iu.col_iters)
    for g, (L, b, x) in enumerate(zip(gs, bs, xs)):
        single = Solver(L, outer_ksp_type="fcg", **kw).solve(b)
        assert _rel(x, single.solution) <= 1e-6, g


def test_work_queue_wait_limit_reports_internal_error():
    from ligmg_gb300._lib import LigmgError
    gs = _graphs()
    bs = [G.rhs(g.n, seed=50 + i) for i, g in enumerate(gs)]
    B = BatchSolver(gs, batch_queue=1, wait_spins=1, kcycle=1)
    with pytest.raises(LigmgError) as e:  # a CTA gives up on its first poll
        B.solve(bs)
    assert e.value.status == 12
    xs, info = BatchSolver(gs, batch_queue=1, kcycle=1).solve(bs)  # the context is intact
    assert info.converged


@pytest.mark.parametrize("queue", [1, 0])
def test_batch_with_graphs_that_vanish_at_coarse_levels(queue):
    # small graphs last: they shrink to nothing while the union is still
    # coarsened, leaving empty trailing segments on the coarse levels
    gs = [G.rgg(3000, seed=7), G.grid2d(24, weights="lognormal", seed=8), G.grid2d(5, seed=9),
          G.rgg(60, seed=10)]
    B = BatchSolver(gs, precision="fp32", kcycle=1, batch_queue=queue)
    bs = [G.rhs(g.n, seed=60 + i) for i, g in enumerate(gs)]
    xs, info = B.solve(bs)
    assert info.converged
    for g, (L, b, x) in enumerate(zip(gs, bs, xs)):
        assert np.isfinite(x).all(), g
        r = b - L.to_scipy() @ x
        assert np.linalg.norm(r) / np.linalg.norm(b) <= 2e-8, g
        xr, _ = O.OracleSolver(L, kcycle=1, outer_ksp_type="fcg").solve(b)
        assert _rel(x, xr) <= 1e-6, g
