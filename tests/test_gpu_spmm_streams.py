"""Products with k >= 8 right-hand sides in the row-stream layout
(spmm_streams = 2: a warp per run of consecutive rows, the next row's first
column indices fetched during this row's last gather step) against a warp
per row (spmm_streams = 0).  Every slot of a warp adds its entries in entry
order in both kernels, so with fixed launch shapes (autotune = 0) whole k = 32
solves must agree bit for bit, in FP32 and FP64, on graphs with hub rows,
short rows and long rows.  With the autotuner (default) the kernel is a timed
candidate; those solves must match to 1e-6."""
import numpy as np
import pytest

from ligmg_gb300 import Solver
from ligmg_gb300 import graphs as G
from ligmg_gb300._lib import LigmgError

pytestmark = pytest.mark.gpu


def _hub_star(n_leaves=6000, width=30):
    """Random cliques on a path plus one vertex joined to every other vertex:
    rows of 2 to ~30 entries and one row far longer than a chunk."""
    rng = np.random.default_rng(2)
    u, v = [], []
    for c in range(n_leaves // width):
        base = c * width
        for i in range(width):
            for j in range(i + 1, width):
                if rng.random() < 0.25 or j == i + 1:
                    u.append(base + i)
                    v.append(base + j)
        if c:
            u.append(base - 1)
            v.append(base)
    hub = n_leaves
    u += [hub] * n_leaves
    v += list(range(n_leaves))
    w = rng.uniform(0.5, 2.0, len(u))
    return G.laplacian_from_edges(n_leaves + 1, np.array(u), np.array(v), w, "hub_star")


GRAPHS = {
    "rmat14": lambda: G.rmat(14, seed=5),
    "grid3d_12": lambda: G.grid3d(12, weights="lognormal", seed=1),
    "hub_star": _hub_star,
}


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
@pytest.mark.parametrize("name", list(GRAPHS))
def test_row_streams_bit_equal_to_row_kernel(name, prec):
    L = GRAPHS[name]()
    B = G.rhs(L.n, k=32, seed=11)
    kw = dict(precision=prec, kcycle=1, outer_ksp_type="fcg", autotune=0)
    a = Solver(L, spmm_streams=2, **kw).solve_batched(B)
    c = Solver(L, spmm_streams=0, **kw).solve_batched(B)
    assert a.converged and c.converged
    assert a.iters() == c.iters()
    assert np.array_equal(a.solution, c.solution)


@pytest.mark.parametrize("name", ["rmat14", "hub_star"])
def test_autotuned_streams_match(name):
    L = GRAPHS[name]()
    B = G.rhs(L.n, k=32, seed=12)
    kw = dict(precision="fp32", kcycle=1, outer_ksp_type="fcg")
    a = Solver(L, spmm_streams=1, **kw).solve_batched(B)
    c = Solver(L, spmm_streams=0, **kw).solve_batched(B)
    assert a.converged and c.converged
    assert np.abs(a.col_iters.astype(int) - c.col_iters.astype(int)).max() <= 1
    x = a.solution - a.solution.mean(axis=0)
    y = c.solution - c.solution.mean(axis=0)
    assert np.linalg.norm(x - y) <= 1e-6 * np.linalg.norm(y)


def test_invalid_stream_option_rejected():
    with pytest.raises(LigmgError) as e:
        Solver(G.grid2d(8), spmm_streams=3)
    assert e.value.status == 2


@pytest.mark.parametrize("prec,k", [("fp32", 32), ("fp32", 8), ("fp64", 16)])
@pytest.mark.parametrize("name", list(GRAPHS))
def test_k_column_tiles_match_row_kernel(name, prec, k):
    # spmm_tiles = 2: tiles of whole rows walked in steps of consecutive
    # entries across row boundaries (segmented sums across the warp's
    # slots); a different fixed summation order than a warp per row, so the
    # solves agree to rounding: same iterations (within one), solutions to
    # 1e-6 (FP32 hierarchy) or 1e-9 (FP64), both at the tolerance
    L = GRAPHS[name]()
    B = G.rhs(L.n, k=k, seed=13).reshape(L.n, k)
    kw = dict(precision=prec, kcycle=1, outer_ksp_type="fcg", autotune=0)
    a = Solver(L, spmm_tiles=2, **kw).solve_batched(B)
    c = Solver(L, spmm_tiles=0, **kw).solve_batched(B)
    assert a.converged and c.converged
    assert abs(a.iters() - c.iters()) <= 1
    assert a.true_rel_residual <= 2e-8
    x = a.solution - a.solution.mean(axis=0)
    y = c.solution - c.solution.mean(axis=0)
    tol = 1e-6 if prec == "fp32" else 1e-9
    assert np.linalg.norm(x - y) <= tol * np.linalg.norm(y)
    # deterministic: a second solve on the same handle is the same bits
    again = Solver(L, spmm_tiles=2, **kw).solve_batched(B)
    assert np.array_equal(again.solution, a.solution)
