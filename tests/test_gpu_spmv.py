"""Single right-hand-side products in the tile layout (spmv_tiles = 1: a warp
per tile of whole rows, a lane per 8 consecutive entries, a segmented scan
across lanes) against the row layout (spmv_tiles = 0) and scipy, on every
level of graphs with ragged, hub and short rows.  FP64 bar: 1e-12 relative to
the largest |y|; the solves must converge in the same number of iterations
(within one) with solutions equal to 1e-6."""
import numpy as np
import pytest
import scipy.sparse as sp

from ligmg_gb300 import Solver
from ligmg_gb300 import graphs as G

pytestmark = pytest.mark.gpu

GRAPHS = {
    "rmat14": lambda: G.rmat(14, seed=5),
    "rmat16": lambda: G.rmat(16, seed=2),
    "grid3d_12": lambda: G.grid3d(12, weights="lognormal", seed=1),
    "rgg3000": lambda: G.rgg(3000, seed=3),
}


@pytest.fixture(scope="module", autouse=True)
def _build():
    from ligmg_gb300 import build
    build.build()


def _hub_star(n_leaves=5000, width=40):
    """A path of `width`-vertex random cliques plus one vertex joined to
    n_leaves vertices: rows from 2 entries up to a hub row far longer than a
    tile holds."""
    rng = np.random.default_rng(1)
    u, v = [], []
    for c in range(n_leaves // width):
        base = c * width
        for i in range(width):
            for j in range(i + 1, width):
                if rng.random() < 0.3 or j == i + 1:
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


@pytest.mark.parametrize("name", list(GRAPHS) + ["hub_star"])
def test_tile_spmv_matches_row_layout_every_level(name):
    L = _hub_star() if name == "hub_star" else GRAPHS[name]()
    T, R = Solver(L, spmv_tiles=1), Solver(L, spmv_tiles=0)
    rng = np.random.default_rng(3)
    for lvl in range(T.num_levels):
        n = T.level_info(lvl)["n"]
        x = rng.standard_normal(n)
        yt, yr = T.spmv(lvl, x), R.spmv(lvl, x)
        rp, ci, v = T.level_matrix(lvl)
        ref = sp.csr_matrix((v, ci, rp), shape=(n, n)) @ x
        scale = max(np.abs(ref).max(), 1e-300)
        assert np.abs(yt - ref).max() <= 1e-12 * scale, (lvl, np.abs(yt - ref).max() / scale)
        assert np.abs(yt - yr).max() <= 1e-12 * scale, lvl
        # same handle, same tiles: bit-identical on a second call
        assert np.array_equal(T.spmv(lvl, x), yt)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("name", ["rmat14", "grid3d_12"])
def test_tile_layout_solve_matches_row_layout(name, prec):
    L = GRAPHS[name]()
    kw = dict(precision=prec, kcycle=1, outer_ksp_type="fcg")
    b = G.rhs(L.n, seed=21)
    a = Solver(L, spmv_tiles=1, **kw).solve(b)
    c = Solver(L, spmv_tiles=0, **kw).solve(b)
    assert a.converged and c.converged
    assert abs(a.iters() - c.iters()) <= 1
    assert a.true_rel_residual <= 2e-8
    x, y = a.solution - a.solution.mean(), c.solution - c.solution.mean()
    assert np.linalg.norm(x - y) <= 1e-6 * np.linalg.norm(y)


@pytest.mark.parametrize("name", list(GRAPHS) + ["hub_star"])
def test_pipelined_tiles_bit_equal_every_level(name):
    # spmv_tiles = 2: the resident grid that fetches a warp's next tile during
    # this tile's gathers; the per-tile arithmetic is the warp-per-tile
    # kernel's, so with fixed shapes (autotune = 0) every level's product and
    # a whole solve are the same bits
    L = _hub_star() if name == "hub_star" else GRAPHS[name]()
    P, W = Solver(L, spmv_tiles=2, autotune=0), Solver(L, spmv_tiles=1, autotune=0)
    rng = np.random.default_rng(4)
    for lvl in range(P.num_levels):
        x = rng.standard_normal(P.level_info(lvl)["n"])
        assert np.array_equal(P.spmv(lvl, x), W.spmv(lvl, x)), lvl
    b = G.rhs(L.n, seed=22)
    a, c = P.solve(b), W.solve(b)
    assert a.converged and a.iters() == c.iters()
    assert np.array_equal(a.solution, c.solution)
