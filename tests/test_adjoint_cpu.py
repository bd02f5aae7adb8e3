"""The adjoint formulas (no reference counterpart), checked on the CPU with
oracle solves: for loss = 0.5 ||x - x_t||^2 with x = L(w)^+ b,
  dloss/dw_ij = -(x_i - x_j)(lam_i - lam_j),  dloss/db = lam (mean-free),
where lam = L^+ (x - x_t).  Central finite differences with step 1e-6
(relative) and FP64 solves to rtol 1e-12 must agree to 1e-5 relative."""
import numpy as np

from ligmg_gb300 import graphs as G
from oracle import oracle as O

KW = dict(kcycle=1, outer_ksp_type="fcg", tol=1e-13)


def solve(n, u, v, w, b):
    L = G.laplacian_from_edges(n, u, v, w)
    x, info = O.OracleSolver(L, **KW).solve(b)
    assert info["status"] == 0
    return x - x.mean()


def loss(n, u, v, w, b, xt):
    x = solve(n, u, v, w, b)
    return 0.5 * np.sum((x - xt) ** 2)


def test_edge_and_rhs_gradients_match_central_differences():
    rng = np.random.default_rng(0)
    L0 = G.rmat(9, seed=3)
    A = L0.to_scipy().tocoo()
    m = A.row < A.col
    u, v, w = A.row[m], A.col[m], -A.data[m]
    n = L0.n
    b = G.rhs(n, seed=1)
    xt = rng.standard_normal(n)
    xt -= xt.mean()
    x = solve(n, u, v, w, b)
    lam = solve(n, u, v, w, x - xt)
    dw = -(x[u] - x[v]) * (lam[u] - lam[v])
    for e in rng.choice(len(w), 12, replace=False):
        h = 1e-6 * w[e]
        wp, wm = w.copy(), w.copy()
        wp[e] += h
        wm[e] -= h
        fd = (loss(n, u, v, wp, b, xt) - loss(n, u, v, wm, b, xt)) / (2 * h)
        assert abs(fd - dw[e]) <= 1e-5 * max(abs(fd), 1e-3 * np.abs(dw).max()), (e, fd, dw[e])
    for i in rng.choice(n, 8, replace=False):
        h = 1e-6
        bp, bm = b.copy(), b.copy()
        bp[i] += h
        bm[i] -= h
        fd = (loss(n, u, v, w, bp, xt) - loss(n, u, v, w, bm, xt)) / (2 * h)
        assert abs(fd - lam[i]) <= 1e-5 * max(abs(fd), 1e-3 * np.abs(lam).max()), (i, fd, lam[i])


def test_require_converged_raises_on_a_non_converged_solve():
    import pytest
    from ligmg_gb300.autograd import NotConvergedError, require_converged
    from ligmg_gb300.solver import ConvergenceInfo
    ok = ConvergenceInfo([1.0, 1e-9], 5, 0.0, 1.0, None, 1e-9, True)
    assert require_converged(ok, "solve") is ok
    bad = ConvergenceInfo([1.0, 0.5], 1, 0.0, 1.0, None, 0.5, False)
    with pytest.raises(NotConvergedError):
        require_converged(bad, "adjoint solve")
