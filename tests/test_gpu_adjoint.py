"""GPU forward/backward pair (ligmg_forward / ligmg_backward) against central
finite differences of GPU solves and against the gradient built from the
oracle's solves."""
import numpy as np
import pytest

from ligmg_gb300 import Solver
from ligmg_gb300 import graphs as G
from oracle import oracle as O

pytestmark = pytest.mark.gpu
KW = dict(kcycle=1, outer_ksp_type="fcg", tol=1e-12)


def _edges(L):
    A = L.to_scipy().tocoo()
    m = A.row < A.col
    return A.row[m], A.col[m], -A.data[m]


def _xsolve(n, u, v, w, b):
    info = Solver(G.laplacian_from_edges(n, u, v, w), **KW).solve(b)
    assert info.converged
    return info.solution - info.solution.mean()


def test_backward_matches_finite_differences_and_oracle():
    from ligmg_gb300.autograd import edge_positions
    rng = np.random.default_rng(1)
    L = G.rmat(12, seed=7)
    u, v, w = _edges(L)
    n = L.n
    b = G.rhs(n, seed=2)
    xt = rng.standard_normal(n)
    xt -= xt.mean()
    S = Solver(L, **KW)
    x = S.forward(b).solution
    x = x - x.mean()
    g = x - xt
    dw_csr, db = S.backward(g)
    dw = dw_csr[edge_positions(L, u, v)]
    # gradient from the oracle's solves
    R = O.OracleSolver(L, **KW)
    xr, _ = R.solve(b)
    xr -= xr.mean()
    lr, _ = R.solve(xr - xt)
    lr -= lr.mean()
    dwr = -(xr[u] - xr[v]) * (lr[u] - lr[v])
    assert np.abs(dw - dwr).max() <= 1e-6 * np.abs(dwr).max()
    assert np.abs(db - lr).max() <= 1e-6 * np.abs(lr).max()

    def f(wv, bv):
        xx = _xsolve(n, u, v, wv, bv)
        return 0.5 * np.sum((xx - xt) ** 2)

    for e in rng.choice(len(w), 8, replace=False):
        h = 1e-6 * w[e]
        wp, wm = w.copy(), w.copy()
        wp[e] += h
        wm[e] -= h
        fd = (f(wp, b) - f(wm, b)) / (2 * h)
        assert abs(fd - dw[e]) <= 1e-5 * max(abs(fd), 1e-3 * np.abs(dw).max()), (e, fd, dw[e])
    for i in rng.choice(n, 8, replace=False):
        bp, bm = b.copy(), b.copy()
        bp[i] += 1e-6
        bm[i] -= 1e-6
        fd = (f(w, bp) - f(w, bm)) / 2e-6
        assert abs(fd - db[i]) <= 1e-5 * max(abs(fd), 1e-3 * np.abs(db).max()), (i, fd, db[i])


def test_autograd_function():
    import torch
    from ligmg_gb300._abi import default_options
    from ligmg_gb300.autograd import LaplacianSolve
    L = G.grid2d(20, weights="lognormal", seed=3)
    u, v, w = _edges(L)
    w_t = torch.tensor(w, requires_grad=True)
    b_t = torch.tensor(G.rhs(L.n, seed=4), requires_grad=True)
    xt = torch.tensor(G.rhs(L.n, seed=5))
    x = LaplacianSolve.apply(w_t, b_t, (u, v), default_options(**KW))
    loss = 0.5 * ((x - xt) ** 2).sum()
    loss.backward()
    assert w_t.grad is not None and b_t.grad is not None
    # directional derivative check along a random direction
    d = np.random.default_rng(6).standard_normal(len(w)) * w * 1e-6
    lp = 0.5 * np.sum((_xsolve(L.n, u, v, w + d, b_t.detach().numpy()) - xt.numpy()) ** 2)
    lm = 0.5 * np.sum((_xsolve(L.n, u, v, w - d, b_t.detach().numpy()) - xt.numpy()) ** 2)
    fd = (lp - lm) / 2
    an = float(np.dot(w_t.grad.numpy(), d))
    assert abs(fd - an) <= 1e-5 * abs(fd)


def test_backward_requires_forward():
    from ligmg_gb300._lib import LigmgError
    S = Solver(G.grid2d(8))
    with pytest.raises(LigmgError):
        S.backward(np.zeros(64))
