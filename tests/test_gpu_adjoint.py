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


def _central_difference(S_of, Lx_of, x, xt, plus, minus, h):
    """Central difference of loss = 0.5 |x - x_t|^2 between two perturbed
    systems, each solved on the GPU to rtol 1e-12.  A perturbed solution is
    written x + d with d solving the perturbed residual equation
    L' d = b' - L' x, so loss(+) - loss(-) = (x - x_t).(d+ - d-) +
    (|d+|^2 - |d-|^2) / 2 carries no cancellation between two losses of size
    ~n (which would bury the O(h) change)."""
    ds = []
    for sys_ in (plus, minus):
        d = S_of(sys_).solve(Lx_of(sys_)).solution
        ds.append(d - d.mean())
    dp, dm = ds
    return (np.dot(x - xt, dp - dm) + 0.5 * (dp @ dp - dm @ dm)) / (2 * h)


@pytest.mark.parametrize("scale,checks", [(12, 16), (15, 32)])
def test_backward_matches_finite_differences_and_oracle(scale, checks):
    from ligmg_gb300.autograd import edge_positions
    rng = np.random.default_rng(1)
    L = G.rmat(scale, seed=7)
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
    assert np.linalg.norm(dw - dwr) <= 1e-9 * np.linalg.norm(dwr)
    assert np.linalg.norm(db - lr) <= 1e-9 * np.linalg.norm(lr)
    A = L.to_scipy()

    def edge_system(wv):
        Lp = G.laplacian_from_edges(n, u, v, wv)
        return Lp, b - Lp.to_scipy() @ x

    for e in rng.choice(len(w), checks, replace=False):
        h = 1e-6 * w[e]
        wp, wm = w.copy(), w.copy()
        wp[e] += h
        wm[e] -= h
        sp_, sm_ = edge_system(wp), edge_system(wm)
        fd = _central_difference(lambda t: Solver(t[0], **KW), lambda t: t[1], x, xt, sp_, sm_, h)
        assert abs(fd - dw[e]) <= 1e-5 * abs(fd), (e, fd, dw[e])
    for i in rng.choice(n, checks, replace=False):
        bp, bm = b.copy(), b.copy()
        bp[i] += 1e-6
        bm[i] -= 1e-6
        fd = _central_difference(lambda t: S, lambda t: t - A @ x, x, xt, bp, bm, 1e-6)
        assert abs(fd - db[i]) <= 1e-5 * abs(fd), (i, fd, db[i])


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
