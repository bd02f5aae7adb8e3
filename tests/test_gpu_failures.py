"""Failure detection without a GPU fault (the reference's error path is
PETSC_CHECK_ERROR throwing std::runtime_error, util.hpp:653-660; here every
failure is an int status at the C ABI).

  * a device-side wait that runs out: the grid-mode coarse-tail kernel's
    barrier waits are bounded by options.wait_spins; with a limit of one poll
    a CTA that is not the last to arrive gives up, every CTA leaves the
    kernel, the call reports LIGMG_ERR_INTERNAL and the context stays usable;
  * a NaN or Inf in the right-hand side: LIGMG_ERR_NONFINITE, not a hang or
    garbage;
  * the iteration limit: LIGMG_NOT_CONVERGED (a soft status, x written),
    which the autograd wrapper turns into NotConvergedError.
"""
import ctypes as C

import numpy as np
import pytest

from ligmg_gb300 import Solver
from ligmg_gb300 import graphs as G
from ligmg_gb300._abi import LIGMG_NOT_CONVERGED
from ligmg_gb300._lib import LigmgError, lib

pytestmark = pytest.mark.gpu

INTERNAL, NONFINITE = 12, 6


@pytest.fixture(scope="module", autouse=True)
def _build():
    from ligmg_gb300 import build
    build.build()


def test_grid_barrier_wait_limit_reports_internal_error():
    # a grid graph has no top elimination: every level from 1 down runs as
    # one cooperative launch of all resident CTAs (autotune off keeps it)
    L = G.grid2d(48, weights="lognormal", seed=2)
    kw = dict(kcycle=1, outer_ksp_type="fcg", tail_rows=1 << 20, autotune=0)
    S = Solver(L, wait_spins=1, **kw)
    b = G.rhs(L.n, seed=3)
    for _ in range(2):  # the barrier state is reset: a retry fails the same way
        with pytest.raises(LigmgError) as e:
            S.solve(b)
        assert e.value.status == INTERNAL
    # the context is intact: a handle with the default limit solves
    ok = Solver(L, **kw).solve(b)
    assert ok.converged and ok.true_rel_residual <= 1e-7


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_nan_rhs_returns_nonfinite(prec):
    L = G.rmat(12, seed=1)
    S = Solver(L, precision=prec, kcycle=1, outer_ksp_type="fcg")
    b = G.rhs(L.n, seed=4)
    b[7] = np.nan
    with pytest.raises(LigmgError) as e:
        S.solve(b)
    assert e.value.status == NONFINITE
    B = G.rhs(L.n, k=4, seed=5)
    B[3, 2] = np.inf
    with pytest.raises(LigmgError) as e:
        S.solve_batched(B)
    assert e.value.status == NONFINITE
    good = S.solve(G.rhs(L.n, seed=4))  # the handle still solves
    assert good.converged


def test_iteration_limit_returns_not_converged():
    L = G.rmat(12, seed=1)
    S = Solver(L, iters=1, kcycle=1, outer_ksp_type="fcg")
    b = G.rhs(L.n, seed=6)
    x = np.empty_like(b)
    st = lib().ligmg_solve(S._h, b.ctypes.data_as(C.c_void_p), x.ctypes.data_as(C.c_void_p), None)
    assert st == LIGMG_NOT_CONVERGED
    assert np.isfinite(x).all()  # the iterate is still written
    info = S.solve(b)
    assert not info.converged and info.iters() == 1


def test_autograd_raises_on_iteration_limit():
    torch = pytest.importorskip("torch")
    from ligmg_gb300._abi import default_options
    from ligmg_gb300.autograd import LaplacianSolve, NotConvergedError
    L0 = G.rmat(9, seed=3)
    A = L0.to_scipy().tocoo()
    m = A.row < A.col
    u, v = A.row[m], A.col[m]
    w = torch.tensor(-A.data[m], dtype=torch.float64, requires_grad=True)
    b = torch.tensor(G.rhs(L0.n, seed=1), dtype=torch.float64)
    with pytest.raises(NotConvergedError):
        LaplacianSolve.apply(w, b, (u, v), default_options(iters=1))
    x = LaplacianSolve.apply(w, b, (u, v), default_options())
    (0.5 * (x ** 2).sum()).backward()
    assert torch.isfinite(w.grad).all()
