"""Launch modes that must not change results: programmatic dependent launch
(pdl = 1: a kernel may be scheduled while its predecessor runs and waits on
the device for it) against ordinary stream order, whole solves compared bit
for bit with fixed shapes."""
import numpy as np
import pytest

from ligmg_gb300 import Solver
from ligmg_gb300 import graphs as G

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec,k", [("fp64", 1), ("fp32", 1), ("fp32", 32)])
def test_dependent_launch_same_bits(prec, k):
    L = G.rmat(14, seed=8)
    B = G.rhs(L.n, k=k, seed=3).reshape(L.n, k)
    kw = dict(precision=prec, kcycle=1, outer_ksp_type="fcg", autotune=0)
    a = Solver(L, pdl=1, **kw).solve_batched(B)
    c = Solver(L, pdl=0, **kw).solve_batched(B)
    assert a.converged and c.converged and a.iters() == c.iters()
    assert np.array_equal(a.solution, c.solution)
