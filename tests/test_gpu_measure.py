"""The gather-ceiling measurement (ligmg_measure_gather_peak) on the GPU and
the error message of a failed call (ligmg_last_error)."""
import numpy as np
import pytest

from ligmg_gb300 import Solver
from ligmg_gb300 import graphs as G
from ligmg_gb300._lib import LigmgError

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("width", [4, 8, 128])
def test_gather_peak_is_plausible(width):
    r = Solver.gather_peak(200000, width, 4_000_000)
    # far above a serial rate, below the L1's one line per SM clock
    assert 1e10 < r < 152 * 2.2e9 * 1.2, r
    assert 1e9 < Solver.gather_peak(200000, width, 4_000_000, blocks_per_sm=1) <= 1.5 * r


def test_failed_call_carries_its_message():
    L = G.grid2d(16)
    S = Solver(L)
    b = G.rhs(L.n, seed=1)
    b[3] = np.nan
    with pytest.raises(LigmgError) as e:
        S.solve(b)
    assert e.value.status == 6
    assert "NaN or Inf" in str(e.value)  # the thrown check's own message
