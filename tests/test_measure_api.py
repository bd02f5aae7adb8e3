"""CPU checks of the measurement entry points that need no GPU: argument
validation of ligmg_measure_gather_peak (rejected before any CUDA call) and
ligmg_last_error."""
import ctypes as C

import pytest

from ligmg_gb300._lib import lib


@pytest.mark.parametrize("rows,width,count,bps", [(0, 8, 10, 0), (10, 16, 10, 0), (10, 8, 0, 0),
                                                  (10, 8, 10, 9), (1 << 40, 4, 10, 0)])
def test_gather_peak_rejects_bad_arguments(rows, width, count, bps):
    out = C.c_double(-1.0)
    assert lib().ligmg_measure_gather_peak(rows, width, count, bps, C.byref(out)) == 2
    assert out.value == -1.0
    assert lib().ligmg_measure_gather_peak(10, 8, 10, 0, None) == 2


def test_last_error_is_a_string():
    assert isinstance(lib().ligmg_last_error(), bytes)
