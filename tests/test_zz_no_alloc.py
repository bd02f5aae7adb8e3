"""ligmg_spmv_device_noalloc: the level SpMV for callers that cannot allocate
device memory at the call (applications whose device memory belongs to their
own pool allocator).

It must give the same y = A x as the allocating entry point ligmg_spmv, on
two calls in a row (the second call finds the shared scratch array holding
the first call's state).  The graph has a hub row longer than the split
threshold, so the scratch array is really used.  This file is collected last
on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from ligmg_gb300 import Solver
from ligmg_gb300 import graphs as G
from ligmg_gb300._lib import check, lib

pytestmark = pytest.mark.gpu


def _hub_graph():
    nx = 64
    idx = np.arange(nx * nx).reshape(nx, nx)
    u = np.concatenate([idx[:, :-1].ravel(), idx[:-1, :].ravel()])
    v = np.concatenate([idx[:, 1:].ravel(), idx[1:, :].ravel()])
    hub = nx * nx
    u = np.concatenate([u, np.full(nx * nx, hub)])
    v = np.concatenate([v, np.arange(nx * nx)])
    w = np.random.default_rng(4).uniform(0.5, 2.0, len(u))
    return G.laplacian_from_edges(nx * nx + 1, u, v, w, "grid64+hub")


def test_noalloc_spmv_matches_allocating_entry_point():
    import torch
    from ligmg_gb300 import build
    build.build()
    L = _hub_graph()
    assert np.diff(L.rowptr).max() > 4096  # a split hub row exercises the scratch
    S = Solver(L)
    rng = np.random.default_rng(0)
    dev = torch.device("cuda", 0)
    for call in range(2):
        x = rng.standard_normal(L.n)
        ref = S.spmv(0, x)
        dx = torch.from_numpy(x).to(dev)
        dy = torch.full((L.n,), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        check(lib().ligmg_spmv_device_noalloc(S._h, 0, C.c_void_p(dx.data_ptr()),
                                              C.c_void_p(dy.data_ptr())), "noalloc spmv")
        torch.cuda.synchronize()
        y = dy.cpu().numpy()
        assert np.isfinite(y).all(), call
        assert np.abs(y - ref).max() <= 1e-12 * np.abs(ref).max(), call
        assert np.abs(y - L.to_scipy() @ x).max() <= 1e-12 * np.abs(ref).max(), call


def test_noalloc_spmv_rejects_bad_arguments():
    L = G.grid2d(8)
    S = Solver(L)
    assert lib().ligmg_spmv_device_noalloc(S._h, 99, C.c_void_p(1), C.c_void_p(1)) == 2
    assert lib().ligmg_spmv_device_noalloc(S._h, 0, None, C.c_void_p(1)) == 2
