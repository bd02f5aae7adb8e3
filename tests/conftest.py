import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


def have_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if have_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


def my_matrix():
    """The reference's example Laplacian (examples/my_matrix.mtx), stored as a
    compact edge list fixture by tests/golden/make_golden.py."""
    from ligmg_gb300.graphs import laplacian_from_edges
    z = np.load(os.path.join(GOLDEN, "my_matrix_edges.npz"))
    return laplacian_from_edges(int(z["n"]), z["u"], z["v"], z["w"], "my_matrix")


@pytest.fixture(scope="session")
def built_lib():
    from ligmg_gb300 import build
    return build.build()
