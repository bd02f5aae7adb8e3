"""Input preparation on the GPU (ligmg_prepare_graph: the reference CLI's --cc
and --adj steps) against the oracle's restatement: integer structure, kept
vertex map and values bit-exact (both sum each row sequentially in column
order)."""
import numpy as np
import pytest
import scipy.sparse as sp

from ligmg_gb300 import graphs as G
from ligmg_gb300 import prepare_graph
from ligmg_gb300._lib import LigmgError
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _adjacency(L):
    A = -L.to_scipy().tocoo()
    m = A.row != A.col
    A = sp.csr_matrix((A.data[m], (A.row[m], A.col[m])), shape=(L.n, L.n))
    A.sort_indices()
    return A.indptr.astype(np.int64), A.indices.astype(np.int32), A.data.astype(np.float64)


def _same(n, rp, ci, cv, lcc, lap):
    got, orig = prepare_graph(n, rp, ci, cv, lcc=lcc, laplacian=lap)
    orp, oci, ocv, oorig = O.prepare_graph(n, rp, ci, cv, lcc=lcc, laplacian=lap)
    assert got.n == len(orp) - 1
    assert np.array_equal(got.rowptr, orp) and np.array_equal(got.col, oci)
    assert np.array_equal(got.val.view(np.int64), ocv.view(np.int64))
    assert np.array_equal(orig, oorig)
    return got


@pytest.mark.parametrize("scale,seed", [(12, 1), (14, 2), (16, 4)])
def test_rmat_components_and_laplacian(scale, seed):
    raw = G.rmat(scale, seed=seed, lcc=False)
    rp, ci, cv = _adjacency(raw)
    lap = _same(raw.n, rp, ci, cv, lcc=True, lap=True)
    ref = G.rmat(scale, seed=seed, lcc=True)  # host pipeline (scipy components)
    assert lap.n == ref.n and np.array_equal(lap.col, ref.col)
    assert np.allclose(lap.val, ref.val, rtol=1e-14, atol=0)
    _same(raw.n, raw.rowptr, raw.col, raw.val, lcc=True, lap=False)  # Laplacian input
    _same(raw.n, rp, ci, cv, lcc=False, lap=True)                    # every component
    _same(raw.n, rp, ci, cv, lcc=False, lap=False)                   # a plain copy


def test_long_path_and_isolated_vertices():
    # a 3000-vertex path (label propagation over a long diameter), isolated
    # vertices around it, and a diagonal entry on one adjacency row
    n = 3100
    u = np.arange(50, 3049)
    A = sp.coo_matrix((np.linspace(0.5, 2.0, len(u)), (u, u + 1)), shape=(n, n))
    A = (A + A.T + sp.coo_matrix(([0.25], ([100], [100])), shape=(n, n))).tocsr()
    A.sort_indices()
    got = _same(n, A.indptr, A.indices, A.data, lcc=True, lap=True)
    assert got.n == 3000


def test_tie_takes_smaller_label():
    u = np.array([0, 2, 1, 3])
    v = np.array([2, 4, 3, 5])
    A = sp.coo_matrix((np.ones(4), (u, v)), shape=(6, 6))
    A = (A + A.T).tocsr()
    A.sort_indices()
    got, orig = prepare_graph(6, A.indptr, A.indices, A.data, lcc=True)
    assert list(orig) == [0, 2, 4] and got.n == 3


def test_prepared_graph_solves():
    # the prepared Laplacian is the solver's input, as in the reference CLI
    from ligmg_gb300 import Solver
    raw = G.rmat(13, seed=6, lcc=False)
    rp, ci, cv = _adjacency(raw)
    L, _ = prepare_graph(raw.n, rp, ci, cv, lcc=True, laplacian=True)
    info = Solver(L, kcycle=1, outer_ksp_type="fcg").solve(G.rhs(L.n, seed=1))
    assert info.converged and info.true_rel_residual <= 1e-8


def test_invalid_inputs():
    rp = np.array([0, 1, 2], np.int64)
    with pytest.raises(LigmgError) as e:
        prepare_graph(2, rp, np.array([1, 5], np.int32), np.ones(2))
    assert e.value.status == 2
    rp = np.array([0, 2, 4], np.int64)
    with pytest.raises(LigmgError) as e:
        prepare_graph(2, rp, np.array([1, 0, 1, 0], np.int32), np.ones(4))
    assert e.value.status == 13
