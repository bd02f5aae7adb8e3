"""CPU tests of the oracle (the CPU restatement of the reference's hot path).

The reference ships no tests or golden vectors for this path; the pins here
are: glibc rand() itself (the generator the reference draws its test vectors
from), the reference's example matrix, dense-algebra identities of every
setup product, and the algorithm's own invariants.
"""
import ctypes
import os

import numpy as np
import pytest
import scipy.sparse as sp

from conftest import GOLDEN, my_matrix
from ligmg_gb300 import graphs as G
from oracle import oracle as O


def dense(rp, ci, cv, n, m=None):
    return sp.csr_matrix((cv, ci, rp), shape=(n, m or n)).toarray()


@pytest.mark.parametrize("seed", [0, 1, 7, 42, 123456789, 2**31 + 5, 2**32 - 1])
def test_glibc_rand_matches_libc(seed):
    libc = ctypes.CDLL("libc.so.6")
    libc.srand(ctypes.c_uint(seed))
    ref = np.array([libc.rand() for _ in range(5000)], dtype=np.int64)
    assert (O.glibc_rand(seed, 5000) == ref).all()
    assert (O.glibc_rand(seed, 100, skip=4900) == ref[4900:]).all()


def test_my_matrix_fixture():
    L = my_matrix()
    assert L.n == 986 and L.nnz == 33114
    A = L.to_scipy()
    assert abs(A - A.T).max() == 0
    assert np.abs(np.asarray(A.sum(axis=1))).max() == 0


def test_oracle_golden_summary():
    from tests.golden.make_golden import digest
    z = np.load(os.path.join(GOLDEN, "oracle_my_matrix.npz"))
    S = O.OracleSolver(my_matrix())
    assert S.num_levels == len(z["types"])
    for l in range(S.num_levels):
        inf = S.level_info(l)
        assert inf["type"] == z["types"][l]
        assert (inf["n"], inf["nnz"], inf["nc"]) == (z["n"][l], z["nnz"][l], z["nc"][l])
        rp, ci, cv = S.level_matrix(l)
        ids = S.level_ids(l) if inf["type"] != "coarse" else np.zeros(0, np.int32)
        assert digest(ids) == z["ids_digest"][l]
        assert digest(rp, ci, cv) == z["mat_digest"][l]


def _level_P(S, l):
    inf = S.level_info(l)
    ids = S.level_ids(l)
    n, nc = inf["n"], inf["nc"]
    if inf["type"] == "agg":
        return sp.csr_matrix((np.ones(n), (np.arange(n), ids)), shape=(n, nc))
    return None


@pytest.mark.parametrize("name", ["grid", "my_matrix", "rmat12"])
def test_galerkin_levels_match_dense_products(name):
    L = {"grid": lambda: G.grid2d(24, weights="lognormal"), "my_matrix": my_matrix,
         "rmat12": lambda: G.rmat(12)}[name]()
    S = O.OracleSolver(L)
    for l in range(S.num_levels - 1):
        inf = S.level_info(l)
        A = dense(*S.level_matrix(l), inf["n"])
        Ac = dense(*S.level_matrix(l + 1), S.level_info(l + 1)["n"])
        assert (Ac == Ac.T).all(), "Galerkin product must be exactly symmetric"
        if inf["type"] == "agg":
            P = _level_P(S, l).toarray()
            ref = P.T @ A @ P
        else:  # elimination: Schur complement on the kept vertices
            ids = S.level_ids(l)
            keep, el = ids >= 0, ids < 0
            Akk, Ake, Aee = A[np.ix_(keep, keep)], A[np.ix_(keep, el)], A[np.ix_(el, el)]
            assert np.count_nonzero(Aee - np.diag(np.diag(Aee))) == 0, "eliminated set independent"
            ref = Akk - Ake @ np.diag(1.0 / np.diag(Aee)) @ Ake.T
        scale = np.abs(A).max()
        assert np.abs(Ac - ref).max() <= 1e-12 * scale
        assert np.abs(Ac.sum(axis=1)).max() <= 1e-10 * scale


def test_elimination_rules():
    L = G.rmat(12)
    S = O.OracleSolver(L)
    inf = S.level_info(0)
    assert inf["type"] == "elim"
    ids = S.level_ids(0)
    A = L.to_scipy()
    deg = np.diff(A.indptr) - 1
    el = np.where(ids < 0)[0]
    assert (deg[el] <= 4).all()
    # new ids of kept vertices are consecutive in index order
    kept = ids[ids >= 0]
    assert (kept == np.arange(len(kept))).all()
    # an eliminated vertex is the smallest candidate of its closed neighbourhood
    cand = deg <= 4
    for i in el[:500]:
        nb = A.indices[A.indptr[i]:A.indptr[i + 1]]
        assert nb[cand[nb]].min() == i


def test_aggregates_are_connected_and_nonempty():
    L = G.grid2d(40, weights="lognormal")
    S = O.OracleSolver(L)
    A = L.to_scipy()
    ids = S.level_ids(0)
    nc = S.level_info(0)["nc"]
    assert ids.min() == 0 and ids.max() == nc - 1
    assert (np.bincount(ids, minlength=nc) > 0).all()
    from scipy.sparse.csgraph import connected_components
    for I in range(0, nc, 7):
        m = np.where(ids == I)[0]
        sub = A[m][:, m]
        assert connected_components(sub, directed=False)[0] == 1


def test_coarse_pseudo_inverse():
    L = G.grid2d(12)
    S = O.OracleSolver(L)
    c = S.num_levels - 1
    assert S.level_info(c)["type"] == "coarse"
    # the coarse cycle is x = L^+ b: L x = b for a mean-free b
    n = S.level_info(c)["n"]
    A = dense(*S.level_matrix(c), n)
    b = np.random.default_rng(0).standard_normal(n)
    b -= b.mean()
    x = S.cycle(c, b)
    assert np.abs(A @ x - b).max() < 1e-10 * np.abs(b).max()
    assert abs(x.mean()) < 1e-12


@pytest.mark.parametrize("kw", [dict(), dict(outer_ksp_type="fcg"),
                                dict(kcycle=1, outer_ksp_type="fcg")])
@pytest.mark.parametrize("name", ["grid", "my_matrix", "rmat12", "rgg"])
def test_oracle_solves(name, kw):
    L = {"grid": lambda: G.grid2d(48), "my_matrix": my_matrix, "rmat12": lambda: G.rmat(12),
         "rgg": lambda: G.rgg(4000, seed=3)}[name]()
    S = O.OracleSolver(L, **kw)
    b = G.rhs(L.n, seed=1)
    x, info = S.solve(b)
    assert info["status"] == 0
    r = b - L.to_scipy() @ x
    assert np.linalg.norm(r) / np.linalg.norm(b) < 1e-7
    assert info["true_rel_residual"] < 1e-7
    assert info["residuals"][-1] <= 1e-8 * info["residuals"][0] * (1 + 1e-12)


def test_oracle_matches_dense_solution():
    L = G.grid2d(20, weights="lognormal", seed=4)
    S = O.OracleSolver(L, kcycle=1, outer_ksp_type="fcg", tol=1e-12)
    b = G.rhs(L.n, seed=2)
    x, _ = S.solve(b)
    xs = np.linalg.pinv(L.to_scipy().toarray(), rcond=1e-10, hermitian=True) @ b
    xs = xs - xs.mean()
    x = x - x.mean()
    assert np.linalg.norm(x - xs) <= 1e-8 * np.linalg.norm(xs)


def test_seed_and_skip_change_test_vectors():
    L = G.grid2d(30, weights="lognormal")
    a = O.OracleSolver(L, seed=1).level_ids(0)
    b = O.OracleSolver(L, seed=1).level_ids(0)
    assert (a == b).all()  # deterministic


def test_invalid_inputs_rejected():
    L = G.grid2d(5)
    v = L.val.copy()
    v[1] = 1.0  # positive off-diagonal, breaks symmetry too
    with pytest.raises(O.OracleError):
        O.OracleSolver(G.Laplacian(L.n, L.rowptr, L.col, v))


def _adjacency(L):
    """Off-diagonal part of a Laplacian as a weighted adjacency CSR."""
    A = -L.to_scipy().tocoo()
    m = A.row != A.col
    import scipy.sparse as sp
    A = sp.csr_matrix((A.data[m], (A.row[m], A.col[m])), shape=L.to_scipy().shape)
    A.sort_indices()
    return A.indptr.astype(np.int64), A.indices.astype(np.int32), A.data.astype(np.float64)


def test_prepare_graph_matches_host_pipeline():
    # R-MAT without the component step has many components; the oracle's
    # --cc/--adj pipeline must give the host generator's LCC Laplacian
    for scale, seed in [(10, 3), (12, 1)]:
        raw = G.rmat(scale, seed=seed, lcc=False)
        ref = G.rmat(scale, seed=seed, lcc=True)
        rp, ci, cv = _adjacency(raw)
        orp, oci, ocv, orig = O.prepare_graph(raw.n, rp, ci, cv, lcc=True, laplacian=True)
        assert len(orp) - 1 == ref.n
        assert np.array_equal(orp, ref.rowptr) and np.array_equal(oci, ref.col)
        assert np.allclose(ocv, ref.val, rtol=1e-14, atol=0)
        assert np.all(np.diff(orig) > 0)
        # laplacian rows sum to zero; lcc-only keeps the input entries
        assert np.abs(ref.to_scipy() @ np.ones(ref.n)).max() <= 1e-12 * np.abs(ref.val).max()
        lrp, lci, lcv, _ = O.prepare_graph(raw.n, raw.rowptr, raw.col, raw.val, lcc=True)
        assert np.array_equal(lrp, ref.rowptr) and np.array_equal(lci, ref.col)


def test_prepare_graph_tie_takes_smaller_label():
    # two paths of 3 vertices: {0, 2, 4} and {1, 3, 5}; labels (largest index)
    # 4 and 5; equal sizes -> the component labelled 4 (max_element, cc.hpp)
    import scipy.sparse as sp
    u = np.array([0, 2, 1, 3])
    v = np.array([2, 4, 3, 5])
    A = sp.coo_matrix((np.ones(4), (u, v)), shape=(6, 6))
    A = (A + A.T).tocsr()
    A.sort_indices()
    rp, ci, cv, orig = O.prepare_graph(6, A.indptr, A.indices, A.data, lcc=True)
    assert list(orig) == [0, 2, 4] and len(rp) == 4 and len(ci) == 4


@pytest.mark.parametrize("iters", [2, 3])
def test_oracle_kcycle_fgmres_matches_dense_solution(iters):
    # K-cycle inner solves by FGMRES (the reference's --kcycle-ksp-type fgmres)
    L = G.grid2d(24, weights="lognormal", seed=4)
    b = G.rhs(L.n, seed=6)
    S = O.OracleSolver(L, kcycle=1, kcycle_ksp_type="fgmres", kcycle_iters=iters,
                       outer_ksp_type="fcg")
    x, info = S.solve(b)
    assert info["status"] == 0 and info["true_rel_residual"] <= 1e-8
    xd = np.linalg.lstsq(L.to_scipy().toarray(), b, rcond=None)[0]
    xd -= xd.mean()
    x = x - x.mean()
    assert np.linalg.norm(x - xd) <= 1e-6 * np.linalg.norm(xd)
    F = O.OracleSolver(L, kcycle=1, kcycle_iters=iters, outer_ksp_type="fcg")
    _, fi = F.solve(b)
    assert abs(info["iters"] - fi["iters"]) <= 3  # same K-cycle, another inner Krylov method


@pytest.mark.parametrize("restart", [30, 3])
def test_oracle_fgmres_matches_dense_solution(restart):
    L = G.grid2d(24, weights="lognormal", seed=4)
    b = G.rhs(L.n, seed=5)
    S = O.OracleSolver(L, kcycle=1, outer_ksp_type="fgmres", gmres_restart=restart)
    x, info = S.solve(b)
    assert info["status"] == 0 and info["true_rel_residual"] <= 1e-8
    xd = np.linalg.lstsq(L.to_scipy().toarray(), b, rcond=None)[0]
    xd -= xd.mean()
    x = x - x.mean()
    assert np.linalg.norm(x - xd) <= 1e-6 * np.linalg.norm(xd)
