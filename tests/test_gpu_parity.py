"""GPU parity tests: the CUDA path (through the C ABI) against the oracle.

Bars:
  * setup (elimination ids, aggregate ids, every level's matrix): bit-exact;
  * Chebyshev eigenvalue estimate: 1e-12 relative;
  * one FP64 cycle from the finest level: 1e-12 relative after projecting
    out the constant;
  * solves: the FP64-recomputed true residual reaches the tolerance, and the
    FP64 solution matches the oracle's to 1e-6 relative (both are solved to
    rtol 1e-8; the difference is bounded by the condition number).
"""
import numpy as np
import pytest

from conftest import my_matrix
from ligmg_gb300 import Solver
from ligmg_gb300 import graphs as G
from ligmg_gb300._lib import LigmgError
from oracle import oracle as O

pytestmark = pytest.mark.gpu

GRAPHS = {
    "grid32": lambda: G.grid2d(32),
    "grid48_logn": lambda: G.grid2d(48, weights="lognormal", seed=2),
    "my_matrix": my_matrix,
    "rmat12": lambda: G.rmat(12, seed=1),
    "rmat14": lambda: G.rmat(14, seed=5),
    "rgg3000": lambda: G.rgg(3000, seed=3),
    "grid3d_12": lambda: G.grid3d(12, weights="lognormal", seed=1),
}


@pytest.fixture(scope="module", autouse=True)
def _build():
    from ligmg_gb300 import build
    build.build()


def _proj(x):
    return x - x.mean()


def _relerr(a, b):
    return np.linalg.norm(_proj(a) - _proj(b)) / max(np.linalg.norm(_proj(b)), 1e-300)


@pytest.mark.parametrize("name", list(GRAPHS))
def test_setup_bit_exact(name):
    L = GRAPHS[name]()
    S = Solver(L)
    R = O.OracleSolver(L)
    assert S.num_levels == R.num_levels
    for l in range(R.num_levels):
        gi, ri = S.level_info(l), R.level_info(l)
        assert gi == ri, (l, gi, ri)
        grp, gci, gv = S.level_matrix(l)
        rrp, rci, rv = R.level_matrix(l)
        assert (grp == rrp).all() and (gci == rci).all(), l
        assert (gv.view(np.int64) == rv.view(np.int64)).all(), f"level {l} values differ"
        if ri["type"] != "coarse":
            assert (S.level_ids(l) == R.level_ids(l)).all(), f"level {l} ids differ"
        if ri["type"] == "agg":
            assert abs(S.level_lmax(l) - R.level_lmax(l)) <= 1e-12 * R.level_lmax(l)


@pytest.mark.parametrize("opt", [dict(aff_scaling="row"), dict(aff_scaling="column"),
                                 dict(aff_scaling="rowcolumn"), dict(aff_scaling="sym"),
                                 dict(aff_scaling="none"), dict(strength_metric="none"),
                                 dict(strength_metric="algebraic-distance"),
                                 dict(max_agg_size=6), dict(rejection_ratio=1.5),
                                 dict(rejection_ratio=1.0, rejection_to_seed=1),
                                 dict(neighbor_of_neighbor=1)])
def test_setup_options_bit_exact(opt):
    L = GRAPHS["rmat12"]()
    S, R = Solver(L, **opt), O.OracleSolver(L, **opt)
    assert S.num_levels == R.num_levels
    for l in range(R.num_levels - 1):
        assert (S.level_ids(l) == R.level_ids(l)).all(), (opt, l)
        assert (S.level_matrix(l)[2].view(np.int64) == R.level_matrix(l)[2].view(np.int64)).all()


@pytest.mark.parametrize("tail", [-1, 0, 1 << 20])
@pytest.mark.parametrize("kcycle", [0, 1])
@pytest.mark.parametrize("name", ["grid48_logn", "my_matrix", "rmat12", "grid3d_12"])
def test_cycle_fp64_matches_oracle(name, kcycle, tail):
    # tail -1: every level launched; 0: the coarse end as the shared-memory
    # program; 1 << 20: every level below the first as the grid-barrier
    # program (autotune off, so the tail runs whatever its speed)
    L = GRAPHS[name]()
    S = Solver(L, kcycle=kcycle, tail_rows=tail, autotune=0 if tail >= 0 else 1)
    R = O.OracleSolver(L, kcycle=kcycle)
    rng = np.random.default_rng(7)
    for level in range(R.num_levels):
        n = R.level_info(level)["n"]
        b = _proj(rng.standard_normal(n))
        xg, xr = S.cycle(level, b), R.cycle(level, b)
        assert _relerr(xg, xr) <= 1e-12, (level, _relerr(xg, xr))


@pytest.mark.parametrize("kcycle", [0, 1])
def test_jacobi_smoother_matches_oracle(kcycle):
    L = GRAPHS["grid48_logn"]()
    kw = dict(smoother_type="jacobi", kcycle=kcycle, outer_ksp_type="fcg")
    S, R = Solver(L, **kw), O.OracleSolver(L, **kw)
    b = _proj(np.random.default_rng(2).standard_normal(L.n))
    assert _relerr(S.cycle(0, b), R.cycle(0, b)) <= 1e-12
    info = S.solve(G.rhs(L.n, seed=3))
    xr, ir = R.solve(G.rhs(L.n, seed=3))
    assert info.converged and abs(info.iters() - ir["iters"]) <= 1
    assert _relerr(info.solution, xr) <= 1e-6


@pytest.mark.parametrize("name", ["grid48_logn", "rmat12"])
def test_cycle_fp32_close_to_oracle(name):
    L = GRAPHS[name]()
    S = Solver(L, precision="fp32", kcycle=1)
    R = O.OracleSolver(L, kcycle=1)
    b = _proj(np.random.default_rng(3).standard_normal(L.n))
    assert _relerr(S.cycle(0, b), R.cycle(0, b)) <= 1e-4


def test_spmv_matches():
    L = GRAPHS["rmat14"]()
    S = Solver(L)
    x = np.random.default_rng(0).standard_normal(L.n)
    y = S.spmv(0, x)
    ref = L.to_scipy() @ x
    assert np.abs(y - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("cfg", [dict(), dict(outer_ksp_type="fcg"),
                                 dict(kcycle=1, outer_ksp_type="fcg")])
@pytest.mark.parametrize("name", ["grid48_logn", "my_matrix", "rmat14", "rgg3000"])
def test_solve_fp64_matches_oracle(name, cfg):
    L = GRAPHS[name]()
    S = Solver(L, **cfg)
    R = O.OracleSolver(L, **cfg)
    b = G.rhs(L.n, seed=11)
    info = S.solve(b)
    xr, ir = R.solve(b)
    assert info.converged
    assert abs(info.iters() - ir["iters"]) <= 1
    assert info.true_rel_residual <= 1e-7
    r = b - L.to_scipy() @ info.solution
    assert np.linalg.norm(r) / np.linalg.norm(b) <= 1e-7
    assert _relerr(info.solution, xr) <= 1e-6


@pytest.mark.parametrize("name", ["grid48_logn", "rmat14", "grid3d_12"])
def test_solve_fp32_hierarchy_reaches_tol(name):
    L = GRAPHS[name]()
    S = Solver(L, precision="fp32", kcycle=1, outer_ksp_type="fcg")
    b = G.rhs(L.n, seed=5)
    info = S.solve(b)
    assert info.converged
    assert info.true_rel_residual <= 2e-8
    r = b - L.to_scipy() @ info.solution
    assert np.linalg.norm(r) / np.linalg.norm(b) <= 2e-8


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("k", [2, 8, 32])
def test_batched_matches_single(prec, k):
    L = GRAPHS["rmat12"]()
    S = Solver(L, precision=prec, kcycle=1, outer_ksp_type="fcg")
    B = G.rhs(L.n, k=k, seed=9)
    info = S.solve_batched(B)
    assert info.converged
    assert (info.col_true_rel_residual <= 2e-8).all()
    for c in (0, k - 1):
        single = S.solve(B[:, c].copy())
        assert _relerr(info.solution[:, c], single.solution) <= 1e-6


def test_graph_replay_matches_direct_launches():
    L = GRAPHS["rmat14"]()
    B = G.rhs(L.n, k=8, seed=3)
    # fixed launch shapes: two handles then run identical kernels
    kw = dict(precision="fp32", kcycle=1, outer_ksp_type="fcg", autotune=0)
    a = Solver(L, **kw).solve_batched(B)
    b = Solver(L, use_graphs=0, **kw).solve_batched(B)
    assert a.iters() == b.iters()
    assert np.array_equal(a.solution, b.solution)


@pytest.mark.parametrize("prec,k", [("fp32", 32), ("fp32", 8), ("fp64", 1), ("fp32", 1),
                                    ("fp32", 4), ("fp32", 2), ("fp64", 2)])
def test_persistent_tail_matches_launched_levels(prec, k):
    # tail_rows = -1: every level launches its own kernels; otherwise the
    # coarse end runs as one persistent kernel (grid barriers for > 0; for 0,
    # column slices of 8, 4 or 1 columns per CTA in shared memory: k = 32 and
    # 8 use 8, k = 4 uses 4, k = 2 and 1 use 1).  Same operations, so the same
    # iterations and solutions equal to rounding of the reductions.
    L = GRAPHS["rmat14"]()
    B = G.rhs(L.n, k=k, seed=9)
    if k == 1:
        B = B.reshape(L.n, 1)
    kw = dict(precision=prec, kcycle=1, outer_ksp_type="fcg", autotune=0)
    a = Solver(L, tail_rows=-1, **kw).solve_batched(B)
    b = Solver(L, tail_rows=1 << 20, **kw).solve_batched(B)
    assert a.converged and b.converged
    assert a.iters() == b.iters()
    tol = 1e-5 if prec == "fp32" else 1e-10
    assert _relerr(a.solution, b.solution) <= tol
    c = Solver(L, tail_rows=500, **kw).solve_batched(B)  # a shorter tail
    assert c.converged and c.iters() == a.iters()
    assert _relerr(a.solution, c.solution) <= tol
    d = Solver(L, tail_rows=0, **kw)  # shared-memory column slices
    S = d.solve_batched(B)
    assert S.converged and S.iters() == a.iters()
    assert _relerr(a.solution, S.solution) <= tol
    S2 = d.solve_batched(B)  # replayed from the captured graph: identical
    assert np.array_equal(S.solution, S2.solution)


def test_autotuned_shapes_match_fixed_shapes():
    # the tuner changes launch shapes and hub-row chunking only: same
    # iterations, solutions equal to rounding
    L = GRAPHS["rmat14"]()
    B = G.rhs(L.n, k=32, seed=5)
    kw = dict(precision="fp32", kcycle=1, outer_ksp_type="fcg")
    a = Solver(L, autotune=1, **kw).solve_batched(B)
    b = Solver(L, autotune=0, **kw).solve_batched(B)
    assert a.converged and b.converged
    assert abs(a.iters() - b.iters()) <= 1
    assert _relerr(a.solution, b.solution) <= 1e-6
    c = Solver(L, autotune=1, precision="fp64", kcycle=1, outer_ksp_type="fcg")
    x1 = c.solve(B[:, 0].copy())
    x2 = c.solve(B[:, 0].copy())  # same handle, same tuned plans: identical
    assert np.array_equal(x1.solution, x2.solution)


def test_profiled_solve_reports_kernels():
    L = GRAPHS["rmat14"]()
    S = Solver(L, precision="fp32", kcycle=1, outer_ksp_type="fcg")
    S.profile(True)
    info = S.solve_batched(G.rhs(L.n, k=32, seed=4))
    st = S.kernel_stats()
    assert info.converged and st
    assert all(r["seconds"] > 0 and r["bytes"] > 0 and r["launches"] > 0 for r in st)
    kinds = {r["kind"] for r in st}
    assert {"cheb_b", "resid", "spmv"} <= kinds


def test_solve_from_level():
    L = GRAPHS["my_matrix"]()
    S = Solver(L, outer_ksp_type="fcg")
    R = O.OracleSolver(L, outer_ksp_type="fcg")
    n1 = R.level_info(1)["n"]
    b = _proj(np.random.default_rng(1).standard_normal(n1))
    info = S.solve(b, from_level=1)
    xr, ir = R.solve(b, from_level=1)
    assert info.converged and _relerr(info.solution, xr) <= 1e-6


def _bad(L, mutate):
    rp, ci, v = L.rowptr.copy(), L.col.copy(), L.val.copy()
    mutate(rp, ci, v)
    return (L.n, rp, ci, v)


def test_invalid_inputs_return_status():
    L = G.grid2d(6)
    off = int(np.where(L.col[: L.rowptr[1]] == 1)[0][0])          # entry (0, 1)
    mirror = int(L.rowptr[1] + np.where(L.col[L.rowptr[1]: L.rowptr[2]] == 0)[0][0])  # (1, 0)

    def positive(rp, ci, v):
        v[off] = 0.5
        v[mirror] = 0.5

    cases = {
        3: lambda rp, ci, v: v.__setitem__(off, -2.0),            # not symmetric
        5: positive,                                              # positive off-diagonal
        6: lambda rp, ci, v: v.__setitem__(0, np.nan),            # non-finite
        4: lambda rp, ci, v: v.__setitem__(0, -1.0),              # bad diagonal
    }
    for code, mut in cases.items():
        with pytest.raises(LigmgError) as e:
            Solver(_bad(L, mut))
        assert e.value.status == code


def test_unsupported_k_rejected():
    L = GRAPHS["grid32"]()
    S = Solver(L)
    with pytest.raises(LigmgError):
        S.solve_batched(np.zeros((L.n, 3)))


@pytest.mark.parametrize("name", ["my_matrix", "rmat12"])
def test_cycle_on_imported_oracle_hierarchy(name, tmp_path):
    """Parity on an exported hierarchy: import the oracle's
    hierarchy (written to PETSc binary and read back) and compare one FP64
    cycle and a full solve with the oracle's."""
    from ligmg_gb300 import petsc_io
    L = GRAPHS[name]()
    kw = dict(kcycle=1, outer_ksp_type="fcg")
    R = O.OracleSolver(L, **kw)
    petsc_io.dump(R.export_levels(), tmp_path)
    S = Solver.import_hierarchy(petsc_io.load(tmp_path), **kw)
    assert S.num_levels == R.num_levels
    for l in range(R.num_levels - 1):
        assert abs(S.level_lmax(l) - R.level_lmax(l)) <= 1e-12 * max(R.level_lmax(l), 1)
    b = _proj(np.random.default_rng(5).standard_normal(L.n))
    assert _relerr(S.cycle(0, b), R.cycle(0, b)) <= 1e-12
    info = S.solve(G.rhs(L.n, seed=6))
    xr, _ = R.solve(G.rhs(L.n, seed=6))
    assert info.converged and _relerr(info.solution, xr) <= 1e-6


def test_gpu_dump_import_round_trip(tmp_path):
    L = GRAPHS["rmat12"]()
    S = Solver(L, kcycle=1, outer_ksp_type="fcg", autotune=0)
    S.dump_hierarchy(str(tmp_path))
    from ligmg_gb300 import petsc_io
    T = Solver.import_hierarchy(petsc_io.load(tmp_path), kcycle=1, outer_ksp_type="fcg",
                                autotune=0)
    b = G.rhs(L.n, seed=8)
    a, c = S.solve(b), T.solve(b)
    assert a.iters() == c.iters() and np.array_equal(a.solution, c.solution)


def test_pcg_jacobi_baseline():
    L = GRAPHS["grid48_logn"]()
    S = Solver(L, iters=5000)
    b = G.rhs(L.n, seed=12)
    info = S.solve_pcg_jacobi(b)
    assert info.converged
    r = b - L.to_scipy() @ info.solution
    assert np.linalg.norm(r) / np.linalg.norm(b) <= 2e-8
    mg = S.solve(b)
    assert mg.iters() < info.iters()  # multigrid needs far fewer iterations


@pytest.mark.parametrize("name", ["grid48_logn", "rmat12"])
def test_kcycle_fgmres_cycle_matches_oracle(name):
    # K-cycle inner solves by FGMRES (--kcycle-ksp-type fgmres): the FP64 cycle
    # of every level against the oracle
    L = GRAPHS[name]()
    kw = dict(kcycle=1, kcycle_ksp_type="fgmres")
    S, R = Solver(L, **kw), O.OracleSolver(L, **kw)
    rng = np.random.default_rng(8)
    for level in range(R.num_levels):
        b = _proj(rng.standard_normal(R.level_info(level)["n"]))
        xg, xr = S.cycle(level, b), R.cycle(level, b)
        assert _relerr(xg, xr) <= 1e-12, (level, _relerr(xg, xr))


@pytest.mark.parametrize("prec,k", [("fp64", 1), ("fp32", 8)])
def test_kcycle_fgmres_solve_matches_oracle(prec, k):
    L = GRAPHS["rmat12"]()
    kw = dict(kcycle=1, kcycle_ksp_type="fgmres", outer_ksp_type="fcg")
    S = Solver(L, precision=prec, **kw)
    R = O.OracleSolver(L, **kw)
    B = G.rhs(L.n, k=k, seed=13)
    if k == 1:
        B = B.reshape(L.n, 1)
    info = S.solve_batched(B)
    assert info.converged and (info.col_true_rel_residual <= 2e-8).all()
    S2 = S.solve_batched(B)  # replayed from the captured graphs: identical
    assert np.array_equal(info.solution, S2.solution)
    for c in (0, k - 1):
        xr, ir = R.solve(B[:, c].copy())
        assert ir["status"] == 0
        assert abs(int(info.col_iters[c]) - ir["iters"]) <= 1
        assert _relerr(info.solution[:, c], xr) <= 1e-6


@pytest.mark.parametrize("prec,k,restart", [("fp64", 1, 30), ("fp32", 8, 30), ("fp64", 1, 3)])
def test_fgmres_outer_matches_oracle(prec, k, restart):
    # FGMRES(m) outer iterations (the reference's --outer-ksp-type fgmres)
    L = GRAPHS["grid48_logn"]()
    kw = dict(kcycle=1, outer_ksp_type="fgmres", gmres_restart=restart)
    S = Solver(L, precision=prec, **kw)
    R = O.OracleSolver(L, **kw)
    B = G.rhs(L.n, k=k, seed=11)
    if k == 1:
        B = B.reshape(L.n, 1)
    info = S.solve_batched(B)
    assert info.converged and (info.col_true_rel_residual <= 2e-8).all()
    for c in (0, k - 1):
        xr, ir = R.solve(B[:, c].copy())
        assert ir["status"] == 0
        assert abs(int(info.col_iters[c]) - ir["iters"]) <= 1
        assert _relerr(info.solution[:, c], xr) <= 1e-6


@pytest.mark.parametrize("scale", [16, 18])
def test_rmat_setup_bit_exact_at_scale(scale):
    # larger R-MAT hierarchies (the headline graph is scale 20; bench.py
    # checks it against the oracle in every run): every level's CSR, value
    # bits and ids
    L = G.rmat(scale, seed=0)
    S, R = Solver(L, kcycle=1, outer_ksp_type="fcg"), O.OracleSolver(L, kcycle=1,
                                                                      outer_ksp_type="fcg")
    assert S.num_levels == R.num_levels
    for l in range(R.num_levels):
        assert S.level_info(l) == R.level_info(l), l
        grp, gci, gv = S.level_matrix(l)
        rrp, rci, rv = R.level_matrix(l)
        assert np.array_equal(grp, rrp) and np.array_equal(gci, rci), l
        assert np.array_equal(gv.view(np.int64), rv.view(np.int64)), l
        if R.level_info(l)["type"] != "coarse":
            assert np.array_equal(S.level_ids(l), R.level_ids(l)), l
    base = 1 if R.level_info(0)["type"] == "elim" else 0
    b = _proj(np.random.default_rng(9).standard_normal(R.level_info(base)["n"]))
    assert _relerr(S.cycle(base, b), R.cycle(base, b)) <= 1e-12


def test_grid256_plain_fp64_vcycle_matches_oracle():
    # the C1 configuration: 256 x 256 5-point grid, unit weights, FP64
    # V-cycle with Chebyshev(2,2) preconditioning FCG to rtol 1e-8
    L = G.grid2d(256)
    kw = dict(kcycle=0, outer_ksp_type="fcg", pre_smooth=2, post_smooth=2)
    S, R = Solver(L, **kw), O.OracleSolver(L, **kw)
    assert S.num_levels == R.num_levels
    for l in range(R.num_levels - 1):
        assert np.array_equal(S.level_ids(l), R.level_ids(l)), l
        assert np.array_equal(S.level_matrix(l)[2].view(np.int64),
                              R.level_matrix(l)[2].view(np.int64)), l
    b = G.rhs(L.n, seed=7)
    assert _relerr(S.cycle(0, b), R.cycle(0, b)) <= 1e-12
    info = S.solve(b)
    xr, ir = R.solve(b)
    assert info.converged and abs(info.iters() - ir["iters"]) <= 1
    assert info.true_rel_residual <= 1e-8
    assert _relerr(info.solution, xr) <= 1e-6
