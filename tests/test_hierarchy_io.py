"""PETSc-binary hierarchy export/import (dump_hierarchy, ligmg.hpp:47-52):
write the oracle's hierarchy, read it back, and check every array."""
import numpy as np

from conftest import my_matrix
from ligmg_gb300 import petsc_io
from oracle import oracle as O


def test_petsc_mat_and_vec_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    rp = np.array([0, 2, 2, 5], np.int64)
    ci = np.array([0, 3, 1, 2, 4], np.int32)
    v = rng.standard_normal(5)
    petsc_io.write_mat(tmp_path / "m.petsc", 3, 5, rp, ci, v)
    m, n, rp2, ci2, v2 = petsc_io.read_mat(tmp_path / "m.petsc")
    assert (m, n) == (3, 5) and (rp2 == rp).all() and (ci2 == ci).all() and (v2 == v).all()
    raw = open(tmp_path / "m.petsc", "rb").read(4)
    assert int.from_bytes(raw, "big") == petsc_io.MAT_CLASSID  # big-endian header
    petsc_io.write_vec(tmp_path / "v.petsc", v)
    assert (petsc_io.read_vec(tmp_path / "v.petsc") == v).all()


def test_dump_and_load_oracle_hierarchy(tmp_path):
    S = O.OracleSolver(my_matrix())
    levels = S.export_levels()
    petsc_io.dump(levels, tmp_path)
    back = petsc_io.load(tmp_path)
    assert [l.type for l in back] == [l.type for l in levels]
    for a, b in zip(levels, back):
        assert a.n == b.n and (a.rowptr == b.rowptr).all() and (a.col == b.col).all()
        assert (a.val == b.val).all()
        if a.type == "agg":
            assert (a.ids == b.ids).all() and a.nc == b.nc
        if a.type == "elim":
            assert (a.prow == b.prow).all() and (a.pcol == b.pcol).all()
            assert (a.pval == b.pval).all() and (a.q == b.q).all()
