"""Hierarchy export/import.

dump_hierarchy (include/ligmg/ligmg.hpp:47-52) writes, for level i, the files
  i_A.petsc  (every level)        i_P.petsc, i_R.petsc  (elimination and
  i_Q.petsc  (elimination)        aggregation levels)
in PETSc's binary format (write_petsc, util.hpp:589-599; big-endian int32
header, row lengths, column indices, FP64 values).  We add i_ids.petsc (the
aggregate / coarse ids as a PETSc Vec) and meta.txt (level types), so a
hierarchy written here, or by a reference run elsewhere, can be read back and
imported with ligmg_import_hierarchy.
"""
import os
from dataclasses import dataclass, field

import numpy as np

MAT_CLASSID = 1211216
VEC_CLASSID = 1211214


@dataclass
class Level:
    type: str
    n: int
    rowptr: np.ndarray
    col: np.ndarray
    val: np.ndarray
    nc: int = 0
    ids: np.ndarray = None
    prow: np.ndarray = None
    pcol: np.ndarray = None
    pval: np.ndarray = None
    q: np.ndarray = None
    extra: dict = field(default_factory=dict)


def write_mat(path, nrows, ncols, rowptr, col, val):
    rowptr = np.asarray(rowptr, dtype=np.int64)
    with open(path, "wb") as f:
        np.array([MAT_CLASSID, nrows, ncols, rowptr[-1]], dtype=">i4").tofile(f)
        np.diff(rowptr).astype(">i4").tofile(f)
        np.asarray(col, dtype=">i4").tofile(f)
        np.asarray(val, dtype=">f8").tofile(f)


def read_mat(path):
    with open(path, "rb") as f:
        hdr = np.fromfile(f, dtype=">i4", count=4)
        if hdr[0] != MAT_CLASSID:
            raise ValueError(f"{path}: not a PETSc Mat")
        m, n, nz = int(hdr[1]), int(hdr[2]), int(hdr[3])
        lens = np.fromfile(f, dtype=">i4", count=m).astype(np.int64)
        col = np.fromfile(f, dtype=">i4", count=nz).astype(np.int32)
        val = np.fromfile(f, dtype=">f8", count=nz).astype(np.float64)
    rowptr = np.zeros(m + 1, dtype=np.int64)
    np.cumsum(lens, out=rowptr[1:])
    return m, n, rowptr, col, val


def write_vec(path, x):
    with open(path, "wb") as f:
        np.array([VEC_CLASSID, len(x)], dtype=">i4").tofile(f)
        np.asarray(x, dtype=">f8").tofile(f)


def read_vec(path):
    with open(path, "rb") as f:
        hdr = np.fromfile(f, dtype=">i4", count=2)
        if hdr[0] != VEC_CLASSID:
            raise ValueError(f"{path}: not a PETSc Vec")
        return np.fromfile(f, dtype=">f8", count=int(hdr[1])).astype(np.float64)


def _transpose(n, nc, rowptr, col, val):
    import scipy.sparse as sp
    T = sp.csr_matrix((val, col, rowptr), shape=(n, nc)).T.tocsr()
    T.sort_indices()
    return T.indptr.astype(np.int64), T.indices.astype(np.int32), T.data


def dump(levels, directory):
    os.makedirs(directory, exist_ok=True)
    with open(os.path.join(directory, "meta.txt"), "w") as f:
        f.write(" ".join(lv.type for lv in levels) + "\n")
    for i, lv in enumerate(levels):
        pre = os.path.join(directory, f"{i}_")
        write_mat(pre + "A.petsc", lv.n, lv.n, lv.rowptr, lv.col, lv.val)
        if lv.type == "coarse":
            continue
        if lv.type == "agg":
            prow = np.arange(lv.n + 1, dtype=np.int64)
            pcol, pval = lv.ids.astype(np.int32), np.ones(lv.n)
            write_vec(pre + "ids.petsc", lv.ids.astype(np.float64))
        else:
            prow, pcol, pval = lv.prow, lv.pcol, lv.pval
            write_mat(pre + "Q.petsc", lv.n, lv.n, np.concatenate([[0], np.cumsum(lv.q != 0)]),
                      np.where(lv.q != 0)[0], lv.q[lv.q != 0])
        write_mat(pre + "P.petsc", lv.n, lv.nc, prow, pcol, pval)
        write_mat(pre + "R.petsc", lv.nc, lv.n, *_transpose(lv.n, lv.nc, prow, pcol, pval))


def load(directory):
    types = open(os.path.join(directory, "meta.txt")).read().split()
    levels = []
    for i, t in enumerate(types):
        pre = os.path.join(directory, f"{i}_")
        n, _, rp, ci, cv = read_mat(pre + "A.petsc")
        lv = Level(t, n, rp, ci, cv)
        if t != "coarse":
            _, nc, prow, pcol, pval = read_mat(pre + "P.petsc")
            lv.nc = nc
            if t == "agg":
                lv.ids = pcol.astype(np.int32)
            else:
                lv.prow, lv.pcol, lv.pval = prow, pcol, pval
                _, _, qr, qc, qv = read_mat(pre + "Q.petsc")
                q = np.zeros(n)
                rows = np.repeat(np.arange(n), np.diff(qr))
                q[rows] = qv
                lv.q = q
        levels.append(lv)
    return levels
