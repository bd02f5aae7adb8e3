"""Generate the committed fixtures under tests/golden/.

1. my_matrix_edges.npz — the reference's only data fixture,
   examples/my_matrix.mtx (a 986-vertex integer graph Laplacian), reduced to
   its strictly-lower edge list (u > v, weight = -L[u, v]).  Read from the
   reference checkout when it is present (this script is the only place that
   reads it).
2. oracle_my_matrix.npz — hierarchy summary produced by the CPU oracle on that
   fixture with default options (level types, sizes, nnz, a digest of every
   level's ids and matrix values).  It pins the oracle against itself across
   builds and hosts (x86_64 here, aarch64 on the GPU host).

Run: python tests/golden/make_golden.py [path/to/reference/checkout]
(the checkout defaults to $LIGMG_REFERENCE; the fixture is its
examples/my_matrix.mtx)
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
REF_ROOT = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LIGMG_REFERENCE", "")
REF_MTX = os.path.join(REF_ROOT, "examples", "my_matrix.mtx") if REF_ROOT else ""


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def make_edges():
    out = os.path.join(HERE, "my_matrix_edges.npz")
    if not REF_MTX or not os.path.exists(REF_MTX):
        if os.path.exists(out):
            return
        raise SystemExit("reference fixture not available")
    import scipy.io
    A = scipy.io.mmread(REF_MTX).tocoo()
    m = A.row > A.col
    u, v, w = A.row[m].astype(np.int32), A.col[m].astype(np.int32), -A.data[m].astype(np.float64)
    np.savez_compressed(out, n=np.int64(A.shape[0]), u=u, v=v, w=w)


def make_oracle_summary():
    from oracle import oracle as O
    from tests.conftest import my_matrix
    L = my_matrix()
    S = O.OracleSolver(L)
    rows = []
    for l in range(S.num_levels):
        inf = S.level_info(l)
        rp, ci, cv = S.level_matrix(l)
        ids = S.level_ids(l) if inf["type"] != "coarse" else np.zeros(0, np.int32)
        rows.append((inf["type"], inf["n"], inf["nnz"], inf["nc"], digest(ids), digest(rp, ci, cv)))
    np.savez(os.path.join(HERE, "oracle_my_matrix.npz"),
             types=np.array([r[0] for r in rows]), n=np.array([r[1] for r in rows]),
             nnz=np.array([r[2] for r in rows]), nc=np.array([r[3] for r in rows]),
             ids_digest=np.array([r[4] for r in rows]), mat_digest=np.array([r[5] for r in rows]))


if __name__ == "__main__":
    make_edges()
    make_oracle_summary()
    print("written to", HERE)
