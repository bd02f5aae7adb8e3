"""Synthetic graph Laplacians and right-hand sides for the solver's workloads.

Host-side input generation (numpy/scipy); it is not part of the solve path.

Workloads (seeded, shapes as named by the benchmark configurations):
  grid2d(256)              2-D 5-point grid, unit weights
  grid3d(128, lognormal)   3-D 7-point grid, weights lognormal(0, 1)
  rmat(scale, 16)          R-MAT (a,b,c,d) = (.57,.19,.19,.05), symmetrised,
                           self-loops and duplicates dropped, largest connected
                           component, weights uniform(0.5, 2.0)
  rgg(n)                   random geometric graph in the unit square, radius
                           for mean degree ~12, weights clip(1/dist, 0.1, 10),
                           largest connected component
The reference reads graphs from MatrixMarket files (src/main.cpp:39) and can
convert adjacency matrices to Laplacians (src/main.cpp:81-110); read_mtx and
laplacian_from_edges cover those inputs.
"""
from dataclasses import dataclass

import numpy as np
import scipy.sparse as sp
from scipy.sparse.csgraph import connected_components


@dataclass
class Laplacian:
    n: int
    rowptr: np.ndarray  # int64[n+1]
    col: np.ndarray     # int32[nnz], ascending per row
    val: np.ndarray     # float64[nnz]
    name: str = ""

    @property
    def nnz(self) -> int:
        return int(self.rowptr[-1])

    def to_scipy(self) -> sp.csr_matrix:
        return sp.csr_matrix((self.val, self.col, self.rowptr), shape=(self.n, self.n))


def laplacian_from_edges(n, u, v, w, name="") -> Laplacian:
    """L = D - W for undirected edges (u, v, w) with u != v, each listed once."""
    u = np.asarray(u, dtype=np.int64)
    v = np.asarray(v, dtype=np.int64)
    w = np.asarray(w, dtype=np.float64)
    rows = np.concatenate([u, v, np.arange(n, dtype=np.int64)])
    cols = np.concatenate([v, u, np.arange(n, dtype=np.int64)])
    deg = np.bincount(u, weights=w, minlength=n) + np.bincount(v, weights=w, minlength=n)
    vals = np.concatenate([-w, -w, deg])
    A = sp.csr_matrix((vals, (rows, cols)), shape=(n, n))
    A.sum_duplicates()
    A.sort_indices()
    return Laplacian(n, A.indptr.astype(np.int64), A.indices.astype(np.int32),
                     A.data.astype(np.float64), name)


def largest_cc_edges(n, u, v, w):
    """Restrict an undirected edge list to its largest connected component
    (the reference's largest_cc, include/ligmg/cc.hpp:24-106), relabelled in
    ascending original order."""
    G = sp.coo_matrix((np.ones(len(u)), (u, v)), shape=(n, n)).tocsr()
    ncomp, labels = connected_components(G, directed=False)
    if ncomp == 1:
        return n, u, v, w
    big = np.bincount(labels).argmax()
    keep = labels == big
    newid = -np.ones(n, dtype=np.int64)
    newid[keep] = np.arange(int(keep.sum()))
    m = keep[u] & keep[v]
    return int(keep.sum()), newid[u[m]], newid[v[m]], w[m]


def grid2d(nx, ny=None, weights="unit", seed=0) -> Laplacian:
    ny = nx if ny is None else ny
    idx = np.arange(nx * ny).reshape(ny, nx)
    u = np.concatenate([idx[:, :-1].ravel(), idx[:-1, :].ravel()])
    v = np.concatenate([idx[:, 1:].ravel(), idx[1:, :].ravel()])
    w = _weights(len(u), weights, seed)
    return laplacian_from_edges(nx * ny, u, v, w, f"grid2d_{nx}x{ny}")


def grid3d(nx, weights="unit", seed=0) -> Laplacian:
    idx = np.arange(nx ** 3).reshape(nx, nx, nx)
    u = np.concatenate([idx[:, :, :-1].ravel(), idx[:, :-1, :].ravel(), idx[:-1, :, :].ravel()])
    v = np.concatenate([idx[:, :, 1:].ravel(), idx[:, 1:, :].ravel(), idx[1:, :, :].ravel()])
    w = _weights(len(u), weights, seed)
    return laplacian_from_edges(nx ** 3, u, v, w, f"grid3d_{nx}")


def _weights(m, law, seed):
    rng = np.random.default_rng(seed + 1)
    if law == "unit":
        return np.ones(m)
    if law == "lognormal":
        return rng.lognormal(0.0, 1.0, m)
    if law == "uniform":
        return rng.uniform(0.5, 2.0, m)
    raise ValueError(law)


def rmat(scale, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=0, weights="uniform",
         lcc=True) -> Laplacian:
    n = 1 << scale
    m = edge_factor * n
    rng = np.random.default_rng(seed)
    u = np.zeros(m, dtype=np.int64)
    v = np.zeros(m, dtype=np.int64)
    ab, abc = a + b, a + b + c
    for bit in range(scale):
        r = rng.random(m)
        ubit = r >= ab                      # quadrants c, d: row bit set
        vbit = ((r >= a) & (r < ab)) | (r >= abc)   # quadrants b, d: col bit set
        u |= ubit.astype(np.int64) << bit
        v |= vbit.astype(np.int64) << bit
    keep = u != v
    u, v = u[keep], v[keep]
    lo, hi = np.minimum(u, v), np.maximum(u, v)
    key = np.unique(lo * n + hi)
    u, v = key // n, key % n
    w = _weights(len(u), weights, seed)
    if lcc:
        n, u, v, w = largest_cc_edges(n, u, v, w)
    return laplacian_from_edges(n, u, v, w, f"rmat{scale}")


def rgg(n, mean_degree=12.0, seed=0, lcc=True) -> Laplacian:
    from scipy.spatial import cKDTree
    rng = np.random.default_rng(seed)
    pts = rng.random((n, 2))
    r = np.sqrt(mean_degree / (np.pi * n))
    pairs = cKDTree(pts).query_pairs(r, output_type="ndarray")
    u, v = pairs[:, 0].astype(np.int64), pairs[:, 1].astype(np.int64)
    d = np.linalg.norm(pts[u] - pts[v], axis=1)
    w = np.clip(1.0 / np.maximum(d, 1e-300), 0.1, 10.0)
    if lcc:
        n, u, v, w = largest_cc_edges(n, u, v, w)
    return laplacian_from_edges(n, u, v, w, f"rgg{n}")


def read_mtx(path, adjacency=False) -> Laplacian:
    """MatrixMarket reader (ParallelReadMM, src/main.cpp:39).  With
    adjacency=True the file holds edge weights and L = D - W is formed."""
    import scipy.io
    A = scipy.io.mmread(path).tocoo()
    n = A.shape[0]
    if adjacency:
        m = A.row < A.col
        return laplacian_from_edges(n, A.row[m], A.col[m], np.abs(A.data[m]).astype(np.float64))
    A = A.tocsr()
    A.sum_duplicates()
    A.sort_indices()
    return Laplacian(n, A.indptr.astype(np.int64), A.indices.astype(np.int32),
                     A.data.astype(np.float64), str(path))


def union(graphs):
    """Block-diagonal union of Laplacians: (vertex_offsets, Laplacian)."""
    offs = np.zeros(len(graphs) + 1, dtype=np.int64)
    for g, L in enumerate(graphs):
        offs[g + 1] = offs[g] + L.n
    rp = [np.zeros(1, dtype=np.int64)]
    base = 0
    for g, L in enumerate(graphs):
        rp.append(L.rowptr[1:] + base)
        base += L.nnz
    col = np.concatenate([L.col.astype(np.int64) + offs[g] for g, L in enumerate(graphs)])
    val = np.concatenate([L.val for L in graphs])
    U = Laplacian(int(offs[-1]), np.concatenate(rp), col.astype(np.int32), val,
                  f"union{len(graphs)}")
    return offs, U


def rgg_batch(count=256, nmin=10_000, nmax=200_000, seed=0):
    """The uneven batch workload: `count` random geometric graphs with vertex
    counts log-uniform in [nmin, nmax], mean degree ~12, weights
    clip(1/dist, 0.1, 10), largest component each."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(nmin), np.log(nmax), count)).astype(np.int64)
    return [rgg(int(n), seed=seed + 1 + g) for g, n in enumerate(sizes)]


def rhs(n, k=1, seed=0) -> np.ndarray:
    """Zero-mean N(0,1) right-hand side(s); k > 1 gives an n x k row-major block."""
    rng = np.random.default_rng(seed + 12345)
    B = rng.standard_normal((n, k))
    B -= B.mean(axis=0, keepdims=True)
    return B[:, 0].copy() if k == 1 else np.ascontiguousarray(B)
