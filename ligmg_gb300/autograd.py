"""PyTorch autograd wrapper of the forward/backward pair (ligmg_forward /
ligmg_backward): x = L(w)^+ b for a graph with a fixed edge list.

    x = LaplacianSolve.apply(w, b, edges, options)

w: edge weights (float64, length m), b: right-hand side (float64, length n),
edges: (u, v) int arrays with u != v, each undirected edge once.  x is the
mean-free solution; gradients flow to w (dloss/dw_e = -(x_u - x_v)(lam_u - lam_v))
and to b (the mean-free adjoint solution).  The solve itself runs in
libligmg_gb300 on the GPU; torch only carries the tensors.

A forward or adjoint solve that stops at the iteration limit
(LIGMG_NOT_CONVERGED) raises NotConvergedError: its x or its gradients would
be wrong, so neither is returned.
"""
import numpy as np

from . import graphs as G
from .solver import Solver

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None


class NotConvergedError(RuntimeError):
    """A solve inside LaplacianSolve reached the iteration limit."""


def edge_positions(L, u, v):
    """CSR position of entry (u[e], v[e]) for every edge."""
    rp, ci = L.rowptr, L.col
    pos = np.empty(len(u), dtype=np.int64)
    for e, (a, b) in enumerate(zip(u, v)):
        lo, hi = rp[a], rp[a + 1]
        pos[e] = lo + np.searchsorted(ci[lo:hi], b)
    return pos


def require_converged(info, what):
    """Raise NotConvergedError unless `info` (a ConvergenceInfo) converged."""
    if not info.converged:
        raise NotConvergedError(
            f"{what} stopped after {info.iters()} iterations without reaching the tolerance "
            f"(true relative residual {info.true_rel_residual:.3e})")
    return info


if torch is not None:
    class LaplacianSolve(torch.autograd.Function):
        @staticmethod
        def forward(ctx, w, b, edges, options=None):
            u, v = edges
            n = b.shape[0]
            L = G.laplacian_from_edges(n, u, v, w.detach().cpu().numpy())
            S = Solver(L, options) if options is not None else Solver(L)
            info = require_converged(S.forward(b.detach().cpu().numpy()), "forward solve")
            x = info.solution - info.solution.mean()
            ctx.solver = S
            ctx.pos = edge_positions(L, np.asarray(u), np.asarray(v))
            return torch.from_numpy(x).to(b.device)

        @staticmethod
        def backward(ctx, gx):
            g = gx.detach().cpu().numpy().astype(np.float64)
            g = g - g.mean()  # x is mean-free: only the mean-free part of g matters
            dw, db, info = ctx.solver.backward(g, with_info=True)
            require_converged(info, "adjoint solve")
            gw = torch.from_numpy(dw[ctx.pos].copy()).to(gx.device)
            gb = torch.from_numpy(db).to(gx.device)
            return gw, gb, None, None
