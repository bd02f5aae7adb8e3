"""Python mirror of the reference's solver interface.

  Solver(A) / Solver(A, options)   ligmg::Solver (include/ligmg/ligmg.hpp:17-28)
  Solver.solve(b)                  ligmg.hpp:31-33
  Solver.solve(b, from_level)      ligmg.hpp:36-38
  Solver.print()                   print_hierarchy (multigrid.hpp:265-292)
  Solver.dump_csv(f, info)         print_csv_header / print_csv (util.hpp:187-205)
  ConvergenceInfo                  util.hpp:143-170

Everything runs through libligmg_gb300.so on the GPU; there is no CPU path.
"""
import ctypes as C
import math
import sys

import numpy as np

from . import _abi
from ._lib import check, lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class ConvergenceInfo:
    """ConvergenceInfo (util.hpp:143-170) plus the FP64 true residual."""

    def __init__(self, residuals, iters, time, work, solution, true_rel_residual, converged,
                 col_iters=None, col_true=None, cycle_complexity_value=0.0):
        self.residuals = np.asarray(residuals)
        self._iters = int(iters)
        self._time = float(time)
        self._work = float(work)
        self.solution = solution
        self.true_rel_residual = float(true_rel_residual)
        self.converged = bool(converged)
        self.col_iters = col_iters
        self.col_true_rel_residual = col_true
        self._cc = cycle_complexity_value

    def iters(self):
        return self._iters

    def time(self):
        return self._time

    def work(self):
        return self._work

    def rel_residual(self):
        return float(self.residuals[-1] / self.residuals[0]) if len(self.residuals) else 0.0

    def cycle_complexity(self):
        return self._work / self._iters if self._iters else self._cc

    def cf(self):
        return self.rel_residual() ** (1.0 / self._iters) if self._iters else 0.0

    def ecf(self):
        if not self._iters or self.cycle_complexity() == 0:
            return 0.0
        return self.rel_residual() ** (1.0 / (self._iters * self.cycle_complexity()))

    def wda(self):
        e = self.ecf()
        return -1.0 / math.log10(e) if 0 < e < 1 else float("inf")

    def __str__(self):
        return ("iters    error  comp  conv econv   wda     time\n"
                f"{self._iters:5d} {self.rel_residual():.2e} {self.cycle_complexity():5.2f} "
                f"{self.cf():.3f} {self.ecf():.3f} {self.wda():5.2f} {self._time:.2e}")


class Solver:
    """GPU LigMG solver for a graph Laplacian given as CSR (int64 rowptr,
    int32 sorted columns, float64 values) or a graphs.Laplacian."""

    def __init__(self, A, options: _abi.Options = None, **kw):
        if hasattr(A, "rowptr"):
            n, rp, ci, v = A.n, A.rowptr, A.col, A.val
        else:
            n, rp, ci, v = A
        self.n = int(n)
        self._rp = np.ascontiguousarray(rp, dtype=np.int64)
        self._ci = np.ascontiguousarray(ci, dtype=np.int32)
        self._v = np.ascontiguousarray(v, dtype=np.float64)
        self.options = options if options is not None else _abi.default_options(**kw)
        h = C.c_void_p()
        check(lib().ligmg_create(self.n, _p(self._rp), _p(self._ci), _p(self._v),
                                 C.byref(self.options), C.byref(h)), "ligmg_create")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().ligmg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- hierarchy ----------------------------------------------------------
    @property
    def num_levels(self):
        x = C.c_int32()
        check(lib().ligmg_hierarchy_levels(self._h, C.byref(x)))
        return x.value

    def level_info(self, level):
        t, n, nnz, nc = C.c_int32(), C.c_int64(), C.c_int64(), C.c_int64()
        check(lib().ligmg_level_info(self._h, level, C.byref(t), C.byref(n), C.byref(nnz),
                                     C.byref(nc)))
        return {"type": _abi.LEVEL_TYPES[t.value], "n": n.value, "nnz": nnz.value, "nc": nc.value}

    def level_matrix(self, level):
        inf = self.level_info(level)
        rp = np.empty(inf["n"] + 1, np.int64)
        ci = np.empty(inf["nnz"], np.int32)
        v = np.empty(inf["nnz"], np.float64)
        check(lib().ligmg_level_matrix(self._h, level, _p(rp), _p(ci), _p(v)))
        return rp, ci, v

    def level_ids(self, level):
        ids = np.empty(self.level_info(level)["n"], np.int32)
        check(lib().ligmg_level_ids(self._h, level, _p(ids)))
        return ids

    SETUP_PHASES = ("validate", "elimination", "aggregation", "galerkin", "solve_data",
                    "smoother", "coarse")

    def setup_times(self):
        """Seconds per setup phase (ligmg_setup_times)."""
        arr = (C.c_double * len(self.SETUP_PHASES))()
        check(lib().ligmg_setup_times(self._h, arr))
        return dict(zip(self.SETUP_PHASES, list(arr)))

    def level_lmax(self, level):
        x = C.c_double()
        check(lib().ligmg_level_lmax(self._h, level, C.byref(x)))
        return x.value

    def print(self, file=sys.stdout):
        """print_hierarchy (multigrid.hpp:265-292) at one GPU."""
        print(f"{'Level':>5}  {'Size':>10}  {'NNZ':>12}  {'Type':>6}", file=file)
        for l in range(self.num_levels):
            i = self.level_info(l)
            print(f"{l:5d}  {i['n']:10d}  {i['nnz']:12d}  {i['type']:>6}", file=file)

    # ---- solve ----------------------------------------------------------------
    def _info(self, k, history=1024):
        info = _abi.Info()
        hist = np.zeros(history)
        ci = np.zeros(k, np.int32)
        ct = np.zeros(k)
        info.residual_history = hist.ctypes.data_as(C.POINTER(C.c_double))
        info.history_capacity = history
        info.col_iters = ci.ctypes.data_as(C.POINTER(C.c_int32))
        info.col_true_rel_residual = ct.ctypes.data_as(C.POINTER(C.c_double))
        return info, hist, ci, ct

    def solve(self, b, from_level=None) -> ConvergenceInfo:
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.empty_like(b)
        info, hist, ci, ct = self._info(1)
        if from_level is None:
            st = check(lib().ligmg_solve(self._h, _p(b), _p(x), C.byref(info)), "ligmg_solve")
        else:
            st = check(lib().ligmg_solve_from(self._h, _p(b), _p(x), int(from_level),
                                              C.byref(info)), "ligmg_solve_from")
        return ConvergenceInfo(hist[: info.history_len].copy(), info.iters, info.solve_seconds,
                               info.work, x, info.true_rel_residual, st == 0, ci, ct,
                               info.cycle_complexity)

    def solve_pcg_jacobi(self, b) -> ConvergenceInfo:
        """Jacobi-preconditioned CG on the input matrix (the reference's
        --test-cg comparison, src/main.cpp:168-180)."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.empty_like(b)
        info, hist, ci, ct = self._info(1, history=self.options.iters + 2)
        st = check(lib().ligmg_solve_pcg_jacobi(self._h, _p(b), _p(x), C.byref(info)),
                   "ligmg_solve_pcg_jacobi")
        return ConvergenceInfo(hist[: info.history_len].copy(), info.iters, info.solve_seconds,
                               info.work, x, info.true_rel_residual, st == 0, ci, ct,
                               info.cycle_complexity)

    def solve_batched(self, B) -> ConvergenceInfo:
        """k right-hand sides as an n x k row-major block (k in 1,2,4,...,64)."""
        B = np.ascontiguousarray(B, dtype=np.float64)
        k = B.shape[1]
        X = np.empty_like(B)
        info, hist, ci, ct = self._info(k)
        st = check(lib().ligmg_solve_batched(self._h, _p(B), k, _p(X), C.byref(info)),
                   "ligmg_solve_batched")
        return ConvergenceInfo(hist[: info.history_len].copy(), info.iters, info.solve_seconds,
                               info.work, X, info.true_rel_residual, st == 0, ci, ct,
                               info.cycle_complexity)

    def cycle(self, level, b):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.empty_like(b)
        check(lib().ligmg_cycle(self._h, level, _p(b), _p(x)), "ligmg_cycle")
        return x

    def spmv(self, level, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        check(lib().ligmg_spmv(self._h, level, _p(x), _p(y)), "ligmg_spmv")
        return y

    # ---- hierarchy export / import --------------------------------------------
    def level_prolongation(self, level):
        inf = self.level_info(level)
        nnz = C.c_int64()
        check(lib().ligmg_level_prolongation(self._h, level, C.byref(nnz), None, None, None,
                                             None))
        rp = np.empty(inf["n"] + 1, np.int64)
        ci = np.empty(nnz.value, np.int32)
        v = np.empty(nnz.value, np.float64)
        q = np.empty(inf["n"], np.float64)
        check(lib().ligmg_level_prolongation(self._h, level, C.byref(nnz), _p(rp), _p(ci),
                                             _p(v), _p(q)))
        return rp, ci, v, q

    def export_levels(self):
        from .petsc_io import Level
        out = []
        for l in range(self.num_levels):
            inf = self.level_info(l)
            rp, ci, v = self.level_matrix(l)
            lv = Level(inf["type"], inf["n"], rp, ci, v, inf["nc"])
            if inf["type"] == "agg":
                lv.ids = self.level_ids(l)
            elif inf["type"] == "elim":
                lv.prow, lv.pcol, lv.pval, lv.q = self.level_prolongation(l)
            out.append(lv)
        return out

    def dump_hierarchy(self, directory):
        """dump_hierarchy (ligmg.hpp:47-52): PETSc binary files per level."""
        from .petsc_io import dump
        dump(self.export_levels(), directory)

    @classmethod
    def import_hierarchy(cls, levels, options: _abi.Options = None, **kw):
        """Handle over an existing hierarchy (list of petsc_io.Level, e.g. from
        petsc_io.load(dir) or an exported hierarchy), without running setup."""
        self = cls.__new__(cls)
        self.options = options if options is not None else _abi.default_options(**kw)
        types = {"elim": 0, "agg": 1, "coarse": 2}
        descs = (_abi.LevelDesc * len(levels))()
        keep = []
        for d, lv in zip(descs, levels):
            arrs = [np.ascontiguousarray(lv.rowptr, np.int64), np.ascontiguousarray(lv.col, np.int32),
                    np.ascontiguousarray(lv.val, np.float64)]
            keep.append(arrs)
            d.type = types[lv.type]
            d.n = lv.n
            d.nnz = int(arrs[0][-1])
            d.rowptr, d.col, d.val = (a.ctypes.data for a in arrs)
            d.nc = lv.nc
            if lv.type == "agg":
                ids = np.ascontiguousarray(lv.ids, np.int32)
                keep.append(ids)
                d.ids = ids.ctypes.data
            elif lv.type == "elim":
                pa = [np.ascontiguousarray(lv.prow, np.int64), np.ascontiguousarray(lv.pcol, np.int32),
                      np.ascontiguousarray(lv.pval, np.float64), np.ascontiguousarray(lv.q, np.float64)]
                keep.append(pa)
                d.prow, d.pcol, d.pval, d.q = (a.ctypes.data for a in pa)
                d.pnnz = int(pa[0][-1])
        h = C.c_void_p()
        check(lib().ligmg_import_hierarchy(len(levels), descs, C.byref(self.options),
                                           C.byref(h)), "ligmg_import_hierarchy")
        self._h = h
        L0 = levels[0]
        self.n = L0.n
        self._rp, self._ci, self._v = keep[0]
        return self

    # ---- differentiation -----------------------------------------------------
    def forward(self, b) -> ConvergenceInfo:
        """Solve L x = b and keep x for backward() (ligmg_forward)."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.empty_like(b)
        info, hist, ci, ct = self._info(1)
        st = check(lib().ligmg_forward(self._h, _p(b), _p(x), C.byref(info)), "ligmg_forward")
        return ConvergenceInfo(hist[: info.history_len].copy(), info.iters, info.solve_seconds,
                               info.work, x, info.true_rel_residual, st == 0, ci, ct,
                               info.cycle_complexity)

    def backward(self, g, with_info=False):
        """Adjoint of the kept forward solve (ligmg_backward): returns (dw, db)
        with dw per stored CSR entry of the input matrix (the edge-weight
        derivative on off-diagonal entries, 0 on the diagonal) and db = dloss/db.
        with_info=True also returns the adjoint solve's ConvergenceInfo (its
        `converged` is False when the adjoint solve stopped at the iteration
        limit, LIGMG_NOT_CONVERGED)."""
        g = np.ascontiguousarray(g, dtype=np.float64)
        dw = np.empty(len(self._ci))
        db = np.empty(self.n)
        info, hist, ci, ct = self._info(1)
        st = check(lib().ligmg_backward(self._h, _p(g), _p(dw), _p(db), C.byref(info)),
                   "ligmg_backward")
        if not with_info:
            return dw, db
        return dw, db, ConvergenceInfo(hist[: info.history_len].copy(), info.iters,
                                       info.solve_seconds, info.work, None,
                                       info.true_rel_residual, st == 0, ci, ct,
                                       info.cycle_complexity)

    # ---- measurement ---------------------------------------------------------
    def profile(self, enable=True):
        check(lib().ligmg_profile_enable(self._h, 1 if enable else 0))

    def kernel_stats(self):
        n = C.c_int32()
        check(lib().ligmg_kernel_stats(self._h, None, 0, C.byref(n)))
        arr = (_abi.KernelStat * max(n.value, 1))()
        check(lib().ligmg_kernel_stats(self._h, arr, n.value, C.byref(n)))
        out = []
        for r in arr[: n.value]:
            out.append({"level": r.level, "kind": _abi.KERNEL_KINDS.get(r.kind, str(r.kind)),
                        "k": r.k, "fp64": bool(r.fp64), "launches": r.launches,
                        "seconds": r.seconds, "bytes": r.bytes})
        return out

    def set_stream(self, stream_ptr):
        check(lib().ligmg_set_stream(self._h, C.c_void_p(stream_ptr)))

    @staticmethod
    def launch_count():
        x = C.c_int64()
        check(lib().ligmg_launch_count(C.byref(x)))
        return x.value

    @staticmethod
    def gather_peak(rows, width, count, blocks_per_sm=0):
        """Random `width`-byte rows (4, 8 or 128) per second that the running
        GPU gathers from a table of `rows` rows (ligmg_measure_gather_peak);
        blocks_per_sm 256-thread blocks per SM (0: every warp slot)."""
        x = C.c_double()
        check(lib().ligmg_measure_gather_peak(int(rows), int(width), int(count),
                                              int(blocks_per_sm), C.byref(x)),
              "ligmg_measure_gather_peak")
        return x.value

    def solve_batched_device(self, b_ptr, k, x_ptr):
        """Device pointers (n x k row-major FP64) on the handle's device."""
        info, hist, ci, ct = self._info(k)
        st = check(lib().ligmg_solve_batched_device(self._h, C.c_void_p(b_ptr), k,
                                                    C.c_void_p(x_ptr), C.byref(info)),
                   "ligmg_solve_batched_device")
        return ConvergenceInfo(hist[: info.history_len].copy(), info.iters, info.solve_seconds,
                               info.work, None, info.true_rel_residual, st == 0, ci, ct,
                               info.cycle_complexity)

    def dump_csv(self, f, info: ConvergenceInfo, graph="graph", setup_time=0.0, nnz=0,
                 header=True):
        """print_csv_header / print_csv (util.hpp:187-205): the options
        columns, then graph, solver, iters, rel_error, cycle_complexity, wda,
        setup_time, solve_time, nnz, nodes (csvout.py)."""
        from . import csvout
        csvout.write(f, self.options, info, graph=graph, setup_time=setup_time,
                     nnz=nnz or len(self._ci), header=header)


def prepare_graph(n, rowptr, col, val, lcc=True, laplacian=False, device=0):
    """The reference CLI's input steps on the GPU (ligmg_prepare_graph):
    keep the largest connected component (lcc) and/or turn a weighted
    adjacency matrix into its Laplacian (laplacian).  Returns
    (graphs.Laplacian, orig) with orig[i] the input index of vertex i."""
    from .graphs import Laplacian
    rowptr = np.ascontiguousarray(rowptr, dtype=np.int64)
    col = np.ascontiguousarray(col, dtype=np.int32)
    val = np.ascontiguousarray(val, dtype=np.float64)
    flags = (1 if lcc else 0) | (2 if laplacian else 0)
    nk, nnz = C.c_int64(), C.c_int64()
    check(lib().ligmg_prepare_graph(n, _p(rowptr), _p(col), _p(val), flags, device,
                                    C.byref(nk), C.byref(nnz), None, None, None, None),
          "ligmg_prepare_graph")
    rp = np.empty(nk.value + 1, np.int64)
    ci = np.empty(nnz.value, np.int32)
    cv = np.empty(nnz.value, np.float64)
    orig = np.empty(nk.value, np.int64)
    check(lib().ligmg_prepare_graph(n, _p(rowptr), _p(col), _p(val), flags, device,
                                    C.byref(nk), C.byref(nnz), _p(rp), _p(ci), _p(cv),
                                    _p(orig)), "ligmg_prepare_graph")
    return Laplacian(int(nk.value), rp, ci, cv, "prepared"), orig


class BatchSolver:
    """A batch of independent graph Laplacians solved together
    (ligmg_batch_create / ligmg_batch_solve): one block-diagonal hierarchy,
    per-graph Krylov scalars and convergence, the whole solve replayed from
    one captured CUDA graph."""

    def __init__(self, graphs, options: _abi.Options = None, **kw):
        from .graphs import union
        kw.setdefault("outer_ksp_type", "fcg")
        self.graphs = list(graphs)
        self.offsets, self.union = union(self.graphs)
        U = self.union
        self.options = options if options is not None else _abi.default_options(**kw)
        h = C.c_void_p()
        self._keep = (self.offsets, U.rowptr, U.col, U.val)
        check(lib().ligmg_batch_create(len(self.graphs), _p(self.offsets), _p(U.rowptr),
                                       _p(U.col), _p(U.val), C.byref(self.options),
                                       C.byref(h)), "ligmg_batch_create")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().ligmg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_levels(self):
        x = C.c_int32()
        check(lib().ligmg_hierarchy_levels(self._h, C.byref(x)))
        return x.value

    def solve(self, bs):
        """bs: one right-hand side per graph (list) or the concatenated vector.
        Returns (list of solutions, ConvergenceInfo with per-graph arrays)."""
        G = len(self.graphs)
        b = np.ascontiguousarray(np.concatenate(bs) if isinstance(bs, (list, tuple)) else bs,
                                 dtype=np.float64)
        x = np.empty_like(b)
        iters = np.zeros(G, np.int32)
        tr = np.zeros(G)
        info = _abi.Info()
        hist = np.zeros(8)
        info.residual_history = hist.ctypes.data_as(C.POINTER(C.c_double))
        info.history_capacity = 8
        st = check(lib().ligmg_batch_solve(self._h, _p(b), _p(x), _p(iters), _p(tr),
                                           C.byref(info)), "ligmg_batch_solve")
        xs = [x[self.offsets[g]:self.offsets[g + 1]].copy() for g in range(G)]
        return xs, ConvergenceInfo(hist[: info.history_len].copy(), info.iters,
                                   info.solve_seconds, info.work, x, info.true_rel_residual,
                                   st == 0, iters, tr, info.cycle_complexity)
