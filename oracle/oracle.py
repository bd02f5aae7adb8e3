"""Python binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg to
check or time against; never by the product package.  Parity status of the
oracle itself: unpinned against the reference (see ligmg_oracle.cpp header).
"""
import ctypes as C
import os
import subprocess

import numpy as np

from ligmg_gb300._abi import Info, Options, default_options

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libligmg_oracle.so")

_lib = None


def build(force=False):
    if force or not os.path.exists(LIB):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        P = C.POINTER
        vp = C.c_void_p
        L.orc_create.argtypes = [C.c_int64, vp, vp, vp, P(Options), P(vp)]
        L.orc_destroy.argtypes = [vp]
        L.orc_num_levels.argtypes = [vp]
        L.orc_level_info.argtypes = [vp, C.c_int, P(C.c_int32), P(C.c_int64), P(C.c_int64),
                                     P(C.c_int64)]
        L.orc_level_matrix.argtypes = [vp, C.c_int, vp, vp, vp]
        L.orc_level_ids.argtypes = [vp, C.c_int, vp]
        L.orc_level_lmax.argtypes = [vp, C.c_int, P(C.c_double)]
        L.orc_level_prolongation.argtypes = [vp, C.c_int, P(C.c_int64), vp, vp, vp, vp]
        L.orc_level_aff_nnz.argtypes = [vp, C.c_int, P(C.c_int64)]
        L.orc_level_aff.argtypes = [vp, C.c_int, vp, vp, vp]
        L.orc_level_debug.argtypes = [vp, C.c_int, C.c_int, vp]
        L.orc_cycle_complexity.argtypes = [vp, C.c_int]
        L.orc_cycle_complexity.restype = C.c_double
        L.orc_setup_seconds.argtypes = [vp]
        L.orc_setup_seconds.restype = C.c_double
        L.orc_cycle.argtypes = [vp, C.c_int, vp, vp]
        L.orc_solve.argtypes = [vp, vp, vp, C.c_int, P(Info)]
        L.orc_spmv.argtypes = [C.c_int64, vp, vp, vp, vp, vp]
        L.orc_glibc_rand.argtypes = [C.c_uint32, C.c_int64, C.c_int64, vp]
        L.orc_galerkin.argtypes = [C.c_int64, vp, vp, vp, C.c_int64, vp, vp, vp,
                                   P(C.c_int64), vp, vp, vp]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_prepare_graph.argtypes = [C.c_int64, vp, vp, vp, C.c_int32, P(C.c_int64),
                                        P(C.c_int64), vp, vp, vp, vp]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def set_threads(n):
    return lib().orc_set_threads(n)


def glibc_rand(seed, count, skip=0):
    out = np.empty(count, dtype=np.int32)
    lib().orc_glibc_rand(seed, skip, count, _p(out))
    return out


def spmv(L, x):
    y = np.empty(L.n)
    x = np.ascontiguousarray(x, dtype=np.float64)
    lib().orc_spmv(L.n, _p(L.rowptr), _p(L.col), _p(L.val), _p(x), _p(y))
    return y


def galerkin(L, nc, prow, pcol, pval):
    prow = np.ascontiguousarray(prow, dtype=np.int64)
    pcol = np.ascontiguousarray(pcol, dtype=np.int32)
    pval = np.ascontiguousarray(pval, dtype=np.float64)
    nnz = C.c_int64()
    lib().orc_galerkin(L.n, _p(L.rowptr), _p(L.col), _p(L.val), nc, _p(prow), _p(pcol),
                       _p(pval), C.byref(nnz), None, None, None)
    rp = np.empty(nc + 1, np.int64)
    ci = np.empty(nnz.value, np.int32)
    cv = np.empty(nnz.value, np.float64)
    lib().orc_galerkin(L.n, _p(L.rowptr), _p(L.col), _p(L.val), nc, _p(prow), _p(pcol),
                       _p(pval), C.byref(nnz), _p(rp), _p(ci), _p(cv))
    return rp, ci, cv


def prepare_graph(n, rowptr, col, val, lcc=True, laplacian=False):
    """Largest connected component and/or adjacency -> Laplacian (the reference
    CLI's --cc and --adj): (rowptr, col, val, orig)."""
    rowptr = np.ascontiguousarray(rowptr, dtype=np.int64)
    col = np.ascontiguousarray(col, dtype=np.int32)
    val = np.ascontiguousarray(val, dtype=np.float64)
    flags = (1 if lcc else 0) | (2 if laplacian else 0)
    nk, nnz = C.c_int64(), C.c_int64()
    lib().orc_prepare_graph(n, _p(rowptr), _p(col), _p(val), flags, C.byref(nk), C.byref(nnz),
                            None, None, None, None)
    rp = np.empty(nk.value + 1, np.int64)
    ci = np.empty(nnz.value, np.int32)
    cv = np.empty(nnz.value, np.float64)
    orig = np.empty(nk.value, np.int64)
    st = lib().orc_prepare_graph(n, _p(rowptr), _p(col), _p(val), flags, C.byref(nk),
                                 C.byref(nnz), _p(rp), _p(ci), _p(cv), _p(orig))
    if st:
        raise OracleError(st)
    return rp, ci, cv, orig


class OracleError(RuntimeError):
    def __init__(self, status):
        super().__init__(f"oracle status {status}")
        self.status = status


class OracleSolver:
    """Hierarchy built by the oracle (make_hierarchy at one rank)."""

    def __init__(self, L, opts: Options = None, **kw):
        self.L = L
        self.opts = opts if opts is not None else default_options(**kw)
        h = C.c_void_p()
        st = lib().orc_create(L.n, _p(L.rowptr), _p(L.col), _p(L.val), C.byref(self.opts),
                              C.byref(h))
        if st != 0:
            raise OracleError(st)
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    @property
    def num_levels(self):
        return lib().orc_num_levels(self.h)

    def level_info(self, l):
        t, n, nnz, nc = C.c_int32(), C.c_int64(), C.c_int64(), C.c_int64()
        st = lib().orc_level_info(self.h, l, C.byref(t), C.byref(n), C.byref(nnz), C.byref(nc))
        if st:
            raise OracleError(st)
        return {"type": ("elim", "agg", "coarse")[t.value], "n": n.value, "nnz": nnz.value,
                "nc": nc.value}

    def level_matrix(self, l):
        inf = self.level_info(l)
        rp = np.empty(inf["n"] + 1, np.int64)
        ci = np.empty(inf["nnz"], np.int32)
        cv = np.empty(inf["nnz"], np.float64)
        lib().orc_level_matrix(self.h, l, _p(rp), _p(ci), _p(cv))
        return rp, ci, cv

    def level_ids(self, l):
        inf = self.level_info(l)
        ids = np.empty(inf["n"], np.int32)
        st = lib().orc_level_ids(self.h, l, _p(ids))
        if st:
            raise OracleError(st)
        return ids

    def level_lmax(self, l):
        x = C.c_double()
        lib().orc_level_lmax(self.h, l, C.byref(x))
        return x.value

    def level_prolongation(self, l):
        inf = self.level_info(l)
        nnz = C.c_int64()
        lib().orc_level_prolongation(self.h, l, C.byref(nnz), None, None, None, None)
        rp = np.empty(inf["n"] + 1, np.int64)
        ci = np.empty(nnz.value, np.int32)
        cv = np.empty(nnz.value, np.float64)
        q = np.empty(inf["n"], np.float64)
        lib().orc_level_prolongation(self.h, l, C.byref(nnz), _p(rp), _p(ci), _p(cv), _p(q))
        return rp, ci, cv, q

    def export_levels(self):
        """Level descriptions (ligmg_gb300.petsc_io.Level) of this hierarchy."""
        from ligmg_gb300.petsc_io import Level
        out = []
        for l in range(self.num_levels):
            inf = self.level_info(l)
            rp, ci, cv = self.level_matrix(l)
            lv = Level(inf["type"], inf["n"], rp, ci, cv, inf["nc"])
            if inf["type"] == "agg":
                lv.ids = self.level_ids(l)
            elif inf["type"] == "elim":
                lv.prow, lv.pcol, lv.pval, lv.q = self.level_prolongation(l)
            out.append(lv)
        return out

    def level_aff(self, l):
        inf = self.level_info(l)
        nnz = C.c_int64()
        lib().orc_level_aff_nnz(self.h, l, C.byref(nnz))
        rp = np.empty(inf["n"] + 1, np.int64)
        ci = np.empty(nnz.value, np.int32)
        cv = np.empty(nnz.value, np.float64)
        lib().orc_level_aff(self.h, l, _p(rp), _p(ci), _p(cv))
        return rp, ci, cv

    def level_debug(self, l, what, size):
        out = np.empty(size, np.float64)
        st = lib().orc_level_debug(self.h, l, what, _p(out))
        if st:
            raise OracleError(st)
        return out

    def cycle_complexity(self, start=0):
        return lib().orc_cycle_complexity(self.h, start)

    @property
    def setup_seconds(self):
        return lib().orc_setup_seconds(self.h)

    def cycle(self, level, b):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.empty_like(b)
        st = lib().orc_cycle(self.h, level, _p(b), _p(x))
        if st:
            raise OracleError(st)
        return x

    def solve(self, b, from_level=0, history=600):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.empty_like(b)
        hist = np.zeros(history)
        info = Info()
        info.residual_history = hist.ctypes.data_as(C.POINTER(C.c_double))
        info.history_capacity = history
        st = lib().orc_solve(self.h, _p(b), _p(x), from_level, C.byref(info))
        if st not in (0, 1):
            raise OracleError(st)
        res = {k: getattr(info, k) for k in ("iters", "converged", "rel_residual",
                                             "true_rel_residual", "cycle_complexity", "work",
                                             "solve_seconds", "setup_seconds")}
        res["status"] = st
        res["residuals"] = hist[: info.history_len].copy()
        return x, res
