"""ctypes binding of libligmg_gb300.so (the C ABI in include/ligmg_gpu.h).

There is no fallback: if the shared library is missing or fails to load,
every entry point raises.  Build it with ligmg_gb300.build.build().
"""
import ctypes as C
import os
import re

from . import build as _build
from ._abi import Info, KernelStat, LevelDesc, Options

HEADER = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "include", "ligmg_gpu.h")

_lib = None


class LigmgError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        msg = _status_string(status)
        super().__init__(f"{what}: {msg} (status {status})" if what else f"{msg} (status {status})")


def _status_string(s):
    try:
        return lib().ligmg_status_string(s).decode()
    except Exception:  # pragma: no cover - only when the library is absent
        from ._abi import STATUS_NAMES
        return STATUS_NAMES.get(s, "unknown")


def header_functions():
    """Names of every function declared in include/ligmg_gpu.h."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(ligmg_\w+)\s*\(", text, flags=re.M)))


def lib(path=None):
    global _lib
    if _lib is not None:
        return _lib
    path = path or _build.LIB
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is not built; call ligmg_gb300.build.build() first")
    L = C.CDLL(path)
    P = C.POINTER
    vp = C.c_void_p
    L.ligmg_default_options.argtypes = [P(Options)]
    L.ligmg_default_options.restype = None
    L.ligmg_status_string.argtypes = [C.c_int]
    L.ligmg_status_string.restype = C.c_char_p
    L.ligmg_create.argtypes = [C.c_int64, vp, vp, vp, P(Options), P(vp)]
    L.ligmg_destroy.argtypes = [vp]
    L.ligmg_solve.argtypes = [vp, vp, vp, P(Info)]
    L.ligmg_solve_from.argtypes = [vp, vp, vp, C.c_int32, P(Info)]
    L.ligmg_solve_batched.argtypes = [vp, vp, C.c_int32, vp, P(Info)]
    L.ligmg_solve_batched_device.argtypes = [vp, vp, C.c_int32, vp, P(Info)]
    L.ligmg_hierarchy_levels.argtypes = [vp, P(C.c_int32)]
    L.ligmg_level_info.argtypes = [vp, C.c_int32, P(C.c_int32), P(C.c_int64), P(C.c_int64),
                                   P(C.c_int64)]
    L.ligmg_level_matrix.argtypes = [vp, C.c_int32, vp, vp, vp]
    L.ligmg_level_ids.argtypes = [vp, C.c_int32, vp]
    L.ligmg_level_lmax.argtypes = [vp, C.c_int32, P(C.c_double)]
    L.ligmg_cycle.argtypes = [vp, C.c_int32, vp, vp]
    L.ligmg_spmv.argtypes = [vp, C.c_int32, vp, vp]
    L.ligmg_profile_enable.argtypes = [vp, C.c_int32]
    L.ligmg_kernel_stats.argtypes = [vp, P(KernelStat), C.c_int32, P(C.c_int32)]
    L.ligmg_set_stream.argtypes = [vp, vp]
    L.ligmg_get_stream.argtypes = [vp, P(vp)]
    L.ligmg_launch_count.argtypes = [P(C.c_int64)]
    L.ligmg_last_error.restype = C.c_char_p
    L.ligmg_last_error.argtypes = []
    L.ligmg_measure_gather_peak.argtypes = [C.c_int64, C.c_int32, C.c_int64, C.c_int32,
                                            P(C.c_double)]
    L.ligmg_spmv_device_noalloc.argtypes = [vp, C.c_int32, vp, vp]
    L.ligmg_forward.argtypes = [vp, vp, vp, P(Info)]
    L.ligmg_solve_pcg_jacobi.argtypes = [vp, vp, vp, P(Info)]
    L.ligmg_prepare_graph.argtypes = [C.c_int64, vp, vp, vp, C.c_int32, C.c_int32,
                                      P(C.c_int64), P(C.c_int64), vp, vp, vp, vp]
    L.ligmg_level_prolongation.argtypes = [vp, C.c_int32, P(C.c_int64), vp, vp, vp, vp]
    L.ligmg_import_hierarchy.argtypes = [C.c_int32, P(LevelDesc), P(Options), P(vp)]
    L.ligmg_batch_create.argtypes = [C.c_int32, vp, vp, vp, vp, P(Options), P(vp)]
    L.ligmg_batch_solve.argtypes = [vp, vp, vp, vp, vp, P(Info)]
    L.ligmg_backward.argtypes = [vp, vp, vp, vp, P(Info)]
    L.ligmg_setup_times.argtypes = [vp, P(C.c_double)]
    for name in header_functions():
        if name not in ("ligmg_default_options", "ligmg_status_string", "ligmg_last_error"):
            getattr(L, name).restype = C.c_int
    _lib = L
    return L


def check(status, what=""):
    if status not in (0, 1):
        msg = lib().ligmg_last_error()
        raise LigmgError(status, f"{what}: {msg.decode()}" if msg else what)
    return status
