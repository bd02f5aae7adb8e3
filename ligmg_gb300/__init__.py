"""GB300-native LigMG: graph-Laplacian multigrid (setup + solve) on one GPU.

The compute path is libligmg_gb300.so (hand-written sm_103a CUDA behind the C
ABI in include/ligmg_gpu.h); this package is its host-side mirror of the
reference interface ligmg::Solver(A) / solve(b).
"""
from ._abi import Info, Options, default_options  # noqa: F401
from .solver import BatchSolver, ConvergenceInfo, Solver, prepare_graph  # noqa: F401
