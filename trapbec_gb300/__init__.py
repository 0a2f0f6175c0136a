"""GB300-native time-stepping engine for the TrapBEC Gross-Pitaevskii solver.

The compute path is libtrapbec.so (CUDA C++ for sm_103a behind a C ABI,
include/trapbec.h); this package is its Python host layer.
"""
from .abi import Params, DiagOut, InitArgs, default_params  # noqa: F401
from .solver import Solver, parse_cparam  # noqa: F401
