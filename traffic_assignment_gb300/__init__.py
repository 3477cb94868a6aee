"""GB300-native Frank-Wolfe user-equilibrium traffic assignment.

A drop-in for the hot path of stivalaa/traffic_assignment (trunk/tap): the
all-origins shortest paths, all-or-nothing loading, BPR cost update, 2^-k
line search and gap / objective / VHT reductions, as hand-written sm_103a
kernels behind the reference's C API (libtapgpu.so, include/tap_gpu.h).

Python entry points:
  Solver            handle API (single scenario, batched scenarios, paths)
  synth, tntp       synthetic workloads and TNTP file formats
  pape              Python 3 drop-in of the reference's ``pape`` extension
  scenarios         net-mod subsets (single / pairs / power set / list)
"""

from . import synth, tntp  # noqa: F401
from ._capi import TapGpuError, load as load_library  # noqa: F401
from .solver import Solver, SolveResult  # noqa: F401

__all__ = ["Solver", "SolveResult", "TapGpuError", "load_library", "synth", "tntp"]
