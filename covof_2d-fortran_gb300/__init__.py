"""GB300-native STANDARD_PROJECTION + geometric VOF hot path of COVOF 2D.

The compute path is libcovof_gpu.so (hand-written sm_103a CUDA behind the C ABI
of include/covof_gpu.h); this package is its Python host mirror: ctypes
bindings (capi), reference-named subroutines over a device handle (solver),
seeded synthetic workloads (cases) and the build recipe (build).

The directory name is not a Python identifier; load the package with
``load_package()`` from __graft_entry__ or by path as ``covof_gb300``.
"""
from . import capi, cases  # noqa: F401
from .capi import CovofError, Params, default_params, load_library  # noqa: F401
from .solver import Batch, Fields, Solver, new_field  # noqa: F401

__all__ = ["capi", "cases", "CovofError", "Params", "Batch", "Fields", "Solver", "default_params",
           "load_library", "new_field"]
