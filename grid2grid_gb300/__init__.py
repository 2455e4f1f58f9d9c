"""grid2grid_gb300: GB300-native transform path of grid2grid.

The product is the C ABI in include/grid2grid_gb300.h, implemented by the
in-tree CUDA library grid2grid_gb300/_lib/libgrid2grid_gb300.so (sm_103a),
plus the C++ facade under grid2grid_gb300/include/grid2grid/. This package
holds the ctypes binding (capi), host-side layout helpers (layouts), seeded
benchmark workloads (workloads) and the build step (build).
"""
from . import capi  # noqa: F401

__all__ = ["capi"]
