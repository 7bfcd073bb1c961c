"""isoext_gb300: GB300-native iso-surface extraction with isoext's Python API.

    import isoext_gb300 as isoext
    grid = isoext.UniformGrid([128] * 3)
    grid.set_values(sdf(grid.get_points()))
    v, f = isoext.marching_cubes(grid)

The extraction functions run hand-written sm_103a kernels through the C ABI of
``_lib/libisoext_gb300.so`` (include/isoext_gb300.h); there is no CPU fallback.
"""

from .grids import FLT_MAX, Grid, UniformGrid
from .mc import marching_cubes

__all__ = [
    "FLT_MAX",
    "Grid",
    "UniformGrid",
    "marching_cubes",
]
