"""isoext_gb300: GB300-native iso-surface extraction with isoext's Python API.

    import isoext_gb300 as isoext
    grid = isoext.UniformGrid([128] * 3)
    grid.set_values(sdf(grid.get_points()))
    v, f = isoext.marching_cubes(grid)

    sparse = isoext.SparseGrid([1024] * 3)
    sparse.add_cells(ids)
    sparse.set_values(sdf(sparse.get_points()))   # [N, 8]
    v, f = isoext.dual_contouring(sparse)

``set_arithmetic("nvcc" | "host")`` picks which of isoext's two builds the
FP32 results equal bit for bit: its CUDA build (default) or its host build.
``set_vertex_order("position")`` numbers vertices as isoext does (sorted by
position), so the returned tensors equal isoext's; the default numbers them by
grid edge or cell (the same mesh after relabelling).

The extraction functions run hand-written sm_103a kernels through the C ABI of
``_lib/libisoext_gb300.so`` (include/isoext_gb300.h); there is no CPU fallback.
"""

from ._ffi import get_arithmetic, get_vertex_order, set_arithmetic, set_vertex_order
from .dc import Intersection, dual_contouring, get_intersection
from .grids import FLT_MAX, Grid, UniformGrid
from .mc import marching_cubes
from .sparse import SparseGrid
from .utils import gaussian_smooth, make_grid, write_obj

__all__ = [
    "FLT_MAX",
    "Grid",
    "Intersection",
    "SparseGrid",
    "UniformGrid",
    "dual_contouring",
    "gaussian_smooth",
    "get_arithmetic",
    "get_intersection",
    "get_vertex_order",
    "make_grid",
    "marching_cubes",
    "set_arithmetic",
    "set_vertex_order",
    "write_obj",
]
