"""marching_cubes: isoext's entry point (src/isoext_ext.cu:95-109) on the CUDA path."""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _ffi
from .grids import SparseGridBase, UniformGrid

METHODS = {"nagae": 0, "lorensen": 1}

# Last seen output sizes per (shape, method, level): the next call sizes its
# buffers from them (10% + a margin), so steady-state calls run once.
_size_cache: dict[tuple, tuple[int, int]] = {}


def method_id(method: str) -> int:
    try:
        return METHODS[method]
    except KeyError:
        raise RuntimeError(f"Unknown method: {method}") from None


def _first_guess(shape) -> tuple[int, int]:
    sx, sy, sz = shape
    area = 2 * (sx * sy + sy * sz + sx * sz)
    cells = max(sx - 1, 0) * max(sy - 1, 0) * max(sz - 1, 0)
    f = min(5 * cells, 2 * area + 4096)
    return f // 2 + 4096, f


def _views(v: torch.Tensor, f: torch.Tensor, nv: int, nf: int):
    if nv == 0 or nf == 0:
        return None, None
    vv, ff = v[:nv], f[:nf]
    # Return exact-size storage when the buffers are much larger than the mesh.
    if v.shape[0] > 2 * nv + 65536:
        vv = vv.clone()
    if f.shape[0] > 2 * nf + 65536:
        ff = ff.clone()
    return vv, ff


def mc_dense_into(values: torch.Tensor, aabb_min, aabb_max, level: float, method: int,
                  vout: torch.Tensor, fout: torch.Tensor, ws: torch.Tensor, small: torch.Tensor,
                  stream: int) -> int:
    """Launch iso_mc_dense into caller-provided buffers (no synchronisation).

    small: int64[4] device tensor; [0:2] receives (V, F), [2] the status word."""
    lib = _ffi.lib()
    nx, ny, nz = values.shape
    return lib.iso_mc_dense(values.data_ptr(), nx, ny, nz, _ffi.fvec3(aabb_min), _ffi.fvec3(aabb_max),
                            float(level), int(method), vout.data_ptr(), vout.shape[0], fout.data_ptr(),
                            fout.shape[0], ws.data_ptr(), ws.numel(), small.data_ptr(),
                            small.data_ptr() + 16, C.c_void_p(stream))


def workspace_bytes(shape, cap_v: int, cap_f: int) -> int:
    return int(_ffi.lib().iso_mc_dense_workspace_size(*shape, cap_v, cap_f))


def coarse_float_grid(shape, aabb_min, aabb_max) -> bool:
    """True when grid spacing is within 64 ulps of the coordinates' magnitude.

    Vertices are identified by grid key; isoext identifies them by exact
    position.  The two agree while neighbouring grid coordinates are many ulps
    apart.  On grids whose spacing approaches float resolution (e.g. a tiny box
    far from the origin) distinct keys can share a position, and the position
    weld of weld_by_position() is applied after extraction.
    """
    for n, a, b in zip(shape, aabb_min, aabb_max):
        if n < 2:
            continue
        a32, b32 = np.float32(a), np.float32(b)
        h = abs(float(b32) - float(a32)) / (n - 1)
        ulp = float(np.spacing(np.float32(max(abs(a32), abs(b32)))))
        if not np.isfinite(h) or h < 64.0 * ulp:
            return True
    return False


def weld_by_position(v: torch.Tensor, f: torch.Tensor):
    """Merge vertices with bit-identical positions (+0 and -0 equal), drop faces
    that became degenerate and vertices no face uses -- the result of isoext's
    position weld (src/utils.cu:32-59 with the degenerate test of
    src/mc/nagae.cu:71) applied to a key-welded mesh.  On the device
    (iso_weld_mesh); the survivors keep their order."""
    if v is None or len(f) == 0:
        return v, f
    return _ffi.weld_mesh(v, f)


def _mc_uniform(grid: UniformGrid, level: float, method: int):
    values = grid._values
    dev = values.device
    key = (tuple(grid.shape), method, float(level), tuple(grid.aabb_min), tuple(grid.aabb_max))
    if key in _size_cache:
        nv, nf = _size_cache[key]
        cap_v, cap_f = nv + nv // 10 + 1024, nf + nf // 10 + 1024
    else:
        cap_v, cap_f = _first_guess(grid.shape)
    with torch.cuda.device(dev):
        stream = torch.cuda.current_stream(dev).cuda_stream
        need = None  # sizes before the snap fix-up shrank them, after a retry
        for _attempt in range(2):
            vout = torch.empty((cap_v, 3), dtype=torch.float32, device=dev)
            fout = torch.empty((cap_f, 3), dtype=torch.int32, device=dev)
            ws = torch.empty(workspace_bytes(grid.shape, cap_v, cap_f), dtype=torch.uint8, device=dev)
            small = torch.zeros(4, dtype=torch.int64, device=dev)
            _ffi.check(mc_dense_into(values, grid.aabb_min, grid.aabb_max, level, method, vout, fout,
                                     ws, small, stream))
            host = small.cpu()
            nv, nf, status = int(host[0]), int(host[1]), int(host[2] & 0xffffffff)
            if status == _ffi.ISO_ERR_OVERFLOW:
                cap_v, cap_f = nv + 1024, nf + 1024
                need = (nv, nf)
                continue
            if status != 0:
                raise RuntimeError(f"isoext_gb300: device error {status} in marching_cubes")
            # counts are final sizes; output buffers must hold the sizes before
            # snapped vertices were merged, which a retry revealed
            _size_cache[key] = need if need is not None else (nv, nf)
            v, f = _views(vout, fout, nv, nf)
            if v is not None and coarse_float_grid(grid.shape, grid.aabb_min, grid.aabb_max):
                v, f = weld_by_position(v, f)
            return v, f
    raise RuntimeError("isoext_gb300: marching_cubes output did not fit after resizing")


def marching_cubes(grid, level: float = 0.0, method: str = "nagae"):
    """Extract an iso-surface with marching cubes.

    Returns (vertices float32 [V, 3], faces int32 [F, 3]) CUDA tensors, or
    (None, None) when the surface is empty -- as isoext.marching_cubes.
    Faces follow isoext's order (ascending cell id, table slot order); vertices
    are in ascending edge-key order, or sorted by position as isoext's after
    set_vertex_order("position").
    """
    mid = method_id(method)
    if isinstance(grid, UniformGrid):
        return _ffi.in_vertex_order(*_mc_uniform(grid, level, mid))
    if isinstance(grid, SparseGridBase):
        return _ffi.in_vertex_order(*grid._marching_cubes(level, mid))
    raise TypeError("grid must be a UniformGrid or SparseGrid")
