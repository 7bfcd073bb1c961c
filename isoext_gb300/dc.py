"""get_intersection / dual_contouring / Intersection with isoext's API
(src/isoext_ext.cu:305-378) on the CUDA path (csrc/dc_dense.cu).

The steps run asynchronously on the current stream; the host synchronises only
to size the next buffers (active cells and crossings, quads, welded vertices).
"""

from __future__ import annotations

import ctypes as C

import torch

from . import _ffi
from .grids import SparseGridBase, UniformGrid, _check_cuda_f32

_vp, _i, _ll, _f, _sz = C.c_void_p, C.c_int, C.c_longlong, C.c_float, C.c_size_t
_fa = C.POINTER(C.c_float)
_ffi.register({
    "iso_dc_workspace_size": ([_i, _i, _i], _sz),
    "iso_dc_classify": ([_vp, _i, _i, _i, _f, _vp, _sz, _vp, _vp], _i),
    "iso_dc_intersect": ([_vp, _i, _i, _i, _fa, _fa, _f, _vp, _ll, _ll, _vp, _vp, _vp, _vp, _vp], _i),
    "iso_dc_normals": ([_vp, _i, _i, _i, _fa, _fa, _vp, _vp, _vp, _ll, _vp, _vp], _i),
    "iso_dc_solve": ([_i, _i, _i, _fa, _fa, _vp, _vp, _vp, _vp, _ll, _f, _f, _vp, _vp], _i),
    "iso_dc_cells": ([_vp, _i, _i, _i, _f, _vp, _vp], _i),
    "iso_dc_quads_count": ([_i, _i, _i, _vp, _vp, _vp], _i),
    "iso_dc_quads_emit": ([_i, _i, _i, _vp, _vp, _vp, _vp], _i),
    "iso_dc_weld_workspace_size": ([_ll], _sz),
    "iso_dc_weld_count": ([_vp, _ll, _vp, _ll, _vp, _sz, _vp, _vp, _vp], _i),
    "iso_dc_weld_write": ([_vp, _ll, _vp, _ll, _vp, _vp, _vp, _vp], _i),
    "iso_dc_weld_write_src": ([_vp, _ll, _vp, _ll, _vp, _vp, _vp, _vp, _vp], _i),
    "iso_dc_intersect_solve": ([_vp, _i, _i, _i, _fa, _fa, _f, _vp, _ll, _ll, _vp, _vp, _f, _f, _vp, _vp], _i),
    "iso_dc_dense_workspace_size": ([_i, _i, _i, _ll, _ll], _sz),
    "iso_dc_dense": ([_vp, _i, _i, _i, _fa, _fa, _f, _f, _f, _vp, _ll, _vp, _ll, _vp, _sz, _vp, _vp, _vp], _i),
})

# Last seen (active cells, quads) per (shape, level, box): the next call sizes its
# buffers from them (10% + a margin), so steady-state calls run once.
_dc_sizes: dict[tuple, tuple[int, int]] = {}


def _p(t):
    return None if t is None else C.c_void_p(t.data_ptr())


class Intersection:
    """Edge/surface crossings of a grid: points, normals and, per active cell,
    the CSR range of its crossings (isoext's Intersection, include/its.cuh:6-26).

    Unlike isoext, the getters do not move the buffers out (isoext's
    get_points() leaves the object without points, src/isoext_ext.cu:50-51)."""

    def __init__(self, points, normals, cell_indices, cell_offsets, level, grid_key, sparse=None):
        self._points = points
        self._normals = normals
        self._cells = cell_indices
        self._offsets = cell_offsets
        self._level = float(level)
        self._grid_key = grid_key
        self._sparse = sparse

    def get_points(self) -> torch.Tensor:
        """Crossing points, float32 [K, 3]."""
        return self._points

    def get_normals(self) -> torch.Tensor:
        """Normals at the crossings, float32 [K, 3] (zeros when none are set)."""
        if self._normals is None:
            return torch.zeros_like(self._points)
        return self._normals

    def has_normals(self) -> bool:
        return self._normals is not None

    def set_normals(self, new_normals: torch.Tensor) -> None:
        _check_cuda_f32(new_normals, ndim=2, last=3, what="new_normals")
        if new_normals.shape != self._points.shape:
            raise RuntimeError("Cannot set values with different shapes")
        self._normals = new_normals.clone()


def _grid_key(grid):
    return (tuple(grid.shape), tuple(grid.aabb_min), tuple(grid.aabb_max), id(grid))


def _stream(dev):
    return C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)


def _classify(grid: UniformGrid, level: float):
    lib = _ffi.lib()
    dev = grid._values.device
    nx, ny, nz = grid.shape
    ws = torch.empty(int(lib.iso_dc_workspace_size(nx, ny, nz)), dtype=torch.uint8, device=dev)
    counts = torch.zeros(2, dtype=torch.int64, device=dev)
    _ffi.check(lib.iso_dc_classify(_p(grid._values), nx, ny, nz, float(level), _p(ws), ws.numel(),
                                   _p(counts), _stream(dev)))
    A, K = (int(x) for x in counts.cpu())
    return ws, A, K


def _intersect_uniform(grid: UniformGrid, level: float, compute_normals: bool):
    lib = _ffi.lib()
    dev = grid._values.device
    nx, ny, nz = grid.shape
    ws, A, K = _classify(grid, level)
    points = torch.empty((K, 3), dtype=torch.float32, device=dev)
    normals = torch.empty((K, 3), dtype=torch.float32, device=dev) if compute_normals else None
    cells = torch.empty(A, dtype=torch.int32, device=dev)
    offs = torch.empty(A + 1, dtype=torch.int32, device=dev)
    _ffi.check(lib.iso_dc_intersect(_p(grid._values), nx, ny, nz, _ffi.fvec3(grid.aabb_min),
                                    _ffi.fvec3(grid.aabb_max), float(level), _p(ws), A, K, _p(points),
                                    _p(normals), _p(cells), _p(offs), _stream(dev)))
    its = Intersection(points, normals, cells, offs, level, _grid_key(grid))
    return its, ws


def get_intersection(grid, level: float = 0.0, compute_normals: bool = False) -> Intersection:
    """Crossings of the grid's edges with the iso-surface (isoext.get_intersection)."""
    if isinstance(grid, UniformGrid):
        return _intersect_uniform(grid, level, compute_normals)[0]
    if isinstance(grid, SparseGridBase):
        return grid._get_intersection(level, compute_normals)
    raise TypeError("grid must be a UniformGrid or SparseGrid")


def _dc_uniform(grid: UniformGrid, level, its: Intersection | None, reg, svd_tol):
    lib = _ffi.lib()
    dev = grid._values.device
    nx, ny, nz = grid.shape
    amin, amax = _ffi.fvec3(grid.aabb_min), _ffi.fvec3(grid.aabb_max)
    st = _stream(dev)
    if its is None:
        return _dc_one_call(grid, level, reg, svd_tol)
    else:
        if its._sparse is not None or its._grid_key[:3] != _grid_key(grid)[:3]:
            raise RuntimeError("intersection was computed for a different grid")
        # the quads follow the intersection's crossings, i.e. its level
        ws, (_, _, Q) = _classify_quads(grid, its._level)
        _ffi.check(lib.iso_dc_cells(_p(grid._values), nx, ny, nz, its._level, _p(ws), st))
    A = int(its._cells.numel())
    normals = its._normals
    if normals is None:
        normals = torch.empty_like(its._points)
        _ffi.check(lib.iso_dc_normals(_p(grid._values), nx, ny, nz, amin, amax, _p(its._points),
                                      _p(its._cells), _p(its._offsets), A, _p(normals), st))
    if A == 0 or Q == 0:
        return None, None
    dual = torch.empty((A, 3), dtype=torch.float32, device=dev)
    _ffi.check(lib.iso_dc_solve(nx, ny, nz, amin, amax, _p(its._points), _p(normals), _p(its._cells),
                                _p(its._offsets), A, float(reg), float(svd_tol), _p(dual), st))
    tri = torch.empty(6 * Q, dtype=torch.int32, device=dev)
    _ffi.check(lib.iso_dc_quads_emit(nx, ny, nz, _p(ws), _p(dual), _p(tri), st))
    return weld_dual(lib, dev, dual, A, tri, st)


def dc_dense_into(values: torch.Tensor, aabb_min, aabb_max, level: float, reg: float, svd_tol: float,
                  vout: torch.Tensor, fout: torch.Tensor, ws: torch.Tensor, small: torch.Tensor, stream: int) -> int:
    """Launch iso_dc_dense into caller-provided buffers (no synchronisation).
    small: int64[8] device tensor; [0:5] receives (V, F, A, K, Q), [6] the status word."""
    nx, ny, nz = values.shape
    return _ffi.lib().iso_dc_dense(_p(values), nx, ny, nz, _ffi.fvec3(aabb_min), _ffi.fvec3(aabb_max),
                                   float(level), float(reg), float(svd_tol), _p(vout), vout.shape[0], _p(fout),
                                   fout.shape[0], _p(ws), ws.numel(), _p(small), C.c_void_p(small.data_ptr() + 48),
                                   C.c_void_p(stream))


def dc_workspace_bytes(shape, cap_v: int, cap_f: int) -> int:
    return int(_ffi.lib().iso_dc_dense_workspace_size(*shape, cap_v, cap_f))


def _dc_one_call(grid: UniformGrid, level, reg, svd_tol):
    """dual_contouring without a caller intersection: iso_dc_dense, one
    synchronisation to read the sizes (a retry with exact capacities if the
    buffers were too small)."""
    from .mc import _first_guess, _views

    dev = grid._values.device
    key = (tuple(grid.shape), float(level), tuple(grid.aabb_min), tuple(grid.aabb_max))
    if key in _dc_sizes:
        a, q = _dc_sizes[key]
        cap_v, cap_f = a + a // 10 + 1024, 2 * q + (2 * q) // 10 + 1024
    else:
        cap_v, cap_f = _first_guess(grid.shape)
    st = torch.cuda.current_stream(dev).cuda_stream
    for _ in range(2):
        vout = torch.empty((cap_v, 3), dtype=torch.float32, device=dev)
        fout = torch.empty((cap_f, 3), dtype=torch.int32, device=dev)
        ws = torch.empty(dc_workspace_bytes(grid.shape, cap_v, cap_f), dtype=torch.uint8, device=dev)
        small = torch.zeros(8, dtype=torch.int64, device=dev)
        _ffi.check(dc_dense_into(grid._values, grid.aabb_min, grid.aabb_max, level, reg, svd_tol, vout, fout, ws,
                                 small, st))
        h = small.cpu()
        V, F, A, Q, status = int(h[0]), int(h[1]), int(h[2]), int(h[4]), int(h[6] & 0xFFFFFFFF)
        _dc_sizes[key] = (A, Q)
        if status == _ffi.ISO_ERR_OVERFLOW:
            cap_v, cap_f = A + 1024, 2 * Q + 1024
            continue
        if status:
            raise RuntimeError(f"isoext_gb300: device error {status} in dual_contouring")
        return _views(vout, fout, V, F)
    raise RuntimeError("isoext_gb300: dual_contouring output did not fit after resizing")


def _classify_quads(grid: UniformGrid, level: float):
    """Workspace after classify + quad count, and (A, K, Q) in one synchronisation."""
    lib = _ffi.lib()
    dev = grid._values.device
    nx, ny, nz = grid.shape
    ws = torch.empty(int(lib.iso_dc_workspace_size(nx, ny, nz)), dtype=torch.uint8, device=dev)
    counts = torch.zeros(4, dtype=torch.int64, device=dev)
    st = _stream(dev)
    _ffi.check(lib.iso_dc_classify(_p(grid._values), nx, ny, nz, float(level), _p(ws), ws.numel(),
                                   _p(counts), st))
    _ffi.check(lib.iso_dc_quads_count(nx, ny, nz, _p(ws), C.c_void_p(counts.data_ptr() + 16), st))
    A, K, Q, _ = (int(x) for x in counts.cpu())
    return ws, (A, K, Q)


def weld_dual(lib, dev, dual, A, tri, st, src=None):
    """Merge the dual vertices faces use by exact position (isoext's sorted weld,
    src/utils.cu:32-59).  Both steps run before the one synchronisation that reads
    V: the vertex buffer is sized A (V <= A) and trimmed after.  src (optional,
    int32 [A]) receives each vertex's dual vertex."""
    wws = torch.empty(int(lib.iso_dc_weld_workspace_size(A)), dtype=torch.uint8, device=dev)
    small = torch.zeros(4, dtype=torch.int64, device=dev)
    vout = torch.empty((A, 3), dtype=torch.float32, device=dev)
    fout = torch.empty((tri.numel() // 3, 3), dtype=torch.int32, device=dev)
    _ffi.check(lib.iso_dc_weld_count(_p(dual), A, _p(tri), tri.numel(), _p(wws), wws.numel(), _p(small),
                                     C.c_void_p(small.data_ptr() + 16), st))
    _ffi.check(lib.iso_dc_weld_write_src(_p(dual), A, _p(tri), tri.numel(), _p(wws), _p(vout), _p(fout), _p(src),
                                         st))
    host = small.cpu()
    V, status = int(host[0]), int(host[2] & 0xffffffff)
    if status:
        raise RuntimeError(f"isoext_gb300: device error {status} in dual_contouring weld")
    v = vout[:V]
    if A > 2 * V + 65536:
        v = v.clone()
    return v, fout


def dual_contouring(grid, level: float = 0.0, intersection: Intersection | None = None,
                    reg: float = 1e-2, svd_tol: float = 1e-6):
    """Extract an iso-surface with dual contouring (isoext.dual_contouring).

    Returns (vertices float32 [V, 3], faces int32 [F, 3]) or (None, None).
    Faces follow isoext's order (quads by crossed edge, two triangles each);
    vertices are ordered by active cell, or sorted by position as isoext's after
    set_vertex_order("position")."""
    if isinstance(grid, UniformGrid):
        return _ffi.in_vertex_order(*_dc_uniform(grid, level, intersection, reg, svd_tol))
    if isinstance(grid, SparseGridBase):
        return _ffi.in_vertex_order(*grid._dual_contouring(level, intersection, reg, svd_tol))
    raise TypeError("grid must be a UniformGrid or SparseGrid")
