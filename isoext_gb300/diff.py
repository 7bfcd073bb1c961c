"""Differentiable extraction: marching cubes and dual contouring whose vertex
positions send gradients back to the grid values.

    values.requires_grad_(True)                      # float32 CUDA [nx, ny, nz]
    v, f = isoext_gb300.diff.marching_cubes(values, aabb_min, aabb_max)
    loss = ((v.norm(dim=-1) - 1) ** 2).mean()
    loss.backward()                                  # values.grad

The forward passes are the library's kernels, so vertices and faces are the
ones marching_cubes / dual_contouring return (bit for bit).  The backward
passes are hand-written kernels (csrc/backward.cu):

* marching cubes: through the edge-interpolation weights of each vertex
  (t = (level - va) / (vb - va), src/mc/nagae.cu:52-56);
* dual contouring: by implicit differentiation of the QEF solve
  (src/dc.cu:14-99), through the crossing points and the normals the grid's
  trilinear interpolant gives (src/its.cu:170-268); zero in clipped coordinates.

Topology (faces, which edges cross, which cells are active) is integer and has
no gradient.  isoext has no differentiable path; this module is an addition.
An empty surface gives empty [0, 3] tensors (not None) so that losses compose.
"""

from __future__ import annotations

import ctypes as C

import torch

from . import _ffi
from .grids import _check_cuda_f32
from .mc import _first_guess, coarse_float_grid, method_id, workspace_bytes

_vp, _i, _ll, _f = C.c_void_p, C.c_int, C.c_longlong, C.c_float
_fa = C.POINTER(C.c_float)
_ffi.register({
    "iso_mc_dense_edges": ([_vp, _i, _i, _i, _fa, _fa, _f, _i, _vp, _ll, _vp, _ll, _vp, C.c_size_t, _vp, _vp, _vp,
                            _vp], _i),
    "iso_mc_backward": ([_vp, _i, _i, _i, _fa, _fa, _f, _vp, _ll, _vp, _vp, _vp], _i),
    "iso_dc_backward": ([_vp, _i, _i, _i, _fa, _fa, _f, _vp, _vp, _ll, _f, _f, _vp, _vp, _vp, _vp, _vp], _i),
})

# Output sizes seen per (shape, box, level, method), for sizing the next call.
_sizes: dict[tuple, tuple[int, int]] = {}


def _p(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream(dev):
    return C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)


def _vec3(v):
    return tuple(float(x) for x in v)


# ---------------------------------------------------------------------------
# marching cubes

def _mc_forward(values: torch.Tensor, amin, amax, level: float, method: int):
    """(vertices, faces, edges): edges[i] = 3 * (low endpoint's point id) + axis of vertex i."""
    lib = _ffi.lib()
    dev = values.device
    shape = tuple(values.shape)
    key = (shape, amin, amax, float(level), method)
    if key in _sizes:
        nv, nf = _sizes[key]
        cap_v, cap_f = nv + nv // 10 + 1024, nf + nf // 10 + 1024
    else:
        cap_v, cap_f = _first_guess(shape)
    st = _stream(dev)
    for _ in range(2):
        vout = torch.empty((cap_v, 3), dtype=torch.float32, device=dev)
        fout = torch.empty((cap_f, 3), dtype=torch.int32, device=dev)
        edges = torch.empty(cap_v, dtype=torch.int64, device=dev)
        ws = torch.empty(workspace_bytes(shape, cap_v, cap_f), dtype=torch.uint8, device=dev)
        small = torch.zeros(4, dtype=torch.int64, device=dev)
        _ffi.check(lib.iso_mc_dense_edges(_p(values), *shape, _ffi.fvec3(amin), _ffi.fvec3(amax), float(level),
                                          int(method), _p(vout), cap_v, _p(fout), cap_f, _p(ws), ws.numel(),
                                          _p(small), C.c_void_p(small.data_ptr() + 16), _p(edges), st))
        h = small.cpu()
        nv, nf, status = int(h[0]), int(h[1]), int(h[2] & 0xFFFFFFFF)
        if status == _ffi.ISO_ERR_OVERFLOW:
            cap_v, cap_f = nv + 1024, nf + 1024
            _sizes[key] = (nv, nf)
            continue
        if status:
            raise RuntimeError(f"isoext_gb300: device error {status} in marching_cubes")
        old = _sizes.get(key, (0, 0))
        _sizes[key] = (max(old[0], nv), max(old[1], nf))
        v, f, e = vout[:nv], fout[:nf], edges[:nv]
        if nv and nf and coarse_float_grid(shape, amin, amax):
            v, f, e = _weld_positions(v, f, e)
        return v.contiguous(), f.contiguous(), e.contiguous()
    raise RuntimeError("isoext_gb300: marching_cubes output did not fit after resizing")


def _weld_positions(v, f, e):
    """mc.weld_by_position, keeping for each vertex the edge of the first vertex
    merged into it."""
    vn = torch.where(v == 0, torch.zeros_like(v), v)
    uniq, inv = torch.unique(vn.view(torch.int32), dim=0, return_inverse=True)
    first = torch.full((len(uniq),), len(v), dtype=torch.int64, device=v.device)
    first.scatter_reduce_(0, inv, torch.arange(len(v), device=v.device), reduce="amin")
    f2 = inv[f.long()]
    keep = (f2[:, 0] != f2[:, 1]) & (f2[:, 0] != f2[:, 2]) & (f2[:, 1] != f2[:, 2])
    f2 = f2[keep]
    used = torch.zeros(len(uniq), dtype=torch.bool, device=v.device)
    used[f2.reshape(-1)] = True
    remap = torch.cumsum(used.to(torch.int64), 0) - 1
    return uniq[used].view(torch.float32), remap[f2].to(torch.int32), e[first[used]]


class _MarchingCubes(torch.autograd.Function):
    @staticmethod
    def forward(ctx, values, amin, amax, level, method):
        v, f, e = _mc_forward(values.detach(), amin, amax, level, method)
        ctx.save_for_backward(values, e)
        ctx.box = (amin, amax, float(level))
        ctx.mark_non_differentiable(f)
        return v, f

    @staticmethod
    def backward(ctx, gv, gf):
        values, e = ctx.saved_tensors
        grad = torch.zeros_like(values)
        if gv is not None and e.numel():
            amin, amax, level = ctx.box
            _ffi.check(_ffi.lib().iso_mc_backward(_p(values), *values.shape, _ffi.fvec3(amin), _ffi.fvec3(amax),
                                                  level, _p(e), e.numel(), _p(gv.contiguous()), _p(grad),
                                                  _stream(values.device)))
        return grad, None, None, None, None


def marching_cubes(values: torch.Tensor, aabb_min=(-1.0, -1.0, -1.0), aabb_max=(1.0, 1.0, 1.0),
                   level: float = 0.0, method: str = "nagae"):
    """Marching cubes of a dense grid of values [nx, ny, nz] over the box, with
    vertices differentiable with respect to values.  Returns (vertices float32
    [V, 3], faces int32 [F, 3]), the same as isoext_gb300.marching_cubes."""
    _check_cuda_f32(values, ndim=3)
    return _MarchingCubes.apply(values, _vec3(aabb_min), _vec3(aabb_max), float(level), method_id(method))


# ---------------------------------------------------------------------------
# dual contouring

class _Values:
    """The attributes of a UniformGrid the dense DC steps read, over a values tensor."""

    def __init__(self, values, amin, amax):
        self._values = values
        self.shape = list(values.shape)
        self.aabb_min, self.aabb_max = list(amin), list(amax)


def _dc_forward(values: torch.Tensor, amin, amax, level: float, reg: float, svd_tol: float):
    """(vertices, faces, cells, offsets, source): cells / offsets are the active
    cells and their crossings' CSR ranges; source[i] = active cell of vertex i."""
    from . import dc

    lib = _ffi.lib()
    dev = values.device
    nx, ny, nz = values.shape
    st = _stream(dev)
    empty = (torch.zeros((0, 3), dtype=torch.float32, device=dev), torch.zeros((0, 3), dtype=torch.int32, device=dev))
    g = _Values(values, amin, amax)
    ws, (A, K, Q) = dc._classify_quads(g, level)
    if A == 0 or Q == 0:
        return (*empty, None, None, None)
    cells = torch.empty(A, dtype=torch.int32, device=dev)
    offs = torch.empty(A + 1, dtype=torch.int32, device=dev)
    dual = torch.empty((A, 3), dtype=torch.float32, device=dev)
    _ffi.check(lib.iso_dc_intersect_solve(_p(values), nx, ny, nz, _ffi.fvec3(amin), _ffi.fvec3(amax), float(level),
                                          _p(ws), A, K, _p(cells), _p(offs), float(reg), float(svd_tol), _p(dual),
                                          st))
    tri = torch.empty(6 * Q, dtype=torch.int32, device=dev)
    _ffi.check(lib.iso_dc_quads_emit(nx, ny, nz, _p(ws), _p(dual), _p(tri), st))
    src = torch.empty(A, dtype=torch.int32, device=dev)
    v, f = dc.weld_dual(lib, dev, dual, A, tri, st, src=src)
    return v, f, cells, offs, src[:len(v)]


class _DualContouring(torch.autograd.Function):
    @staticmethod
    def forward(ctx, values, amin, amax, level, reg, svd_tol):
        v, f, cells, offs, src = _dc_forward(values.detach(), amin, amax, level, reg, svd_tol)
        ctx.save_for_backward(values, cells, offs, src)
        ctx.meta = (amin, amax, float(level), float(reg), float(svd_tol))
        ctx.mark_non_differentiable(f)
        return v, f

    @staticmethod
    def backward(ctx, gv, gf):
        values, cells, offs, src = ctx.saved_tensors
        grad = torch.zeros_like(values)
        if gv is None or cells is None or src.numel() == 0:
            return grad, None, None, None, None, None
        amin, amax, level, reg, svd_tol = ctx.meta
        A = cells.numel()
        gdual = torch.zeros((A, 3), dtype=torch.float32, device=values.device)
        gdual[src.long()] = gv.to(torch.float32)  # each dual vertex is the source of at most one vertex
        _ffi.check(_ffi.lib().iso_dc_backward(_p(values), *values.shape, _ffi.fvec3(amin), _ffi.fvec3(amax), level,
                                              _p(cells), _p(offs), A, reg, svd_tol, None, _p(gdual), _p(grad), None,
                                              _stream(values.device)))
        return grad, None, None, None, None, None


def dual_contouring(values: torch.Tensor, aabb_min=(-1.0, -1.0, -1.0), aabb_max=(1.0, 1.0, 1.0),
                    level: float = 0.0, reg: float = 1e-2, svd_tol: float = 1e-6):
    """Dual contouring of a dense grid of values [nx, ny, nz] over the box, with
    normals from the grid (as isoext.dual_contouring without an intersection)
    and vertices differentiable with respect to values.  Returns (vertices
    float32 [V, 3], faces int32 [F, 3]), the same as
    isoext_gb300.dual_contouring."""
    _check_cuda_f32(values, ndim=3)
    return _DualContouring.apply(values, _vec3(aabb_min), _vec3(aabb_max), float(level), float(reg),
                                 float(svd_tol))
