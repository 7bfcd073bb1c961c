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
    "iso_dc_dense_ex": ([_vp, _i, _i, _i, _fa, _fa, _f, _f, _f, _vp, _ll, _vp, _ll, _vp, C.c_size_t, _vp, _vp, _vp, _vp,
                         _vp, _vp], _i),
    "iso_mc_dense_edges": ([_vp, _i, _i, _i, _fa, _fa, _f, _i, _vp, _ll, _vp, _ll, _vp, C.c_size_t, _vp, _vp, _vp,
                            _vp], _i),
    "iso_mc_backward": ([_vp, _i, _i, _i, _fa, _fa, _f, _vp, _ll, _vp, _vp, _vp], _i),
    "iso_dc_backward": ([_vp, _i, _i, _i, _fa, _fa, _f, _vp, _vp, _ll, _f, _f, _vp, _vp, _vp, _vp, _vp], _i),
    "iso_dc_backward_src": ([_vp, _i, _i, _i, _fa, _fa, _f, _vp, _vp, _ll, _f, _f, _vp, _ll, _vp, _vp, _vp, _vp],
                            _i),
})

# Output sizes seen per (shape, box, level, method), for sizing the next call.
_sizes: dict[tuple, tuple[int, int]] = {}


def _p(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream(dev):
    return C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)


def _vec3(v):
    return tuple(float(x) for x in v)


class _Launch:
    """The buffers of one queued extraction; `small` receives its sizes."""

    def __init__(self, kind, values, key, **buf):
        self.kind, self.values, self.key = kind, values, key
        self.__dict__.update(buf)


# ---------------------------------------------------------------------------
# marching cubes

def _mc_launch(values: torch.Tensor, amin, amax, level: float, method: int, caps=None, small=None) -> _Launch:
    """Queues iso_mc_dense_edges on the current stream (no synchronisation).
    small: a zeroed int64[8] device tensor for the sizes (one is made if None)."""
    lib = _ffi.lib()
    dev = values.device
    shape = tuple(values.shape)
    key = (shape, amin, amax, float(level), method)
    if caps is None:
        if key in _sizes:
            nv, nf = _sizes[key]
            caps = (nv + nv // 10 + 1024, nf + nf // 10 + 1024)
        else:
            caps = _first_guess(shape)
    cap_v, cap_f = caps
    L = _Launch("mc", values, key, amin=amin, amax=amax, level=level, method=method,
                vout=torch.empty((cap_v, 3), dtype=torch.float32, device=dev),
                fout=torch.empty((cap_f, 3), dtype=torch.int32, device=dev),
                edges=torch.empty(cap_v, dtype=torch.int64, device=dev),
                ws=torch.empty(workspace_bytes(shape, cap_v, cap_f), dtype=torch.uint8, device=dev),
                small=small if small is not None else torch.zeros(8, dtype=torch.int64, device=dev))
    _ffi.check(lib.iso_mc_dense_edges(_p(values), *shape, _ffi.fvec3(amin), _ffi.fvec3(amax), float(level),
                                      int(method), _p(L.vout), cap_v, _p(L.fout), cap_f, _p(L.ws), L.ws.numel(),
                                      _p(L.small), C.c_void_p(L.small.data_ptr() + 16), _p(L.edges), _stream(dev)))
    return L


def _mc_finish(L: _Launch, h):
    """(vertices, faces, edges) from the sizes h, or None and the capacities to
    retry with."""
    nv, nf, status = int(h[0]), int(h[1]), int(h[2] & 0xFFFFFFFF)
    if status == _ffi.ISO_ERR_OVERFLOW:
        _sizes[L.key] = (nv, nf)
        return None, (nv + 1024, nf + 1024)
    if status:
        raise RuntimeError(f"isoext_gb300: device error {status} in marching_cubes")
    old = _sizes.get(L.key, (0, 0))
    _sizes[L.key] = (max(old[0], nv), max(old[1], nf))
    v, f, e = L.vout[:nv], L.fout[:nf], L.edges[:nv]
    if nv and nf and coarse_float_grid(L.values.shape, L.amin, L.amax):
        v, f, e = _weld_positions(v, f, e)
    return (v.contiguous(), f.contiguous(), e.contiguous()), None


def _weld_positions(v, f, e):
    """mc.weld_by_position, keeping for each vertex the edge of the first vertex
    merged into it (iso_weld_mesh reports each survivor's input vertex)."""
    v2, f2, src = _ffi.weld_mesh(v, f, want_source=True)
    if v2 is None:
        return v[:0], f[:0], e[:0]
    return v2, f2, e[src.long()]


def _smalls(values_list):
    """A zeroed int64 [8] size record per extraction: rows of one tensor when the
    grids share a device."""
    devs = {x.device for x in values_list}
    if len(devs) == 1:
        return list(torch.zeros((len(values_list), 8), dtype=torch.int64, device=devs.pop()).unbind(0))
    return [torch.zeros(8, dtype=torch.int64, device=x.device) for x in values_list]


def _collect(launches, relaunch):
    """One synchronisation for all queued launches; launches whose buffers were
    too small are queued again with exact capacities (a second one)."""
    if not launches:
        return []
    sizes = torch.stack([L.small for L in launches]).cpu()
    finish = {"mc": _mc_finish, "dc": _dc_finish}
    out, again = [None] * len(launches), []
    for i, (L, h) in enumerate(zip(launches, sizes)):
        res, caps = finish[L.kind](L, h)
        if res is None:
            again.append((i, relaunch(L, caps)))
        else:
            out[i] = res
    if again:
        sizes = torch.stack([L.small for _, L in again]).cpu()
        for (i, L), h in zip(again, sizes):
            res, _ = finish[L.kind](L, h)
            if res is None:
                raise RuntimeError(f"isoext_gb300: {L.kind} output did not fit after resizing")
            out[i] = res
    return out


class _MarchingCubes(torch.autograd.Function):
    @staticmethod
    def forward(ctx, values, res, box):
        v, f, e = res
        ctx.save_for_backward(values, e)
        ctx.box = box
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
        return grad, None, None


def _mc_relaunch(L, caps):
    return _mc_launch(L.values, L.amin, L.amax, L.level, L.method, caps)


def _mc_forward(values: torch.Tensor, amin, amax, level: float, method: int):
    """(vertices, faces, edges): edges[i] = 3 * (low endpoint's point id) + axis of vertex i."""
    return _collect([_mc_launch(values, amin, amax, level, method)], _mc_relaunch)[0]


def marching_cubes(values: torch.Tensor, aabb_min=(-1.0, -1.0, -1.0), aabb_max=(1.0, 1.0, 1.0),
                   level: float = 0.0, method: str = "nagae"):
    """Marching cubes of a dense grid of values [nx, ny, nz] over the box, with
    vertices differentiable with respect to values.  Returns (vertices float32
    [V, 3], faces int32 [F, 3]), the same as isoext_gb300.marching_cubes."""
    return marching_cubes_batch([values], aabb_min, aabb_max, level, method)[0]


def marching_cubes_batch(values_list, aabb_min=(-1.0, -1.0, -1.0), aabb_max=(1.0, 1.0, 1.0),
                         level: float = 0.0, method: str = "nagae"):
    """marching_cubes of several grids: every extraction is queued before one
    synchronisation reads all their sizes.  Returns a list of (vertices, faces)."""
    amin, amax, mid = _vec3(aabb_min), _vec3(aabb_max), method_id(method)
    for x in values_list:
        _check_cuda_f32(x, ndim=3)
    smalls = _smalls(values_list)  # the sizes of all the batch's extractions, zeroed at once
    res = _collect([_mc_launch(x.detach(), amin, amax, float(level), mid, small=smalls[i])
                    for i, x in enumerate(values_list)], _mc_relaunch)
    return [_MarchingCubes.apply(x, r, (amin, amax, float(level))) for x, r in zip(values_list, res)]


# ---------------------------------------------------------------------------
# dual contouring

def _dc_launch(values: torch.Tensor, amin, amax, level: float, reg: float, svd_tol: float, caps=None,
               small=None) -> _Launch:
    """Queues iso_dc_dense_ex on the current stream (no synchronisation).
    small: a zeroed int64[8] device tensor for the sizes (one is made if None)."""
    from . import dc

    lib = _ffi.lib()
    dev = values.device
    shape = tuple(values.shape)
    key = (shape, float(level), tuple(amin), tuple(amax))
    if caps is None:
        if key in dc._dc_sizes:
            a, q = dc._dc_sizes[key]
            caps = (a + a // 10 + 1024, 2 * q + (2 * q) // 10 + 1024)
        else:
            caps = _first_guess(shape)
    cap_v, cap_f = caps
    L = _Launch("dc", values, key, amin=amin, amax=amax, level=level, reg=reg, svd_tol=svd_tol,
                vout=torch.empty((cap_v, 3), dtype=torch.float32, device=dev),
                fout=torch.empty((cap_f, 3), dtype=torch.int32, device=dev),
                cells=torch.empty(cap_v, dtype=torch.int32, device=dev),
                offs=torch.empty(cap_v + 1, dtype=torch.int32, device=dev),
                src=torch.empty(cap_v, dtype=torch.int32, device=dev),
                ws=torch.empty(dc.dc_workspace_bytes(shape, cap_v, cap_f), dtype=torch.uint8, device=dev),
                small=small if small is not None else torch.zeros(8, dtype=torch.int64, device=dev))
    _ffi.check(lib.iso_dc_dense_ex(_p(values), *shape, _ffi.fvec3(amin), _ffi.fvec3(amax), float(level), float(reg),
                                   float(svd_tol), _p(L.vout), cap_v, _p(L.fout), cap_f, _p(L.ws), L.ws.numel(),
                                   _p(L.small), C.c_void_p(L.small.data_ptr() + 48), _p(L.cells), _p(L.offs),
                                   _p(L.src), _stream(dev)))
    return L


def _dc_finish(L: _Launch, h):
    """(vertices, faces, cells, offsets, source) from the sizes h, or None and
    the capacities to retry with."""
    from . import dc

    V, F, A, Q, status = int(h[0]), int(h[1]), int(h[2]), int(h[4]), int(h[6] & 0xFFFFFFFF)
    dc._dc_sizes[L.key] = (A, Q)
    if status == _ffi.ISO_ERR_OVERFLOW:
        return None, (A + 1024, 2 * Q + 1024)
    if status:
        raise RuntimeError(f"isoext_gb300: device error {status} in dual_contouring")
    if V == 0 or F == 0:
        dev = L.values.device
        return (torch.zeros((0, 3), dtype=torch.float32, device=dev), torch.zeros((0, 3), dtype=torch.int32, device=dev),
                None, None, None), None
    return (L.vout[:V], L.fout[:F], L.cells[:A], L.offs[:A + 1], L.src[:V]), None


def _dc_relaunch(L, caps):
    return _dc_launch(L.values, L.amin, L.amax, L.level, L.reg, L.svd_tol, caps)


def _dc_forward(values: torch.Tensor, amin, amax, level: float, reg: float, svd_tol: float):
    """(vertices, faces, cells, offsets, source): cells / offsets are the active
    cells and their crossings' CSR ranges; source[i] = active cell of vertex i."""
    return _collect([_dc_launch(values, amin, amax, level, reg, svd_tol)], _dc_relaunch)[0]


class _DualContouring(torch.autograd.Function):
    @staticmethod
    def forward(ctx, values, res, meta):
        v, f, cells, offs, src = res
        ctx.save_for_backward(values, cells, offs, src)
        ctx.meta = meta
        ctx.mark_non_differentiable(f)
        return v, f

    @staticmethod
    def backward(ctx, gv, gf):
        values, cells, offs, src = ctx.saved_tensors
        if gv is None or cells is None or src.numel() == 0:
            return torch.zeros_like(values), None, None
        amin, amax, level, reg, svd_tol = ctx.meta
        A = cells.numel()
        grad = torch.empty_like(values)  # zeroed by the call
        gdual = torch.empty((A, 3), dtype=torch.float32, device=values.device)
        gvc = gv.to(torch.float32).contiguous()
        # each dual vertex is the source of at most one vertex: the call scatters
        # grad_vertices to their source cells, then differentiates the solve
        _ffi.check(_ffi.lib().iso_dc_backward_src(_p(values), *values.shape, _ffi.fvec3(amin), _ffi.fvec3(amax),
                                                  level, _p(cells), _p(offs), A, reg, svd_tol, _p(src), src.numel(),
                                                  _p(gvc), _p(gdual), _p(grad), _stream(values.device)))
        return grad, None, None


def dual_contouring(values: torch.Tensor, aabb_min=(-1.0, -1.0, -1.0), aabb_max=(1.0, 1.0, 1.0),
                    level: float = 0.0, reg: float = 1e-2, svd_tol: float = 1e-6):
    """Dual contouring of a dense grid of values [nx, ny, nz] over the box, with
    normals from the grid (as isoext.dual_contouring without an intersection)
    and vertices differentiable with respect to values.  Returns (vertices
    float32 [V, 3], faces int32 [F, 3]), the same as
    isoext_gb300.dual_contouring."""
    return dual_contouring_batch([values], aabb_min, aabb_max, level, reg, svd_tol)[0]


def dual_contouring_batch(values_list, aabb_min=(-1.0, -1.0, -1.0), aabb_max=(1.0, 1.0, 1.0),
                          level: float = 0.0, reg: float = 1e-2, svd_tol: float = 1e-6):
    """dual_contouring of several grids with one synchronisation (see
    marching_cubes_batch).  Returns a list of (vertices, faces)."""
    amin, amax = _vec3(aabb_min), _vec3(aabb_max)
    for x in values_list:
        _check_cuda_f32(x, ndim=3)
    smalls = _smalls(values_list)  # the sizes of all the batch's extractions, zeroed at once
    res = _collect([_dc_launch(x.detach(), amin, amax, float(level), float(reg), float(svd_tol), small=smalls[i])
                    for i, x in enumerate(values_list)],
                   _dc_relaunch)
    meta = (amin, amax, float(level), float(reg), float(svd_tol))
    return [_DualContouring.apply(x, r, meta) for x, r in zip(values_list, res)]
