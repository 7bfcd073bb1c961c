"""ctypes binding of libisoext_gb300.so (the C ABI in include/isoext_gb300.h).

The library is the product's only compute path: if it cannot be loaded the
import of the extraction functions fails loudly -- there is no CPU fallback.
"""

from __future__ import annotations

import ctypes as C
import threading

from . import _build

_lock = threading.Lock()
_lib: C.CDLL | None = None

ISO_OK = 0
ISO_ERR_ARG = 1
ISO_ERR_CUDA = 2
ISO_ERR_TIMEOUT = 3
ISO_ERR_LOOKUP = 4
ISO_ERR_WORKSPACE = 5
ISO_ERR_OVERFLOW = 6

_vp = C.c_void_p
_i = C.c_int
_ll = C.c_longlong
_f = C.c_float
_fa = C.POINTER(C.c_float)


def _declare(lib: C.CDLL) -> None:
    lib.iso_last_error.restype = C.c_char_p
    lib.iso_abi_version.restype = _i
    lib.iso_mc_set_config.argtypes = [_i]
    lib.iso_mc_get_config.argtypes = [C.POINTER(_i)]
    lib.iso_tune_set.argtypes = [C.c_char_p, _i]
    lib.iso_tune_get.argtypes = [C.c_char_p, C.POINTER(_i)]
    lib.iso_profile_enable.argtypes = [_i]
    lib.iso_profile_reset.restype = None
    lib.iso_profile_read.argtypes = [C.c_char_p, C.POINTER(_ll), C.POINTER(C.c_double)]
    lib.iso_profile_kernels.argtypes = [C.c_char_p, C.POINTER(_ll)]
    lib.iso_mc_dense_workspace_size.argtypes = [_i, _i, _i, _ll, _ll]
    lib.iso_mc_dense_workspace_size.restype = C.c_size_t
    lib.iso_mc_dense.argtypes = [_vp, _i, _i, _i, _fa, _fa, _f, _i, _vp, _ll, _vp, _ll, _vp,
                                 C.c_size_t, _vp, _vp, _vp]
    lib.iso_set_arith.argtypes = [_i]
    lib.iso_get_arith.restype = _i
    lib.iso_axis_coords.argtypes = [_vp, _i, _f, _f, _vp]
    lib.iso_weld_mesh_workspace_size.argtypes = [_ll, _ll]
    lib.iso_weld_mesh_workspace_size.restype = C.c_size_t
    lib.iso_weld_mesh.argtypes = [_vp, _ll, _vp, _ll, _vp, _vp, _vp, _vp, _vp, _vp, C.c_size_t, _vp]
    lib.iso_sort_vertices_workspace_size.argtypes = [_ll]
    lib.iso_sort_vertices_workspace_size.restype = C.c_size_t
    lib.iso_sort_vertices.argtypes = [_vp, _ll, _vp, _ll, _vp, C.c_size_t, _vp]
    _apply(lib, _EXTRA)


def _apply(lib: C.CDLL, entries: dict) -> None:
    for name, args in entries.items():
        fn = getattr(lib, name, None)
        if fn is not None:
            fn.argtypes = args[0]
            if args[1] is not None:
                fn.restype = args[1]


# Declarations of further entry points (added by the modules that use them).
_EXTRA: dict[str, tuple[list, object]] = {}


def register(entries: dict) -> None:
    """Declare entry points {name: (argtypes, restype)}; applies at once if loaded."""
    _EXTRA.update(entries)
    if _lib is not None:
        _apply(_lib, entries)


def lib() -> C.CDLL:
    """Load (building first if the sources are newer) the CUDA library."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            path = _build.build()
            handle = C.CDLL(str(path))
            _declare(handle)
            _lib = handle
    return _lib


def last_error() -> str:
    return lib().iso_last_error().decode(errors="replace")


def check(rc: int) -> None:
    if rc == ISO_OK:
        return
    msg = last_error()
    if rc == ISO_ERR_ARG:
        raise RuntimeError(msg)
    raise RuntimeError(f"isoext_gb300 error {rc}: {msg}")


ARITH = {"host": 0, "nvcc": 1}


def set_arithmetic(mode: str) -> None:
    """Which reading of isoext's FP32 expressions the kernels compute (process-wide).

    ``"nvcc"`` (default): the arithmetic of isoext's CUDA build, whose compiler
    fuses multiply-adds in its grid positions, lerps, normal stencil and norms;
    vertices, intersection points and normals equal that build's bit for bit.
    ``"host"``: every operation rounded on its own, as isoext's host build (and
    the reference's source read literally) computes.  No counterpart in isoext,
    which has one arithmetic per build."""
    if mode not in ARITH:
        raise ValueError(f"arithmetic must be one of {sorted(ARITH)}, not {mode!r}")
    check(lib().iso_set_arith(ARITH[mode]))


def get_arithmetic() -> str:
    m = lib().iso_get_arith()
    return next(k for k, v in ARITH.items() if v == m)


ORDERS = ("edge", "position")
_vertex_order = "edge"


def set_vertex_order(order: str) -> None:
    """How extraction results number their vertices (process-wide).

    ``"edge"`` (default): by grid edge (marching cubes) or by cell (dual
    contouring), as the kernels produce them; the mesh is isoext's after
    relabelling.  ``"position"``: sorted by position, lexicographically in
    (x, y, z), which is isoext's own numbering, so the returned tensors equal
    isoext's.  Faces are in isoext's order either way.  No counterpart in
    isoext (one order only)."""
    global _vertex_order
    if order not in ORDERS:
        raise ValueError(f"vertex order must be one of {ORDERS}, not {order!r}")
    _vertex_order = order


def get_vertex_order() -> str:
    return _vertex_order


def in_vertex_order(v, f):
    """(v, f) renumbered in the current vertex order (in place when sorting)."""
    if _vertex_order == "edge" or v is None or f is None or v.shape[0] < 2:
        return v, f
    import torch

    v = v.contiguous()
    f = f.contiguous()
    ws = torch.empty(lib().iso_sort_vertices_workspace_size(v.shape[0]), dtype=torch.uint8, device=v.device)
    with torch.cuda.device(v.device):
        check(lib().iso_sort_vertices(v.data_ptr(), v.shape[0], f.data_ptr(), f.shape[0], ws.data_ptr(), ws.numel(),
                                      C.c_void_p(torch.cuda.current_stream(v.device).cuda_stream)))
    return v, f


def fvec3(xs) -> C.Array:
    return (C.c_float * 3)(*[float(x) for x in xs])


def profile_read(kernel: str | None) -> tuple[int, float]:
    """(timed groups, total ms) recorded under a name since the last reset."""
    n, t = _ll(), C.c_double()
    check(lib().iso_profile_read(kernel.encode() if kernel else None, C.byref(n), C.byref(t)))
    return n.value, t.value


def profile_kernels(kernel: str | None) -> int:
    """Kernels launched under a name (None: all) since the last reset."""
    n = _ll()
    check(lib().iso_profile_kernels(kernel.encode() if kernel else None, C.byref(n)))
    return n.value


def weld_mesh(v, f, want_source: bool = False):
    """isoext's exact-position weld of a mesh on the device (iso_weld_mesh):
    vertices with bit-equal positions merge into the first, faces with two
    equal vertices and vertices no face uses are dropped, order kept.  Returns
    (vertices, faces) or (None, None) for an empty result, and with want_source
    each output vertex's input index as a third element."""
    import torch

    V, F = len(v), len(f)
    dev = v.device
    vout = torch.empty((V, 3), dtype=torch.float32, device=dev)
    fout = torch.empty((F, 3), dtype=torch.int32, device=dev)
    src = torch.empty(V, dtype=torch.int32, device=dev) if want_source else None
    small = torch.zeros(3, dtype=torch.int64, device=dev)
    ws = torch.empty(int(lib().iso_weld_mesh_workspace_size(V, F)), dtype=torch.uint8, device=dev)
    vv, ff = v.contiguous(), f.to(torch.int32).contiguous()
    check(lib().iso_weld_mesh(C.c_void_p(vv.data_ptr()), V, C.c_void_p(ff.data_ptr()), F,
                              C.c_void_p(vout.data_ptr()), C.c_void_p(fout.data_ptr()),
                              C.c_void_p(src.data_ptr()) if src is not None else None,
                              C.c_void_p(small.data_ptr()), C.c_void_p(small.data_ptr() + 16),
                              C.c_void_p(ws.data_ptr()), ws.numel(),
                              C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)))
    h = small.cpu()
    nv, nf, status = int(h[0]), int(h[1]), int(h[2] & 0xFFFFFFFF)
    if status:
        raise RuntimeError(f"isoext_gb300: device error {status} in the position weld")
    if nf == 0:
        return (None, None, None) if want_source else (None, None)
    out = (vout[:nv], fout[:nf])
    return out + (src[:nv],) if want_source else out
