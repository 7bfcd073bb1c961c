"""iso_mc_dense_noalloc (fixed library scratch) against iso_mc_dense (caller
workspace), through the C ABI.

The two entry points run the same kernels, so the tolerance is exact equality
of counts, vertices and faces.  Two calls in a row on one stream, with no
synchronisation between them, must each equal the workspace entry point's
result.  Both calls share the scratch.
"""

import ctypes as C
import os
import re

import numpy as np
import pytest
import torch

from helpers import sphere, torus
from isoext_gb300 import _ffi

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LO, HI = (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0)


def _lib():
    lib = _ffi.lib()
    vp, i, ll, f = C.c_void_p, C.c_int, C.c_longlong, C.c_float
    fa = C.POINTER(C.c_float)
    lib.iso_mc_dense_noalloc.argtypes = [vp, i, i, i, fa, fa, f, i, vp, ll, vp, ll, vp, vp, vp]
    return lib


def _header_limit() -> int:
    src = open(os.path.join(ROOT, "include", "isoext_gb300.h")).read()
    m = re.search(r"#define ISO_MC_NOALLOC_SCRATCH_BYTES \((\d+)u << (\d+)\)", src)
    return int(m.group(1)) << int(m.group(2))


class Out:
    def __init__(self, cap_v, cap_f):
        self.v = torch.full((cap_v, 3), float("nan"), device="cuda")
        self.f = torch.full((cap_f, 3), -7, dtype=torch.int32, device="cuda")
        self.small = torch.zeros(4, dtype=torch.int64, device="cuda")

    def mesh(self):
        nv, nf, st = (int(x) for x in self.small[:3].cpu())
        assert st & 0xFFFFFFFF == 0, f"device status {st}"
        return nv, nf, self.v[:nv].cpu(), self.f[:nf].cpu()


def _with_workspace(vals, cap_v, cap_f, level=0.0, method=0):
    lib = _ffi.lib()
    nx, ny, nz = vals.shape
    o = Out(cap_v, cap_f)
    ws = torch.empty(lib.iso_mc_dense_workspace_size(nx, ny, nz, cap_v, cap_f), dtype=torch.uint8,
                     device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    rc = lib.iso_mc_dense(vals.data_ptr(), nx, ny, nz, _ffi.fvec3(LO), _ffi.fvec3(HI), level, method,
                          o.v.data_ptr(), cap_v, o.f.data_ptr(), cap_f, ws.data_ptr(), ws.numel(),
                          o.small.data_ptr(), o.small.data_ptr() + 16, C.c_void_p(s))
    assert rc == 0, _ffi.last_error()
    torch.cuda.synchronize()
    return o.mesh()


def _noalloc(lib, vals, o, level=0.0, method=0):
    nx, ny, nz = vals.shape
    s = torch.cuda.current_stream().cuda_stream
    return lib.iso_mc_dense_noalloc(vals.data_ptr(), nx, ny, nz, _ffi.fvec3(LO), _ffi.fvec3(HI), level,
                                    method, o.v.data_ptr(), o.v.shape[0], o.f.data_ptr(), o.f.shape[0],
                                    o.small.data_ptr(), o.small.data_ptr() + 16, C.c_void_p(s))


def _same(a, b, what):
    nv, nf, v, f = a
    nv2, nf2, v2, f2 = b
    assert (nv, nf) == (nv2, nf2), f"{what}: counts {(nv, nf)} vs {(nv2, nf2)}"
    assert nf > 0, what
    assert torch.equal(v, v2), f"{what}: vertices differ"
    assert torch.equal(f, f2), f"{what}: faces differ"


def test_noalloc_two_calls_in_a_row_match_workspace_entry():
    lib = _lib()
    a = torch.from_numpy(sphere((96, 96, 96), 0.7, center=(0.03, -0.02, 0.01))).cuda()
    b = torch.from_numpy(np.ascontiguousarray(torus((80, 72, 64), 0.5, 0.2))).cuda()
    ref_a = _with_workspace(a, 60000, 120000)
    ref_b = _with_workspace(b, 60000, 120000, method=1)
    oa, ob = Out(60000, 120000), Out(60000, 120000)
    # two calls back to back on one stream; they share the scratch
    assert _noalloc(lib, a, oa) == 0, _ffi.last_error()
    assert _noalloc(lib, b, ob, method=1) == 0, _ffi.last_error()
    torch.cuda.synchronize()
    _same(oa.mesh(), ref_a, "first call (sphere, nagae)")
    _same(ob.mesh(), ref_b, "second call (torus, lorensen)")
    # and again, after the scratch holds the second call's data
    oc = Out(60000, 120000)
    assert _noalloc(lib, a, oc) == 0, _ffi.last_error()
    torch.cuda.synchronize()
    _same(oc.mesh(), ref_a, "third call (sphere again)")


def test_noalloc_rejects_sizes_beyond_its_scratch():
    lib = _lib()
    limit = _header_limit()
    vals = torch.from_numpy(sphere((64, 64, 64), 0.5)).cuda()
    cap_v, cap_f = 1 << 21, 1 << 22  # real buffers, so nothing could run out of bounds
    need = lib.iso_mc_dense_workspace_size(64, 64, 64, cap_v, cap_f)
    assert need > limit
    o = Out(cap_v, cap_f)
    o.small.fill_(-1)  # a sentinel that any queued kernel or clear would overwrite
    torch.cuda.synchronize()
    rc = _noalloc(lib, vals, o)
    assert rc == _ffi.ISO_ERR_WORKSPACE
    msg = _ffi.last_error()
    assert "scratch" in msg and str(limit) in msg and str(need) in msg, msg
    torch.cuda.synchronize()
    assert (o.small == -1).all(), "a rejected call queued work"  # nothing was queued


def test_noalloc_accepts_sizes_just_under_its_scratch():
    """Capacities whose workspace is the largest that fits the header's limit run
    and equal the workspace entry point (the library's own limit is the header's)."""
    lib = _lib()
    limit = _header_limit()
    vals = torch.from_numpy(sphere((64, 64, 64), 0.5)).cuda()
    lo, hi = 1, 1 << 22  # largest vertex capacity (faces twice as many) that fits
    while lo < hi:
        mid = (lo + hi + 1) // 2
        if lib.iso_mc_dense_workspace_size(64, 64, 64, mid, 2 * mid) <= limit:
            lo = mid
        else:
            hi = mid - 1
    cap_v, cap_f = lo, 2 * lo
    assert lib.iso_mc_dense_workspace_size(64, 64, 64, cap_v, cap_f) <= limit
    assert lib.iso_mc_dense_workspace_size(64, 64, 64, cap_v + 1, cap_f + 2) > limit
    o = Out(cap_v, cap_f)
    assert _noalloc(lib, vals, o) == 0, _ffi.last_error()
    torch.cuda.synchronize()
    _same(o.mesh(), _with_workspace(vals, cap_v, cap_f), "capacities at the scratch limit")
