"""The oracle: CPU restatement of isoext's MC / DC path, and the reference itself.

TEST INFRASTRUCTURE ONLY.  Imported by ``tests/``, ``__graft_entry__.smoke()``
and ``bench.py`` (its ``cpu_baseline`` leg and ``--impl reference``); never by
the ``isoext_gb300`` package.

* :class:`Oracle` wraps ``iso_oracle.c`` (plain C, FP32 with every operation
  rounded separately, built with ``-ffp-contract=off``; FP64 least squares for
  DC).  It builds on any machine with gcc.
* :class:`Reference` wraps the reference's own sources compiled for the host
  CPU by ``build_ref.sh`` (``oracle/_ref/libisoext_ref.so``).  It exists only
  where the isoext checkout was present at build time.
"""

from __future__ import annotations

import ctypes as C
import os
import pathlib
import subprocess

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
BUILD = HERE / "_build"
ORACLE_SO = BUILD / "libiso_oracle.so"
REF_SO = HERE / "_ref" / "libisoext_ref.so"
# The isoext checkout to build the reference from: an argument of
# build_reference(), else the ISOEXT_REFERENCE environment variable.
REF_ENV = "ISOEXT_REFERENCE"

_f = C.POINTER(C.c_float)
_i32 = C.POINTER(C.c_int32)
_u32 = C.POINTER(C.c_uint32)
_u8 = C.POINTER(C.c_uint8)
_d = C.POINTER(C.c_double)
_i64 = C.c_int64


def build_oracle(force: bool = False) -> pathlib.Path:
    """Compile iso_oracle.c (seconds)."""
    src = HERE / "iso_oracle.c"
    hdr = HERE.parent / "isoext_gb300" / "csrc" / "luts.h"
    if (not force and ORACLE_SO.exists()
            and ORACLE_SO.stat().st_mtime > max(src.stat().st_mtime, hdr.stat().st_mtime)):
        return ORACLE_SO
    BUILD.mkdir(exist_ok=True)
    tmp = ORACLE_SO.with_suffix(f".{os.getpid()}.tmp")
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-std=c11",
                           "-o", str(tmp), str(src), "-lm"])
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_reference(src: str | os.PathLike | None = None, force: bool = False) -> pathlib.Path | None:
    """Compile the reference's own sources for the host.

    ``src`` is the isoext checkout (else ``$ISOEXT_REFERENCE``).  Returns None
    when neither names a checkout and no earlier build exists."""
    if REF_SO.exists() and not force:
        return REF_SO
    src = src or os.environ.get(REF_ENV)
    if not src or not (pathlib.Path(src) / "src").is_dir():
        return None
    subprocess.check_call(["bash", str(HERE / "build_ref.sh"), str(src)],
                          stdout=subprocess.DEVNULL)
    return REF_SO


def _fp(a: np.ndarray):
    return a.ctypes.data_as(_f)


def _take(ptr, n: int, dtype, shape, free) -> np.ndarray:
    """Copy a malloc'd C array into numpy and free it."""
    count = int(np.prod(shape)) if len(shape) else 1
    if n == 0 or count == 0:
        free(ptr)
        return np.zeros(shape, dtype=dtype)
    buf = np.ctypeslib.as_array(ptr, shape=(count,)).copy().astype(dtype, copy=False)
    free(ptr)
    return buf.reshape(shape)


class _ItsT(C.Structure):
    _fields_ = [("ncross", C.c_int64), ("nactive", C.c_int64), ("points", _f), ("normals", _f),
                ("edges", _u32), ("is_out", _u8), ("cells", _u32), ("offsets", _u32)]


ARITH = {"host": 0, "nvcc": 1}


class Oracle:
    """CPU restatement (iso_oracle.c).  All arrays are numpy, C-contiguous.

    ``arith`` is the reading of the reference's FP32 expressions: ``"nvcc"``
    (its CUDA build, the default) or ``"host"`` (its host build)."""

    def __init__(self, arith: str = "nvcc"):
        if arith not in ARITH:
            raise ValueError(f"arith must be one of {sorted(ARITH)}")
        self.arith = arith
        lib = C.CDLL(str(build_oracle()))
        lib.ora_set_arith.argtypes = [C.c_int]
        lib.ora_axis_coords.argtypes = [C.c_int, C.c_float, C.c_float, _f]
        lib.ora_mc_dense.argtypes = [_f, C.c_int, C.c_int, C.c_int, _f, _f, C.c_float, C.c_int,
                                     C.POINTER(_f), C.POINTER(_i64), C.POINTER(_i32),
                                     C.POINTER(_i64), C.POINTER(_u32)]
        lib.ora_mc_sparse.argtypes = [_i32, _f, _i64, C.c_int, C.c_int, C.c_int, _f, _f,
                                      C.c_float, C.c_int, C.POINTER(_f), C.POINTER(_i64),
                                      C.POINTER(_i32), C.POINTER(_i64), C.POINTER(_u32)]
        lib.ora_intersection_dense.argtypes = [_f, C.c_int, C.c_int, C.c_int, _f, _f, C.c_float,
                                               C.c_int, C.POINTER(_ItsT)]
        lib.ora_intersection_sparse.argtypes = [_i32, _f, _i64, C.c_int, C.c_int, C.c_int, _f, _f,
                                                C.c_float, C.c_int, C.POINTER(_ItsT)]
        lib.ora_dc.argtypes = [_f, _i32, _i64, C.c_int, C.c_int, C.c_int, C.c_int, _f, _f,
                               C.POINTER(_ItsT), C.c_float, C.c_float, C.POINTER(_f),
                               C.POINTER(_i64), C.POINTER(_i32), C.POINTER(_i64),
                               C.POINTER(_d)]
        lib.ora_qef.argtypes = [_f, _f, _u32, _i64, C.c_float, _f, _f]
        lib.ora_its_free.argtypes = [C.POINTER(_ItsT)]
        lib.ora_free.argtypes = [C.c_void_p]
        self._lib = lib

    @property
    def lib(self):
        """The C library, set to this oracle's arithmetic reading (the setting is
        the library's own, so it is made before every call)."""
        self._lib.ora_set_arith(ARITH[self.arith])
        return self._lib

    def axis_coords(self, n: int, lo: float = -1.0, hi: float = 1.0) -> np.ndarray:
        """The FP32 coordinates of the n points of one axis over [lo, hi]."""
        out = np.empty(max(n, 0), np.float32)
        if n > 0:
            self.lib.ora_axis_coords(n, lo, hi, _fp(out))
        return out

    def qef(self, points, normals, offsets, reg=1e-2):
        """(ATA [A, 9], ATb [A, 3]) of each cell's crossings (src/dc.cu:14-65)."""
        points = np.ascontiguousarray(points, np.float32)
        normals = np.ascontiguousarray(normals, np.float32)
        offsets = np.ascontiguousarray(offsets, np.uint32)
        A = len(offsets) - 1
        ata = np.zeros((max(A, 0), 9), np.float32)
        atb = np.zeros((max(A, 0), 3), np.float32)
        if A > 0:
            self.lib.ora_qef(_fp(points), _fp(normals), offsets.ctypes.data_as(_u32), A, reg, _fp(ata), _fp(atb))
        return ata, atb

    def grid_points(self, shape, lo=(-1, -1, -1), hi=(1, 1, 1)) -> np.ndarray:
        """Point positions [nx, ny, nz, 3] as the reference's get_points gives them."""
        ax = [self.axis_coords(shape[k], lo[k], hi[k]) for k in range(3)]
        X, Y, Z = np.meshgrid(*ax, indexing="ij")
        return np.stack([X, Y, Z], axis=-1)

    def _free(self, p):
        self.lib.ora_free(C.cast(p, C.c_void_p))

    def _mesh(self, vp, nv, fp, nf, ep):
        v = _take(vp, nv.value, np.float32, (nv.value, 3), self._free)
        f = _take(fp, nf.value, np.int32, (nf.value, 3), self._free)
        e = _take(ep, nv.value, np.uint32, (nv.value, 2), self._free)
        return v, f, e

    def mc_dense(self, values, aabb_min=(-1, -1, -1), aabb_max=(1, 1, 1), level=0.0,
                 method="nagae"):
        """Returns (vertices [V,3] f32, faces [F,3] i32, vertex source edges [V,2] u32)."""
        values = np.ascontiguousarray(values, dtype=np.float32)
        nx, ny, nz = values.shape
        amin = np.asarray(aabb_min, np.float32)
        amax = np.asarray(aabb_max, np.float32)
        vp, fp, ep = _f(), _i32(), _u32()
        nv, nf = _i64(), _i64()
        rc = self.lib.ora_mc_dense(_fp(values), nx, ny, nz, _fp(amin), _fp(amax), level,
                                   _method_id(method), C.byref(vp), C.byref(nv), C.byref(fp),
                                   C.byref(nf), C.byref(ep))
        if rc:
            raise MemoryError("oracle mc_dense failed")
        return self._mesh(vp, nv, fp, nf, ep)

    def mc_sparse(self, cell_ids, values, shape, aabb_min=(-1, -1, -1), aabb_max=(1, 1, 1),
                  level=0.0, method="nagae"):
        ids = np.ascontiguousarray(cell_ids, dtype=np.int32)
        vals = np.ascontiguousarray(values, dtype=np.float32).reshape(-1, 8)
        amin = np.asarray(aabb_min, np.float32)
        amax = np.asarray(aabb_max, np.float32)
        vp, fp, ep = _f(), _i32(), _u32()
        nv, nf = _i64(), _i64()
        rc = self.lib.ora_mc_sparse(ids.ctypes.data_as(_i32), _fp(vals), len(ids), *shape,
                                    _fp(amin), _fp(amax), level, _method_id(method),
                                    C.byref(vp), C.byref(nv), C.byref(fp), C.byref(nf),
                                    C.byref(ep))
        if rc:
            raise MemoryError("oracle mc_sparse failed")
        return self._mesh(vp, nv, fp, nf, ep)

    def _its_out(self, its: _ItsT) -> dict:
        k, a = its.ncross, its.nactive

        def grab(p, shape, dt):
            n = int(np.prod(shape))
            return (np.ctypeslib.as_array(p, shape=(n,)).copy().astype(dt).reshape(shape)
                    if n else np.zeros(shape, dt))

        out = {
            "points": grab(its.points, (k, 3), np.float32),
            "normals": grab(its.normals, (k, 3), np.float32),
            "edges": grab(its.edges, (k, 2), np.uint32),
            "is_out": grab(its.is_out, (k,), np.uint8).astype(bool),
            "cell_indices": grab(its.cells, (a,), np.uint32),
            "cell_offsets": grab(its.offsets, (a + 1,), np.uint32),
        }
        self.lib.ora_its_free(C.byref(its))
        return out

    def intersection_dense(self, values, aabb_min=(-1, -1, -1), aabb_max=(1, 1, 1), level=0.0,
                           normals=True) -> dict:
        values = np.ascontiguousarray(values, dtype=np.float32)
        amin = np.asarray(aabb_min, np.float32)
        amax = np.asarray(aabb_max, np.float32)
        its = _ItsT()
        if self.lib.ora_intersection_dense(_fp(values), *values.shape, _fp(amin), _fp(amax),
                                           level, int(normals), C.byref(its)):
            raise MemoryError("oracle intersection failed")
        return self._its_out(its)

    def intersection_sparse(self, cell_ids, values, shape, aabb_min=(-1, -1, -1),
                            aabb_max=(1, 1, 1), level=0.0, normals=True) -> dict:
        ids = np.ascontiguousarray(cell_ids, dtype=np.int32)
        vals = np.ascontiguousarray(values, dtype=np.float32).reshape(-1, 8)
        amin = np.asarray(aabb_min, np.float32)
        amax = np.asarray(aabb_max, np.float32)
        its = _ItsT()
        if self.lib.ora_intersection_sparse(ids.ctypes.data_as(_i32), _fp(vals), len(ids),
                                            *shape, _fp(amin), _fp(amax), level, int(normals),
                                            C.byref(its)):
            raise MemoryError("oracle intersection failed")
        return self._its_out(its)

    def dc(self, its: dict, shape, aabb_min=(-1, -1, -1), aabb_max=(1, 1, 1), reg=1e-2,
           svd_tol=1e-6, values=None, cell_ids=None):
        """Dual contouring from an intersection dict (points, normals, edges, is_out,
        cell_indices, cell_offsets).  Dense: values [nx,ny,nz]; sparse: cell_ids +
        values [N,8].  Returns (v, f, dual64 [A,3] FP64 QEF solutions)."""
        sparse = cell_ids is not None
        vals = np.ascontiguousarray(values, dtype=np.float32)
        ids = np.ascontiguousarray(cell_ids if sparse else np.zeros(1), dtype=np.int32)
        amin = np.asarray(aabb_min, np.float32)
        amax = np.asarray(aabb_max, np.float32)
        keep = {k: np.ascontiguousarray(its[k]) for k in its}
        pts = keep["points"].astype(np.float32)
        nrm = keep["normals"].astype(np.float32)
        edg = keep["edges"].astype(np.uint32)
        iso = keep["is_out"].astype(np.uint8)
        cel = keep["cell_indices"].astype(np.uint32)
        off = keep["cell_offsets"].astype(np.uint32)
        st = _ItsT(len(pts), len(cel), _fp(pts), _fp(nrm), edg.ctypes.data_as(_u32),
                   iso.ctypes.data_as(_u8), cel.ctypes.data_as(_u32), off.ctypes.data_as(_u32))
        vp, fp, dp = _f(), _i32(), _d()
        nv, nf = _i64(), _i64()
        rc = self.lib.ora_dc(_fp(vals), ids.ctypes.data_as(_i32), len(ids) if sparse else 0,
                             int(sparse), *shape, _fp(amin), _fp(amax), C.byref(st), reg,
                             svd_tol, C.byref(vp), C.byref(nv), C.byref(fp), C.byref(nf),
                             C.byref(dp))
        if rc:
            raise MemoryError("oracle dc failed")
        v = _take(vp, nv.value, np.float32, (nv.value, 3), self._free)
        f = _take(fp, nf.value, np.int32, (nf.value, 3), self._free)
        d = _take(dp, len(cel), np.float64, (len(cel), 3), self._free)
        return v, f, d

    def dc_dense(self, values, aabb_min=(-1, -1, -1), aabb_max=(1, 1, 1), level=0.0, reg=1e-2,
                 svd_tol=1e-6, normals=None):
        its = self.intersection_dense(values, aabb_min, aabb_max, level, normals is None)
        if normals is not None:
            its["normals"] = np.asarray(normals, np.float32).reshape(-1, 3)
        return self.dc(its, np.shape(values), aabb_min, aabb_max, reg, svd_tol, values=values)


def _method_id(method: str) -> int:
    if method == "nagae":
        return 0
    if method == "lorensen":
        return 1
    raise RuntimeError(f"Unknown method: {method}")


class Reference:
    """The reference's own code compiled for the host (build_ref.sh)."""

    def __init__(self):
        so = build_reference()
        if so is None or not so.exists():
            raise FileNotFoundError("reference host build unavailable (no isoext sources)")
        lib = C.CDLL(str(so))
        P = C.POINTER
        ll = C.c_longlong
        lib.ref_mc_dense.argtypes = [_f, C.c_int, C.c_int, C.c_int, _f, _f, C.c_float, C.c_char_p,
                                     P(_f), P(ll), P(_i32), P(ll)]
        lib.ref_mc_sparse.argtypes = [_i32, _f, ll, C.c_int, C.c_int, C.c_int, _f, _f, C.c_float,
                                      C.c_char_p, P(_f), P(ll), P(_i32), P(ll)]
        lib.ref_intersection_dense.argtypes = [_f, C.c_int, C.c_int, C.c_int, _f, _f, C.c_float,
                                               C.c_int, P(_f), P(_f), P(_u32), P(_u8), P(_u32),
                                               P(_u32), P(ll), P(ll)]
        lib.ref_dc_dense.argtypes = [_f, C.c_int, C.c_int, C.c_int, _f, _f, C.c_float, _f, ll,
                                     C.c_float, C.c_float, P(_f), P(ll), P(_i32), P(ll)]
        lib.ref_dc_sparse.argtypes = [_i32, _f, ll, C.c_int, C.c_int, C.c_int, _f, _f, C.c_float,
                                      C.c_float, C.c_float, P(_f), P(ll), P(_i32), P(ll)]
        lib.ref_free.argtypes = [C.c_void_p]
        lib.ref_last_error.restype = C.c_char_p
        self.lib = lib

    def _free(self, p):
        self.lib.ref_free(C.cast(p, C.c_void_p))

    def _check(self, rc):
        if rc:
            raise RuntimeError(self.lib.ref_last_error().decode())

    def _mesh(self, vp, nv, fp, nf):
        v = _take(vp, nv.value, np.float32, (nv.value, 3), self._free)
        f = _take(fp, nf.value, np.int32, (nf.value, 3), self._free)
        return v, f

    def mc_dense(self, values, aabb_min=(-1, -1, -1), aabb_max=(1, 1, 1), level=0.0,
                 method="nagae"):
        values = np.ascontiguousarray(values, dtype=np.float32)
        amin = np.asarray(aabb_min, np.float32)
        amax = np.asarray(aabb_max, np.float32)
        vp, fp, nv, nf = _f(), _i32(), C.c_longlong(), C.c_longlong()
        self._check(self.lib.ref_mc_dense(_fp(values), *values.shape, _fp(amin), _fp(amax), level,
                                          method.encode(), C.byref(vp), C.byref(nv), C.byref(fp),
                                          C.byref(nf)))
        return self._mesh(vp, nv, fp, nf)

    def mc_sparse(self, cell_ids, values, shape, aabb_min=(-1, -1, -1), aabb_max=(1, 1, 1),
                  level=0.0, method="nagae"):
        ids = np.ascontiguousarray(cell_ids, dtype=np.int32)
        vals = np.ascontiguousarray(values, dtype=np.float32).reshape(-1, 8)
        amin = np.asarray(aabb_min, np.float32)
        amax = np.asarray(aabb_max, np.float32)
        vp, fp, nv, nf = _f(), _i32(), C.c_longlong(), C.c_longlong()
        self._check(self.lib.ref_mc_sparse(ids.ctypes.data_as(_i32), _fp(vals), len(ids), *shape,
                                           _fp(amin), _fp(amax), level, method.encode(),
                                           C.byref(vp), C.byref(nv), C.byref(fp), C.byref(nf)))
        return self._mesh(vp, nv, fp, nf)

    def intersection_dense(self, values, aabb_min=(-1, -1, -1), aabb_max=(1, 1, 1), level=0.0,
                           normals=True) -> dict:
        values = np.ascontiguousarray(values, dtype=np.float32)
        amin = np.asarray(aabb_min, np.float32)
        amax = np.asarray(aabb_max, np.float32)
        pp, np_, ep, ip, cp, op = _f(), _f(), _u32(), _u8(), _u32(), _u32()
        k, a = C.c_longlong(), C.c_longlong()
        self._check(self.lib.ref_intersection_dense(
            _fp(values), *values.shape, _fp(amin), _fp(amax), level, int(normals), C.byref(pp),
            C.byref(np_), C.byref(ep), C.byref(ip), C.byref(cp), C.byref(op), C.byref(k),
            C.byref(a)))
        K, A = k.value, a.value
        return {
            "points": _take(pp, K, np.float32, (K, 3), self._free),
            "normals": _take(np_, K, np.float32, (K, 3), self._free),
            "edges": _take(ep, K, np.uint32, (K, 2), self._free),
            "is_out": _take(ip, K, np.uint8, (K,), self._free).astype(bool),
            "cell_indices": _take(cp, A, np.uint32, (A,), self._free),
            "cell_offsets": _take(op, A + 1, np.uint32, (A + 1,), self._free),
        }

    def dc_dense(self, values, aabb_min=(-1, -1, -1), aabb_max=(1, 1, 1), level=0.0, reg=1e-2,
                 svd_tol=1e-6, normals=None):
        values = np.ascontiguousarray(values, dtype=np.float32)
        amin = np.asarray(aabb_min, np.float32)
        amax = np.asarray(aabb_max, np.float32)
        nrm = None if normals is None else np.ascontiguousarray(normals, np.float32).reshape(-1, 3)
        vp, fp, nv, nf = _f(), _i32(), C.c_longlong(), C.c_longlong()
        self._check(self.lib.ref_dc_dense(
            _fp(values), *values.shape, _fp(amin), _fp(amax), level,
            None if nrm is None else _fp(nrm), 0 if nrm is None else len(nrm), reg, svd_tol,
            C.byref(vp), C.byref(nv), C.byref(fp), C.byref(nf)))
        return self._mesh(vp, nv, fp, nf)

    def dc_sparse(self, cell_ids, values, shape, aabb_min=(-1, -1, -1), aabb_max=(1, 1, 1),
                  level=0.0, reg=1e-2, svd_tol=1e-6):
        ids = np.ascontiguousarray(cell_ids, dtype=np.int32)
        vals = np.ascontiguousarray(values, dtype=np.float32).reshape(-1, 8)
        amin = np.asarray(aabb_min, np.float32)
        amax = np.asarray(aabb_max, np.float32)
        vp, fp, nv, nf = _f(), _i32(), C.c_longlong(), C.c_longlong()
        self._check(self.lib.ref_dc_sparse(ids.ctypes.data_as(_i32), _fp(vals), len(ids), *shape,
                                           _fp(amin), _fp(amax), level, reg, svd_tol, C.byref(vp),
                                           C.byref(nv), C.byref(fp), C.byref(nf)))
        return self._mesh(vp, nv, fp, nf)
