"""The default arithmetic equals isoext's CUDA build, bit for bit.

isoext's GPU build is compiled by nvcc with default flags, whose FMA
contraction fuses multiply-adds in the grid positions, the lerp of each
crossing and the normal stencil.  tests/nvcc_expr.cu restates those device
expressions in the reference's own source shape and is compiled here with
nvcc's defaults (no -fmad flag, no rounding intrinsics), as the reference's
CMake build does.  Its outputs on the same inputs must equal, to the last bit:

* the library's grid coordinates (UniformGrid.get_points);
* every intersection point of get_intersection, in order;
* every normal of get_intersection(compute_normals=True);
* every marching-cubes vertex (each is one of the crossing points);
* the QEF (ATA, ATb) of every active cell, against the oracle's CUDA-build
  reading, which spells out the same fused accumulation as the library's
  dual-contouring kernels.

Each case also checks that the host-build reading gives different bits on some
crossings, so the comparison can tell the two builds apart.
"""

import ctypes as C
import os
import subprocess

import numpy as np
import pytest
import torch

import isoext_gb300 as iso
from helpers import noise, sphere, torus

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "nvcc_expr.cu")
OUT = os.path.join(HERE, "_build", "libnvcc_expr.so")


def _nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


@pytest.fixture(scope="module")
def nx():
    if not os.path.exists(OUT) or os.path.getmtime(OUT) < os.path.getmtime(SRC):
        os.makedirs(os.path.dirname(OUT), exist_ok=True)
        tmp = f"{OUT}.{os.getpid()}.tmp"
        # nvcc's defaults for device arithmetic, as isoext's build: no -fmad,
        # -prec-div or -use_fast_math flag
        subprocess.check_call([_nvcc(), "-O3", "-std=c++17", "-shared", "-Xcompiler", "-fPIC",
                               "-gencode", "arch=compute_103a,code=sm_103a", "-o", tmp, SRC])
        os.replace(tmp, OUT)
    lib = C.CDLL(OUT)
    vp, i, f = C.c_void_p, C.c_int, C.c_float
    fa = C.POINTER(C.c_float)
    lib.nx_points.argtypes = [i, i, i, fa, fa, vp, vp]
    lib.nx_crossings.argtypes = [i, i, i, vp, vp, vp, vp, i, vp, f, vp, vp, vp]
    lib.nx_normals.argtypes = [i, i, i, vp, vp, vp, vp, i, vp, vp, vp]
    lib.nx_qef.argtypes = [vp, vp, vp, i, f, vp, vp, vp]
    iso.set_arithmetic("nvcc")
    yield lib
    iso.set_arithmetic("nvcc")


def _edges_table():
    import sys

    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "isoext_gb300", "csrc"))
    import gen_luts

    return torch.tensor([c for pair in gen_luts.EDGE_PAIRS for c in pair], dtype=torch.int32, device="cuda")


def _bits(t: torch.Tensor) -> np.ndarray:
    return t.contiguous().cpu().numpy().view(np.int32)


def _reference_outputs(lib, values, lo, hi, level, its):
    """Points, crossing points and normals as isoext's CUDA build computes them."""
    nx_, ny_, nz_ = values.shape
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    pts = torch.empty((nx_ * ny_ * nz_, 3), dtype=torch.float32, device="cuda")
    assert lib.nx_points(nx_, ny_, nz_, iso._ffi.fvec3(lo), iso._ffi.fvec3(hi), pts.data_ptr(), s) == 0
    cells = its._cells.to(torch.int32).contiguous()
    offs = its._offsets.to(torch.int32).contiguous()
    A, K = cells.numel(), int(offs[-1]) if offs.numel() else 0
    xp = torch.zeros((K, 3), dtype=torch.float32, device="cuda")
    nrm = torch.zeros((K, 3), dtype=torch.float32, device="cuda")
    bad = torch.zeros(1, dtype=torch.int32, device="cuda")
    table = _edges_table()
    assert lib.nx_crossings(nx_, ny_, nz_, values.data_ptr(), pts.data_ptr(), cells.data_ptr(), offs.data_ptr(),
                            A, table.data_ptr(), float(level), xp.data_ptr(), bad.data_ptr(), s) == 0
    assert lib.nx_normals(nx_, ny_, nz_, values.data_ptr(), pts.data_ptr(), cells.data_ptr(), offs.data_ptr(),
                          A, xp.data_ptr(), nrm.data_ptr(), s) == 0
    torch.cuda.synchronize()
    assert int(bad) == 0, "crossing counts of the restatement differ from the intersection's offsets"
    return pts.view(nx_, ny_, nz_, 3), xp, nrm


def _check(lib, vals_np, level=0.0, lo=(-1, -1, -1), hi=(1, 1, 1), what="", expect_host_diff=True):
    iso.set_arithmetic("nvcc")
    vals = torch.from_numpy(np.ascontiguousarray(vals_np, dtype=np.float32)).cuda()
    g = iso.UniformGrid(vals.shape, lo, hi)
    g.set_values(vals)
    its = iso.get_intersection(g, level=level, compute_normals=True)
    pts, xp, nrm = _reference_outputs(lib, vals, lo, hi, level, its)
    assert np.array_equal(_bits(g.get_points()), _bits(pts)), f"{what}: grid points differ"
    assert np.array_equal(_bits(its.get_points()), _bits(xp)), f"{what}: crossing points differ"
    assert np.array_equal(_bits(its.get_normals()), _bits(nrm)), f"{what}: normals differ"
    # QEF accumulation of the crossings (dual contouring's first step)
    A = int(its._cells.numel())
    if A:
        offs = its._offsets.to(torch.int32).contiguous()
        ata = torch.zeros((A, 9), dtype=torch.float32, device="cuda")
        atb = torch.zeros((A, 3), dtype=torch.float32, device="cuda")
        assert lib.nx_qef(xp.data_ptr(), nrm.data_ptr(), offs.data_ptr(), A, 1e-2, ata.data_ptr(), atb.data_ptr(),
                          C.c_void_p(torch.cuda.current_stream().cuda_stream)) == 0
        torch.cuda.synchronize()
        from oracle import Oracle

        oa, ob = Oracle("nvcc").qef(xp.cpu().numpy(), nrm.cpu().numpy(), offs.cpu().numpy(), 1e-2)
        assert np.array_equal(_bits(ata), oa.view(np.int32)), f"{what}: QEF ATA differs"
        assert np.array_equal(_bits(atb), ob.view(np.int32)), f"{what}: QEF ATb differs"
    v, f = iso.marching_cubes(g, level=level)
    if v is not None:
        cross = np.unique(_bits(xp).reshape(-1, 3), axis=0)
        vb = _bits(v).reshape(-1, 3)
        rows = np.ascontiguousarray(cross).view(np.dtype((np.void, 12))).ravel()
        vr = np.ascontiguousarray(vb).view(np.dtype((np.void, 12))).ravel()
        assert np.isin(vr, rows).all(), f"{what}: MC vertices not among the CUDA build's crossing points"
    # the other reading differs, so this comparison separates the two builds
    iso.set_arithmetic("host")
    try:
        its_h = iso.get_intersection(g, level=level, compute_normals=True)
        diff_p = int((_bits(its_h.get_points()) != _bits(xp)).any(axis=1).sum())
        diff_n = int((_bits(its_h.get_normals()) != _bits(nrm)).any(axis=1).sum())
    finally:
        iso.set_arithmetic("nvcc")
    K = int(xp.shape[0])
    print(f"{what}: K={K} crossings bit-equal to the CUDA build; the host-build reading differs on "
          f"{diff_p} points and {diff_n} normals")
    if expect_host_diff:
        assert diff_p + diff_n > 0, f"{what}: the host reading gives the same bits; the case separates nothing"
    return K


def test_default_is_the_cuda_build():
    assert iso.get_arithmetic() == "nvcc"


def test_sphere_512_metric_grid(nx):
    """The 512^3 sphere |p| - 0.8 of the benchmark."""
    n = 512
    ax = torch.linspace(-1, 1, n, device="cuda")  # inputs only; any values do
    x, y, z = torch.meshgrid(ax, ax, ax, indexing="ij")
    vals = (torch.sqrt(x * x + y * y + z * z) - 0.8).contiguous()
    K = _check(nx, vals.cpu().numpy(), what="sphere 512")
    assert K > 3_000_000


@pytest.mark.parametrize("seed", [0, 1])
def test_noise_with_exact_zeros(nx, seed):
    _check(nx, noise((37, 41, 45), seed=seed, zero_frac=0.3), what=f"noise {seed}")


@pytest.mark.parametrize("seed", range(2))
def test_extreme_magnitudes(nx, seed):
    g = np.random.default_rng(100 + seed)
    shape = (21, 26, 33)
    mag = 10.0 ** g.uniform(-38, 38, size=shape)
    vals = (np.sign(g.uniform(-1, 1, size=shape)) * mag).astype(np.float32)
    _check(nx, vals, what=f"extreme {seed}", expect_host_diff=False)


def test_far_offset_box(nx):
    _check(nx, noise((17, 18, 19), seed=5, zero_frac=0.2), lo=(1000.0, -500.0, 2.0), hi=(1001.0, -499.5, 2.001),
           what="far box")


def test_boxes_whose_coordinates_fuse(nx):
    # sizes that are not powers of two: amin + pos * size rounds differently
    # when fused, so grid positions themselves differ between the builds
    _check(nx, torus((64, 57, 49), 0.5, 0.2), lo=(-3.7, 0.25, 10.0), hi=(11.2, 1.0, 10.5), what="odd box")
    _check(nx, sphere((33, 40, 29), 0.6), level=0.05, lo=(-0.5, -2.0, 0.0), hi=(1.5, 1.0, 0.25),
           what="torus box")
