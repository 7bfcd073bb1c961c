"""Marching cubes on the GPU against the oracle and the reference's fixtures.

Parity bar: bit-exact.  Every vertex position must equal a reference vertex to
the last bit and the face sequence must be identical after relabelling vertex
indices (faces in the same order with the same corner order).  Only the order of
the vertex list differs (isoext sorts vertices by position; this path keeps
them in edge-key order).

Tests with the ``oracle`` fixture run in both readings of isoext's FP32
arithmetic: its CUDA build's (nvcc's fused multiply-adds, the library's
default) and its host build's.  The golden fixtures were made by the host
build and are compared in that reading.
"""

import glob
import os

import numpy as np
import pytest
import torch

import isoext_gb300 as iso
from helpers import assert_same_mesh, noise, sphere, torus

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
DENSE = sorted(p for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
               if not os.path.basename(p).startswith(("sparse", "cuboid", "sdf_", "luts")))


def run_mc(values, level=0.0, method="nagae", lo=(-1, -1, -1), hi=(1, 1, 1)):
    g = iso.UniformGrid(values.shape, lo, hi)
    g.set_values(torch.from_numpy(np.ascontiguousarray(values)).cuda())
    v, f = iso.marching_cubes(g, level=level, method=method)
    if v is None:
        return np.zeros((0, 3), np.float32), np.zeros((0, 3), np.int32)
    assert v.dtype == torch.float32 and f.dtype == torch.int32 and v.is_cuda and f.is_cuda
    return v.cpu().numpy(), f.cpu().numpy()


def check(oracle, values, level=0.0, method="nagae", lo=(-1, -1, -1), hi=(1, 1, 1), what=""):
    v, f = run_mc(values, level, method, lo, hi)
    vo, fo, _ = oracle.mc_dense(values, lo, hi, level, method)
    assert_same_mesh(v, f, vo, fo, what)
    return v, f


@pytest.fixture(autouse=True)
def _default_config():
    lib = iso._ffi.lib()
    lib.iso_mc_set_config(256)
    yield
    lib.iso_mc_set_config(256)


@pytest.mark.parametrize("path", DENSE, ids=lambda p: os.path.basename(p)[:-4])
@pytest.mark.parametrize("method", ["nagae", "lorensen"])
def test_mc_matches_reference_fixture(path, method, host_arith):
    g = np.load(path)
    v, f = run_mc(g["values"], float(g["level"]), method)
    assert_same_mesh(v, f, g[f"mc_{method}_v"], g[f"mc_{method}_f"], os.path.basename(path))


@pytest.mark.parametrize("n,r", [(32, 0.5), (64, 0.7), (128, 0.8), (97, 0.45)])
@pytest.mark.parametrize("method", ["nagae", "lorensen"])
def test_mc_sphere(oracle, n, r, method):
    check(oracle, sphere((n, n, n), r), method=method, what=f"sphere{n}")


def test_mc_config1_counts(oracle):
    v, f = check(oracle, sphere((128,) * 3, 0.8), what="config1")
    assert (len(v), len(f)) == (48576, 97148)


@pytest.mark.parametrize("shape", [(16, 32, 48), (8, 64, 16), (33, 7, 130), (2, 2, 2), (3, 50, 5),
                                   (40, 3, 2), (5, 5, 1000)])
def test_mc_anisotropic(oracle, shape):
    check(oracle, sphere(shape, 0.6), what=str(shape))
    check(oracle, sphere(shape, 0.6, center=(0.1, -0.2, 0.05)), level=0.05, what=str(shape))


@pytest.mark.parametrize("seed", range(4))
@pytest.mark.parametrize("method", ["nagae", "lorensen"])
def test_mc_noise_with_exact_zeros(oracle, seed, method):
    # many vertices land exactly on grid points: exercises snapping,
    # degenerate triangles and corner-keyed vertices
    check(oracle, noise((23, 19, 37), seed=seed, zero_frac=0.3), method=method, what=f"noise{seed}")


def test_mc_levels_and_box(oracle):
    vals = torus((40, 40, 40), 0.5, 0.2)
    for lvl in [-0.1, 0.0, 0.07]:
        check(oracle, vals, level=lvl, what=f"torus level {lvl}")
    check(oracle, vals, lo=(-0.5, -2.0, 0.0), hi=(1.5, 1.0, 0.25), what="torus box")


def test_mc_flt_max_default(oracle):
    # UniformGrid's default value is FLT_MAX; crossings towards it round onto
    # the finite corner
    vals = sphere((30, 30, 30), 0.5)
    vals[:, :, 20:] = np.finfo(np.float32).max
    check(oracle, vals, what="fltmax")
    g = iso.UniformGrid([12, 12, 12])
    v, f = iso.marching_cubes(g)
    assert v is None and f is None


def test_mc_empty_and_full():
    assert run_mc(np.ones((10, 10, 10), np.float32))[0].shape == (0, 3)
    assert run_mc(-np.ones((10, 10, 10), np.float32))[0].shape == (0, 3)
    g = iso.UniformGrid([1, 5, 5])
    assert iso.marching_cubes(g) == (None, None)


@pytest.mark.parametrize("threads", [128, 256])
def test_mc_block_sizes(oracle, threads):
    lib = iso._ffi.lib()
    assert lib.iso_mc_set_config(threads) == 0
    for shape in [(31, 45, 29), (64, 64, 64), (9, 10, 101)]:
        check(oracle, sphere(shape, 0.7), what=f"{shape} T{threads}")
        check(oracle, noise(shape, seed=7, zero_frac=0.1), method="lorensen", what=f"noise {shape}")


@pytest.mark.parametrize("nz", [31, 32, 33, 63, 64, 65, 150])
def test_mc_word_boundaries(oracle, nz):
    # z extents around multiples of the 32-bit word: edges and cells that span
    # two words, partial last words
    check(oracle, sphere((20, 24, nz), 0.8), what=f"nz {nz}")
    check(oracle, noise((9, 10, nz), seed=nz, zero_frac=0.2), what=f"noise nz {nz}")


def test_mc_long_rows(oracle):
    # rows longer than 2048 words (nz > 65536) take the two-pass sign + count path
    for shape in [(3, 3, 70001), (2, 4, 66000)]:
        check(oracle, noise(shape, seed=11, zero_frac=0.05), what=f"long rows {shape}")


def test_mc_thin_grids(oracle):
    # fewer point words than grid coordinates (the count kernel also writes those)
    for shape in [(2, 2, 300), (2, 300, 2), (300, 2, 2), (3, 3, 1000)]:
        check(oracle, noise(shape, seed=5, zero_frac=0.1), what=f"thin {shape}")


def test_mc_unknown_method():
    g = iso.UniformGrid([8, 8, 8])
    with pytest.raises(RuntimeError, match="Unknown method: foo"):
        iso.marching_cubes(g, method="foo")


def test_mc_512_properties(oracle):
    # full benchmark size: counts equal the oracle's and the mesh is closed
    vals = sphere((512,) * 3, 0.8)
    v, f = run_mc(vals)
    vo, fo, _ = oracle.mc_dense(vals)
    assert_same_mesh(v, f, vo, fo, "512")
    assert (len(v), len(f)) == (787464, 1574924)
    e = np.sort(np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]]), axis=1)
    _, cnt = np.unique(e[:, 0].astype(np.int64) * len(v) + e[:, 1], return_counts=True)
    assert (cnt == 2).all()
    assert len(v) - len(cnt) + len(f) == 2  # Euler characteristic of a sphere


def test_mc_repeat_is_deterministic():
    vals = torch.from_numpy(noise((40, 41, 42), seed=11, zero_frac=0.05)).cuda()
    g = iso.UniformGrid(vals.shape)
    g.set_values(vals)
    a = iso.marching_cubes(g)
    b = iso.marching_cubes(g)
    assert torch.equal(a[0], b[0]) and torch.equal(a[1], b[1])


@pytest.mark.parametrize("seed", range(3))
def test_mc_extreme_magnitudes(oracle, seed):
    # values spanning 1e-38 .. 1e38: many edge parameters t are tiny but not
    # zero, so vertices round onto grid points without an exact zero value
    g = np.random.default_rng(100 + seed)
    shape = (21, 26, 33)
    mag = 10.0 ** g.uniform(-38, 38, size=shape)
    vals = (np.sign(g.uniform(-1, 1, size=shape)) * mag).astype(np.float32)
    for m in ["nagae", "lorensen"]:
        check(oracle, vals, method=m, what=f"extreme {seed} {m}")


def test_mc_far_offset_box(oracle):
    # coordinates far from the origin relative to the cell size
    vals = noise((17, 18, 19), seed=5, zero_frac=0.2)
    check(oracle, vals, lo=(1000.0, -500.0, 2.0), hi=(1001.0, -499.5, 2.001), what="far box")
    check(oracle, sphere((30, 30, 30), 0.3) * 1e-3, lo=(1000.0, 1000.0, 1000.0),
          hi=(1000.002, 1000.002, 1000.002), what="far sphere")


def test_set_values_from_host_tensors():
    vals = sphere((20, 21, 22), 0.6)
    ref = iso.UniformGrid([20, 21, 22])
    ref.set_values(torch.from_numpy(vals).cuda())
    for host in (torch.from_numpy(vals), torch.from_numpy(vals).pin_memory()):
        g = iso.UniformGrid([20, 21, 22])
        g.set_values(host)
        assert torch.equal(g.get_values(), ref.get_values())
    g = iso.UniformGrid([20, 21, 22])
    with pytest.raises(TypeError):
        g.set_values(torch.from_numpy(vals).double())
    with pytest.raises(RuntimeError, match="different shapes"):
        g.set_values(torch.zeros((20, 21, 23)))


def test_launch_parameters_do_not_change_results():
    """Every value of every autotuner knob gives the same meshes (MC and DC)."""
    from isoext_gb300 import tune

    vals = sphere((70, 65, 90), 0.55) + 0.02 * noise((70, 65, 90), seed=2)
    g = iso.UniformGrid(list(vals.shape))
    g.set_values(torch.from_numpy(vals.astype(np.float32)).cuda())
    old = tune.current()
    try:
        ref_mc, ref_dc = iso.marching_cubes(g), iso.dual_contouring(g)
        for key, values in tune.KNOBS.items():
            for v in values:
                tune.set(key, v)
                mc, dc = iso.marching_cubes(g), iso.dual_contouring(g)
                assert torch.equal(mc[0], ref_mc[0]) and torch.equal(mc[1], ref_mc[1]), (key, v)
                assert torch.equal(dc[0], ref_dc[0]) and torch.equal(dc[1], ref_dc[1]), (key, v)
            tune.set(key, old[key])
        rep = tune.autotune(g, repeats=3)
        assert all(rep["best"][k] in tune.KNOBS[k] for k in tune.KNOBS)
        assert tune.current() == rep["best"]
    finally:
        tune.apply(old)


def test_autotune_cache_applies_stored_results(tmp_path):
    from isoext_gb300 import tune

    vals = sphere((64, 64, 64), 0.6)
    g = iso.UniformGrid(list(vals.shape))
    g.set_values(torch.from_numpy(vals).cuda())
    old = tune.current()
    path = str(tmp_path / "tune.json")
    try:
        first = tune.autotune(g, kinds=("mc",), repeats=2, cache=path)
        assert not first["cached"]
        tune.apply({k: tune.KNOBS[k][0] for k in tune.KNOBS})  # anything else
        second = tune.autotune(g, kinds=("mc",), repeats=2, cache=path)
        assert second["cached"]
        assert {k: v for k, v in second["best"].items() if k.startswith("mc.")} == \
            {k: v for k, v in first["best"].items() if k.startswith("mc.")}
    finally:
        tune.apply(old)


def test_bounded_wait_times_out_with_a_status():
    """A look-back wait on states nobody publishes gives up after its limit and
    reports ISO_ERR_TIMEOUT; the context stays usable."""
    import ctypes

    from isoext_gb300 import _ffi

    lib = _ffi.lib()
    lib.iso_test_wait_timeout.argtypes = [ctypes.c_uint, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p]
    state = torch.zeros(64, dtype=torch.int64, device="cuda")
    status = torch.zeros(2, dtype=torch.int32, device="cuda")
    out = torch.zeros(2, dtype=torch.int64, device="cuda")
    rc = lib.iso_test_wait_timeout(4096, ctypes.c_void_p(state.data_ptr()), ctypes.c_void_p(status.data_ptr()),
                                   ctypes.c_void_p(out.data_ptr()),
                                   ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0
    torch.cuda.synchronize()
    assert int(status[0]) == _ffi.ISO_ERR_TIMEOUT
    assert lib.iso_test_wait_timeout(1 << 21, ctypes.c_void_p(state.data_ptr()), ctypes.c_void_p(status.data_ptr()),
                                     ctypes.c_void_p(out.data_ptr()), None) == _ffi.ISO_ERR_ARG
    v, f = run_mc(sphere((24, 24, 24), 0.5))
    assert len(f) > 0


def _weld_mesh_np(v, f):
    """isoext's position weld restated: the first vertex of each position
    (bits, -0 read as +0), faces with two equal vertices dropped, unused
    vertices dropped, order kept."""
    vn = np.where(v == 0, np.float32(0), v).astype(np.float32)
    bits = vn.view(np.uint32)
    first = {}
    rep = np.empty(len(v), np.int64)
    for i, key in enumerate(map(bytes, bits)):
        rep[i] = first.setdefault(key, i)
    f2 = rep[f]
    keep = (f2[:, 0] != f2[:, 1]) & (f2[:, 0] != f2[:, 2]) & (f2[:, 1] != f2[:, 2])
    f2 = f2[keep]
    used = np.zeros(len(v), bool)
    used[f2.ravel()] = True
    num = np.cumsum(used) - 1
    return v[used], num[f2].astype(np.int32), np.nonzero(used)[0]


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_weld_mesh_matches_the_position_weld(seed):
    """iso_weld_mesh (the path of grids whose spacing comes within a few ulps of
    their coordinates) against the restated weld, with repeated positions, -0
    against +0, faces that become degenerate and vertices no face uses."""
    from isoext_gb300 import _ffi

    rng = np.random.default_rng(seed)
    pool = rng.integers(-3, 4, size=(400, 3)).astype(np.float32) * np.float32(0.25)
    pool[rng.random(400) < 0.1, 0] = np.float32(-0.0)
    v = pool[rng.integers(0, 400, size=3000)]
    f = rng.integers(0, 3000, size=(5000, 3)).astype(np.int32)
    vo, fo, so = _weld_mesh_np(v, f)
    vg, fg, sg = _ffi.weld_mesh(torch.from_numpy(v).cuda(), torch.from_numpy(f).cuda(), want_source=True)
    assert np.array_equal(vg.cpu().numpy().view(np.uint32), vo.view(np.uint32))
    assert np.array_equal(fg.cpu().numpy(), fo)
    assert np.array_equal(sg.cpu().numpy(), so)
