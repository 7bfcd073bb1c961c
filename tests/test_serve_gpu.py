"""The served loop on the GPU: grid evaluation of a union matches its FP32
formula, and every served result equals the one-call-per-grid result, bit for
bit, whether the request ran alone or among others."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _union_np(points, prims):
    """The union's value at float32 points [..., 3]: sphere |p - c| - r and box
    |max(q, 0)| + min(max q, 0), q = |p - c| - h, each operation rounded to float32."""
    f = np.float32
    d = np.full(points.shape[:-1], np.finfo(np.float32).max, np.float32)
    for row in prims.astype(np.float32):
        dx, dy, dz = (points[..., k] - row[1 + k] for k in range(3))
        if row[0] == 0:
            dk = np.sqrt((dx * dx + dy * dy) + dz * dz) - row[4]
        else:
            qx, qy, qz = np.abs(dx) - row[4], np.abs(dy) - row[5], np.abs(dz) - row[6]
            ox, oy, oz = (np.maximum(q, f(0)) for q in (qx, qy, qz))
            dk = np.sqrt((ox * ox + oy * oy) + oz * oz) + np.minimum(np.maximum(qx, np.maximum(qy, qz)), f(0))
        d = np.minimum(d, dk.astype(np.float32))
    return d


@pytest.mark.parametrize("shape,req", [((33, 40, 47), 3), ((64, 64, 64), 3)] +
                         [((29, 31, 67), r) for r in range(8)])
def test_union_grid_matches_formula(shape, req):
    """Bit for bit against the formula, for unions of 1 to 16 spheres and boxes
    (a warp per grid row, its lanes along z, rows shorter and longer than a
    warp)."""
    import ctypes as C

    from isoext_gb300 import UniformGrid, _ffi
    from isoext_gb300.serve import HI, LO, prims_buffer, random_requests

    prims = random_requests(8, seed=11)[req].prims
    grid = UniformGrid(list(shape), LO, HI)
    dev = torch.from_numpy(prims_buffer(prims)).cuda()
    _ffi.check(_ffi.lib().iso_sdf_union_grid(C.c_void_p(dev.data_ptr()), *shape, _ffi.fvec3(LO), _ffi.fvec3(HI),
                                             C.c_void_p(grid._values.data_ptr()),
                                             C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    got = grid.get_values().cpu().numpy()
    want = _union_np(grid.get_points().cpu().numpy(), prims)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def _same(a, b):
    return a[0].shape == b[0].shape and np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_served_results_equal_plain_results():
    from isoext_gb300.serve import Server, random_requests, solve_plain

    reqs = random_requests(24, seed=5, sizes=(32, 48, 64))
    solo = [solve_plain(r) for r in reqs]
    srv = Server(slots=3, budget_bytes=1 << 30)
    srv.warmup((32, 48, 64))
    futs = [srv.submit(r) for r in reqs]
    served = [f.result(timeout=300) for f in futs]
    srv.close()
    assert srv.max_running > 1  # requests were on the device together
    for r, s, p in zip(reqs, served, solo):
        assert s.rid == r.rid
        assert len(p[1]) > 0
        assert _same((s.vertices, s.faces), p), (r.rid, r.kind, r.n)


def test_served_overflow_reruns_with_exact_sizes(monkeypatch):
    from isoext_gb300 import serve

    reqs = serve.random_requests(24, seed=9, sizes=(48,))
    plain = [serve.solve_plain(r) for r in reqs]
    big = [(r, p) for r, p in zip(reqs, plain) if len(p[1]) > 64 and r.kind == "mc"][:2]
    big += [(r, p) for r, p in zip(reqs, plain) if len(p[1]) > 64 and r.kind == "dc"][:2]
    assert len(big) == 4
    monkeypatch.setattr(serve, "_mc_caps", lambda n: (64, 64))
    srv = serve.Server(slots=2, budget_bytes=1 << 30)
    out = [f.result(timeout=300) for f in [srv.submit(r) for r, _ in big]]
    srv.close()
    for (r, p), s in zip(big, out):
        assert _same((s.vertices, s.faces), p)


def test_native_server_results_equal_plain_results():
    from isoext_gb300.serve import NativeServer, random_requests, solve_plain

    reqs = random_requests(24, seed=5, sizes=(32, 48, 64))
    solo = [solve_plain(r) for r in reqs]
    srv = NativeServer(slots=3, budget_bytes=1 << 30, warm_sizes=(32, 48, 64))
    futs = [srv.submit(r) for r in reqs]
    served = [f.result(timeout=300) for f in futs]
    stats = srv.stats()
    srv.close()
    assert stats["completed"] == len(reqs) and stats["max_running"] > 1
    for r, s, p in zip(reqs, served, solo):
        assert s.rid == r.rid
        assert _same((s.vertices, s.faces), p), (r.rid, r.kind, r.n)


def test_native_server_buckets_equal_plain_results():
    """Length buckets: same-key requests queued together run as parallel branches
    of one graph launch; every result equals the plain path's, bit for bit."""
    from isoext_gb300.serve import NativeServer, random_requests, solve_plain

    reqs = random_requests(40, seed=21, sizes=(32, 48))
    solo = [solve_plain(r) for r in reqs]
    srv = NativeServer(slots=2, budget_bytes=1 << 30, warm_sizes=(32, 48), bucket=8)
    futs = [srv.submit(r) for r in reqs]
    served = [f.result(timeout=300) for f in futs]
    stats = srv.stats()
    srv.close()
    assert stats["completed"] == len(reqs)
    assert stats["bucket_launches"] > 0 and stats["bucketed_requests"] >= 2 * stats["bucket_launches"]
    for r, s, p in zip(reqs, served, solo):
        assert s.rid == r.rid
        assert _same((s.vertices, s.faces), p), (r.rid, r.kind, r.n)


def test_native_server_buckets_grow_together():
    """A bucket whose meshes outgrow its buffers grows every branch to the
    largest counted sizes and runs again."""
    import ctypes

    from isoext_gb300 import _ffi
    from isoext_gb300.serve import NativeServer, random_requests, solve_plain

    reqs = random_requests(16, seed=23, sizes=(40,))
    srv = NativeServer(slots=1, budget_bytes=1 << 30, warm_sizes=(), tune=False, bucket=4)
    assert _ffi.lib().iso_serve_set_capacity_scale(srv._h, ctypes.c_double(1e-4)) == 0
    out = [f.result(timeout=300) for f in [srv.submit(r) for r in reqs]]
    stats = srv.stats()
    srv.close()
    assert stats["grown"] > 0 and stats["bucket_launches"] > 0
    for r, s in zip(reqs, out):
        assert _same((s.vertices, s.faces), solve_plain(r)), (r.rid, r.kind)


def test_native_server_bucket_sizes():
    from isoext_gb300 import _ffi
    from isoext_gb300.serve import NativeServer

    srv = NativeServer(slots=1, budget_bytes=1 << 28, warm_sizes=(), tune=False)
    try:
        for b in (1, 2, 4, 8):
            assert _ffi.lib().iso_serve_set_bucket(srv._h, b) == 0
        for b in (0, 3, 16, -1):
            assert _ffi.lib().iso_serve_set_bucket(srv._h, b) == _ffi.ISO_ERR_ARG
    finally:
        srv.close()


def test_native_server_reruns_meshes_larger_than_its_buffers():
    import ctypes

    from isoext_gb300 import _ffi
    from isoext_gb300.serve import NativeServer, random_requests, solve_plain

    reqs = random_requests(8, seed=9, sizes=(48,))
    srv = NativeServer(slots=2, budget_bytes=1 << 30, warm_sizes=(), tune=False)
    assert _ffi.lib().iso_serve_set_capacity_scale(srv._h, ctypes.c_double(1e-4)) == 0
    out = [f.result(timeout=300) for f in [srv.submit(r) for r in reqs]]
    stats = srv.stats()
    srv.close()
    assert stats["grown"] > 0  # entries built too small grew from the sizes their run counted
    for r, s in zip(reqs, out):
        assert _same((s.vertices, s.faces), solve_plain(r)), (r.rid, r.kind)


def test_native_server_memory_stays_within_budget():
    """50 requests of distinct (size, level) keys, each needing an entry of its
    own, under a budget that holds a few: entries are sized by a count pass,
    the least recently used idle ones are evicted, the bytes held never exceed
    the budget, and every result equals the plain path's."""
    from isoext_gb300.serve import NativeServer, random_requests, solve_plain

    reqs = random_requests(50, seed=21, sizes=(24, 32, 40, 48, 56, 64, 72, 80))
    for i, r in enumerate(reqs):
        r.level = float(np.float32(-0.05 + 0.002 * i))
    budget = 48 << 20
    srv = NativeServer(slots=3, budget_bytes=budget, warm_sizes=(), tune=False)
    out = [f.result(timeout=300) for f in [srv.submit(r) for r in reqs]]
    stats = srv.stats()
    srv.close()
    assert stats["completed"] == len(reqs)
    assert stats["max_held_bytes"] <= budget, stats
    assert stats["evictions"] > 0 and stats["count_passes"] == len(reqs), stats
    for r, s in zip(reqs, out):
        assert _same((s.vertices, s.faces), solve_plain(r)), (r.rid, r.kind, r.n, r.level)


def test_native_server_refuses_bad_requests():
    import numpy as np

    from isoext_gb300.serve import NativeServer, Request

    srv = NativeServer(slots=1, budget_bytes=64 << 20, warm_sizes=(), tune=False)
    with pytest.raises(ValueError, match="budget"):
        srv.submit(Request("mc", 400, np.zeros((1, 7), np.float32)))
    with pytest.raises(ValueError):
        srv.submit(Request("mc", 32, np.zeros((0, 7), np.float32)))
    srv.close()
