"""SparseGrid on the GPU against the reference's fixtures and the oracle.

MC: bit-exact positions, faces equal after relabelling (isoext welds by
position; here vertices come in first-occurrence order).  Intersections:
bit-exact.  DC: positions within 1e-4 * h of the FP64 oracle, quads as in
test_dc_gpu.  Tests with the ``oracle`` fixture run in both readings of
isoext's FP32 arithmetic; the golden fixtures (host build) in the host one.
"""

import os

import numpy as np
import pytest
import torch

import isoext_gb300 as iso
from helpers import assert_same_mesh, grid_points, sphere, torus
from test_dc_gpu import assert_dc_match, cell_h

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def sparse_from_dense(values, keep="active", extra=0, seed=0, level=0.0):
    """(ids, vals [N, 8]) of the cells of a dense grid whose corners straddle the
    level, plus `extra` random other cells (consistent values)."""
    shape = values.shape
    n = np.asarray(shape)
    cx, cy, cz = np.meshgrid(*[np.arange(k - 1) for k in shape], indexing="ij")
    vals = np.stack([values[cx + (k >> 2), cy + ((k >> 1) & 1), cz + (k & 1)] for k in range(8)], -1)
    ids = ((cx * (n[1] - 1) + cy) * (n[2] - 1) + cz).astype(np.int64)
    neg = (vals < level).sum(-1)
    mask = (neg > 0) & (neg < 8) if keep == "active" else np.ones_like(neg, bool)
    if extra:
        rng = np.random.default_rng(seed)
        flat = np.nonzero(~mask.ravel())[0]
        pick = rng.choice(flat, size=min(extra, len(flat)), replace=False)
        m2 = mask.ravel().copy()
        m2[pick] = True
        mask = m2.reshape(mask.shape)
    sel_ids = ids[mask].astype(np.int32)
    sel_vals = vals[mask].astype(np.float32)
    order = np.argsort(sel_ids)
    return sel_ids[order], np.ascontiguousarray(sel_vals[order])


def make_sparse(shape, ids, vals, lo=(-1, -1, -1), hi=(1, 1, 1)):
    g = iso.SparseGrid(shape, lo, hi)
    g.add_cells(torch.from_numpy(np.asarray(ids, np.int32)).cuda())
    g.set_values(torch.from_numpy(np.asarray(vals, np.float32)).cuda())
    return g


# --- fixtures from the reference's host build -----------------------------------

@pytest.mark.parametrize("method", ["nagae", "lorensen"])
def test_sparse_mc_matches_reference_fixture(method, host_arith):
    gd = np.load(os.path.join(GOLDEN, "sparse16.npz"))
    shape = tuple(int(x) for x in gd["shape"])
    g = make_sparse(shape, gd["cell_ids"], gd["values"])
    v, f = iso.marching_cubes(g, method=method)
    assert_same_mesh(v.cpu().numpy(), f.cpu().numpy(), gd[f"mc_{method}_v"], gd[f"mc_{method}_f"], method)


def test_sparse_dc_matches_reference_fixture(host_arith):
    gd = np.load(os.path.join(GOLDEN, "sparse16.npz"))
    shape = tuple(int(x) for x in gd["shape"])
    g = make_sparse(shape, gd["cell_ids"], gd["values"])
    v, f = iso.dual_contouring(g)
    assert_dc_match(v.cpu().numpy(), f.cpu().numpy(), gd["dc_v"], gd["dc_f"], cell_h(shape), "sparse16")


# --- against the oracle ------------------------------------------------------------

@pytest.mark.parametrize("method", ["nagae", "lorensen"])
@pytest.mark.parametrize("extra", [0, 500])
def test_sparse_mc_matches_oracle(oracle, method, extra):
    vals = torus((40, 36, 44), 0.5, 0.2)
    ids, cv = sparse_from_dense(vals, extra=extra, seed=extra)
    g = make_sparse(vals.shape, ids, cv)
    v, f = iso.marching_cubes(g, method=method)
    vo, fo, _ = oracle.mc_sparse(ids, cv, vals.shape, method=method)
    assert_same_mesh(v.cpu().numpy(), f.cpu().numpy(), vo, fo, f"{method} extra {extra}")


@pytest.mark.parametrize("shape", [(30, 4, 50), (33, 31, 3), (3, 40, 40), (2, 2, 2), (25, 2, 37), (41, 23, 4)])
def test_sparse_mc_thin_grids(oracle, shape):
    """Grids one or two cells thick along an axis: the owner of an edge is
    looked for at y - 1 and z +- 1 only where those cells exist (y > 0, z > 0,
    z + 1 < nz - 1), and chunk ends cut neighbours apart."""
    rng = np.random.default_rng(sum(shape))
    vals = (rng.standard_normal(shape) * 0.3 + sphere(shape, 0.5)).astype(np.float32) \
        if min(shape) > 2 else rng.uniform(-1, 1, size=shape).astype(np.float32)
    ids, cv = sparse_from_dense(vals, extra=50, seed=1)
    if len(ids) == 0:
        pytest.skip("no crossed cell")
    g = make_sparse(shape, ids, cv)
    for method in ("nagae", "lorensen"):
        v, f = iso.marching_cubes(g, method=method)
        vo, fo, _ = oracle.mc_sparse(ids, cv, shape, method=method)
        if v is None:
            assert len(fo) == 0
            continue
        assert_same_mesh(v.cpu().numpy(), f.cpu().numpy(), vo, fo, f"{method} {shape}")


def test_sparse_mc_missing_neighbours(oracle):
    """Consistent values, but a random half of the crossed cells left out: an
    edge's earlier cells are often absent, and the first present one owns it."""
    vals = torus((44, 40, 48), 0.5, 0.2)
    ids, cv = sparse_from_dense(vals)
    keep = np.random.default_rng(4).random(len(ids)) < 0.5
    ids, cv = ids[keep], np.ascontiguousarray(cv[keep])
    g = make_sparse(vals.shape, ids, cv)
    v, f = iso.marching_cubes(g)
    vo, fo, _ = oracle.mc_sparse(ids, cv, vals.shape)
    assert_same_mesh(v.cpu().numpy(), f.cpu().numpy(), vo, fo, "half the cells")


@pytest.mark.parametrize("seed,drop,shape", [(0, 0.2, (40, 44, 36)), (1, 0.5, (36, 40, 44)),
                                             (2, 0.8, (44, 36, 40)), (3, 0.3, (96, 90, 100))])
def test_sparse_mc_dropped_and_perturbed_cells(oracle, seed, drop, shape):
    """Random cells left out and one corner value in ten moved by an ulp: every
    pattern of present, absent, compatible and incompatible cells around an
    edge (and, on the largest grid, chunk ends through them) must give the
    oracle's mesh."""
    vals = torus(shape, 0.5, 0.2)
    ids, cv = sparse_from_dense(vals, extra=200, seed=seed)
    rng = np.random.default_rng(100 + seed)
    keep = rng.random(len(ids)) >= drop
    ids, cv = ids[keep], np.ascontiguousarray(cv[keep])
    moved = rng.random(cv.shape) < 0.1
    cv[moved] = np.nextafter(cv[moved], np.float32(np.inf))
    g = make_sparse(shape, ids, cv)
    for method in ("nagae", "lorensen"):
        v, f = iso.marching_cubes(g, method=method)
        vo, fo, _ = oracle.mc_sparse(ids, cv, shape, method=method)
        assert_same_mesh(v.cpu().numpy(), f.cpu().numpy(), vo, fo, f"{method} seed {seed}")


def test_sparse_mc_inconsistent_values(oracle):
    # independent random values per cell: shared corners disagree, so welding
    # by exact position is all that joins cells
    rng = np.random.default_rng(7)
    shape = (12, 10, 14)
    ncell = 11 * 9 * 13
    ids = np.sort(rng.choice(ncell, size=600, replace=False)).astype(np.int32)
    cv = rng.standard_normal((600, 8)).astype(np.float32)
    cv[rng.random((600, 8)) < 0.05] = 0.0  # exact zeros: vertices on grid points
    g = make_sparse(shape, ids, cv)
    for method in ("nagae", "lorensen"):
        v, f = iso.marching_cubes(g, method=method)
        vo, fo, _ = oracle.mc_sparse(ids, cv, shape, method=method)
        assert_same_mesh(v.cpu().numpy(), f.cpu().numpy(), vo, fo, method)


def test_sparse_mc_neighbours_disagree_by_an_ulp(oracle):
    # consistent cells, then one corner value of some cells moved by one ulp:
    # those cells' shared edges give positions that differ from the
    # neighbour's (or not, where the lerp rounds them together), and only
    # exact position equality may join them
    vals = torus((36, 40, 44), 0.5, 0.2)
    ids, cv = sparse_from_dense(vals, extra=300, seed=5)
    rng = np.random.default_rng(11)
    pick = rng.random(len(ids)) < 0.15
    corner = rng.integers(0, 8, len(ids))
    rows = np.nonzero(pick)[0]
    cv[rows, corner[rows]] = np.nextafter(cv[rows, corner[rows]], np.float32(np.inf))
    g = make_sparse(vals.shape, ids, cv)
    for method in ("nagae", "lorensen"):
        v, f = iso.marching_cubes(g, method=method)
        vo, fo, _ = oracle.mc_sparse(ids, cv, vals.shape, method=method)
        assert_same_mesh(v.cpu().numpy(), f.cpu().numpy(), vo, fo, method)


def test_sparse_mc_every_edge_crossed(oracle):
    # a checkerboard field crosses all 12 edges of every cell: a chunk of the
    # cell list then holds far more vertex entries and triangles than a CTA
    # stages, so the direct writes (and no CTA-local weld) carry the output
    rng = np.random.default_rng(3)
    shape = (26, 22, 30)
    x, y, z = np.meshgrid(*[np.arange(k) for k in shape], indexing="ij")
    vals = np.where((x + y + z) % 2 == 0, 1.0, -1.0) * (0.5 + rng.random(shape))
    ids, cv = sparse_from_dense(vals.astype(np.float32))
    assert len(ids) == np.prod([k - 1 for k in shape])
    g = make_sparse(shape, ids, cv)
    for method in ("nagae", "lorensen"):
        v, f = iso.marching_cubes(g, method=method)
        vo, fo, _ = oracle.mc_sparse(ids, cv, shape, method=method)
        assert_same_mesh(v.cpu().numpy(), f.cpu().numpy(), vo, fo, method)


def test_sparse_intersection_matches_oracle(oracle):
    vals = sphere((36, 36, 36), 0.6, center=(0.02, -0.03, 0.01))
    ids, cv = sparse_from_dense(vals, extra=300, seed=3)
    g = make_sparse(vals.shape, ids, cv)
    for normals in (False, True):
        its = iso.get_intersection(g, compute_normals=normals)
        ref = oracle.intersection_sparse(ids, cv, vals.shape, normals=normals)
        assert np.array_equal(its.get_points().cpu().numpy(), ref["points"])
        if normals:
            assert np.array_equal(its.get_normals().cpu().numpy(), ref["normals"])
        assert np.array_equal(its._cells.cpu().numpy().astype(np.uint32), ref["cell_indices"])
        assert np.array_equal(its._offsets.cpu().numpy().astype(np.uint32), ref["cell_offsets"])


@pytest.mark.parametrize("extra", [0, 400])
def test_sparse_dc_matches_oracle(oracle, extra):
    vals = sphere((40, 40, 40), 0.6, center=(0.03, 0.01, -0.02))
    ids, cv = sparse_from_dense(vals, extra=extra, seed=11)
    g = make_sparse(vals.shape, ids, cv)
    v, f = iso.dual_contouring(g)
    its = oracle.intersection_sparse(ids, cv, vals.shape)
    vo, fo, _ = oracle.dc(its, vals.shape, values=cv, cell_ids=ids)
    assert_dc_match(v.cpu().numpy(), f.cpu().numpy(), vo, fo, cell_h(vals.shape), f"extra {extra}")


def _populate_like_the_reference(g, sdf, level):
    """The reference tests' population loop (tests/conftest.py:39-61): the
    potential cells in one chunk, those whose corners straddle the level kept,
    then every kept cell's SDF values."""
    n = g.get_shape()
    for chunk in g.get_potential_cell_indices(n[0] * n[1] * n[2]):
        kept = g.filter_cell_indices(chunk, sdf(g.get_points_by_cell_indices(chunk)), level=level)
        if len(kept) > 0:
            g.add_cells(kept)
    if g.get_num_cells() > 0:
        g.set_values(sdf(g.get_points()))


@pytest.mark.parametrize("level", [-0.1, 0.0, 0.1])
def test_sparse_levels_match_oracle(oracle, level):
    """tests/test_marching_cubes.py:166-180 and tests/test_dual_contouring.py's
    sparse level sweep, each mesh against the oracle."""
    g = iso.SparseGrid([32, 32, 32], aabb_min=[-1, -1, -1], aabb_max=[1, 1, 1])
    _populate_like_the_reference(g, lambda p: p.norm(dim=-1) - 0.5, level)
    assert g.get_num_cells() > 0
    ids = g.get_cell_indices().cpu().numpy()
    cv = g.get_values().cpu().numpy()
    for method in ("nagae", "lorensen"):
        v, f = iso.marching_cubes(g, level=level, method=method)
        vo, fo, _ = oracle.mc_sparse(ids, cv, (32, 32, 32), level=level, method=method)
        assert_same_mesh(v.cpu().numpy(), f.cpu().numpy(), vo, fo, f"{method} level {level}")
    v, f = iso.dual_contouring(g, level=level)
    its = oracle.intersection_sparse(ids, cv, (32, 32, 32), level=level)
    vo, fo, _ = oracle.dc(its, (32, 32, 32), values=cv, cell_ids=ids)
    assert_dc_match(v.cpu().numpy(), f.cpu().numpy(), vo, fo, cell_h((32, 32, 32)), f"level {level}")


def test_sparse_dc_user_intersection(oracle):
    vals = torus((36, 36, 36), 0.5, 0.2)
    ids, cv = sparse_from_dense(vals)
    g = make_sparse(vals.shape, ids, cv)
    its = iso.get_intersection(g)
    assert not its.has_normals()
    v, f = iso.dual_contouring(g, intersection=its)  # normals computed from the grid
    ref = oracle.intersection_sparse(ids, cv, vals.shape)
    vo, fo, _ = oracle.dc(ref, vals.shape, values=cv, cell_ids=ids)
    assert_dc_match(v.cpu().numpy(), f.cpu().numpy(), vo, fo, cell_h(vals.shape), "auto normals")
    pts = its.get_points()
    n = torch.nn.functional.normalize(pts - pts.mean(0), dim=-1).contiguous()
    its.set_normals(n)
    v, f = iso.dual_contouring(g, intersection=its)
    ref["normals"] = n.cpu().numpy()
    vo, fo, _ = oracle.dc(ref, vals.shape, values=cv, cell_ids=ids)
    assert_dc_match(v.cpu().numpy(), f.cpu().numpy(), vo, fo, cell_h(vals.shape), "user normals")


# --- sparse over all active cells == dense ----------------------------------------

@pytest.mark.parametrize("n", [64, 128])
def test_sparse_equals_dense_mc(n):
    vals = sphere((n, n, n), 0.7, center=(0.01, 0.02, -0.01))
    ids, cv = sparse_from_dense(vals)
    g = make_sparse(vals.shape, ids, cv)
    d = iso.UniformGrid(vals.shape)
    d.set_values(torch.from_numpy(vals).cuda())
    for method in ("nagae", "lorensen"):
        v, f = iso.marching_cubes(g, method=method)
        vd, fd = iso.marching_cubes(d, method=method)
        assert_same_mesh(v.cpu().numpy(), f.cpu().numpy(), vd.cpu().numpy(), fd.cpu().numpy(), method)


def test_sparse_equals_dense_dc():
    vals = torus((64, 64, 64), 0.5, 0.2)
    ids, cv = sparse_from_dense(vals)
    g = make_sparse(vals.shape, ids, cv)
    d = iso.UniformGrid(vals.shape)
    d.set_values(torch.from_numpy(vals).cuda())
    v, f = iso.dual_contouring(g)
    vd, fd = iso.dual_contouring(d)
    assert_dc_match(v.cpu().numpy(), f.cpu().numpy(), vd.cpu().numpy(), fd.cpu().numpy(), cell_h(vals.shape))


# --- the container API ---------------------------------------------------------------

def test_sparse_container_api():
    g = iso.SparseGrid([8, 9, 10], default_value=5.0)
    assert g.get_num_cells() == 0 and g.get_num_points() == 0
    g.add_cells(torch.tensor([30, 5, 30, 7], dtype=torch.int32, device="cuda"))
    assert g.get_cell_indices().tolist() == [5, 7, 30]
    assert g.get_num_points() == 24
    assert torch.equal(g.get_values(), torch.full((3, 8), 5.0, device="cuda"))
    g.set_values(torch.arange(24, dtype=torch.float32, device="cuda").view(3, 8))
    g.add_cells(torch.tensor([6], dtype=torch.int32, device="cuda"))
    assert g.get_cell_indices().tolist() == [5, 6, 7, 30]
    assert (g.get_values() == 5.0).all()  # isoext resets every value on add/remove
    g.remove_cells(torch.tensor([7, 100], dtype=torch.int32, device="cuda"))
    assert g.get_cell_indices().tolist() == [5, 6, 30]
    assert g.get_cells().tolist()[1] == list(range(8, 16))
    with pytest.raises(RuntimeError, match="New values size does not match number of points"):
        g.set_values(torch.zeros((2, 8), device="cuda"))
    with pytest.raises(TypeError):
        g.set_values(torch.zeros((3, 8)))
    with pytest.raises(TypeError):
        g.add_cells(torch.tensor([1], dtype=torch.int64, device="cuda"))
    with pytest.raises(RuntimeError, match="max int"):
        iso.SparseGrid([2048, 2048, 2048])


def test_sparse_points_and_chunks():
    shape = (17, 12, 9)
    g = iso.SparseGrid(shape, (-1, -0.5, 0.0), (1, 0.5, 2.0))
    ids = torch.tensor([0, 3, 57, 11 * 16 * 8 - 1], dtype=torch.int32, device="cuda")
    g.add_cells(ids)
    pts = g.get_points().cpu().numpy()
    dense = grid_points(shape, (-1, -0.5, 0.0), (1, 0.5, 2.0))
    for r, c in enumerate(ids.tolist()):
        z = c % 8
        y = (c // 8) % 11
        x = c // 88
        for k in range(8):
            assert np.array_equal(pts[r, k], dense[x + (k >> 2), y + ((k >> 1) & 1), z + (k & 1)])
    assert torch.equal(g.get_points_by_cell_indices(ids[1:3].contiguous()), g.get_points()[1:3])
    chunks = g.get_potential_cell_indices(1000)
    total = 17 * 12 * 9
    assert len(chunks) == (total + 999) // 1000
    assert torch.equal(torch.cat(chunks), torch.arange(total, dtype=torch.int32, device="cuda"))


def test_sparse_population_loop_matches_dense():
    # isoext's documented loop (doc/grids.ipynb): potential ids -> points -> SDF ->
    # filter -> add -> set values -> extract
    n = 48
    g = iso.SparseGrid([n] * 3)
    keep = []
    for chunk in g.get_potential_cell_indices(20000):
        p = g.get_points_by_cell_indices(chunk)
        sdf = (p.norm(dim=-1) - 0.6).contiguous()
        keep.append(g.filter_cell_indices(chunk, sdf))
    g.add_cells(torch.cat(keep))
    g.set_values((g.get_points().norm(dim=-1) - 0.6).contiguous())
    d = iso.UniformGrid([n] * 3)
    d.set_values((d.get_points().norm(dim=-1) - 0.6).contiguous())
    v, f = iso.marching_cubes(g)
    vd, fd = iso.marching_cubes(d)
    assert_same_mesh(v.cpu().numpy(), f.cpu().numpy(), vd.cpu().numpy(), fd.cpu().numpy(), "population")


def test_sparse_empty():
    g = iso.SparseGrid([16, 16, 16])
    assert iso.marching_cubes(g) == (None, None)
    assert iso.dual_contouring(g) == (None, None)
    assert iso.get_intersection(g).get_points().shape == (0, 3)
    g.add_cells(torch.tensor([1, 2, 3], dtype=torch.int32, device="cuda"))  # FLT_MAX values
    assert iso.marching_cubes(g) == (None, None)


# --- device-side population ---------------------------------------------------------

def _spheres(count, seed, k=0.05):
    from isoext_gb300 import sdf as S

    rng = np.random.default_rng(seed)
    prims = [S.TranslationOp(S.SphereSDF(float(r)), [float(x) for x in c])
             for c, r in zip(rng.uniform(-0.7, 0.7, size=(count, 3)), rng.uniform(0.05, 0.25, size=count))]
    return S.SmoothUnionOp(prims, k)


def test_populate_surface_equals_the_documented_loop():
    shape = (40, 33, 47)
    f = _spheres(12, seed=4)
    g1 = iso.SparseGrid(shape)
    g1.populate(f, mode="surface", brick=4)
    g2 = iso.SparseGrid(shape)
    ncells = 39 * 32 * 46
    for ids in g2.get_potential_cell_indices(5000):
        ids = ids[ids < ncells].contiguous()
        vals = f(g2.get_points_by_cell_indices(ids)).contiguous()
        kept = g2.filter_cell_indices(ids, vals)
        if kept.numel():
            g2.add_cells(kept)
    g2.set_values(f(g2.get_points()).contiguous())
    assert g1.get_num_cells() > 1000
    assert torch.equal(g1.get_cell_indices(), g2.get_cell_indices())
    assert torch.equal(g1.get_values(), g2.get_values())
    v1, f1 = iso.marching_cubes(g1)
    v2, f2 = iso.marching_cubes(g2)
    assert torch.equal(v1, v2) and torch.equal(f1, f2)


def test_populate_brick_mode_keeps_whole_bricks_around_the_surface():
    shape = (50, 50, 50)
    f = _spheres(6, seed=8)
    g = iso.SparseGrid(shape)
    g.populate(f, mode="brick", brick=8)
    s = iso.SparseGrid(shape)
    s.populate(f, mode="surface", brick=8)
    ids = g.get_cell_indices().long().cpu().numpy()
    assert np.all(np.diff(ids) > 0)
    assert np.isin(s.get_cell_indices().cpu().numpy(), ids).all()
    n = 49
    x, y, z = ids // (n * n), (ids // n) % n, ids % n
    b = (x // 8) * 49 + (y // 8) * 7 + z // 8
    counts = np.bincount(b)
    full = [min(8, n - 8 * k) for k in range(7)]
    for bid in np.nonzero(counts)[0]:
        bx, by, bz = bid // 49, (bid // 7) % 7, bid % 7
        assert counts[bid] == full[bx] * full[by] * full[bz]
    # values are the SDF at the cells' corners, as set_values(sdf(get_points())) gives
    assert torch.equal(g.get_values(), f(g.get_points()).contiguous())


def test_populate_brick_size_does_not_change_the_mesh():
    """The brick edge (an autotuner knob) decides only which empty cells near the
    surface are kept: MC and DC meshes are the same for every brick size."""
    from isoext_gb300 import tune

    shape = (72, 64, 80)
    f = _spheres(10, seed=12)
    meshes = {}
    for b in tune.BRICKS:
        g = iso.SparseGrid(shape)
        g.populate(f, mode="brick", brick=b)
        meshes[b] = (iso.marching_cubes(g), iso.dual_contouring(g), g.get_num_cells())
    (mc0, dc0, n0) = meshes[tune.BRICKS[0]]
    assert len({n for _, _, n in meshes.values()}) > 1  # the kept cells differ
    for b, (mc, dc, _) in meshes.items():
        assert torch.equal(mc[0], mc0[0]) and torch.equal(mc[1], mc0[1]), b
        assert torch.equal(dc[0], dc0[0]) and torch.equal(dc[1], dc0[1]), b


def test_autotune_populate_picks_a_brick(tmp_path):
    from isoext_gb300 import tune

    old = tune.populate_brick()
    try:
        rep = tune.autotune_populate((96, 96, 96), _spheres(8, seed=3), repeats=1, cache=str(tmp_path / "t.json"))
        assert rep["best"]["sparse.brick"] in tune.BRICKS and tune.populate_brick() == rep["best"]["sparse.brick"]
        again = tune.autotune_populate((96, 96, 96), _spheres(8, seed=3), cache=str(tmp_path / "t.json"))
        assert again["cached"] and again["best"] == rep["best"]
    finally:
        tune.set_populate_brick(old)


def test_sparse_mc_retries_when_buffers_are_small():
    vals = sphere((40, 40, 40), 0.6)
    ids, cv = sparse_from_dense(vals, extra=200, seed=1)
    g = make_sparse((40, 40, 40), ids, cv)
    v0, f0 = iso.marching_cubes(g)
    g._mc_sizes = {(g.get_num_cells(), 0.0, 0): (4, 4)}
    v1, f1 = iso.marching_cubes(g)
    assert torch.equal(v0, v1) and torch.equal(f0, f1)
    g._mc_sizes = {(g.get_num_cells(), 0.0, 0): (4, len(f0))}  # faces fit, vertices do not
    v2, f2 = iso.marching_cubes(g)
    assert torch.equal(v0, v2) and torch.equal(f0, f2)


def test_sparse_mc_weld_overflow_reports_a_vertex_count_that_fits():
    """A vertex capacity far below the mesh's: the weld's table (sized from it)
    fills, the call reports ISO_ERR_OVERFLOW with a vertex count at least the
    true one, and a rerun sized from that count gives the mesh."""
    import ctypes as C

    from isoext_gb300 import _ffi
    from isoext_gb300.sparse import _p, _stream

    vals = torus((40, 44, 36), 0.5, 0.2)
    ids, cv = sparse_from_dense(vals, extra=300, seed=2)
    g = make_sparse(vals.shape, ids, cv)
    v0, f0 = iso.marching_cubes(g)
    lib = _ffi.lib()
    n = g.get_num_cells()
    sx, sy, sz, lo, hi = g._geom()

    def run(cap_v, cap_f):
        vout = torch.empty((cap_v, 3), dtype=torch.float32, device="cuda")
        fout = torch.empty((cap_f, 3), dtype=torch.int32, device="cuda")
        ws = torch.empty(int(lib.iso_sparse_mc_workspace_size(n, cap_v, cap_f)), dtype=torch.uint8, device="cuda")
        small = torch.zeros(4, dtype=torch.int64, device="cuda")
        _ffi.check(lib.iso_sparse_mc(_p(g._ids), _p(g._values), n, sx, sy, sz, lo, hi, 0.0, 0, _p(vout), cap_v,
                                     _p(fout), cap_f, _p(ws), ws.numel(), _p(small),
                                     C.c_void_p(small.data_ptr() + 24), _stream(torch.device("cuda"))))
        h = small.cpu()
        return vout, fout, int(h[0]), int(h[1]), int(h[3] & 0xFFFFFFFF)

    cap_f = len(f0) + 16
    _, _, V, _, status = run(16, cap_f)
    assert status == _ffi.ISO_ERR_OVERFLOW
    assert V >= len(v0)
    vout, fout, V1, F1, status1 = run(V, cap_f)
    assert status1 == 0 and V1 == len(v0) and F1 == len(f0)
    assert torch.equal(vout[:V1], v0) and torch.equal(fout[:F1], f0)
