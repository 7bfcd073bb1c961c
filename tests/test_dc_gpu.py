"""Intersections and dual contouring on the GPU against the oracle.

Intersections (points, normals, active cells, offsets) must equal the
reference's bit for bit.  Dual-contouring vertices come from a 3x3 solve: the
oracle solves in FP64, this path in FP32 refined with an FP64 residual, and
positions must agree within 1e-4 * h (h = smallest cell size).  Faces must
match quad by quad; a quad may use the other diagonal only where its two
diagonals are equally long within that tolerance.

Tests with the ``oracle`` fixture run in both readings of isoext's FP32
arithmetic (its CUDA build's, the default, and its host build's); the golden
fixtures come from the host build and are compared in that reading.
"""

import os

import numpy as np
import pytest
import torch

import isoext_gb300 as iso
from helpers import grid_points, noise, sphere, torus

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def make_grid(values, lo=(-1, -1, -1), hi=(1, 1, 1)):
    g = iso.UniformGrid(values.shape, lo, hi)
    g.set_values(torch.from_numpy(np.ascontiguousarray(values)).cuda())
    return g


def cell_h(shape, lo=(-1, -1, -1), hi=(1, 1, 1)):
    return min((hi[k] - lo[k]) / (shape[k] - 1) for k in range(3))


def assert_dc_match(v, f, vo, fo, h, what=""):
    v = np.asarray(v, np.float64)
    vo = np.asarray(vo, np.float64)
    f = np.asarray(f, np.int64)
    fo = np.asarray(fo, np.int64)
    tol = 1e-4 * h
    assert f.shape == fo.shape, f"{what}: F {len(f)} vs {len(fo)}"
    assert v.shape == vo.shape, f"{what}: V {len(v)} vs {len(vo)}"
    # vertex map by nearest position
    from scipy.spatial import cKDTree

    d, perm = cKDTree(vo).query(v)
    assert d.max() <= tol, f"{what}: max vertex error {d.max() / h:.3g} h"
    assert len(np.unique(perm)) == len(perm), f"{what}: vertex map not a bijection"
    m = perm[f]
    for q in range(len(f) // 2):
        t0, t1 = tuple(m[2 * q]), tuple(m[2 * q + 1])
        r0, r1 = tuple(fo[2 * q]), tuple(fo[2 * q + 1])
        if (t0, t1) == (r0, r1):
            continue
        a0, a1, a2 = t0
        b2 = t1[2]
        alt = {(b2, a2, a0), (a2, b2, a1)}
        assert {r0, r1} == alt, f"{what}: quad {q} differs: {t0, t1} vs {r0, r1}"
        dd = abs(np.linalg.norm(vo[a2] - vo[b2]) - np.linalg.norm(vo[a0] - vo[a1]))
        assert dd <= 4 * tol, f"{what}: quad {q} split differs with diagonals {dd / h:.3g} h apart"


def check_dc(oracle, values, level=0.0, lo=(-1, -1, -1), hi=(1, 1, 1), what=""):
    g = make_grid(values, lo, hi)
    v, f = iso.dual_contouring(g, level=level)
    vo, fo, _ = oracle.dc_dense(values, lo, hi, level)
    if v is None:
        assert len(fo) == 0, what
        return
    assert_dc_match(v.cpu().numpy(), f.cpu().numpy(), vo, fo, cell_h(values.shape, lo, hi), what)


@pytest.mark.parametrize("name", ["sphere20", "torus24", "aniso"])
def test_intersection_matches_reference_fixture(name, host_arith):
    gd = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    g = make_grid(gd["values"])
    its = iso.get_intersection(g, level=float(gd["level"]), compute_normals=True)
    assert its.has_normals()
    assert np.array_equal(its.get_points().cpu().numpy(), gd["its_points"])
    assert np.array_equal(its.get_normals().cpu().numpy(), gd["its_normals"])
    assert np.array_equal(its._cells.cpu().numpy().astype(np.uint32), gd["its_cell_indices"])
    assert np.array_equal(its._offsets.cpu().numpy().astype(np.uint32), gd["its_cell_offsets"])


@pytest.mark.parametrize("shape,r", [((32, 32, 32), 0.5), ((45, 37, 61), 0.6), ((64, 64, 64), 0.7),
                                     ((16, 32, 48), 0.5), ((8, 64, 16), 0.5)])
def test_intersection_matches_oracle(oracle, shape, r):
    vals = sphere(shape, r, center=(0.05, -0.03, 0.02))
    g = make_grid(vals)
    for normals in (False, True):
        its = iso.get_intersection(g, compute_normals=normals)
        ref = oracle.intersection_dense(vals, normals=normals)
        assert np.array_equal(its.get_points().cpu().numpy(), ref["points"])
        if normals:
            assert np.array_equal(its.get_normals().cpu().numpy(), ref["normals"])
        else:
            assert not its.has_normals()
        assert np.array_equal(its._offsets.cpu().numpy().astype(np.uint32), ref["cell_offsets"])


@pytest.mark.parametrize("name", ["sphere20", "torus24", "aniso"])
def test_dc_matches_reference_fixture(name, host_arith):
    gd = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    g = make_grid(gd["values"])
    v, f = iso.dual_contouring(g, level=float(gd["level"]))
    assert_dc_match(v.cpu().numpy(), f.cpu().numpy(), gd["dc_v"], gd["dc_f"], cell_h(gd["values"].shape), name)


def test_dc_cuboid_fixture(host_arith):
    gd = np.load(os.path.join(GOLDEN, "cuboid24.npz"))
    g = make_grid(gd["values"])
    v, f = iso.dual_contouring(g)
    assert_dc_match(v.cpu().numpy(), f.cpu().numpy(), gd["dc_v"], gd["dc_f"], cell_h((24, 24, 24)), "cuboid")


@pytest.mark.parametrize("shape,r", [((32, 32, 32), 0.5), ((48, 40, 56), 0.6), ((96, 96, 96), 0.7),
                                     ((16, 32, 48), 0.5), ((8, 64, 16), 0.5)])
def test_dc_sphere(oracle, shape, r):
    check_dc(oracle, sphere(shape, r, center=(0.02, 0.01, -0.03)), what=f"sphere {shape}")


def test_dc_levels_torus(oracle):
    vals = torus((48, 48, 48), 0.5, 0.2)
    for lvl in (-0.05, 0.0, 0.05):
        check_dc(oracle, vals, level=lvl, what=f"torus {lvl}")


def test_dc_known_answer_cuboid64(oracle):
    # doc/dual_contouring.ipynb: cuboid 1.0 on 64^3 -> K 24576, V 6146, F 12288
    p = torch.from_numpy(grid_points((64, 64, 64)))
    q = p.abs() - 0.5
    d = (torch.clamp(q, min=0).norm(dim=-1) + torch.clamp(q.max(dim=-1).values, max=0)).numpy()
    g = make_grid(d)
    its = iso.get_intersection(g)
    assert its.get_points().shape == (24576, 3)
    v, f = iso.dual_contouring(g)
    assert v.shape == (6146, 3) and f.shape == (12288, 3)
    vo, fo, _ = oracle.dc_dense(d)
    assert_dc_match(v.cpu().numpy(), f.cpu().numpy(), vo, fo, cell_h((64,) * 3), "cuboid64")


def test_dc_custom_normals(oracle):
    # isoext's documented flow: intersection -> analytic normals -> DC
    vals = sphere((40, 40, 40), 0.6)
    g = make_grid(vals)
    its = iso.get_intersection(g)
    pts = its.get_points()
    n = torch.nn.functional.normalize(pts, dim=-1).contiguous()
    its.set_normals(n)
    v, f = iso.dual_contouring(g, intersection=its)
    ref = oracle.intersection_dense(vals, normals=False)
    ref["normals"] = n.cpu().numpy()
    vo, fo, _ = oracle.dc(ref, vals.shape, values=vals)
    assert_dc_match(v.cpu().numpy(), f.cpu().numpy(), vo, fo, cell_h((40,) * 3), "custom normals")
    # the intersection is not consumed: a second call gives the same mesh
    v2, f2 = iso.dual_contouring(g, intersection=its)
    assert torch.equal(v, v2) and torch.equal(f, f2)


def test_dc_intersection_without_normals(oracle):
    vals = torus((40, 40, 40), 0.5, 0.2)
    g = make_grid(vals)
    its = iso.get_intersection(g, compute_normals=False)
    v, f = iso.dual_contouring(g, intersection=its)
    vo, fo, _ = oracle.dc_dense(vals)
    assert_dc_match(v.cpu().numpy(), f.cpu().numpy(), vo, fo, cell_h((40,) * 3), "auto normals later")


def test_dc_reg_and_tol(oracle):
    vals = sphere((36, 36, 36), 0.55)
    g = make_grid(vals)
    for reg, tol in [(1e-1, 1e-6), (1e-3, 1e-6), (1e-2, 1e-2)]:
        v, f = iso.dual_contouring(g, reg=reg, svd_tol=tol)
        vo, fo, _ = oracle.dc_dense(vals, reg=reg, svd_tol=tol)
        assert_dc_match(v.cpu().numpy(), f.cpu().numpy(), vo, fo, cell_h((36,) * 3), f"reg {reg} tol {tol}")


def test_dc_empty():
    g = make_grid(np.ones((10, 10, 10), np.float32))
    assert iso.dual_contouring(g) == (None, None)
    its = iso.get_intersection(g)
    assert its.get_points().shape == (0, 3)


def test_intersection_set_normals_checks():
    g = make_grid(sphere((16, 16, 16), 0.5))
    its = iso.get_intersection(g)
    with pytest.raises(TypeError):
        its.set_normals(torch.zeros((3, 3)))
    with pytest.raises(RuntimeError, match="different shapes"):
        its.set_normals(torch.zeros((3, 3), device="cuda"))


@pytest.mark.parametrize("values", ["sphere", "noise"])
def test_dc_one_pass_solve_equals_intersection_then_solve(values):
    """dual_contouring(grid) solves each cell without writing the intersection;
    it must give the bits of get_intersection(normals) -> dual_contouring(its)."""
    vals = sphere((41, 37, 45), 0.55) if values == "sphere" else noise((24, 30, 33), seed=4)
    g = make_grid(vals)
    v0, f0 = iso.dual_contouring(g)
    its = iso.get_intersection(g, compute_normals=True)
    v1, f1 = iso.dual_contouring(g, intersection=its)
    assert torch.equal(v0, v1) and torch.equal(f0, f1)


def test_dc_one_call_retries_when_buffers_are_small():
    """dual_contouring sizes its buffers from the last call; when they are too
    small the device reports the sizes and the call reruns with them."""
    from isoext_gb300 import dc

    vals = sphere((48, 50, 52), 0.7)
    g = make_grid(vals)
    v0, f0 = iso.dual_contouring(g)
    key = (tuple(g.shape), 0.0, tuple(g.aabb_min), tuple(g.aabb_max))
    dc._dc_sizes[key] = (8, 8)
    v1, f1 = iso.dual_contouring(g)
    assert torch.equal(v0, v1) and torch.equal(f0, f1)
    assert dc._dc_sizes[key][0] >= len(v0)


def _cuboid_sdf(shape, half=0.5, lo=(-1, -1, -1), hi=(1, 1, 1)):
    p = torch.from_numpy(grid_points(shape, lo, hi)).double()
    c = torch.tensor([(lo[k] + hi[k]) / 2 for k in range(3)], dtype=torch.float64)
    q = (p - c).abs() - half * torch.tensor([(hi[k] - lo[k]) / 2 for k in range(3)], dtype=torch.float64)
    return (torch.clamp(q, min=0).norm(dim=-1) + torch.clamp(q.max(dim=-1).values, max=0)).float().numpy()


@pytest.mark.parametrize("case", ["cuboid", "zeros", "repeated_coords"])
def test_dc_one_call_weld_equals_hash_weld(case):
    """The one-call path welds a dual vertex that lies on a face of its cell by
    comparing it with the cells around that face; the call sequence hashes every
    position.  Both must give the same bits: on a cuboid whose vertices clip to
    cell faces, on noise with exact zeros (crossings on grid points), and on a
    grid finer than FP32 resolves at its coordinates (coordinates repeat, so
    more than the neighbouring cells share a face position)."""
    lo, hi = (-1, -1, -1), (1, 1, 1)
    if case == "cuboid":
        vals = _cuboid_sdf((33, 29, 31))
    elif case == "zeros":
        vals = noise((26, 22, 30), seed=9, zero_frac=0.3)
    else:
        lo, hi = (1000.0, -1.0, 1000.0), (1000.001, 1.0, 1000.002)
        vals = _cuboid_sdf((24, 20, 28), 0.6, lo, hi)
    g = make_grid(vals, lo, hi)
    v0, f0 = iso.dual_contouring(g)
    its = iso.get_intersection(g, compute_normals=True)
    v1, f1 = iso.dual_contouring(g, intersection=its)
    assert v0 is not None and len(f0) > 0
    assert torch.equal(v0, v1) and torch.equal(f0, f1)
    if case == "repeated_coords":  # the grid does repeat coordinates, and the weld merged across them
        pts = g.get_points().reshape(-1, 3)
        assert len(torch.unique(pts[:, 0])) < g.shape[0]


@pytest.mark.parametrize("shape", [(2, 2, 2), (3, 3, 3), (2, 5, 33), (5, 3, 32), (37, 41, 128), (33, 29, 97)])
def test_dc_one_call_shapes(oracle, shape):
    """The one-call path numbers cells over the flat point-word bitmap, four words
    per lane with 16-byte loads when rows hold a multiple of 4 words (nz in
    97..128 here) and scalar loads otherwise; rows of one word (nz <= 33) and the
    smallest grids exercise the edges of that walk.  The mesh must equal the call
    sequence's bit for bit and the oracle's within the tolerance."""
    rng = np.random.default_rng(sum(shape))
    vals = sphere(shape, 0.45, center=(0.05, -0.02, 0.01)) if min(shape) > 3 else \
        rng.uniform(-1, 1, size=shape).astype(np.float32)
    g = make_grid(vals)
    v0, f0 = iso.dual_contouring(g)
    its = iso.get_intersection(g, compute_normals=True)
    v1, f1 = iso.dual_contouring(g, intersection=its)
    if v0 is None:
        assert v1 is None
        return
    assert torch.equal(v0, v1) and torch.equal(f0, f1)
    vo, fo, _ = oracle.dc_dense(vals)
    assert_dc_match(v0.cpu().numpy(), f0.cpu().numpy(), vo, fo, cell_h(shape), f"shape {shape}")
