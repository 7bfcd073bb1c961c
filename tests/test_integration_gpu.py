"""The reference's integration tests (tests/test_integration.py:16-137), compared
with the oracle: composite SDFs built from the sdf module's primitives and
operators, evaluated on the grid's points, then extracted by marching cubes and
dual contouring.

The reference's tests check only the output shapes.  Here every mesh is
compared with the oracle on the same values: marching cubes bit for bit after
relabelling, dual contouring with vertices within 1e-4 of a cell of the
oracle's and the same quads.  Each test runs in both readings of isoext's FP32
arithmetic (the ``oracle`` fixture).
"""

import numpy as np
import pytest
import torch

import isoext_gb300 as iso
from isoext_gb300.sdf import (
    IntersectionOp,
    NegationOp,
    RotationOp,
    SphereSDF,
    TorusSDF,
    TranslationOp,
    UnionOp,
    get_sdf_normal,
)
from helpers import assert_same_mesh
from test_dc_gpu import assert_dc_match, cell_h

pytestmark = pytest.mark.gpu


def _holed_sphere():
    """A sphere with three orthogonal toroidal holes (tests/test_integration.py:18-22)."""
    torus_a = TorusSDF(R=0.75, r=0.15)
    torus_b = RotationOp(sdf=torus_a, axis=[1, 0, 0], angle=90)
    torus_c = RotationOp(sdf=torus_a, axis=[0, 1, 0], angle=90)
    sphere_a = SphereSDF(radius=0.75)
    return IntersectionOp([sphere_a, NegationOp(UnionOp([torus_a, torus_b, torus_c]))])


def _grid(sdf, res):
    g = iso.UniformGrid([res] * 3, aabb_min=[-1, -1, -1], aabb_max=[1, 1, 1])
    g.set_values(sdf(g.get_points()))
    return g, g.get_values().cpu().numpy()


def _mc(oracle, sdf, res, method="nagae"):
    g, vals = _grid(sdf, res)
    v, f = iso.marching_cubes(g, level=0.0, method=method)
    assert v is not None and v.shape[1] == 3 and f.shape[1] == 3 and len(f) > 0
    vo, fo, _ = oracle.mc_dense(vals, (-1, -1, -1), (1, 1, 1), 0.0, method)
    assert_same_mesh(v.cpu().numpy(), f.cpu().numpy(), vo, fo, f"{type(sdf).__name__} {res}")


@pytest.mark.parametrize("method", ["nagae", "lorensen"])
def test_complex_shape_marching_cubes(oracle, method):
    _mc(oracle, _holed_sphere(), 64, method)


def test_complex_shape_dual_contouring(oracle):
    g, vals = _grid(_holed_sphere(), 64)
    v, f = iso.dual_contouring(g, level=0.0)
    assert v.shape[1] == 3 and f.shape[1] == 3
    vo, fo, _ = oracle.dc_dense(vals)
    assert_dc_match(v.cpu().numpy(), f.cpu().numpy(), vo, fo, cell_h((64,) * 3), "holed sphere")


def test_complex_shape_dual_contouring_custom_normals(oracle):
    sdf = _holed_sphere()
    g, vals = _grid(sdf, 64)
    its = iso.get_intersection(g, level=0.0)
    points = its.get_points()
    assert len(points) > 0
    normals = get_sdf_normal(sdf, points)
    its.set_normals(normals)
    v, f = iso.dual_contouring(g, level=0.0, intersection=its)
    assert v.shape[1] == 3 and f.shape[1] == 3
    ref = oracle.intersection_dense(vals, normals=False)
    np.testing.assert_array_equal(ref["points"], points.cpu().numpy())
    ref["normals"] = normals.cpu().numpy()
    vo, fo, _ = oracle.dc(ref, vals.shape, values=vals)
    assert_dc_match(v.cpu().numpy(), f.cpu().numpy(), vo, fo, cell_h((64,) * 3), "holed sphere, SDF normals")


def test_multiple_spheres_union(oracle):
    spheres = [TranslationOp(SphereSDF(radius=0.3), offset=[x, 0.0, 0.0]) for x in (-0.5, 0.0, 0.5)]
    _mc(oracle, UnionOp(spheres), 48)


def test_nested_operations(oracle):
    union = UnionOp([SphereSDF(radius=0.4), TranslationOp(SphereSDF(radius=0.4), offset=[0.3, 0.0, 0.0])])
    _mc(oracle, IntersectionOp([union, SphereSDF(radius=0.5)]), 32)


def test_rotated_translated_shape(oracle):
    rotated = RotationOp(TorusSDF(R=0.5, r=0.2), axis=[1, 0, 0], angle=45)
    _mc(oracle, TranslationOp(rotated, offset=[0.3, 0.0, 0.0]), 32)


def test_make_grid_on_the_device():
    """tests/test_grid_utils.py:11-27 on the GPU: the grid's points as a
    [X, Y, Z, 3] tensor, corners at the box's corners."""
    from isoext_gb300.utils import make_grid

    grid = make_grid([-1, -1, -1, 1, 1, 1], res=32, device="cuda")
    assert grid.shape == (32, 32, 32, 3) and grid.device.type == "cuda"
    assert torch.equal(grid[0, 0, 0].cpu(), torch.tensor([-1.0, -1.0, -1.0]))
    assert torch.allclose(grid[-1, -1, -1].cpu(), torch.tensor([1.0, 1.0, 1.0]), atol=1e-5)
    assert make_grid([-1, -1, -1, 1, 1, 1], res=[16, 32, 64], device="cuda").shape == (16, 32, 64, 3)
