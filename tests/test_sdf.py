"""isoext_gb300.sdf against isoext's sdf module (src/isoext/sdf.py): values and
normals at seeded points equal the reference's (fixture written by
tests/golden/make_sdf_golden.py)."""

import os

import numpy as np
import pytest
import torch

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "sdf_cases.npz")

CASES = {
    "sphere": lambda m: m.SphereSDF(0.5),
    "torus": lambda m: m.TorusSDF(0.5, 0.2),
    "cuboid": lambda m: m.CuboidSDF([0.5, 0.7, 0.9]),
    "union": lambda m: m.UnionOp([m.SphereSDF(0.3), m.TranslationOp(m.CuboidSDF([0.4, 0.4, 0.4]), [0.2, 0.0, 0.0])]),
    "smooth_union": lambda m: m.SmoothUnionOp([m.SphereSDF(0.3), m.TranslationOp(m.SphereSDF(0.2), [0.3, 0.1, 0.0])], 0.05),
    "intersection": lambda m: m.IntersectionOp([m.SphereSDF(0.6), m.NegationOp(m.SphereSDF(0.3))]),
    "rotation": lambda m: m.RotationOp(m.TorusSDF(0.5, 0.1), [1.0, 1.0, 0.0], 30),
    "rotation_rad": lambda m: m.RotationOp(m.CuboidSDF([0.3, 0.6, 0.2]), [0.0, 0.0, 1.0], 0.4, use_degree=False),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_sdf_matches_reference(name):
    from isoext_gb300 import sdf

    g = np.load(GOLDEN)
    p = torch.from_numpy(g["points"])
    s = CASES[name](sdf)
    assert np.array_equal(s(p).numpy(), g[f"{name}_value"])
    n = sdf.get_sdf_normal(s, p.clone()).numpy()
    assert np.allclose(n, g[f"{name}_normal"], atol=1e-6, rtol=0)


def test_sdf_normal_leaves_input_untouched():
    from isoext_gb300 import sdf

    p = torch.rand(10, 3)
    sdf.get_sdf_normal(sdf.SphereSDF(0.5), p)
    assert not p.requires_grad


# tests/test_sdf_utils.py's cases (sphere radius 0.5, torus R=0.5 r=0.2, unit
# cuboid), on host tensors, with the exact gradients where they are known.


def test_sdf_grad_sphere_and_cuboid_point_outward():
    from isoext_gb300 import sdf

    p = torch.tensor([[0.0, 0.0, 0.0], [0.5, 0.0, 0.0], [1.0, 0.0, 0.0]])
    for s in (sdf.SphereSDF(radius=0.5), sdf.CuboidSDF(size=[1.0, 1.0, 1.0])):
        g = sdf.get_sdf_grad(s, p)
        assert g.shape == (3, 3)
        assert torch.norm(g[0]) < 1e-5  # the centre
        assert g[1, 0] > 0 and g[2, 0] > 0  # outward on and outside the surface
    g = sdf.get_sdf_grad(sdf.SphereSDF(radius=0.5), p)
    assert torch.equal(g[1:], torch.tensor([[1.0, 0.0, 0.0], [1.0, 0.0, 0.0]]))


def test_sdf_normals_are_unit_and_outward():
    from isoext_gb300 import sdf

    axes = torch.tensor([[0.5, 0.0, 0.0], [0.0, 0.5, 0.0], [0.0, 0.0, 0.5]])
    for s in (sdf.SphereSDF(radius=0.5), sdf.CuboidSDF(size=[1.0, 1.0, 1.0])):
        n = sdf.get_sdf_normal(s, axes.clone())
        assert n.shape == (3, 3)
        assert torch.allclose(n, torch.eye(3), atol=1e-6)
    torus = sdf.TorusSDF(R=0.5, r=0.2)
    assert sdf.get_sdf_grad(torus, torch.tensor([[0.5, 0.0, 0.0], [0.0, 0.0, 0.0]])).shape == (2, 3)
    n = sdf.get_sdf_normal(torus, torch.tensor([[0.6, 0.1, 0.0], [0.4, 0.1, 0.0], [0.5, 0.2, 0.0]]))
    assert torch.allclose(torch.norm(n, dim=-1), torch.ones(3), atol=1e-5)
    # in the ring's plane (z = 0; the torus lies around z) the normal is radial,
    # away from the tube's centre circle of radius 0.5
    for k, (x, y) in enumerate([(0.6, 0.1), (0.4, 0.1), (0.5, 0.2)]):
        rho = (x * x + y * y) ** 0.5
        sign = 1.0 if rho > 0.5 else -1.0
        assert torch.allclose(n[k], torch.tensor([sign * x / rho, sign * y / rho, 0.0]), atol=1e-6)


def test_sdf_normal_keeps_batch_shape():
    from isoext_gb300 import sdf

    p = torch.from_numpy(np.random.default_rng(5).standard_normal((2, 3, 3)).astype(np.float32))
    n = sdf.get_sdf_normal(sdf.SphereSDF(radius=0.5), p)
    assert n.shape == (2, 3, 3)
    assert torch.allclose(torch.norm(n, dim=-1), torch.ones(2, 3), atol=1e-5)
    assert torch.allclose(n, p / torch.norm(p, dim=-1, keepdim=True), atol=1e-6)
