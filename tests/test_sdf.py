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
