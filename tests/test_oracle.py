"""The oracle is pinned before it is trusted: against fixtures produced by the
reference's own code (tests/golden) and against the counts published in the
reference's notebooks (doc/*.ipynb)."""

import glob
import os

import numpy as np
import pytest
import torch

from helpers import assert_same_mesh, grid_points, sphere

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
DENSE = sorted(p for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
               if not os.path.basename(p).startswith(("sparse", "cuboid", "sdf_", "luts")))


@pytest.mark.parametrize("path", DENSE, ids=lambda p: os.path.basename(p)[:-4])
@pytest.mark.parametrize("method", ["nagae", "lorensen"])
def test_oracle_mc_matches_reference_fixture(host_oracle, path, method):
    g = np.load(path)
    v, f, _ = host_oracle.mc_dense(g["values"], level=float(g["level"]), method=method)
    # The oracle also welds like the reference, so even the vertex order matches.
    assert np.array_equal(v, g[f"mc_{method}_v"])
    assert np.array_equal(f, g[f"mc_{method}_f"])


@pytest.mark.parametrize("name", ["sphere20", "torus24", "aniso"])
def test_oracle_intersection_and_dc_match_reference_fixture(host_oracle, name):
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    its = host_oracle.intersection_dense(g["values"], level=float(g["level"]), normals=True)
    for k in ["points", "normals", "edges", "is_out", "cell_indices", "cell_offsets"]:
        assert np.array_equal(its[k], g[f"its_{k}"]), k
    v, f, _ = host_oracle.dc_dense(g["values"], level=float(g["level"]))
    assert np.array_equal(v, g["dc_v"]) and np.array_equal(f, g["dc_f"])


def test_oracle_dc_cuboid_fixture(host_oracle):
    g = np.load(os.path.join(GOLDEN, "cuboid24.npz"))
    v, f, _ = host_oracle.dc_dense(g["values"])
    assert np.array_equal(v, g["dc_v"]) and np.array_equal(f, g["dc_f"])


@pytest.mark.parametrize("method", ["nagae", "lorensen"])
def test_oracle_sparse_fixture(host_oracle, method):
    g = np.load(os.path.join(GOLDEN, "sparse16.npz"))
    shape = tuple(int(x) for x in g["shape"])
    v, f, _ = host_oracle.mc_sparse(g["cell_ids"], g["values"], shape, method=method)
    assert np.array_equal(v, g[f"mc_{method}_v"]) and np.array_equal(f, g[f"mc_{method}_f"])
    its = host_oracle.intersection_sparse(g["cell_ids"], g["values"], shape)
    v, f, _ = host_oracle.dc(its, shape, values=g["values"], cell_ids=g["cell_ids"])
    assert np.array_equal(v, g["dc_v"]) and np.array_equal(f, g["dc_f"])


# --- known answers from the reference's notebooks (run on its CUDA build), in
# both readings of its arithmetic -------------------------------------------

def _torch_points(n):
    return torch.from_numpy(grid_points((n, n, n)))


def test_known_answer_sphere64(oracle):
    # doc/marching_cubes.ipynb: 64^3, |p| - 0.7 -> V 9168, F 18332 (both tables)
    vals = (_torch_points(64).norm(dim=-1) - 0.7).numpy()
    for m in ["nagae", "lorensen"]:
        v, f, _ = oracle.mc_dense(vals, method=m)
        assert (len(v), len(f)) == (9168, 18332)
    # levels -0.2 / +0.2 -> 4728 / 15072 vertices
    assert len(oracle.mc_dense(vals, level=-0.2)[0]) == 4728
    assert len(oracle.mc_dense(vals, level=0.2)[0]) == 15072


def test_known_answer_gyroid64(oracle):
    # doc/grids.ipynb: gyroid, scale 6 -> 38760 vertices
    p = _torch_points(64) * 6.0
    x, y, z = p[..., 0], p[..., 1], p[..., 2]
    g = torch.sin(x) * torch.cos(y) + torch.sin(y) * torch.cos(z) + torch.sin(z) * torch.cos(x)
    v, f, _ = oracle.mc_dense(g.numpy())
    assert len(v) == 38760


def test_known_answer_occupancy(oracle):
    # doc/occupancy_grids.ipynb: binary occupancy at level 0.5 -> 9168 / 18332
    occ = ((_torch_points(64).norm(dim=-1) - 0.7) < 0).float()
    v, f, _ = oracle.mc_dense(occ.numpy(), level=0.5)
    assert (len(v), len(f)) == (9168, 18332)
    from isoext_gb300.utils import gaussian_smooth

    sm = gaussian_smooth(occ, sigma=5.0)
    v, f, _ = oracle.mc_dense(sm.numpy(), level=0.5)
    assert (len(v), len(f)) == (8232, 16460)


def test_known_answer_dc_cuboid64(oracle):
    # doc/dual_contouring.ipynb: cuboid 1.0 on 64^3 -> K 24576, V 6146, F 12288
    p = _torch_points(64)
    q = p.abs() - 0.5
    d = torch.clamp(q, min=0).norm(dim=-1) + torch.clamp(q.max(dim=-1).values, max=0)
    its = oracle.intersection_dense(d.numpy())
    assert len(its["points"]) == 24576
    v, f, _ = oracle.dc_dense(d.numpy())
    assert (len(v), len(f)) == (6146, 12288)


def test_known_answer_config1_sphere128(oracle):
    # the 128^3 sphere |p| - 0.8 used as the first benchmark configuration
    v, f, _ = oracle.mc_dense(sphere((128,) * 3, 0.8))
    assert (len(v), len(f)) == (48576, 97148)


def test_oracle_matches_reference_build_random(host_oracle, reference):
    # random fields with exact zeros, both tables, compared with the reference's
    # own code compiled for the host (skipped where that build is unavailable)
    from helpers import noise

    for seed in range(3):
        vals = noise((10, 11, 9), seed=seed, zero_frac=0.25)
        for m in ["nagae", "lorensen"]:
            v, f, _ = host_oracle.mc_dense(vals, method=m)
            rv, rf = reference.mc_dense(vals, method=m)
            assert np.array_equal(v, rv) and np.array_equal(f, rf)
            assert_same_mesh(v, f, rv, rf)
