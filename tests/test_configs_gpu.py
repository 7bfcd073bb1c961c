"""The benchmark configurations themselves against the oracle.

* Dual contouring of the 256^3 seeded CSG (box minus sphere, union torus):
  with normals from the grid, and with the analytic SDF normals handed over
  through Intersection.set_normals (isoext's documented flow).
* Dual contouring of the 512^3 sphere |p| - 0.8 (the metric's DC grid).
* Sparse marching cubes and dual contouring of the smooth-min union of 64
  seeded spheres (k = 0.05), cells of 8^3 bricks within 2 h of the surface, on
  a 256^3 lattice (the 1024^3 benchmark's field at a size the oracle checks in
  seconds).

Tolerances are the suite's: MC bit-exact after relabelling, intersections
bit-exact, DC vertices within 1e-4 * h of the oracle's FP64 solve with quads
matching (the other diagonal only where both diagonals are equal within that
tolerance).  Each runs in both readings of isoext's arithmetic (the oracle
fixture).
"""

import numpy as np
import pytest
import torch

import isoext_gb300 as iso
from helpers import assert_same_mesh, csg_shape, smoothmin_spheres
from test_dc_gpu import assert_dc_match, cell_h

pytestmark = pytest.mark.gpu


def _csg_grid(n, seed):
    shape = csg_shape(seed)
    g = iso.UniformGrid([n] * 3)
    g.set_values(shape(g.get_points()).contiguous())
    return g, shape


@pytest.mark.parametrize("seed", [7, 3])
def test_config2_csg_dc_with_grid_normals(oracle, seed):
    g, _ = _csg_grid(256, seed)
    v, f = iso.dual_contouring(g)
    vals = g.get_values().cpu().numpy()
    vo, fo, _ = oracle.dc_dense(vals)
    assert len(fo) > 100_000
    assert_dc_match(v.cpu().numpy(), f.cpu().numpy(), vo, fo, cell_h(vals.shape), f"csg {seed} grid normals")


@pytest.mark.parametrize("seed", [7, 3])
def test_config2_csg_dc_with_analytic_normals(oracle, seed):
    from isoext_gb300 import sdf

    g, shape = _csg_grid(256, seed)
    its = iso.get_intersection(g)
    normals = sdf.get_sdf_normal(shape, its.get_points()).contiguous()
    its.set_normals(normals)
    v, f = iso.dual_contouring(g, intersection=its)
    vals = g.get_values().cpu().numpy()
    ref = oracle.intersection_dense(vals, normals=False)
    assert np.array_equal(its.get_points().cpu().numpy(), ref["points"])  # same crossings, bit for bit
    ref["normals"] = normals.cpu().numpy()
    vo, fo, _ = oracle.dc(ref, vals.shape, values=vals)
    assert_dc_match(v.cpu().numpy(), f.cpu().numpy(), vo, fo, cell_h(vals.shape), f"csg {seed} analytic normals")


def test_dc_512_sphere_matches_oracle(oracle):
    n = 512
    g = iso.UniformGrid([n] * 3)
    p = g.get_points()
    g.set_values((torch.sqrt((p * p).sum(-1)) - 0.8).contiguous())
    del p
    v, f = iso.dual_contouring(g)
    vals = g.get_values().cpu().numpy()
    vo, fo, _ = oracle.dc_dense(vals)
    assert len(vo) == len(v) and len(fo) == len(f)
    assert_dc_match(v.cpu().numpy(), f.cpu().numpy(), vo, fo, cell_h(vals.shape), "sphere 512")


@pytest.fixture(scope="module")
def smoothmin_256():
    n = 256
    field = smoothmin_spheres(seed=0)
    sg = iso.SparseGrid([n] * 3)
    sg.populate(field, mode="brick", band=2 * 2.0 / (n - 1), brick=8)
    return sg


def test_config3_smoothmin_sparse_mc(oracle, smoothmin_256):
    sg = smoothmin_256
    ids = sg.get_cell_indices().cpu().numpy()
    vals = sg.get_values().cpu().numpy()
    assert 0.01 < len(ids) / 255 ** 3 < 0.5  # a band of whole bricks, not the lattice
    for method in ("nagae", "lorensen"):
        v, f = iso.marching_cubes(sg, method=method)
        vo, fo, _ = oracle.mc_sparse(ids, vals, sg.get_shape(), method=method)
        assert len(fo) > 100_000
        assert_same_mesh(v.cpu().numpy(), f.cpu().numpy(), vo, fo, f"smooth-min 256 {method}")


def test_config3_smoothmin_sparse_dc(oracle, smoothmin_256):
    sg = smoothmin_256
    ids = sg.get_cell_indices().cpu().numpy()
    vals = sg.get_values().cpu().numpy()
    shape = sg.get_shape()
    v, f = iso.dual_contouring(sg)
    its = oracle.intersection_sparse(ids, vals, shape)
    vo, fo, _ = oracle.dc(its, shape, values=vals, cell_ids=ids)
    assert_dc_match(v.cpu().numpy(), f.cpu().numpy(), vo, fo, cell_h(shape), "smooth-min 256 dc")
