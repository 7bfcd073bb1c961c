"""set_vertex_order("position"): vertices numbered as isoext numbers them
(sorted by position, src/utils.cu:32-59), so the returned tensors equal the
reference's exactly -- not only after relabelling."""

import glob
import os

import numpy as np
import pytest
import torch

import isoext_gb300 as iso
from helpers import noise, sphere, torus

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
DENSE = sorted(p for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
               if not os.path.basename(p).startswith(("sparse", "cuboid", "sdf_", "luts")))


@pytest.fixture
def by_position():
    iso.set_vertex_order("position")
    yield
    iso.set_vertex_order("edge")


def _grid(values):
    g = iso.UniformGrid(values.shape)
    g.set_values(torch.from_numpy(np.ascontiguousarray(values, np.float32)).cuda())
    return g


@pytest.mark.parametrize("path", DENSE, ids=lambda p: os.path.basename(p)[:-4])
@pytest.mark.parametrize("method", ["nagae", "lorensen"])
def test_mc_tensors_equal_the_reference_fixture(path, method, by_position, host_arith):
    g = np.load(path)
    v, f = iso.marching_cubes(_grid(g["values"]), level=float(g["level"]), method=method)
    assert np.array_equal(v.cpu().numpy(), g[f"mc_{method}_v"])
    assert np.array_equal(f.cpu().numpy(), g[f"mc_{method}_f"])


def test_sparse_mc_tensors_equal_the_reference_fixture(by_position, host_arith):
    g = np.load(os.path.join(GOLDEN, "sparse16.npz"))
    sg = iso.SparseGrid(tuple(int(x) for x in g["shape"]))
    sg.add_cells(torch.from_numpy(g["cell_ids"]).cuda())
    sg.set_values(torch.from_numpy(g["values"]).cuda())
    for m in ("nagae", "lorensen"):
        v, f = iso.marching_cubes(sg, method=m)
        assert np.array_equal(v.cpu().numpy(), g[f"mc_{m}_v"]) and np.array_equal(f.cpu().numpy(), g[f"mc_{m}_f"])


@pytest.mark.parametrize("case", ["sphere", "torus", "noise"])
def test_mc_tensors_equal_the_oracle(case, by_position, oracle):
    vals = {"sphere": sphere((96, 80, 112), 0.7), "torus": torus((64, 64, 64), 0.5, 0.2),
            "noise": noise((33, 35, 37), seed=4, zero_frac=0.3)}[case]
    v, f = iso.marching_cubes(_grid(vals))
    vo, fo, _ = oracle.mc_dense(vals)  # the oracle welds as isoext does: sorted by position
    assert np.array_equal(v.cpu().numpy(), vo) and np.array_equal(f.cpu().numpy(), fo)


def test_dc_vertex_order_sorts_and_keeps_the_mesh(by_position):
    vals = sphere((48, 48, 48), 0.6)
    v, f = iso.dual_contouring(_grid(vals))
    iso.set_vertex_order("edge")
    ve, fe = iso.dual_contouring(_grid(vals))
    vn = v.cpu().numpy()
    keys = [tuple(r) for r in vn.tolist()]
    assert keys == sorted(keys)  # lexicographic by (x, y, z)
    # the same mesh: equal face sequences once both are written with positions
    assert np.array_equal(vn[f.cpu().numpy()], ve.cpu().numpy()[fe.cpu().numpy()])
