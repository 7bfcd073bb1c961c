"""Size-independent properties at the benchmark sizes, where the oracle is too
slow to compare mesh by mesh: a closed surface gives a closed 2-manifold with
the right Euler characteristic, one vertex per sign-changing grid edge, and
every vertex on its edge."""

import numpy as np
import pytest
import torch

import isoext_gb300 as iso

pytestmark = pytest.mark.gpu


def _sphere_grid(n, r):
    ax = torch.arange(n, device="cuda", dtype=torch.float32)
    c = ax / torch.tensor(float(n - 1), device="cuda") * torch.tensor(2.0, device="cuda") + torch.tensor(-1.0, device="cuda")
    x, y, z = c.view(-1, 1, 1), c.view(1, -1, 1), c.view(1, 1, -1)
    g = iso.UniformGrid([n] * 3)
    g.set_values((torch.sqrt((x * x + y * y) + z * z) - r).contiguous())
    return g


def _edges_crossed(vals, level=0.0):
    b = vals < level
    return int((b[1:] != b[:-1]).sum() + (b[:, 1:] != b[:, :-1]).sum() + (b[:, :, 1:] != b[:, :, :-1]).sum())


def _manifold(f):
    """(closed 2-manifold, Euler characteristic) of a triangle mesh."""
    f = f.long()
    e = torch.cat([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
    key = torch.minimum(e[:, 0], e[:, 1]) * (int(f.max()) + 1) + torch.maximum(e[:, 0], e[:, 1])
    _, counts = torch.unique(key, return_counts=True)
    V = int(torch.unique(f).numel())
    return bool((counts == 2).all()), V - len(counts) + len(f)


@pytest.mark.parametrize("n", [512, 700])
def test_mc_sphere_is_a_closed_genus_0_surface(n):
    g = _sphere_grid(n, 0.8)
    v, f = iso.marching_cubes(g)
    crossed = _edges_crossed(g._values)
    if int((g._values == 0).sum()) == 0:
        assert len(v) == crossed  # one vertex per crossed edge
    else:
        assert len(v) <= crossed  # vertices on grid points are shared
    closed, chi = _manifold(f)
    assert closed and chi == 2
    h = 2.0 / (n - 1)
    assert float((v.norm(dim=-1) - 0.8).abs().max()) < h  # on the surface to within a cell


def test_dc_sphere_at_512_is_closed():
    g = _sphere_grid(512, 0.8)
    v, f = iso.dual_contouring(g)
    closed, chi = _manifold(f)
    assert closed and chi == 2
    assert float((v.norm(dim=-1) - 0.8).abs().max()) < 2 * 2.0 / 511  # within its cell (diagonal < 2 h)


def test_sparse_surface_cells_give_the_dense_mesh_at_1024():
    """populate(mode='surface') keeps the cells the surface crosses, so sparse MC
    over them is the dense mesh (same positions, same faces up to vertex order)."""
    n = 1024

    def sdf(p):
        return torch.sqrt((p[..., 0] * p[..., 0] + p[..., 1] * p[..., 1]) + p[..., 2] * p[..., 2]) - 0.7

    sg = iso.SparseGrid([n] * 3)
    sg.populate(sdf, mode="surface", brick=8)
    vs, fs = iso.marching_cubes(sg)
    from isoext_gb300.grids import grid_positions

    ax = grid_positions(torch.arange(n, device="cuda"), n, -1.0, 1.0)  # the lattice's FP32 coordinates
    x, y, z = ax.view(-1, 1, 1), ax.view(1, -1, 1), ax.view(1, 1, -1)
    dg = iso.UniformGrid([n] * 3)
    dg.set_values((torch.sqrt((x * x + y * y) + z * z) - 0.7).contiguous())  # sdf's arithmetic, broadcast
    vd, fd = iso.marching_cubes(dg)
    assert vs.shape == vd.shape and fs.shape == fd.shape
    # same vertex set (bit-equal positions) and the same faces after relabelling
    bits_s = vs.view(torch.int32).cpu().numpy().view(np.dtype((np.void, 12))).ravel()
    bits_d = vd.view(torch.int32).cpu().numpy().view(np.dtype((np.void, 12))).ravel()
    order = np.argsort(bits_d)
    pos = np.searchsorted(bits_d[order], bits_s)
    assert (bits_d[order][np.clip(pos, 0, len(bits_d) - 1)] == bits_s).all()
    perm = torch.from_numpy(order[pos]).cuda()
    assert torch.equal(perm[fs.long()], fd.long())
