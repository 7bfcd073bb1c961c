"""The FP64 gradient reference (tests/grad_ref.py) is pinned before it is used:
its positions agree with the oracle's, and its autograd gradients agree with
central finite differences of itself (no GPU)."""

import numpy as np
import pytest
import torch

from grad_ref import dc_crossed, dc_duals, mc_vertices, sphere_loss
from helpers import axis_coords, fourier_sphere, grid_points

N = 20
LO, HI = (0.1, 0.1, 0.1), (0.7, 0.66, 0.74)


@pytest.fixture(scope="module")
def crop():
    return fourier_sphere(grid_points((N, N, N), LO, HI), seed=3)


def _mc_edges(e, shape):
    nx, ny, nz = shape
    a, b = e[:, 0].astype(np.int64), e[:, 1].astype(np.int64)
    lo, hi = np.minimum(a, b), np.maximum(a, b)
    ax = np.select([hi - lo == ny * nz, hi - lo == nz], [0, 1], 2)
    return torch.from_numpy(3 * lo + ax)


def test_mc_reference_positions_match_oracle(oracle, crop):
    v, f, e = oracle.mc_dense(crop, LO, HI)
    assert len(f) > 100
    ref = mc_vertices(torch.from_numpy(crop).double(), _mc_edges(e, crop.shape), LO, HI).numpy()
    h = (HI[0] - LO[0]) / (N - 1)
    # the oracle rounds each lerp step to FP32: a few ulps of the coordinates
    assert np.abs(ref - v).max() <= 1e-6 * h + 4 * np.spacing(np.float32(max(HI)))


def test_dc_reference_duals_match_oracle(oracle, crop):
    its = oracle.intersection_dense(crop, LO, HI)
    _, _, d64 = oracle.dc(its, crop.shape, LO, HI, values=crop)
    cells = torch.from_numpy(its["cell_indices"].astype(np.int64))
    vals = torch.from_numpy(crop).double()
    crossed = dc_crossed(vals, cells)
    assert np.array_equal(crossed.sum(1).numpy(), np.diff(its["cell_offsets"].astype(np.int64)))
    ref = dc_duals(vals, cells, crossed, LO, HI).numpy()
    # the oracle's solutions are before clipping
    ax = [axis_coords(N, LO[k], HI[k]).astype(np.float64) for k in range(3)]
    c = its["cell_indices"].astype(np.int64)
    ci = [c // ((N - 1) ** 2), (c // (N - 1)) % (N - 1), c % (N - 1)]
    lo = np.stack([ax[k][ci[k]] for k in range(3)], -1)
    hi = np.stack([ax[k][ci[k] + 1] for k in range(3)], -1)
    want = np.minimum(np.maximum(d64, lo), hi)
    h = (HI[0] - LO[0]) / (N - 1)
    # The oracle accumulates the QEF in FP32 as the reference does (src/dc.cu:26-62);
    # the reference here is exact.  On a flat patch the tangential eigenvalues are
    # reg, so a rounding of 6e-8 relative in M or r moves x by about
    # 6e-8 * K * |x| / reg = 1e-3 h on this grid.
    assert np.abs(ref - want).max() <= 2e-3 * h


def _fd_check(loss_of, vals, idx, eps=1e-6):
    x = vals.clone().requires_grad_(True)
    loss_of(x).backward()
    g = x.grad.reshape(-1)
    flat = vals.reshape(-1)
    for i in idx:
        hi, lo = flat.clone(), flat.clone()
        hi[i] += eps
        lo[i] -= eps
        fd = (loss_of(hi.reshape(vals.shape)) - loss_of(lo.reshape(vals.shape))) / (2 * eps)
        assert abs(float(fd) - float(g[i])) <= 1e-6 * float(g.abs().max()) + 1e-12, (i, float(fd), float(g[i]))
    return g


def test_reference_autograd_matches_finite_differences(oracle, crop):
    vals = torch.from_numpy(crop).double()
    _, _, e = oracle.mc_dense(crop, LO, HI)
    edges = _mc_edges(e, crop.shape)
    rng = np.random.default_rng(0)
    g = _fd_check(lambda x: sphere_loss(mc_vertices(x, edges, LO, HI)), vals, [])
    nz = torch.nonzero(g).reshape(-1).numpy()
    _fd_check(lambda x: sphere_loss(mc_vertices(x, edges, LO, HI)), vals, rng.choice(nz, 12, replace=False))
    its = oracle.intersection_dense(crop, LO, HI)
    cells = torch.from_numpy(its["cell_indices"].astype(np.int64))
    crossed = dc_crossed(vals, cells)
    loss = lambda x: sphere_loss(dc_duals(x, cells, crossed, LO, HI))  # noqa: E731
    g = _fd_check(loss, vals, [])
    nz = torch.nonzero(g).reshape(-1).numpy()
    _fd_check(loss, vals, rng.choice(nz, 12, replace=False))
