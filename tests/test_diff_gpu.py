"""Differentiable extraction on the GPU: the forward results equal the plain
functions' bit for bit, and the backward kernels' gradients of a loss on the
vertices match the FP64 autograd reference (tests/grad_ref.py) and FP64 central
finite differences, on a 32^3 crop of the |p| - 0.6 + Fourier-features field."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from grad_ref import dc_crossed, dc_duals, mc_vertices, sphere_loss  # noqa: E402
from helpers import axis_coords, fourier_sphere, grid_points  # noqa: E402

FULL = 256
I0 = (190, 112, 112)  # the crop's first point in the 256^3 grid over [-1, 1]^3


def _crop(seed=1):
    ax = axis_coords(FULL)
    lo = tuple(float(ax[i]) for i in I0)
    hi = tuple(float(ax[i + 31]) for i in I0)
    return fourier_sphere(grid_points((32, 32, 32), lo, hi), seed), lo, hi


def _grad(fn, vals, lo, hi):
    x = torch.from_numpy(vals).cuda().requires_grad_(True)
    v, f = fn(x, lo, hi)
    sphere_loss(v).backward()
    return v.detach(), f, x.grad.double().cpu()


def _fd(loss_of, vals64, idx, eps=1e-6):
    flat = vals64.reshape(-1)
    out = []
    for i in idx:
        up, dn = flat.clone(), flat.clone()
        up[i] += eps
        dn[i] -= eps
        out.append(float(loss_of(up.reshape(vals64.shape)) - loss_of(dn.reshape(vals64.shape))) / (2 * eps))
    return np.array(out)


def test_mc_forward_equals_plain_marching_cubes():
    import isoext_gb300 as iso
    from isoext_gb300 import diff

    vals, lo, hi = _crop()
    grid = iso.UniformGrid([32] * 3, lo, hi)
    grid.set_values(torch.from_numpy(vals).cuda())
    v0, f0 = iso.marching_cubes(grid)
    v1, f1 = diff.marching_cubes(torch.from_numpy(vals).cuda(), lo, hi)
    assert torch.equal(v0, v1) and torch.equal(f0, f1)


def test_mc_gradient_matches_fp64_reference_and_finite_differences():
    from isoext_gb300 import diff

    vals, lo, hi = _crop()
    v, f, g = _grad(diff.marching_cubes, vals, lo, hi)
    _, _, e = diff._mc_forward(torch.from_numpy(vals).cuda(), lo, hi, 0.0, 0)
    x64 = torch.from_numpy(vals).double().requires_grad_(True)
    vr = mc_vertices(x64, e.cpu(), lo, hi)
    h = (hi[0] - lo[0]) / 31
    assert (vr.detach() - v.cpu().double()).abs().max() <= 1e-6 * h + 4 * np.spacing(np.float32(1.0))
    sphere_loss(vr).backward()
    gr = x64.grad
    scale = float(gr.abs().max())
    assert scale > 0
    assert float((g - gr).abs().max()) <= 1e-4 * scale
    nz = torch.nonzero(gr.reshape(-1)).reshape(-1).numpy()
    idx = np.random.default_rng(0).choice(nz, 24, replace=False)
    base = torch.from_numpy(vals).double()
    fd = _fd(lambda x: sphere_loss(mc_vertices(x, e.cpu(), lo, hi)), base, idx)
    assert np.abs(fd - g.reshape(-1)[idx].numpy()).max() <= 2e-4 * scale
    # values that feed no vertex get no gradient
    assert float(g.reshape(-1)[gr.reshape(-1) == 0].abs().max()) == 0.0


def test_dc_forward_equals_plain_dual_contouring():
    import isoext_gb300 as iso
    from isoext_gb300 import diff

    vals, lo, hi = _crop()
    grid = iso.UniformGrid([32] * 3, lo, hi)
    grid.set_values(torch.from_numpy(vals).cuda())
    v0, f0 = iso.dual_contouring(grid)
    v1, f1 = diff.dual_contouring(torch.from_numpy(vals).cuda(), lo, hi)
    assert torch.equal(v0, v1) and torch.equal(f0, f1)


def test_dc_gradient_matches_fp64_reference_and_finite_differences():
    from isoext_gb300 import diff

    vals, lo, hi = _crop()
    v, f, g = _grad(diff.dual_contouring, vals, lo, hi)
    _, _, cells, offs, src = diff._dc_forward(torch.from_numpy(vals).cuda(), lo, hi, 0.0, 1e-2, 1e-6)
    cells, offs, src = cells.cpu().long(), offs.cpu().long(), src.cpu().long()
    base = torch.from_numpy(vals).double()
    crossed = dc_crossed(base, cells)
    assert torch.equal(crossed.sum(1), offs[1:] - offs[:-1])
    x64 = base.clone().requires_grad_(True)
    vr = dc_duals(x64, cells, crossed, lo, hi)[src]
    # The kernel accumulates the QEF in FP32 as the reference does (src/dc.cu:26-62);
    # the FP64 restatement is exact.  With tangential eigenvalues equal to reg, a
    # rounding of 6e-8 relative moves x by about 6e-8 * K * |x| / reg: 1.4e-5 for
    # K = 4, |x| = 0.6, reg = 0.01, whatever the cell size.
    assert float((vr.detach() - v.cpu().double()).abs().max()) <= 4e-5
    sphere_loss(vr).backward()
    gr = x64.grad
    scale = float(gr.abs().max())
    assert scale > 0
    err = float((g - gr).abs().max())
    assert err <= 2e-3 * scale, (err, scale)
    nz = torch.nonzero(gr.reshape(-1)).reshape(-1).numpy()
    idx = np.random.default_rng(1).choice(nz, 24, replace=False)
    fd = _fd(lambda x: sphere_loss(dc_duals(x, cells, crossed, lo, hi)[src]), base, idx)
    assert np.abs(fd - g.reshape(-1)[idx].numpy()).max() <= 2e-3 * scale


def test_empty_surface_gives_empty_tensors_and_zero_gradient():
    from isoext_gb300 import diff

    x = torch.ones((16, 16, 16), device="cuda", requires_grad=True)
    for fn in (diff.marching_cubes, diff.dual_contouring):
        v, f = fn(x)
        assert v.shape == (0, 3) and f.shape == (0, 3)
        v.sum().backward()
        assert float(x.grad.abs().max()) == 0.0
        x.grad = None


def test_batched_extraction_equals_one_by_one():
    """The batch entry points queue every grid before one synchronisation; the
    meshes and gradients are those of one call per grid."""
    from isoext_gb300 import diff

    grids = [_crop(seed)[0] for seed in (1, 2, 3)]
    _, lo, hi = _crop(1)
    xs = [torch.from_numpy(g).cuda().requires_grad_(True) for g in grids]
    mcs = diff.marching_cubes_batch(xs, lo, hi)
    dcs = diff.dual_contouring_batch(xs, lo, hi)
    sum(sphere_loss(v) for v, _ in mcs + dcs).backward()
    for g, x, (vm, fm), (vd, fd) in zip(grids, xs, mcs, dcs):
        y = torch.from_numpy(g).cuda().requires_grad_(True)
        vm1, fm1 = diff.marching_cubes(y, lo, hi)
        vd1, fd1 = diff.dual_contouring(y, lo, hi)
        (sphere_loss(vm1) + sphere_loss(vd1)).backward()
        assert torch.equal(vm, vm1) and torch.equal(fm, fm1) and torch.equal(vd, vd1) and torch.equal(fd, fd1)
        # atomics make the summation order vary: equal to FP32 rounding
        assert torch.allclose(x.grad, y.grad, rtol=1e-5, atol=1e-7 * float(y.grad.abs().max()))
