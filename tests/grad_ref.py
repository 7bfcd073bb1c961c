"""FP64 PyTorch restatements of the vertex positions the differentiable forward
passes produce, given the topology the kernels found.  They are the reference
gradient (torch autograd) and the function finite differences are taken of.

* marching cubes: v = (1 - t) pa + t pb, t = (level - va) / (vb - va), for each
  vertex's edge (src/mc/nagae.cu:52-56, include/math.cuh:77-81);
* dual contouring: crossing points by the same lerp, normals from the cell's
  trilinear interpolant with the +-0.02 stencil clamped to [0.01, 0.99]
  (src/its.cu:170-268), the QEF normal equations with reg times the distance to
  the mean point (src/dc.cu:14-65), solved exactly (reg > 0 keeps the system
  regular), clipped to the cell (src/dc.cu:82-99).
Grid coordinates are the FP32 ones the kernels use, widened to FP64.
"""

from __future__ import annotations

import os
import sys

import numpy as np
import torch

from helpers import axis_coords

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "isoext_gb300", "csrc"))
from gen_luts import EDGE_PAIRS  # noqa: E402


def _coords(shape, lo, hi):
    return [torch.from_numpy(axis_coords(shape[k], lo[k], hi[k]).astype(np.float64)) for k in range(3)]


def mc_vertices(values: torch.Tensor, edges: torch.Tensor, lo, hi, level: float = 0.0) -> torch.Tensor:
    """Positions [V, 3] of the vertices on edges (3 * low point id + axis)."""
    nx, ny, nz = values.shape
    cx, cy, cz = _coords(values.shape, lo, hi)
    e = edges.long().cpu()
    ia, ax = e // 3, e % 3
    step = torch.tensor([ny * nz, nz, 1])[ax]
    flat = values.reshape(-1)
    va, vb = flat[ia], flat[ia + step]
    t = ((level - va) / (vb - va))[:, None]
    x, y, z = ia // (ny * nz), (ia // nz) % ny, ia % nz
    pa = torch.stack([cx[x], cy[y], cz[z]], -1)
    pb = torch.stack([cx[x + (ax == 0)], cy[y + (ax == 1)], cz[z + (ax == 2)]], -1)
    return (1 - t) * pa + t * pb


def _cell_corners(values, cells):
    nx, ny, nz = values.shape
    c = cells.long().cpu()
    cz = c % (nz - 1)
    r = c // (nz - 1)
    cy, cx = r % (ny - 1), r // (ny - 1)
    idx = []
    for j in range(8):
        x, y, z = cx + (j >> 2), cy + ((j >> 1) & 1), cz + (j & 1)
        idx.append((x * ny + y) * nz + z)
    return torch.stack(idx, -1), (cx, cy, cz)


def dc_crossed(values: torch.Tensor, cells: torch.Tensor, level: float = 0.0) -> torch.Tensor:
    """[A, 12] crossed edges of each active cell (the topology, kept fixed)."""
    idx, _ = _cell_corners(values, cells)
    c = values.detach().reshape(-1)[idx]
    below = (c - level) < 0
    return torch.stack([below[:, a] != below[:, b] for a, b in EDGE_PAIRS], -1)


def _trilin(c, t):
    """c [A, 8], t [A, 12, 3] -> [A, 12]."""
    out = 0
    for j in range(8):
        w = 1.0
        for a, bit in enumerate(((j >> 2) & 1, (j >> 1) & 1, j & 1)):
            w = w * (t[..., a] if bit else 1 - t[..., a])
        out = out + c[:, None, j] * w
    return out


def dc_duals(values: torch.Tensor, cells: torch.Tensor, crossed: torch.Tensor, lo, hi, level: float = 0.0,
             reg: float = 1e-2) -> torch.Tensor:
    """Clipped QEF solutions [A, 3] of the active cells, normals from the grid."""
    idx, (cx, cy, cz) = _cell_corners(values, cells)
    c = values.reshape(-1)[idx]  # [A, 8]
    X, Y, Z = _coords(values.shape, lo, hi)
    P = torch.stack([torch.stack([X[cx + (j >> 2)], Y[cy + ((j >> 1) & 1)], Z[cz + (j & 1)]], -1)
                     for j in range(8)], 1)  # [A, 8, 3]
    ca = [a for a, _ in EDGE_PAIRS]
    cb = [b for _, b in EDGE_PAIRS]
    va, vb = c[:, ca], c[:, cb]  # [A, 12]
    m = crossed.to(values.dtype)
    t = torch.where(crossed, (level - va) / torch.where(crossed, vb - va, torch.ones_like(va)), torch.zeros_like(va))
    p = (1 - t)[..., None] * P[:, ca] + t[..., None] * P[:, cb]  # [A, 12, 3]
    cmin, csz = P[:, 0], P[:, 7] - P[:, 0]
    tt = ((p - cmin[:, None]) / csz[:, None]).clamp(0.01, 0.99)
    d = []
    for a in range(3):
        tp, tm = tt.clone(), tt.clone()
        tp[..., a] = (tt[..., a] + 0.02).clamp(max=0.99)
        tm[..., a] = (tt[..., a] - 0.02).clamp(min=0.01)
        d.append((_trilin(c, tp) - _trilin(c, tm)) / ((tp[..., a] - tm[..., a]) * csz[:, None, a]))
    d = torch.stack(d, -1)
    ln = d.norm(dim=-1, keepdim=True)
    z = torch.tensor([0.0, 0.0, 1.0], dtype=values.dtype)
    n = torch.where(ln > 1e-8, d / ln.clamp(min=1e-30), z)
    K = m.sum(1)
    eye = torch.eye(3, dtype=values.dtype)
    M = torch.einsum("ak,aki,akj->aij", m, n, n) + reg * eye
    pm = (m[..., None] * p).sum(1) / K[:, None]
    r = torch.einsum("ak,aki,ak->ai", m, n, (n * p).sum(-1)) + reg * pm
    x = torch.linalg.solve(M, r)
    lo_c = P[:, 0]
    hi_c = P[:, 7]
    return torch.minimum(torch.maximum(x, lo_c), hi_c)


def sphere_loss(v: torch.Tensor) -> torch.Tensor:
    """Mean squared distance of the vertices to the unit sphere."""
    return ((v.norm(dim=-1) - 1.0) ** 2).mean()
