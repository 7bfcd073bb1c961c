"""Test helpers: reference-exact grid coordinates, synthetic fields, mesh comparison."""

from __future__ import annotations

import numpy as np


def axis_coords(n: int, lo: float = -1.0, hi: float = 1.0) -> np.ndarray:
    """lo + (i / (float)(n - 1)) * (hi - lo), each step rounded in FP32."""
    i = np.arange(n, dtype=np.float32)
    size = np.float32(hi) - np.float32(lo)
    return (np.float32(lo) + (i / np.float32(n - 1)) * size).astype(np.float32)


def grid_points(shape, lo=(-1, -1, -1), hi=(1, 1, 1)) -> np.ndarray:
    ax = [axis_coords(shape[k], lo[k], hi[k]) for k in range(3)]
    X, Y, Z = np.meshgrid(*ax, indexing="ij")
    return np.stack([X, Y, Z], axis=-1)


def sphere(shape, r, lo=(-1, -1, -1), hi=(1, 1, 1), center=(0, 0, 0)) -> np.ndarray:
    p = grid_points(shape, lo, hi) - np.asarray(center, np.float32)
    return (np.sqrt((p * p).sum(-1)) - np.float32(r)).astype(np.float32)


def torus(shape, R, r) -> np.ndarray:
    p = grid_points(shape)
    q = np.sqrt(p[..., 0] ** 2 + p[..., 1] ** 2) - np.float32(R)
    return (np.sqrt(q * q + p[..., 2] ** 2) - np.float32(r)).astype(np.float32)


def noise(shape, seed: int, zero_frac: float = 0.0) -> np.ndarray:
    """Uniform noise in [-1, 1] with a fraction of exact zeros (exercises vertices
    that round onto grid points and degenerate triangles)."""
    g = np.random.default_rng(seed)
    v = g.uniform(-1, 1, size=shape).astype(np.float32)
    if zero_frac:
        v[g.random(shape) < zero_frac] = 0.0
    return v


def assert_same_mesh(v, f, vo, fo, what: str = "") -> None:
    """Bit-exact equality up to vertex order: every vertex position must appear in
    the other mesh with identical float bits, and the face index sequences must be
    identical after relabelling (same faces, same order, same corner order)."""
    v = np.asarray(v, np.float32).reshape(-1, 3)
    vo = np.asarray(vo, np.float32).reshape(-1, 3)
    f = np.asarray(f, np.int64).reshape(-1, 3)
    fo = np.asarray(fo, np.int64).reshape(-1, 3)
    assert v.shape == vo.shape, f"{what}: V {v.shape[0]} vs {vo.shape[0]}"
    assert f.shape == fo.shape, f"{what}: F {f.shape[0]} vs {fo.shape[0]}"
    if len(v) == 0:
        return
    vb = np.ascontiguousarray(v).view(np.dtype((np.void, 12))).ravel()
    vob = np.ascontiguousarray(vo).view(np.dtype((np.void, 12))).ravel()
    order = np.argsort(vob)
    pos = np.searchsorted(vob[order], vb)
    pos = np.clip(pos, 0, len(vo) - 1)
    found = vob[order][pos] == vb
    assert found.all(), f"{what}: {int((~found).sum())} vertices not in the other mesh"
    perm = order[pos]
    assert len(np.unique(perm)) == len(perm), f"{what}: vertex map is not a bijection"
    mapped = perm[f]
    bad = np.nonzero((mapped != fo).any(axis=1))[0]
    assert len(bad) == 0, f"{what}: {len(bad)} faces differ, first at {bad[:5]}"


def fourier_sphere(points: np.ndarray, seed: int, k: int = 32) -> np.ndarray:
    """|p| - 0.6 plus k random Fourier features a sin(w . p + phi), w ~ N(0, 3^2)
    per axis, a ~ N(0, 0.02^2), phi ~ U[0, 2 pi] (seeded); FP64, rounded to FP32."""
    g = np.random.default_rng(seed)
    w = g.normal(0.0, 3.0, size=(k, 3))
    a = g.normal(0.0, 0.02, size=k)
    phi = g.uniform(0.0, 2 * np.pi, size=k)
    p = np.asarray(points, np.float64)
    out = np.sqrt((p * p).sum(-1)) - 0.6
    for i in range(k):
        out += a[i] * np.sin(p @ w[i] + phi[i])
    return out.astype(np.float32)


def csg_shape(seed: int):
    """The dual-contouring benchmark's seeded CSG (an isoext_gb300.sdf callable on
    torch points): (box with half-extents U[0.3,0.6]) minus (sphere, r U[0.2,0.4]),
    unioned with (torus R U[0.3,0.5], r U[0.05,0.15]); centres U[-0.3,0.3]^3."""
    import torch

    from isoext_gb300 import sdf

    g = torch.Generator().manual_seed(seed)

    def u(lo, hi, k=1):
        return (lo + (hi - lo) * torch.rand(k, generator=g)).tolist()

    half = u(0.3, 0.6, 3)
    rs = u(0.2, 0.4)[0]
    big, small = u(0.3, 0.5)[0], u(0.05, 0.15)[0]
    c_box, c_sph, c_tor = u(-0.3, 0.3, 3), u(-0.3, 0.3, 3), u(-0.3, 0.3, 3)
    box = sdf.TranslationOp(sdf.CuboidSDF([2 * h for h in half]), c_box)
    hole = sdf.NegationOp(sdf.TranslationOp(sdf.SphereSDF(rs), c_sph))
    ring = sdf.TranslationOp(sdf.TorusSDF(big, small), c_tor)
    return sdf.UnionOp([sdf.IntersectionOp([box, hole]), ring])


def smoothmin_spheres(seed: int, spheres: int = 64, k: float = 0.05):
    """The sparse benchmark's field: smooth-min (k) union of seeded spheres,
    centres U[-0.7, 0.7]^3, radii U[0.05, 0.25] (an isoext_gb300.sdf callable)."""
    from isoext_gb300 import sdf as S

    rng = np.random.default_rng(seed)
    c = rng.uniform(-0.7, 0.7, size=(spheres, 3))
    r = rng.uniform(0.05, 0.25, size=spheres)
    return S.SmoothUnionOp([S.TranslationOp(S.SphereSDF(float(ri)), [float(x) for x in ci]) for ci, ri in zip(c, r)],
                           k)
