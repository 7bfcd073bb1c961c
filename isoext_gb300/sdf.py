"""Signed distance functions in torch, with isoext's names and formulas
(src/isoext/sdf.py): primitives, CSG operations and autograd normals.

These are plain torch expressions evaluated wherever the points live; they build
grids for the extraction functions and give analytic normals for
dual_contouring (isoext's documented flow: get_intersection -> get_sdf_normal
at the crossing points -> Intersection.set_normals).
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Protocol

import torch


class SDFProtocol(Protocol):
    def __call__(self, p: torch.Tensor) -> torch.Tensor: ...


def get_sdf_grad(sdf: SDFProtocol, p: torch.Tensor) -> torch.Tensor:
    """Gradient of sdf at points p [..., 3] (src/isoext/sdf.py:23-36)."""
    p = p.detach().requires_grad_(True)
    with torch.enable_grad():
        d = sdf(p)
        (g,) = torch.autograd.grad(d, p, grad_outputs=torch.ones_like(d))
    return g


def get_sdf_normal(sdf: SDFProtocol, p: torch.Tensor) -> torch.Tensor:
    """Unit gradient of sdf at points p (src/isoext/sdf.py:39-50)."""
    return torch.nn.functional.normalize(get_sdf_grad(sdf, p), dim=-1)


class SDF:
    """Base of the SDFs: a callable from points [..., 3] to distances [...]."""

    def __call__(self, p: torch.Tensor) -> torch.Tensor:  # pragma: no cover - abstract
        raise NotImplementedError


@dataclass
class SphereSDF(SDF):
    """Sphere of the given radius at the origin."""

    radius: float

    def __call__(self, p):
        return p.norm(dim=-1) - self.radius


@dataclass
class TorusSDF(SDF):
    """Torus around the z axis: major radius R in the xy plane, tube radius r."""

    R: float
    r: float

    def __call__(self, p):
        ring = p[..., :2].norm(dim=-1) - self.R
        return torch.stack([ring, p[..., 2]], dim=-1).norm(dim=-1) - self.r


@dataclass
class CuboidSDF(SDF):
    """Axis-aligned box at the origin; size = full edge lengths (x, y, z)."""

    size: list

    def __call__(self, p):
        half = torch.as_tensor(self.size, dtype=p.dtype, device=p.device) * 0.5
        q = p.abs() - half
        outside = q.clamp(min=0).norm(dim=-1)
        inside = q.max(dim=-1).values.clamp(max=0)
        return outside + inside


@dataclass
class UnionOp(SDF):
    """Union: the smallest of the distances."""

    sdf_list: list

    def __call__(self, p):
        d = self.sdf_list[0](p)
        for s in self.sdf_list[1:]:
            d = torch.minimum(d, s(p))
        return d


@dataclass
class SmoothUnionOp(SDF):
    """Smooth union, folded left: d <- -k log(exp(-d / k) + exp(-d_i / k)).
    As in isoext the expression is evaluated directly (it overflows once a
    distance exceeds about 88 k in magnitude)."""

    sdf_list: list
    k: float

    def __call__(self, p):
        d = self.sdf_list[0](p)
        for s in self.sdf_list[1:]:
            d = -self.k * torch.log(torch.exp(-d / self.k) + torch.exp(-s(p) / self.k))
        return d


@dataclass
class IntersectionOp(SDF):
    """Intersection: the largest of the distances."""

    sdf_list: list

    def __call__(self, p):
        d = self.sdf_list[0](p)
        for s in self.sdf_list[1:]:
            d = torch.maximum(d, s(p))
        return d


@dataclass
class NegationOp(SDF):
    """Complement: the distance with its sign flipped."""

    sdf: SDF

    def __call__(self, p):
        return -self.sdf(p)


@dataclass
class TranslationOp(SDF):
    """The shape moved by offset."""

    sdf: SDF
    offset: list

    def __call__(self, p):
        return self.sdf(p - torch.as_tensor(self.offset, dtype=p.dtype, device=p.device))


@dataclass
class RotationOp(SDF):
    """The shape rotated about axis by angle (degrees unless use_degree is False):
    points are mapped by p @ R with R the rotation matrix of Rodrigues' formula."""

    sdf: SDF
    axis: list
    angle: float
    use_degree: bool = True
    R: torch.Tensor = field(init=False, repr=False)

    def __post_init__(self):
        # float32 throughout, as isoext builds it (src/isoext/sdf.py:199-218)
        a = torch.nn.functional.normalize(torch.tensor(self.axis).float(), dim=0).reshape(3, 1)
        theta = torch.tensor(self.angle).float()
        if self.use_degree:
            theta = torch.deg2rad(theta)
        c, s = torch.cos(theta), torch.sin(theta)
        k = torch.zeros((3, 3))
        k[0, 1], k[0, 2] = -a[2, 0], a[1, 0]
        k[1, 0], k[1, 2] = a[2, 0], -a[0, 0]
        k[2, 0], k[2, 1] = -a[1, 0], a[0, 0]
        self.R = c * torch.eye(3) + s * k + (1 - c) * (a @ a.T)

    def __call__(self, p):
        return self.sdf(p @ self.R.to(dtype=p.dtype, device=p.device))
