"""Input/output helpers with isoext's signatures (src/isoext/utils.py).

Not on the extraction path: plain torch / file code, provided so that code
written for isoext keeps working.
"""

from __future__ import annotations

import torch
import torch.nn.functional as F


def gaussian_smooth(field: torch.Tensor, sigma: float = 1.0, kernel_size: int | None = None) -> torch.Tensor:
    """Gaussian blur of a 3D scalar field [X, Y, Z] (src/isoext/utils.py:5-39).

    The kernel is the outer product of a normalised 1D Gaussian of odd size
    (default int(6 * sigma) | 1), applied as one 3D convolution with
    replicate padding -- the same arithmetic as isoext, so meshes extracted
    from the result match.
    """
    if kernel_size is None:
        kernel_size = int(6 * sigma) | 1
    half = kernel_size // 2
    x = torch.arange(kernel_size, device=field.device, dtype=field.dtype) - half
    k1 = torch.exp(-0.5 * (x / sigma) ** 2)
    k1 = k1 / k1.sum()
    k3 = (k1[:, None, None] * k1[None, :, None] * k1[None, None, :]).view(
        1, 1, kernel_size, kernel_size, kernel_size)
    f5 = F.pad(field.view(1, 1, *field.shape), [half] * 6, mode="replicate")
    return F.conv3d(f5, k3).reshape(field.shape)


def write_obj(obj_path: str, v: torch.Tensor, f: torch.Tensor) -> None:
    """Write a triangle mesh as Wavefront OBJ (1-based face indices).

    An empty or missing mesh writes an empty file (src/isoext/utils.py:42-63)."""
    with open(obj_path, "w") as fh:
        if v is None or f is None or v.numel() == 0 or f.numel() == 0:
            return
        vl = v.detach().cpu().tolist()
        fl = (f.detach().cpu().to(torch.int64) + 1).tolist()
        fh.writelines([f"v {a} {b} {c}\n" for a, b, c in vl])
        fh.writelines([f"f {a} {b} {c}\n" for a, b, c in fl])


def make_grid(aabb: list[float], res, device: str = "cuda") -> torch.Tensor:
    """Point coordinates [X, Y, Z, 3] of a regular grid over
    aabb = [xmin, ymin, zmin, xmax, ymax, zmax] (src/isoext/utils.py:66-83)."""
    if isinstance(res, int):
        res = [res] * 3
    axes = [torch.linspace(aabb[i], aabb[i + 3], res[i], device=device) for i in range(3)]
    return torch.stack(torch.meshgrid(axes, indexing="ij"), dim=-1)
