"""Grid containers with isoext's Python API (src/isoext_ext.cu:111-303).

``shape`` is the number of grid POINTS per axis (isoext's docstrings say
"cells"; its code, src/grid/uniform.cu:8-20, uses points).  Values live in a
torch CUDA float32 tensor owned by the grid.
"""

from __future__ import annotations

import numpy as np
import torch

FLT_MAX = float(np.finfo(np.float32).max)
_INT_MAX = 2147483647


def _shape3(shape) -> list[int]:
    s = [int(v) for v in shape]
    if len(s) != 3:
        raise TypeError("shape must have 3 entries")
    if any(v < 0 for v in s):
        raise TypeError("shape entries must be non-negative")
    return s


def _vec3(v) -> list[float]:
    out = [float(np.float32(x)) for x in v]
    if len(out) != 3:
        raise TypeError("expected 3 floats")
    return out


def _check_cuda_f32(t, ndim: int | None = None, last: int | None = None, what: str = "values"):
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{what} must be a torch.Tensor")
    if t.dtype != torch.float32 or not t.is_cuda or not t.is_contiguous():
        raise TypeError(f"{what} must be a C-contiguous float32 CUDA tensor")
    if ndim is not None and t.dim() != ndim:
        raise TypeError(f"{what} must have {ndim} dimensions")
    if last is not None and t.shape[-1] != last:
        raise TypeError(f"{what} must have shape (-1, {last})")


def grid_positions(index: torch.Tensor, n: int, amin: float, amax: float) -> torch.Tensor:
    """Coordinate of grid index i along one axis of n points over [amin, amax]:
    amin + (i / (float)(n - 1)) * (amax - amin) in FP32, as isoext computes it
    (include/utils.cuh:62-80), in the library's current arithmetic reading
    (``set_arithmetic``).  ``index`` is an integer CUDA tensor."""
    from . import _ffi

    table = torch.empty(max(int(n), 0), dtype=torch.float32, device=index.device)
    with torch.cuda.device(index.device):
        _ffi.check(_ffi.lib().iso_axis_coords(table.data_ptr(), int(n), float(amin), float(amax),
                                              torch.cuda.current_stream(index.device).cuda_stream))
    return table[index.long()]


class Grid:
    """Common base of UniformGrid and SparseGrid (isoext ``Grid``)."""

    def get_num_cells(self) -> int:  # pragma: no cover - abstract
        raise NotImplementedError

    def get_num_points(self) -> int:  # pragma: no cover - abstract
        raise NotImplementedError


class UniformGrid(Grid):
    """Dense grid of float32 values at ``shape`` points over an axis-aligned box.

    Mirrors isoext.UniformGrid (src/isoext_ext.cu:128-168, src/grid/uniform.cu).
    """

    def __init__(self, shape, aabb_min=(-1.0, -1.0, -1.0), aabb_max=(1.0, 1.0, 1.0),
                 default_value: float = FLT_MAX, device=None):
        s = _shape3(shape)
        if s[0] * s[1] * s[2] > _INT_MAX:
            raise RuntimeError("Number of points exceeds maximum value 2147483647 (max int)")
        self.shape = s
        self.aabb_min = _vec3(aabb_min)
        self.aabb_max = _vec3(aabb_max)
        # aabb_max - aabb_min in FP32, as the reference's float3 subtraction
        self._size = [float(np.float32(b) - np.float32(a)) for a, b in zip(self.aabb_min, self.aabb_max)]
        dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self._values = torch.full(s, float(np.float32(default_value)), dtype=torch.float32, device=dev)

    @property
    def device(self) -> torch.device:
        return self._values.device

    def get_num_cells(self) -> int:
        sx, sy, sz = self.shape
        return max(sx - 1, 0) * max(sy - 1, 0) * max(sz - 1, 0)

    def get_num_points(self) -> int:
        sx, sy, sz = self.shape
        return sx * sy * sz

    def get_shape(self) -> list[int]:
        return list(self.shape)

    def get_points(self) -> torch.Tensor:
        """Grid point positions, float32 [sx, sy, sz, 3]."""
        dev = self._values.device
        axes = []
        for k in range(3):
            idx = torch.arange(self.shape[k], device=dev, dtype=torch.int64)
            axes.append(grid_positions(idx, self.shape[k], self.aabb_min[k], self.aabb_max[k]))
        gx, gy, gz = torch.meshgrid(axes[0], axes[1], axes[2], indexing="ij")
        return torch.stack([gx, gy, gz], dim=-1).contiguous()

    def get_values(self) -> torch.Tensor:
        """A copy of the values (isoext deep-copies too, include/ndarray.cuh:32-36)."""
        return self._values.clone()

    def set_values(self, new_values: torch.Tensor) -> None:
        """Copy new values [sx, sy, sz] float32 into the grid.

        isoext takes a CUDA tensor only.  Here a C-contiguous float32 host
        tensor is also accepted and copied straight into the grid's device
        storage (one H2D copy, at full speed from pinned memory); the call
        returns once the copy is done."""
        if isinstance(new_values, torch.Tensor) and not new_values.is_cuda:
            if new_values.dtype != torch.float32 or not new_values.is_contiguous() or new_values.dim() != 3:
                raise TypeError("new_values must be a C-contiguous float32 tensor with 3 dimensions")
        else:
            _check_cuda_f32(new_values, ndim=3, what="new_values")
        if list(new_values.shape) != self.shape:
            raise RuntimeError("Cannot set values with different shapes")
        self._values.copy_(new_values)

    def get_cells(self) -> torch.Tensor:
        """8 corner point ids per cell (Morton order), [sx-1, sy-1, sz-1, 8]."""
        sx, sy, sz = self.shape
        dev = self._values.device
        x = torch.arange(max(sx - 1, 0), device=dev).view(-1, 1, 1)
        y = torch.arange(max(sy - 1, 0), device=dev).view(1, -1, 1)
        z = torch.arange(max(sz - 1, 0), device=dev).view(1, 1, -1)
        base = (x * sy + y) * sz + z
        off = torch.tensor([0, 1, sz, sz + 1, sy * sz, sy * sz + 1, sy * sz + sz, sy * sz + sz + 1],
                           device=dev)
        cells = base.unsqueeze(-1) + off
        return cells.to(torch.int32)


class SparseGridBase(Grid):
    """Base of SparseGrid (defined in sparse.py); lets callers dispatch on type."""

    def _marching_cubes(self, level: float, method: int):  # pragma: no cover - abstract
        raise NotImplementedError
