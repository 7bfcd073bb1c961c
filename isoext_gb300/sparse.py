"""SparseGrid with isoext's API (src/isoext_ext.cu:170-303, src/grid/sparse.cu:9-246)
and its marching cubes / intersection / dual contouring on the CUDA path
(csrc/sparse.cu).

A sparse grid holds a sorted list of cell ids on the lattice of a ``shape``-point
grid and 8 corner values per cell ([N, 8], corner k = 4x + 2y + z).  Cells do not
share storage, so -- as in isoext -- MC vertices are welded by exact position and
every cell uses its own 8 values.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _ffi
from .grids import FLT_MAX, SparseGridBase, _INT_MAX, _check_cuda_f32, _shape3, _vec3

_vp, _i, _ll, _f, _sz = C.c_void_p, C.c_int, C.c_longlong, C.c_float, C.c_size_t
_fa = C.POINTER(C.c_float)
_ffi.register({
    "iso_sparse_blocks_size": ([_ll], _sz),
    "iso_sparse_mc_count": ([_vp, _vp, _ll, _i, _i, _i, _fa, _fa, _f, _i, _vp, _vp, _vp], _i),
    "iso_sparse_mc_emit": ([_vp, _vp, _ll, _i, _i, _i, _fa, _fa, _f, _i, _vp, _vp, _vp], _i),
    "iso_sparse_its_count": ([_vp, _ll, _f, _vp, _vp, _vp], _i),
    "iso_sparse_its_emit": ([_vp, _vp, _ll, _i, _i, _i, _fa, _fa, _f, _vp, _ll, _ll, _vp, _vp, _vp, _vp,
                             _vp, _vp, _vp], _i),
    "iso_sparse_normals": ([_vp, _vp, _i, _i, _i, _fa, _fa, _vp, _vp, _ll, _vp, _vp, _vp], _i),
    "iso_sparse_quads_count": ([_vp, _vp, _ll, _i, _i, _i, _f, _vp, _vp, _vp, _vp], _i),
    "iso_sparse_quads_emit": ([_vp, _vp, _ll, _i, _i, _i, _f, _vp, _vp, _vp, _vp, _vp], _i),
    "iso_sparse_points": ([_vp, _ll, _i, _i, _i, _fa, _fa, _vp, _vp], _i),
    "iso_sparse_filter_count": ([_vp, _ll, _f, _vp, _vp, _vp], _i),
    "iso_sparse_filter_write": ([_vp, _vp, _ll, _f, _vp, _vp, _vp], _i),
    "iso_sparse_mc_workspace_size": ([_ll, _ll, _ll], _sz),
    "iso_sparse_mc": ([_vp, _vp, _ll, _i, _i, _i, _fa, _fa, _f, _i, _vp, _ll, _vp, _ll, _vp, _sz, _vp, _vp, _vp], _i),
})


def _p(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream(dev):
    return C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)


def _check_ids(t, what="new_cell_indices"):
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{what} must be a torch.Tensor")
    if t.dtype != torch.int32 or not t.is_cuda or not t.is_contiguous() or t.dim() != 1:
        raise TypeError(f"{what} must be a 1D C-contiguous int32 CUDA tensor")


def _as_uint(ids: torch.Tensor) -> torch.Tensor:
    """int32 ids read as uint32 (isoext casts the binding's int32 to uint), int64."""
    return ids.to(torch.int64) & 0xFFFFFFFF


def _from_uint(u: torch.Tensor) -> torch.Tensor:
    return torch.where(u >= 2**31, u - 2**32, u).to(torch.int32).contiguous()


class SparseGrid(SparseGridBase):
    """Sparse grid of cells over a ``shape``-point lattice (isoext.SparseGrid).

    ``shape`` counts lattice points per axis: cell (x, y, z) has id
    x (sy-1)(sz-1) + y (sz-1) + z and corners at points (x..x+1, y..y+1, z..z+1).
    """

    def __init__(self, shape, aabb_min=(-1.0, -1.0, -1.0), aabb_max=(1.0, 1.0, 1.0),
                 default_value: float = FLT_MAX, device=None):
        s = _shape3(shape)
        if s[0] * s[1] * s[2] > _INT_MAX:
            raise RuntimeError("Maximum number of points exceeds maximum value 2147483647 (max int)")
        self.shape = s
        self.aabb_min = _vec3(aabb_min)
        self.aabb_max = _vec3(aabb_max)
        self.default_value = float(np.float32(default_value))
        dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self._ids = torch.empty(0, dtype=torch.int32, device=dev)   # ascending as uint32
        self._values = torch.empty((0, 8), dtype=torch.float32, device=dev)

    @property
    def device(self) -> torch.device:
        return self._ids.device

    # -- container API --------------------------------------------------------------

    def get_num_cells(self) -> int:
        return int(self._ids.numel())

    def get_num_points(self) -> int:
        return 8 * int(self._ids.numel())

    def get_shape(self) -> list[int]:
        return list(self.shape)

    def get_cell_indices(self) -> torch.Tensor:
        return self._ids.clone()

    def get_values(self) -> torch.Tensor:
        return self._values.clone()

    def set_values(self, new_values: torch.Tensor) -> None:
        _check_cuda_f32(new_values, ndim=2, last=8, what="new_values")
        if new_values.numel() != self.get_num_points():
            raise RuntimeError("New values size does not match number of points")
        self._values.copy_(new_values)

    def get_cells(self) -> torch.Tensor:
        """Point ids of each cell's corners in get_points() order: arange(8N).view(N, 8)."""
        n = self.get_num_cells()
        return torch.arange(8 * n, dtype=torch.int32, device=self.device).view(n, 8)

    def _reset_values(self):
        # isoext refills every value with the default after add/remove (src/grid/sparse.cu:94-95)
        self._values = torch.full((self.get_num_cells(), 8), self.default_value, dtype=torch.float32,
                                  device=self.device)

    def add_cells(self, new_cell_indices: torch.Tensor) -> None:
        """Union with new ids (sorted, unique); all values reset to default_value."""
        _check_ids(new_cell_indices)
        u = torch.cat([_as_uint(self._ids), _as_uint(new_cell_indices)])
        self._ids = _from_uint(torch.unique(u, sorted=True))
        self._reset_values()

    def remove_cells(self, new_cell_indices: torch.Tensor) -> None:
        """Set difference; all values reset to default_value."""
        _check_ids(new_cell_indices)
        keep = ~torch.isin(_as_uint(self._ids), _as_uint(new_cell_indices))
        self._ids = self._ids[keep].contiguous()
        self._reset_values()

    def get_potential_cell_indices(self, chunk_size: int) -> list[torch.Tensor]:
        """All ids 0 .. sx*sy*sz - 1 in chunks of chunk_size (src/grid/sparse.cu:128-142;
        isoext counts sx*sy*sz ids although the lattice has (sx-1)(sy-1)(sz-1) cells)."""
        chunk = int(chunk_size)
        if chunk <= 0:
            raise RuntimeError("chunk_size must be positive")
        total = self.shape[0] * self.shape[1] * self.shape[2]
        return [torch.arange(s, min(s + chunk, total), dtype=torch.int32, device=self.device)
                for s in range(0, total, chunk)]

    def populate(self, sdf, level: float = 0.0, mode: str = "brick", band: float | None = None,
                 brick: int | None = None, max_points: int = 1 << 23) -> None:
        """Builds the grid's cells and values from an SDF on the device, replacing
        both.  No counterpart in isoext: it stands in for the documented loop
        get_potential_cell_indices -> get_points_by_cell_indices -> sdf ->
        filter_cell_indices -> add_cells -> set_values (src/grid/sparse.cu:71-179),
        which visits every lattice cell.

        The lattice is tiled by bricks of brick^3 cells (brick defaults to the
        autotuner's choice, tune.populate_brick(), 8 until tuned).  A brick is a candidate
        when |sdf(centre) - level| <= band + its half-diagonal; sdf must therefore
        be 1-Lipschitz (a distance or a lower bound of one).  band defaults to 2 h
        (h the longest cell edge).  The SDF is evaluated once per lattice point of
        each candidate brick ((brick + 1)^3 points) and gathered into the
        per-cell [N, 8] layout; positions are the lattice's FP32 positions, the
        same as get_points() gives.
          mode "brick":   every cell of the bricks with a lattice point where
                          |sdf - level| < band;
          mode "surface": only the cells whose 8 values straddle level, i.e. the
                          cells the documented loop keeps.
        sdf: callable on float32 CUDA points [..., 3] returning [...] distances."""
        if mode not in ("brick", "surface"):
            raise ValueError('mode must be "brick" or "surface"')
        if brick is None:
            from .tune import populate_brick

            brick = populate_brick()
        if brick < 1:
            raise ValueError("brick must be positive")
        dev = self.device
        shape = self.shape
        ncell = [max(n - 1, 0) for n in shape]
        if min(ncell) < 1:
            self._ids = torch.empty(0, dtype=torch.int32, device=dev)
            self._values = torch.empty((0, 8), dtype=torch.float32, device=dev)
            return
        from .grids import grid_positions

        size = [float(np.float32(b) - np.float32(a)) for a, b in zip(self.aabb_min, self.aabb_max)]
        axes = [grid_positions(torch.arange(shape[k], device=dev), shape[k], self.aabb_min[k], self.aabb_max[k])
                for k in range(3)]
        h = [abs(size[k]) / (shape[k] - 1) for k in range(3)]
        band = 2.0 * max(h) if band is None else float(band)
        radius = 0.5 * brick * float(np.sqrt(sum(x * x for x in h)))
        nb = [(ncell[k] + brick - 1) // brick for k in range(3)]
        # 1. active bricks, a slab of x at a time
        per_slab = nb[1] * nb[2]
        step = max(1, (1 << 22) // max(per_slab, 1))
        active = []
        for x0 in range(0, nb[0], step):
            bx = torch.arange(x0, min(x0 + step, nb[0]), device=dev)
            b = torch.stack(torch.meshgrid(bx, torch.arange(nb[1], device=dev), torch.arange(nb[2], device=dev),
                                           indexing="ij"), -1).reshape(-1, 3)
            lo_pt = b * brick
            hi_pt = torch.minimum(lo_pt + brick, torch.tensor(ncell, device=dev))
            centre = torch.stack([0.5 * (axes[k][lo_pt[:, k]] + axes[k][hi_pt[:, k]]) for k in range(3)], -1)
            d = sdf(centre)
            keep = (d - level).abs() <= band + radius
            active.append(b[keep])
        bricks = torch.cat(active)
        # 2. lattice values of the active bricks, gathered per cell
        L = brick + 1
        o = torch.arange(L, device=dev)
        oc = torch.arange(brick, device=dev)
        corner = [(j >> 2, (j >> 1) & 1, j & 1) for j in range(8)]
        ids_parts, val_parts = [], []
        chunk = max(1, max_points // (L ** 3))
        for s in range(0, len(bricks), chunk):
            bb = bricks[s:s + chunk]
            pts_idx = [torch.clamp(bb[:, k, None] * brick + o, max=shape[k] - 1) for k in range(3)]  # [nb, L]
            P = torch.stack(torch.broadcast_tensors(axes[0][pts_idx[0]][:, :, None, None],
                                                    axes[1][pts_idx[1]][:, None, :, None],
                                                    axes[2][pts_idx[2]][:, None, None, :]), -1)
            vals = sdf(P).to(torch.float32)  # [nb, L, L, L]
            if mode == "brick":
                # the brick stays if one of its lattice points lies within the band
                near = (vals - level).abs().amin(dim=(1, 2, 3)) < band
                bb, vals = bb[near], vals[near]
            cv = torch.stack([vals[:, dx:dx + brick, dy:dy + brick, dz:dz + brick] for dx, dy, dz in corner], -1)
            cx, cy, cz = (bb[:, k, None] * brick + oc for k in range(3))  # [nb, brick]
            ok = (cx[:, :, None, None] < ncell[0]) & (cy[:, None, :, None] < ncell[1]) & \
                (cz[:, None, None, :] < ncell[2])
            ids = (cx[:, :, None, None] * ncell[1] + cy[:, None, :, None]) * ncell[2] + cz[:, None, None, :]
            ids, cv = ids[ok], cv[ok]
            if mode == "surface":
                below = (cv - level) < 0
                straddle = below.any(-1) & ~below.all(-1)
                ids, cv = ids[straddle], cv[straddle]
            ids_parts.append(ids)
            val_parts.append(cv)
        ids = torch.cat(ids_parts) if ids_parts else torch.empty(0, dtype=torch.int64, device=dev)
        vals = torch.cat(val_parts) if val_parts else torch.empty((0, 8), dtype=torch.float32, device=dev)
        ids, order = torch.sort(ids)
        self._ids = ids.to(torch.int32).contiguous()
        self._values = vals[order].contiguous()

    def get_points_by_cell_indices(self, cell_indices: torch.Tensor) -> torch.Tensor:
        """Corner positions [M, 8, 3] of the given cell ids."""
        _check_ids(cell_indices, "cell_indices")
        return self._points_of(cell_indices)

    def get_points(self) -> torch.Tensor:
        """Corner positions [N, 8, 3] of the grid's cells."""
        return self._points_of(self._ids)

    def _points_of(self, ids: torch.Tensor) -> torch.Tensor:
        m = int(ids.numel())
        out = torch.empty((m, 8, 3), dtype=torch.float32, device=ids.device)
        if m:
            sx, sy, sz = self.shape
            _ffi.check(_ffi.lib().iso_sparse_points(_p(ids), m, sx, sy, sz, _ffi.fvec3(self.aabb_min),
                                                    _ffi.fvec3(self.aabb_max), _p(out), _stream(ids.device)))
        return out

    def filter_cell_indices(self, cell_indices: torch.Tensor, values: torch.Tensor,
                            level: float = 0.0) -> torch.Tensor:
        """Ids whose 8 values straddle ``level`` (case not 0 or 255), in input order."""
        _check_ids(cell_indices, "cell_indices")
        _check_cuda_f32(values, ndim=2, last=8, what="values")
        m = int(cell_indices.numel())
        if values.shape[0] != m:
            raise RuntimeError("values must have one row of 8 per cell index")
        lib = _ffi.lib()
        dev = cell_indices.device
        st = _stream(dev)
        blk = torch.empty(int(lib.iso_sparse_blocks_size(m)), dtype=torch.uint8, device=dev)
        counts = torch.zeros(2, dtype=torch.int64, device=dev)
        _ffi.check(lib.iso_sparse_filter_count(_p(values), m, float(level), _p(blk), _p(counts), st))
        k = int(counts[0].item())
        out = torch.empty(k, dtype=torch.int32, device=dev)
        if k:
            _ffi.check(lib.iso_sparse_filter_write(_p(cell_indices), _p(values), m, float(level), _p(blk),
                                                   _p(out), st))
        return out

    # -- extraction --------------------------------------------------------------

    def _geom(self):
        sx, sy, sz = self.shape
        return sx, sy, sz, _ffi.fvec3(self.aabb_min), _ffi.fvec3(self.aabb_max)

    def _marching_cubes(self, level: float, method: int):
        """iso_sparse_mc in one call, sized from the last call on this grid (one
        synchronisation; a retry with exact capacities when they were small)."""
        from .mc import _views

        lib = _ffi.lib()
        dev = self.device
        n = self.get_num_cells()
        if n == 0:
            return None, None
        st = _stream(dev)
        sx, sy, sz, lo, hi = self._geom()
        key = (n, float(level), int(method))
        if getattr(self, "_mc_sizes", None) and key in self._mc_sizes:
            v, f = self._mc_sizes[key]
            cap_v, cap_f = v + v // 10 + 1024, f + f // 10 + 1024
        else:
            cap_f = 2 * n + 1024
            cap_v = cap_f
        for _ in range(2):
            vout = torch.empty((cap_v, 3), dtype=torch.float32, device=dev)
            fout = torch.empty((cap_f, 3), dtype=torch.int32, device=dev)
            ws = torch.empty(int(lib.iso_sparse_mc_workspace_size(n, cap_v, cap_f)), dtype=torch.uint8, device=dev)
            small = torch.zeros(4, dtype=torch.int64, device=dev)
            _ffi.check(lib.iso_sparse_mc(_p(self._ids), _p(self._values), n, sx, sy, sz, lo, hi, float(level),
                                         int(method), _p(vout), cap_v, _p(fout), cap_f, _p(ws), ws.numel(),
                                         _p(small), C.c_void_p(small.data_ptr() + 24), st))
            h = small.cpu()
            V, F, Fneed, status = int(h[0]), int(h[1]), int(h[2]), int(h[3] & 0xFFFFFFFF)
            if not getattr(self, "_mc_sizes", None):
                self._mc_sizes = {}
            self._mc_sizes[key] = (max(V, 1), max(Fneed, 1))
            if status == _ffi.ISO_ERR_OVERFLOW:
                cap_f = Fneed + 1024
                cap_v = max(V, 3 * Fneed if V == 0 else V) + 1024
                continue
            if status:
                raise RuntimeError(f"isoext_gb300: device error {status} in marching_cubes")
            return _views(vout, fout, V, F)
        raise RuntimeError("isoext_gb300: marching_cubes output did not fit after resizing")

    def _intersect(self, level: float, compute_normals: bool):
        from .dc import Intersection

        lib = _ffi.lib()
        dev = self.device
        n = self.get_num_cells()
        st = _stream(dev)
        sx, sy, sz, lo, hi = self._geom()
        blk = torch.empty(int(lib.iso_sparse_blocks_size(n)), dtype=torch.uint8, device=dev)
        counts = torch.zeros(2, dtype=torch.int64, device=dev)
        _ffi.check(lib.iso_sparse_its_count(_p(self._values), n, float(level), _p(blk), _p(counts), st))
        A, K = (int(x) for x in counts.cpu())
        points = torch.empty((K, 3), dtype=torch.float32, device=dev)
        normals = torch.empty((K, 3), dtype=torch.float32, device=dev) if compute_normals else None
        act = torch.empty(A, dtype=torch.int32, device=dev)
        act_lattice = torch.empty(A, dtype=torch.int32, device=dev)
        offs = torch.empty(A + 1, dtype=torch.int32, device=dev)
        rank = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
        _ffi.check(lib.iso_sparse_its_emit(_p(self._ids), _p(self._values), n, sx, sy, sz, lo, hi,
                                           float(level), _p(blk), A, K, _p(points), _p(normals), _p(act),
                                           _p(act_lattice), _p(offs), _p(rank), st))
        key = (tuple(self.shape), tuple(self.aabb_min), tuple(self.aabb_max), id(self))
        sparse = {"lattice": act_lattice, "rank": rank, "n": n}
        return Intersection(points, normals, act, offs, level, key, sparse=sparse)

    def _get_intersection(self, level: float, compute_normals: bool):
        return self._intersect(level, compute_normals)

    def _dual_contouring(self, level, its, reg, svd_tol):
        from .dc import weld_dual

        lib = _ffi.lib()
        dev = self.device
        st = _stream(dev)
        sx, sy, sz, lo, hi = self._geom()
        if its is None:
            its = self._intersect(level, True)
        elif its._sparse is None or its._grid_key[:3] != (tuple(self.shape), tuple(self.aabb_min),
                                                            tuple(self.aabb_max)) \
                or its._sparse["n"] != self.get_num_cells():
            raise RuntimeError("intersection was computed for a different grid")
        A = int(its._cells.numel())
        n = self.get_num_cells()
        normals = its._normals
        if normals is None:
            normals = torch.empty_like(its._points)
            _ffi.check(lib.iso_sparse_normals(_p(self._ids), _p(self._values), sx, sy, sz, lo, hi,
                                              _p(its._cells), _p(its._offsets), A, _p(its._points),
                                              _p(normals), st))
        if A == 0:
            return None, None
        dual = torch.empty((A, 3), dtype=torch.float32, device=dev)
        _ffi.check(lib.iso_dc_solve(sx, sy, sz, lo, hi, _p(its._points), _p(normals),
                                    _p(its._sparse["lattice"]), _p(its._offsets), A, float(reg),
                                    float(svd_tol), _p(dual), st))
        blk = torch.empty(int(lib.iso_sparse_blocks_size(n)), dtype=torch.uint8, device=dev)
        counts = torch.zeros(2, dtype=torch.int64, device=dev)
        rank = its._sparse["rank"]
        _ffi.check(lib.iso_sparse_quads_count(_p(self._ids), _p(self._values), n, sx, sy, sz,
                                              float(its._level), _p(rank), _p(blk), _p(counts), st))
        Q = int(counts[0].item())
        if Q == 0:
            return None, None
        tri = torch.empty(6 * Q, dtype=torch.int32, device=dev)
        _ffi.check(lib.iso_sparse_quads_emit(_p(self._ids), _p(self._values), n, sx, sy, sz,
                                             float(its._level), _p(rank), _p(blk), _p(dual), _p(tri), st))
        return weld_dual(lib, dev, dual, A, tri, st)
