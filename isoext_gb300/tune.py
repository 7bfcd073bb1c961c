"""Autotuner of the library's launch parameters on the GPU at hand.

    from isoext_gb300 import tune
    report = tune.autotune(grid)            # a UniformGrid with its values set
    tune.apply(report["best"])              # done by autotune; also for a saved report

The knobs (C ABI iso_tune_set) change launch shapes only, never results:
  "mc.emit_threads"     threads per CTA of the MC emit kernel
  "mc.sign_ctas_per_sm" CTAs per SM of the sign pass
  "mc.count_threads"    threads per CTA of the MC count kernel (and so the
                        scan's segment: 4 point words per thread)
  "dc.cell_threads"     threads per CTA of the per-active-cell DC kernels
Each knob is timed in turn (coordinate descent) with CUDA events over the
extraction it affects, on the caller's grid, the others held at their current
best.  For sparse grids, autotune_populate picks the brick size of
SparseGrid.populate (the bricks change which empty cells are kept, never the
mesh).

Results persist in a JSON cache keyed by (GPU name, extraction, grid shape,
level): autotune(..., cache=True) (or a path, or $ISOEXT_GB300_TUNE_CACHE)
applies a stored result without timing and stores new ones.  isoext has no
tunables; this module is an addition.
"""

from __future__ import annotations

import ctypes as C
import json
import os

import torch

from . import _ffi

KNOBS = {
    "mc.emit_threads": (128, 256),
    "mc.sign_ctas_per_sm": (8, 16, 32, 64),
    "mc.count_threads": (128, 256),
    "dc.cell_threads": (64, 128, 256),
}
# which extraction a knob's time is measured on
_TARGET = {"mc.emit_threads": "mc", "mc.sign_ctas_per_sm": "mc", "mc.count_threads": "mc", "dc.cell_threads": "dc"}
BRICKS = (4, 8, 16)  # brick edges (cells) autotune_populate tries
CACHE_ENV = "ISOEXT_GB300_TUNE_CACHE"
_populate_brick = 8


def get(key: str) -> int:
    v = C.c_int()
    _ffi.check(_ffi.lib().iso_tune_get(key.encode(), C.byref(v)))
    return v.value


def set(key: str, value: int) -> None:  # noqa: A001 - mirrors the C name
    _ffi.check(_ffi.lib().iso_tune_set(key.encode(), int(value)))


def current() -> dict:
    return {k: get(k) for k in KNOBS}


def apply(best: dict) -> None:
    for k, v in best.items():
        set(k, v)


# A knob keeps the value in force unless another is faster by more than this
# fraction: single-grid timings differ by a few percent from run to run, and a
# choice within that noise can suit concurrent streams worse (the served loop).
MARGIN = 0.03


def choose(times: dict, incumbent):
    """The value autotune keeps for one knob, given {value: ms}: the fastest,
    unless the incumbent (the value in force) is within MARGIN of it."""
    fastest = min(times, key=times.get)
    if incumbent in times and times[fastest] >= times[incumbent] * (1.0 - MARGIN):
        return incumbent
    return fastest


def _time(fn, repeats: int) -> float:
    """Mean ms of fn() over repeats calls, after two warm-up calls."""
    for _ in range(2):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(repeats):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / repeats


def populate_brick() -> int:
    """The brick edge SparseGrid.populate uses when none is given."""
    return _populate_brick


def set_populate_brick(brick: int) -> None:
    global _populate_brick
    if int(brick) < 1:
        raise ValueError("brick must be positive")
    _populate_brick = int(brick)


# ---------------------------------------------------------------------------
# the persistent cache

def cache_path(cache=None) -> str | None:
    """The cache file: `cache` if it is a path, the default file if it is True,
    else $ISOEXT_GB300_TUNE_CACHE (None when unset)."""
    if isinstance(cache, (str, os.PathLike)):
        return os.fspath(cache)
    if cache is True:
        return os.environ.get(CACHE_ENV) or os.path.join(os.path.expanduser("~"), ".cache", "isoext_gb300",
                                                         "tune.json")
    return os.environ.get(CACHE_ENV)


def gpu_name() -> str:
    return torch.cuda.get_device_name(torch.cuda.current_device())


def cache_key(kind: str, shape, level: float, gpu: str | None = None) -> str:
    """(GPU name, extraction, grid shape, level) as one string."""
    return f"{gpu or gpu_name()}|{kind}|{'x'.join(str(int(n)) for n in shape)}|level={float(level)!r}"


def cache_lookup(path: str | None, key: str) -> dict | None:
    if not path or not os.path.exists(path):
        return None
    try:
        with open(path) as fh:
            return json.load(fh).get(key)
    except (OSError, ValueError):
        return None


def cache_store(path: str | None, key: str, report: dict) -> None:
    """Adds report under key (written to a temporary file, then renamed)."""
    if not path:
        return
    data = {}
    if os.path.exists(path):
        try:
            with open(path) as fh:
                data = json.load(fh)
        except (OSError, ValueError):
            data = {}
    data[key] = report
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    tmp = f"{path}.{os.getpid()}.tmp"
    with open(tmp, "w") as fh:
        json.dump(data, fh, indent=1, sort_keys=True)
    os.replace(tmp, path)


def _json_report(report: dict) -> dict:
    return {"best": report["best"], "ms": {k: {str(v): t for v, t in d.items()} for k, d in report["ms"].items()}}


def autotune(grid, level: float = 0.0, kinds=("mc", "dc"), repeats: int = 10, knobs: dict | None = None,
             cache=None) -> dict:
    """Times each knob's values on this grid and keeps the fastest (the value in
    force unless another beats it by more than MARGIN, see choose); returns
    {"best": {knob: value}, "ms": {knob: {value: ms}}} and leaves the best set.
    With a cache (see cache_path), a stored result for this GPU, grid shape,
    extractions and level is applied instead ("cached": True), and a new one is
    stored."""
    from .dc import dual_contouring
    from .mc import marching_cubes

    knobs = knobs or KNOBS
    path = cache_path(cache)
    key = cache_key("+".join(kinds), grid.shape, level)
    hit = cache_lookup(path, key)
    if hit and all(k in hit.get("best", {}) for k in knobs if _TARGET[k] in kinds):
        apply({k: v for k, v in hit["best"].items() if k in KNOBS})
        return {"best": current(), "ms": hit.get("ms", {}), "cached": True}
    run = {"mc": lambda: marching_cubes(grid, level), "dc": lambda: dual_contouring(grid, level)}
    best = current()
    times: dict = {}
    for k, values in knobs.items():
        if _TARGET[k] not in kinds:
            continue
        times[k] = {}
        for v in values:
            set(k, v)
            times[k][v] = round(_time(run[_TARGET[k]], repeats), 5)
        best[k] = choose(times[k], best[k])
        set(k, best[k])
    report = {"best": best, "ms": times, "cached": False}
    cache_store(path, key, _json_report(report))
    return report


def autotune_populate(shape, sdf, level: float = 0.0, band: float | None = None, bricks=BRICKS,
                      aabb_min=(-1.0, -1.0, -1.0), aabb_max=(1.0, 1.0, 1.0), repeats: int = 2, cache=None) -> dict:
    """Picks SparseGrid.populate's brick edge for this lattice and SDF: each
    brick size is timed over populate + marching_cubes, and the fastest becomes
    the default (set_populate_brick).  Every brick size gives the same mesh:
    bricks only decide which empty cells near the surface are kept.  Returns
    {"best": {"sparse.brick": b}, "ms": {"sparse.brick": {b: ms}}}; cached like
    autotune."""
    import time

    from .mc import marching_cubes
    from .sparse import SparseGrid

    path = cache_path(cache)
    key = cache_key("sparse", shape, level)
    hit = cache_lookup(path, key)
    if hit and "sparse.brick" in hit.get("best", {}):
        set_populate_brick(hit["best"]["sparse.brick"])
        return {"best": {"sparse.brick": populate_brick()}, "ms": hit.get("ms", {}), "cached": True}
    times = {}
    for b in bricks:
        g = SparseGrid(list(shape), aabb_min, aabb_max)

        def step():
            g.populate(sdf, level, mode="brick", band=band, brick=b)
            marching_cubes(g, level)

        step()  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(repeats):
            step()
        torch.cuda.synchronize()
        times[b] = round(1e3 * (time.perf_counter() - t0) / repeats, 4)
    best = min(times, key=times.get)
    set_populate_brick(best)
    report = {"best": {"sparse.brick": best}, "ms": {"sparse.brick": times}, "cached": False}
    cache_store(path, key, _json_report(report))
    return report


def save(report: dict, path: str) -> None:
    with open(path, "w") as fh:
        json.dump(_json_report(report), fh, indent=1)


def load(path: str) -> dict:
    with open(path) as fh:
        rep = json.load(fh)
    apply({k: v for k, v in rep["best"].items() if k in KNOBS})
    return rep
