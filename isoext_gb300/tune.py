"""Autotuner of the library's launch parameters on the GPU at hand.

    from isoext_gb300 import tune
    report = tune.autotune(grid)            # a UniformGrid with its values set
    tune.apply(report["best"])              # done by autotune; also for a saved report

The knobs (C ABI iso_tune_set) change launch shapes only, never results:
  "mc.emit_threads"     threads per CTA of the MC emit kernel
  "mc.sign_ctas_per_sm" CTAs per SM of the sign pass
  "dc.cell_threads"     threads per CTA of the per-active-cell DC kernels
Each knob is timed in turn (coordinate descent) with CUDA events over the
extraction it affects, on the caller's grid, the others held at their current
best.  isoext has no tunables; this module is an addition.
"""

from __future__ import annotations

import ctypes as C
import json

import torch

from . import _ffi

KNOBS = {
    "mc.emit_threads": (128, 256),
    "mc.sign_ctas_per_sm": (8, 16, 32, 64),
    "dc.cell_threads": (64, 128, 256),
}
# which extraction a knob's time is measured on
_TARGET = {"mc.emit_threads": "mc", "mc.sign_ctas_per_sm": "mc", "dc.cell_threads": "dc"}


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


def autotune(grid, level: float = 0.0, kinds=("mc", "dc"), repeats: int = 10, knobs: dict | None = None) -> dict:
    """Times each knob's values on this grid and keeps the fastest; returns
    {"best": {knob: value}, "ms": {knob: {value: ms}}} and leaves the best set."""
    from .dc import dual_contouring
    from .mc import marching_cubes

    run = {"mc": lambda: marching_cubes(grid, level), "dc": lambda: dual_contouring(grid, level)}
    knobs = knobs or KNOBS
    best = current()
    times: dict = {}
    for key, values in knobs.items():
        if _TARGET[key] not in kinds:
            continue
        times[key] = {}
        for v in values:
            set(key, v)
            times[key][v] = round(_time(run[_TARGET[key]], repeats), 5)
        best[key] = min(times[key], key=times[key].get)
        set(key, best[key])
    return {"best": best, "ms": times}


def save(report: dict, path: str) -> None:
    with open(path, "w") as fh:
        json.dump(report, fh, indent=1)


def load(path: str) -> dict:
    with open(path) as fh:
        rep = json.load(fh)
    apply(rep["best"])
    return rep
