"""Benchmark: dense 512^3 FP32 marching cubes (sphere |p| - 0.8) in Gcells/s.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload mc512|mc128|dc512|dc256|serve|grad|sparse1024|sparse768] [--mc-only]

One step is one extraction of the whole grid (511^3 = 133,432,831 cells).
  value  device-timed throughput with the grid resident in HBM (C ABI call with
         device buffers; CUDA events on the launching stream).
  e2e    the same through the public API with host buffers: pinned host values
         -> device, UniformGrid.set_values, marching_cubes, result -> host.
  roofline  of the kernel with the largest event-timed share: its algorithmic
         bytes per launch over its duration, against the measured HBM copy
         bandwidth; beside it the whole extraction's 4*N^3 + 12*V + 12*F bytes
         over the step time.
  cpu_baseline  the oracle's C restatement of the reference's algorithm on all
         host cores (x slabs on threads; rank 0 only).
  dc512, serve, sparse1024  (default run on one GPU) the metric's other halves
         in the same line: dual contouring of the same grid (value, roofline,
         e2e, its own CPU baseline), a short served mixed stream against the
         plain path (req/s, p50 / p99), and sparse marching cubes of the 1024^3
         smooth-min band.
--impl reference runs the reference's algorithm on the CPU (the oracle port:
the isoext sources are not available on the GPU host) and prints the same line.
Multi-GPU runs are independent replicas (the path has no exchange step).
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

WORKLOADS = {
    "mc512": dict(kind="mc", n=512, r=0.8, desc="mc_dense_512_sphere_r0.8"),
    "mc128": dict(kind="mc", n=128, r=0.8, desc="mc_dense_128_sphere_r0.8"),
    "dc512": dict(kind="dc1", n=512, r=0.8, desc="dc_dense_512_sphere_r0.8"),
    "dc384": dict(kind="dc1", n=384, r=0.8, desc="dc_dense_384_sphere_r0.8"),
    "dc256": dict(kind="dc", n=256, seed=7, desc="dc_dense_256_csg_seed7"),
    "serve": dict(kind="serve", count=512, seed=2026, sizes=(64, 96, 128, 192, 256), mc_share=0.7,
                  slots=8, budget_gb=40, desc="served_mixed_512req_n64-256_mc70"),
    "grad": dict(kind="grad", n=256, batch=8, seed=5, desc="diff_mc_dc_8x256_fourier"),
    "sparse1024": dict(kind="sparse", n=1024, brick=8, spheres=64, k=0.05, seed=3,
                       desc="sparse_mc_1024_bricks8_smoothmin64"),
    # the same field on a 768^3 lattice (32 M cells): the case ncu section captures run on
    "sparse768": dict(kind="sparse", n=768, brick=8, spheres=64, k=0.05, seed=3,
                      desc="sparse_mc_768_bricks8_smoothmin64"),
}
METRIC = "MC/DC Gcells/s @512^3 fp32"


def max_over_ranks(ms: float, world: int, dev=None) -> float:
    """The slowest rank's step time (replicas: every rank times its own steps)."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist

    t = torch.tensor([ms], dtype=torch.float64, device=dev if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(units_per_rank: float, ms: float, world: int) -> float:
    """Whole-job throughput: the units all ranks processed over the slowest rank's time."""
    return world * units_per_rank / (ms * 1e-3)


def peaks() -> dict:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for name, val in zip(names, parts[4:8]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def csg_sdf(seed: int):
    """Seeded CSG of the DC workload (tests/helpers.py csg_shape)."""
    from helpers import csg_shape

    return csg_shape(seed)


def sphere_values(n: int, r: float) -> np.ndarray:
    from helpers import sphere

    return sphere((n, n, n), r)


# ---------------------------------------------------------------------------

def kernel_bytes(kind: str, n: int, nv: int, nf: int) -> dict:
    """Algorithmic bytes per launch of each kernel of the MC pipeline."""
    pts = n ** 3
    words = n * n * ((n + 31) // 32)
    segs = (words + 1023) // 1024
    return {
        "mc_signs": 4 * pts + 4 * words,           # values once, sign bitmap once
        "mc_count": 4 * words + 4 * words,         # bitmap once, per-word entries once
        "mc_scan": 32 * segs,                      # segment sums read, offsets written
        "mc_emit": 16 * nv + 12 * nv + 8 * nf + 12 * nf,  # entries and endpoint values; vertices, faces
    }


def profiled_traffic(workload: str, kernel: str):
    """DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) recorded
    from an ncu capture in profiles/traffic.txt ("workload kernel bytes" lines)."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    if not os.path.exists(path):
        return None
    with open(path) as fh:
        for ln in fh:
            parts = ln.split()
            if len(parts) == 3 and parts[0] == workload and parts[1] == kernel:
                return int(parts[2])
    return None


def run_ours(args, wl, rank, world) -> dict | None:
    import torch

    import isoext_gb300 as iso
    from isoext_gb300 import _ffi
    from isoext_gb300.mc import mc_dense_into, workspace_bytes

    if wl["kind"] == "dc":
        return run_dc(args, wl, rank, world)
    if wl["kind"] == "serve":
        return run_serve(args, wl, rank)
    if wl["kind"] == "dc1":
        return run_dc_one_call(args, wl, rank, world)
    if wl["kind"] == "grad":
        return run_grad(args, wl, rank, world)
    if wl["kind"] == "sparse":
        return run_sparse(args, wl, rank, world)
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    n = wl["n"]
    vals_np = sphere_values(n, wl["r"])
    vals = torch.from_numpy(vals_np).to(dev)
    cells = (n - 1) ** 3
    lib = _ffi.lib()
    stream = torch.cuda.current_stream(dev)
    # size outputs with one call, then time K back-to-back calls
    grid = iso.UniformGrid([n] * 3, device=dev)
    grid.set_values(vals)
    v, f = iso.marching_cubes(grid)
    nv, nf = len(v), len(f)
    capv, capf = nv + 1024, nf + 1024
    vout = torch.empty((capv, 3), dtype=torch.float32, device=dev)
    fout = torch.empty((capf, 3), dtype=torch.int32, device=dev)
    ws = torch.empty(workspace_bytes([n] * 3, capv, capf), dtype=torch.uint8, device=dev)
    small = torch.zeros(4, dtype=torch.int64, device=dev)
    amin, amax = (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0)

    def step():
        _ffi.check(mc_dense_into(vals, amin, amax, 0.0, 0, vout, fout, ws, small, stream.cuda_stream))

    algo_bytes = 4 * n ** 3 + 12 * nv + 12 * nf
    kbytes = kernel_bytes("mc", n, nv, nf)
    kernels = list(kbytes)
    # launch parameters for this GPU and grid (isoext_gb300.tune), before timing
    from isoext_gb300 import tune
    tuned = tune.autotune(grid, kinds=("mc",), repeats=10)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    with ClockSampler(dev.index) as clk:
        # The timed region lasts milliseconds, shorter than the sampler's period:
        # keep the GPU busy with the same step for ~0.6 s first, so the clock
        # samples are taken under this load (they run on through the timed region).
        t_end = time.perf_counter() + (0.0 if args.quick else 0.6)
        while time.perf_counter() < t_end:
            for _ in range(50):
                step()
            torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    # per-kernel times in a separate pass: the timing hooks put events between
    # the kernels, which the timed region above does not have
    lib.iso_profile_reset()
    lib.iso_profile_enable(1)
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    lib.iso_profile_enable(0)
    host = small.cpu()
    assert int(host[2] & 0xffffffff) == 0, f"device status {int(host[2])}"
    assert (int(host[0]), int(host[1])) == (nv, nf)
    kt = {k: _ffi.profile_read(k) for k in kernels}
    launches = sum(_ffi.profile_kernels(k) for k in kt)  # kernels, not timed groups
    # per extraction: the sum of the kernel's launches in one call
    kavg = {k: t / args.steps for k, (c, t) in kt.items()}
    top = max(kavg, key=kavg.get)
    ms = max_over_ranks(ms, world, dev)

    # e2e through the public API with host buffers: pinned values copied into the
    # grid (set_values with a host tensor: one H2D copy), marching_cubes, the mesh
    # read into pinned host buffers
    pinned = torch.from_numpy(vals_np).pin_memory()
    grid = iso.UniformGrid([n] * 3, device=dev)
    vh = torch.empty((capv, 3), dtype=torch.float32).pin_memory()
    fh = torch.empty((capf, 3), dtype=torch.int32).pin_memory()
    e2e_times, h2d_t, d2h_t = [], [], []
    h2d = pinned.numel() * 4
    d2h = 0
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        grid.set_values(pinned)
        t1 = time.perf_counter()
        v, f = iso.marching_cubes(grid)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        vh[:len(v)].copy_(v)
        fh[:len(f)].copy_(f)
        t3 = time.perf_counter()
        if i >= args.warmup:
            e2e_times.append(t3 - t0)
            h2d_t.append(t1 - t0)
            d2h_t.append(t3 - t2)
        d2h = v.numel() * 4 + f.numel() * 4 + 32
    e2e_ms = 1e3 * statistics.mean(e2e_times)
    e2e_split = {"h2d_ms": round(1e3 * statistics.mean(h2d_t), 3), "d2h_ms": round(1e3 * statistics.mean(d2h_t), 3),
                 "h2d_gbs": round(h2d / statistics.mean(h2d_t) / 1e9, 1)}

    if rank != 0:
        return None
    pk = peaks()
    achieved = kbytes[top] / (kavg[top] * 1e-3) / 1e9
    pipeline = algo_bytes / (ms * 1e-3) / 1e9
    out = {
        "metric": METRIC, "value": round(world * cells / (ms * 1e-3) / 1e9, 3), "unit": "Gcells/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: sphere SDF |p|-0.8 on [-1,1]^3",
        "config": {"workload": wl["desc"], "grid": [n, n, n], "cells": cells, "method": "nagae",
                   "vertices": nv, "faces": nf, "parallelism": f"replicas x{world}",
                   "tuned": {k: v for k, v in tuned["best"].items() if k.startswith("mc.")},
                   "l2": f"inputs larger than L2 (values {4 * n ** 3 / 1e6:.0f} MB > 129 MB L2)"
                         if 4 * n ** 3 > 129e6 else "inputs smaller than L2 (not flushed)"},
        "e2e": {"value": round(world * cells / (e2e_ms * 1e-3) / 1e9, 3), "unit": "Gcells/s",
                "ms_per_step": round(e2e_ms, 3), "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                **e2e_split},
        "roofline": {"bound": "hbm", "kernel": top, "achieved": round(achieved, 1),
                     "peak": pk["hbm_gbs"], "unit": "GB/s", "frac": round(achieved / pk["hbm_gbs"], 4),
                     "peak_source": pk["source"], "algorithmic_bytes": kbytes[top],
                     "kernel_ms": round(kavg[top], 4), "traffic": profiled_traffic(wl["desc"], top),
                     "pipeline": {"algorithmic_bytes": algo_bytes, "achieved": round(pipeline, 1),
                                  "frac": round(pipeline / pk["hbm_gbs"], 4)}},
        "kernel_ms": {k: round(v_, 4) for k, v_ in kavg.items()},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(vals_np, cells)
    if wl["desc"] == WORKLOADS["mc512"]["desc"] and not args.mc_only and world == 1:
        # the metric's other halves, measured in the same run: dense DC of the
        # same grid, and the served stream against the plain path (one GPU; the
        # replicas run of N > 1 times MC alone)
        dc = run_dc_one_call(args, WORKLOADS["dc512"], rank, world)
        out["dc512"] = {k: dc[k] for k in ("value", "unit", "ms_per_step", "config", "e2e", "roofline",
                                           "kernel_ms", "gpu_launches", "clocks", "cpu_baseline") if k in dc}
        out["serve"] = serve_summary(args, dev)
        # config 3: sparse MC of the 1024^3 smooth-min band (57.2 M cells)
        sp = run_sparse(args, WORKLOADS["sparse1024"], rank, world)
        out["sparse1024"] = {k: sp[k] for k in ("value", "unit", "ms_per_step", "config", "e2e", "roofline",
                                                "kernel_ms", "gpu_launches", "clocks", "cpu_baseline") if k in sp}
    return out


DC_KERNELS = ["mc_signs", "dc_classify", "dc_intersect", "dc_normals", "dc_solve", "dc_quads", "dc_weld"]


def fourier_values(n: int, seed: int, dev, k: int = 32):
    """helpers.fourier_sphere on the n^3 grid over [-1, 1]^3, evaluated on the device
    in FP64 (same seeded parameters), rounded to FP32."""
    import torch
    from helpers import axis_coords

    g = np.random.default_rng(seed)
    w = torch.from_numpy(g.normal(0.0, 3.0, size=(k, 3))).to(dev)
    a = g.normal(0.0, 0.02, size=k)
    phi = g.uniform(0.0, 2 * np.pi, size=k)
    ax = torch.from_numpy(axis_coords(n).astype(np.float64)).to(dev)
    X, Y, Z = torch.meshgrid(ax, ax, ax, indexing="ij")
    out = torch.sqrt(X * X + Y * Y + Z * Z) - 0.6
    for i in range(k):
        out += a[i] * torch.sin(X * w[i, 0] + Y * w[i, 1] + Z * w[i, 2] + phi[i])
    return out.float().contiguous()


GRAD_KERNELS = ["mc_signs", "mc_count", "mc_scan", "mc_emit", "mc_backward", "dc_classify", "dc_intersect",
                "dc_solve", "dc_quads", "dc_weld", "dc_backward"]


def run_grad(args, wl, rank, world) -> dict | None:
    """One step: differentiable marching cubes and dual contouring of the batch's
    grids (isoext_gb300.diff, batched: one synchronisation per kind), loss = sum
    over the meshes of the mean squared distance of their vertices to the unit
    sphere, backward to the grid values (hand-written backward kernels)."""
    import torch

    from isoext_gb300 import _ffi, diff

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    n, B = wl["n"], wl["batch"]
    lo, hi = (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0)
    xs = [fourier_values(n, wl["seed"] + i, dev).requires_grad_(True) for i in range(B)]
    lib = _ffi.lib()
    stream = torch.cuda.current_stream(dev)
    nverts = []

    def loss_of(v):
        return ((v.norm(dim=-1) - 1.0) ** 2).mean()

    def step():
        nverts.clear()
        for x in xs:
            x.grad = None
        # every grid's extraction is queued before one synchronisation per kind
        mcs = diff.marching_cubes_batch(xs, lo, hi)
        dcs = diff.dual_contouring_batch(xs, lo, hi)
        loss = sum(loss_of(vm) + loss_of(vd) for (vm, _), (vd, _) in zip(mcs, dcs))
        loss.backward()
        nverts.extend((len(vm), len(vd)) for (vm, _), (vd, _) in zip(mcs, dcs))

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    with ClockSampler(dev.index) as clk:
        t_end = time.perf_counter() + (0.0 if args.quick else 0.6)
        while time.perf_counter() < t_end:
            step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    lib.iso_profile_reset()  # per-kernel times in a separate pass (events between kernels)
    lib.iso_profile_enable(1)
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    lib.iso_profile_enable(0)
    kt = {k: _ffi.profile_read(k) for k in GRAD_KERNELS}
    kavg = {k: t / max(c, 1) for k, (c, t) in kt.items() if c}
    launches = sum(_ffi.profile_kernels(k) for k in kt)  # kernels, not timed groups
    # e2e: grids from pinned host memory, gradients back to the host
    hosts = [x.detach().cpu().pin_memory() for x in xs]
    outs = [torch.empty_like(h).pin_memory() for h in hosts]
    e2e_t = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for x, h in zip(xs, hosts):
            with torch.no_grad():
                x.copy_(h, non_blocking=True)
        step()
        for x, o in zip(xs, outs):
            o.copy_(x.grad, non_blocking=True)
        torch.cuda.synchronize()
        if i >= args.warmup:
            e2e_t.append(time.perf_counter() - t0)
    e2e_ms = 1e3 * statistics.mean(e2e_t)
    if rank != 0:
        return None
    cells = B * (n - 1) ** 3
    pk = peaks()
    top = "mc_backward" if "mc_backward" in kavg else None
    V = sum(a for a, _ in nverts) // B
    bw_bytes = V * (8 + 12 + 8 + 8)  # edge key, vertex gradient, two endpoint values (read) + two atomics
    roof = None
    if top:
        ach = bw_bytes / (kavg[top] * 1e-3) / 1e9
        roof = {"bound": "hbm", "kernel": top, "achieved": round(ach, 1), "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": round(ach / pk["hbm_gbs"], 4), "peak_source": pk["source"], "algorithmic_bytes": bw_bytes,
                "kernel_ms": round(kavg[top], 4), "traffic": profiled_traffic(wl["desc"], top)}
    out = {
        "metric": "differentiable MC+DC Gcells/s (forward + backward)", "value": round(cells / (ms * 1e-3) / 1e9, 3),
        "unit": "Gcells/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic: |p| - 0.6 + 32 seeded Fourier features on [-1,1]^3",
        "config": {"workload": wl["desc"], "batch": B, "grid": [n, n, n], "cells_per_step": cells,
                   "loss": "mean (|v| - 1)^2 per mesh, MC + DC", "vertices_mc_dc": nverts[0],
                   "l2": "each grid 67 MB < L2; 8 grids 537 MB > 129 MB L2, visited in turn"},
        "e2e": {"value": round(cells / (e2e_ms * 1e-3) / 1e9, 3), "unit": "Gcells/s", "ms_per_step": round(e2e_ms, 3),
                "h2d_bytes_per_step": B * 4 * n ** 3, "d2h_bytes_per_step": B * 4 * n ** 3},
        "roofline": roof,
        "kernel_ms": {k: round(v_, 4) for k, v_ in kavg.items()},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline_grad(wl)
    return out


def cpu_baseline_grad(wl) -> dict:
    """The FP64 autograd restatement (tests/grad_ref.py) of the same forward and
    backward on a 64^3 sample of the first grid, on the host's threads."""
    import torch
    from grad_ref import dc_crossed, dc_duals, mc_vertices, sphere_loss
    from helpers import axis_coords, fourier_sphere, grid_points

    from oracle import Oracle

    m = 64
    ax = axis_coords(wl["n"])
    lo, hi = (float(ax[190]),) + (float(ax[96]),) * 2, (float(ax[190 + m - 1]),) + (float(ax[96 + m - 1]),) * 2
    vals = fourier_sphere(grid_points((m, m, m), lo, hi), wl["seed"])
    ora = Oracle()
    t0 = time.perf_counter()
    _, _, e = ora.mc_dense(vals, lo, hi)
    its = ora.intersection_dense(vals, lo, hi)
    a, b = e[:, 0].astype(np.int64), e[:, 1].astype(np.int64)
    low, d = np.minimum(a, b), np.abs(a - b)
    edges = torch.from_numpy(3 * low + np.select([d == m * m, d == m], [0, 1], 2))
    cells = torch.from_numpy(its["cell_indices"].astype(np.int64))
    x = torch.from_numpy(vals).double().requires_grad_(True)
    crossed = dc_crossed(x, cells)
    loss = sphere_loss(mc_vertices(x, edges, lo, hi)) + sphere_loss(dc_duals(x, cells, crossed, lo, hi))
    loss.backward()
    sec = time.perf_counter() - t0
    c = (m - 1) ** 3
    return {"value": round(c / sec / 1e9, 6), "unit": "Gcells/s", "cores": torch.get_num_threads(), "kind": "port",
            "sample": f"one {m}^3 crop of the first grid: oracle C port forward (topology) + FP64 torch "
                      f"restatement forward and autograd backward, {sec:.2f} s; isoext has no backward"}


def smoothmin_spheres(wl):
    """Smooth-min union of the sparse workload's seeded spheres (tests/helpers.py)."""
    from helpers import smoothmin_spheres as field

    return field(wl["seed"], wl["spheres"], wl["k"])


def run_sparse(args, wl, rank, world) -> dict | None:
    """Sparse-grid marching cubes at n^3 virtual resolution: cells of the 8^3
    bricks within 2 h of the surface (SparseGrid.populate on the device), then
    K timed extractions."""
    import torch

    import isoext_gb300 as iso
    from isoext_gb300 import _ffi

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    n = wl["n"]
    f = smoothmin_spheres(wl)
    grid = iso.SparseGrid([n] * 3, device=dev)
    builds = []
    for _ in range(2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        grid.populate(f, mode="brick", brick=wl["brick"])
        torch.cuda.synchronize()
        builds.append(time.perf_counter() - t0)
    N = grid.get_num_cells()
    lib = _ffi.lib()
    stream = torch.cuda.current_stream(dev)
    v, fa = iso.marching_cubes(grid)
    nv, nf = len(v), len(fa)
    # the timed step: one iso_sparse_mc call with device buffers sized from the
    # first call (no host synchronisation between steps), as the dense workloads
    import ctypes as C

    cap_v, cap_f = nv + 1024, nf + 1024
    vout = torch.empty((cap_v, 3), dtype=torch.float32, device=dev)
    fout = torch.empty((cap_f, 3), dtype=torch.int32, device=dev)
    ws = torch.empty(int(lib.iso_sparse_mc_workspace_size(N, cap_v, cap_f)), dtype=torch.uint8, device=dev)
    small = torch.zeros(4, dtype=torch.int64, device=dev)
    sx, sy, sz, lo, hi = grid._geom()

    def step():
        _ffi.check(lib.iso_sparse_mc(C.c_void_p(grid._ids.data_ptr()), C.c_void_p(grid._values.data_ptr()), N,
                                     sx, sy, sz, lo, hi, 0.0, 0, C.c_void_p(vout.data_ptr()), cap_v,
                                     C.c_void_p(fout.data_ptr()), cap_f, C.c_void_p(ws.data_ptr()), ws.numel(),
                                     C.c_void_p(small.data_ptr()), C.c_void_p(small.data_ptr() + 24),
                                     C.c_void_p(stream.cuda_stream)))

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    with ClockSampler(dev.index) as clk:
        t_end = time.perf_counter() + (0.0 if args.quick else 0.6)
        while time.perf_counter() < t_end:
            for _ in range(10):
                step()
            torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    h = small.cpu()
    assert int(h[3] & 0xFFFFFFFF) == 0 and (int(h[0]), int(h[1])) == (nv, nf), "sparse sizes"
    lib.iso_profile_reset()  # per-kernel times in a separate pass (events between kernels)
    lib.iso_profile_enable(1)
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    lib.iso_profile_enable(0)
    kt = {k: _ffi.profile_read(k) for k in ("sparse_mc", "dc_weld")}
    kavg = {k: t / args.steps for k, (c, t) in kt.items() if c}  # per extraction (a name may time several groups)
    launches = sum(_ffi.profile_kernels(k) for k in kt)  # kernels, not timed groups
    # e2e: ids and values from pinned host memory, the mesh back
    ids_h = grid.get_cell_indices().cpu().pin_memory()
    vals_h = grid.get_values().cpu().pin_memory()
    e2e_t = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g2 = iso.SparseGrid([n] * 3, device=dev)
        g2._ids = ids_h.to(dev, non_blocking=True)  # sorted ids, as add_cells leaves them
        g2._values = vals_h.to(dev, non_blocking=True)
        vv, ff = iso.marching_cubes(g2)
        vh, fh = vv.cpu(), ff.cpu()
        if i >= args.warmup:
            e2e_t.append(time.perf_counter() - t0)
    e2e_ms = 1e3 * statistics.mean(e2e_t)
    if rank != 0:
        return None
    pk = peaks()
    mc_bytes = N * (4 + 32) + 12 * nv + 12 * nf  # ids and values read, vertices and faces written
    top = "sparse_mc" if "sparse_mc" in kavg else None
    roof = None
    if top:
        ach = mc_bytes / (kavg[top] * 1e-3) / 1e9
        roof = {"bound": "hbm", "kernel": top, "achieved": round(ach, 1), "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": round(ach / pk["hbm_gbs"], 4), "peak_source": pk["source"], "algorithmic_bytes": mc_bytes,
                "kernel_ms": round(kavg[top], 4), "traffic": profiled_traffic(wl["desc"], top)}
    out = {
        "metric": "sparse MC Gcells/s (active cells)", "value": round(N / (ms * 1e-3) / 1e9, 3), "unit": "Gcells/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": f"synthetic: smooth-min (k={wl['k']}) of {wl['spheres']} seeded spheres on [-1,1]^3",
        "config": {"workload": wl["desc"], "virtual_grid": [n, n, n], "active_cells": N,
                   "occupancy": round(N / (n - 1) ** 3, 4), "brick": wl["brick"], "vertices": nv, "faces": nf,
                   "virtual_gcells_s": round((n - 1) ** 3 / (ms * 1e-3) / 1e9, 2),
                   "populate_s": round(min(builds), 3),
                   "l2": f"values {N * 32 / 1e9:.2f} GB > 129 MB L2"},
        "e2e": {"value": round(N / (e2e_ms * 1e-3) / 1e9, 3), "unit": "Gcells/s", "ms_per_step": round(e2e_ms, 3),
                "h2d_bytes_per_step": N * 36, "d2h_bytes_per_step": nv * 12 + nf * 12},
        "roofline": roof,
        "kernel_ms": {k: round(v_, 4) for k, v_ in kavg.items()},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline_sparse(grid, N)
    return out


def cpu_baseline_sparse(grid, N) -> dict:
    """The oracle's sparse MC on a contiguous sample of the grid's cells (host threads, one slice each)."""
    import concurrent.futures as cf

    from oracle import Oracle

    ora = Oracle()
    m = min(N, 4_000_000)
    ids = grid.get_cell_indices()[:m].cpu().numpy()
    vals = grid.get_values()[:m].cpu().numpy()
    threads = os.cpu_count() or 1
    cuts = np.linspace(0, m, threads + 1).astype(int)
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(lambda i: ora.mc_sparse(ids[cuts[i]:cuts[i + 1]], vals[cuts[i]:cuts[i + 1]], grid.shape),
                    range(threads)))
    sec = time.perf_counter() - t0
    return {"value": round(m / sec / 1e9, 5), "unit": "Gcells/s", "cores": threads, "kind": "port",
            "sample": f"the first {m} active cells, {threads} slices on {threads} threads (each welded on its "
                      f"own), oracle C port, {sec:.2f} s"}


def _digest(v, f) -> str:
    import hashlib

    h = hashlib.blake2b(digest_size=16)
    h.update(np.ascontiguousarray(v).tobytes())
    h.update(np.ascontiguousarray(f).tobytes())
    return h.hexdigest()


def _serve_pass(srv, reqs, arrivals):
    """Submits reqs at their arrival offsets (s); returns (req/s, latencies s, digests)."""
    t0 = time.perf_counter()
    futs = []
    for r, a in zip(reqs, arrivals):
        d = t0 + a - time.perf_counter()
        if d > 0:
            time.sleep(d)
        futs.append(srv.submit(r))
    res = [f.result() for f in futs]
    lat = [x.t_done - (t0 + a) for x, a in zip(res, arrivals)]
    span = max(x.t_done for x in res) - t0
    nbytes = sum(x.vertices.nbytes + x.faces.nbytes for x in res)
    return len(reqs) / span, lat, [_digest(x.vertices, x.faces) for x in res], nbytes


def _plain_pass(reqs, arrivals, solve):
    """The same arrivals served one call per grid, first come first served."""
    t0 = time.perf_counter()
    lat, dig = [], []
    for r, a in zip(reqs, arrivals):
        d = t0 + a - time.perf_counter()
        if d > 0:
            time.sleep(d)
        v, f = solve(r)
        lat.append(time.perf_counter() - (t0 + a))
        dig.append(_digest(v, f))
    return len(reqs) / (time.perf_counter() - t0), lat, dig


def _pct(xs, q):
    return round(1e3 * float(np.percentile(np.asarray(xs), q)), 3)


def run_serve(args, wl, rank) -> dict | None:
    """The served mixed stream against the plain one-call-per-grid path.

    Both paths see the same requests at the same Poisson arrival times.  Two loads:
    a saturating one (mean gap 50 us, far below either path's service time) gives
    each path's requests/s, and a load of 0.8 x the plain path's capacity gives
    the latencies at a rate both sustain.  Every served result is compared with
    the plain result of the same request (digest of the vertex and face bytes)."""
    import torch

    from isoext_gb300 import serve

    if rank != 0:
        return None
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    sizes = tuple(wl["sizes"])
    reqs = serve.random_requests(wl["count"], wl["seed"], sizes, wl["mc_share"])
    warm = serve.random_requests(max(3, args.warmup) * 8, wl["seed"] + 1, sizes, wl["mc_share"])
    rng = np.random.default_rng(wl["seed"] + 2)
    gaps = rng.exponential(1.0, size=len(reqs))
    srv = serve.Server(slots=wl["slots"], budget_bytes=int(wl["budget_gb"] * (1 << 30)), device=dev)
    t_cap = time.perf_counter()
    tuned = srv.warmup(sizes)
    t_cap = time.perf_counter() - t_cap
    for r in warm:  # first calls of each size on both paths
        serve.solve_plain(r, dev)
    for f in [srv.submit(r) for r in warm]:
        f.result()
    repeats = max(1, min(args.steps, 3))
    with ClockSampler(dev.index) as clk:
        sat = np.cumsum(gaps) * 50e-6
        plain_sat = [_plain_pass(reqs, sat, lambda r: serve.solve_plain(r, dev)) for _ in range(repeats)]
        served_sat = [_serve_pass(srv, reqs, sat) for _ in range(repeats)]
        p_rate = statistics.median(x[0] for x in plain_sat)
        s_rate = statistics.median(x[0] for x in served_sat)
        load = np.cumsum(gaps) / (0.8 * p_rate)
        plain_load = _plain_pass(reqs, load, lambda r: serve.solve_plain(r, dev))
        served_load = _serve_pass(srv, reqs, load)
        srv.close()
        # the same loop in C++ (iso_serve_*): no interpreter on the request path
        nsrv = serve.NativeServer(slots=wl["slots"], budget_bytes=int(wl["budget_gb"] * (1 << 30)),
                                  warm_sizes=sizes, tune=False, device=dev)
        for f in [nsrv.submit(r) for r in warm]:
            f.result()
        native_sat = [_serve_pass(nsrv, reqs, sat) for _ in range(repeats)]
        n_rate = statistics.median(x[0] for x in native_sat)
        native_load = _serve_pass(nsrv, reqs, load)
        n_stats = nsrv.stats()
        nsrv.close()
        # the C++ loop with length buckets: same-key requests queued together
        # run as the parallel branches of one graph launch (up to 8)
        bsrv = serve.NativeServer(slots=wl["slots"], budget_bytes=int(wl["budget_gb"] * (1 << 30)),
                                  warm_sizes=sizes, tune=False, device=dev, bucket=8)
        for f in [bsrv.submit(r) for r in warm]:
            f.result()
        _serve_pass(bsrv, reqs, sat)  # builds the bucket entries (their count passes and graphs), untimed
        bucket_sat = [_serve_pass(bsrv, reqs, sat) for _ in range(repeats)]
        b_rate = statistics.median(x[0] for x in bucket_sat)
        bucket_load = _serve_pass(bsrv, reqs, load)
        b_stats = bsrv.stats()
        bsrv.close()
    same = sum(a == b for a, b in zip(plain_sat[0][2], served_sat[0][2]))
    same_load = sum(a == b for a, b in zip(plain_sat[0][2], served_load[2]))
    same_native = sum(a == b for a, b in zip(plain_sat[0][2], native_sat[0][2]))
    same_bucket = sum(a == b for a, b in zip(plain_sat[0][2], bucket_sat[0][2]))
    n_mc = sum(r.kind == "mc" for r in reqs)
    cells = sum((r.n - 1) ** 3 for r in reqs)
    ms_step = 1e3 / n_rate
    return {
        "metric": "served requests/s (mixed MC/DC stream)", "value": round(n_rate, 1), "unit": "req/s",
        "n_gpus": 1, "steps": repeats, "warmup": args.warmup, "ms_per_step": round(ms_step, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded unions of 1-16 spheres/boxes (sizes U[0.05,0.4]) on [-1,1]^3",
        "config": {"workload": wl["desc"], "requests": len(reqs), "sizes": list(sizes), "mc": n_mc,
                   "dc": len(reqs) - n_mc, "slots": wl["slots"], "budget_gb": wl["budget_gb"],
                   "cells_per_stream": cells, "warmup_s": round(t_cap, 2),
                   "tuned": tuned["best"] if tuned else None,
                   "l2": "each request's grid is written and read once; not flushed"},
        "served": {"req_s": round(n_rate, 1), "p50_ms": _pct(native_sat[0][1], 50),
                   "p99_ms": _pct(native_sat[0][1], 99), "gcells_s": round(cells * n_rate / len(reqs) / 1e9, 3),
                   "loop": "C++ (iso_serve_*)", "max_running": int(n_stats["max_running"]),
                   "max_admitted_gb": round(n_stats["max_admitted_bytes"] / 2 ** 30, 3)},
        "served_bucketed": {"req_s": round(b_rate, 1), "p50_ms": _pct(bucket_sat[0][1], 50),
                            "p99_ms": _pct(bucket_sat[0][1], 99), "loop": "C++, length buckets of up to 8",
                            "bucket_launches": int(b_stats["bucket_launches"]),
                            "bucketed_requests": int(b_stats["bucketed_requests"]),
                            "max_admitted_gb": round(b_stats["max_admitted_bytes"] / 2 ** 30, 3)},
        "served_python": {"req_s": round(s_rate, 1), "p50_ms": _pct(served_sat[0][1], 50),
                          "p99_ms": _pct(served_sat[0][1], 99), "max_running": srv.max_running,
                          "max_admitted_gb": round(srv.max_reserved / 2 ** 30, 3)},
        "plain": {"req_s": round(p_rate, 1), "p50_ms": _pct(plain_sat[0][1], 50),
                  "p99_ms": _pct(plain_sat[0][1], 99)},
        "at_load": {"rate_req_s": round(0.8 * p_rate, 1),
                    "served": {"p50_ms": _pct(native_load[1], 50), "p99_ms": _pct(native_load[1], 99)},
                    "served_bucketed": {"p50_ms": _pct(bucket_load[1], 50), "p99_ms": _pct(bucket_load[1], 99)},
                    "served_python": {"p50_ms": _pct(served_load[1], 50), "p99_ms": _pct(served_load[1], 99)},
                    "plain": {"p50_ms": _pct(plain_load[1], 50), "p99_ms": _pct(plain_load[1], 99)}},
        "identical_results": {"saturated": f"{same_native}/{len(reqs)}",
                              "saturated_bucketed": f"{same_bucket}/{len(reqs)}",
                              "saturated_python": f"{same}/{len(reqs)}", "at_load_python": f"{same_load}/{len(reqs)}"},
        "e2e": {"value": round(n_rate, 1), "unit": "req/s", "h2d_bytes_per_step": 4 * (1 + 7 * serve.MAX_PRIMS),
                "d2h_bytes_per_step": int(native_sat[0][3] / len(reqs)),
                "note": "a step is one request: its primitives host -> device, its mesh device -> host"},
        "roofline": None,
        "gpu_launches": repeats * (serve.KERNELS_PER_REQUEST["mc"] * n_mc
                                   + serve.KERNELS_PER_REQUEST["dc"] * (len(reqs) - n_mc)),
        "clocks": clk.summary(),
    }


def serve_summary(args, dev, count: int = 128) -> dict:
    """A short run of the served mixed stream (config of the serve workload, first
    `count` requests): the C++ serving loop against the plain one-call-per-grid
    path, saturated (req/s) and at 0.8 x the plain capacity (p50 / p99)."""
    from isoext_gb300 import serve

    wl = WORKLOADS["serve"]
    sizes = tuple(wl["sizes"])
    reqs = serve.random_requests(count, wl["seed"], sizes, wl["mc_share"])
    warm = serve.random_requests(16, wl["seed"] + 1, sizes, wl["mc_share"])
    gaps = np.random.default_rng(wl["seed"] + 2).exponential(1.0, size=len(reqs))
    nsrv = serve.NativeServer(slots=wl["slots"], budget_bytes=int(wl["budget_gb"] * (1 << 30)),
                              warm_sizes=sizes, tune=False, device=dev)
    try:
        for r in warm:
            serve.solve_plain(r, dev)
        for f in [nsrv.submit(r) for r in warm]:
            f.result()
        sat = np.cumsum(gaps) * 50e-6
        plain_sat = _plain_pass(reqs, sat, lambda r: serve.solve_plain(r, dev))
        native_sat = _serve_pass(nsrv, reqs, sat)
        load = np.cumsum(gaps) / (0.8 * plain_sat[0])
        plain_load = _plain_pass(reqs, load, lambda r: serve.solve_plain(r, dev))
        native_load = _serve_pass(nsrv, reqs, load)
    finally:
        nsrv.close()
    same = sum(a == b for a, b in zip(plain_sat[2], native_sat[2]))
    return {"workload": f"{wl['desc']} (first {count} requests)", "served_req_s": round(native_sat[0], 1),
            "plain_req_s": round(plain_sat[0], 1), "speedup": round(native_sat[0] / plain_sat[0], 2),
            "saturated": {"served_p50_ms": _pct(native_sat[1], 50), "served_p99_ms": _pct(native_sat[1], 99),
                          "plain_p50_ms": _pct(plain_sat[1], 50), "plain_p99_ms": _pct(plain_sat[1], 99)},
            "at_load": {"rate_req_s": round(0.8 * plain_sat[0], 1),
                        "served_p50_ms": _pct(native_load[1], 50), "served_p99_ms": _pct(native_load[1], 99),
                        "plain_p50_ms": _pct(plain_load[1], 50), "plain_p99_ms": _pct(plain_load[1], 99)},
            "identical_results": f"{same}/{len(reqs)}", "loop": "C++ (iso_serve_*)"}


def run_dc(args, wl, rank, world) -> dict | None:
    """One step: get_intersection -> analytic normals (autograd of the SDF, FP32)
    -> set_normals -> dual_contouring, the flow of isoext's DC notebook."""
    import torch

    import isoext_gb300 as iso
    from isoext_gb300 import _ffi, sdf

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    n = wl["n"]
    shape = csg_sdf(wl["seed"])
    grid = iso.UniformGrid([n] * 3, device=dev)
    vals = shape(grid.get_points()).contiguous()
    grid.set_values(vals)
    cells = (n - 1) ** 3
    lib = _ffi.lib()
    stream = torch.cuda.current_stream(dev)

    def step():
        its = iso.get_intersection(grid)
        its.set_normals(sdf.get_sdf_normal(shape, its.get_points()).contiguous())
        return iso.dual_contouring(grid, intersection=its)

    v, f = step()
    nv, nf = len(v), len(f)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    with ClockSampler(dev.index) as clk:
        t_end = time.perf_counter() + (0.0 if args.quick else 0.6)
        while time.perf_counter() < t_end:
            step()
        torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    lib.iso_profile_reset()  # per-kernel times in a separate pass (events between kernels)
    lib.iso_profile_enable(1)
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    lib.iso_profile_enable(0)
    kt = {k: _ffi.profile_read(k) for k in DC_KERNELS}
    kavg = {k: t / max(c, 1) for k, (c, t) in kt.items() if c}
    launches = sum(_ffi.profile_kernels(k) for k in kt)  # kernels, not timed groups
    ms = max_over_ranks(ms, world, dev)

    # e2e: host values -> device -> grid -> the step -> mesh to host
    host = vals.cpu().pin_memory()
    e2e_t = []
    d2h = 0
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        grid.set_values(host.to(dev, non_blocking=True))
        vv, ff = step()
        vh, fh = vv.cpu(), ff.cpu()
        t1 = time.perf_counter()
        if i >= args.warmup:
            e2e_t.append(t1 - t0)
        d2h = vh.numel() * 4 + fh.numel() * 4 + 64
    e2e_ms = 1e3 * statistics.mean(e2e_t)
    if rank != 0:
        return None
    K = int(iso.get_intersection(grid).get_points().shape[0])
    pts, words = n ** 3, n * n * ((n + 31) // 32)
    kbytes = {"mc_signs": 4 * pts + 4 * words, "dc_intersect": 8 * K + 12 * K + 8 * K,
              "dc_solve": 24 * K + 12 * K // 3, "dc_quads": 4 * words + 24 * nf // 2,
              "dc_weld": 24 * K // 3 + 24 * nf}
    top = max((k for k in kavg if k in kbytes), key=lambda k: kavg[k])
    pk = peaks()
    achieved = kbytes[top] / (kavg[top] * 1e-3) / 1e9
    algo = 4 * pts + 12 * nv + 12 * nf + 24 * K
    out = {
        "metric": METRIC, "value": round(world * cells / (ms * 1e-3) / 1e9, 3), "unit": "Gcells/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": f"synthetic: seeded CSG (box - sphere) U torus, seed {wl['seed']}, on [-1,1]^3",
        "config": {"workload": wl["desc"], "grid": [n, n, n], "cells": cells, "normals": "analytic (autograd)",
                   "vertices": nv, "faces": nf, "crossings": K, "parallelism": f"replicas x{world}",
                   "l2": "values 67 MB < 129 MB L2, not flushed between steps"},
        "e2e": {"value": round(world * cells / (e2e_ms * 1e-3) / 1e9, 3), "unit": "Gcells/s",
                "ms_per_step": round(e2e_ms, 3), "h2d_bytes_per_step": host.numel() * 4,
                "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "hbm", "kernel": top, "achieved": round(achieved, 1), "peak": pk["hbm_gbs"],
                     "unit": "GB/s", "frac": round(achieved / pk["hbm_gbs"], 4), "peak_source": pk["source"],
                     "algorithmic_bytes": kbytes[top], "kernel_ms": round(kavg[top], 4),
                     "traffic": profiled_traffic(wl["desc"], top),
                     "pipeline": {"algorithmic_bytes": algo, "achieved": round(algo / (ms * 1e-3) / 1e9, 1),
                                  "frac": round(algo / (ms * 1e-3) / 1e9 / pk["hbm_gbs"], 4)}},
        "kernel_ms": {k: round(v_, 4) for k, v_ in kavg.items()},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline_dc(vals.cpu().numpy(), shape, cells)
    return out


DC1_KERNELS = ["mc_signs", "dc_classify", "dc_solve", "dc_weld", "dc_quads"]


def run_dc_one_call(args, wl, rank, world) -> dict | None:
    """Dense dual contouring of the sphere |p| - r with normals from the grid
    (isoext.dual_contouring(grid) without an intersection), one call
    (iso_dc_dense) per step with device buffers."""
    import torch

    import isoext_gb300 as iso
    from isoext_gb300 import _ffi
    from isoext_gb300.dc import dc_dense_into, dc_workspace_bytes

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    n = wl["n"]
    vals_np = sphere_values(n, wl["r"])
    vals = torch.from_numpy(vals_np).to(dev)
    cells = (n - 1) ** 3
    lib = _ffi.lib()
    stream = torch.cuda.current_stream(dev)
    grid = iso.UniformGrid([n] * 3, device=dev)
    grid.set_values(vals)
    # launch parameters for this GPU and grid (isoext_gb300.tune), before timing
    from isoext_gb300 import tune
    tuned = tune.autotune(grid, kinds=("dc",), repeats=10)
    v, f = iso.dual_contouring(grid)
    nv, nf = len(v), len(f)
    from isoext_gb300 import dc as dcmod
    A, Q = dcmod._dc_sizes[(tuple(grid.shape), 0.0, tuple(grid.aabb_min), tuple(grid.aabb_max))]
    capv, capf = A + 1024, 2 * Q + 1024
    vout = torch.empty((capv, 3), dtype=torch.float32, device=dev)
    fout = torch.empty((capf, 3), dtype=torch.int32, device=dev)
    ws = torch.empty(dc_workspace_bytes([n] * 3, capv, capf), dtype=torch.uint8, device=dev)
    small = torch.zeros(8, dtype=torch.int64, device=dev)
    lo, hi = (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0)

    def step():
        _ffi.check(dc_dense_into(vals, lo, hi, 0.0, 1e-2, 1e-6, vout, fout, ws, small, stream.cuda_stream))

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    with ClockSampler(dev.index) as clk:
        t_end = time.perf_counter() + (0.0 if args.quick else 0.6)
        while time.perf_counter() < t_end:
            for _ in range(20):
                step()
            torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, world, dev)
    h = small.cpu()
    assert int(h[6] & 0xFFFFFFFF) == 0 and (int(h[0]), int(h[1])) == (nv, nf), "dc512 sizes"
    lib.iso_profile_reset()  # per-kernel times in a separate pass (events between kernels)
    lib.iso_profile_enable(1)
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    lib.iso_profile_enable(0)
    kt = {k: _ffi.profile_read(k) for k in DC1_KERNELS}
    kstep = {k: t / args.steps for k, (c, t) in kt.items() if c}
    launches = sum(_ffi.profile_kernels(k) for k in kt)  # kernels, not timed groups
    # e2e: pinned host values -> a grid, dual_contouring, mesh into pinned buffers
    pinned = torch.from_numpy(vals_np).pin_memory()
    egrid = iso.UniformGrid([n] * 3, device=dev)
    vh = torch.empty((capv, 3), dtype=torch.float32).pin_memory()
    fh = torch.empty((capf, 3), dtype=torch.int32).pin_memory()
    e2e_t, h2d_t, d2h_t = [], [], []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        egrid.set_values(pinned)
        t1 = time.perf_counter()
        vv, ff = iso.dual_contouring(egrid)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        vh[:len(vv)].copy_(vv)
        fh[:len(ff)].copy_(ff)
        t3 = time.perf_counter()
        if i >= args.warmup:
            e2e_t.append(t3 - t0)
            h2d_t.append(t1 - t0)
            d2h_t.append(t3 - t2)
    e2e_ms = 1e3 * statistics.mean(e2e_t)
    e2e_split = {"h2d_ms": round(1e3 * statistics.mean(h2d_t), 3), "d2h_ms": round(1e3 * statistics.mean(d2h_t), 3)}
    if rank != 0:
        return None
    pts, words = n ** 3, n * n * ((n + 31) // 32)
    # per kernel: the bitmap / values it must read and what it must write
    kbytes = {"mc_signs": 4 * pts + 4 * words, "dc_classify": 4 * words + 8 * words + 8 * A,
              "dc_solve": 4 * A + 32 * A + 12 * A + A, "dc_weld": A + 12 * A + 4 * A + 4 * A + 12 * nv,
              "dc_quads": 8 * A + 12 * A + 4 * A + 24 * Q}
    top = max(kstep, key=kstep.get)
    pk = peaks()
    achieved = kbytes[top] / (kstep[top] * 1e-3) / 1e9
    algo = 4 * pts + 12 * nv + 12 * nf
    out = {
        "metric": METRIC, "value": round(world * cells / (ms * 1e-3) / 1e9, 3), "unit": "Gcells/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": f"synthetic: sphere SDF |p|-{wl['r']} on [-1,1]^3",
        "config": {"workload": wl["desc"], "grid": [n, n, n], "cells": cells, "normals": "from the grid",
                   "vertices": nv, "faces": nf, "active_cells": A, "parallelism": f"replicas x{world}",
                   "tuned": {k: v_ for k, v_ in tuned["best"].items() if k.startswith("dc.")},
                   "tuning_ms": tuned["ms"],
                   "l2": f"inputs larger than L2 (values {4 * pts / 1e6:.0f} MB > 129 MB L2)"},
        "e2e": {"value": round(world * cells / (e2e_ms * 1e-3) / 1e9, 3), "unit": "Gcells/s",
                "ms_per_step": round(e2e_ms, 3), "h2d_bytes_per_step": 4 * pts, "d2h_bytes_per_step": 12 * (nv + nf),
                **e2e_split},
        "roofline": {"bound": "hbm", "kernel": top, "achieved": round(achieved, 1), "peak": pk["hbm_gbs"],
                     "unit": "GB/s", "frac": round(achieved / pk["hbm_gbs"], 4), "peak_source": pk["source"],
                     "algorithmic_bytes": kbytes[top], "kernel_ms": round(kstep[top], 4),
                     "traffic": profiled_traffic(wl["desc"], top),
                     "pipeline": {"algorithmic_bytes": algo, "achieved": round(algo / (ms * 1e-3) / 1e9, 1),
                                  "frac": round(algo / (ms * 1e-3) / 1e9 / pk["hbm_gbs"], 4)}},
        "kernel_ms": {k: round(v_, 4) for k, v_ in kstep.items()},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if not args.no_cpu:
        from oracle import Oracle

        threads = os.cpu_count() or 1
        sec = cpu_dc_slabs(Oracle(), vals_np, threads)
        out["cpu_baseline"] = {"value": round(cells / sec / 1e9, 5), "unit": "Gcells/s", "cores": threads,
                               "kind": "port",
                               "sample": f"one dual contouring of the same grid ({cells} cells): oracle C port "
                                         f"(FP64 QEF) over {threads} x-slabs on {threads} threads, {sec:.2f} s"}
    return out


def cpu_dc_slabs(ora, vals_np, threads: int) -> float:
    """Seconds for one dual contouring of the grid by the oracle's C port, split
    into x slabs (one point plane shared by neighbours, so each slab's cells are
    the grid's cells once) run on `threads` host threads (ctypes releases the
    GIL).  Quads whose four cells straddle two slabs are not formed: a timing of
    the same per-cell work, not a mesh."""
    import concurrent.futures as cf

    n = vals_np.shape[0]
    slabs = _slabs(n, threads)
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(lambda ab: ora.dc_dense(np.ascontiguousarray(vals_np[ab[0]:ab[1] + 1])), slabs))
    return time.perf_counter() - t0


def cpu_dc(ora, vals_np, shape) -> float:
    """Seconds for the oracle's C port of the same DC step on one host thread."""
    import torch

    from isoext_gb300 import sdf

    t0 = time.perf_counter()
    its = ora.intersection_dense(vals_np, normals=False)
    its["normals"] = sdf.get_sdf_normal(shape, torch.from_numpy(its["points"])).numpy()
    ora.dc(its, vals_np.shape, values=vals_np)
    return time.perf_counter() - t0


def cpu_baseline_dc(vals_np, shape, cells) -> dict:
    from oracle import Oracle

    sec = cpu_dc(Oracle(), vals_np, shape)
    return {"value": round(cells / sec / 1e9, 5), "unit": "Gcells/s", "cores": 1, "kind": "port",
            "sample": f"one full DC step of the same grid ({cells} cells): oracle C port (FP64 QEF solve), "
                      f"1 thread, {sec:.2f} s"}


def _slabs(n: int, parts: int):
    """x ranges [a, b] (point planes, inclusive) whose cells partition the grid's."""
    parts = max(1, min(parts, n - 1))
    cuts = [round(i * (n - 1) / parts) for i in range(parts + 1)]
    return [(cuts[i], cuts[i + 1]) for i in range(parts)]


def cpu_extract(ora, vals_np, threads: int) -> float:
    """Seconds for one extraction of the grid by the oracle's C port, split into
    x slabs (one point plane shared by neighbours) run on `threads` host threads.
    ctypes releases the GIL during each call, so the slabs run in parallel.  Each
    slab is welded on its own; its cells are the grid's cells exactly once."""
    import concurrent.futures as cf

    n = vals_np.shape[0]
    slabs = _slabs(n, threads)
    t0 = time.perf_counter()
    if threads == 1:
        ora.mc_dense(vals_np)
    else:
        with cf.ThreadPoolExecutor(max_workers=threads) as ex:
            list(ex.map(lambda ab: ora.mc_dense(np.ascontiguousarray(vals_np[ab[0]:ab[1] + 1])), slabs))
    return time.perf_counter() - t0


def cpu_baseline(vals_np, cells) -> dict:
    from oracle import Oracle

    ora = Oracle()
    threads = os.cpu_count() or 1
    sec = min(cpu_extract(ora, vals_np, threads) for _ in range(2))
    return {"value": round(cells / sec / 1e9, 5), "unit": "Gcells/s", "cores": threads, "kind": "port",
            "sample": f"one full extraction of the same grid ({cells} cells) per repeat, best of 2: "
                      f"oracle C port over {threads} x-slabs on {threads} threads, {sec:.3f} s"}


def run_reference(args, wl, rank) -> dict | None:
    if rank != 0:
        return None
    from oracle import Oracle

    if wl["kind"] in ("sparse", "grad", "serve", "dc1"):
        return run_reference_other(args, wl)
    n = wl["n"]
    if wl["kind"] == "dc":
        return run_reference_dc(args, wl)
    vals_np = sphere_values(n, wl["r"])
    cells = (n - 1) ** 3
    ora = Oracle()
    threads = os.cpu_count() or 1
    times = []
    for i in range(args.warmup + args.steps):
        dt = cpu_extract(ora, vals_np, threads)
        if i >= args.warmup:
            times.append(dt)
    sec = statistics.mean(times)
    val = round(cells / sec / 1e9, 5)
    return {
        "metric": METRIC, "impl": "reference", "value": val, "unit": "Gcells/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(sec * 1e3, 2),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: sphere SDF |p|-0.8 on [-1,1]^3",
        "config": {"workload": wl["desc"], "grid": [n, n, n], "cells": cells, "method": "nagae"},
        "cpu_baseline": {"value": val, "unit": "Gcells/s", "cores": threads, "kind": "port",
                         "sample": f"full grid per step as {threads} x-slabs on {threads} threads; the "
                                   "reference's algorithm restated in C (oracle/iso_oracle.c); isoext's "
                                   "sources are not on the GPU host"},
        "e2e": {"value": val, "unit": "Gcells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def _union_np(points, prims):
    """iso_sdf_union_grid's formula on the host (FP32 operations)."""
    f = np.float32
    d = np.full(points.shape[:-1], np.finfo(np.float32).max, np.float32)
    for row in prims.astype(np.float32):
        dx, dy, dz = (points[..., k] - row[1 + k] for k in range(3))
        if row[0] == 0:
            dk = np.sqrt((dx * dx + dy * dy) + dz * dz) - row[4]
        else:
            q = [np.abs(dx) - row[4], np.abs(dy) - row[5], np.abs(dz) - row[6]]
            o = [np.maximum(x, f(0)) for x in q]
            dk = np.sqrt((o[0] * o[0] + o[1] * o[1]) + o[2] * o[2]) + np.minimum(np.maximum(q[0], np.maximum(q[1], q[2])), f(0))
        d = np.minimum(d, dk.astype(np.float32))
    return d


def run_reference_other(args, wl) -> dict:
    """The oracle port (the reference's algorithms on the host) on a bounded
    sample of the sparse, grad or serve workload, all host threads."""
    import concurrent.futures as cf

    import torch
    from helpers import grid_points

    from oracle import Oracle

    ora = Oracle()
    threads = os.cpu_count() or 1
    if wl["kind"] == "dc1":
        m = 256  # a bounded sample of the same sphere, one slab per host thread
        sv = sphere_values(m, wl["r"])
        slabs = _slabs(m, threads)

        def one():
            with cf.ThreadPoolExecutor(max_workers=threads) as ex:
                list(ex.map(lambda ab: ora.dc_dense(np.ascontiguousarray(sv[ab[0]:ab[1] + 1])), slabs))
        units, unit, metric = (m - 1) ** 3 / 1e9, "Gcells/s", METRIC
        sample = f"the same sphere on {m}^3 per step as {threads} x-slabs on {threads} threads (oracle C port)"
    elif wl["kind"] == "sparse":
        import isoext_gb300 as iso

        g = iso.SparseGrid([wl["n"]] * 3, device="cpu")
        g.populate(smoothmin_spheres(wl), mode="brick", brick=wl["brick"])
        m = min(g.get_num_cells(), 4_000_000)
        ids, vals = g._ids[:m].numpy(), g._values[:m].numpy()
        cuts = np.linspace(0, m, threads + 1).astype(int)

        def one():
            with cf.ThreadPoolExecutor(max_workers=threads) as ex:
                list(ex.map(lambda i: ora.mc_sparse(ids[cuts[i]:cuts[i + 1]], vals[cuts[i]:cuts[i + 1]], g.shape),
                            range(threads)))
        units, unit, metric = m / 1e9, "Gcells/s", "sparse MC Gcells/s (active cells)"
        sample = f"the first {m} active cells of the populated grid per step, {threads} slices on {threads} threads"
    elif wl["kind"] == "grad":
        def one():
            cpu_baseline_grad(wl)
        units, unit, metric = 63 ** 3 / 1e9, "Gcells/s", "differentiable MC+DC Gcells/s (forward + backward)"
        sample = "one 64^3 crop per step: oracle forward topology + FP64 torch forward and autograd backward"
        threads = torch.get_num_threads()
    else:
        from isoext_gb300.serve import random_requests

        reqs = random_requests(16, wl["seed"], tuple(wl["sizes"]), wl["mc_share"])
        grids = {r.n: grid_points((r.n,) * 3) for r in reqs}
        vals = [_union_np(grids[r.n], r.prims) for r in reqs]

        def solve(i):
            r = reqs[i]
            if r.kind == "mc":
                ora.mc_dense(vals[i])
            else:
                ora.dc_dense(vals[i])

        def one():
            with cf.ThreadPoolExecutor(max_workers=threads) as ex:
                list(ex.map(solve, range(len(reqs))))
        units, unit, metric = len(reqs), "req/s", "served requests/s (mixed MC/DC stream)"
        sample = f"the first {len(reqs)} requests of the stream per step, one per host thread"
    times = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        one()
        if i >= args.warmup:
            times.append(time.perf_counter() - t0)
    sec = statistics.mean(times)
    val = round(units / sec, 6 if unit == "Gcells/s" else 1)
    return {
        "metric": metric, "impl": "reference", "value": val, "unit": unit, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(sec * 1e3, 2), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": {"workload": wl["desc"]},
        "cpu_baseline": {"value": val, "unit": unit, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": val, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def run_reference_dc(args, wl) -> dict:
    import torch
    from helpers import grid_points

    from oracle import Oracle

    n = wl["n"]
    shape = csg_sdf(wl["seed"])
    vals_np = shape(torch.from_numpy(grid_points((n, n, n)))).contiguous().numpy()
    cells = (n - 1) ** 3
    ora = Oracle()
    times = [cpu_dc(ora, vals_np, shape) for _ in range(args.warmup + args.steps)][args.warmup:]
    sec = statistics.mean(times)
    val = round(cells / sec / 1e9, 5)
    return {
        "metric": METRIC, "impl": "reference", "value": val, "unit": "Gcells/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(sec * 1e3, 2),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": f"synthetic: seeded CSG (box - sphere) U torus, seed {wl['seed']}, on [-1,1]^3",
        "config": {"workload": wl["desc"], "grid": [n, n, n], "cells": cells, "normals": "analytic (autograd)"},
        "cpu_baseline": {"value": val, "unit": "Gcells/s", "cores": 1, "kind": "port",
                         "sample": "full DC step per step on one thread; the reference's algorithm restated "
                                   "in C with an FP64 QEF solve (oracle/iso_oracle.c)"},
        "e2e": {"value": val, "unit": "Gcells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="mc512")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--mc-only", action="store_true",
                    help="mc512: leave out the DC 512^3 and served-stream blocks of the default line")
    ap.add_argument("--slots", type=int, default=None, help="serve workload: worker slots (default 8)")
    ap.add_argument("--quick", action="store_true",
                    help="no load phase before the timed region (for profiler runs; clocks are not sampled under load)")
    args = ap.parse_args()
    wl = dict(WORKLOADS[args.workload])
    if args.slots is not None and wl["kind"] == "serve":
        wl["slots"] = args.slots
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1 and args.impl == "ours":
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        dist.init_process_group("nccl")
    if args.impl == "reference":
        out = run_reference(args, wl, rank)
    else:
        out = run_ours(args, wl, rank, world)
    if out is not None:
        print(json.dumps(out), flush=True)
    if world > 1 and args.impl == "ours":
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
