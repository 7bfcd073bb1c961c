"""Served extraction: continuous batching of marching-cubes and dual-contouring
requests on one GPU.

A request names a grid (cubic, ``n`` points per axis over [-1, 1]^3) given as
a union of spheres and boxes, and an extraction (``"mc"`` or ``"dc"``).  The
server keeps ``slots`` workers, each with its own CUDA stream and its own
device buffers, resident across requests.  Requests are admitted in arrival
order as soon as a slot is free and the device-memory budget holds the
request's worst case; the requests on different slots run concurrently on the
GPU.  A request replays a CUDA graph captured for its slot, kind and grid size:
grid evaluation + extraction, no host work in between (iso_mc_dense for
marching cubes, iso_dc_dense for dual contouring).  A mesh larger than the
slot's buffers reruns through the plain path.

Each result equals the one-call-per-grid result (``solve_plain``) bit for bit:
the same kernels run on the same inputs, only concurrently.

The scheduling (``Scheduler``) is plain host code, testable without a GPU.
"""

from __future__ import annotations

import concurrent.futures as cf
import ctypes as C
import threading
import time
from collections import deque
from dataclasses import dataclass

import numpy as np

from . import _ffi

_vp, _i, _fa = C.c_void_p, C.c_int, C.POINTER(C.c_float)
_ffi.register({"iso_sdf_union_grid": ([_vp, _i, _i, _i, _fa, _fa, _vp, _vp], _i)})

MAX_PRIMS = 32
DC_REG, DC_SVD_TOL = 1e-2, 1e-6  # dual_contouring's defaults (isoext)
LO, HI = (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0)


@dataclass
class Request:
    """kind "mc" or "dc"; n points per axis; prims float [k, 7] rows of
    (kind 0 sphere / 1 box, centre xyz, radius | half-extents xyz)."""

    kind: str
    n: int
    prims: np.ndarray
    level: float = 0.0
    method: str = "nagae"
    rid: int = 0


@dataclass
class Result:
    rid: int
    vertices: np.ndarray
    faces: np.ndarray
    t_submit: float
    t_start: float
    t_done: float
    slot: int = -1

    @property
    def latency(self) -> float:
        return self.t_done - self.t_submit


def prims_buffer(prims: np.ndarray) -> np.ndarray:
    """The device layout of iso_sdf_union_grid: [count, rows of 7 ...], padded."""
    p = np.asarray(prims, np.float32).reshape(-1, 7)
    if not 1 <= len(p) <= MAX_PRIMS:
        raise ValueError(f"a request has 1 .. {MAX_PRIMS} primitives")
    out = np.zeros(1 + 7 * MAX_PRIMS, np.float32)
    out[0] = len(p)
    out[1:1 + p.size] = p.ravel()
    return out


# Kernels of this library one request launches: marching cubes = grid evaluation
# + mc_signs, mc_count, mc_scan, mc_emit; dual contouring = grid evaluation +
# mc_signs, cell count, scan and write, solve, weld flags, scan and numbering,
# quads.
KERNELS_PER_REQUEST = {"mc": 5, "dc": 10}


# ---------------------------------------------------------------------------
# scheduling (host only)

class Scheduler:
    """FIFO admission of requests to `slots` workers under a byte budget.

    need(req) is the request's worst-case device memory; a request starts when a
    worker is free and the bytes of the running requests plus its own fit the
    budget.  The head of the queue waits for room: later requests never pass it.
    run(slot, req) performs the request and returns (vertices, faces)."""

    def __init__(self, slots: int, budget_bytes: int, need, run):
        if slots < 1:
            raise ValueError("slots >= 1")
        self.budget = int(budget_bytes)
        self._need, self._run = need, run
        self._queue: deque = deque()
        self._cv = threading.Condition()
        self._reserved = 0
        self._closed = False
        self.max_reserved = 0
        self.max_running = 0
        self._running = 0
        self._threads = [threading.Thread(target=self._worker, args=(i,), daemon=True) for i in range(slots)]
        for t in self._threads:
            t.start()

    def submit(self, req) -> cf.Future:
        need = int(self._need(req))
        if need > self.budget:
            raise ValueError(f"request needs {need} bytes, more than the budget {self.budget}")
        fut: cf.Future = cf.Future()
        with self._cv:
            if self._closed:
                raise RuntimeError("scheduler is closed")
            self._queue.append((req, need, fut, time.perf_counter()))
            self._cv.notify_all()
        return fut

    def _worker(self, slot: int) -> None:
        while True:
            with self._cv:
                while True:
                    if self._queue and self._reserved + self._queue[0][1] <= self.budget:
                        req, need, fut, t_submit = self._queue.popleft()
                        self._reserved += need
                        self._running += 1
                        self.max_reserved = max(self.max_reserved, self._reserved)
                        self.max_running = max(self.max_running, self._running)
                        break
                    if self._closed and not self._queue:
                        return
                    self._cv.wait()
            t_start = time.perf_counter()
            try:
                v, f = self._run(slot, req)
                fut.set_result(Result(getattr(req, "rid", 0), v, f, t_submit, t_start, time.perf_counter(), slot))
            except BaseException as exc:  # noqa: BLE001 - the future carries it
                fut.set_exception(exc)
            finally:
                with self._cv:
                    self._reserved -= need
                    self._running -= 1
                    self._cv.notify_all()

    def close(self) -> None:
        with self._cv:
            self._closed = True
            self._cv.notify_all()
        for t in self._threads:
            t.join()


# ---------------------------------------------------------------------------
# GPU execution

def _mc_caps(n: int) -> tuple[int, int]:
    # the faces of a closed surface inside the box stay below twice the grid's
    # face area in cells (and the output check catches the rest)
    f = 4 * 6 * (n - 1) ** 2 + 4096
    return f // 2 + 4096, f


def request_bytes(req: Request) -> int:
    """Worst-case device bytes of a request: grid values, workspace and outputs
    at the capacity bound."""
    from .dc import dc_workspace_bytes
    from .mc import workspace_bytes

    n = req.n
    cap_v, cap_f = _mc_caps(n)
    ws = (workspace_bytes if req.kind == "mc" else dc_workspace_bytes)((n, n, n), cap_v, cap_f)
    return 4 * n ** 3 + ws + 12 * cap_v + 12 * cap_f + 4096


class _GraphSlot:
    """A slot's buffers for one kind and grid size, and the captured graph
    (grid evaluation + iso_mc_dense or iso_dc_dense) that fills them."""

    def __init__(self, kind: str, n: int, method: int, level: float, prims_dev, stream, device, use_graph: bool):
        import torch

        from .dc import dc_workspace_bytes
        from .mc import workspace_bytes

        self.kind, self.n, self.method, self.level = kind, n, method, level
        self.cap_v, self.cap_f = _mc_caps(n)
        wsb = (workspace_bytes if kind == "mc" else dc_workspace_bytes)((n, n, n), self.cap_v, self.cap_f)
        self.values = torch.empty((n, n, n), dtype=torch.float32, device=device)
        self.vout = torch.empty((self.cap_v, 3), dtype=torch.float32, device=device)
        self.fout = torch.empty((self.cap_f, 3), dtype=torch.int32, device=device)
        self.ws = torch.empty(wsb, dtype=torch.uint8, device=device)
        self.small = torch.zeros(8, dtype=torch.int64, device=device)
        self.small_host = torch.zeros(8, dtype=torch.int64).pin_memory()
        self.prims_dev = prims_dev
        self.stream = stream
        self.graph = None
        if use_graph:
            with torch.cuda.stream(stream):
                self._launch()  # once outside the graph: module loading, first-use set-up
            stream.synchronize()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=stream, capture_error_mode="thread_local"):
                self._launch()
            self.graph = g

    def _launch(self):
        from .dc import dc_dense_into
        from .mc import mc_dense_into

        lib = _ffi.lib()
        s = self.stream.cuda_stream
        self.small.zero_()
        _ffi.check(lib.iso_sdf_union_grid(C.c_void_p(self.prims_dev.data_ptr()), self.n, self.n, self.n,
                                          _ffi.fvec3(LO), _ffi.fvec3(HI), C.c_void_p(self.values.data_ptr()),
                                          C.c_void_p(s)))
        if self.kind == "mc":
            _ffi.check(mc_dense_into(self.values, LO, HI, self.level, self.method, self.vout, self.fout, self.ws,
                                     self.small, s))
        else:
            _ffi.check(dc_dense_into(self.values, LO, HI, self.level, DC_REG, DC_SVD_TOL, self.vout, self.fout,
                                     self.ws, self.small, s))

    def run(self):
        """Returns (V, F, status) after the extraction; outputs stay on the device."""
        import torch

        with torch.cuda.stream(self.stream):
            if self.graph is not None:
                self.graph.replay()
            else:
                self._launch()
            self.small_host.copy_(self.small, non_blocking=True)
        self.stream.synchronize()
        h = self.small_host
        status = int(h[2] if self.kind == "mc" else h[6]) & 0xFFFFFFFF
        return int(h[0]), int(h[1]), status


class Server(Scheduler):
    """Continuous-batching server of Requests on one GPU.

    slots: concurrent workers (streams).  budget_bytes: device memory admitted
    at once (request_bytes per running request).  use_graphs: marching cubes
    replays a captured graph per slot and grid size."""

    def __init__(self, slots: int = 8, budget_bytes: int = 40 << 30, device=None, use_graphs: bool = True):
        import torch

        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.use_graphs = use_graphs
        self._slot_state = [dict() for _ in range(slots)]
        self._streams = [torch.cuda.Stream(self.device) for _ in range(slots)]
        self._prims_dev = [torch.zeros(1 + 7 * MAX_PRIMS, dtype=torch.float32, device=self.device)
                           for _ in range(slots)]
        self._prims_host = [torch.zeros(1 + 7 * MAX_PRIMS, dtype=torch.float32).pin_memory() for _ in range(slots)]
        self._lock = threading.Lock()  # graph capture is done one at a time
        super().__init__(slots, budget_bytes, request_bytes, self._execute)

    def warmup(self, sizes, method: str = "nagae", level: float = 0.0, tune: bool = True,
               kinds=("mc", "dc")) -> dict | None:
        """Builds every slot's buffers and graphs for the given grid sizes up front.
        With tune, the launch parameters are first tuned (isoext_gb300.tune) on a
        grid of the largest size, so the captured graphs use them; returns the
        tuning report."""
        import torch

        from .mc import method_id

        report = None
        if tune:
            from . import tune as tuner

            n = int(max(sizes))
            req = random_requests(1, seed=0, sizes=(n,))[0]
            prims = torch.from_numpy(prims_buffer(req.prims)).to(self.device)
            report = _tune_on(n, prims, self.device, level, tuner)
        for slot in range(len(self._streams)):
            for n in sizes:
                for kind in kinds:
                    self._slot(slot, kind, int(n), method_id(method), float(level))
        return report

    def _slot(self, slot: int, kind: str, n: int, method: int, level: float) -> _GraphSlot:
        key = (kind, n, method if kind == "mc" else 0, level)
        st = self._slot_state[slot]
        if key not in st:
            with self._lock:
                st[key] = _GraphSlot(kind, n, method, level, self._prims_dev[slot], self._streams[slot], self.device,
                                     self.use_graphs)
        return st[key]

    def _upload_prims(self, slot: int, prims) -> None:
        import torch

        host = self._prims_host[slot]
        host.copy_(torch.from_numpy(prims_buffer(prims)))
        with torch.cuda.stream(self._streams[slot]):
            self._prims_dev[slot].copy_(host, non_blocking=True)

    def _execute(self, slot: int, req: Request):
        import torch

        from .mc import method_id

        stream = self._streams[slot]
        self._upload_prims(slot, req.prims)
        gs = self._slot(slot, req.kind, req.n, method_id(req.method), float(req.level))
        V, F, status = gs.run()
        if status == _ffi.ISO_ERR_OVERFLOW:
            # larger than the slot's buffers: the plain path on this stream
            with torch.cuda.stream(stream):
                return _solve_on_stream(req, self._prims_dev[slot], self.device)
        if status != 0:
            raise RuntimeError(f"isoext_gb300: device error {status} in a served request")
        if V == 0 or F == 0:
            return np.zeros((0, 3), np.float32), np.zeros((0, 3), np.int32)
        with torch.cuda.stream(stream):
            v = gs.vout[:V].to("cpu").numpy().copy()
            f = gs.fout[:F].to("cpu").numpy().copy()
        return v, f


class _ServeRequest(C.Structure):
    _fields_ = [("kind", C.c_int), ("n", C.c_int), ("method", C.c_int), ("level", C.c_float),
                ("num_prims", C.c_int), ("prims", C.POINTER(C.c_float))]


class _ServeResult(C.Structure):
    _fields_ = [("ticket", C.c_longlong), ("status", C.c_int), ("slot", C.c_int), ("num_vertices", C.c_longlong),
                ("num_faces", C.c_longlong), ("vertices", C.POINTER(C.c_float)), ("faces", C.POINTER(C.c_int)),
                ("t_submit", C.c_double), ("t_start", C.c_double), ("t_done", C.c_double)]


_ffi.register({
    "iso_serve_create": ([C.c_int, C.c_longlong, C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_void_p)], C.c_int),
    "iso_serve_submit": ([C.c_void_p, C.POINTER(_ServeRequest)], C.c_longlong),
    "iso_serve_wait": ([C.c_void_p, C.c_longlong, C.c_double, C.POINTER(_ServeResult)], C.c_int),
    "iso_serve_free_result": ([C.POINTER(_ServeResult)], None),
    "iso_serve_stats": ([C.c_void_p, C.POINTER(C.c_longlong)], C.c_int),
    "iso_serve_stats_ex": ([C.c_void_p, C.POINTER(C.c_longlong), C.c_int], C.c_int),
    "iso_serve_destroy": ([C.c_void_p], C.c_int),
    "iso_serve_set_capacity_scale": ([C.c_void_p, C.c_double], C.c_int),
    "iso_serve_set_bucket": ([C.c_void_p, C.c_int], C.c_int),
})


class _NativeFuture:
    def __init__(self, server, ticket: int, rid: int):
        self._server, self._ticket, self._rid = server, ticket, rid
        self._result = None

    def result(self, timeout: float | None = None) -> Result:
        if self._result is None:
            self._result = self._server._wait(self._ticket, self._rid, timeout)
        return self._result


class NativeServer:
    """The served loop in C++ (iso_serve_*): worker threads, streams, per-slot
    buffers and CUDA graphs and the admission all run natively, without the
    Python interpreter; Python submits requests and collects meshes.  Same
    requests and results as Server (and solve_plain), bit for bit.

    Device memory stays within budget_bytes, cached buffers included: entries
    are sized from a count pass on their first request, evicted least recently
    used when a new one needs room, and grown when a later mesh is larger.

    warm_sizes: grid sizes whose buffers and graphs are built up front (the
    launch parameters are tuned first on the largest, as Server.warmup does).
    bucket: requests of one kind, grid size, method and level that one launch
    may run together (1, 2, 4 or 8; a graph with a parallel branch per
    request)."""

    def __init__(self, slots: int = 8, budget_bytes: int = 40 << 30, warm_sizes=(), tune: bool = True,
                 device=None, bucket: int = 1):
        import torch

        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.tuned = None
        torch.cuda.set_device(self.device)
        if tune and warm_sizes:
            from . import tune as tuner

            n = int(max(warm_sizes))
            req = random_requests(1, seed=0, sizes=(n,))[0]
            prims = torch.from_numpy(prims_buffer(req.prims)).to(self.device)
            self.tuned = _tune_on(n, prims, self.device, 0.0, tuner)
        sizes = (C.c_int * max(1, len(warm_sizes)))(*[int(n) for n in warm_sizes])
        handle = C.c_void_p()
        _ffi.check(_ffi.lib().iso_serve_create(int(slots), int(budget_bytes), sizes, len(warm_sizes), C.byref(handle)))
        self._h = handle
        self.budget = int(budget_bytes)
        if bucket != 1:
            _ffi.check(_ffi.lib().iso_serve_set_bucket(self._h, int(bucket)))

    def submit(self, req: Request) -> _NativeFuture:
        p = np.ascontiguousarray(np.asarray(req.prims, np.float32).reshape(-1, 7))
        from .mc import method_id

        q = _ServeRequest(0 if req.kind == "mc" else 1, int(req.n), method_id(req.method), float(req.level), len(p),
                          p.ctypes.data_as(C.POINTER(C.c_float)))
        t = _ffi.lib().iso_serve_submit(self._h, C.byref(q))
        if t < 0:
            if -t == _ffi.ISO_ERR_WORKSPACE:
                raise ValueError(f"request needs more than the budget {self.budget}")
            raise ValueError(f"isoext_gb300: request refused (error {-t})")
        return _NativeFuture(self, int(t), req.rid)

    def _wait(self, ticket: int, rid: int, timeout: float | None) -> Result:
        r = _ServeResult()
        rc = _ffi.lib().iso_serve_wait(self._h, ticket, -1.0 if timeout is None else float(timeout), C.byref(r))
        if rc == _ffi.ISO_ERR_TIMEOUT:
            raise TimeoutError(f"request {rid} not done after {timeout} s")
        _ffi.check(rc)
        try:
            if r.status:
                raise RuntimeError(f"isoext_gb300: device error {r.status} in a served request")
            V, F = int(r.num_vertices), int(r.num_faces)
            v = np.ctypeslib.as_array(r.vertices, shape=(V, 3)).copy() if V else np.zeros((0, 3), np.float32)
            f = np.ctypeslib.as_array(r.faces, shape=(F, 3)).copy() if F else np.zeros((0, 3), np.int32)
        finally:
            _ffi.lib().iso_serve_free_result(C.byref(r))
        return Result(rid, v, f, r.t_submit, r.t_start, r.t_done, int(r.slot))

    def stats(self) -> dict:
        """Counters of the loop.  Device bytes: every byte the server holds
        (slot buffers and cached entries) counts against the budget."""
        s = (C.c_longlong * 12)()
        _ffi.check(_ffi.lib().iso_serve_stats_ex(self._h, s, 12))
        return {"completed": s[0], "max_running": s[1], "max_held_bytes": s[2], "max_admitted_bytes": s[2],
                "queued": s[3], "held_bytes": s[4], "evictions": s[5], "entries": s[6], "count_passes": s[7],
                "grown": s[8], "budget": s[9], "bucket_launches": s[10], "bucketed_requests": s[11]}

    @property
    def max_running(self) -> int:
        return int(self.stats()["max_running"])

    @property
    def max_reserved(self) -> int:
        return int(self.stats()["max_admitted_bytes"])

    def close(self) -> None:
        if self._h:
            _ffi.lib().iso_serve_destroy(self._h)
            self._h = None


def _tune_on(n: int, prims_dev, device, level: float, tuner) -> dict:
    """Tunes the launch parameters on an n^3 grid of the union in prims_dev."""
    import torch

    from .grids import UniformGrid

    grid = UniformGrid([n] * 3, LO, HI, device=device)
    s = torch.cuda.current_stream(device).cuda_stream
    _ffi.check(_ffi.lib().iso_sdf_union_grid(C.c_void_p(prims_dev.data_ptr()), n, n, n, _ffi.fvec3(LO),
                                             _ffi.fvec3(HI), C.c_void_p(grid._values.data_ptr()), C.c_void_p(s)))
    return tuner.autotune(grid, level, repeats=5)


def _solve_on_stream(req: Request, prims_dev, device):
    """The public API on the current stream: grid from the union, then
    marching_cubes or dual_contouring (isoext's defaults); results copied to the host."""
    import torch

    from .dc import dual_contouring
    from .grids import UniformGrid
    from .mc import marching_cubes

    n = req.n
    grid = UniformGrid([n] * 3, LO, HI, device=device)
    s = torch.cuda.current_stream(device).cuda_stream
    _ffi.check(_ffi.lib().iso_sdf_union_grid(C.c_void_p(prims_dev.data_ptr()), n, n, n, _ffi.fvec3(LO),
                                             _ffi.fvec3(HI), C.c_void_p(grid._values.data_ptr()), C.c_void_p(s)))
    if req.kind == "mc":
        v, f = marching_cubes(grid, req.level, req.method)
    else:
        v, f = dual_contouring(grid, req.level, reg=DC_REG, svd_tol=DC_SVD_TOL)
    if v is None:
        return np.zeros((0, 3), np.float32), np.zeros((0, 3), np.int32)
    return v.cpu().numpy(), f.cpu().numpy()


def solve_plain(req: Request, device=None):
    """The one-call-per-grid path: one request at a time on the current stream."""
    import torch

    device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    prims_dev = torch.from_numpy(prims_buffer(req.prims)).to(device)
    return _solve_on_stream(req, prims_dev, device)


def random_requests(count: int, seed: int, sizes=(64, 96, 128, 192, 256), mc_share: float = 0.7):
    """The mixed stream: grid edge uniform over `sizes`, mc with probability
    mc_share, each grid a union of 1..16 spheres / boxes of size U[0.05, 0.4]
    centred in U[-0.5, 0.5]^3 (seeded)."""
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(count):
        k = int(rng.integers(1, 17))
        prims = np.zeros((k, 7), np.float32)
        prims[:, 0] = rng.integers(0, 2, size=k)
        prims[:, 1:4] = rng.uniform(-0.5, 0.5, size=(k, 3))
        size = rng.uniform(0.05, 0.4, size=(k, 1))
        # spheres use the first size; boxes get three half-extents around it
        prims[:, 4:7] = np.where(prims[:, :1] == 0, size, size * rng.uniform(0.5, 1.0, size=(k, 3)))
        kind = "mc" if rng.random() < mc_share else "dc"
        reqs.append(Request(kind, int(rng.choice(sizes)), prims, rid=i))
    return reqs
