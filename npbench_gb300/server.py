"""Continuous-batching server for stencil solves on one GPU.

A request is one grid solve, the reference's ``kernel(TSTEPS, A, B)`` of
polybench/jacobi_2d/jacobi_2d_numpy.py:4-10 (2D) or
polybench/heat_3d/heat_3d_numpy.py:4-20 (3D), in float32 or float64, with its
own size and step count.

Requests flow through four stages, each advanced by the serving thread
without ever waiting for the GPU:

* **admission**: queued requests are admitted oldest first while their device
  arrays fit in the HBM budget (``AdmissionController``); their arrays are
  allocated and their inputs uploaded on a copy stream (an event marks the
  upload done);
* **dispatch**: an uploaded grid below ``direct_cells`` cells is folded into
  the device-side tile work queue (``npbench_gb300.queue``, libnpbgb's
  ``npbgb_queue_*``), whose persistent worker kernel takes it in while it runs:
  its tiles interleave with those of every other small grid, whatever their
  sizes, kinds and precisions, and its next half-sweep starts as soon as its
  own previous one is done.  A larger grid fills the GPU by itself and goes to
  a big-grid lane (its own stream) that runs it with the tuned single-grid
  kernels (TMA pipelines, the binary64 Jacobi-2D loop in one launch), in
  the tuned lane order; the queue's CTAs share the SMs with those launches;
* **completion**: the worker writes a completion word to host memory when a
  grid's last half-sweep is done, and a lane records an event; the serving
  thread polls both;
* **return**: results are copied back on the copy stream (or handed over as
  device tensors), the budget is released and the future resolved.

Arrivals never wait for a round to end: the worker kernel keeps running while
new grids are folded in (and ends by itself only when it has nothing left),
and small requests never wait behind a large one.

**Float64 guard.**  A float32 request whose float32 error against float64 is
predicted to exceed NPBench's acceptance bound (``npbench_gb300.precision``)
runs in float64 on the GPU: the queue widens its float32 inputs exactly,
sweeps in float64 and rounds the result to float32 once.  ``run_sequential``,
the comparator (the same requests one at a time with plain per-grid launches,
in arrival order), applies the same guard.

A grid's result is the same alone and in the mix, bit for bit (the tests check
it): the queue applies the same arithmetic in the same order per point.
"""
import collections
import concurrent.futures
import itertools
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import _lib, precision, stencils

__all__ = ["AdmissionController", "Request", "StencilServer", "run_sequential", "latency_stats",
           "guarded"]


class AdmissionController:
    """Byte budget for resident grids.  Host logic only (no GPU)."""

    def __init__(self, budget_bytes):
        if budget_bytes <= 0:
            raise ValueError("budget must be positive")
        self.budget = int(budget_bytes)
        self.in_use = 0
        self.peak = 0
        self._lock = threading.Lock()

    def fits_ever(self, nbytes):
        return nbytes <= self.budget

    def try_admit(self, nbytes):
        with self._lock:
            if self.in_use + nbytes > self.budget:
                return False
            self.in_use += nbytes
            self.peak = max(self.peak, self.in_use)
            return True

    def release(self, nbytes):
        with self._lock:
            if nbytes > self.in_use:
                raise RuntimeError("released more bytes than admitted")
            self.in_use -= nbytes


def guarded(kind, dtype, tsteps, fp64_guard=True):
    """True when a request of this kind, dtype and TSTEPS runs in float64 for accuracy."""
    return (fp64_guard and np.dtype(dtype) == np.float32 and
            precision.needs_fp64(kind, int(tsteps)))


@dataclass
class Request:
    """One solve.  Give host arrays ``a`` (and ``b`` for 2D), or a ``seed``
    from which the server draws U[0,1) inputs on the device."""
    shape: tuple
    dtype: object
    tsteps: int
    a: np.ndarray = None
    b: np.ndarray = None
    seed: int = None
    return_host: bool = True
    # filled in by the server
    id: int = -1
    t_submit: float = 0.0
    t_admit: float = 0.0
    t_done: float = 0.0
    promoted: bool = False
    path: str = ""        # "queue" (tile queue) or "lane" (big-grid lane)
    dev: dict = field(default=None, repr=False)
    out: tuple = field(default=None, repr=False)
    future: concurrent.futures.Future = field(default=None, repr=False)

    @property
    def kind(self):
        return "jacobi2d" if len(self.shape) == 2 else "heat3d"

    @property
    def cells(self):
        return int(np.prod(self.shape))

    @property
    def nbytes(self):
        """Device bytes while resident: the pair in the request's dtype, plus the
        float64 pair of a promoted float32 request."""
        n = 2 * self.cells * np.dtype(self.dtype).itemsize
        return n + (2 * self.cells * 8 if self.promoted else 0)

    @property
    def updates(self):
        inner = int(np.prod([max(0, s - 2) for s in self.shape]))
        return max(0, 2 * (self.tsteps - 1)) * inner


def _validate(req):
    if len(req.shape) not in (2, 3):
        raise ValueError("requests are 2D (Jacobi) or 3D (heat) grids")
    if np.dtype(req.dtype) not in (np.dtype(np.float32), np.dtype(np.float64)):
        raise TypeError(f"unsupported dtype {req.dtype}")
    if req.a is None and req.seed is None:
        raise ValueError("a request needs input arrays or a seed")
    if req.a is not None:
        if tuple(req.a.shape) != tuple(req.shape):
            raise ValueError("input shape does not match the request")
        if len(req.shape) == 2 and req.b is None:
            raise ValueError("Jacobi-2D requests need both A and B")


def _tdtype(dtype):
    import torch
    return torch.float64 if np.dtype(dtype) == np.float64 else torch.float32


def _materialise(req, device, stream=None):
    """Device arrays (A, B) of a request in its dtype, inputs uploaded or drawn on
    `stream` (default: the current stream)."""
    import torch
    tdt = _tdtype(req.dtype)
    ctx = torch.cuda.stream(stream) if stream is not None else _nullctx()
    with ctx:
        if req.a is not None:
            A = torch.empty(req.shape, dtype=tdt, device=device)
            A.copy_(_host(req.a, req.dtype), non_blocking=True)
            B = torch.empty_like(A)
            B.copy_(_host(req.b if req.b is not None else req.a, req.dtype), non_blocking=True)
        else:
            g = torch.Generator(device=device)
            g.manual_seed(int(req.seed))
            A = torch.rand(req.shape, dtype=torch.float64, device=device, generator=g).to(tdt)
            B = (torch.rand(req.shape, dtype=torch.float64, device=device, generator=g).to(tdt)
                 if len(req.shape) == 2 else A.clone())
    return A, B


class _nullctx:
    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False


def _host(x, dtype):
    import torch
    arr = np.ascontiguousarray(x, dtype=dtype)
    t = torch.from_numpy(arr)
    return t


class StencilServer:
    """Serving thread with an HBM admission budget, feeding the device-side tile queue."""

    def __init__(self, device=0, hbm_budget_bytes=150e9, max_slots=4096, tile_rows=0,
                 tile_planes=0, ctas_per_sm=None, idle_us=500, fp64_guard=True,
                 reserve_bytes=8 << 30, poll_s=2e-4, direct_cells=None, big_lanes=None,
                 lane_order=None, age_s=0.25):
        """direct_cells (grids from this many cells go to a big-grid lane),
        ctas_per_sm (the queue worker's CTAs per SM), big_lanes (big grids run
        concurrently, one per lane) and lane_order ("sjf": shortest job first;
        "fifo"; "aged": shortest first unless the oldest has waited longer than
        age_s) default to the tuned settings of the serving loop
        (``autotune.server_settings``)."""
        from . import autotune
        tuned = autotune.server_settings()
        direct_cells = tuned["direct_cells"] if direct_cells is None else direct_cells
        ctas_per_sm = tuned["ctas_per_sm"] if ctas_per_sm is None else ctas_per_sm
        big_lanes = tuned["big_lanes"] if big_lanes is None else big_lanes
        lane_order = tuned.get("lane_order", "sjf") if lane_order is None else lane_order
        import torch
        self.device = torch.device("cuda", device) if isinstance(device, int) else \
            torch.device(device)
        self.admission = AdmissionController(hbm_budget_bytes)
        self.max_slots = int(max_slots)
        self.tile_rows, self.tile_planes = int(tile_rows), int(tile_planes)
        self.ctas_per_sm, self.idle_us = int(ctas_per_sm), int(idle_us)
        self.fp64_guard = bool(fp64_guard)
        self.reserve_bytes = int(min(reserve_bytes, hbm_budget_bytes))
        self.poll_s = float(poll_s)
        self.direct_cells = int(direct_cells)
        self.big_lanes = max(1, int(big_lanes))
        if lane_order not in ("sjf", "fifo", "aged"):
            raise ValueError("lane_order: 'sjf' (shortest job first), 'fifo' or 'aged' "
                             "(shortest first, but a job waiting longer than age_s goes first)")
        self.lane_order = lane_order
        self.age_s = float(age_s)
        self.queued_small = self.ran_big = 0
        self._queue = collections.deque()
        self._cv = threading.Condition()
        self._stop = False
        self._ids = itertools.count()
        self._thread = None
        self.completed = []
        self.error = None
        self.promoted = 0
        self.launches = 0

    # -- client side ------------------------------------------------------
    def submit(self, req):
        _validate(req)
        req.promoted = guarded(req.kind, req.dtype, req.tsteps, self.fp64_guard)
        if not self.admission.fits_ever(req.nbytes):
            raise ValueError(f"request needs {req.nbytes} bytes, above the HBM budget "
                             f"{self.admission.budget}")
        req.id = next(self._ids)
        req.t_submit = time.perf_counter()
        req.future = concurrent.futures.Future()
        with self._cv:
            if self._stop:
                raise RuntimeError("server stopped")
            if self.error is not None:
                raise RuntimeError("server failed") from self.error
            self._queue.append(req)
            self._cv.notify()
        return req.future

    def start(self):
        _lib.load()
        self._thread = threading.Thread(target=self._serve, name="npbgb-server", daemon=True)
        self._thread.start()
        return self

    def stop(self, drain=True):
        """Stop after the queued and resident requests finish (drain) or now."""
        with self._cv:
            self._stop = True
            if not drain:
                for r in list(self._queue):
                    r.future.cancel()
                self._queue.clear()
            self._cv.notify()
        if self._thread is not None:
            self._thread.join()

    def __enter__(self):
        return self.start()

    def __exit__(self, *exc):
        self.stop(drain=exc[0] is None)

    # -- serving thread ---------------------------------------------------
    def _upload(self, req):
        """Allocates the request's device arrays and queues its input upload."""
        import torch
        A, B = _materialise(req, self.device, self._copy)
        dev = {"A": A, "B": B}
        if req.promoted:
            with torch.cuda.stream(self._copy):
                dev["A64"] = torch.empty(req.shape, dtype=torch.float64, device=self.device)
                dev["B64"] = torch.empty(req.shape, dtype=torch.float64, device=self.device)
        ev = torch.cuda.Event()
        ev.record(self._copy)
        req.dev = dev
        return ev

    def _fold(self, req):
        """Hands an uploaded grid to the tile queue; returns its slot (-1: nothing to do)."""
        d = req.dev
        if req.promoted:
            return self.tq.submit(d["A64"], d["B64"], req.tsteps, a32=d["A"], b32=d["B"])
        return self.tq.submit(d["A"], d["B"], req.tsteps)

    def _pick(self, ready):
        """The next large grid for a free lane (``ready`` is in arrival order)."""
        if self.lane_order == "fifo":
            return ready[0]
        if self.lane_order == "aged":
            now = time.perf_counter()
            if now - ready[0].t_submit > self.age_s:
                return ready[0]  # the oldest has waited long enough: it goes first
        return min(ready, key=lambda r: r.updates)  # shortest job first

    def _run_big(self, req, stream):
        """Queues a large grid's whole run on a big-grid lane; returns its end event."""
        import torch
        d = req.dev
        fn = stencils.jacobi_2d_kernel if len(req.shape) == 2 else stencils.heat_3d_kernel
        with torch.cuda.stream(stream):
            if req.promoted:
                _lib.convert(d["A64"], d["A"], stream)
                _lib.convert(d["B64"], d["B"], stream)
                fn(req.tsteps, d["A64"], d["B64"])
                _lib.convert(d["A"], d["A64"], stream)
                _lib.convert(d["B"], d["B64"], stream)
            else:
                fn(req.tsteps, d["A"], d["B"])
        ev = torch.cuda.Event()
        ev.record(stream)
        return ev

    def _deliver(self, req):
        """Starts returning a finished request's result; returns an event that marks it."""
        import torch
        A, B = req.dev["A"], req.dev["B"]
        if req.return_host:
            with torch.cuda.stream(self._copy):
                hA = torch.empty(A.shape, dtype=A.dtype, pin_memory=True)
                hB = torch.empty(B.shape, dtype=B.dtype, pin_memory=True)
                hA.copy_(A, non_blocking=True)
                hB.copy_(B, non_blocking=True)
            req.out = (hA, hB)
        else:
            req.out = (A, B)
        ev = torch.cuda.Event()
        ev.record(self._copy)
        return ev

    def _resolve(self, req):
        if req.return_host:
            out = (req.out[0].numpy(), req.out[1].numpy())
        else:
            out = req.out
        req.dev = None
        req.out = None
        self.admission.release(req.nbytes)
        req.t_done = time.perf_counter()
        self.completed.append(req)
        req.future.set_result(out)

    def _serve(self):
        import torch

        from .queue import TileQueue
        torch.cuda.set_device(self.device)
        self._copy = torch.cuda.Stream(self.device)
        self._compute = torch.cuda.Stream(self.device)
        if self.reserve_bytes > 0:
            # One cached block for the copy stream's allocations: later arrays are
            # carved out of it without a cudaMalloc while the worker runs.
            with torch.cuda.stream(self._copy):
                blk = torch.empty(self.reserve_bytes, dtype=torch.uint8, device=self.device)
            del blk
        self.tq = TileQueue(max_slots=self.max_slots, tile_rows=self.tile_rows,
                            tile_planes=self.tile_planes, ctas_per_sm=self.ctas_per_sm,
                            idle_us=self.idle_us, device=self.device)
        lanes = [{"stream": torch.cuda.Stream(self.device), "req": None, "ev": None}
                 for _ in range(self.big_lanes)]
        staging = []     # (request, upload event)
        big_ready = []   # uploaded large grids waiting for a lane
        resident = {}    # slot -> request
        returning = []   # (request, delivery event)
        try:
            while True:
                with self._cv:
                    busy = any(ln["req"] is not None for ln in lanes)
                    if self._stop and not (self._queue or staging or big_ready or resident or
                                           returning or busy):
                        return
                moved = False
                # admission, oldest first; later requests wait behind one that does not fit
                # (a request leaves the client queue only once admitted, so stop(drain=False)
                # can still cancel the rest)
                while True:
                    with self._cv:
                        if not self._queue:
                            break
                        req = self._queue[0]
                        if req.future.cancelled():
                            self._queue.popleft()
                            continue
                        if not self.admission.try_admit(req.nbytes):
                            break
                        self._queue.popleft()
                    req.t_admit = time.perf_counter()
                    self.promoted += int(req.promoted)
                    staging.append((req, self._upload(req)))
                    moved = True
                # dispatch: large grids to a lane, small ones into the running queue
                still = []
                for req, ev in staging:
                    if not ev.query():
                        still.append((req, ev))
                        continue
                    if req.cells >= self.direct_cells and req.updates > 0:
                        req.path = "lane"
                        big_ready.append(req)
                        moved = True
                        continue
                    try:
                        slot = self._fold(req)
                    except _lib.NpbgbError as e:
                        if e.status != _lib.NPBGB_ERR_NOMEM:
                            raise
                        still.append((req, ev))  # every slot busy: fold it later
                        continue
                    moved = True
                    if slot < 0:
                        returning.append((req, self._deliver(req)))
                    else:
                        resident[slot] = req
                        req.path = "queue"
                        self.queued_small += 1
                staging = still
                for ln in lanes:
                    if ln["req"] is not None and ln["ev"].query():
                        returning.append((ln["req"], self._deliver(ln["req"])))
                        ln["req"] = None
                        moved = True
                    if ln["req"] is None and big_ready:
                        nxt = self._pick(big_ready)
                        big_ready.remove(nxt)
                        ln["req"], ln["ev"] = nxt, self._run_big(nxt, ln["stream"])
                        self.ran_big += 1
                        moved = True
                if resident:
                    self.tq.kick(self._compute)
                    for slot in self.tq.poll():
                        req = resident.pop(slot)
                        returning.append((req, self._deliver(req)))
                        moved = True
                still = []
                for req, ev in returning:
                    if ev.query():
                        self._resolve(req)
                        moved = True
                    else:
                        still.append((req, ev))
                returning = still
                if not moved:
                    with self._cv:
                        if not self._stop:
                            self._cv.wait(timeout=self.poll_s)
        except Exception as e:  # fail every outstanding request loudly
            self.error = e
            with self._cv:
                pending = list(self._queue) + [r for r, _ in staging] + big_ready + \
                    list(resident.values()) + [r for r, _ in returning] + \
                    [ln["req"] for ln in lanes if ln["req"] is not None]
                self._queue.clear()
            for r in pending:
                if not r.future.done():
                    r.future.set_exception(e)
        finally:
            try:
                self.launches = self.tq.state()["launches"]
            except Exception:
                pass
            self.tq.destroy()


def run_sequential(requests, arrivals, device=0, fp64_guard=True):
    """Comparator: the requests one at a time, in arrival order, each with plain
    per-grid launches (``stencils.jacobi_2d_kernel`` / ``heat_3d_kernel``), under
    the same float64 guard as the server.  ``arrivals`` are offsets in seconds
    from the start.  Returns the requests with t_submit/t_done filled in."""
    import torch
    dev = torch.device("cuda", device) if isinstance(device, int) else device
    t0 = time.perf_counter()
    for req, at in zip(requests, arrivals):
        now = time.perf_counter() - t0
        if at > now:
            time.sleep(at - now)
        req.t_submit = t0 + at
        req.promoted = guarded(req.kind, req.dtype, req.tsteps, fp64_guard)
        A, B = _materialise(req, dev)
        fn = stencils.jacobi_2d_kernel if A.dim() == 2 else stencils.heat_3d_kernel
        if req.promoted:
            A64, B64 = A.double(), B.double()
            fn(req.tsteps, A64, B64)
            A.copy_(A64)
            B.copy_(B64)
            del A64, B64
        else:
            fn(req.tsteps, A, B)
        if req.return_host:
            req.out = (A.cpu().numpy(), B.cpu().numpy())
        else:
            req.out = (A, B)
        torch.cuda.synchronize(dev)
        req.t_done = time.perf_counter()
    return requests


def latency_stats(requests):
    lat = np.array([r.t_done - r.t_submit for r in requests])
    if lat.size == 0:
        return {"p50_ms": None, "p99_ms": None, "count": 0}
    span = max(r.t_done for r in requests) - min(r.t_submit for r in requests)
    ups = sum(r.updates for r in requests)
    return {"count": int(lat.size), "p50_ms": float(np.percentile(lat, 50) * 1e3),
            "p99_ms": float(np.percentile(lat, 99) * 1e3), "mean_ms": float(lat.mean() * 1e3),
            "span_s": float(span), "updates": int(ups),
            "updates_per_s": float(ups / span) if span > 0 else None}
