"""Device-side tile work queue (libnpbgb's ``npbgb_queue_*``): grids added while it runs.

    q = TileQueue(max_slots=1024)
    slot = q.submit(A, B, TSTEPS)       # CUDA tensors (2D: Jacobi-2D, 3D: Heat-3D)
    q.kick()                            # starts the worker kernel if none runs
    ...
    for slot in q.poll():               # grids finished since the last poll
        ...

One persistent worker kernel claims tiles of grid half-sweeps from a ring in
device memory; grids submitted while it runs are taken in from an inbox in
pinned host memory, without a launch or a synchronisation per grid.  A grid
leaves the queue bit-identical to ``kernel(TSTEPS, A, B)`` of
polybench/jacobi_2d/jacobi_2d_numpy.py:4-10 or
polybench/heat_3d/heat_3d_numpy.py:4-20 run on it alone.  The tensors must
stay alive until their slot is reported by ``poll``.
"""
import ctypes

from . import _lib

__all__ = ["TileQueue"]


class TileQueue:
    def __init__(self, max_slots=1024, tile_rows=0, tile_planes=0, ctas_per_sm=0, idle_us=2000,
                 device=None):
        import torch
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None else \
            torch.device(device)
        self._h = None
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(_lib.load().npbgb_queue_create(int(max_slots), int(tile_rows),
                                                      int(tile_planes), int(ctas_per_sm),
                                                      int(idle_us), ctypes.byref(h)),
                       "npbgb_queue_create")
        self._h = h
        self.max_slots = int(max_slots)
        self._keep = {}
        self._buf = (ctypes.c_int32 * self.max_slots)()

    def submit(self, A, B, tsteps, step0=0, nsteps=0, band_rows=0, a32=None, b32=None):
        """Queue one grid; returns its slot, or -1 if it has nothing to do.

        With ``a32``/``b32`` (float32 tensors of A's shape), A and B are a
        float64 pair: the queue widens a32/b32 into them, runs the grid in
        float64 and rounds the result back into a32/b32."""
        import torch
        if self._h is None:
            raise RuntimeError("queue destroyed")
        if not (isinstance(A, torch.Tensor) and isinstance(B, torch.Tensor)):
            raise TypeError("queue grids must be CUDA tensors")
        if A.device != self.device or B.device != self.device:
            raise ValueError(f"queue grids must be on {self.device}")
        if A.dim() not in (2, 3) or A.shape != B.shape or A.dtype != B.dtype:
            raise ValueError("A and B must be 2D or 3D with equal shape and dtype")
        if not (A.is_contiguous() and B.is_contiguous()):
            raise ValueError("tensors must be contiguous")
        if A.dtype == torch.float64:
            code = _lib.NPBGB_F64
        elif A.dtype == torch.float32:
            code = _lib.NPBGB_F32
        else:
            raise TypeError(f"unsupported dtype {A.dtype}")
        g = _lib.Grid()
        g.a, g.b = A.data_ptr(), B.data_ptr()
        if A.dim() == 2:
            g.n0, g.n1, g.n2 = A.shape[0], A.shape[1], 1
            g.kind = _lib.NPBGB_KIND_JACOBI2D
        else:
            g.n0, g.n1, g.n2 = A.shape
            g.kind = _lib.NPBGB_KIND_HEAT3D
        g.dtype = code
        g.tsteps = int(tsteps)
        g.band_rows = int(band_rows)
        g.step0, g.nsteps = int(step0), int(nsteps)
        keep = (A, B)
        if a32 is not None or b32 is not None:
            if a32 is None or b32 is None:
                raise ValueError("give both a32 and b32")
            for x in (a32, b32):
                if (not isinstance(x, torch.Tensor) or x.dtype != torch.float32 or
                        x.shape != A.shape or x.device != self.device or not x.is_contiguous()):
                    raise ValueError("a32/b32 must be contiguous float32 tensors of A's shape "
                                     "on the queue's device")
            if A.dtype != torch.float64:
                raise TypeError("a grid with float32 arrays runs in float64: A and B must be "
                                "float64")
            g.a32, g.b32 = a32.data_ptr(), b32.data_ptr()
            keep = (A, B, a32, b32)
        slot = ctypes.c_int32(-1)
        _lib.check(_lib.load().npbgb_queue_submit(self._h, ctypes.byref(g), ctypes.byref(slot)),
                   "npbgb_queue_submit")
        if slot.value >= 0:
            self._keep[slot.value] = keep
        return slot.value

    def kick(self, stream=None):
        """Launch the worker on `stream` (default: the device's current stream) unless one runs."""
        import torch
        if stream is None:
            stream = torch.cuda.current_stream(self.device)
        ptr = stream.cuda_stream if hasattr(stream, "cuda_stream") else stream
        _lib.check(_lib.load().npbgb_queue_kick(self._h, ptr), "npbgb_queue_kick")

    def poll(self):
        """Slots finished since the last poll (their grids are complete on the device)."""
        n = ctypes.c_int32(0)
        _lib.check(_lib.load().npbgb_queue_poll(self._h, self._buf, self.max_slots,
                                                ctypes.byref(n)), "npbgb_queue_poll")
        out = [int(self._buf[i]) for i in range(n.value)]
        for s in out:
            self._keep.pop(s, None)
        return out

    def state(self):
        """{"running": bool, "busy": slots in use, "launches": worker launches so far}."""
        r, b, n = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int64()
        _lib.check(_lib.load().npbgb_queue_state(self._h, ctypes.byref(r), ctypes.byref(b),
                                                 ctypes.byref(n)), "npbgb_queue_state")
        return {"running": bool(r.value), "busy": b.value, "launches": n.value}

    def close(self):
        """No more grids: a running worker ends once the queued ones are done."""
        if self._h is not None:
            _lib.check(_lib.load().npbgb_queue_close(self._h), "npbgb_queue_close")

    def destroy(self):
        if self._h is not None:
            _lib.load().npbgb_queue_destroy(self._h)
            self._h = None
            self._keep.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.destroy()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass
