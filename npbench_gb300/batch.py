"""Many independent grids advanced by one persistent launch (libnpbgb batches).

    with Batch([(A0, B0, T0), (A1, B1, T1), ...]) as batch:
        batch.launch()              # one counter reset + one cooperative persistent kernel
        batch.launch(graph=True)    # the same, captured once into a CUDA graph and replayed

Batches of 2^24 cells or more run in the stepped form (one chained launch per
half-sweep over all grids still active), smaller ones in the persistent form;
``mode="queue"`` runs the batch as one launch of the device-side tile work
queue, and NPBGB_CFG_BATCH_MODE or ``mode`` forces any form.  ``guard=True``
runs float32 grids whose float32 error would exceed NPBench's bound in float64
(stepped or queue form).  Every entry (A, B, TSTEPS) is a pair of CUDA tensors of one dtype (float32 or
float64) with its own step count: 2D pairs are Jacobi-2D grids, 3D pairs
Heat-3D grids.  After a launch each pair holds what ``kernel(TSTEPS, A, B)``
of polybench/jacobi_2d/jacobi_2d_numpy.py:4-10 or
polybench/heat_3d/heat_3d_numpy.py:4-20 leaves, bit for bit.  An entry
(A, B, TSTEPS, step0, nsteps) resumes a run after step0 half-sweeps and
performs at most nsteps (0 = all remaining).  The tensors must stay alive
while the batch is used.
"""
import ctypes
import threading

from . import _lib

__all__ = ["Batch"]

_MODES = {None: 0, "auto": 0, "persistent": _lib.NPBGB_BATCH_PERSISTENT,
          "stepped": _lib.NPBGB_BATCH_STEPPED, "queue": _lib.NPBGB_BATCH_QUEUE}
_plan_lock = threading.Lock()


def _planned(mode, fn):
    """Runs fn() (a create or replan) with the batch form `mode` in force."""
    code = _MODES[mode]
    if code == 0:
        return fn()
    with _plan_lock:
        old = _lib.set_config(_lib.NPBGB_CFG_BATCH_MODE, code)
        try:
            return fn()
        finally:
            _lib.set_config(_lib.NPBGB_CFG_BATCH_MODE, old)


class Batch:
    def __init__(self, grids, band_rows=0, band_rows_of=None, mode=None, guard=False):
        """grids: iterable of (A, B, TSTEPS); band_rows_of(A) may pick rows per band;
        mode: None (by size), "persistent", "stepped" or "queue".

        guard=True applies the float64 guard (``npbench_gb300.precision``): a
        float32 grid whose float32 error is predicted above NPBench's bound runs
        in float64 (widened exactly, rounded back once at the end), which the
        stepped and queue forms do (by default such a batch is stepped)."""
        self._h = None
        self.guard = bool(guard)
        self.promoted = 0
        if self.guard:
            mode = self._guard_mode(grids, mode)
        arr = self._structs(grids, band_rows_of)
        h = ctypes.c_void_p()
        _planned(mode, lambda: _lib.check(
            _lib.load().npbgb_batch_create(arr, len(grids), int(band_rows), ctypes.byref(h)),
            "npbgb_batch_create"))
        self._h = h

    def replan(self, grids, band_rows=0, band_rows_of=None, mode=None):
        """Re-plan this batch for a new grid list, reusing its device buffers."""
        if self._h is None:
            raise RuntimeError("batch destroyed")
        if self.guard:
            mode = self._guard_mode(grids, mode)
        arr = self._structs(grids, band_rows_of)
        _planned(mode, lambda: _lib.check(
            _lib.load().npbgb_batch_replan(self._h, arr, len(grids), int(band_rows)),
            "npbgb_batch_replan"))

    def _promote(self, A, entry):
        import torch
        from . import precision
        if not self.guard or A.dtype != torch.float32:
            return False
        return precision.needs_fp64("jacobi2d" if A.dim() == 2 else "heat3d", int(entry[2]))

    def _guard_mode(self, grids, mode):
        if mode == "persistent" and any(self._promote(e[0], e) for e in grids):
            raise ValueError("float32 grids promoted to float64 need the stepped or queue form")
        return mode

    def _structs(self, grids, band_rows_of):
        import torch
        self._keep = []
        self.promoted = 0
        arr = (_lib.Grid * max(1, len(grids)))()
        for n, entry in enumerate(grids):
            A, B, T = entry[:3]
            step0, nsteps = (entry[3], entry[4]) if len(entry) > 3 else (0, 0)
            if not (isinstance(A, torch.Tensor) and isinstance(B, torch.Tensor)):
                raise TypeError("batch grids must be CUDA tensors")
            if A.device.type != "cuda" or B.device != A.device:
                raise ValueError("batch grids must be on one CUDA device")
            if A.dim() not in (2, 3) or A.shape != B.shape or A.dtype != B.dtype:
                raise ValueError(f"grid {n}: A and B must be 2D or 3D with equal shape and dtype")
            if not (A.is_contiguous() and B.is_contiguous()):
                raise ValueError(f"grid {n}: tensors must be contiguous")
            if A.dtype == torch.float64:
                code = _lib.NPBGB_F64
            elif A.dtype == torch.float32:
                code = _lib.NPBGB_F32
            else:
                raise TypeError(f"grid {n}: unsupported dtype {A.dtype}")
            g = arr[n]
            g.a, g.b = A.data_ptr(), B.data_ptr()
            if A.dim() == 2:
                g.n0, g.n1, g.n2 = A.shape[0], A.shape[1], 1
                g.kind = _lib.NPBGB_KIND_JACOBI2D
            else:
                g.n0, g.n1, g.n2 = A.shape
                g.kind = _lib.NPBGB_KIND_HEAT3D
            g.step0, g.nsteps = int(step0), int(nsteps)
            g.dtype = code
            g.tsteps = int(T)
            g.band_rows = int(band_rows_of(A)) if band_rows_of else 0
            self._keep.append((A, B))
            if self._promote(A, entry):
                # run in float64: the queue widens A/B into this pair and rounds back
                A64 = torch.empty(A.shape, dtype=torch.float64, device=A.device)
                B64 = torch.empty_like(A64)
                g.a, g.b = A64.data_ptr(), B64.data_ptr()
                g.a32, g.b32 = A.data_ptr(), B.data_ptr()
                g.dtype = _lib.NPBGB_F64
                self._keep.append((A64, B64))
                self.promoted += 1
        self.device = self._keep[0][0].device if self._keep else None
        return arr

    def launch(self, graph=False, stream=None):
        import torch
        if self._h is None:
            raise RuntimeError("batch destroyed")
        if stream is None and self.device is not None:
            stream = torch.cuda.current_stream(self.device).cuda_stream
        _lib.check(_lib.load().npbgb_batch_launch(self._h, 1 if graph else 0, stream),
                   "npbgb_batch_launch")

    def info(self):
        """{"mode": "persistent" | "stepped", "bands", "ctas", "updates"}; in the
        stepped form "bands" counts tiles and "ctas" launches."""
        nb, nc, up = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        lib = _lib.load()
        _lib.check(lib.npbgb_batch_info(self._h, ctypes.byref(nb), ctypes.byref(nc),
                                        ctypes.byref(up)), "npbgb_batch_info")
        mode = ctypes.c_int32()
        _lib.check(lib.npbgb_batch_mode(self._h, ctypes.byref(mode)), "npbgb_batch_mode")
        name = {_lib.NPBGB_BATCH_STEPPED: "stepped",
                _lib.NPBGB_BATCH_QUEUE: "queue"}.get(mode.value, "persistent")
        return {"mode": name, "bands": nb.value, "ctas": nc.value, "updates": up.value}

    def close(self):
        if self._h is not None:
            _lib.load().npbgb_batch_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
