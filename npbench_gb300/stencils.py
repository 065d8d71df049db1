"""NPBench-signature stencil kernels running on libnpbgb's sm_103a CUDA code.

These are drop-ins for the reference NumPy kernels:

* ``jacobi_2d_kernel(TSTEPS, A, B)``   -- polybench/jacobi_2d/jacobi_2d_numpy.py:4
* ``heat_3d_kernel(TSTEPS, A, B)``     -- polybench/heat_3d/heat_3d_numpy.py:4
* ``hdiff(in_field, out_field, coeff)`` -- weather_stencils/hdiff/hdiff_numpy.py:5
* ``jacobi_1d_kernel(TSTEPS, A, B)``   -- polybench/jacobi_1d/jacobi_1d_numpy.py:4
* ``fdtd_2d_kernel(TMAX, ex, ey, hz, _fict_)`` -- polybench/fdtd_2d/fdtd_2d_numpy.py:4
* ``vadv(utens_stage, u_stage, wcon, u_pos, utens, dtr_stage)`` --
  weather_stencils/vadv/vadv_numpy.py:9
* ``cavity_flow(nx, ny, nt, nit, u, v, dt, dx, dy, p, rho, nu)`` --
  cavity_flow/cavity_flow_numpy.py:41
* ``channel_flow(nit, u, v, dt, dx, dy, p, rho, nu, F)`` --
  channel_flow/channel_flow_numpy.py:69 (returns the step count)

Arguments are updated in place and nothing is returned, as in the reference.
They may be

* ``torch.Tensor`` on a CUDA device (the framework plugin's path): the kernels
  run on the tensors' current stream and return without synchronising;
* ``numpy.ndarray`` (host): the arrays are copied to the current CUDA device,
  updated there and copied back into the same NumPy arrays before returning.

With ``npbench_gb300.autotune`` enabled, Jacobi-2D and Heat-3D calls run with
the launch settings cached for their shape (settings change speed, not bits).

Results are bit-identical to the reference NumPy kernels for float64 and
float32 (hdiff, vadv, cavity_flow and channel_flow: float64 only).  Errors raise ``TypeError`` (dtype),
``ValueError`` (shape, device, aliasing) or ``npbench_gb300.NpbgbError``
(a status from the library).  There is no CPU fallback: without a CUDA device
or without libnpbgb.so these functions raise.
"""
import numpy as np

from . import _lib

__all__ = ["jacobi_2d_kernel", "heat_3d_kernel", "hdiff", "jacobi_1d_kernel", "fdtd_2d_kernel",
           "vadv", "cavity_flow", "channel_flow"]


def _torch():
    import torch
    return torch


def _dtype_code(dtype, allowed=(np.float64, np.float32)):
    torch = _torch()
    table = {torch.float64: _lib.NPBGB_F64, torch.float32: _lib.NPBGB_F32,
             np.dtype(np.float64): _lib.NPBGB_F64, np.dtype(np.float32): _lib.NPBGB_F32}
    allowed_codes = {_lib.NPBGB_F64 if a == np.float64 else _lib.NPBGB_F32 for a in allowed}
    code = table.get(dtype)
    if code is None or code not in allowed_codes:
        raise TypeError(f"unsupported dtype {dtype}; expected one of "
                        f"{[np.dtype(a).name for a in allowed]}")
    return code


class _DeviceView:
    """Contiguous CUDA tensors standing for the caller's arrays during one call.

    For CUDA tensors that are already contiguous the tensors themselves are
    used (no copy).  Otherwise a contiguous device copy is made and written
    back on ``finish()`` into the caller's object, which keeps its identity.
    """

    def __init__(self, arrays, writable):
        torch = _torch()
        self.orig = arrays
        self.writable = writable
        self.dev = []
        first = arrays[0]
        if isinstance(first, torch.Tensor):
            if not all(isinstance(a, torch.Tensor) for a in arrays):
                raise TypeError("mix of torch tensors and other arrays")
            device = first.device
            if device.type != "cuda":
                raise ValueError(f"tensors must be on a CUDA device, got {device}")
            for a in arrays:
                if a.device != device:
                    raise ValueError("all tensors must be on the same device")
                self.dev.append(a if a.is_contiguous() else a.contiguous())
            self.device = device
            self.host = False
        else:
            if not torch.cuda.is_available():
                raise RuntimeError("no CUDA device available (no CPU fallback)")
            self.device = torch.device("cuda", torch.cuda.current_device())
            for o, w in zip(arrays, writable):
                if w and not isinstance(o, np.ndarray):
                    raise TypeError("output arguments must be numpy arrays or CUDA tensors")
            arrs = [np.asarray(a) for a in arrays]
            self.dev = [torch.from_numpy(np.ascontiguousarray(a)).to(self.device) for a in arrs]
            self.host = True

    @property
    def stream(self):
        return _torch().cuda.current_stream(self.device).cuda_stream

    def ptr(self, i):
        return self.dev[i].data_ptr()

    def finish(self):
        for i, (o, d) in enumerate(zip(self.orig, self.dev)):
            if not self.writable[i]:
                continue
            if self.host:
                np.copyto(o, d.cpu().numpy())
            elif d is not o:
                o.copy_(d)


def _check_same(arrays, names):
    a0 = arrays[0]
    for a, n in zip(arrays[1:], names[1:]):
        if tuple(a.shape) != tuple(a0.shape):
            raise ValueError(f"{n} has shape {tuple(a.shape)}, {names[0]} has {tuple(a0.shape)}")
        if a.dtype != a0.dtype:
            raise TypeError(f"{n} has dtype {a.dtype}, {names[0]} has {a0.dtype}")


def _shares_memory(x, y):
    torch = _torch()
    if isinstance(x, torch.Tensor):
        if x.numel() == 0 or y.numel() == 0:
            return False
        xs, xe = x.data_ptr(), x.data_ptr() + x.numel() * x.element_size()
        ys, ye = y.data_ptr(), y.data_ptr() + y.numel() * y.element_size()
        return xs < ye and ys < xe
    return np.shares_memory(x, y)


def _pingpong(name, entry, ndim, TSTEPS, A, B, tuned=None):
    _check_same((A, B), ("A", "B"))
    if len(A.shape) != ndim:
        raise ValueError(f"{name}: expected {ndim}-D arrays, got shape {tuple(A.shape)}")
    code = _dtype_code(A.dtype)
    T = int(TSTEPS)
    if not (-2**31 <= T < 2**31):
        raise ValueError(f"{name}: TSTEPS out of int32 range")
    if _shares_memory(A, B):
        raise ValueError(f"{name}: A and B share memory")
    lib = _lib.load()
    torch = _torch()
    view = _DeviceView((A, B), (True, True))
    from . import autotune
    with torch.cuda.device(view.device), autotune.applied(tuned or name, A.shape, A.dtype):
        st = entry(lib)(view.ptr(0), view.ptr(1), *[int(s) for s in A.shape], T, code, view.stream)
        _lib.check(st, name)
        view.finish()


def jacobi_2d_kernel(TSTEPS, A, B):
    """``kernel(TSTEPS, A, B)`` of polybench/jacobi_2d/jacobi_2d_numpy.py:4-10, on the GPU."""
    _pingpong("jacobi_2d", lambda lib: lib.npbgb_jacobi2d, 2, TSTEPS, A, B)


def heat_3d_kernel(TSTEPS, A, B):
    """``kernel(TSTEPS, A, B)`` of polybench/heat_3d/heat_3d_numpy.py:4-20, on the GPU."""
    _pingpong("heat_3d", lambda lib: lib.npbgb_heat3d, 3, TSTEPS, A, B)


def hdiff(in_field, out_field, coeff):
    """``hdiff(in_field, out_field, coeff)`` of weather_stencils/hdiff/hdiff_numpy.py:5-29."""
    I, J, K = (int(s) for s in out_field.shape)
    if tuple(in_field.shape) != (I + 4, J + 4, K):
        raise ValueError(f"hdiff: in_field shape {tuple(in_field.shape)}, expected "
                         f"{(I + 4, J + 4, K)}")
    if tuple(coeff.shape) != (I, J, K):
        raise ValueError(f"hdiff: coeff shape {tuple(coeff.shape)}, expected {(I, J, K)}")
    for n, a in (("in_field", in_field), ("coeff", coeff)):
        if a.dtype != out_field.dtype:
            raise TypeError(f"hdiff: {n} dtype {a.dtype} differs from out_field {out_field.dtype}")
        if _shares_memory(a, out_field):
            raise ValueError(f"hdiff: {n} shares memory with out_field")
    code = _dtype_code(out_field.dtype, allowed=(np.float64,))
    lib = _lib.load()
    torch = _torch()
    view = _DeviceView((in_field, out_field, coeff), (False, True, False))
    with torch.cuda.device(view.device):
        st = lib.npbgb_hdiff(view.ptr(0), view.ptr(1), view.ptr(2), I, J, K, code, view.stream)
        _lib.check(st, "hdiff")
        view.finish()


def jacobi_1d_kernel(TSTEPS, A, B):
    """``kernel(TSTEPS, A, B)`` of polybench/jacobi_1d/jacobi_1d_numpy.py:4-8, on the GPU."""
    _pingpong("jacobi_1d", lambda lib: lib.npbgb_jacobi1d, 1, TSTEPS, A, B)


def fdtd_2d_kernel(TMAX, ex, ey, hz, _fict_):
    """``kernel(TMAX, ex, ey, hz, _fict_)`` of polybench/fdtd_2d/fdtd_2d_numpy.py:4-11."""
    _check_same((ex, ey, hz), ("ex", "ey", "hz"))
    if len(ex.shape) != 2:
        raise ValueError(f"fdtd_2d: expected 2-D fields, got shape {tuple(ex.shape)}")
    if len(_fict_.shape) != 1 or _fict_.dtype != ex.dtype:
        raise TypeError("fdtd_2d: _fict_ must be 1-D with the fields' dtype")
    T = int(TMAX)
    if T > _fict_.shape[0]:
        raise IndexError(f"fdtd_2d: _fict_ has {_fict_.shape[0]} entries, TMAX is {T}")
    for x, y, nx, ny in (("ex", "ey", ex, ey), ("ex", "hz", ex, hz), ("ey", "hz", ey, hz)):
        if _shares_memory(nx, ny):
            raise ValueError(f"fdtd_2d: {x} and {y} share memory")
    code = _dtype_code(ex.dtype)
    lib = _lib.load()
    torch = _torch()
    view = _DeviceView((ex, ey, hz, _fict_), (True, True, True, False))
    with torch.cuda.device(view.device):
        st = lib.npbgb_fdtd2d(view.ptr(0), view.ptr(1), view.ptr(2), view.ptr(3),
                              int(_fict_.shape[0]), int(ex.shape[0]), int(ex.shape[1]), T, code,
                              view.stream)
        _lib.check(st, "fdtd_2d")
        view.finish()


def vadv(utens_stage, u_stage, wcon, u_pos, utens, dtr_stage):
    """``vadv(utens_stage, u_stage, wcon, u_pos, utens, dtr_stage)`` of
    weather_stencils/vadv/vadv_numpy.py:9-78; writes ``utens_stage``.

    The solve's coefficient workspace (8*(K-1)*I*J bytes) is taken from
    PyTorch's caching allocator on the call's stream.  K < 2 raises
    IndexError, as the reference does.
    """
    I, J, K = (int(s) for s in utens_stage.shape)
    for n, a in (("u_stage", u_stage), ("u_pos", u_pos), ("utens", utens)):
        if tuple(a.shape) != (I, J, K):
            raise ValueError(f"vadv: {n} shape {tuple(a.shape)}, expected {(I, J, K)}")
    if tuple(wcon.shape) != (I + 1, J, K):
        raise ValueError(f"vadv: wcon shape {tuple(wcon.shape)}, expected {(I + 1, J, K)}")
    for n, a in (("u_stage", u_stage), ("wcon", wcon), ("u_pos", u_pos), ("utens", utens)):
        if a.dtype != utens_stage.dtype:
            raise TypeError(f"vadv: {n} dtype {a.dtype} differs from utens_stage "
                            f"{utens_stage.dtype}")
        if _shares_memory(a, utens_stage):
            raise ValueError(f"vadv: {n} shares memory with utens_stage")
    code = _dtype_code(utens_stage.dtype, allowed=(np.float64,))
    if K < 2:
        raise IndexError(f"vadv: K = {K}; the solve reads level 1")
    lib = _lib.load()
    torch = _torch()
    view = _DeviceView((utens_stage, u_stage, wcon, u_pos, utens),
                       (True, False, False, False, False))
    with torch.cuda.device(view.device):
        nbytes = int(lib.npbgb_vadv_workspace_bytes(I, J, K))
        ws = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=view.device)
        st = lib.npbgb_vadv(view.ptr(0), view.ptr(1), view.ptr(2), view.ptr(3), view.ptr(4),
                            float(dtr_stage), I, J, K, code, ws.data_ptr(), nbytes, view.stream)
        _lib.check(st, "vadv")
        view.finish()


def cavity_flow(nx, ny, nt, nit, u, v, dt, dx, dy, p, rho, nu):
    """``cavity_flow(nx, ny, nt, nit, u, v, dt, dx, dy, p, rho, nu)`` of
    cavity_flow/cavity_flow_numpy.py:41-82; updates u, v and p in place.

    The whole time loop is one persistent launch; its workspace (four fields
    and the band counters) comes from PyTorch's caching allocator.  Sizes the
    reference's boundary statements cannot index raise IndexError, as there.
    """
    ny, nx, nt, nit = int(ny), int(nx), int(nt), int(nit)
    _check_same((u, v, p), ("u", "v", "p"))
    if tuple(u.shape) != (ny, nx):
        raise ValueError(f"cavity_flow: arrays are {tuple(u.shape)}, expected (ny, nx) = "
                         f"{(ny, nx)}")
    code = _dtype_code(u.dtype, allowed=(np.float64,))
    for x, y, a, b in (("u", "v", u, v), ("u", "p", u, p), ("v", "p", v, p)):
        if _shares_memory(a, b):
            raise ValueError(f"cavity_flow: {x} and {y} share memory")
    if nt > 0 and (ny < 1 or nx < 1 or (nit > 0 and (ny < 2 or nx < 2))):
        raise IndexError(f"cavity_flow: a ({ny}, {nx}) grid is too small for the boundary "
                         "statements")
    if nt < 0 or nit < 0:
        raise ValueError("cavity_flow: negative nt or nit")
    lib = _lib.load()
    torch = _torch()
    view = _DeviceView((u, v, p), (True, True, True))
    with torch.cuda.device(view.device):
        nbytes = int(lib.npbgb_cavity_flow_workspace_bytes(ny, nx))
        ws = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=view.device)
        st = lib.npbgb_cavity_flow(view.ptr(0), view.ptr(1), view.ptr(2), ny, nx, nt, nit,
                                   float(dt), float(dx), float(dy), float(rho), float(nu), code,
                                   ws.data_ptr(), nbytes, view.stream)
        _lib.check(st, "cavity_flow")
        view.finish()


def channel_flow(nit, u, v, dt, dx, dy, p, rho, nu, F, max_steps=1_000_000):
    """``channel_flow(nit, u, v, dt, dx, dy, p, rho, nu, F)`` of
    channel_flow/channel_flow_numpy.py:69-152; updates u, v, p in place and
    returns the step count, which matches the reference's because its
    convergence sums are np.sum's bit for bit.

    ``max_steps`` bounds the loop (the reference's has no bound); reaching it
    without convergence raises RuntimeError, with u, v, p left at that step.
    """
    import ctypes
    nit = int(nit)
    _check_same((u, v, p), ("u", "v", "p"))
    if len(u.shape) != 2:
        raise ValueError(f"channel_flow: expected 2-D arrays, got shape {tuple(u.shape)}")
    ny, nx = (int(x) for x in u.shape)
    code = _dtype_code(u.dtype, allowed=(np.float64,))
    for x, y, a, b in (("u", "v", u, v), ("u", "p", u, p), ("v", "p", v, p)):
        if _shares_memory(a, b):
            raise ValueError(f"channel_flow: {x} and {y} share memory")
    if nx < 2 or ny < 1 or (nit > 0 and ny < 2):
        raise IndexError(f"channel_flow: a ({ny}, {nx}) grid is too small for the boundary "
                         "statements")
    if nit < 0 or int(max_steps) < 1:
        raise ValueError("channel_flow: negative nit or max_steps < 1")
    lib = _lib.load()
    torch = _torch()
    view = _DeviceView((u, v, p), (True, True, True))
    steps = ctypes.c_int64(0)
    with torch.cuda.device(view.device):
        nbytes = int(lib.npbgb_channel_flow_workspace_bytes(ny, nx))
        ws = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=view.device)
        st = lib.npbgb_channel_flow(view.ptr(0), view.ptr(1), view.ptr(2), ny, nx, nit,
                                    float(dt), float(dx), float(dy), float(rho), float(nu),
                                    float(F), int(max_steps), code, ws.data_ptr(), nbytes,
                                    ctypes.byref(steps), view.stream)
        _lib.check(st, "channel_flow")
        view.finish()
    if steps.value < 0:
        raise RuntimeError(f"channel_flow: no convergence within {max_steps} steps")
    return int(steps.value)
