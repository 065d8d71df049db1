"""ctypes binding of the C oracle (oracle/stencils.c) -- TEST INFRASTRUCTURE ONLY.

``load()`` builds ``oracle/_build/liboracle.so`` with ``make`` when it is
missing and returns wrappers that take NumPy arrays and mutate them in place,
with the same call shapes as the reference kernels:

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
* ``numpy_sum(a)`` -- ``np.sum`` of a contiguous float64 array
"""
import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lock = threading.Lock()
_lib = None


def build(force=False):
    """Compile the C oracle with its Makefile; returns the .so path."""
    if force or not os.path.exists(_LIB_PATH):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def _bind(lib):
    i64, i32, vp = ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p
    for sfx in ("f64", "f32"):
        getattr(lib, "oracle_jacobi2d_" + sfx).argtypes = [vp, vp, i64, i64, i32]
        getattr(lib, "oracle_jacobi2d_half_" + sfx).argtypes = [vp, vp, i64, i64]
        getattr(lib, "oracle_heat3d_" + sfx).argtypes = [vp, vp, i64, i64, i64, i32]
        getattr(lib, "oracle_heat3d_half_" + sfx).argtypes = [vp, vp, i64, i64, i64]
    lib.oracle_hdiff_f64.argtypes = [vp, vp, vp, i64, i64, i64]
    for sfx in ("f64", "f32"):
        getattr(lib, "oracle_jacobi1d_" + sfx).argtypes = [vp, vp, i64, i32]
        getattr(lib, "oracle_fdtd2d_" + sfx).argtypes = [vp, vp, vp, vp, i64, i64, i32]
    lib.oracle_vadv_f64.argtypes = [vp, vp, vp, vp, vp, ctypes.c_double, i64, i64, i64]
    d = ctypes.c_double
    lib.oracle_cavity_flow_f64.argtypes = [vp, vp, vp, i64, i64, i32, i32, d, d, d, d, d, vp]
    lib.oracle_channel_flow_f64.argtypes = [vp, vp, vp, i64, i64, i32, d, d, d, d, d, d, vp, i64]
    lib.oracle_channel_flow_f64.restype = i64
    lib.oracle_numpy_sum_f64.argtypes = [vp, i64]
    lib.oracle_numpy_sum_f64.restype = d
    return lib


def lib():
    global _lib
    with _lock:
        if _lib is None:
            _lib = _bind(ctypes.CDLL(build()))
    return _lib


def _sfx(*arrays):
    dt = arrays[0].dtype
    for a in arrays:
        if a.dtype != dt or not a.flags.c_contiguous:
            raise ValueError("oracle wants C-contiguous arrays of one dtype")
    if dt == np.float64:
        return "f64"
    if dt == np.float32:
        return "f32"
    raise TypeError(f"unsupported dtype {dt}")


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def jacobi_2d_kernel(TSTEPS, A, B):
    sfx = _sfx(A, B)
    getattr(lib(), "oracle_jacobi2d_" + sfx)(_p(A), _p(B), A.shape[0], A.shape[1], int(TSTEPS))


def heat_3d_kernel(TSTEPS, A, B):
    sfx = _sfx(A, B)
    getattr(lib(), "oracle_heat3d_" + sfx)(_p(A), _p(B), *A.shape, int(TSTEPS))


def jacobi_2d_half_sweep(src, dst):
    sfx = _sfx(src, dst)
    getattr(lib(), "oracle_jacobi2d_half_" + sfx)(_p(src), _p(dst), *src.shape)


def heat_3d_half_sweep(src, dst):
    sfx = _sfx(src, dst)
    getattr(lib(), "oracle_heat3d_half_" + sfx)(_p(src), _p(dst), *src.shape)


def hdiff(in_field, out_field, coeff):
    if _sfx(in_field, out_field, coeff) != "f64":
        raise TypeError("hdiff oracle is float64 only")
    I, J, K = out_field.shape
    if in_field.shape != (I + 4, J + 4, K) or coeff.shape != (I, J, K):
        raise ValueError("hdiff shapes: in (I+4, J+4, K), out/coeff (I, J, K)")
    lib().oracle_hdiff_f64(_p(in_field), _p(out_field), _p(coeff), I, J, K)


def jacobi_1d_kernel(TSTEPS, A, B):
    sfx = _sfx(A, B)
    getattr(lib(), "oracle_jacobi1d_" + sfx)(_p(A), _p(B), A.shape[0], int(TSTEPS))


def fdtd_2d_kernel(TMAX, ex, ey, hz, _fict_):
    sfx = _sfx(ex, ey, hz, _fict_)
    if int(TMAX) > _fict_.shape[0]:
        raise ValueError("_fict_ shorter than TMAX")
    getattr(lib(), "oracle_fdtd2d_" + sfx)(_p(ex), _p(ey), _p(hz), _p(_fict_), ex.shape[0],
                                          ex.shape[1], int(TMAX))


def vadv(utens_stage, u_stage, wcon, u_pos, utens, dtr_stage):
    if _sfx(utens_stage, u_stage, wcon, u_pos, utens) != "f64":
        raise TypeError("vadv oracle is float64 only")
    I, J, K = utens_stage.shape
    if wcon.shape != (I + 1, J, K) or any(a.shape != (I, J, K) for a in (u_stage, u_pos, utens)):
        raise ValueError("vadv shapes: wcon (I+1, J, K), the others (I, J, K)")
    if K < 2:
        raise IndexError(f"vadv needs K >= 2 (reads level 1), got K={K}")
    lib().oracle_vadv_f64(_p(utens_stage), _p(u_stage), _p(wcon), _p(u_pos), _p(utens),
                          float(dtr_stage), I, J, K)


_CFD_KEYS = ("two_dx", "two_dy", "inv_dt", "dx2", "dy2", "pD", "pC", "k1u", "k1v", "k2", "k3")


def cavity_flow(nx, ny, nt, nit, u, v, dt, dx, dy, p, rho, nu):
    from .stencils_np import cfd_constants
    if _sfx(u, v, p) != "f64":
        raise TypeError("cavity_flow oracle is float64 only")
    if u.shape != (ny, nx) or v.shape != (ny, nx) or p.shape != (ny, nx):
        raise ValueError("cavity_flow arrays must be (ny, nx)")
    if int(nt) > 0 and int(nit) > 0 and (ny < 2 or nx < 2):
        raise IndexError("cavity_flow: the pressure boundaries need ny >= 2 and nx >= 2")
    k = cfd_constants(dt, dx, dy, rho)
    kc = np.array([k[n] for n in _CFD_KEYS], dtype=np.float64)
    lib().oracle_cavity_flow_f64(_p(u), _p(v), _p(p), ny, nx, int(nt), int(nit), float(dt),
                                 float(dx), float(dy), float(rho), float(nu), _p(kc))


def numpy_sum(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return lib().oracle_numpy_sum_f64(_p(a), a.size)


def channel_flow(nit, u, v, dt, dx, dy, p, rho, nu, F, max_steps=10**7):
    from .stencils_np import cfd_constants
    if _sfx(u, v, p) != "f64":
        raise TypeError("channel_flow oracle is float64 only")
    ny, nx = u.shape
    if v.shape != (ny, nx) or p.shape != (ny, nx):
        raise ValueError("channel_flow arrays must share one (ny, nx) shape")
    if ny < 1 or (int(nit) > 0 and ny < 2) or nx < 2:
        raise IndexError("channel_flow: the boundary statements need ny >= 2 and nx >= 2")
    k = cfd_constants(dt, dx, dy, rho)
    kc = np.array([k[n] for n in _CFD_KEYS], dtype=np.float64)
    steps = lib().oracle_channel_flow_f64(_p(u), _p(v), _p(p), ny, nx, int(nit), float(dt),
                                          float(dx), float(dy), float(rho), float(nu),
                                          float(F * dt), _p(kc), int(max_steps))
    if steps < 0:
        raise RuntimeError(f"channel_flow did not converge in {max_steps} steps")
    return int(steps)
