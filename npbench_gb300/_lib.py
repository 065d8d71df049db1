"""ctypes binding of libnpbgb.so (the C ABI declared in include/npbgb.h).

The library is loaded from this package directory.  There is no fallback: if
it is missing or fails to load, every entry point raises ``RuntimeError``
telling how to build it (``python -m npbench_gb300.build``).
"""
import ctypes
import os
import threading

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libnpbgb.so")

NPBGB_OK = 0
NPBGB_ERR_ARG = 1
NPBGB_ERR_DTYPE = 2
NPBGB_ERR_CUDA = 3
NPBGB_ERR_TIMEOUT = 4
NPBGB_ERR_NOMEM = 5
NPBGB_ERR_STATE = 6
NPBGB_F64 = 0
NPBGB_F32 = 1
NPBGB_CFG_F64_EMULATION = 1
NPBGB_CFG_HEAT_CHUNK = 2
NPBGB_CFG_HEAT_TMA = 3
NPBGB_CFG_JACOBI_CHUNK = 4
NPBGB_CFG_HEAT_ROWS = 5
NPBGB_CFG_HEAT_HW_ROWS = 6
NPBGB_CFG_F64_CVT = 7
NPBGB_CFG_JACOBI_HW_WARPS = 8
NPBGB_CFG_BATCH_CTAS_PER_SM = 9
NPBGB_CFG_PDL = 10
NPBGB_CFG_BATCH_MODE = 11
NPBGB_CFG_HDIFF_EMU = 12
NPBGB_CFG_JACOBI1D_CTAS = 14
NPBGB_CFG_JACOBI1D_DEPTH = 15
NPBGB_CFG_HEAT_TB = 16
NPBGB_CFG_HEAT_TB_CHUNK = 17
NPBGB_CFG_JACOBI_BANDS = 18
NPBGB_CFG_JACOBI_BANDS_WARPS = 19
NPBGB_CFG_HEAT_STAGES = 20
NPBGB_CFG_LAUNCHES = 21
NPBGB_CFG_HEAT_MAD_ROWS = 22
NPBGB_CFG_QUEUE_WHOLE_CELLS = 23
NPBGB_CFG_JACOBI_FX_MUL = 24
NPBGB_CFG_JACOBI_FX_ADDS = 25
NPBGB_CFG_JACOBI_TMA = 26
NPBGB_CFG_BATCH_TMA = 27
NPBGB_BATCH_PERSISTENT = 1
NPBGB_BATCH_STEPPED = 2
NPBGB_BATCH_QUEUE = 3

NPBGB_KIND_JACOBI2D = 0
NPBGB_KIND_HEAT3D = 1


class Grid(ctypes.Structure):
    """npbgb_grid of include/npbgb.h."""
    _fields_ = [("a", ctypes.c_void_p), ("b", ctypes.c_void_p), ("n0", ctypes.c_int64),
                ("n1", ctypes.c_int64), ("n2", ctypes.c_int64), ("kind", ctypes.c_int32),
                ("dtype", ctypes.c_int32), ("tsteps", ctypes.c_int32),
                ("band_rows", ctypes.c_int32), ("step0", ctypes.c_int32),
                ("nsteps", ctypes.c_int32), ("a32", ctypes.c_void_p), ("b32", ctypes.c_void_p)]


# Every symbol include/npbgb.h declares, with its ctypes signature.
_i32, _i64, _vp, _cp = ctypes.c_int32, ctypes.c_int64, ctypes.c_void_p, ctypes.c_char_p
SIGNATURES = {
    "npbgb_version": (_cp, []),
    "npbgb_last_error": (_cp, []),
    "npbgb_status_string": (_cp, [_i32]),
    "npbgb_set_config": (_i32, [_i32, _i64]),
    "npbgb_get_config": (_i32, [_i32, ctypes.POINTER(_i64)]),
    "npbgb_device_status": (_i32, [_vp]),
    "npbgb_selftest_wait_timeout": (_i32, [_i64, _vp]),
    "npbgb_batch_create": (_i32, [ctypes.POINTER(Grid), _i64, _i32, ctypes.POINTER(_vp)]),
    "npbgb_batch_launch": (_i32, [_vp, _i32, _vp]),
    "npbgb_batch_replan": (_i32, [_vp, ctypes.POINTER(Grid), _i64, _i32]),
    "npbgb_batch_mode": (_i32, [_vp, ctypes.POINTER(_i32)]),
    "npbgb_batch_info": (_i32, [_vp, ctypes.POINTER(_i64), ctypes.POINTER(_i64),
                                 ctypes.POINTER(_i64)]),
    "npbgb_batch_destroy": (_i32, [_vp]),
    "npbgb_batch_run_noalloc": (_i32, [ctypes.POINTER(Grid), _i64, _i32, _vp]),
    "npbgb_queue_create": (_i32, [_i32, _i32, _i32, _i32, _i64, ctypes.POINTER(_vp)]),
    "npbgb_queue_submit": (_i32, [_vp, ctypes.POINTER(Grid), ctypes.POINTER(_i32)]),
    "npbgb_queue_kick": (_i32, [_vp, _vp]),
    "npbgb_queue_poll": (_i32, [_vp, ctypes.POINTER(_i32), _i32, ctypes.POINTER(_i32)]),
    "npbgb_queue_state": (_i32, [_vp, ctypes.POINTER(_i32), ctypes.POINTER(_i32),
                                 ctypes.POINTER(_i64)]),
    "npbgb_queue_close": (_i32, [_vp]),
    "npbgb_queue_destroy": (_i32, [_vp]),
    "npbgb_probe_pipe": (_i32, [_i32, _i64, _i32, _vp, _vp]),
    "npbgb_convert": (_i32, [_vp, _i32, _vp, _i32, _i64, _vp]),
    "npbgb_jacobi2d": (_i32, [_vp, _vp, _i64, _i64, _i32, _i32, _vp]),
    "npbgb_heat3d": (_i32, [_vp, _vp, _i64, _i64, _i64, _i32, _i32, _vp]),
    "npbgb_hdiff": (_i32, [_vp, _vp, _vp, _i64, _i64, _i64, _i32, _vp]),
    "npbgb_jacobi1d": (_i32, [_vp, _vp, _i64, _i32, _i32, _vp]),
    "npbgb_fdtd2d": (_i32, [_vp, _vp, _vp, _vp, _i64, _i64, _i64, _i32, _i32, _vp]),
    "npbgb_vadv_workspace_bytes": (_i64, [_i64, _i64, _i64]),
    "npbgb_cavity_flow_workspace_bytes": (_i64, [_i64, _i64]),
    "npbgb_channel_flow_workspace_bytes": (_i64, [_i64, _i64]),
    "npbgb_channel_flow": (_i32, [_vp, _vp, _vp, _i64, _i64, _i32] + [ctypes.c_double] * 6 +
                           [_i64, _i32, _vp, _i64, ctypes.POINTER(ctypes.c_int64), _vp]),
    "npbgb_cavity_flow": (_i32, [_vp, _vp, _vp, _i64, _i64, _i32, _i32, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                 ctypes.c_double, _i32, _vp, _i64, _vp]),
    "npbgb_vadv": (_i32, [_vp, _vp, _vp, _vp, _vp, ctypes.c_double, _i64, _i64, _i64, _i32, _vp,
                          _i64, _vp]),
}

_lock = threading.Lock()
_lib = None


class NpbgbError(RuntimeError):
    """A libnpbgb entry point returned a non-OK status."""

    def __init__(self, status, where, message):
        super().__init__(f"{where}: {message} (status {status})")
        self.status = status


def load():
    """Load and bind libnpbgb.so (once per process)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(
                    f"{LIB_PATH} is not built; run `python -m npbench_gb300.build` "
                    "(or __graft_entry__.build()) -- there is no CPU fallback")
            lib = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


def check(status, where):
    """Raise NpbgbError for a non-OK status, with the library's message."""
    if status != NPBGB_OK:
        lib = load()
        msg = lib.npbgb_last_error().decode(errors="replace")
        if not msg:
            msg = lib.npbgb_status_string(status).decode()
        raise NpbgbError(status, where, msg)


def set_config(key, value):
    """Set a library knob (NPBGB_CFG_*); returns the previous value."""
    old = get_config(key)
    check(load().npbgb_set_config(key, int(value)), "npbgb_set_config")
    return old


def get_config(key):
    v = _i64(0)
    check(load().npbgb_get_config(key, ctypes.byref(v)), "npbgb_get_config")
    return v.value


def launches():
    """Kernels the library has put on a stream so far (NPBGB_CFG_LAUNCHES)."""
    return get_config(NPBGB_CFG_LAUNCHES)


def device_status(stream=None):
    """Synchronise and raise NpbgbError if a kernel gave up a bounded device wait."""
    check(load().npbgb_device_status(stream), "device_status")


def version():
    return load().npbgb_version().decode()


def convert(dst, src, stream=None):
    """dst <- src between float32 and float64 CUDA tensors of one size (libnpbgb kernel)."""
    import torch
    codes = {torch.float64: NPBGB_F64, torch.float32: NPBGB_F32}
    if dst.numel() != src.numel() or not (dst.is_contiguous() and src.is_contiguous()):
        raise ValueError("convert: contiguous tensors of one size")
    if stream is None:
        stream = torch.cuda.current_stream(dst.device)
    check(load().npbgb_convert(dst.data_ptr(), codes[dst.dtype], src.data_ptr(), codes[src.dtype],
                               dst.numel(), stream.cuda_stream), "npbgb_convert")
