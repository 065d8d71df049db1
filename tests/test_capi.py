"""The C-ABI library loads, exports every declared symbol, and validates arguments on the host.

No test here launches a kernel: argument errors and no-op sizes return before
any CUDA call, so these run on machines without a GPU.
"""
import ctypes
import os
import re

import pytest

from npbench_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for fn in os.listdir(inc):
        if fn.endswith(".h"):
            with open(os.path.join(inc, fn)) as f:
                names |= set(re.findall(r"NPBGB_API\s+[\w\s\*]+?\b(npbgb_\w+)\s*\(", f.read()))
    return names


def test_header_declares_the_bound_symbols():
    declared = _declared_symbols()
    assert declared, "no NPBGB_API declarations found"
    assert declared == set(_lib.SIGNATURES), (declared ^ set(_lib.SIGNATURES))


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(_lib.LIB_PATH)
    for name in _declared_symbols():
        assert hasattr(lib, name), name


def test_version_and_status_strings():
    lib = _lib.load()
    assert lib.npbgb_version().decode().startswith("npbgb ")
    assert "sm_103a" in lib.npbgb_version().decode()
    assert lib.npbgb_status_string(_lib.NPBGB_OK) == b"ok"
    assert lib.npbgb_status_string(_lib.NPBGB_ERR_TIMEOUT) == b"device wait timed out"
    assert lib.npbgb_status_string(12345) == b"unknown status"


def test_argument_errors_are_status_codes_not_crashes():
    lib = _lib.load()
    assert lib.npbgb_jacobi2d(None, None, -1, 4, 5, _lib.NPBGB_F64, None) == _lib.NPBGB_ERR_ARG
    assert b"negative" in lib.npbgb_last_error()
    assert lib.npbgb_heat3d(None, None, 4, -4, 4, 5, _lib.NPBGB_F32, None) == _lib.NPBGB_ERR_ARG
    assert lib.npbgb_hdiff(None, None, None, 4, 4, 4, _lib.NPBGB_F32, None) == _lib.NPBGB_ERR_DTYPE
    assert lib.npbgb_hdiff(None, None, None, 4, 4, 4, _lib.NPBGB_F64, None) == _lib.NPBGB_ERR_ARG
    assert lib.npbgb_jacobi2d(None, None, 8, 8, 3, _lib.NPBGB_F64, None) == _lib.NPBGB_ERR_ARG
    assert b"null" in lib.npbgb_last_error()
    assert lib.npbgb_jacobi2d(ctypes.c_void_p(4096), ctypes.c_void_p(4096), 8, 8, 3,
                              _lib.NPBGB_F64, None) == _lib.NPBGB_ERR_ARG
    assert b"alias" in lib.npbgb_last_error()
    assert lib.npbgb_heat3d(ctypes.c_void_p(4096), ctypes.c_void_p(8192), 8, 8, 8, 3, 7,
                            None) == _lib.NPBGB_ERR_DTYPE
    assert lib.npbgb_vadv(None, None, None, None, None, 0.15, 4, 4, 4, _lib.NPBGB_F32, None, 0,
                          None) == _lib.NPBGB_ERR_DTYPE
    assert lib.npbgb_vadv(None, None, None, None, None, 0.15, 4, 4, 1, _lib.NPBGB_F64, None, 0,
                          None) == _lib.NPBGB_ERR_ARG
    assert b"level 1" in lib.npbgb_last_error()
    assert lib.npbgb_vadv(None, None, None, None, None, 0.15, 4, 4, 4, _lib.NPBGB_F64, None, 0,
                          None) == _lib.NPBGB_ERR_ARG
    assert b"null" in lib.npbgb_last_error()
    p = [ctypes.c_void_p(4096 * (i + 1)) for i in range(5)]
    assert lib.npbgb_vadv(p[0], p[1], p[2], p[3], p[0], 0.15, 4, 4, 4, _lib.NPBGB_F64, None, 0,
                          None) == _lib.NPBGB_ERR_ARG
    assert b"alias" in lib.npbgb_last_error()
    assert lib.npbgb_vadv(*p, 0.15, 4, 4, 4, _lib.NPBGB_F64, ctypes.c_void_p(65536), 8,
                          None) == _lib.NPBGB_ERR_ARG
    assert b"workspace" in lib.npbgb_last_error()
    assert lib.npbgb_vadv_workspace_bytes(256, 256, 160) == 8 * 159 * 256 * 256
    assert lib.npbgb_vadv_workspace_bytes(4, 4, 1) == 0
    assert lib.npbgb_set_config(_lib.NPBGB_CFG_PDL, 2) == _lib.NPBGB_ERR_ARG
    assert lib.npbgb_set_config(_lib.NPBGB_CFG_HDIFF_EMU, 1 << 24) == _lib.NPBGB_ERR_ARG
    assert lib.npbgb_set_config(_lib.NPBGB_CFG_HDIFF_EMU, -2) == _lib.NPBGB_ERR_ARG
    old = _lib.get_config(_lib.NPBGB_CFG_HDIFF_EMU)
    assert old == -1  # the library's default mask
    assert _lib.set_config(_lib.NPBGB_CFG_HDIFF_EMU, 0xabcdef) == -1
    assert _lib.set_config(_lib.NPBGB_CFG_HDIFF_EMU, old) == 0xabcdef
    for key, bad in ((_lib.NPBGB_CFG_JACOBI1D_CTAS, 9), (_lib.NPBGB_CFG_JACOBI1D_DEPTH, 33),
                     (_lib.NPBGB_CFG_JACOBI1D_DEPTH, 66), (_lib.NPBGB_CFG_JACOBI1D_CTAS, -1)):
        assert lib.npbgb_set_config(key, bad) == _lib.NPBGB_ERR_ARG
    for key, bad in ((_lib.NPBGB_CFG_HEAT_STAGES, 5), (_lib.NPBGB_CFG_HEAT_STAGES, 2),
                     (_lib.NPBGB_CFG_JACOBI_BANDS_WARPS, 12), (_lib.NPBGB_CFG_JACOBI_BANDS, 3),
                     (_lib.NPBGB_CFG_LAUNCHES, 7), (_lib.NPBGB_CFG_HEAT_MAD_ROWS, 65),
                     (_lib.NPBGB_CFG_HEAT_MAD_ROWS, -1), (_lib.NPBGB_CFG_JACOBI_TMA, 3),
                     (_lib.NPBGB_CFG_JACOBI_TMA, -1), (_lib.NPBGB_CFG_BATCH_TMA, 2),
                     (_lib.NPBGB_CFG_BATCH_CTAS_PER_SM, 6), (_lib.NPBGB_CFG_BATCH_CTAS_PER_SM, 1)):
        assert lib.npbgb_set_config(key, bad) == _lib.NPBGB_ERR_ARG
    # the rings: automatic for large binary64 Jacobi-2D grids, off for batches by default
    assert _lib.get_config(_lib.NPBGB_CFG_JACOBI_TMA) == 1
    assert _lib.get_config(_lib.NPBGB_CFG_BATCH_TMA) == 0
    assert _lib.get_config(_lib.NPBGB_CFG_BATCH_CTAS_PER_SM) == 5
    assert _lib.get_config(_lib.NPBGB_CFG_HEAT_STAGES) == 0
    assert _lib.get_config(_lib.NPBGB_CFG_JACOBI_BANDS_WARPS) == 0


def test_launch_counter_counts_only_launched_kernels():
    """The library's launch counter resets to 0 and does not move for calls that
    launch nothing (no-op sizes and argument errors)."""
    lib = _lib.load()
    _lib.set_config(_lib.NPBGB_CFG_LAUNCHES, 0)
    assert _lib.launches() == 0
    assert lib.npbgb_jacobi2d(None, None, 100, 100, 1, _lib.NPBGB_F64, None) == _lib.NPBGB_OK
    assert lib.npbgb_heat3d(None, None, 100, 2, 100, 50, _lib.NPBGB_F64, None) == _lib.NPBGB_OK
    assert lib.npbgb_set_config(_lib.NPBGB_CFG_PDL, 2) == _lib.NPBGB_ERR_ARG
    assert _lib.launches() == 0


def test_noop_sizes_return_ok_without_touching_memory():
    lib = _lib.load()
    # tsteps <= 1 and empty interiors are no-ops, exactly as the reference's loops are.
    assert lib.npbgb_jacobi2d(None, None, 100, 100, 1, _lib.NPBGB_F64, None) == _lib.NPBGB_OK
    assert lib.npbgb_jacobi2d(None, None, 2, 100, 50, _lib.NPBGB_F32, None) == _lib.NPBGB_OK
    assert lib.npbgb_heat3d(None, None, 100, 2, 100, 50, _lib.NPBGB_F64, None) == _lib.NPBGB_OK
    assert lib.npbgb_hdiff(None, None, None, 0, 5, 5, _lib.NPBGB_F64, None) == _lib.NPBGB_OK
    assert lib.npbgb_vadv(None, None, None, None, None, 0.15, 0, 5, 5, _lib.NPBGB_F64, None, 0,
                          None) == _lib.NPBGB_OK


def test_python_errors_mirror_reference_behaviour():
    import numpy as np
    from npbench_gb300 import stencils
    with pytest.raises(ValueError):
        stencils.jacobi_2d_kernel(3, np.zeros((4, 4)), np.zeros((4, 5)))
    with pytest.raises(TypeError):
        stencils.jacobi_2d_kernel(3, np.zeros((4, 4), np.int64), np.zeros((4, 4), np.int64))
    with pytest.raises(TypeError):
        stencils.hdiff(np.zeros((8, 8, 2), np.float32), np.zeros((4, 4, 2), np.float32),
                       np.zeros((4, 4, 2), np.float32))
    with pytest.raises(ValueError):
        stencils.hdiff(np.zeros((8, 9, 2)), np.zeros((4, 4, 2)), np.zeros((4, 4, 2)))
    a = np.zeros((6, 6))
    with pytest.raises(ValueError):
        stencils.jacobi_2d_kernel(3, a, a)
    with pytest.raises(ValueError):
        stencils.heat_3d_kernel(3, np.zeros((4, 4)), np.zeros((4, 4)))
    z = np.zeros((3, 4, 5))
    with pytest.raises(ValueError):
        stencils.vadv(z.copy(), z, np.zeros((3, 4, 5)), z, z, 0.15)   # wcon must be (I+1, J, K)
    with pytest.raises(TypeError):
        stencils.vadv(z.astype(np.float32), z.astype(np.float32), np.zeros((4, 4, 5), np.float32),
                      z.astype(np.float32), z.astype(np.float32), 0.15)
    with pytest.raises(ValueError):
        stencils.vadv(z, z, np.zeros((4, 4, 5)), z.copy(), z.copy(), 0.15)  # output aliases input
    z1 = np.zeros((3, 4, 1))
    with pytest.raises(IndexError):
        stencils.vadv(z1.copy(), z1, np.zeros((4, 4, 1)), z1, z1, 0.15)


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "libnpbgb.so"))
    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _lib.load()
