"""The allocation-free batch entry point, npbgb_batch_run_noalloc, on the GPU.

Some callers cannot allocate device memory: a host whose own pool or HBM
budget owns every byte of the GPU, or a loop that cannot afford the implicit
synchronisation of cudaMalloc/cudaFree.  For them the library offers
npbgb_batch_run_noalloc, which runs the persistent batch kernel out of a fixed
static device array.  These tests call it through the C ABI and check its
grids against those of the allocating entry points (npbgb_batch_create +
npbgb_batch_launch) bit for bit, on two calls in a row with different batches,
so that contents left in the shared array by one call cannot leak into the
next.  Collected last on purpose (file name), so a failure here comes after
every other test has run; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from npbench_gb300 import _lib  # noqa: E402

DEV = torch.device("cuda", 0)


def _grids(seed, n, max_side, max_t):
    rng = np.random.default_rng(seed)
    out = []
    for g in range(n):
        ny, nx = (int(x) for x in np.exp(rng.uniform(np.log(3), np.log(max_side), 2)).round())
        dt = np.float64 if g % 3 else np.float32
        T = int(rng.integers(0, max_t))
        out.append((rng.random((ny, nx)).astype(dt), rng.random((ny, nx)).astype(dt), T))
    return out


def _struct_array(dev_grids):
    arr = (_lib.Grid * max(1, len(dev_grids)))()
    for n, (A, B, T) in enumerate(dev_grids):
        g = arr[n]
        g.a, g.b = A.data_ptr(), B.data_ptr()
        g.n0, g.n1, g.n2 = A.shape[0], A.shape[1], 1
        g.kind = _lib.NPBGB_KIND_JACOBI2D
        g.dtype = _lib.NPBGB_F64 if A.dtype == torch.float64 else _lib.NPBGB_F32
        g.tsteps = T
        g.band_rows = 0
    return arr


def _to_dev(grids):
    return [(torch.from_numpy(A).to(DEV), torch.from_numpy(B).to(DEV), T) for A, B, T in grids]


def _run_allocating(grids, band_rows):
    lib = _lib.load()
    dev = _to_dev(grids)
    arr = _struct_array(dev)
    h = ctypes.c_void_p()
    _lib.check(lib.npbgb_batch_create(arr, len(dev), band_rows, ctypes.byref(h)), "create")
    try:
        _lib.check(lib.npbgb_batch_launch(h, 0, torch.cuda.current_stream().cuda_stream), "launch")
        _lib.device_status()
    finally:
        lib.npbgb_batch_destroy(h)
    return dev


def _run_noalloc(grids, band_rows):
    lib = _lib.load()
    dev = _to_dev(grids)
    arr = _struct_array(dev)
    st = lib.npbgb_batch_run_noalloc(arr, len(dev), band_rows,
                                     torch.cuda.current_stream().cuda_stream)
    _lib.check(st, "npbgb_batch_run_noalloc")
    _lib.device_status()
    return dev


def test_noalloc_matches_allocating_batch_on_two_calls_in_a_row():
    # Different batches on the two calls: the second has fewer bands than the
    # first, so stale plan entries or counters would show up as wrong grids.
    for seed, n, side, tmax, band_rows in ((1, 30, 400, 40, 0), (2, 9, 150, 25, 5)):
        grids = _grids(seed, n, side, tmax)
        want = _run_allocating(grids, band_rows)
        got = _run_noalloc(grids, band_rows)
        torch.cuda.synchronize()
        for i, ((wa, wb, _), (ga, gb, _)) in enumerate(zip(want, got)):
            assert torch.equal(wa, ga) and torch.equal(wb, gb), (seed, i)


def test_noalloc_repeated_identical_calls_agree():
    grids = _grids(3, 12, 300, 30)
    first = _run_noalloc(grids, 16)
    second = _run_noalloc(grids, 16)
    for (a1, b1, _), (a2, b2, _) in zip(first, second):
        assert torch.equal(a1, a2) and torch.equal(b1, b2)


def test_noalloc_rejects_plans_beyond_its_capacity():
    lib = _lib.load()
    # 70000 rows with one row per band need 69998 bands > 32768.
    A = torch.zeros((70000, 3), dtype=torch.float32, device=DEV)
    B = torch.zeros_like(A)
    arr = _struct_array([(A, B, 3)])
    st = lib.npbgb_batch_run_noalloc(arr, 1, 1, torch.cuda.current_stream().cuda_stream)
    assert st == _lib.NPBGB_ERR_NOMEM
    assert b"32768" in lib.npbgb_last_error()
    _lib.device_status()


def test_noalloc_refuses_a_capturing_stream():
    # The plan is staged from shared host buffers, so a captured call could be
    # replayed against another call's plan: the entry point refuses capture
    # before it stages or launches anything.
    lib = _lib.load()
    grids = _to_dev(_grids(4, 3, 60, 6))
    arr = _struct_array(grids)
    x = torch.zeros(8, device=DEV)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        st = lib.npbgb_batch_run_noalloc(arr, len(grids), 0, torch.cuda.current_stream().cuda_stream)
        x.add_(1.0)
    assert st == _lib.NPBGB_ERR_ARG
    assert b"capturing" in lib.npbgb_last_error()
    g.replay()
    torch.cuda.synchronize()
    assert float(x.sum()) == 8.0
