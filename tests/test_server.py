"""Continuous-batching server: admission logic on the CPU, mixed serving on the GPU.

The GPU test is the one the served configuration asks for: requests of mixed
dimension, size, dtype and step count arrive while others run, are admitted as
memory frees up under a small HBM budget, are folded into the running
device-side tile queue, and each result is bit-identical to the same request
run alone (under the same float64 guard).  The guard's own test runs a float32
request above the calibrated error bound (promoted to float64) and one below
it (kept float32), both within 1e-5 of the float64 oracle.
"""
import threading
import time

import numpy as np
import pytest

from npbench_gb300 import precision
from npbench_gb300.server import AdmissionController, guarded


def test_admission_budget_and_peak():
    a = AdmissionController(100)
    assert a.fits_ever(100) and not a.fits_ever(101)
    assert a.try_admit(60)
    assert not a.try_admit(50)
    assert a.try_admit(40)
    assert a.in_use == 100 and a.peak == 100
    a.release(60)
    assert a.try_admit(50) and a.in_use == 90
    with pytest.raises(RuntimeError):
        a.release(1000)
    with pytest.raises(ValueError):
        AdmissionController(0)


def test_admission_is_thread_safe():
    a = AdmissionController(1000)
    got = []

    def worker():
        for _ in range(200):
            if a.try_admit(7):
                got.append(7)

    ts = [threading.Thread(target=worker) for _ in range(8)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert sum(got) <= 1000 and a.in_use == sum(got)


def test_float32_error_model_and_guard_threshold():
    """The calibrated table: Jacobi-2D float32 error grows with TSTEPS and crosses the
    bound (with its safety margin) between TSTEPS 100 and 200; Heat-3D never does."""
    prev = 0.0
    for T in (2, 10, 50, 100, 150, 200, 500, 1000, 3000):
        e = precision.predicted_rel_l2("jacobi2d", T)
        assert e >= prev
        prev = e
    assert not precision.needs_fp64("jacobi2d", 100) and precision.needs_fp64("jacobi2d", 200)
    assert not any(precision.needs_fp64("heat3d", T) for T in (2, 100, 1000, 2000))
    assert precision.predicted_rel_l2((10, 10), 1) == 0.0
    assert guarded("jacobi2d", np.float32, 500) and not guarded("jacobi2d", np.float64, 500)
    assert not guarded("jacobi2d", np.float32, 500, fp64_guard=False)
    assert not guarded("heat3d", np.float32, 1000)


def _requests(n, seed):
    from npbench_gb300.server import Request
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n):
        dt = np.float32 if rng.random() < 0.7 else np.float64
        if i % 2:
            shape = tuple(int(x) for x in rng.integers(3, 160, 2))
            a, b = rng.random(shape).astype(dt), rng.random(shape).astype(dt)
        else:
            shape = tuple(int(x) for x in rng.integers(3, 40, 3))
            a = rng.random(shape).astype(dt)
            b = None
        # 2D runs up to TSTEPS 200, so float32 ones above the error bound get promoted
        T = int(rng.integers(0, 200 if i % 2 else 60))
        reqs.append(Request(shape=shape, dtype=dt, tsteps=T, a=a, b=b))
    return reqs


def _alone(r):
    """The request run alone with per-grid launches, under the same float64 guard."""
    import torch
    from npbench_gb300 import stencils
    a = torch.from_numpy(r.a).cuda()
    b = torch.from_numpy(r.b if r.b is not None else r.a.copy()).cuda()
    fn = stencils.jacobi_2d_kernel if a.dim() == 2 else stencils.heat_3d_kernel
    if r.promoted:
        a64, b64 = a.double(), b.double()
        fn(r.tsteps, a64, b64)
        a.copy_(a64)
        b.copy_(b64)
    else:
        fn(r.tsteps, a, b)
    return a.cpu().numpy(), b.cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("tile_rows,direct_cells", [(0, 1 << 20), (5, 1 << 20), (0, 3000)])
def test_served_mix_equals_alone(tile_rows, direct_cells):
    """Requests arrive from three client threads while others run, wait for
    memory under a small budget, and each result equals the request run alone
    (all through the tile queue, or the larger ones through a big-grid lane)."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from npbench_gb300.server import StencilServer
    reqs = _requests(40, seed=3)
    budget = max(2 * r.cells * 16 for r in reqs) * 3  # small: forces waiting for memory
    futures = []
    with StencilServer(hbm_budget_bytes=budget, tile_rows=tile_rows, tile_planes=tile_rows,
                       reserve_bytes=budget, direct_cells=direct_cells, big_lanes=2) as srv:
        def client(part):
            for r in part:
                futures.append((r, srv.submit(r)))
                time.sleep(0.002)
        ts = [threading.Thread(target=client, args=(reqs[k::3],)) for k in range(3)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
        results = [(r, f.result(timeout=300)) for r, f in futures]
    assert srv.admission.peak <= budget and srv.admission.in_use == 0
    assert srv.queued_small + srv.ran_big <= len(reqs) and srv.queued_small >= 1
    if direct_cells < 10000:
        assert srv.ran_big >= 1
    for r, (A, B) in results:
        a, b = _alone(r)
        assert np.array_equal(a, A) and np.array_equal(b, B), (r.shape, r.dtype, r.tsteps)


@pytest.mark.gpu
def test_float64_guard_promotes_long_float32_runs():
    """A float32 Jacobi-2D run above the calibrated error bound runs in float64
    (and ends within 1e-5 of the float64 oracle, where plain float32 does not);
    one below it stays float32 and is bit-identical to the float32 oracle."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from npbench_gb300 import precision
    from npbench_gb300.server import Request, StencilServer, guarded
    from oracle import cref
    rng = np.random.default_rng(12)
    A64, B64 = rng.random((300, 260)), rng.random((300, 260))
    A32, B32 = A64.astype(np.float32), B64.astype(np.float32)
    long_T, short_T = 900, 40
    assert guarded("jacobi2d", np.float32, long_T) and not guarded("jacobi2d", np.float32, short_T)
    assert precision.predicted_rel_l2("jacobi2d", long_T) > precision.BOUND
    with StencilServer(hbm_budget_bytes=1 << 30, reserve_bytes=1 << 28) as srv:
        f_long = srv.submit(Request(shape=A32.shape, dtype=np.float32, tsteps=long_T, a=A32, b=B32))
        f_short = srv.submit(Request(shape=A32.shape, dtype=np.float32, tsteps=short_T, a=A32, b=B32))
        (la, lb), (sa, sb) = f_long.result(timeout=120), f_short.result(timeout=120)
    assert srv.promoted == 1
    assert la.dtype == np.float32 and sa.dtype == np.float32

    def rel(x, ref):
        return float(np.linalg.norm(x.astype(np.float64) - ref) / np.linalg.norm(ref))
    # float64 oracle of the float32 inputs (widened exactly)
    for T, (ra, rb) in ((long_T, (la, lb)), (short_T, (sa, sb))):
        oa, ob = A32.astype(np.float64), B32.astype(np.float64)
        cref.jacobi_2d_kernel(T, oa, ob)
        assert rel(ra, oa) <= 1e-5 and rel(rb, ob) <= 1e-5, T
    # the promoted result is the float64 run rounded once
    oa, ob = A32.astype(np.float64), B32.astype(np.float64)
    cref.jacobi_2d_kernel(long_T, oa, ob)
    assert np.array_equal(la, oa.astype(np.float32)) and np.array_equal(lb, ob.astype(np.float32))
    # plain float32 would have missed the bound on the long run
    pa, pb = A32.copy(), B32.copy()
    cref.jacobi_2d_kernel(long_T, pa, pb)
    assert rel(pa, oa) > 1e-5
    # the short run stayed float32: bit-identical to the float32 oracle
    qa, qb = A32.copy(), B32.copy()
    cref.jacobi_2d_kernel(short_T, qa, qb)
    assert np.array_equal(sa, qa) and np.array_equal(sb, qb)


@pytest.mark.gpu
def test_server_rejects_oversized_and_cancels_on_stop():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from npbench_gb300.server import Request, StencilServer
    big = Request(shape=(100, 100), dtype=np.float64, tsteps=5, seed=1)
    srv = StencilServer(hbm_budget_bytes=big.nbytes - 1, reserve_bytes=0).start()
    with pytest.raises(ValueError):
        srv.submit(big)
    srv.stop()
    # a long queue behind a budget that holds one grid (each takes tens of
    # milliseconds); stop without draining cancels the rest
    one = Request(shape=(1024, 1024), dtype=np.float64, tsteps=3000, seed=0)
    srv = StencilServer(hbm_budget_bytes=one.nbytes, reserve_bytes=0).start()
    futs = [srv.submit(Request(shape=(1024, 1024), dtype=np.float64, tsteps=3000, seed=i,
                               return_host=False))
            for i in range(6)]
    time.sleep(0.02)
    srv.stop(drain=False)
    assert any(f.cancelled() for f in futs)
    for f in futs:
        if not f.cancelled():
            A, B = f.result(timeout=60)
            assert tuple(A.shape) == (1024, 1024)
