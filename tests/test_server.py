"""Continuous-batching server: admission logic on the CPU, mixed serving on the GPU.

The GPU test is the one the served configuration asks for: requests of mixed
dimension, size, dtype and step count arrive while others run, are admitted as
memory frees up under a small HBM budget, share persistent launches, and each
result is bit-identical to the same request run alone.
"""
import threading
import time

import numpy as np
import pytest

from npbench_gb300.server import AdmissionController


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
        reqs.append(Request(shape=shape, dtype=dt, tsteps=int(rng.integers(0, 60)), a=a, b=b))
    return reqs


@pytest.mark.gpu
@pytest.mark.parametrize("direct_cells,round_updates", [(1 << 20, 2e9), (600, 2e4)])
def test_served_mix_equals_alone(direct_cells, round_updates):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from npbench_gb300 import stencils
    from npbench_gb300.server import StencilServer
    reqs = _requests(40, seed=3)
    budget = max(r.nbytes for r in reqs) * 3  # small: forces waiting for memory
    futures = []
    with StencilServer(hbm_budget_bytes=budget, quantum=6, direct_cells=direct_cells,
                       round_updates=round_updates) as srv:
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
    assert srv.admission.peak <= budget
    assert srv.rounds > 1
    for r, (A, B) in results:
        a = torch.from_numpy(r.a).cuda()
        b = torch.from_numpy(r.b if r.b is not None else r.a.copy()).cuda()
        (stencils.jacobi_2d_kernel if a.dim() == 2 else stencils.heat_3d_kernel)(r.tsteps, a, b)
        assert np.array_equal(a.cpu().numpy(), A) and np.array_equal(b.cpu().numpy(), B), (
            r.shape, r.dtype, r.tsteps)


@pytest.mark.gpu
def test_server_rejects_oversized_and_cancels_on_stop():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from npbench_gb300.server import Request, StencilServer
    big = Request(shape=(100, 100), dtype=np.float64, tsteps=5, seed=1)
    srv = StencilServer(hbm_budget_bytes=big.nbytes - 1).start()
    with pytest.raises(ValueError):
        srv.submit(big)
    srv.stop()
    # a long queue behind a budget that holds one grid; stop without draining cancels the rest
    srv = StencilServer(hbm_budget_bytes=big.nbytes, quantum=2).start()
    futs = [srv.submit(Request(shape=(100, 100), dtype=np.float64, tsteps=400, seed=i))
            for i in range(6)]
    time.sleep(0.05)
    srv.stop(drain=False)
    assert any(f.cancelled() for f in futs)
    for f in futs:
        if not f.cancelled():
            A, B = f.result(timeout=60)
            assert A.shape == (100, 100)
