"""The device-side tile work queue with grids added while its worker runs.

Grids of both kinds and precisions, ragged shapes and step counts are
submitted one at a time, some while the worker kernel is already running,
cut into tiles or run whole;
each must end bit for bit as the oracle (the C restatement of the
reference's NumPy kernels) leaves it, which is also what the grid gives when
run alone.  The worker ends by itself once idle and is launched again for
later grids.  A full queue refuses a grid with a status, not a crash.
"""
import time

import numpy as np
import pytest

from conftest import bits_equal, first_diff

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from npbench_gb300 import _lib, stencils  # noqa: E402
from npbench_gb300.queue import TileQueue  # noqa: E402
from oracle import cref  # noqa: E402

DEV = torch.device("cuda", 0)


@pytest.fixture(autouse=True, params=[0, 65536, 1 << 40], ids=["tiles", "small-whole", "all-whole"])
def whole_cells(request):
    """Every test with no grid run whole, with the default (grids up to 65536 cells
    run whole: one CTA per half-sweep, running on to the next ones), and with every
    grid run whole."""
    old = _lib.set_config(_lib.NPBGB_CFG_QUEUE_WHOLE_CELLS, request.param)
    yield request.param
    _lib.set_config(_lib.NPBGB_CFG_QUEUE_WHOLE_CELLS, old)


def _grids(n, seed, max2d=260, max3d=36, max_t=25):
    rng = np.random.default_rng(seed)
    out = []
    for g in range(n):
        dt = np.float32 if g % 2 else np.float64
        T = int(rng.integers(0, max_t))
        if g % 3 == 2:
            shape = tuple(int(x) for x in np.exp(rng.uniform(np.log(3), np.log(max3d), 3)).round())
            A = rng.random(shape).astype(dt)
            out.append((A, A.copy(), T))
        else:
            shape = tuple(int(x) for x in np.exp(rng.uniform(np.log(3), np.log(max2d), 2)).round())
            out.append((rng.random(shape).astype(dt), rng.random(shape).astype(dt), T))
    return out


def _oracle(A, B, T):
    ra, rb = A.copy(), B.copy()
    (cref.jacobi_2d_kernel if A.ndim == 2 else cref.heat_3d_kernel)(T, ra, rb)
    return ra, rb


def _drain(q, pending, limit_s=60.0):
    t0 = time.perf_counter()
    while pending:
        q.kick()
        for s in q.poll():
            pending.discard(s)
        assert time.perf_counter() - t0 < limit_s, "queue did not drain"
        time.sleep(0.0005)
    assert q.state()["busy"] == 0


@pytest.mark.parametrize("tile_rows", [0, 3])
def test_grids_submitted_while_running_match_the_oracle(tile_rows):
    grids = _grids(36, seed=tile_rows + 1)
    dev = [(torch.from_numpy(A).to(DEV), torch.from_numpy(B).to(DEV), T) for A, B, T in grids]
    torch.cuda.synchronize()
    with TileQueue(max_slots=64, tile_rows=tile_rows, tile_planes=tile_rows) as q:
        pending = set()
        for n, (a, b, T) in enumerate(dev):
            slot = q.submit(a, b, T)
            if slot >= 0:
                pending.add(slot)
            q.kick()
            if n % 5 == 4:
                time.sleep(0.002)  # later grids arrive while earlier ones run
        _drain(q, pending)
        _lib.device_status()
    for n, ((A, B, T), (a, b, _)) in enumerate(zip(grids, dev)):
        ra, rb = _oracle(A, B, T)
        assert bits_equal(a.cpu().numpy(), ra), (n, A.shape, A.dtype, T,
                                                 first_diff(a.cpu().numpy(), ra))
        assert bits_equal(b.cpu().numpy(), rb), (n, A.shape, A.dtype, T)


def test_mixed_run_equals_each_grid_alone():
    grids = _grids(20, seed=40, max2d=400, max3d=48, max_t=40)
    dev = [(torch.from_numpy(A).to(DEV), torch.from_numpy(B).to(DEV), T) for A, B, T in grids]
    with TileQueue(max_slots=32) as q:
        pending = {q.submit(a, b, T) for a, b, T in dev} - {-1}
        _drain(q, pending)
    for (A, B, T), (a, b, _) in zip(grids, dev):
        sa, sb = torch.from_numpy(A).to(DEV), torch.from_numpy(B).to(DEV)
        (stencils.jacobi_2d_kernel if A.ndim == 2 else stencils.heat_3d_kernel)(T, sa, sb)
        assert torch.equal(sa, a) and torch.equal(sb, b)


def test_resumed_pieces_through_the_queue_equal_one_run():
    grids = _grids(9, seed=77, max_t=30)
    dev = [(torch.from_numpy(A).to(DEV), torch.from_numpy(B).to(DEV), T) for A, B, T in grids]
    total = [max(0, 2 * (T - 1)) for _, _, T in grids]
    done = [0] * len(dev)
    with TileQueue(max_slots=16) as q:
        while any(d < t for d, t in zip(done, total)):
            pending = set()
            for n, (a, b, T) in enumerate(dev):
                if done[n] < total[n]:
                    s = q.submit(a, b, T, step0=done[n], nsteps=4)
                    assert s >= 0
                    pending.add(s)
            _drain(q, pending)
            done = [min(t, d + 4) for d, t in zip(done, total)]
    for (A, B, T), (a, b, _) in zip(grids, dev):
        ra, rb = _oracle(A, B, T)
        assert bits_equal(a.cpu().numpy(), ra) and bits_equal(b.cpu().numpy(), rb)


def test_long_runs_pass_through_the_ring_many_times():
    """Grids of 598 half-sweeps: a whole grid goes back to the ring every 256 of them
    (and a tiled one every half-sweep); each still ends as the oracle leaves it."""
    rng = np.random.default_rng(12)
    grids = []
    for shape, dt in (((40, 41), np.float64), ((33, 70), np.float32), ((10, 12, 9), np.float64),
                      ((7, 34, 40), np.float32)):
        A = rng.random(shape).astype(dt)
        B = rng.random(shape).astype(dt) if len(shape) == 2 else A.copy()
        grids.append((A, B, 300))
    dev = [(torch.from_numpy(A).to(DEV), torch.from_numpy(B).to(DEV), T) for A, B, T in grids]
    with TileQueue(max_slots=8) as q:
        pending = {q.submit(a, b, T) for a, b, T in dev} - {-1}
        _drain(q, pending)
        _lib.device_status()
    for (A, B, T), (a, b, _) in zip(grids, dev):
        ra, rb = _oracle(A, B, T)
        assert bits_equal(a.cpu().numpy(), ra) and bits_equal(b.cpu().numpy(), rb), A.shape


def test_worker_ends_when_idle_and_is_launched_again():
    grids = _grids(4, seed=5, max_t=10)
    dev = [(torch.from_numpy(A).to(DEV), torch.from_numpy(B).to(DEV), T) for A, B, T in grids]
    with TileQueue(max_slots=8, idle_us=1000) as q:
        pending = {q.submit(a, b, T) for a, b, T in dev[:2]} - {-1}
        _drain(q, pending)
        torch.cuda.synchronize()  # the worker ends within its idle limit
        assert not q.state()["running"]
        first = q.state()["launches"]
        pending = {q.submit(a, b, T) for a, b, T in dev[2:]} - {-1}
        _drain(q, pending)
        assert q.state()["launches"] == first + 1
    for (A, B, T), (a, b, _) in zip(grids, dev):
        ra, rb = _oracle(A, B, T)
        assert bits_equal(a.cpu().numpy(), ra) and bits_equal(b.cpu().numpy(), rb)


def test_full_queue_refuses_with_a_status():
    grids = _grids(3, seed=9, max_t=8)
    dev = [(torch.from_numpy(A).to(DEV), torch.from_numpy(B).to(DEV), max(T, 3))
           for A, B, T in grids]
    with TileQueue(max_slots=2) as q:
        s0 = q.submit(*dev[0])
        s1 = q.submit(*dev[1])
        with pytest.raises(_lib.NpbgbError) as e:
            q.submit(*dev[2])
        assert e.value.status == _lib.NPBGB_ERR_NOMEM
        _drain(q, {s0, s1} - {-1})
        s2 = q.submit(*dev[2])
        _drain(q, {s2} - {-1})
    for (A, B, _), (a, b, T) in zip(grids, dev):
        ra, rb = _oracle(A, B, T)
        assert bits_equal(a.cpu().numpy(), ra) and bits_equal(b.cpu().numpy(), rb)


def test_batch_guard_promotes_long_float32_grids():
    """Batch(guard=True): float32 Jacobi-2D grids above the calibrated float32 error
    bound run in float64 and equal the float64 oracle rounded once; the others stay
    float32, bit-identical to the float32 oracle; all are within 1e-5 of float64."""
    from npbench_gb300.batch import Batch
    rng = np.random.default_rng(21)
    cases = [((200, 150), np.float32, 600), ((120, 90), np.float32, 30),
             ((90, 70), np.float64, 300), ((20, 30, 24), np.float32, 300)]
    host, dev = [], []
    for shape, dt, T in cases:
        A = rng.random(shape).astype(dt)
        B = rng.random(shape).astype(dt) if len(shape) == 2 else A.copy()
        host.append((A, B, T))
        dev.append((torch.from_numpy(A).to(DEV), torch.from_numpy(B).to(DEV), T))
    init = [(a.clone(), b.clone()) for a, b, _ in dev]
    for mode, name in ((None, "stepped"), ("queue", "queue"), ("stepped", "stepped")):
        for (a0, b0), (a, b, _) in zip(init, dev):
            a.copy_(a0)
            b.copy_(b0)
        with Batch(dev, guard=True, mode=mode) as bt:
            assert bt.promoted == 1 and bt.info()["mode"] == name
            bt.launch()
            _lib.device_status()
        _check_guarded(host, dev)
    with pytest.raises(ValueError):
        Batch(dev, guard=True, mode="persistent")


def _check_guarded(host, dev):
    for n, ((A, B, T), (a, b, _)) in enumerate(zip(host, dev)):
        ga, gb = a.cpu().numpy(), b.cpu().numpy()
        oa, ob = A.astype(np.float64), B.astype(np.float64)
        (cref.jacobi_2d_kernel if A.ndim == 2 else cref.heat_3d_kernel)(T, oa, ob)
        rel = np.linalg.norm(ga.astype(np.float64) - oa) / np.linalg.norm(oa)
        assert rel <= 1e-5, (n, rel)
        if n == 0:
            assert np.array_equal(ga, oa.astype(np.float32)) and np.array_equal(gb, ob.astype(np.float32))
        else:
            ra, rb = _oracle(A, B, T)
            assert bits_equal(ga, ra) and bits_equal(gb, rb), n
