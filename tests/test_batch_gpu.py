"""Batched launches == per-grid launches == the oracle, on the GPU.

Every test runs three times: with the batch forced into its persistent form
(one cooperative launch, neighbour counters), into its stepped form (one
chained launch per half-sweep index) and into its queue form (one launch of the
device-side tile work queue), which must all leave the same bits.
"""
import numpy as np
import pytest

from conftest import bits_equal, first_diff

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from npbench_gb300 import _lib, stencils  # noqa: E402
from npbench_gb300.batch import Batch  # noqa: E402
from oracle import cref  # noqa: E402

DEV = torch.device("cuda", 0)


@pytest.fixture(autouse=True, params=[_lib.NPBGB_BATCH_PERSISTENT, _lib.NPBGB_BATCH_STEPPED,
                                      _lib.NPBGB_BATCH_QUEUE],
                ids=["persistent", "stepped", "queue"])
def batch_mode(request):
    old = _lib.set_config(_lib.NPBGB_CFG_BATCH_MODE, request.param)
    yield request.param
    _lib.set_config(_lib.NPBGB_CFG_BATCH_MODE, old)


def _mixed_batch(n, seed, max_side=300, max_t=40):
    rng = np.random.default_rng(seed)
    grids = []
    for g in range(n):
        ny, nx = (int(x) for x in np.exp(rng.uniform(np.log(3), np.log(max_side), 2)).round())
        dt = np.float32 if g % 2 else np.float64
        T = int(rng.integers(0, max_t))
        A = rng.random((ny, nx)).astype(dt)
        B = rng.random((ny, nx)).astype(dt)
        grids.append((A, B, T))
    return grids


@pytest.mark.parametrize("band_rows", [0, 1, 7, 64])
def test_batch_matches_oracle_and_single_launches(band_rows):
    grids = _mixed_batch(40, seed=band_rows)
    dev = [(torch.from_numpy(A).to(DEV), torch.from_numpy(B).to(DEV), T) for A, B, T in grids]
    with Batch(dev, band_rows=band_rows) as b:
        info = b.info()
        assert info["ctas"] >= 1
        b.launch()
        _lib.device_status()
    for n, ((A, B, T), (dA, dB, _)) in enumerate(zip(grids, dev)):
        ra, rb = A.copy(), B.copy()
        cref.jacobi_2d_kernel(T, ra, rb)
        assert bits_equal(dA.cpu().numpy(), ra), (n, A.shape, A.dtype, T, first_diff(dA.cpu().numpy(), ra))
        assert bits_equal(dB.cpu().numpy(), rb), (n, A.shape, A.dtype, T)
        sA, sB = torch.from_numpy(A).to(DEV), torch.from_numpy(B).to(DEV)
        stencils.jacobi_2d_kernel(T, sA, sB)
        assert torch.equal(sA, dA) and torch.equal(sB, dB), n


@pytest.mark.parametrize("tma", [1, 0])
def test_stepped_batch_tma_rings_match_oracle(batch_mode, tma):
    """The stepped form's binary64 Jacobi-2D tiles through each warp's TMA ring (rows
    of a 16-byte multiple, on request) or plain loads: the oracle's bits on uniform and
    mixed-range fields, even and odd widths, tiles of 1, 7 and 32 rows."""
    if batch_mode != _lib.NPBGB_BATCH_STEPPED:
        pytest.skip("the TMA rings belong to the stepped form")
    rng = np.random.default_rng(7 + tma)
    grids = []
    for g, (ny, nx) in enumerate([(3, 4), (9, 30), (40, 34), (130, 258), (77, 64), (65, 65), (200, 17)]):
        A = rng.random((ny, nx))
        B = rng.random((ny, nx))
        if g % 3 == 1:  # values outside the fixed-point range take the hardware path
            flat = A.reshape(-1)
            flat[rng.choice(flat.size, size=max(1, flat.size // 20), replace=False)] = -0.5
        grids.append((A, B, int(rng.integers(2, 12))))
    old = _lib.set_config(_lib.NPBGB_CFG_BATCH_TMA, tma)
    try:
        for rows in (1, 7, 32):
            dev = [(torch.from_numpy(A).to(DEV), torch.from_numpy(B).to(DEV), T) for A, B, T in grids]
            with Batch(dev, band_rows=rows) as b:
                b.launch()
                _lib.device_status()
            for n, ((A, B, T), (dA, dB, _)) in enumerate(zip(grids, dev)):
                ra, rb = A.copy(), B.copy()
                cref.jacobi_2d_kernel(T, ra, rb)
                assert bits_equal(dA.cpu().numpy(), ra), (tma, rows, n, A.shape, T,
                                                          first_diff(dA.cpu().numpy(), ra))
                assert bits_equal(dB.cpu().numpy(), rb), (tma, rows, n, A.shape, T)
    finally:
        _lib.set_config(_lib.NPBGB_CFG_BATCH_TMA, old)


def test_batch_graph_replay_is_repeatable():
    grids = _mixed_batch(25, seed=99, max_side=500, max_t=30)
    init = [(torch.from_numpy(A).to(DEV), torch.from_numpy(B).to(DEV), T) for A, B, T in grids]
    work = [(a.clone(), b.clone(), T) for a, b, T in init]
    results = []
    with Batch(work) as b:
        for rep in range(3):
            for (a0, b0, _), (a, bb, _) in zip(init, work):
                a.copy_(a0)
                bb.copy_(b0)
            b.launch(graph=True)
            _lib.device_status()
            results.append([(a.clone(), bb.clone()) for a, bb, _ in work])
    for rep in (1, 2):
        for (a1, b1), (a2, b2) in zip(results[0], results[rep]):
            assert torch.equal(a1, a2) and torch.equal(b1, b2)
    for (A, B, T), (a, bb) in zip(grids, results[0]):
        ra, rb = A.copy(), B.copy()
        cref.jacobi_2d_kernel(T, ra, rb)
        assert bits_equal(a.cpu().numpy(), ra) and bits_equal(bb.cpu().numpy(), rb)


def test_batch_f64_emulation_off_matches():
    grids = _mixed_batch(12, seed=5)
    dev = [(torch.from_numpy(A).to(DEV), torch.from_numpy(B).to(DEV), T) for A, B, T in grids]
    old = _lib.set_config(_lib.NPBGB_CFG_F64_EMULATION, 0)
    try:
        with Batch(dev) as b:
            b.launch()
            _lib.device_status()
    finally:
        _lib.set_config(_lib.NPBGB_CFG_F64_EMULATION, old)
    for (A, B, T), (dA, dB, _) in zip(grids, dev):
        ra, rb = A.copy(), B.copy()
        cref.jacobi_2d_kernel(T, ra, rb)
        assert bits_equal(dA.cpu().numpy(), ra) and bits_equal(dB.cpu().numpy(), rb)


def test_empty_and_trivial_batches():
    with Batch([]) as b:
        b.launch()
    A = torch.rand(2, 9, dtype=torch.float64, device=DEV)
    B = torch.rand(2, 9, dtype=torch.float64, device=DEV)
    a0 = A.clone()
    with Batch([(A, B, 50)]) as b:  # no interior: nothing to do, as in the reference
        b.launch()
        assert b.info()["bands"] == 0
    assert torch.equal(A, a0)


def _heat_grids(n, seed, max_side=40, max_t=12):
    rng = np.random.default_rng(seed)
    grids = []
    for g in range(n):
        shape = tuple(int(x) for x in np.exp(rng.uniform(np.log(3), np.log(max_side), 3)).round())
        dt = np.float32 if g % 2 else np.float64
        T = int(rng.integers(0, max_t))
        A = rng.random(shape).astype(dt)
        grids.append((A, A.copy(), T))
    return grids


@pytest.mark.parametrize("band_rows", [0, 1, 5])
def test_batch_mixed_jacobi_and_heat(band_rows):
    grids = _mixed_batch(15, seed=7, max_side=200, max_t=20) + _heat_grids(15, seed=8)
    dev = [(torch.from_numpy(A).to(DEV), torch.from_numpy(B).to(DEV), T) for A, B, T in grids]
    with Batch(dev, band_rows=band_rows) as b:
        b.launch()
        _lib.device_status()
    for n, ((A, B, T), (dA, dB, _)) in enumerate(zip(grids, dev)):
        ra, rb = A.copy(), B.copy()
        (cref.jacobi_2d_kernel if A.ndim == 2 else cref.heat_3d_kernel)(T, ra, rb)
        assert bits_equal(dA.cpu().numpy(), ra), (n, A.shape, A.dtype, T, first_diff(dA.cpu().numpy(), ra))
        assert bits_equal(dB.cpu().numpy(), rb), (n, A.shape, A.dtype, T)


def test_batch_resumed_in_pieces_equals_one_run():
    """step0/nsteps: a run split over several launches gives the uninterrupted bits."""
    grids = _mixed_batch(8, seed=11, max_side=120, max_t=30) + _heat_grids(8, seed=12, max_t=20)
    dev = [(torch.from_numpy(A).to(DEV), torch.from_numpy(B).to(DEV), T) for A, B, T in grids]
    done = [0] * len(dev)
    total = [max(0, 2 * (T - 1)) for _, _, T in grids]
    piece = 3
    while any(d < t for d, t in zip(done, total)):
        entries = [(a, b, T, done[n], piece) for n, (a, b, T) in enumerate(dev) if done[n] < total[n]]
        with Batch(entries) as b:
            b.launch()
            _lib.device_status()
        for n in range(len(dev)):
            done[n] = min(total[n], done[n] + piece)
    for n, ((A, B, T), (dA, dB, _)) in enumerate(zip(grids, dev)):
        ra, rb = A.copy(), B.copy()
        (cref.jacobi_2d_kernel if A.ndim == 2 else cref.heat_3d_kernel)(T, ra, rb)
        assert bits_equal(dA.cpu().numpy(), ra) and bits_equal(dB.cpu().numpy(), rb), n


def test_batch_reports_its_form(batch_mode):
    A = torch.rand((40, 50), dtype=torch.float64, device=DEV)
    B = A.clone()
    with Batch([(A, B, 5)]) as bt:
        info = bt.info()
    assert info["mode"] == {_lib.NPBGB_BATCH_STEPPED: "stepped",
                            _lib.NPBGB_BATCH_QUEUE: "queue"}.get(batch_mode, "persistent")
    assert info["updates"] == 8 * 38 * 48


def test_batch_form_can_be_chosen_per_batch(batch_mode):
    """Batch(..., mode=...) overrides the configured form for that plan only."""
    A = torch.rand((40, 50), dtype=torch.float32, device=DEV)
    B = A.clone()
    for name in ("persistent", "stepped", "queue"):
        with Batch([(A, B, 3)], mode=name) as bt:
            assert bt.info()["mode"] == name
            bt.replan([(A, B, 4)], mode=name)
            assert bt.info()["mode"] == name
    assert _lib.get_config(_lib.NPBGB_CFG_BATCH_MODE) == batch_mode
