"""npbench_gb300.autotune: the per-shape cache of launch settings.

CPU: cache keys, the JSON round trip, and that a cached setting is applied for
exactly the duration of a call and restored after it (the library's knobs are
host-side state, so this needs no GPU).  GPU: tuning a small grid stores a
setting, every candidate it timed left the default setting's bits, and a
tuned call still matches the oracle bit for bit.
"""
import json

import numpy as np
import pytest

from npbench_gb300 import _lib, autotune


@pytest.fixture
def cache(tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    monkeypatch.setenv("NPBGB_TUNE_CACHE", str(path))
    autotune.load_cache(refresh=True)
    was = autotune.enabled()
    yield path
    (autotune.enable if was else autotune.disable)()
    monkeypatch.delenv("NPBGB_TUNE_CACHE")
    autotune.load_cache(refresh=True)


def test_keys_name_benchmark_dtype_and_shape_class():
    assert autotune.shape_class((2800, 2800)) == (11, 11)
    assert autotune.key("jacobi_2d", (2800, 2800), np.float64) == "jacobi_2d/float64/c11x11"
    assert autotune.key("heat_3d", [120, 120, 120], "float32") == "heat_3d/float32/c6x6x6"
    # grids within a factor of two share a class
    assert autotune.key("heat_3d", (256,) * 3, "float64") == autotune.key("heat_3d", (511, 300, 257),
                                                                         "float64")
    assert autotune.key("heat_3d", (256,) * 3, "float64") != autotune.key("heat_3d", (255, 256, 256),
                                                                         "float64")
    torch = pytest.importorskip("torch")
    assert autotune.key("heat_3d", (4, 5, 6), torch.float64) == "heat_3d/float64/c2x2x2"


def test_search_spaces():
    sp = autotune._space("jacobi_2d", np.float64)
    assert {"JACOBI_HW_WARPS": 4, "JACOBI_CHUNK": 3, "JACOBI_BANDS": 0} in sp and len(sp) == 65
    # binary64: the chained launches, the whole loop in one launch (bands), or the
    # chained launches with each warp's TMA ring forced on
    assert {"JACOBI_HW_WARPS": 4, "JACOBI_CHUNK": 0, "JACOBI_BANDS": 2} in sp
    assert {"JACOBI_HW_WARPS": 3, "JACOBI_CHUNK": 16, "JACOBI_BANDS": 0, "JACOBI_TMA": 2} in sp
    assert all("JACOBI_TMA" not in c for c in autotune._space("jacobi_2d", np.float32))
    f32j = autotune._space("jacobi_2d", np.float32)
    assert all(c["JACOBI_HW_WARPS"] == -1 and "JACOBI_BANDS" not in c for c in f32j)
    heat = autotune._space("heat_3d", np.float64)
    assert all("HEAT_TB" not in c for c in heat)
    f32 = autotune._space("heat_3d", np.float32)
    assert {c["HEAT_TB"] for c in f32} == {1, 2}  # temporal depth is a knob in binary32
    assert {"HEAT_ROWS": 2, "HEAT_HW_ROWS": 4, "HEAT_CHUNK": 8} in heat
    assert {"HEAT_ROWS": 2, "HEAT_HW_ROWS": 5, "HEAT_CHUNK": 8} in heat
    assert {"HEAT_ROWS": 2, "HEAT_HW_ROWS": 7, "HEAT_CHUNK": 8} in heat
    with pytest.raises(ValueError):
        autotune._space("hdiff", np.float64)


def test_cached_setting_applies_for_the_call_only(cache):
    cache.write_text(json.dumps({"jacobi_2d/float64/c5x5": {
        "config": {"JACOBI_HW_WARPS": 6, "JACOBI_CHUNK": 5}, "ms": 1.0, "default_ms": 2.0}}))
    autotune.load_cache(refresh=True)
    before = (_lib.get_config(_lib.NPBGB_CFG_JACOBI_HW_WARPS),
              _lib.get_config(_lib.NPBGB_CFG_JACOBI_CHUNK))
    autotune.disable()
    with autotune.applied("jacobi_2d", (40, 50), np.float64) as cfg:
        assert cfg is None
    autotune.enable()
    with autotune.applied("jacobi_2d", (40, 50), np.float64) as cfg:
        assert cfg == {"JACOBI_HW_WARPS": 6, "JACOBI_CHUNK": 5}
        assert _lib.get_config(_lib.NPBGB_CFG_JACOBI_HW_WARPS) == 6
        assert _lib.get_config(_lib.NPBGB_CFG_JACOBI_CHUNK) == 5
    # an unseen shape of the same class gets the setting; another class does not
    with autotune.applied("jacobi_2d", (61, 33), np.float64) as cfg:
        assert cfg == {"JACOBI_HW_WARPS": 6, "JACOBI_CHUNK": 5}
        assert _lib.get_config(_lib.NPBGB_CFG_JACOBI_CHUNK) == 5
    with autotune.applied("jacobi_2d", (64, 50), np.float64) as cfg:
        assert cfg is None
    assert (_lib.get_config(_lib.NPBGB_CFG_JACOBI_HW_WARPS),
            _lib.get_config(_lib.NPBGB_CFG_JACOBI_CHUNK)) == before


def test_batch_and_server_settings_by_class(cache):
    """The batch's tile rows and the server's split come from the class of the batch
    (grid count, median size, dtype mix) and of the stream; an unseen batch of the
    same class gets the tuned rows."""
    batch = [((100 + i, 200), np.float32 if i % 2 else np.float64) for i in range(300)]
    k = autotune.batch_key(batch)
    assert k == "batch/mixed/n8/m15"
    cache.write_text(json.dumps({
        k: {"config": {"rows": 64, "JACOBI_HW_WARPS": 6}},
        "serve/mixed": {"config": {"direct_cells": 262144, "ctas_per_sm": 2, "big_lanes": 1}}}))
    autotune.load_cache(refresh=True)
    autotune.enable()
    other = [((120, 150 + i), np.float64 if i % 3 else np.float32) for i in range(400)]
    assert autotune.batch_key(other) == k
    got = autotune.batch_settings(other)
    assert got == {"rows": 64, "JACOBI_HW_WARPS": 6}
    before = _lib.get_config(_lib.NPBGB_CFG_JACOBI_HW_WARPS)
    with autotune.batch_applied(got):
        assert _lib.get_config(_lib.NPBGB_CFG_JACOBI_HW_WARPS) == 6
    assert _lib.get_config(_lib.NPBGB_CFG_JACOBI_HW_WARPS) == before
    assert autotune.batch_settings([((10, 10), np.float32)])["rows"] == 128  # no entry: default
    assert autotune.server_settings() == {"direct_cells": 262144, "ctas_per_sm": 2,
                                          "big_lanes": 1}
    autotune.disable()
    assert autotune.server_settings()["direct_cells"] == 1 << 18


def test_shipped_table_is_consulted_after_the_user_cache(cache, monkeypatch, tmp_path):
    shipped = tmp_path / "shipped.json"
    shipped.write_text(json.dumps({"heat_3d/float64/c8x8x8": {"config": {"HEAT_CHUNK": 8}},
                                   "heat_3d/float32/c8x8x8": {"config": {"HEAT_TB": 2}}}))
    original = autotune.SHIPPED_PATH
    monkeypatch.setattr(autotune, "SHIPPED_PATH", str(shipped))
    cache.write_text(json.dumps({"heat_3d/float32/c8x8x8": {"config": {"HEAT_TB": 1}}}))
    autotune.load_cache(refresh=True)
    assert autotune.lookup("heat_3d/float64/c8x8x8")["config"] == {"HEAT_CHUNK": 8}
    assert autotune.lookup("heat_3d/float32/c8x8x8")["config"] == {"HEAT_TB": 1}
    monkeypatch.setattr(autotune, "SHIPPED_PATH", original)
    autotune.load_cache(refresh=True)


def test_shipped_table_names_known_knobs_with_accepted_values():
    """Every setting in the shipped table is a knob the library accepts (set and read back
    through the C ABI), a batch's tile rows, or one of the serving loop's parameters."""
    import json
    from npbench_gb300 import _lib
    with open(autotune.SHIPPED_PATH) as f:
        table = json.load(f)
    server_keys = set(autotune._SERVER_DEFAULT)
    for key, entry in table.items():
        cfg = entry["config"]
        if key.startswith("serve/"):
            assert set(cfg) <= server_keys, key
            continue
        for name, value in cfg.items():
            if key.startswith("batch/") and name == "rows":
                assert value > 0, key
                continue
            assert name in autotune._KNOBS, (key, name)
            old = _lib.get_config(autotune._KNOBS[name])
            try:
                _lib.set_config(autotune._KNOBS[name], value)  # raises for a refused value
                assert _lib.get_config(autotune._KNOBS[name]) == value, (key, name)
            finally:
                _lib.set_config(autotune._KNOBS[name], old)


def test_store_merges_entries(cache):
    autotune._store("a/float64/1x1", {"config": {}, "ms": 1.0})
    autotune._store("b/float64/2x2", {"config": {}, "ms": 2.0})
    data = json.loads(cache.read_text())
    assert set(data) == {"a/float64/1x1", "b/float64/2x2"}


@pytest.mark.gpu
def test_tune_then_tuned_call_is_bit_exact(cache):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from conftest import bits_equal
    from npbench_gb300 import stencils, workloads
    from oracle import cref
    space = [{"JACOBI_HW_WARPS": hw, "JACOBI_CHUNK": ch} for hw in (0, 4, 8) for ch in (0, 3)]
    entry = autotune.tune("jacobi_2d", (130, 300), np.float64, tsteps=5, space=space)
    assert entry["candidates"] == 6 and entry["ms"] <= entry["default_ms"]
    assert autotune.key("jacobi_2d", (130, 300), np.float64) in json.loads(cache.read_text())
    autotune.enable()
    A, B = workloads.uniform_pair((130, 300), np.float64, seed=5)
    dA = torch.from_numpy(A).cuda()
    dB = torch.from_numpy(B).cuda()
    stencils.jacobi_2d_kernel(9, dA, dB)
    cref.jacobi_2d_kernel(9, A, B)
    assert bits_equal(dA.cpu().numpy(), A) and bits_equal(dB.cpu().numpy(), B)
    heat = autotune.tune("heat_3d", (20, 30, 70), np.float32, tsteps=4,
                         space=[{"HEAT_ROWS": r, "HEAT_HW_ROWS": -1, "HEAT_CHUNK": c}
                                for r in (1, 4) for c in (0, 4)])
    assert heat["candidates"] == 4
