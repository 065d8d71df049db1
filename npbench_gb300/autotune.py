"""Tuning of libnpbgb's launch settings by shape class, with a JSON cache.

    python -m npbench_gb300.autotune --bench jacobi_2d --preset paper
    python -m npbench_gb300.autotune --bench heat_3d --shape 256 256 256 --dtype float32
    python -m npbench_gb300.autotune --batch          # the 4096-grid batch's tiles
    python -m npbench_gb300.autotune --server         # the serving loop's split
    python -m npbench_gb300.autotune --ship FILE      # all of the above into FILE

The kernels take knobs that change speed, never results (``NPBGB_CFG_*``): for
binary64 Jacobi-2D the warps per CTA on the hardware binary64 path, the
rows per CTA and whether the whole loop runs in one launch with bands of rows
in shared memory; for Heat-3D the tile rows per warp, the rows on hardware
binary64, the planes per CTA and, in binary32, the half-sweeps per launch
(temporal depth, 1 or 2).  Batches have their tile rows and hardware warps;
the server its split between the tile queue and the big-grid lanes.

Settings are keyed by **shape class**, not exact shape: a grid's class is the
integer part of log2 of each extent (256^3 and 300^3 share ``c8x8x8``), so a
setting tuned on one grid applies to every grid of its class.  A batch's class
is the log2 of its grid count and of its median grid size and its dtype mix;
the server has one class per stream description.

``tune(...)``, ``tune_batch(...)`` and ``tune_server(...)`` time every
candidate with CUDA events, check that each leaves exactly the bits of the
default (the knobs must not change results; a mismatch raises) and store the
fastest.  Lookups read the user cache (NPBGB_TUNE_CACHE, else
~/.cache/npbench_gb300/tune.json) and then ``tuned.json`` shipped in this
package, measured on GB300 by ``--ship``.  Tuned settings are applied by
default; NPBGB_AUTOTUNE=0 in the environment, or ``disable()``, turns that off.
"""
import argparse
import contextlib
import json
import math
import os
import threading
import time

import numpy as np

from . import _lib

__all__ = ["tune", "tune_batch", "tune_server", "enable", "disable", "enabled", "applied",
           "cache_path", "load_cache", "key", "shape_class", "lookup", "batch_key",
           "batch_settings", "batch_applied", "server_key", "server_settings", "SHIPPED_PATH"]

SHIPPED_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuned.json")

_lock = threading.RLock()
_state = {"enabled": os.environ.get("NPBGB_AUTOTUNE", "1") not in ("", "0"), "cache": None,
          "shipped": None}

# Knob name -> NPBGB_CFG_* key, and the candidates each benchmark sweeps.
_KNOBS = {
    "JACOBI_HW_WARPS": _lib.NPBGB_CFG_JACOBI_HW_WARPS,
    "JACOBI_CHUNK": _lib.NPBGB_CFG_JACOBI_CHUNK,
    "HEAT_ROWS": _lib.NPBGB_CFG_HEAT_ROWS,
    "HEAT_HW_ROWS": _lib.NPBGB_CFG_HEAT_HW_ROWS,
    "HEAT_CHUNK": _lib.NPBGB_CFG_HEAT_CHUNK,
    "HEAT_TB": _lib.NPBGB_CFG_HEAT_TB,
    "JACOBI_BANDS": _lib.NPBGB_CFG_JACOBI_BANDS,
    "JACOBI_TMA": _lib.NPBGB_CFG_JACOBI_TMA,
}


def _space(bench, dtype):
    """Candidate settings (dicts of knob -> value) for a benchmark and dtype."""
    f64 = np.dtype(dtype) == np.float64
    out = []
    if bench == "jacobi_2d":
        for hw in ((0, 2, 3, 4, 5, 6, 8) if f64 else (-1,)):
            for ch in (0, 3, 4, 6, 8, 16, 32):
                cfg = {"JACOBI_HW_WARPS": hw, "JACOBI_CHUNK": ch}
                if f64:
                    cfg["JACOBI_BANDS"] = 0  # chained launches
                out.append(cfg)
            if f64:  # the whole loop in one launch where the bands fit
                out.append({"JACOBI_HW_WARPS": hw, "JACOBI_CHUNK": 0, "JACOBI_BANDS": 2})
        if f64:  # each warp's TMA ring on grids below the size where it is automatic
            for hw in (2, 3, 4):
                for ch in (8, 16, 32):
                    out.append({"JACOBI_HW_WARPS": hw, "JACOBI_CHUNK": ch, "JACOBI_BANDS": 0,
                                "JACOBI_TMA": 2})
    elif bench == "heat_3d":
        for rows in (1, 2, 4):
            tj = 8 * rows
            for hw in (sorted({0, tj // 8, tj // 4, 5 * tj // 16, 3 * tj // 8, 7 * tj // 16})
                       if f64 else (-1,)):
                for ch in (0, 4, 5, 8, 16, 32):
                    for tb in ((1,) if f64 else (1, 2)):
                        cfg = {"HEAT_ROWS": rows, "HEAT_HW_ROWS": hw, "HEAT_CHUNK": ch}
                        if not f64:
                            cfg["HEAT_TB"] = tb
                        out.append(cfg)
    else:
        raise ValueError(f"no tunable knobs for {bench!r}")
    return out


def cache_path():
    p = os.environ.get("NPBGB_TUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "npbench_gb300", "tune.json")


def _dtype_name(dtype):
    name = str(dtype)
    if name.startswith("torch."):
        return name[len("torch."):]
    return np.dtype(dtype).name


def shape_class(shape):
    """Integer log2 of each extent: grids within a factor of two share a class."""
    return tuple(int(math.floor(math.log2(max(1, int(s))))) for s in shape)


def key(bench, shape, dtype):
    return f"{bench}/{_dtype_name(dtype)}/c{'x'.join(str(c) for c in shape_class(shape))}"


def _read_json(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def load_cache(refresh=False):
    with _lock:
        if _state["cache"] is None or refresh:
            _state["cache"] = _read_json(cache_path())
        if _state["shipped"] is None or refresh:
            _state["shipped"] = _read_json(SHIPPED_PATH)
        return _state["cache"]


def lookup(k):
    """The entry for key k: the user cache first, then the shipped table."""
    cache = load_cache()
    return cache.get(k) or _state["shipped"].get(k)


def _store(k, entry, path=None):
    with _lock:
        path = path or cache_path()
        cache = _read_json(path)
        cache[k] = entry
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(cache, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
        if path == cache_path():
            _state["cache"] = cache


def enable():
    _state["enabled"] = True


def disable():
    _state["enabled"] = False


def enabled():
    return _state["enabled"]


@contextlib.contextmanager
def _settings(config):
    config = {k: v for k, v in config.items() if k in _KNOBS}
    old = {name: _lib.set_config(_KNOBS[name], value) for name, value in config.items()}
    try:
        yield
    finally:
        for name, value in old.items():
            _lib.set_config(_KNOBS[name], value)


@contextlib.contextmanager
def applied(bench, shape, dtype):
    """The tuned setting of this call's shape class, if tuning is enabled and one exists."""
    entry = lookup(key(bench, shape, dtype)) if _state["enabled"] else None
    if not entry:
        yield None
        return
    with _lock, _settings(entry["config"]):
        yield entry["config"]


def _defaults(bench, dtype=np.float64):
    f64 = np.dtype(dtype) == np.float64
    if bench == "jacobi_2d":
        names = ("JACOBI_HW_WARPS", "JACOBI_CHUNK") + (("JACOBI_BANDS",) if f64 else ())
    else:
        names = ("HEAT_ROWS", "HEAT_HW_ROWS", "HEAT_CHUNK") + (() if f64 else ("HEAT_TB",))
    return {n: _lib.get_config(_KNOBS[n]) for n in names}


def _events_ms(fn, sync_dev, repeats):
    import torch
    ts = []
    for _ in range(repeats):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize(sync_dev)
        ts.append(e0.elapsed_time(e1))
    return float(np.median(ts))


def tune(bench, shape, dtype, tsteps=None, repeats=3, space=None, store=True, path=None):
    """Times every candidate setting for (bench, shape, dtype); returns the cache entry
    (stored under the shape's class).

    Each candidate must leave exactly the bits the default setting leaves (else
    RuntimeError).  tsteps defaults to 21 (40 half-sweeps).
    """
    import torch

    from . import stencils, workloads
    if not torch.cuda.is_available():
        raise RuntimeError("autotune needs a CUDA device")
    dev = torch.device("cuda", torch.cuda.current_device())
    shape = tuple(int(s) for s in shape)
    dtype = np.dtype(_dtype_name(dtype))
    kern = {"jacobi_2d": stencils.jacobi_2d_kernel, "heat_3d": stencils.heat_3d_kernel}[bench]
    if bench == "jacobi_2d":
        A0, B0 = workloads.uniform_pair(shape, dtype.type, seed=1)
    else:
        A0, B0 = workloads.uniform_heat(shape, dtype.type, seed=1)
    T = int(tsteps) if tsteps else 21
    pA, pB = torch.from_numpy(A0).to(dev), torch.from_numpy(B0).to(dev)
    A, B = torch.empty_like(pA), torch.empty_like(pB)
    was_enabled = _state["enabled"]
    _state["enabled"] = False  # the kernels must see exactly the settings below

    def run():
        A.copy_(pA)
        B.copy_(pB)
        kern(T, A, B)

    def timed():
        run()
        torch.cuda.synchronize(dev)

        def once():
            kern(T, A, B)
        ms = []
        for _ in range(repeats):
            A.copy_(pA)
            B.copy_(pB)
            ms.append(_events_ms(once, dev, 1))
        return float(np.median(ms))

    try:
        base_cfg = _defaults(bench, dtype)
        run()
        ref = (A.clone(), B.clone())
        base_ms = timed()
        results = []
        for cfg in (space or _space(bench, dtype)):
            with _settings(cfg):
                run()
                if not (torch.equal(A.view(torch.int8), ref[0].view(torch.int8)) and
                        torch.equal(B.view(torch.int8), ref[1].view(torch.int8))):
                    raise RuntimeError(f"setting {cfg} changed the results of {bench}")
                results.append((timed(), cfg))
        best_ms, best = min(results, key=lambda r: r[0])
        if best_ms >= base_ms:
            best_ms, best = base_ms, base_cfg
        entry = {"config": best, "ms": best_ms, "default_ms": base_ms, "tsteps": T,
                 "tuned_on": list(shape), "gpu": torch.cuda.get_device_name(dev),
                 "library": _lib.version(), "candidates": len(results)}
        if store:
            _store(key(bench, shape, dtype), entry, path)
        return entry
    finally:
        _state["enabled"] = was_enabled


# ---------------------------------------------------------------------------
# Batches
# ---------------------------------------------------------------------------
def batch_key(shapes_dtypes):
    """Class of a batch: log2 of its grid count and of its median grid size, and
    whether it holds float32, float64 or both."""
    n = len(shapes_dtypes)
    cells = sorted(int(np.prod(s)) for s, _ in shapes_dtypes) or [1]
    kinds = {np.dtype(d).name for _, d in shapes_dtypes}
    mix = "mixed" if len(kinds) > 1 else (kinds.pop() if kinds else "none")
    return (f"batch/{mix}/n{int(math.log2(max(1, n)))}"
            f"/m{int(math.log2(max(1, cells[len(cells) // 2])))}")


_BATCH_DEFAULT = {"rows": 128, "JACOBI_HW_WARPS": -1}


def batch_settings(shapes_dtypes):
    """{"rows": tile rows, "JACOBI_HW_WARPS": ...} for a batch of (shape, dtype)."""
    entry = lookup(batch_key(shapes_dtypes)) if _state["enabled"] else None
    return dict(entry["config"]) if entry else dict(_BATCH_DEFAULT)


@contextlib.contextmanager
def batch_applied(settings):
    """The knobs of batch_settings() in force (tile rows are passed to the batch)."""
    with _lock, _settings({k: v for k, v in settings.items() if k != "rows"}):
        yield settings


def tune_batch(n_grids=512, seed=0, rows=(32, 64, 128, 256), hw_warps=(-1, 2, 3, 6), repeats=2,
               store=True, path=None, guard=True, full_grids=4096):
    """Tunes the stepped batch's tile rows and binary64 hardware warps on the first
    n_grids of the batched configuration (its distribution: sides log-uniform in
    [64, 2048], float32/float64, TSTEPS in [10, 500]); stores the result under the
    class of the full batch."""
    import torch

    from . import workloads
    from .batch import Batch
    dev = torch.device("cuda", torch.cuda.current_device())
    full = workloads.batch_jacobi_specs(full_grids, seed=seed)
    specs = full[:n_grids]
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    init, work = [], []
    for (ny, nx), dt, T in specs:
        tdt = torch.float64 if dt == np.float64 else torch.float32
        a = torch.rand((ny, nx), dtype=tdt, device=dev, generator=gen)
        b = torch.rand((ny, nx), dtype=tdt, device=dev, generator=gen)
        init.append((a, b))
        work.append((a.clone(), b.clone(), T))

    def reset():
        for (a0, b0), (a, b, _) in zip(init, work):
            a.copy_(a0)
            b.copy_(b0)
    was = _state["enabled"]
    _state["enabled"] = False
    results, ref = [], None
    try:
        for r in rows:
            for hw in hw_warps:
                cfg = {"rows": r, "JACOBI_HW_WARPS": hw}
                with batch_applied(cfg), Batch(work, band_rows=r, mode="stepped",
                                               guard=guard) as bt:
                    reset()
                    bt.launch(graph=True)
                    torch.cuda.synchronize(dev)
                    out = [a.clone() for a, _, _ in work]
                    if ref is None:
                        ref = out
                    elif not all(torch.equal(x, y) for x, y in zip(out, ref)):
                        raise RuntimeError(f"batch setting {cfg} changed the results")
                    ms = []
                    for _ in range(repeats):
                        reset()
                        ms.append(_events_ms(lambda: bt.launch(graph=True), dev, 1))
                    results.append((float(np.median(ms)), cfg))
    finally:
        _state["enabled"] = was
    best_ms, best = min(results, key=lambda x: x[0])
    default_ms = next((m for m, c in results if c == _BATCH_DEFAULT), None)
    entry = {"config": best, "ms": best_ms, "default_ms": default_ms,
             "tuned_on": f"first {n_grids} grids of the {full_grids}-grid batch",
             "candidates": len(results), "gpu": torch.cuda.get_device_name(dev),
             "library": _lib.version()}
    if store:
        _store(batch_key([(s, d) for s, d, _ in full]), entry, path)
    return entry


# ---------------------------------------------------------------------------
# The server
# ---------------------------------------------------------------------------
_SERVER_DEFAULT = {"direct_cells": 1 << 18, "ctas_per_sm": 1, "big_lanes": 3, "lane_order": "fifo"}


def server_key(stream="mixed"):
    return f"serve/{stream}"


def server_settings(stream="mixed"):
    """{"direct_cells", "ctas_per_sm", "big_lanes", "lane_order"} for the serving loop."""
    entry = lookup(server_key(stream)) if _state["enabled"] else None
    return dict(entry["config"]) if entry else dict(_SERVER_DEFAULT)


def tune_server(n_requests=100, rates=(200.0, 1000.0), direct_cells=(1 << 16, 1 << 18),
                ctas_per_sm=(1,), big_lanes=(2, 3, 4), lane_order=("sjf", "fifo", "aged"),
                store=True, path=None):
    """Serves the mixed stream (workloads.served_requests) at each rate once per
    candidate split, next to the same requests run one at a time with per-grid
    launches (``server.run_sequential``).  Keeps the candidate with the highest
    throughput at its worst rate among those whose p50 and p99 are no worse than
    sequential at every rate (if none is, the highest throughput alone)."""
    import torch

    from . import workloads
    from .server import Request, StencilServer, latency_stats, run_sequential
    _, specs = workloads.served_requests(n_requests, rates[0], seed=0)
    host = []
    for s, dt, T, sd in specs:
        rng = np.random.default_rng(sd)
        tdt = torch.float32 if dt == np.float32 else torch.float64
        a = torch.empty(s, dtype=tdt, pin_memory=True).numpy()
        rng.random(s, dtype=dt, out=a)
        b = None
        if len(s) == 2:
            b = torch.empty(s, dtype=tdt, pin_memory=True).numpy()
            rng.random(s, dtype=dt, out=b)
        host.append((a, b))

    def make():
        return [Request(shape=s, dtype=dt, tsteps=T, a=h[0], b=h[1], return_host=False)
                for (s, dt, T, _), h in zip(specs, host)]

    def serve(rate, cand):
        arrivals, _ = workloads.served_requests(n_requests, rate, seed=0)
        reqs = make()
        srv = StencilServer(**cand).start()
        t0 = time.perf_counter()
        futs = []
        for r, at in zip(reqs, arrivals):
            now = time.perf_counter() - t0
            if at > now:
                time.sleep(at - now)
            futs.append(srv.submit(r))
        for f in futs:
            f.result()
        srv.stop()
        st = latency_stats(reqs)
        del reqs, futs
        torch.cuda.empty_cache()
        return {k: st[k] for k in ("updates_per_s", "p50_ms", "p99_ms")}

    seq = {}
    for rate in rates:
        arrivals, _ = workloads.served_requests(n_requests, rate, seed=0)
        q = make()
        run_sequential(q, arrivals)
        st = latency_stats(q)
        seq[rate] = {k: st[k] for k in ("updates_per_s", "p50_ms", "p99_ms")}
        del q
        torch.cuda.empty_cache()
    cands = [{"direct_cells": dc, "ctas_per_sm": cps, "big_lanes": lanes, "lane_order": order}
             for dc in direct_cells for cps in ctas_per_sm for lanes in big_lanes
             for order in lane_order]
    results = []
    for cand in cands:
        per = {rate: serve(rate, cand) for rate in rates}
        worst = min(per[r]["updates_per_s"] / seq[r]["updates_per_s"] for r in rates)
        no_worse = all(per[r]["p50_ms"] <= seq[r]["p50_ms"] and per[r]["p99_ms"] <= seq[r]["p99_ms"]
                       for r in rates)
        results.append({"config": cand, "worst_ratio": worst, "latency_no_worse": no_worse,
                        "rates": {str(r): per[r] for r in rates}})
    pool = [r for r in results if r["latency_no_worse"]] or results
    best = max(pool, key=lambda r: r["worst_ratio"])
    entry = {"config": best["config"], "worst_ratio_over_sequential": best["worst_ratio"],
             "latency_no_worse_than_sequential": best["latency_no_worse"],
             "tuned_on": f"{n_requests} requests of the mixed stream at "
                         f"{', '.join(f'{r:g}' for r in rates)} req/s",
             "sequential": {str(r): seq[r] for r in rates}, "candidates": results,
             "gpu": torch.cuda.get_device_name(torch.cuda.current_device()),
             "library": _lib.version()}
    if store:
        _store(server_key(), entry, path)
    return entry


def main(argv=None):
    from . import workloads
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawTextHelpFormatter)
    ap.add_argument("--bench", choices=["jacobi_2d", "heat_3d"])
    ap.add_argument("--preset", choices=["S", "M", "L", "paper"])
    ap.add_argument("--shape", type=int, nargs="+")
    ap.add_argument("--dtype", default="float64", choices=["float64", "float32"])
    ap.add_argument("--batch", action="store_true")
    ap.add_argument("--server", action="store_true")
    ap.add_argument("--ship", metavar="FILE", help="tune the benchmark classes into FILE")
    ap.add_argument("--out", metavar="FILE",
                    help="store a --bench/--batch/--server result in FILE, not the user cache")
    a = ap.parse_args(argv)
    if a.ship:
        grids = [("heat_3d", (256,) * 3, "float64"), ("heat_3d", (256,) * 3, "float32"),
                 ("heat_3d", (512,) * 3, "float32"), ("heat_3d", (120,) * 3, "float64"),
                 ("jacobi_2d", (1000, 1000), "float64"), ("jacobi_2d", (2800, 2800), "float64"),
                 ("jacobi_2d", (2800, 2800), "float32"), ("jacobi_2d", (4096, 4096), "float64")]
        for bench, shape, dt in grids:
            e = tune(bench, shape, dt, path=a.ship)
            print(json.dumps({key(bench, shape, dt): e}), flush=True)
        print(json.dumps({"batch": tune_batch(path=a.ship)}), flush=True)
        print(json.dumps({"server": tune_server(path=a.ship)}), flush=True)
        return
    if a.batch:
        print(json.dumps(tune_batch(path=a.out)))
        return
    if a.server:
        print(json.dumps(tune_server(path=a.out)))
        return
    if not a.bench:
        ap.error("give --bench, --batch, --server or --ship")
    if a.shape:
        shape = tuple(a.shape)
    elif a.preset:
        n = workloads.PRESETS[a.bench][a.preset]["N"]
        shape = (n, n) if a.bench == "jacobi_2d" else (n, n, n)
    else:
        ap.error("give --preset or --shape")
    entry = tune(a.bench, shape, a.dtype, path=a.out)
    print(json.dumps({key(a.bench, shape, a.dtype): entry}))


if __name__ == "__main__":
    main()
