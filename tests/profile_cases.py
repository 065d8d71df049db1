"""Small single-kernel cases for ncu captures (the recipe behind the profile summaries).

    python tests/profile_cases.py <case>

Each case runs one kernel family on an input still larger than L2 where the
real workload is, with few launches, so that one capture
(``ncu --set full --clock-control none -k regex:<kernel> -s <n> -c 1``) ends in
seconds.  Run the case once without ncu first; capture it only after that run
exited 0:

========== ============================================== ===================
case       what                                           kernel to capture
========== ============================================== ===================
heat_f64   Heat-3D 256^3 float64, TSTEPS=3 (4 launches)   heat3d_tma, -s 2
heat_f32   Heat-3D 256^3 float32, TSTEPS=3                heat3d_tma, -s 2
jacobi_f64 Jacobi-2D 4096^2 float64, TSTEPS=3             jacobi2d_strip, -s 2
jacobi_f32 Jacobi-2D 4096^2 float32, TSTEPS=3             jacobi2d_strip, -s 2
hdiff      hdiff 256x256x160 float64, 3 calls             hdiff_tile, -s 1
vadv       vadv 256x256x160 float64, 3 calls              vadv_columns, -s 1
cavity     cavity_flow 101x101, nt=20, nit=50, 2 calls    cavity_bands, -s 1
batch      256 mixed Jacobi-2D grids, 2 launches          batch_persistent, -s 1
batch_step 256 mixed grids, stepped form, one pass        batch_step, -s 20
jacobi_f64_1000  Jacobi-2D 1000^2 float64, TSTEPS=3       jacobi2d_strip, -s 2
jacobi1d   Jacobi-1D N=32000 float64, TSTEPS=64           jacobi1d_block, -s 2
fdtd       FDTD-2D 1000x1200 float64, TMAX=3 (6 launches) fdtd_e / fdtd_h, -s 1
heat_f32_tb Heat-3D 416^3 float32, TSTEPS=6: 4 two-step   heat3d_tb2, -s 1
           launches, then one single-step pair
heat_f32_384 Heat-3D 384^3 float32, TSTEPS=3, one step    heat3d_tma, -s 2
           per launch
heat_f32_512 Heat-3D 512^3 float32, TSTEPS=3 (automatic   heat3d_tma, -s 2
           5-plane chunks)
heat_f32_chunks  timing sweep (CUDA events, no ncu) of    -
           the binary32 Heat-3D plane chunks and forms,
           256^3 to 640^3, TSTEPS=21; one JSON line per size
jacobi_bands_1000  Jacobi-2D 1000^2 float64, TSTEPS=10,   jacobi2d_bands, -c 1
           one launch with the bands in shared memory
jacobi_f64_fx  Jacobi-2D 4096^2 float64, TSTEPS=3, every  jacobi2d_strip, -s 2
           warp in fixed point
jacobi_f64_hw  the same, every warp on hardware binary64  jacobi2d_strip, -s 2
batch1024  the first 1024 grids of the 4096-grid batch,   batch_step, -s 100
           stepped form, TSTEPS as drawn, tuned tile rows,
           float64 guard (about 5 GB)
queue_mix  240 small mixed grids through the tile queue   queue_worker, -c 1
pipes      the seven pipe-rate probes                     pipe_probe, -c 7
========== ============================================== ===================
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _heat_f32_chunks(dev, sizes=(256, 384, 416, 512, 640), T=21):
    """Median CUDA-event time of kernel(T, A, B) per binary32 Heat-3D setting, its
    fraction of the measured copy bandwidth at 8 bytes per update, and the library's
    kernel launches for one call."""
    import json

    import torch

    from npbench_gb300 import _lib, autotune, stencils, workloads
    autotune.disable()
    peak = 6687.5
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak = float(json.load(f)["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        pass
    keys = {k: getattr(_lib, "NPBGB_CFG_" + k) for k in ("HEAT_TB", "HEAT_TB_CHUNK", "HEAT_CHUNK")}
    settings = ([("auto", {})] + [(f"chunk {c}", {"HEAT_TB": 1, "HEAT_CHUNK": c})
                                  for c in (4, 5, 6, 8, 16, 32, 64, 128)] +
                [(f"two-step chunk {c}", {"HEAT_TB": 2, "HEAT_TB_CHUNK": c}) for c in (8, 16, 32)])
    st = torch.cuda.current_stream(dev)
    for n in sizes:
        A0, _ = workloads.uniform_heat((n,) * 3, np.float32, seed=1)
        pa = torch.from_numpy(A0).to(dev)
        del A0
        a, b = torch.empty_like(pa), torch.empty_like(pa)
        row = {}
        for name, cfg in settings:
            old = {k: _lib.set_config(keys[k], v) for k, v in cfg.items()}
            ts = []
            for rep in range(5):
                a.copy_(pa)
                b.copy_(pa)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                n_launch = _lib.launches()
                e0.record(st)
                stencils.heat_3d_kernel(T, a, b)
                e1.record(st)
                e1.synchronize()
                n_launch = _lib.launches() - n_launch
                if rep >= 2:
                    ts.append(e0.elapsed_time(e1))
            for k, v in old.items():
                _lib.set_config(keys[k], v)
            ms = float(np.median(ts))
            frac = 2 * (T - 1) * (n - 2) ** 3 * 8 / (ms * 1e-3) / 1e9 / peak
            row[name] = [round(ms, 3), round(frac, 3), n_launch]
        print(json.dumps({"n": n, "TSTEPS": T, "peak_gbs": peak, "ms_and_frac": row}), flush=True)
        del pa, a, b
        torch.cuda.empty_cache()


def run(case):
    import torch

    from npbench_gb300 import _lib, stencils, workloads
    dev = torch.device("cuda", 0)
    if case in ("heat_f64", "heat_f32"):
        dt = np.float64 if case.endswith("64") else np.float32
        A, B = workloads.uniform_heat((256,) * 3, dt, seed=0)
        a, b = torch.from_numpy(A).to(dev), torch.from_numpy(B).to(dev)
        stencils.heat_3d_kernel(3, a, b)
    elif case in ("jacobi_f64", "jacobi_f32"):
        dt = np.float64 if case.endswith("64") else np.float32
        A, B = workloads.uniform_pair((4096, 4096), dt, seed=0)
        a, b = torch.from_numpy(A).to(dev), torch.from_numpy(B).to(dev)
        stencils.jacobi_2d_kernel(3, a, b)
    elif case == "hdiff":
        inf, out, co = workloads.init_hdiff(256, 256, 160)
        x, y, z = (torch.from_numpy(t).to(dev) for t in (inf, out, co))
        for _ in range(3):
            stencils.hdiff(x, y, z)
    elif case == "vadv":
        dtr, us, u, w, up, ut = workloads.init_vadv(256, 256, 160)
        a, b, c, d, e = (torch.from_numpy(t).to(dev) for t in (us, u, w, up, ut))
        for _ in range(3):
            stencils.vadv(a, b, c, d, e, dtr)
    elif case == "cavity":
        u, v, p, dx, dy, dt = workloads.init_cavity_flow(101, 101)
        a, b, c = (torch.from_numpy(t).to(dev) for t in (u, v, p))
        for _ in range(2):
            stencils.cavity_flow(101, 101, 20, 50, a, b, dt, dx, dy, c, 1.0, 0.1)
    elif case == "jacobi_f64_1000":
        A, B = workloads.uniform_pair((1000, 1000), np.float64, seed=11)
        a, b = torch.from_numpy(A).to(dev), torch.from_numpy(B).to(dev)
        stencils.jacobi_2d_kernel(3, a, b)
    elif case == "jacobi1d":
        A, B = workloads.init_jacobi_1d(32000, np.float64)
        a, b = torch.from_numpy(A).to(dev), torch.from_numpy(B).to(dev)
        stencils.jacobi_1d_kernel(64, a, b)
    elif case == "fdtd":
        fields = workloads.init_fdtd_2d(3, 1000, 1200)
        ex, ey, hz, fict = (torch.from_numpy(t).to(dev) for t in fields)
        stencils.fdtd_2d_kernel(3, ex, ey, hz, fict)
    elif case == "batch_step":
        from npbench_gb300.batch import Batch
        specs = workloads.batch_jacobi_specs(256, seed=0, tsteps=(10, 40))
        g = torch.Generator(device=dev)
        g.manual_seed(0)
        work = []
        for (ny, nx), dtp, T in specs:
            tdt = torch.float64 if dtp == np.float64 else torch.float32
            work.append((torch.rand((ny, nx), dtype=tdt, device=dev, generator=g),
                         torch.rand((ny, nx), dtype=tdt, device=dev, generator=g), T))
        with Batch(work, mode="stepped") as bt:
            bt.launch()
    elif case == "batch":
        from npbench_gb300.batch import Batch
        specs = workloads.batch_jacobi_specs(256, seed=0, tsteps=(10, 40))
        g = torch.Generator(device=dev)
        g.manual_seed(0)
        work = []
        for (ny, nx), dtp, T in specs:
            tdt = torch.float64 if dtp == np.float64 else torch.float32
            work.append((torch.rand((ny, nx), dtype=tdt, device=dev, generator=g),
                         torch.rand((ny, nx), dtype=tdt, device=dev, generator=g), T))
        with Batch(work, band_rows=64) as bt:
            bt.launch()
            bt.launch()
    elif case in ("heat_f32_tb", "heat_f32_384"):
        n, T = (416, 6) if case == "heat_f32_tb" else (384, 3)
        A, B = workloads.uniform_heat((n,) * 3, np.float32, seed=0)
        a, b = torch.from_numpy(A).to(dev), torch.from_numpy(B).to(dev)
        stencils.heat_3d_kernel(T, a, b)
    elif case == "heat_f32_512":
        A, B = workloads.uniform_heat((512,) * 3, np.float32, seed=0)
        a, b = torch.from_numpy(A).to(dev), torch.from_numpy(B).to(dev)
        stencils.heat_3d_kernel(3, a, b)
    elif case == "heat_f32_chunks":
        _heat_f32_chunks(dev)
    elif case in ("jacobi_f64_fx", "jacobi_f64_hw"):
        from npbench_gb300 import autotune
        autotune.disable()
        _lib.set_config(_lib.NPBGB_CFG_JACOBI_HW_WARPS, 0 if case.endswith("fx") else 8)
        A, B = workloads.uniform_pair((4096, 4096), np.float64, seed=0)
        a, b = torch.from_numpy(A).to(dev), torch.from_numpy(B).to(dev)
        stencils.jacobi_2d_kernel(3, a, b)
    elif case == "jacobi_bands_1000":
        from npbench_gb300 import autotune
        autotune.disable()
        _lib.set_config(_lib.NPBGB_CFG_JACOBI_BANDS, 2)
        A, B = workloads.uniform_pair((1000, 1000), np.float64, seed=0)
        a, b = torch.from_numpy(A).to(dev), torch.from_numpy(B).to(dev)
        stencils.jacobi_2d_kernel(10, a, b)
    elif case == "batch1024":
        from npbench_gb300.batch import Batch
        specs = workloads.batch_jacobi_specs(4096, seed=0)[:1024]
        g = torch.Generator(device=dev)
        g.manual_seed(0)
        work = []
        for (ny, nx), dtp, T in specs:
            tdt = torch.float64 if dtp == np.float64 else torch.float32
            work.append((torch.rand((ny, nx), dtype=tdt, device=dev, generator=g),
                         torch.rand((ny, nx), dtype=tdt, device=dev, generator=g), T))
        # the batched configuration's settings: its tuned tile rows and knobs, the float64 guard
        from npbench_gb300 import autotune
        tuned = autotune.batch_settings([(s_, dt_) for s_, dt_, _ in workloads.batch_jacobi_specs(4096, seed=0)])
        with autotune.batch_applied(tuned), Batch(work, band_rows=tuned.get("rows", 64), mode="stepped",
                                                  guard=True) as bt:
            bt.launch()
    elif case == "queue_mix":
        from npbench_gb300.queue import TileQueue
        rng = np.random.default_rng(0)
        grids = []
        for n in range(240):
            dtp = torch.float32 if n % 3 else torch.float64
            if n % 2:
                shape = tuple(int(x) for x in rng.integers(64, 700, 2))
            else:
                shape = tuple(int(x) for x in rng.integers(16, 90, 3))
            a = torch.rand(shape, dtype=dtp, device=dev)
            grids.append((a, a.clone(), int(rng.integers(20, 200))))
        with TileQueue(max_slots=256, ctas_per_sm=1) as q:
            pending = {q.submit(a, b, T) for a, b, T in grids} - {-1}
            while pending:
                q.kick()
                pending -= set(q.poll())
    elif case == "pipes":
        from npbench_gb300 import pipes
        pipes.measure(target_ms=1.0, repeats=0)
    else:
        raise SystemExit(f"unknown case {case!r}")
    torch.cuda.synchronize()
    _lib.device_status()
    print("ok", case)


if __name__ == "__main__":
    run(sys.argv[1])
