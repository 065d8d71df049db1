"""Benchmark of the structured-grid stencil path on GB300: lattice updates/s and HBM roofline.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Workload (one "step"): Heat-3D, 256^3 grid, TSTEPS=100 (198 half-sweeps of
254^3 interior updates), seeded U[0,1) input (B = copy of A), float64 -- the
3D 7-point heat configuration.  Each timed step starts from the same seeded
field (restored on the device between steps, outside the timed interval).
The two 128 MiB arrays exceed the 129 MB L2, so no L2 flush is needed.

* ``value``     updates/s over the K timed steps, inputs resident in HBM;
* ``e2e``       the same through the public kernel call with host buffers:
                pinned host -> device copies of A and B, the kernel, and device
                -> host copies of A and B, all inside the timed interval;
* ``roofline``  algorithmic bytes (16 B per float64 update: read one value,
                write one) of one half-sweep launch over its measured duration;
* ``fp64_roofline`` the reference's 13 binary64 operations per update at the
                achieved rate against the binary64 pipe's rate, measured in the
                same run by a probe kernel (npbench_gb300.pipes);
* ``compute_roofline`` the kernel's instructions per update on each pipe (ncu)
                against each pipe's measured rate: the arithmetic ceiling;
* ``fp32``      the same workload in float32 with its error against float64;
* ``cpu_baseline`` the reference's arithmetic on the host: the C restatement
                (oracle/stencils.c, bit-identical to the reference's NumPy code)
                with OpenMP on all host threads, the whole workload 10 times;
                ``numpy_1core`` beside it times the NumPy restatement on one core
                (NumPy's elementwise ufuncs are single-threaded).

* ``batch``     configuration 4 (4096 mixed Jacobi-2D grids, float32 and
                float64, in one batch per step), with plain per-grid launches of
                the same grids beside it and the float32 grids' error against
                float64 runs; its own step counts are stated in the block;
* ``serve``     configuration 5 (100 Poisson-arrival mixed solves through the
                serving loop at 200, 1000 and 5000 req/s) with p50/p99 latency,
                the same requests run one at a time with per-grid launches beside
                it, and the float32 requests' error against float64.

``--impl reference`` times only that CPU implementation (the C restatement on
all host threads, one whole workload per step) and prints its line with
``"impl": "reference"``.

With N > 1 (torchrun), every rank runs an independent replica on its own GPU
(the path has no exchange between independent grids): ``value`` is the total
updates of all ranks over the slowest rank's time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "lattice_updates_per_s"
UNIT = "updates/s"
N_GRID = 256
TSTEPS = 100
HALF_SWEEPS = 2 * (TSTEPS - 1)
INTERIOR = (N_GRID - 2) ** 3
UPDATES_PER_STEP = HALF_SWEEPS * INTERIOR
FALLBACK_HBM_GBS = 6800.0
# Separately rounded binary64 operations per Heat-3D update as the reference
# writes it: 2*c once, then per axis a subtraction, an addition and the product
# by 0.125, and three additions joining the axes.
HEAT_FP64_OPS = 13


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp32", action="store_true")
    ap.add_argument("--no-batch", action="store_true",
                    help="default workload: leave out the batched block (configuration 4)")
    ap.add_argument("--no-serve", action="store_true",
                    help="default workload: leave out the served-stream block (configuration 5)")
    ap.add_argument("--workload", default="heat3d",
                    choices=["heat3d", "jacobi2d", "hdiff", "batch", "serve", "jacobi1d", "fdtd2d",
                             "vadv", "cavity", "channel"],
                    help="heat3d (default): Heat-3D 256^3; jacobi2d: Jacobi-2D 1000^2 float64, "
                         "TSTEPS=100; hdiff: 256x256x160 float64, one call per step; batch: "
                         "4096 mixed Jacobi-2D grids in one persistent launch; serve: "
                         "Poisson-arrival mixed solves through the continuous-batching server; "
                         "jacobi1d / fdtd2d / vadv / cavity / channel: NPBench paper presets")
    ap.add_argument("--batch-grids", type=int, default=4096)
    ap.add_argument("--compare", action="store_true",
                    help="batch/serve: also time the per-grid / sequential comparator")
    ap.add_argument("--requests", type=int, default=200)
    ap.add_argument("--rate", type=float, default=1000.0)
    ap.add_argument("--stream", choices=["mixed", "small"], default="mixed",
                    help="serve workload: the mixed stream of configuration 5, or grids "
                         "small enough for the tile queue")
    return ap.parse_args()


def dist_info():
    from npbench_gb300 import replicas
    return replicas.dist_info()


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def _ncu_record(kernel_key):
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as f:
            return json.load(f).get(kernel_key, {})
    except Exception:
        return {}


def ncu_traffic(kernel_key):
    """DRAM bytes per launch recorded from an ncu capture (profiles/ncu_traffic.json)."""
    return _ncu_record(kernel_key).get("dram_bytes_per_launch")


# Which probe measures each pipe's throughput (npbench_gb300.pipes): the integer
# ALU pipe retires LOP3, the binary64 pipe DADD/DMUL/DFMA; the stencils' FMA-pipe
# instructions are integer multiply-adds on its heavy half, whose rate IMAD measures.
PIPE_PROBES = {"alu": "lop3", "fp64": "dadd", "fma": "imad"}


def compute_roofline(kernel_key, achieved_ups, rates):
    """The arithmetic roof of a binary64 kernel: thread instructions per lattice
    update on each pipe (ncu's sm__inst_executed_pipe_*.sum of one launch x 32 /
    updates per launch, profiles/ncu_traffic.json) against each pipe's throughput
    measured in this run (pipe probes), and the issue rate of one instruction
    per scheduler per clock.  The ceiling is the update rate at which the
    busiest pipe (or issue) saturates."""
    rec = _ncu_record(kernel_key).get("inst_per_update")
    if not rec or not rates:
        return None
    limits = {}
    for pipe, probe in PIPE_PROBES.items():
        n = rec.get(pipe, 0.0)
        if n > 0 and rates.get(probe):
            limits[pipe] = rates[probe] / n
    if rec.get("issue") and rates.get("issue_slots"):
        limits["issue"] = rates["issue_slots"] / rec["issue"]
    if not limits:
        return None
    bound = min(limits, key=limits.get)
    return {"bound": bound, "ceiling_updates_per_s": limits[bound], "achieved": achieved_ups,
            "frac": achieved_ups / limits[bound], "unit": "updates/s",
            "per_pipe_ceiling_updates_per_s": limits, "inst_per_update": rec,
            "pipe_rates_ops_per_s": {k: rates.get(v) for k, v in PIPE_PROBES.items()},
            "source": _ncu_record(kernel_key).get("inst_source")}


def measure_pipes():
    """Live pipe throughputs on this GPU (a fraction of a second), plus issue slots."""
    import torch
    from npbench_gb300 import pipes
    rates = pipes.measure(target_ms=3.0, repeats=2)
    props = torch.cuda.get_device_properties(0)
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            clk = float(json.load(f)["sm_max_mhz"]) * 1e6
    except Exception:
        clk = 2.07e9  # GB300's maximum SM clock
    # one warp instruction per scheduler (4 per SM) per clock = 128 thread instructions
    rates["issue_slots"] = props.multi_processor_count * 4 * 32 * clk
    return rates


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.15)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


def cpu_numpy_sample(dtype=np.float64, half_sweeps=2, seed=0):
    """Times the NumPy restatement of the reference kernel on a bounded sample."""
    from npbench_gb300 import workloads
    from oracle import stencils_np
    A, B = workloads.uniform_heat((N_GRID,) * 3, dtype, seed=seed)
    t0 = time.perf_counter()
    for h in range(half_sweeps):
        if h % 2 == 0:
            stencils_np.heat_3d_half_sweep(A, B)
        else:
            stencils_np.heat_3d_half_sweep(B, A)
    dt = time.perf_counter() - t0
    return half_sweeps * INTERIOR / dt, dt


def host_threads():
    """Threads the OpenMP loops of the C restatement use (OMP_NUM_THREADS, else all cores)."""
    try:
        return max(1, int(os.environ.get("OMP_NUM_THREADS", "")))
    except ValueError:
        return os.cpu_count() or 1


def cpu_port(setup, run, units, what, parallel=True, reps=3, numpy=None):
    """Times the C restatement of the reference's arithmetic (oracle/stencils.c,
    bit-identical to the reference's NumPy code) on the host cores.

    setup() returns fresh arguments (untimed), run(*args) is timed; the median
    of ``reps`` runs gives ``units / s``.  ``parallel``: the C loops use OpenMP
    on all host threads (False for the kernels whose C form is sequential).
    ``numpy``: optional (setup, run, units, what) timed once with the NumPy
    restatement, one core, reported beside it as ``numpy_1core``.
    """
    run(*setup())  # warm-up: builds the library and starts the thread pool
    dts = []
    for _ in range(reps):
        a = setup()
        t0 = time.perf_counter()
        run(*a)
        dts.append(time.perf_counter() - t0)
    dt = statistics.median(dts)
    cores = host_threads() if parallel else 1
    out = {"value": units / dt, "unit": UNIT, "cores": cores, "kind": "port",
           "sample": f"{what}: C restatement of the reference (OpenMP, {cores} of "
                     f"{os.cpu_count()} host threads), median of {reps} runs, {dt:.2f} s each"}
    if numpy is not None:
        n_setup, n_run, n_units, n_what = numpy
        a = n_setup()
        t0 = time.perf_counter()
        n_run(*a)
        ndt = time.perf_counter() - t0
        out["numpy_1core"] = {"value": n_units / ndt, "unit": UNIT, "cores": 1,
                              "sample": f"{n_what}: NumPy restatement (single-threaded ufuncs), "
                                        f"{ndt:.2f} s"}
    return out


def heat_config(world):
    """The headline workload's config, identical in both arms."""
    return {"workload": "heat_3d 256^3 float64, TSTEPS=100 (198 half-sweeps)",
            "grid": [N_GRID] * 3, "TSTEPS": TSTEPS, "updates_per_step": UPDATES_PER_STEP,
            "l2": "inputs larger than L2 (2 x 128 MiB), no flush",
            "parallelism": "replicas" if world > 1 else "single"}


def run_reference(args, world, rank):
    """The reference's CPU path: heat_3d(TSTEPS=100) on the 256^3 float64 grid, each
    step one whole workload through the C restatement of heat_3d_numpy.py (bit-identical
    to it) on all host threads; NumPy's own single-threaded rate is reported beside it."""
    if rank != 0:
        return
    from npbench_gb300 import workloads
    from oracle import cref
    A0, B0 = workloads.uniform_heat((N_GRID,) * 3, np.float64, seed=0)
    A, B = A0.copy(), B0.copy()
    for _ in range(max(0, args.warmup)):
        np.copyto(A, A0)
        np.copyto(B, B0)
        cref.heat_3d_kernel(TSTEPS, A, B)
    t_total = 0.0
    for _ in range(args.steps):
        np.copyto(A, A0)
        np.copyto(B, B0)
        t0 = time.perf_counter()
        cref.heat_3d_kernel(TSTEPS, A, B)
        t_total += time.perf_counter() - t0
    value = UPDATES_PER_STEP * args.steps / t_total
    cores = host_threads()
    v_np, dt_np = cpu_numpy_sample(half_sweeps=2)
    sample = (f"the whole workload (TSTEPS={TSTEPS}, {HALF_SWEEPS} half-sweeps) per step, C "
              f"restatement of heat_3d_numpy.py (OpenMP, {cores} of {os.cpu_count()} host threads)")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic U[0,1) from default_rng(0)",
        "config": heat_config(world),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": sample},
        "numpy_1core": {"value": v_np, "unit": UNIT, "cores": 1,
                        "sample": f"2 half-sweeps through the NumPy restatement, {dt_np:.2f} s"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gb300(args, world, rank, local):
    import torch
    from npbench_gb300 import stencils, workloads

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    stream = torch.cuda.current_stream(dev)

    def timed(dtype):
        A0, _ = workloads.uniform_heat((N_GRID,) * 3, dtype, seed=rank)
        pA = torch.from_numpy(A0).to(dev)
        A = torch.empty_like(pA)
        B = torch.empty_like(pA)

        def reset():
            A.copy_(pA)
            B.copy_(pA)

        for _ in range(args.warmup):
            reset()
            stencils.heat_3d_kernel(TSTEPS, A, B)
        torch.cuda.synchronize(dev)
        barrier()
        n0 = _library_launches()
        ev = []
        for _ in range(args.steps):
            reset()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            stencils.heat_3d_kernel(TSTEPS, A, B)
            e1.record(stream)
            ev.append((e0, e1))
        torch.cuda.synchronize(dev)
        barrier()
        _LAUNCHES["last"] = _library_launches() - n0
        ms = sum(a.elapsed_time(b) for a, b in ev)
        return ms, A, B, A0

    with ClockSampler(local) as clk:
        ms64, A64, B64, A0 = timed(np.float64)
    clocks = clk.summary()
    launches = _LAUNCHES["last"]
    from npbench_gb300 import replicas
    ms_max = replicas.max_over_ranks(ms64, device=dev)
    ms_per_step = ms_max / args.steps
    value = replicas.job_throughput(UPDATES_PER_STEP * args.steps, world, ms_max * 1e-3)

    # Roofline of the dominant kernel (one half-sweep launch).
    peak, peak_kind = measured_peaks()
    launch_ms = ms_per_step / HALF_SWEEPS
    alg_bytes = 16.0 * INTERIOR
    achieved = alg_bytes / (launch_ms * 1e-3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_kind": peak_kind,
                "traffic": ncu_traffic("heat3d_f64_256"),
                "kernel": "heat3d half-sweep float64", "alg_bytes_per_launch": alg_bytes,
                "launch_ms": launch_ms}
    # The arithmetic bounds.  fp64_roofline: the reference's 13 binary64
    # operations per update at the achieved rate, against what the binary64 pipe
    # alone retires (measured now by the DADD probe); above 1 because most
    # additions run exactly in fixed point on the integer pipes.
    # compute_roofline: the kernel's own instruction mix against every pipe.
    rates = measure_pipes() if rank == 0 else {}
    fp64_equiv = HEAT_FP64_OPS * INTERIOR / (launch_ms * 1e-3)
    fp64_roof = None
    if rates.get("dadd"):
        fp64_roof = {"ops_per_update": HEAT_FP64_OPS, "achieved_ops_per_s": fp64_equiv,
                     "fp64_pipe_ops_per_s": rates["dadd"], "frac": fp64_equiv / rates["dadd"],
                     "peak_kind": "DADD pipe probe (npbench_gb300.pipes), measured in this run"}
    comp_roof = compute_roofline("heat3d_f64_256", INTERIOR / (launch_ms * 1e-3), rates)

    # End to end through the public call with host buffers.
    hA = torch.from_numpy(A0).pin_memory()
    hB = hA.clone().pin_memory()
    oA = torch.empty_like(hA).pin_memory()
    oB = torch.empty_like(hA).pin_memory()
    dA = torch.empty_like(A64)
    dB = torch.empty_like(A64)
    e2e_ms = 0.0
    for it in range(args.warmup + args.steps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        dA.copy_(hA, non_blocking=True)
        dB.copy_(hB, non_blocking=True)
        stencils.heat_3d_kernel(TSTEPS, dA, dB)
        oA.copy_(dA, non_blocking=True)
        oB.copy_(dB, non_blocking=True)
        e1.record(stream)
        e1.synchronize()
        if it >= args.warmup:
            e2e_ms += e0.elapsed_time(e1)
    e2e_value = UPDATES_PER_STEP * args.steps / (e2e_ms * 1e-3)
    if world > 1:
        e2e_value *= world  # replicas run the same host-buffer path concurrently
    assert torch.equal(oA, A64.cpu()), "e2e result differs from the device-resident run"

    fp32 = None
    if not args.no_fp32:
        ms32, A32, _, _ = timed(np.float32)
        a64 = A64.double()
        diff = A32.double() - a64
        fp32 = {"value": UPDATES_PER_STEP * args.steps / (ms32 * 1e-3),
                "ms_per_step": ms32 / args.steps, "dtype": "f32",
                "roofline_frac": (8.0 * INTERIOR / (ms32 / args.steps / HALF_SWEEPS * 1e-3) / 1e9)
                / peak,
                "max_abs_err_vs_f64": float(diff.abs().max()),
                "rel_l2_err_vs_f64": float(diff.norm() / a64.norm())}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import cref, stencils_np
        hA = A0.copy()
        cpu = cpu_port(lambda: (hA.copy(), hA.copy()),
                       lambda a, b: cref.heat_3d_kernel(TSTEPS, a, b), UPDATES_PER_STEP,
                       f"the whole workload (TSTEPS={TSTEPS}) on the same 256^3 float64 grid",
                       reps=10,
                       numpy=(lambda: (hA.copy(), hA.copy()),
                              lambda a, b: stencils_np.heat_3d_kernel(3, a, b), 4 * INTERIOR,
                              "TSTEPS=3 (4 half-sweeps) on the same grid"))

    # Configurations 4 and 5 as blocks of the same line (one GPU only: under
    # torchrun the replicas report the headline workload alone).
    batch_block = serve_block = None
    if world == 1 and not args.no_batch:
        batch_block = batch_measure()
        batch_block["workload"] = BATCH_WORKLOAD.format(n=4096)
    if world == 1 and not args.no_serve:
        serve_block = serve_measure()
        serve_block["workload"] = SERVE_WORKLOAD.format(n=100, rate=0).replace(
            "Poisson 0 req/s", "Poisson arrivals at each rate")
        small = serve_measure(rates=(SMALL_RATE,), n_requests=SMALL_REQUESTS, stream=SMALL_STREAM)
        small["workload"] = SMALL_WORKLOAD.format(n=SMALL_REQUESTS, rate=SMALL_RATE)
        serve_block["small_grids"] = small

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic U[0,1) from numpy default_rng(rank), B = copy of A",
            "config": heat_config(world),
            "roofline": roofline,
            "fp64_roofline": fp64_roof,
            "compute_roofline": comp_roof,
            "pipe_rates_ops_per_s": dict(rates) if rates else None,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 2 * A64.nbytes,
                    "d2h_bytes_per_step": 2 * A64.nbytes},
            "gpu_launches": launches,
            "clocks": clocks,
            "fp32": fp32,
            "cpu_baseline": cpu,
            "batch": batch_block,
            "serve": serve_block,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


_LAUNCHES = {"last": None}


def _library_launches():
    """Kernels libnpbgb has put on a stream so far (its own counter)."""
    from npbench_gb300 import _lib
    return _lib.launches()


def _timed_steps(torch, dev, stream, step, reset, steps, warmup, flush=None):
    """Event time (ms) of `steps` calls of step(); reset() and flush() run untimed.
    The library's kernel launches inside the timed calls land in _LAUNCHES["last"]."""
    for _ in range(warmup):
        reset()
        step()
    torch.cuda.synchronize(dev)
    n0 = _library_launches()
    ev = []
    for _ in range(steps):
        reset()
        if flush is not None:
            flush()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        ev.append((e0, e1))
    torch.cuda.synchronize(dev)
    _LAUNCHES["last"] = _library_launches() - n0
    return sum(a.elapsed_time(b) for a, b in ev)


def _base_line(args, metric_value, ms_per_step, dtype, workload, extra_config, **kw):
    line = {"metric": METRIC, "value": metric_value, "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": dtype,
            "data": "synthetic U[0,1), seeded",
            "config": {"workload": workload, **extra_config}}
    line.update(kw)
    return line


def run_jacobi2d(args):
    """Jacobi-2D 1000^2 float64, TSTEPS=100 (16 MB: L2-resident, so L2 is flushed per step)."""
    import torch
    from npbench_gb300 import stencils, workloads
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    n, T = 1000, 100
    A0, B0 = workloads.uniform_pair((n, n), np.float64, seed=0)
    pA, pB = torch.from_numpy(A0).to(dev), torch.from_numpy(B0).to(dev)
    A, B = torch.empty_like(pA), torch.empty_like(pB)
    scrub = torch.empty(256 * 2**20 // 4, dtype=torch.float32, device=dev)

    def reset():
        A.copy_(pA)
        B.copy_(pB)

    with ClockSampler(0) as clk:
        ms = _timed_steps(torch, dev, stream, lambda: stencils.jacobi_2d_kernel(T, A, B), reset,
                          args.steps, args.warmup, flush=lambda: scrub.fill_(1.0))
    hs = 2 * (T - 1)
    ups = hs * (n - 2) ** 2
    ms_step = ms / args.steps
    peak, kind = measured_peaks()
    ach = 16.0 * (n - 2) ** 2 / (ms_step / hs * 1e-3) / 1e9
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import cref, stencils_np
        cpu = cpu_port(lambda: (A0.copy(), B0.copy()), lambda a, b: cref.jacobi_2d_kernel(T, a, b),
                       ups, f"the whole workload (TSTEPS={T}) on the same grid", reps=5,
                       numpy=(lambda: (A0.copy(), B0.copy()),
                              lambda a, b: stencils_np.jacobi_2d_kernel(11, a, b),
                              20 * (n - 2) ** 2, "TSTEPS=11 (20 half-sweeps)"))
    print(json.dumps(_base_line(
        args, ups * args.steps / (ms * 1e-3), ms_step, "f64",
        "jacobi_2d 1000^2 float64, TSTEPS=100 (198 half-sweeps)",
        {"grid": [n, n], "TSTEPS": T, "l2": "16 MB grid is L2-resident; 256 MB scrub written "
         "between timed steps"},
        roofline={"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                  "peak_kind": kind, "traffic": ncu_traffic("jacobi2d_f64_1000"),
                  "note": "inputs live in L2 within a step; frac may exceed what HBM alone allows"},
        gpu_launches=_LAUNCHES["last"], clocks=clk.summary(), cpu_baseline=cpu)), flush=True)


def run_hdiff(args):
    """hdiff 256x256x160 float64, one call per step (the harness repeats it)."""
    import torch
    from npbench_gb300 import stencils, workloads
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    I, J, K = 256, 256, 160
    inf, out0, coeff = workloads.init_hdiff(I, J, K)
    dIn, dOut, dC = (torch.from_numpy(x).to(dev) for x in (inf, out0, coeff))
    scrub = torch.empty(256 * 2**20 // 4, dtype=torch.float32, device=dev)
    with ClockSampler(0) as clk:
        ms = _timed_steps(torch, dev, stream, lambda: stencils.hdiff(dIn, dOut, dC), lambda: None,
                          args.steps, args.warmup, flush=lambda: scrub.fill_(1.0))
    ms_step = ms / args.steps
    pts = I * J * K
    alg = 8.0 * ((I + 4) * (J + 4) * K + 2 * I * J * K)
    peak, kind = measured_peaks()
    ach = alg / (ms_step * 1e-3) / 1e9
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import cref, stencils_np
        cpu = cpu_port(lambda: (out0.copy(),), lambda o: cref.hdiff(inf, o, coeff), pts,
                       "one call on the same 256x256x160 input", reps=5,
                       numpy=(lambda: (out0.copy(),), lambda o: stencils_np.hdiff(inf, o, coeff),
                              pts, "one call"))
    print(json.dumps(_base_line(
        args, pts * args.steps / (ms * 1e-3), ms_step, "f64",
        "hdiff 256x256x160 float64 (reference initialize), one call per step",
        {"shape": [I, J, K], "l2": "253 MB of inputs+output; 256 MB scrub between steps"},
        unit_note="value counts output points per second",
        roofline={"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                  "peak_kind": kind, "traffic": ncu_traffic("hdiff_f64_256"),
                  "alg_bytes_per_launch": alg},
        gpu_launches=_LAUNCHES["last"], clocks=clk.summary(), cpu_baseline=cpu)), flush=True)


def run_jacobi1d(args):
    """Jacobi-1D at NPBench's paper preset (N=32000, TSTEPS=4000), float64."""
    import torch
    from npbench_gb300 import stencils, workloads
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    n, T = 32000, 4000
    A0, B0 = workloads.init_jacobi_1d(n)
    pA, pB = torch.from_numpy(A0).to(dev), torch.from_numpy(B0).to(dev)
    A, B = torch.empty_like(pA), torch.empty_like(pB)

    def reset():
        A.copy_(pA)
        B.copy_(pB)

    with ClockSampler(0) as clk:
        ms = _timed_steps(torch, dev, stream, lambda: stencils.jacobi_1d_kernel(T, A, B), reset,
                          args.steps, args.warmup)
    ups = 2 * (T - 1) * (n - 2)
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import cref, stencils_np
        cpu = cpu_port(lambda: (A0.copy(), B0.copy()), lambda a, b: cref.jacobi_1d_kernel(T, a, b),
                       ups, f"the whole workload (TSTEPS={T})", parallel=False,
                       numpy=(lambda: (A0.copy(), B0.copy()),
                              lambda a, b: stencils_np.jacobi_1d_kernel(T, a, b), ups,
                              f"the whole workload (TSTEPS={T})"))
    peak, kind = measured_peaks()
    ach = 16.0 * ups / (ms / args.steps * 1e-3) / 1e9
    from npbench_gb300 import _lib
    depth = _lib.get_config(_lib.NPBGB_CFG_JACOBI1D_DEPTH)  # half-sweeps per launch in effect
    print(json.dumps(_base_line(
        args, ups * args.steps / (ms * 1e-3), ms / args.steps, "f64",
        "jacobi_1d N=32000 float64, TSTEPS=4000 (paper preset, reference initialize)",
        {"n": n, "TSTEPS": T, "l2": "256 KB arrays are L2-resident"},
        roofline={"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                  "peak_kind": kind, "traffic": None,
                  "note": f"16 B per update; {depth} half-sweeps per launch run in shared "
                          "memory, so the binary64 pipe, not HBM, bounds it"},
        gpu_launches=_LAUNCHES["last"], clocks=clk.summary(),
        cpu_baseline=cpu)), flush=True)


def run_vadv(args):
    """vadv 256x256x160 float64 (paper preset, reference initialize), one call per step."""
    import torch
    from npbench_gb300 import stencils, workloads
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    I, J, K = 256, 256, 160
    dtr, us0, u, w, up, ut = workloads.init_vadv(I, J, K)
    pristine = torch.from_numpy(us0).to(dev)
    dUs = pristine.clone()
    dU, dW, dUp, dUt = (torch.from_numpy(x).to(dev) for x in (u, w, up, ut))

    def reset():
        dUs.copy_(pristine)

    with ClockSampler(0) as clk:
        ms = _timed_steps(torch, dev, stream,
                          lambda: stencils.vadv(dUs, dU, dW, dUp, dUt, dtr), reset,
                          args.steps, args.warmup)
    ms_step = ms / args.steps
    pts = I * J * K
    # read utens_stage, u_stage, u_pos, utens and wcon once, write utens_stage once
    alg = 8.0 * (5 * I * J * K + (I + 1) * J * K)
    peak, kind = measured_peaks()
    ach = alg / (ms_step * 1e-3) / 1e9
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import cref, stencils_np
        cpu = cpu_port(lambda: (us0.copy(),), lambda o: cref.vadv(o, u, w, up, ut, dtr), pts,
                       "one call on the same 256x256x160 input",
                       numpy=(lambda: (us0.copy(),), lambda o: stencils_np.vadv(o, u, w, up, ut, dtr),
                              pts, "one call"))
    print(json.dumps(_base_line(
        args, pts * args.steps / (ms * 1e-3), ms_step, "f64",
        "vadv 256x256x160 float64 (paper preset, reference initialize), one call per step",
        {"shape": [I, J, K], "l2": "420 MB of inputs+output, larger than L2"},
        unit_note="value counts output points per second",
        roofline={"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                  "peak_kind": kind, "traffic": ncu_traffic("vadv_f64_256"),
                  "alg_bytes_per_launch": alg},
        gpu_launches=_LAUNCHES["last"], clocks=clk.summary(), cpu_baseline=cpu)), flush=True)


def run_cavity(args):
    """cavity_flow at NPBench's paper preset (101 x 101, nt=700, nit=50), float64, one
    call (the whole time loop) per step."""
    import torch
    from npbench_gb300 import stencils, workloads
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    ny, nx, nt, nit, rho, nu = 101, 101, 700, 50, 1.0, 0.1
    u0, v0, p0, dx, dy, dt = workloads.init_cavity_flow(ny, nx)
    pristine = [torch.from_numpy(x).to(dev) for x in (u0, v0, p0)]
    work = [x.clone() for x in pristine]

    def reset():
        for w, p in zip(work, pristine):
            w.copy_(p)

    with ClockSampler(0) as clk:
        ms = _timed_steps(torch, dev, stream,
                          lambda: stencils.cavity_flow(nx, ny, nt, nit, work[0], work[1], dt, dx,
                                                       dy, work[2], rho, nu),
                          reset, args.steps, args.warmup)
    ms_step = ms / args.steps
    sweeps = nt * (nit + 2)                   # b, nit pressure iterations, u/v per step
    ups = sweeps * (ny - 2) * (nx - 2)
    # per interior point and sweep: pressure reads p and pC*b, writes p (24 B); b reads u, v and
    # writes pC*b (24 B); u/v read un, vn, p and write u, v (40 B)
    alg = nt * (ny - 2) * (nx - 2) * (24.0 * nit + 24.0 + 40.0)
    peak, kind = measured_peaks()
    ach = alg / (ms_step * 1e-3) / 1e9
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import cref, stencils_np
        fresh = lambda: tuple(x.copy() for x in (u0, v0, p0))  # noqa: E731
        cpu = cpu_port(fresh,
                       lambda u, v, p: cref.cavity_flow(nx, ny, nt, nit, u, v, dt, dx, dy, p, rho,
                                                        nu),
                       ups, f"the whole workload (nt={nt}, nit={nit})", parallel=False,
                       numpy=(fresh,
                              lambda u, v, p: stencils_np.cavity_flow(nx, ny, 20, nit, u, v, dt,
                                                                      dx, dy, p, rho, nu),
                              20 * (nit + 2) * (ny - 2) * (nx - 2), "nt=20 of the same problem"))
    print(json.dumps(_base_line(
        args, ups * args.steps / (ms * 1e-3), ms_step, "f64",
        "cavity_flow 101x101 float64, nt=700, nit=50 (paper preset, reference initialize), "
        "one call per step",
        {"shape": [ny, nx], "nt": nt, "nit": nit, "sweeps_per_call": sweeps,
         "unit_note": "value counts interior points x sweeps (b, each pressure iteration, u/v) "
                      "per second",
         "l2": "four 82 KB fields are L2-resident"},
        roofline={"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                  "peak_kind": kind, "traffic": None,
                  "note": "36,400 dependent sweeps of a 10K-point grid in one launch: bound by "
                          "the latency of each sweep's neighbour hand-off, not by bytes"},
        gpu_launches=_LAUNCHES["last"], clocks=clk.summary(), cpu_baseline=cpu)), flush=True)


def run_channel(args):
    """channel_flow at NPBench's paper preset (101 x 101, nit=50, run to convergence: 989
    steps), float64, one call per step."""
    import torch
    from npbench_gb300 import stencils, workloads
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    ny, nx, nit, rho, nu, F = 101, 101, 50, 1.0, 0.1, 1.0
    u0, v0, p0, dx, dy, dt = workloads.init_channel_flow(ny, nx)
    pristine = [torch.from_numpy(x).to(dev) for x in (u0, v0, p0)]
    work = [x.clone() for x in pristine]
    steps = []

    def reset():
        for w, p in zip(work, pristine):
            w.copy_(p)

    def call():
        steps.append(stencils.channel_flow(nit, work[0], work[1], dt, dx, dy, work[2], rho, nu, F))

    with ClockSampler(0) as clk:
        ms = _timed_steps(torch, dev, stream, call, reset, args.steps, args.warmup)
    ms_step = ms / args.steps
    nsteps = steps[-1]
    sweeps = nsteps * (nit + 2)
    ups = sweeps * (ny - 2) * nx
    alg = nsteps * (ny - 2) * nx * (24.0 * nit + 24.0 + 40.0)
    peak, kind = measured_peaks()
    ach = alg / (ms_step * 1e-3) / 1e9
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import cref, stencils_np
        fresh = lambda: tuple(x.copy() for x in (u0, v0, p0))  # noqa: E731
        cpu = cpu_port(fresh,
                       lambda u, v, p: cref.channel_flow(nit, u, v, dt, dx, dy, p, rho, nu, F),
                       ups, f"the whole run ({nsteps} steps)", parallel=False,
                       numpy=(fresh,
                              lambda u, v, p: stencils_np.channel_flow(nit, u, v, dt, dx, dy, p,
                                                                       rho, nu, F),
                              ups, f"the whole run ({nsteps} steps)"))
    print(json.dumps(_base_line(
        args, ups * args.steps / (ms * 1e-3), ms_step, "f64",
        "channel_flow 101x101 float64, nit=50, to convergence (paper preset, reference "
        "initialize), one call per step",
        {"shape": [ny, nx], "nit": nit, "steps_to_convergence": nsteps,
         "sweeps_per_call": sweeps,
         "unit_note": "value counts row points x sweeps (b, each pressure iteration, u/v) per "
                      "second; each step also sums u exactly as np.sum does",
         "l2": "four 82 KB fields are L2-resident"},
        roofline={"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                  "peak_kind": kind, "traffic": None,
                  "note": "dependent sweeps of a 10K-point grid in one launch: bound by the "
                          "latency of each sweep's neighbour hand-off, not by bytes"},
        gpu_launches=_LAUNCHES["last"], clocks=clk.summary(), cpu_baseline=cpu)), flush=True)


def run_fdtd2d(args):
    """FDTD-2D at NPBench's paper preset (TMAX=500, 1000 x 1200), float64."""
    import torch
    from npbench_gb300 import stencils, workloads
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    T, nx, ny = 500, 1000, 1200
    host = workloads.init_fdtd_2d(T, nx, ny)
    pristine = [torch.from_numpy(x).to(dev) for x in host]
    work = [x.clone() for x in pristine]

    def reset():
        for w, p in zip(work[:3], pristine[:3]):
            w.copy_(p)

    with ClockSampler(0) as clk:
        ms = _timed_steps(torch, dev, stream, lambda: stencils.fdtd_2d_kernel(T, *work), reset,
                          args.steps, args.warmup)
    cells = T * nx * ny  # cell-steps (each updates ex, ey and hz)
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import cref, stencils_np
        fresh = lambda: tuple(x.copy() for x in host)  # noqa: E731
        cpu = cpu_port(fresh, lambda ex, ey, hz, fict: cref.fdtd_2d_kernel(T, ex, ey, hz, fict),
                       cells, f"the whole workload (TMAX={T})",
                       numpy=(fresh,
                              lambda ex, ey, hz, fict: stencils_np.fdtd_2d_kernel(20, ex, ey, hz,
                                                                                  fict),
                              20 * nx * ny, "TMAX=20 on the same fields"))
    peak, kind = measured_peaks()
    ach = 48.0 * cells / (ms / args.steps * 1e-3) / 1e9
    print(json.dumps(_base_line(
        args, cells * args.steps / (ms * 1e-3), ms / args.steps, "f64",
        "fdtd_2d 1000x1200 float64, TMAX=500 (paper preset, reference initialize)",
        {"shape": [nx, ny], "TMAX": T, "unit_note": "value counts cell-steps per second",
         "l2": "the three 9.6 MB fields are L2-resident"},
        roofline={"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                  "peak_kind": kind, "traffic": None,
                  "note": "48 B per cell-step (ex, ey, hz read and written once)"},
        gpu_launches=_LAUNCHES["last"], clocks=clk.summary(), cpu_baseline=cpu)), flush=True)


def _rel_err(low, ref):
    """(max-abs, relative L2) of a low-precision result against its float64 run."""
    d = low.double() - ref
    nrm = float(ref.norm())
    return float(d.abs().max()) if d.numel() else 0.0, (float(d.norm()) / nrm if nrm > 0 else 0.0)


def _fp32_error_report(pairs):
    """pairs: (TSTEPS, float32 result, float64 result of the same grid).  Worst error
    overall and per TSTEPS range, with the grid count."""
    bins = [(0, 100), (100, 250), (250, 10**9)]
    out = {"grids": len(pairs), "max_abs": 0.0, "rel_l2_max": 0.0, "rel_l2_max_tsteps": None,
           "by_tsteps": {}}
    for lo, hi in bins:
        out["by_tsteps"][f"{lo}-{hi if hi < 10**9 else 'max'}"] = {"grids": 0, "rel_l2_max": 0.0}
    for T, low, ref in pairs:
        mx, rl = _rel_err(low, ref)
        out["max_abs"] = max(out["max_abs"], mx)
        if rl >= out["rel_l2_max"]:
            out["rel_l2_max"], out["rel_l2_max_tsteps"] = rl, T
        for lo, hi in bins:
            if lo <= T < hi:
                b = out["by_tsteps"][f"{lo}-{hi if hi < 10**9 else 'max'}"]
                b["grids"] += 1
                b["rel_l2_max"] = max(b["rel_l2_max"], rl)
    return out


BATCH_FORM = "stepped"
BATCH_TILE_ROWS = 128


def _per_grid_guarded(work, guard):
    """Plain per-grid launches of the batch's grids, under the same float64 guard:
    a promoted float32 grid is widened, run in float64 and rounded back."""
    import torch
    from npbench_gb300 import precision, stencils
    for a, b, T in work:
        if guard and a.dtype == torch.float32 and precision.needs_fp64("jacobi2d", T):
            a64, b64 = a.double(), b.double()
            stencils.jacobi_2d_kernel(T, a64, b64)
            a.copy_(a64)
            b.copy_(b64)
        else:
            stencils.jacobi_2d_kernel(T, a, b)


def batch_measure(n_grids=4096, steps=2, warmup=1, compare=True, compare_steps=1,
                  compare_warmup=1, fp32_error=True, cpu=False, guard=True, form=None,
                  tile_rows=None):
    """Configuration 4: ``n_grids`` independent Jacobi-2D grids (sides log-uniform in
    [64, 2048] per axis, half float32 and half float64, TSTEPS uniform in [10, 500])
    advanced by one batch per step.  With ``guard`` the float32 grids whose float32
    error would exceed 1e-5 run in float64 (both arms).  Returns the measurement."""
    import torch
    from npbench_gb300 import _lib, stencils, workloads
    from npbench_gb300.batch import Batch
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    specs = workloads.batch_jacobi_specs(n_grids, seed=0)
    gen = torch.Generator(device=dev)
    gen.manual_seed(0)
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

    from npbench_gb300 import autotune, precision
    form = form or BATCH_FORM
    tuned = autotune.batch_settings([(s, dt) for s, dt, _ in specs])
    rows = tile_rows or tuned.get("rows") or BATCH_TILE_ROWS
    promoted = [guard and dt == np.float32 and precision.needs_fp64("jacobi2d", T)
                for _, dt, T in specs]
    ups = sum(2 * (T - 1) * (s[0] - 2) * (s[1] - 2) for s, _, T in specs)
    # algorithmic bytes: 2 x the element size per update, in the precision it runs in
    alg = sum(2 * (T - 1) * (s[0] - 2) * (s[1] - 2) * 2 * (8 if p else np.dtype(dt).itemsize)
              for (s, dt, T), p in zip(specs, promoted))
    with autotune.batch_applied(tuned), Batch(work, band_rows=rows, mode=form,
                                              guard=guard) as batch:
        info = batch.info()
        with ClockSampler(0) as clk:
            ms = _timed_steps(torch, dev, stream, lambda: batch.launch(graph=True), reset,
                              steps, warmup)
        launches = _LAUNCHES["last"]
        _lib.device_status()
    ms_step = ms / steps
    peak, kind = measured_peaks()
    ach = alg / (ms_step * 1e-3) / 1e9
    out = {"value": ups / (ms_step * 1e-3), "unit": UNIT, "ms_per_step": ms_step,
           "steps": steps, "warmup": warmup, "updates_per_step": ups,
           "cells": sum(s[0] * s[1] for s, _, _ in specs), "form": info["mode"],
           "tiles" if info["mode"] != "persistent" else "bands": info["bands"],
           "launches" if info["mode"] == "stepped" else "ctas": info["ctas"],
           "rows_per_tile": rows, "graph": True,
           "tuned": {"class": autotune.batch_key([(s, dt) for s, dt, _ in specs]),
                     "settings": dict(tuned, rows=rows)},
           "fp64_guard": {"on": bool(guard), "float32_grids_run_in_float64": int(sum(promoted)),
                          "float32_grids": int(sum(dt == np.float32 for _, dt, _ in specs))},
           "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                        "frac": ach / peak, "peak_kind": kind,
                        "traffic": ncu_traffic("batch_4096"),
                        "traffic_over_algorithmic":
                            _ncu_record("batch_4096").get("traffic_over_algorithmic")},
           "clocks": clk.summary(), "gpu_launches": launches}
    if compare:
        ms_pg = _timed_steps(torch, dev, stream, lambda: _per_grid_guarded(work, guard), reset,
                             compare_steps, compare_warmup)
        ms_pg /= compare_steps
        out["per_grid"] = {"value": ups / (ms_pg * 1e-3), "ms_per_step": ms_pg,
                           "steps": compare_steps, "warmup": compare_warmup,
                           "kernel_launches": _LAUNCHES["last"],
                           "what": "one jacobi_2d_kernel call per grid (tuned single-grid "
                                   "kernels: chained launches, or one launch with the bands "
                                   "in shared memory), same inputs, steps and float64 guard"}
        out["batched_over_per_grid"] = ms_pg / ms_step
    if fp32_error:
        # The float32 grids (as the batch left them, guard included) against float64
        # runs of the same inputs, widened exactly.
        reset()
        with Batch(work, band_rows=rows, mode=form, guard=guard) as batch:
            batch.launch()
        f32 = [(g, T) for g, ((_, dt, T), _) in enumerate(zip(specs, work)) if dt == np.float32]
        shadow = [(init[g][0].double(), init[g][1].double(), T) for g, T in f32]
        with Batch(shadow, band_rows=rows, mode=form) as sb:
            sb.launch()
        torch.cuda.synchronize(dev)
        out["fp32_error_vs_fp64"] = _fp32_error_report(
            [(T, work[g][0], shadow[n][0]) for n, (g, T) in enumerate(f32)])
        del shadow
    if cpu:
        # The first 64 grids of the same configuration, seeded host inputs: timed
        # through the C restatement on all host threads, and run as a GPU batch
        # that must match it bit for bit.
        from oracle import cref
        sample = specs[:64]
        rng = np.random.default_rng(1)
        host = [(rng.random(sh).astype(dt), rng.random(sh).astype(dt), T) for sh, dt, T in sample]
        gpu = [(torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev), T) for a, b, T in host]
        with Batch(gpu) as sb:
            sb.launch()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for a, b, T in host:
            cref.jacobi_2d_kernel(T, a, b)
        dt_cpu = time.perf_counter() - t0
        exact = all(np.array_equal(a.view(np.uint8), ga.cpu().numpy().view(np.uint8)) and
                    np.array_equal(b.view(np.uint8), gb.cpu().numpy().view(np.uint8))
                    for (a, b, _), (ga, gb, _) in zip(host, gpu))
        ups_s = sum(2 * (T - 1) * (sh[0] - 2) * (sh[1] - 2) for sh, _, T in sample)
        out["cpu_baseline"] = {
            "value": ups_s / dt_cpu, "unit": UNIT, "cores": host_threads(), "kind": "port",
            "sample": f"the first {len(sample)} grids of the batch ({ups_s:.3g} updates), C "
                      f"restatement on {host_threads()} host threads, {dt_cpu:.2f} s; the GPU "
                      f"batch of the same grids {'matches it bit for bit' if exact else 'DIFFERS'}"}
    del init, work
    torch.cuda.empty_cache()
    return out


BATCH_WORKLOAD = ("batched jacobi_2d: {n} grids, sides log-uniform [64, 2048], half float32 / "
                  "half float64, TSTEPS uniform [10, 500]")


def run_batch(args):
    """Configuration 4 on its own line (``--workload batch``)."""
    b = batch_measure(args.batch_grids, steps=args.steps, warmup=args.warmup,
                      compare=args.compare, cpu=not args.no_cpu_baseline)
    extra = {k: b[k] for k in ("cells", "updates_per_step", "form", "rows_per_tile", "graph")}
    print(json.dumps(_base_line(
        args, b["value"], b["ms_per_step"], "f32+f64", BATCH_WORKLOAD.format(n=args.batch_grids),
        dict(extra, l2=f"{b['cells'] * 6 * 2 / 1e9:.1f} GB resident, far above L2"),
        roofline=b["roofline"], comparator=b.get("per_grid"),
        batched_over_per_grid=b.get("batched_over_per_grid"),
        fp32_error_vs_fp64=b.get("fp32_error_vs_fp64"), gpu_launches=b["gpu_launches"],
        clocks=b["clocks"], cpu_baseline=b.get("cpu_baseline"))), flush=True)


SERVE_WORKLOAD = ("served stream: {n} requests, Poisson {rate:g} req/s, 2D Jacobi 128^2-4096^2 "
                  "and 3D heat 32^3-384^3 (log-uniform per axis), 70% float32, TSTEPS 20-1000")

# A stream of grids small enough for the tile queue: every request is folded
# into the running worker kernel, none takes a big-grid lane.
SMALL_STREAM = {"side2d": (32, 224), "side3d": (12, 36)}
SMALL_REQUESTS, SMALL_RATE = 1000, 20000.0
SMALL_WORKLOAD = ("small-grid stream: {n} requests, Poisson {rate:g} req/s, 2D Jacobi 32^2-224^2 "
                  "and 3D heat 12^3-36^3 (log-uniform per axis), 70% float32, TSTEPS 20-1000")


def serve_measure(rates=(200.0, 1000.0, 5000.0), n_requests=100, compare=True, fp32_error=True,
                  cpu=False, stream=None):
    """Configuration 5: Poisson arrivals of mixed solves through the continuous-batching
    server at each rate, beside the same requests run one at a time with per-grid
    launches.  `stream` overrides the request sizes (workloads.served_requests keywords).
    Returns {"rates": [...], "fp32_error_vs_fp64": ...}."""
    stream = dict(stream or {})
    import torch
    from npbench_gb300 import stencils, workloads
    from npbench_gb300.server import (Request, StencilServer, latency_stats, run_sequential,
                                      _materialise)
    with StencilServer() as warm:
        warm.submit(Request(shape=(64, 64), dtype=np.float32, tsteps=5, seed=1)).result()
    from npbench_gb300 import autotune
    out = {"requests_per_rate": n_requests, "hbm_budget_gb": 150, "rates": [],
           "tuned": {"class": autotune.server_key(), "settings": autotune.server_settings()},
           "inputs": "seeded U[0,1) host arrays in pinned memory, uploaded by the server "
                     "(and by the comparator) inside the measured span; results stay on "
                     "the device"}
    kept = None
    # The same requests at every rate (only the arrival times scale).
    _, specs = workloads.served_requests(n_requests, rates[0], seed=0, **stream)
    host = [_pinned_inputs(s, dt, sd) for s, dt, T, sd in specs]
    for rate in rates:
        arrivals, _ = workloads.served_requests(n_requests, rate, seed=0, **stream)

        def make():
            return [Request(shape=s, dtype=dt, tsteps=T, a=h[0], b=h[1], return_host=False)
                    for (s, dt, T, sd), h in zip(specs, host)]
        reqs = make()
        torch.cuda.synchronize()
        n_launch0 = _library_launches()
        srv = StencilServer(hbm_budget_bytes=150e9).start()
        futs = []
        with ClockSampler(0) as clk:
            # The arrival clock starts once the sampler runs (its start-up wait
            # would otherwise turn the first arrivals into one burst).
            t0 = time.perf_counter()
            for r, at in zip(reqs, arrivals):
                now = time.perf_counter() - t0
                if at > now:
                    time.sleep(at - now)
                futs.append(srv.submit(r))
            results = [f.result() for f in futs]
            srv.stop()
        torch.cuda.synchronize()
        n_launch = _library_launches() - n_launch0
        st = latency_stats(reqs)
        entry = {"rate_hz": rate, "served": {k: st[k] for k in ("updates_per_s", "p50_ms",
                                                                  "p99_ms", "mean_ms", "span_s")},
                 "worker_launches": srv.launches, "float32_requests_run_in_float64": srv.promoted,
                 "paths": {"tile_queue": srv.queued_small, "big_grid_lanes": srv.ran_big},
                 "gpu_launches": n_launch,
                 "peak_resident_gb": srv.admission.peak / 1e9, "clocks": clk.summary()}
        if compare:
            seq = make()
            run_sequential(seq, arrivals)
            sq = latency_stats(seq)
            entry["sequential"] = {k: sq[k] for k in ("updates_per_s", "p50_ms", "p99_ms",
                                                      "mean_ms", "span_s")}
            entry["served_over_sequential"] = st["updates_per_s"] / sq["updates_per_s"]
        out["rates"].append(entry)
        if fp32_error and kept is None:
            kept = (reqs, results)
        else:
            del results
        torch.cuda.empty_cache()
    out["stream_updates"] = sum(r.updates for r in reqs)
    if kept is not None:
        reqs, results = kept
        dev = torch.device("cuda", 0)
        pairs = []
        for r, (A, B) in zip(reqs, results):
            if np.dtype(r.dtype) != np.float32 or r.tsteps <= 1:
                continue
            a64, b64 = _materialise(r, dev)
            a64, b64 = a64.double(), b64.double()
            (stencils.jacobi_2d_kernel if a64.dim() == 2 else stencils.heat_3d_kernel)(
                r.tsteps, a64, b64)
            pairs.append((r.tsteps, A, a64))
        torch.cuda.synchronize(dev)
        rep = _fp32_error_report(pairs)
        rep["what"] = ("float32 requests of the stream (float64 guard on) against float64 "
                       "runs of the same inputs, widened exactly")
        out["fp32_error_vs_fp64"] = rep
        del pairs, kept, results
        torch.cuda.empty_cache()
    if cpu:
        # The stream's requests in arrival order, up to about 2e10 updates,
        # through the C restatement on all host threads.
        from oracle import cref
        _, specs = workloads.served_requests(n_requests, rates[0], seed=0, **stream)
        rng = np.random.default_rng(2)
        done_ups, t_cpu, n = 0, 0.0, 0
        for shape, dt, T, _ in specs:
            if done_ups > 2e10:
                break
            a = rng.random(shape).astype(dt)
            b = a.copy() if len(shape) == 3 else rng.random(shape).astype(dt)
            t0 = time.perf_counter()
            (cref.jacobi_2d_kernel if len(shape) == 2 else cref.heat_3d_kernel)(T, a, b)
            t_cpu += time.perf_counter() - t0
            done_ups += 2 * (T - 1) * int(np.prod([x - 2 for x in shape]))
            n += 1
        out["cpu_baseline"] = {
            "value": done_ups / t_cpu, "unit": UNIT, "cores": host_threads(), "kind": "port",
            "sample": f"the stream's first {n} requests ({done_ups:.3g} updates), C "
                      f"restatement on {host_threads()} host threads, {t_cpu:.2f} s"}
    return out


def _pinned_inputs(shape, dt, seed):
    """Seeded U[0,1) inputs of one request in pinned host memory: A, and B for 2D."""
    import torch
    tdt = torch.float32 if dt == np.float32 else torch.float64
    rng = np.random.default_rng(seed)
    a = torch.empty(shape, dtype=tdt, pin_memory=True).numpy()
    rng.random(shape, dtype=dt, out=a)
    if len(shape) != 2:
        return a, None
    b = torch.empty(shape, dtype=tdt, pin_memory=True).numpy()
    rng.random(shape, dtype=dt, out=b)
    return a, b


def run_serve(args):
    """Configuration 5 on its own line (``--workload serve``) at ``--rate``."""
    small = args.stream == "small"
    s = serve_measure(rates=(args.rate,), n_requests=args.requests, compare=args.compare,
                      cpu=not args.no_cpu_baseline, stream=SMALL_STREAM if small else None)
    e = s["rates"][0]
    print(json.dumps(_base_line(
        args, e["served"]["updates_per_s"], e["served"]["span_s"] * 1e3, "f32+f64",
        (SMALL_WORKLOAD if small else SERVE_WORKLOAD).format(n=args.requests, rate=args.rate),
        {"hbm_budget_gb": 150, "worker_launches": e["worker_launches"], "paths": e["paths"],
         "float32_requests_run_in_float64": e["float32_requests_run_in_float64"],
         "peak_resident_gb": e["peak_resident_gb"]},
        latency={k: e["served"][k] for k in ("p50_ms", "p99_ms", "mean_ms")},
        comparator=e.get("sequential"), served_over_sequential=e.get("served_over_sequential"),
        fp32_error_vs_fp64=s.get("fp32_error_vs_fp64"), clocks=e["clocks"],
        cpu_baseline=s.get("cpu_baseline"))), flush=True)


def main():
    args = parse()
    world, rank, local = dist_info()
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.workload == "heat3d":
        run_gb300(args, world, rank, local)
    elif rank == 0:
        {"jacobi2d": run_jacobi2d, "hdiff": run_hdiff, "batch": run_batch,
         "serve": run_serve, "jacobi1d": run_jacobi1d, "fdtd2d": run_fdtd2d, "vadv": run_vadv,
         "cavity": run_cavity, "channel": run_channel}[args.workload](args)


if __name__ == "__main__":
    main()
