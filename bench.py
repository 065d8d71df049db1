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
* ``fp32``      the same workload in float32 with its error against float64;
* ``cpu_baseline`` the NumPy restatement of the reference kernel on a bounded
                sample (16 half-sweeps of the same grid), one host core
                (NumPy's elementwise ufuncs are single-threaded).

``--impl reference`` times only that CPU implementation (the reference's own
arithmetic) on the host cores and prints its line with ``"impl": "reference"``.

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


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp32", action="store_true")
    return ap.parse_args()


def dist_info():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic(kernel_key):
    """DRAM bytes per launch recorded from an ncu capture (profiles/ncu_traffic.json)."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as f:
            d = json.load(f)
        return d.get(kernel_key, {}).get("dram_bytes_per_launch")
    except Exception:
        return None


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


def run_reference(args, world, rank):
    if rank != 0:
        return
    ups = []
    for _ in range(max(0, args.warmup)):
        cpu_numpy_sample()
    t_total = 0.0
    for _ in range(args.steps):
        v, dt = cpu_numpy_sample()
        ups.append(v)
        t_total += dt
    value = 2 * INTERIOR * args.steps / t_total
    sample = (f"2 half-sweeps of the 256^3 float64 heat grid per step "
              f"(heat_3d_numpy.py arithmetic via its NumPy restatement)")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic U[0,1) from default_rng(0)",
        "config": {"workload": "heat_3d 256^3 float64 (bounded sample: 2 half-sweeps per step)",
                   "TSTEPS": TSTEPS, "grid": [N_GRID] * 3},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": sample},
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
        ms = sum(a.elapsed_time(b) for a, b in ev)
        return ms, A, B, A0

    with ClockSampler(local) as clk:
        ms64, A64, B64, A0 = timed(np.float64)
    clocks = clk.summary()
    ms_max = ms64
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms64], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_max = float(t.item())
    ms_per_step = ms_max / args.steps
    value = world * UPDATES_PER_STEP * args.steps / (ms_max * 1e-3)

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
        v, dt = cpu_numpy_sample(half_sweeps=16)
        cpu = {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"16 half-sweeps of the 256^3 float64 grid, NumPy restatement of "
                         f"heat_3d_numpy.py, {dt:.1f} s; host has {os.cpu_count()} cores, "
                         f"NumPy ufuncs use one"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic U[0,1) from numpy default_rng(rank), B = copy of A",
            "config": {"workload": "heat_3d 256^3 float64, TSTEPS=100 (198 half-sweeps)",
                       "grid": [N_GRID] * 3, "TSTEPS": TSTEPS,
                       "updates_per_step": UPDATES_PER_STEP,
                       "l2": "inputs larger than L2 (2 x 128 MiB), no flush",
                       "parallelism": "replicas" if world > 1 else "single"},
            "roofline": roofline,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 2 * A64.nbytes,
                    "d2h_bytes_per_step": 2 * A64.nbytes},
            "gpu_launches": HALF_SWEEPS * args.steps,
            "clocks": clocks,
            "fp32": fp32,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    args = parse()
    world, rank, local = dist_info()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_gb300(args, world, rank, local)


if __name__ == "__main__":
    main()
