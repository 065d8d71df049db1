"""bench.py's output contract: one JSON line with the keys the measurement needs.

CPU: the reference arm (the reference's arithmetic on the host's threads) prints
its line, and under torchrun with two ranks only rank 0 prints it.  GPU: a short
run of the default workload carries the roofline, end-to-end, clock and launch
fields next to the metric.
"""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BASE_KEYS = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
             "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config"}


def _lines(out):
    return [json.loads(ln) for ln in out.splitlines() if ln.startswith("{")]


def _run(args, timeout=900, env=None):
    e = dict(os.environ)
    e.update(env or {})
    r = subprocess.run([sys.executable] + args, cwd=ROOT, capture_output=True, text=True,
                       timeout=timeout, env=e)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def test_reference_arm_line():
    (line,) = _lines(_run(["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"],
                          env={"OMP_NUM_THREADS": "2"}))
    assert BASE_KEYS <= set(line)
    assert line["impl"] == "reference" and line["metric"] == "lattice_updates_per_s"
    assert line["value"] > 0 and line["higher_is_better"] is True and line["dtype"] == "f64"
    cpu = line["cpu_baseline"]
    assert cpu["value"] == line["value"] and cpu["kind"] == "port" and cpu["cores"] == 2
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"],
                           "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert line["numpy_1core"]["cores"] == 1 and line["numpy_1core"]["value"] > 0
    assert "TSTEPS=100" in line["config"]["workload"]


def test_reference_arm_prints_once_under_torchrun():
    out = _run(["-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                "--master-addr", "127.0.0.1", "--master-port", "29631", "bench.py", "--impl",
                "reference", "--gpus", "2", "--steps", "1", "--warmup", "0"],
               env={"OMP_NUM_THREADS": "2"})
    lines = _lines(out)
    assert len(lines) == 1 and lines[0]["impl"] == "reference" and lines[0]["n_gpus"] == 2


def test_compute_roofline_from_committed_instruction_mix():
    """The arithmetic roof of the headline kernel: the committed ncu instruction counts per
    update against given pipe rates; the tightest pipe is the bound."""
    import bench
    rates = {"lop3": 2.0e13, "dadd": 5.26e11, "imad": 2.0e13, "issue_slots": 4.03e13}
    rec = bench._ncu_record("heat3d_f64_256")["inst_per_update"]
    r = bench.compute_roofline("heat3d_f64_256", 1.3e11, rates)
    limits = r["per_pipe_ceiling_updates_per_s"]
    assert limits["alu"] == pytest.approx(2.0e13 / rec["alu"])
    assert limits["fp64"] == pytest.approx(5.26e11 / rec["fp64"])
    assert limits["issue"] == pytest.approx(4.03e13 / rec["issue"])
    assert r["ceiling_updates_per_s"] == min(limits.values())
    assert r["bound"] == min(limits, key=limits.get)
    assert r["frac"] == pytest.approx(1.3e11 / r["ceiling_updates_per_s"])
    assert bench.compute_roofline("no_such_kernel", 1.0, rates) is None


@pytest.mark.gpu
def test_default_run_line():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    (line,) = _lines(_run(["bench.py", "--steps", "2", "--warmup", "3", "--no-fp32",
                           "--no-cpu-baseline"]))
    assert BASE_KEYS <= set(line) and "impl" not in line
    assert line["n_gpus"] == 1 and line["steps"] == 2 and line["warmup"] == 3
    roof = line["roofline"]
    assert roof["bound"] == "hbm" and roof["unit"] == "GB/s" and roof["peak"] > 0
    assert roof["frac"] == pytest.approx(roof["achieved"] / roof["peak"])
    assert line["fp64_roofline"]["frac"] > 0
    e2e = line["e2e"]
    assert e2e["value"] > 0 and e2e["h2d_bytes_per_step"] == 2 * 8 * 256 ** 3
    assert e2e["d2h_bytes_per_step"] == 2 * 8 * 256 ** 3
    assert line["gpu_launches"] == 2 * 198
    assert "sm_mhz" in line["clocks"] and "reasons" in line["clocks"]


@pytest.mark.gpu
def test_batch_and_serve_blocks():
    """The default line's configuration 4 and 5 blocks, on a few grids and requests."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import bench
    b = bench.batch_measure(n_grids=48, steps=1, warmup=1, compare_steps=1, compare_warmup=0)
    assert b["value"] > 0 and b["per_grid"]["value"] > 0
    assert b["batched_over_per_grid"] == pytest.approx(b["per_grid"]["ms_per_step"] /
                                                       b["ms_per_step"])
    err = b["fp32_error_vs_fp64"]
    assert err["grids"] == 24 and 0 < err["rel_l2_max"] < 1e-3
    assert sum(v["grids"] for v in err["by_tsteps"].values()) == 24
    s = bench.serve_measure(rates=(2000.0,), n_requests=6)
    (e,) = s["rates"]
    assert e["served"]["updates_per_s"] > 0 and e["sequential"]["updates_per_s"] > 0
    assert e["served"]["p50_ms"] <= e["served"]["p99_ms"]
    assert s["fp32_error_vs_fp64"]["grids"] >= 1
