"""When float32 storage is accurate enough: the error model behind the float64 guard.

A float32 run of ``kernel(TSTEPS, A, B)`` (polybench/jacobi_2d/jacobi_2d_numpy.py:4-10,
polybench/heat_3d/heat_3d_numpy.py:4-20) rounds every operator to float32, so
its result drifts from the float64 run of the same inputs as TSTEPS grows.
NPBench accepts a result whose relative L2 error against the reference is at
most 1e-5 (npbench/infrastructure/utilities.py:154-180).  The batch and the
server keep a float32 request in float32 only while the error predicted for it
stays below that bound; above it the request runs in float64 on the GPU (its
float32 inputs widened exactly) and its result is rounded to float32 once at
the end.

The prediction comes from ``fp32_error_model.json``, measured on the GPU by
``python -m npbench_gb300.precision --calibrate``: for each kind and a range of
grid sizes, the relative L2 error of float32 against float64 runs of the same
U[0,1) inputs (the float32 inputs are the float64 draw rounded) at TSTEPS from
2 to 2000.  ``predicted_rel_l2`` takes the largest error over the calibrated
sizes at each calibrated TSTEPS, interpolates linearly in log-log between
them, and beyond the last calibrated TSTEPS carries the last segment's power
law on.  ``needs_fp64`` compares it, times a safety factor, with the bound.

Measured on GB300: Jacobi-2D grows about linearly, 4.5e-6 at TSTEPS=100 and
4.6e-5 at 1000, within 10% across grid sizes 128^2 to 4096^2 (the table keeps
the worst), so with a safety factor of 1.25 float32 Jacobi-2D runs above about
TSTEPS=175 run in float64; Heat-3D stays below 3.5e-6 up to TSTEPS=2000 and
always runs in float32.
"""
import argparse
import json
import math
import os

import numpy as np

__all__ = ["BOUND", "SAFETY", "model", "predicted_rel_l2", "needs_fp64", "calibrate"]

BOUND = 1e-5   # NPBench's relative L2 acceptance bound (utilities.py:154-180)
SAFETY = 1.25  # margin between the calibrated error (worst of five grid sizes) and the bound
MODEL_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "fp32_error_model.json")

_model = None


def model():
    """The calibrated table: {"jacobi2d": {"tsteps": [...], "rel_l2": [[per size] per T]}, ...}."""
    global _model
    if _model is None:
        with open(MODEL_PATH) as f:
            _model = json.load(f)
    return _model


def _kind(kind_or_shape):
    if isinstance(kind_or_shape, str):
        return kind_or_shape
    return "jacobi2d" if len(kind_or_shape) == 2 else "heat3d"


def predicted_rel_l2(kind, tsteps):
    """Predicted relative L2 error of a float32 run against float64 after TSTEPS."""
    if tsteps <= 1:
        return 0.0
    m = model()[_kind(kind)]
    ts = m["tsteps"]
    worst = [max(max(row), 1e-30) for row in m["rel_l2"]]
    if tsteps <= ts[0]:
        return float(worst[0])
    k = 1
    while k < len(ts) - 1 and tsteps > ts[k]:
        k += 1
    t0, t1, e0, e1 = ts[k - 1], ts[k], worst[k - 1], worst[k]
    slope = math.log(e1 / e0) / math.log(t1 / t0)
    if tsteps > t1:
        slope = max(0.0, slope)  # beyond the table: no decrease assumed
    return float(e0 * (tsteps / t0) ** slope)


def needs_fp64(kind, tsteps, bound=BOUND, safety=SAFETY):
    """True when a float32 run of this kind and TSTEPS may exceed the relative L2 bound."""
    return predicted_rel_l2(kind, tsteps) * safety > bound


def _rel_l2(low, ref):
    d = low.double() - ref
    n = float(ref.norm())
    return float(d.norm()) / n if n > 0 else 0.0


def calibrate(tsteps=(2, 5, 10, 20, 50, 100, 200, 500, 1000, 2000), seed=0):
    """Measures the float32 error table on the current CUDA device (a few seconds)."""
    import torch
    from . import stencils
    dev = torch.device("cuda", torch.cuda.current_device())
    sizes = {"jacobi2d": [(128, 128), (500, 300), (1000, 1000), (2048, 1536), (4096, 4096)],
             "heat3d": [(32, 32, 32), (64, 100, 80), (128, 128, 128), (256, 256, 256)]}
    out = {"what": "relative L2 error of float32 against float64 runs of the same U[0,1) "
                   "inputs (float32 inputs = the float64 draw rounded), per TSTEPS (rows) and "
                   "grid size (columns)",
           "bound": BOUND, "safety": SAFETY}
    for kind, shapes in sizes.items():
        fn = stencils.jacobi_2d_kernel if kind == "jacobi2d" else stencils.heat_3d_kernel
        table = []
        for T in tsteps:
            row = []
            for n, shape in enumerate(shapes):
                g = torch.Generator(device=dev)
                g.manual_seed(seed + n)
                a64 = torch.rand(shape, dtype=torch.float64, device=dev, generator=g)
                b64 = (torch.rand(shape, dtype=torch.float64, device=dev, generator=g)
                       if kind == "jacobi2d" else a64.clone())
                a32, b32 = a64.float(), b64.float()
                fn(T, a32, b32)
                fn(T, a64, b64)
                row.append(_rel_l2(a32, a64))
            table.append(row)
        out[kind] = {"shapes": [list(s) for s in shapes], "tsteps": list(tsteps), "rel_l2": table}
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__,
                                 formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--calibrate", action="store_true", help="measure on the GPU and write --out")
    ap.add_argument("--out", default=MODEL_PATH)
    a = ap.parse_args(argv)
    if a.calibrate:
        tab = calibrate()
        with open(a.out, "w") as f:
            json.dump(tab, f, indent=1)
        print(json.dumps({k: v for k, v in tab.items() if k in ("jacobi2d", "heat3d")}))
    else:
        for kind in ("jacobi2d", "heat3d"):
            for T in (10, 100, 500, 1000):
                print(kind, T, f"{predicted_rel_l2(kind, T):.3g}", needs_fp64(kind, T))


if __name__ == "__main__":
    main()
