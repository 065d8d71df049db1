"""Measured throughput of GB300's arithmetic pipes (libnpbgb's ``npbgb_probe_pipe``).

    python -m npbench_gb300.pipes          # prints the rates as JSON

The binary64 stencils are bound by arithmetic issue, not by HBM: GB300's
binary64 pipe retires far fewer operations per clock than its binary32 and
integer pipes.  ``measure()`` times each probe kernel (independent dependency
chains of one instruction kind, every SM filled) with CUDA events and returns
operations per second for the whole GPU; these are the compute roofs the
binary64 kernels are stated against (``compute_roofline`` in bench.py).
"""
import json

from . import _lib

__all__ = ["OPS", "measure"]

OPS = {"dadd": 0, "dmul": 1, "dfma": 2, "ffma": 3, "lop3": 4, "iadd": 5, "imad": 6}


def measure(ops=tuple(OPS), target_ms=5.0, ctas_per_sm=8, repeats=3):
    """{op: operations per second} on the current CUDA device (best of `repeats`)."""
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    ctas = sms * ctas_per_sm
    threads = ctas * 256
    sink = torch.empty(threads, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    lib = _lib.load()
    out = {}
    for name in ops:
        op = OPS[name]
        iters = 256
        best = None
        for attempt in range(8):
            times = []
            for _ in range(max(1, repeats) + 1):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                _lib.check(lib.npbgb_probe_pipe(op, iters, ctas, sink.data_ptr(),
                                                stream.cuda_stream), "npbgb_probe_pipe")
                e1.record(stream)
                e1.synchronize()
                times.append(e0.elapsed_time(e1))
            best = min(times[1:])
            if best >= target_ms:
                break
            iters = int(iters * max(2.0, target_ms / max(best, 1e-3)))
        out[name] = threads * 8 * iters / (best * 1e-3)
    return out


def main():
    rates = measure()
    print(json.dumps({k: float(f"{v:.4g}") for k, v in rates.items()}))


if __name__ == "__main__":
    main()
