# NPBench framework plugin for npbench_gb300 (GB300, sm_103a).
#
# Installed as npbench/infrastructure/gb300_framework.py next to the other
# plugins, with `from .gb300_framework import *` in
# npbench/infrastructure/__init__.py and framework_info/gb300.json.  It follows
# the Framework interface of npbench/infrastructure/framework.py:12-162:
#
# * copy_func moves each array argument to the current CUDA device as a
#   torch.Tensor in the untimed setup (the device crossing the CuPy and APPy
#   plugins also do there, cupy_framework.py:26-30, appy_framework.py:28-34);
# * setup_str and exec_str end with torch.cuda.synchronize(), so the timed
#   statement covers the kernels and nothing queued before them
#   (cupy_framework.py:32-58);
# * copy_back_func brings validated outputs back as NumPy arrays;
# * version() reports the library instead of asking pkg_resources, which does
#   not know this framework's name (framework.py:33-35).
from typing import Any, Callable, Dict

from npbench.infrastructure import Benchmark, Framework

__all__ = ["GB300Framework"]


class GB300Framework(Framework):
    """Runs NPBench's stencil kernels on libnpbgb's hand-written sm_103a CUDA kernels."""

    def __init__(self, fname: str):
        super().__init__(fname)

    def version(self) -> str:
        import npbench_gb300
        return npbench_gb300.version()

    def imports(self) -> Dict[str, Any]:
        import torch
        import npbench_gb300
        npbench_gb300.load()  # fail here, loudly, if the CUDA library is missing
        return {"torch": torch}

    def copy_func(self) -> Callable:
        import numpy as np
        import torch

        def to_device(arr):
            if isinstance(arr, np.ndarray):
                return torch.from_numpy(np.ascontiguousarray(arr)).to("cuda")
            return arr
        return to_device

    def copy_back_func(self) -> Callable:
        def to_host(x):
            if type(x).__module__.startswith("torch"):
                return x.cpu().numpy()
            return x
        return to_host

    def setup_str(self, bench: Benchmark, impl: Callable = None) -> str:
        sync = "torch.cuda.synchronize()"
        if len(bench.info["array_args"]):
            copies = ", ".join("__npb_copy({})".format(a) for a in bench.info["array_args"])
            return self.out_arg_str(bench, impl) + " = " + copies + "; " + sync
        return sync

    def exec_str(self, bench: Benchmark, impl: Callable = None) -> str:
        call = "__npb_result = __npb_impl({a})".format(a=self.arg_str(bench, impl))
        return call + "; torch.cuda.synchronize()"
