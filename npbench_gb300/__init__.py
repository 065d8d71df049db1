"""npbench_gb300 -- GB300-native (sm_103a) structured-grid stencil time-stepping.

A drop-in for NPBench's stencil kernels (Jacobi-2D, Heat-3D, hdiff, and
Jacobi-1D, FDTD-2D, vadv, cavity_flow and channel_flow beside them): the
functions in ``npbench_gb300.stencils`` keep the reference NumPy signatures
and run hand-written CUDA kernels from ``libnpbgb.so`` through its C ABI
(``include/npbgb.h``).  ``npbench_gb300.plugin`` holds the NPBench framework
plugin (``framework_info`` JSON, ``Framework`` subclass, kernel modules).
"""
from ._lib import NpbgbError, load, version  # noqa: F401
from .stencils import (fdtd_2d_kernel, hdiff, heat_3d_kernel, jacobi_1d_kernel,  # noqa: F401
                       jacobi_2d_kernel, vadv, cavity_flow, channel_flow)

__all__ = ["NpbgbError", "load", "version", "jacobi_2d_kernel", "heat_3d_kernel", "hdiff",
           "jacobi_1d_kernel", "fdtd_2d_kernel", "vadv", "cavity_flow", "channel_flow"]
