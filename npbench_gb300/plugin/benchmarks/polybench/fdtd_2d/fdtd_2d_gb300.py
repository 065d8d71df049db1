# NPBench implementation file for the gb300 framework: the FDTD-2D time loop
# of fdtd_2d_numpy.py, run by libnpbgb's sm_103a kernels on CUDA tensors.
from npbench_gb300.stencils import fdtd_2d_kernel


def kernel(TMAX, ex, ey, hz, _fict_):
    fdtd_2d_kernel(TMAX, ex, ey, hz, _fict_)
