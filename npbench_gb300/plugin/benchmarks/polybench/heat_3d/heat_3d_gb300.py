# NPBench implementation file for the gb300 framework: the Heat-3D time loop
# of heat_3d_numpy.py, run by libnpbgb's sm_103a kernels on CUDA tensors.
from npbench_gb300.stencils import heat_3d_kernel


def kernel(TSTEPS, A, B):
    heat_3d_kernel(TSTEPS, A, B)
