# NPBench implementation file for the gb300 framework: the Jacobi-2D time loop
# of jacobi_2d_numpy.py, run by libnpbgb's sm_103a kernels on CUDA tensors.
from npbench_gb300.stencils import jacobi_2d_kernel


def kernel(TSTEPS, A, B):
    jacobi_2d_kernel(TSTEPS, A, B)
