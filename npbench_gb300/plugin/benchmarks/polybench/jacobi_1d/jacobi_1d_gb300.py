# NPBench implementation file for the gb300 framework: the Jacobi-1D time loop
# of jacobi_1d_numpy.py, run by libnpbgb's sm_103a kernels on CUDA tensors.
from npbench_gb300.stencils import jacobi_1d_kernel


def kernel(TSTEPS, A, B):
    jacobi_1d_kernel(TSTEPS, A, B)
