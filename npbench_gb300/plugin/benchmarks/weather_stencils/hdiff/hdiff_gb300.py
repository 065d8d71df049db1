# NPBench implementation file for the gb300 framework: horizontal diffusion
# (hdiff_numpy.py), run by libnpbgb's sm_103a kernel on CUDA tensors.
from npbench_gb300.stencils import hdiff as _hdiff


def hdiff(in_field, out_field, coeff):
    _hdiff(in_field, out_field, coeff)
