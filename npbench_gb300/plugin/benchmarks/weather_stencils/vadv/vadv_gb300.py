# NPBench implementation file for the gb300 framework: vertical advection
# (vadv_numpy.py), run by libnpbgb's sm_103a kernel on CUDA tensors.
from npbench_gb300.stencils import vadv as _vadv


def vadv(utens_stage, u_stage, wcon, u_pos, utens, dtr_stage):
    _vadv(utens_stage, u_stage, wcon, u_pos, utens, dtr_stage)
