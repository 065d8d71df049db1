# NPBench implementation file for the gb300 framework: lid-driven cavity flow
# (cavity_flow_numpy.py), the whole time loop in one persistent sm_103a launch.
from npbench_gb300.stencils import cavity_flow as _cavity_flow


def cavity_flow(nx, ny, nt, nit, u, v, dt, dx, dy, p, rho, nu):
    _cavity_flow(nx, ny, nt, nit, u, v, dt, dx, dy, p, rho, nu)
