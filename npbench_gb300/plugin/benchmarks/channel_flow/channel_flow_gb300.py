# NPBench implementation file for the gb300 framework: channel flow
# (channel_flow_numpy.py), the whole convergence loop in one persistent
# sm_103a launch; returns the step count as the reference does.
from npbench_gb300.stencils import channel_flow as _channel_flow


def channel_flow(nit, u, v, dt, dx, dy, p, rho, nu, F):
    return _channel_flow(nit, u, v, dt, dx, dy, p, rho, nu, F)
