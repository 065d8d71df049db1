"""Synthetic inputs for the stencil path: the reference's initializers and seeded U[0,1) grids.

* ``init_jacobi_2d(N, dtype)`` restates polybench/jacobi_2d/jacobi_2d.py:6-10:
  ``A = i*(j+2)/N``, ``B = i*(j+3)/N`` evaluated in ``dtype``.
* ``init_heat_3d(N, dtype)`` restates polybench/heat_3d/heat_3d.py:6-11:
  ``A = (i+j+(N-k))*10/N``, ``B = copy(A)``.
* ``init_hdiff(I, J, K)`` restates weather_stencils/hdiff/hdiff.py:6-15:
  ``default_rng(42)`` draws ``in_field (I+4,J+4,K)``, ``out_field (I,J,K)``,
  ``coeff (I,J,K)`` in that order.
* ``init_vadv(I, J, K)`` restates weather_stencils/vadv/vadv.py:6-19:
  ``dtr_stage = 3/20`` and ``default_rng(42)`` draws ``utens_stage``,
  ``u_stage``, ``wcon (I+1,J,K)``, ``u_pos``, ``utens`` in that order.
* ``init_cavity_flow(ny, nx)`` restates cavity_flow/cavity_flow.py:6-13:
  zero u, v, p and ``dx = 2/(nx-1)``, ``dy = 2/(ny-1)``,
  ``dt = .1/((nx-1)*(ny-1))``.
* ``init_channel_flow(ny, nx)`` restates channel_flow/channel_flow.py:6-13
  (as cavity_flow's, but p = 1).
* ``uniform_pair`` / ``uniform_heat`` draw U[0,1) fields from
  ``numpy.random.default_rng(seed)`` (float32 forms are casts of the float64
  draw, so both precisions see the same field).
"""
import numpy as np

PRESETS = {
    "jacobi_2d": {"S": {"TSTEPS": 50, "N": 150}, "M": {"TSTEPS": 80, "N": 350},
                  "L": {"TSTEPS": 200, "N": 700}, "paper": {"TSTEPS": 1000, "N": 2800}},
    "heat_3d": {"S": {"TSTEPS": 25, "N": 25}, "M": {"TSTEPS": 50, "N": 40},
                "L": {"TSTEPS": 100, "N": 70}, "paper": {"TSTEPS": 500, "N": 120}},
    "hdiff": {"S": {"I": 64, "J": 64, "K": 60}, "M": {"I": 128, "J": 128, "K": 160},
              "L": {"I": 384, "J": 384, "K": 160}, "paper": {"I": 256, "J": 256, "K": 160}},
    "jacobi_1d": {"S": {"TSTEPS": 800, "N": 3200}, "M": {"TSTEPS": 3000, "N": 12000},
                  "L": {"TSTEPS": 8500, "N": 34000}, "paper": {"TSTEPS": 4000, "N": 32000}},
    "cavity_flow": {"S": {"ny": 61, "nx": 61, "nt": 25, "nit": 5, "rho": 1.0, "nu": 0.1},
                    "M": {"ny": 121, "nx": 121, "nt": 50, "nit": 10, "rho": 1.0, "nu": 0.1},
                    "L": {"ny": 201, "nx": 201, "nt": 100, "nit": 20, "rho": 1.0, "nu": 0.1},
                    "paper": {"ny": 101, "nx": 101, "nt": 700, "nit": 50, "rho": 1.0,
                              "nu": 0.1}},
    "channel_flow": {"S": {"ny": 61, "nx": 61, "nit": 5, "rho": 1.0, "nu": 0.1, "F": 1.0},
                     "M": {"ny": 121, "nx": 121, "nit": 10, "rho": 1.0, "nu": 0.1, "F": 1.0},
                     "L": {"ny": 201, "nx": 201, "nit": 20, "rho": 1.0, "nu": 0.1, "F": 1.0},
                     "paper": {"ny": 101, "nx": 101, "nit": 50, "rho": 1.0, "nu": 0.1,
                               "F": 1.0}},
    "vadv": {"S": {"I": 60, "J": 60, "K": 40}, "M": {"I": 112, "J": 112, "K": 80},
             "L": {"I": 180, "J": 180, "K": 160}, "paper": {"I": 256, "J": 256, "K": 160}},
    "fdtd_2d": {"S": {"TMAX": 20, "NX": 200, "NY": 220}, "M": {"TMAX": 60, "NX": 400, "NY": 450},
                "L": {"TMAX": 150, "NX": 800, "NY": 900},
                "paper": {"TMAX": 500, "NX": 1000, "NY": 1200}},
}


def init_jacobi_2d(N, dtype=np.float64):
    A = np.fromfunction(lambda i, j: i * (j + 2) / N, (N, N), dtype=dtype)
    B = np.fromfunction(lambda i, j: i * (j + 3) / N, (N, N), dtype=dtype)
    return A, B


def init_heat_3d(N, dtype=np.float64):
    A = np.fromfunction(lambda i, j, k: (i + j + (N - k)) * 10 / N, (N, N, N), dtype=dtype)
    return A, np.copy(A)


def init_jacobi_1d(N, dtype=np.float64):
    """polybench/jacobi_1d/jacobi_1d.py:6-10: A = (i+2)/N, B = (i+3)/N."""
    A = np.fromfunction(lambda i: (i + 2) / N, (N,), dtype=dtype)
    B = np.fromfunction(lambda i: (i + 3) / N, (N,), dtype=dtype)
    return A, B


def init_fdtd_2d(TMAX, NX, NY, dtype=np.float64):
    """polybench/fdtd_2d/fdtd_2d.py:6-17: ex = i(j+1)/NX, ey = i(j+2)/NY,
    hz = i(j+3)/NX, _fict_ = i."""
    ex = np.fromfunction(lambda i, j: (i * (j + 1)) / NX, (NX, NY), dtype=dtype)
    ey = np.fromfunction(lambda i, j: (i * (j + 2)) / NY, (NX, NY), dtype=dtype)
    hz = np.fromfunction(lambda i, j: (i * (j + 3)) / NX, (NX, NY), dtype=dtype)
    fict = np.fromfunction(lambda i: i, (TMAX,), dtype=dtype)
    return ex, ey, hz, fict


def init_hdiff(I, J, K):
    rng = np.random.default_rng(42)
    in_field = rng.random((I + 4, J + 4, K))
    out_field = rng.random((I, J, K))
    coeff = rng.random((I, J, K))
    return in_field, out_field, coeff


def init_vadv(I, J, K):
    """Returns (dtr_stage, utens_stage, u_stage, wcon, u_pos, utens)."""
    rng = np.random.default_rng(42)
    dtr_stage = 3. / 20.
    utens_stage = rng.random((I, J, K))
    u_stage = rng.random((I, J, K))
    wcon = rng.random((I + 1, J, K))
    u_pos = rng.random((I, J, K))
    utens = rng.random((I, J, K))
    return dtr_stage, utens_stage, u_stage, wcon, u_pos, utens


def init_cavity_flow(ny, nx):
    """Returns (u, v, p, dx, dy, dt)."""
    u = np.zeros((ny, nx), dtype=np.float64)
    v = np.zeros((ny, nx), dtype=np.float64)
    p = np.zeros((ny, nx), dtype=np.float64)
    dx = 2 / (nx - 1)
    dy = 2 / (ny - 1)
    dt = .1 / ((nx - 1) * (ny - 1))
    return u, v, p, dx, dy, dt


def init_channel_flow(ny, nx):
    """channel_flow/channel_flow.py:6-13: u = v = 0, p = 1; returns (u, v, p, dx, dy, dt)."""
    u = np.zeros((ny, nx), dtype=np.float64)
    v = np.zeros((ny, nx), dtype=np.float64)
    p = np.ones((ny, nx), dtype=np.float64)
    dx = 2 / (nx - 1)
    dy = 2 / (ny - 1)
    dt = .1 / ((nx - 1) * (ny - 1))
    return u, v, p, dx, dy, dt


def uniform_pair(shape, dtype=np.float64, seed=0):
    """Jacobi-2D inputs: A and B independent U[0,1) draws."""
    rng = np.random.default_rng(seed)
    A = rng.random(shape)
    B = rng.random(shape)
    return A.astype(dtype, copy=False), B.astype(dtype, copy=False)


def uniform_heat(shape, dtype=np.float64, seed=0):
    """Heat-3D inputs: A a U[0,1) draw, B a copy of A."""
    rng = np.random.default_rng(seed)
    A = rng.random(shape).astype(dtype, copy=False)
    return A, A.copy()


def uniform_hdiff(I, J, K, seed=0):
    rng = np.random.default_rng(seed)
    return rng.random((I + 4, J + 4, K)), rng.random((I, J, K)), rng.random((I, J, K))


def batch_jacobi_specs(n_grids=4096, seed=0, side=(64, 2048), tsteps=(10, 500)):
    """Batched Jacobi-2D configuration: per grid (shape, dtype, TSTEPS).

    Side lengths are drawn log-uniform in [side[0], side[1]] per axis (non-square),
    half the grids float32 and half float64 (alternating), TSTEPS uniform in
    [tsteps[0], tsteps[1]].
    """
    rng = np.random.default_rng(seed)
    lo, hi = np.log(side[0]), np.log(side[1])
    shapes = np.exp(rng.uniform(lo, hi, size=(n_grids, 2))).round().astype(np.int64)
    steps = rng.integers(tsteps[0], tsteps[1] + 1, size=n_grids)
    return [((int(s[0]), int(s[1])), np.float32 if g % 2 else np.float64, int(t))
            for g, (s, t) in enumerate(zip(shapes, steps))]


def served_requests(n, rate_hz, seed=0, side2d=(128, 4096), side3d=(32, 384),
                    tsteps=(20, 1000), f32_share=0.7):
    """Served-stream configuration: Poisson arrivals and mixed solves.

    Returns (arrival_offsets_s, [(shape, dtype, TSTEPS, data_seed)]): half the
    requests 2D Jacobi with sides log-uniform in side2d, half 3D heat with
    sides log-uniform in side3d, 70% float32 / 30% float64, TSTEPS uniform in
    tsteps, inter-arrival times exponential with mean 1/rate_hz.
    """
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate_hz, size=n))
    out = []
    for i in range(n):
        if rng.random() < 0.5:
            lo, hi = np.log(side2d[0]), np.log(side2d[1])
            shape = tuple(int(x) for x in np.exp(rng.uniform(lo, hi, 2)).round())
        else:
            lo, hi = np.log(side3d[0]), np.log(side3d[1])
            shape = tuple(int(x) for x in np.exp(rng.uniform(lo, hi, 3)).round())
        dt = np.float32 if rng.random() < f32_share else np.float64
        out.append((shape, dt, int(rng.integers(tsteps[0], tsteps[1] + 1)), int(rng.integers(1 << 31))))
    return arrivals, out
