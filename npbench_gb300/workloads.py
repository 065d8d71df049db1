"""Synthetic inputs for the stencil path: the reference's initializers and seeded U[0,1) grids.

* ``init_jacobi_2d(N, dtype)`` restates polybench/jacobi_2d/jacobi_2d.py:6-10:
  ``A = i*(j+2)/N``, ``B = i*(j+3)/N`` evaluated in ``dtype``.
* ``init_heat_3d(N, dtype)`` restates polybench/heat_3d/heat_3d.py:6-11:
  ``A = (i+j+(N-k))*10/N``, ``B = copy(A)``.
* ``init_hdiff(I, J, K)`` restates weather_stencils/hdiff/hdiff.py:6-15:
  ``default_rng(42)`` draws ``in_field (I+4,J+4,K)``, ``out_field (I,J,K)``,
  ``coeff (I,J,K)`` in that order.
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
}


def init_jacobi_2d(N, dtype=np.float64):
    A = np.fromfunction(lambda i, j: i * (j + 2) / N, (N, N), dtype=dtype)
    B = np.fromfunction(lambda i, j: i * (j + 3) / N, (N, N), dtype=dtype)
    return A, B


def init_heat_3d(N, dtype=np.float64):
    A = np.fromfunction(lambda i, j, k: (i + j + (N - k)) * 10 / N, (N, N, N), dtype=dtype)
    return A, np.copy(A)


def init_hdiff(I, J, K):
    rng = np.random.default_rng(42)
    in_field = rng.random((I + 4, J + 4, K))
    out_field = rng.random((I, J, K))
    coeff = rng.random((I, J, K))
    return in_field, out_field, coeff


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
