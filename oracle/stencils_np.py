"""NumPy restatement of NPBench's stencil kernels -- TEST INFRASTRUCTURE ONLY.

Each function evaluates the same IEEE operations, in the same order, as the
reference kernel it cites, so that its result is bit-identical to the
reference's for any input.  Scalars follow NumPy's promotion rules: for float32
arrays the constants 0.2, 2.0, 0.125 and 4.0 are applied as float32 (NEP 50;
NumPy 1.x value-based casting gives the same), for float64 arrays as float64.

Evaluation orders restated here:

* Jacobi-2D, polybench/jacobi_2d/jacobi_2d_numpy.py:6-10 --
  ``dst = 0.2 * ((((c + w) + e) + s) + n)`` where ``w/e`` are the column
  neighbours ``j-1/j+1`` and ``s/n`` the row neighbours ``i+1/i-1``; one
  iteration is a half-sweep A->B followed by B->A, and ``kernel(T, A, B)``
  runs ``T-1`` iterations.
* Heat-3D, polybench/heat_3d/heat_3d_numpy.py:6-20 --
  ``dst = ((ti + tj) + tk) + c`` with
  ``tx = 0.125 * ((next_x - 2.0 * c) + prev_x)``.
* hdiff, weather_stencils/hdiff/hdiff_numpy.py:5-29 -- see ``hdiff``.
* vadv, weather_stencils/vadv/vadv_numpy.py:9-78 -- see ``vadv``.
"""
import numpy as np

__all__ = ["jacobi_2d_kernel", "heat_3d_kernel", "hdiff", "jacobi_2d_half_sweep",
           "heat_3d_half_sweep", "jacobi_1d_kernel", "fdtd_2d_kernel", "vadv"]


def jacobi_2d_half_sweep(src, dst):
    """One Jacobi-2D update of the interior of ``dst`` from ``src``.

    Follows polybench/jacobi_2d/jacobi_2d_numpy.py:7-8 operator by operator.
    """
    k = src.dtype.type(0.2)
    centre = src[1:-1, 1:-1]
    west, east = src[1:-1, :-2], src[1:-1, 2:]
    south, north = src[2:, 1:-1], src[:-2, 1:-1]
    acc = np.add(centre, west)
    np.add(acc, east, out=acc)
    np.add(acc, south, out=acc)
    np.add(acc, north, out=acc)
    np.multiply(k, acc, out=dst[1:-1, 1:-1])


def jacobi_2d_kernel(TSTEPS, A, B):
    """``kernel(TSTEPS, A, B)`` of polybench/jacobi_2d/jacobi_2d_numpy.py:4-10.

    In place: after the call A holds the newest field and B the one before.
    """
    for _ in range(1, TSTEPS):
        jacobi_2d_half_sweep(A, B)
        jacobi_2d_half_sweep(B, A)


def _heat_axis_term(nxt, ctr, prv, two, eighth):
    # 0.125 * ((next - 2.0 * centre) + prev), heat_3d_numpy.py:8-13
    t = np.multiply(two, ctr)
    np.subtract(nxt, t, out=t)
    np.add(t, prv, out=t)
    np.multiply(eighth, t, out=t)
    return t


def heat_3d_half_sweep(src, dst):
    """One Heat-3D update of the interior of ``dst`` from ``src``.

    Follows polybench/heat_3d/heat_3d_numpy.py:7-13 operator by operator.
    """
    two, eighth = src.dtype.type(2.0), src.dtype.type(0.125)
    c = src[1:-1, 1:-1, 1:-1]
    ti = _heat_axis_term(src[2:, 1:-1, 1:-1], c, src[:-2, 1:-1, 1:-1], two, eighth)
    tj = _heat_axis_term(src[1:-1, 2:, 1:-1], c, src[1:-1, :-2, 1:-1], two, eighth)
    tk = _heat_axis_term(src[1:-1, 1:-1, 2:], c, src[1:-1, 1:-1, :-2], two, eighth)
    np.add(ti, tj, out=ti)
    np.add(ti, tk, out=ti)
    np.add(ti, c, out=dst[1:-1, 1:-1, 1:-1])


def heat_3d_kernel(TSTEPS, A, B):
    """``kernel(TSTEPS, A, B)`` of polybench/heat_3d/heat_3d_numpy.py:4-20."""
    for _ in range(1, TSTEPS):
        heat_3d_half_sweep(A, B)
        heat_3d_half_sweep(B, A)


def hdiff(in_field, out_field, coeff):
    """``hdiff(in_field, out_field, coeff)`` of weather_stencils/hdiff/hdiff_numpy.py:5-29.

    ``in_field`` is (I+4, J+4, K) with a halo of two in I and J; ``out_field``
    and ``coeff`` are (I, J, K).  K is the contiguous axis.  Steps:

    * Laplacian on the (I+2, J+2) ring-1 region (hdiff_numpy.py:7-9):
      ``lap = 4*c - (((in[i+1] + in[i-1]) + in[j+1]) + in[j-1])``.
    * x-flux (hdiff_numpy.py:11-17): ``res = lap[i+1] - lap[i]`` over
      (I+1, J), replaced by +0.0 where ``res * (in[i+1] - in[i]) > 0``.
    * y-flux (hdiff_numpy.py:19-25): the same along j over (I, J+1).
    * update (hdiff_numpy.py:27-29):
      ``out = c - coeff * (((flx[i] - flx[i-1]) + fly[j]) - fly[j-1])``.
    """
    I, J, K = out_field.shape
    f = in_field
    four = f.dtype.type(4.0)
    lap = np.multiply(four, f[1:I + 3, 1:J + 3, :])
    nb = np.add(f[2:I + 4, 1:J + 3, :], f[0:I + 2, 1:J + 3, :])
    np.add(nb, f[1:I + 3, 2:J + 4, :], out=nb)
    np.add(nb, f[1:I + 3, 0:J + 2, :], out=nb)
    np.subtract(lap, nb, out=lap)

    res = np.subtract(lap[1:, 1:J + 1, :], lap[:-1, 1:J + 1, :])
    grad = np.subtract(f[2:I + 3, 2:J + 2, :], f[1:I + 2, 2:J + 2, :])
    flx = np.where(np.multiply(res, grad) > 0, 0, res)

    res = np.subtract(lap[1:I + 1, 1:, :], lap[1:I + 1, :-1, :])
    grad = np.subtract(f[2:I + 2, 2:J + 3, :], f[2:I + 2, 1:J + 2, :])
    fly = np.where(np.multiply(res, grad) > 0, 0, res)

    div = np.subtract(flx[1:, :, :], flx[:-1, :, :])
    np.add(div, fly[:, 1:, :], out=div)
    np.subtract(div, fly[:, :-1, :], out=div)
    np.multiply(coeff, div, out=div)
    np.subtract(f[2:I + 2, 2:J + 2, :], div, out=out_field)


def jacobi_1d_kernel(TSTEPS, A, B):
    """``kernel(TSTEPS, A, B)`` of polybench/jacobi_1d/jacobi_1d_numpy.py:4-8.

    dst[1:-1] = 0.33333 * ((src[:-2] + src[1:-1]) + src[2:]), A->B then B->A.
    """
    k = A.dtype.type(0.33333)

    def half(src, dst):
        acc = np.add(src[:-2], src[1:-1])
        np.add(acc, src[2:], out=acc)
        np.multiply(k, acc, out=dst[1:-1])

    for _ in range(1, TSTEPS):
        half(A, B)
        half(B, A)


def fdtd_2d_kernel(TMAX, ex, ey, hz, _fict_):
    """``kernel(TMAX, ex, ey, hz, _fict_)`` of polybench/fdtd_2d/fdtd_2d_numpy.py:4-11.

    Per step, in place and in this order: ey[0,:] = fict[t];
    ey[1:,:] -= 0.5 * (hz[1:,:] - hz[:-1,:]); ex[:,1:] -= 0.5 * (hz[:,1:] - hz[:,:-1]);
    hz[:-1,:-1] -= 0.7 * (((ex[:-1,1:] - ex[:-1,:-1]) + ey[1:,:-1]) - ey[:-1,:-1]).
    """
    half, c07 = ex.dtype.type(0.5), ex.dtype.type(0.7)
    for t in range(TMAX):
        ey[0, :] = _fict_[t]
        d = np.subtract(hz[1:, :], hz[:-1, :])
        np.multiply(half, d, out=d)
        np.subtract(ey[1:, :], d, out=ey[1:, :])
        d = np.subtract(hz[:, 1:], hz[:, :-1])
        np.multiply(half, d, out=d)
        np.subtract(ex[:, 1:], d, out=ex[:, 1:])
        d = np.subtract(ex[:-1, 1:], ex[:-1, :-1])
        np.add(d, ey[1:, :-1], out=d)
        np.subtract(d, ey[:-1, :-1], out=d)
        np.multiply(c07, d, out=d)
        np.subtract(hz[:-1, :-1], d, out=hz[:-1, :-1])


def vadv(utens_stage, u_stage, wcon, u_pos, utens, dtr_stage):
    """``vadv(utens_stage, u_stage, wcon, u_pos, utens, dtr_stage)`` of
    weather_stencils/vadv/vadv_numpy.py:9-78 (float64; K contiguous).

    A tridiagonal (Thomas) solve along K for every (i, j) column, written into
    ``utens_stage``.  With ``w_k = wcon[i+1, j, k] + wcon[i, j, k]`` the
    reference forms ``gcv = 0.25*w_{k+1}``, ``gav = -0.25*w_k`` and their
    halves (BET_M = BET_P = 0.5), then per level k, in this order:

    * ``bcol = (dtr - acol) - ccol_k`` (no ``acol`` at k = 0, no ``ccol_k`` at
      k = K-1);
    * ``corr = (-as)*(u[k-1] - u[k]) - cs*(u[k+1] - u[k])`` (one-sided at the
      ends);
    * ``dcol_k = ((dtr*u_pos[k] + utens[k]) + utens_stage[k]) + corr``;
    * ``divided = 1.0 / (bcol - ccol_{k-1}*acol)``; ``ccol_k *= divided``;
      ``dcol_k = (dcol_k - dcol_{k-1}*acol) * divided``;

    then back substitution ``data = dcol_k - ccol_k*data`` from K-2 down to 0
    (``data = dcol_{K-1}`` at the top) with
    ``utens_stage[k] = dtr*(data - u_pos[k])``.  K < 2 raises IndexError, as
    the reference does (it reads level 1 unconditionally).
    """
    I, J, K = utens_stage.shape
    if K < 2:
        raise IndexError(f"vadv needs K >= 2 (reads level 1), got K={K}")
    dtr = float(dtr_stage)
    ccol = np.empty((I, J, K))
    dcol = np.empty((I, J, K))

    def wsum(k):
        return np.add(wcon[1:, :, k], wcon[:-1, :, k])

    def dfirst(k, corr):
        d = np.multiply(dtr, u_pos[:, :, k])
        np.add(d, utens[:, :, k], out=d)
        np.add(d, utens_stage[:, :, k], out=d)
        np.add(d, corr, out=d)
        return d

    for k in range(K):
        if k + 1 < K:
            gcv = np.multiply(0.25, wsum(k + 1))
            cs = np.multiply(gcv, 0.5)
            ccol[:, :, k] = np.multiply(gcv, 0.5)
        if k > 0:
            gav = np.multiply(-0.25, wsum(k))
            as_ = np.multiply(gav, 0.5)
            acol = np.multiply(gav, 0.5)
        # bcol and the correction term
        if k == 0:
            bcol = np.subtract(dtr, ccol[:, :, k])
            corr = np.multiply(np.negative(cs), np.subtract(u_stage[:, :, 1], u_stage[:, :, 0]))
        elif k < K - 1:
            bcol = np.subtract(np.subtract(dtr, acol), ccol[:, :, k])
            lo = np.multiply(np.negative(as_), np.subtract(u_stage[:, :, k - 1], u_stage[:, :, k]))
            hi = np.multiply(cs, np.subtract(u_stage[:, :, k + 1], u_stage[:, :, k]))
            corr = np.subtract(lo, hi)
        else:
            bcol = np.subtract(dtr, acol)
            corr = np.multiply(np.negative(as_), np.subtract(u_stage[:, :, k - 1], u_stage[:, :, k]))
        dcol[:, :, k] = dfirst(k, corr)
        # forward elimination
        if k == 0:
            divided = np.divide(1.0, bcol)
            np.multiply(ccol[:, :, k], divided, out=ccol[:, :, k])
            np.multiply(dcol[:, :, k], divided, out=dcol[:, :, k])
        else:
            divided = np.divide(1.0, np.subtract(bcol, np.multiply(ccol[:, :, k - 1], acol)))
            if k < K - 1:
                np.multiply(ccol[:, :, k], divided, out=ccol[:, :, k])
            t = np.subtract(dcol[:, :, k], np.multiply(dcol[:, :, k - 1], acol))
            np.multiply(t, divided, out=dcol[:, :, k])

    data = dcol[:, :, K - 1].copy()
    utens_stage[:, :, K - 1] = np.multiply(dtr, np.subtract(data, u_pos[:, :, K - 1]))
    for k in range(K - 2, -1, -1):
        data = np.subtract(dcol[:, :, k], np.multiply(ccol[:, :, k], data))
        utens_stage[:, :, k] = np.multiply(dtr, np.subtract(data, u_pos[:, :, k]))
