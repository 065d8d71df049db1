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
* cavity_flow, cavity_flow/cavity_flow_numpy.py:13-82 -- see ``cavity_flow``.
* channel_flow, channel_flow/channel_flow_numpy.py:13-152 -- see ``channel_flow``.
"""
import numpy as np

__all__ = ["jacobi_2d_kernel", "heat_3d_kernel", "hdiff", "jacobi_2d_half_sweep",
           "heat_3d_half_sweep", "jacobi_1d_kernel", "fdtd_2d_kernel", "vadv",
           "cavity_flow", "cfd_constants", "channel_flow"]


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


def cfd_constants(dt, dx, dy, rho):
    """The scalars cavity_flow_numpy.py forms with Python float arithmetic.

    ``dx**2`` is Python's float power, i.e. the C library's ``pow(dx, 2.0)``,
    which is not always the correctly rounded ``dx*dx``; every user of these
    constants must take them from ``pow`` as well.
    """
    dx2, dy2 = dx ** 2, dy ** 2
    return {
        "two_dx": 2 * dx, "two_dy": 2 * dy, "inv_dt": 1 / dt,       # build_up_b, :15-21
        "dx2": dx2, "dy2": dy2,                                     # pressure_poisson, :30-33
        "pD": 2 * (dx2 + dy2), "pC": dx2 * dy2 / (2 * (dx2 + dy2)),
        "k1u": dt / (2 * rho * dx), "k1v": dt / (2 * rho * dy),     # the u/v updates, :53-74
        "k2": dt / dx2, "k3": dt / dy2,
    }


def cavity_flow(nx, ny, nt, nit, u, v, dt, dx, dy, p, rho, nu):
    """``cavity_flow(nx, ny, nt, nit, u, v, dt, dx, dy, p, rho, nu)`` of
    cavity_flow/cavity_flow_numpy.py:41-82 (float64; u, v, p updated in place).

    Per time step, in the reference's order:

    * ``build_up_b`` (:13-21) on the interior, with x1 = (u_e - u_w)/(2dx),
      x2 = (v_s - v_n)/(2dy), z = (((u_s - u_n)/(2dy))*(v_e - v_w))/(2dx):
      ``b = rho*((((1/dt)*(x1 + x2) - x1**2) - 2*z) - x2**2)``;
    * ``pressure_poisson`` (:24-38), nit times: the interior
      ``(((p_e + p_w)*dy**2 + (p_s + p_n)*dx**2) / (2*(dx**2 + dy**2))) - c*b``
      from the previous iterate, then ``p[:, -1] = p[:, -2]``,
      ``p[0, :] = p[1, :]``, ``p[:, 0] = p[:, 1]``, ``p[-1, :] = 0``;
    * the u and v updates (:53-74) from copies un, vn and the new p, then the
      walls (:75-82): u = 0 on three sides and 1 on the lid (row -1), v = 0.

    Here ``_e/_w`` are columns j+1/j-1 and ``_s/_n`` rows i+1/i-1.
    """
    k = cfd_constants(dt, dx, dy, rho)
    b = np.zeros((ny, nx))
    for _ in range(nt):
        un = u.copy()
        vn = v.copy()
        _cfd_build_up_b(b, rho, u, v, k)
        _cfd_pressure_poisson(nit, p, b, k)
        _cfd_velocity(u, v, un, vn, p, dt, dx, dy, nu, k)
        u[0, :] = 0
        u[:, 0] = 0
        u[:, -1] = 0
        u[-1, :] = 1
        v[0, :] = 0
        v[-1, :] = 0
        v[:, 0] = 0
        v[:, -1] = 0


def _cfd_build_up_b(b, rho, u, v, k):
    x1 = np.divide(np.subtract(u[1:-1, 2:], u[1:-1, 0:-2]), k["two_dx"])
    x2 = np.divide(np.subtract(v[2:, 1:-1], v[0:-2, 1:-1]), k["two_dy"])
    r = np.multiply(k["inv_dt"], np.add(x1, x2))
    np.subtract(r, np.multiply(x1, x1), out=r)
    z = np.divide(np.subtract(u[2:, 1:-1], u[0:-2, 1:-1]), k["two_dy"])
    np.multiply(z, np.subtract(v[1:-1, 2:], v[1:-1, 0:-2]), out=z)
    np.divide(z, k["two_dx"], out=z)
    np.subtract(r, np.multiply(2, z), out=r)
    np.subtract(r, np.multiply(x2, x2), out=r)
    b[1:-1, 1:-1] = np.multiply(rho, r)


def _cfd_pressure_poisson(nit, p, b, k):
    cb = np.multiply(k["pC"], b[1:-1, 1:-1])
    for _ in range(nit):
        pn = p.copy()
        t = np.multiply(np.add(pn[1:-1, 2:], pn[1:-1, 0:-2]), k["dy2"])
        np.add(t, np.multiply(np.add(pn[2:, 1:-1], pn[0:-2, 1:-1]), k["dx2"]), out=t)
        np.divide(t, k["pD"], out=t)
        p[1:-1, 1:-1] = np.subtract(t, cb)
        p[:, -1] = p[:, -2]
        p[0, :] = p[1, :]
        p[:, 0] = p[:, 1]
        p[-1, :] = 0


def _cfd_component(c, f, p_diff, dt, dx, dy, nu, k1, k):
    """(((f - ((ua*dt)/dx)*(f - f_w)) - ((vn*dt)/dy)*(f - f_n)) - k1*p_diff)
    + nu*(k2*((f_e - 2f) + f_w) + k3*((f_s - 2f) + f_n)) on the interior, where
    ``c`` is the (un, vn) pair and ``f`` the advected field."""
    un, vn = c
    fc = f[1:-1, 1:-1]
    a = np.multiply(np.divide(np.multiply(un[1:-1, 1:-1], dt), dx),
                    np.subtract(fc, f[1:-1, 0:-2]))
    bb = np.multiply(np.divide(np.multiply(vn[1:-1, 1:-1], dt), dy),
                     np.subtract(fc, f[0:-2, 1:-1]))
    out = np.subtract(fc, a)
    np.subtract(out, bb, out=out)
    np.subtract(out, np.multiply(k1, p_diff), out=out)
    two_f = np.multiply(2, fc)
    d1 = np.multiply(k["k2"], np.add(np.subtract(f[1:-1, 2:], two_f), f[1:-1, 0:-2]))
    d2 = np.multiply(k["k3"], np.add(np.subtract(f[2:, 1:-1], two_f), f[0:-2, 1:-1]))
    np.add(out, np.multiply(nu, np.add(d1, d2)), out=out)
    return out


def _cfd_velocity(u, v, un, vn, p, dt, dx, dy, nu, k):
    u[1:-1, 1:-1] = _cfd_component((un, vn), un, np.subtract(p[1:-1, 2:], p[1:-1, 0:-2]),
                                   dt, dx, dy, nu, k["k1u"], k)
    v[1:-1, 1:-1] = _cfd_component((un, vn), vn, np.subtract(p[2:, 1:-1], p[0:-2, 1:-1]),
                                   dt, dx, dy, nu, k["k1v"], k)


def _wrap_cols(f):
    """(east, west) neighbours of every column with periodic wrap in x."""
    return np.roll(f, -1, axis=1), np.roll(f, 1, axis=1)


def channel_flow(nit, u, v, dt, dx, dy, p, rho, nu, F):
    """``channel_flow(nit, u, v, dt, dx, dy, p, rho, nu, F)`` of
    channel_flow/channel_flow_numpy.py:69-152; returns the step count.

    The cavity_flow arithmetic with a periodic x direction: build_up_b (:13-39),
    the pressure iterations (:42-66) and the u/v updates (:80-143) evaluate the
    same expressions at every column, the neighbours of columns 0 and -1
    wrapping around; the pressure walls copy row -2 to row -1, then row 1 to
    row 0; u gains ``+ F*dt`` and the walls zero rows 0 and -1 of u and v.
    The loop runs while ``(sum(u) - sum(un)) / sum(u) > .001`` (``np.sum``,
    NumPy's pairwise summation).
    """
    ny, nx = u.shape
    # The reference indexes column -2 (channel_flow_numpy.py:24), row -2 of p
    # (:65, when nit >= 1) and row 0 (:144): IndexError below these sizes.
    if nx < 2 or ny < 1 or (nit > 0 and ny < 2):
        raise IndexError(f"channel_flow: a ({ny}, {nx}) grid is too small for the boundaries")
    k = cfd_constants(dt, dx, dy, rho)
    Fdt = F * dt
    udiff = 1
    stepcount = 0
    while udiff > .001:
        un = u.copy()
        vn = v.copy()
        b = np.zeros_like(u)
        _chan_build_up_b(b, rho, u, v, k)
        _chan_pressure(nit, p, b, k)
        _chan_velocity(u, v, un, vn, p, dt, dx, dy, nu, Fdt, k)
        u[0, :] = 0
        u[-1, :] = 0
        v[0, :] = 0
        v[-1, :] = 0
        udiff = (np.sum(u) - np.sum(un)) / np.sum(u)
        stepcount += 1
    return stepcount


def _chan_build_up_b(b, rho, u, v, k):
    ue, uw = _wrap_cols(u)
    ve, vw = _wrap_cols(v)
    x1 = np.divide(np.subtract(ue[1:-1], uw[1:-1]), k["two_dx"])
    x2 = np.divide(np.subtract(v[2:], v[0:-2]), k["two_dy"])
    r = np.multiply(k["inv_dt"], np.add(x1, x2))
    np.subtract(r, np.multiply(x1, x1), out=r)
    z = np.divide(np.subtract(u[2:], u[0:-2]), k["two_dy"])
    np.multiply(z, np.subtract(ve[1:-1], vw[1:-1]), out=z)
    np.divide(z, k["two_dx"], out=z)
    np.subtract(r, np.multiply(2, z), out=r)
    np.subtract(r, np.multiply(x2, x2), out=r)
    b[1:-1, :] = np.multiply(rho, r)


def _chan_pressure(nit, p, b, k):
    cb = np.multiply(k["pC"], b[1:-1])
    for _ in range(nit):
        pn = p.copy()
        pe, pw = _wrap_cols(pn)
        t = np.multiply(np.add(pe[1:-1], pw[1:-1]), k["dy2"])
        np.add(t, np.multiply(np.add(pn[2:], pn[0:-2]), k["dx2"]), out=t)
        np.divide(t, k["pD"], out=t)
        p[1:-1, :] = np.subtract(t, cb)
        p[-1, :] = p[-2, :]
        p[0, :] = p[1, :]


def _chan_component(un, vn, f, p_diff, dt, dx, dy, nu, k1, k):
    fe, fw = _wrap_cols(f)
    fc = f[1:-1]
    a = np.multiply(np.divide(np.multiply(un[1:-1], dt), dx), np.subtract(fc, fw[1:-1]))
    bb = np.multiply(np.divide(np.multiply(vn[1:-1], dt), dy), np.subtract(fc, f[0:-2]))
    out = np.subtract(fc, a)
    np.subtract(out, bb, out=out)
    np.subtract(out, np.multiply(k1, p_diff), out=out)
    two_f = np.multiply(2, fc)
    d1 = np.multiply(k["k2"], np.add(np.subtract(fe[1:-1], two_f), fw[1:-1]))
    d2 = np.multiply(k["k3"], np.add(np.subtract(f[2:], two_f), f[0:-2]))
    np.add(out, np.multiply(nu, np.add(d1, d2)), out=out)
    return out


def _chan_velocity(u, v, un, vn, p, dt, dx, dy, nu, Fdt, k):
    pe, pw = _wrap_cols(p)
    nu_ = _chan_component(un, vn, un, np.subtract(pe[1:-1], pw[1:-1]), dt, dx, dy, nu, k["k1u"], k)
    u[1:-1, :] = np.add(nu_, Fdt)
    v[1:-1, :] = _chan_component(un, vn, vn, np.subtract(p[2:], p[0:-2]), dt, dx, dy, nu,
                                 k["k1v"], k)
