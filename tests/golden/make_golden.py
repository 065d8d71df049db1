"""Generate the golden vectors for the stencil path from the reference itself.

Run with a directory holding the NPBench sources (``--ref``, or the
NPBENCH_SRC environment variable):

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py --ref DIR

It imports the reference's own NumPy kernels

* ``npbench.benchmarks.polybench.jacobi_2d.jacobi_2d_numpy.kernel``
* ``npbench.benchmarks.polybench.heat_3d.heat_3d_numpy.kernel``
* ``npbench.benchmarks.weather_stencils.hdiff.hdiff_numpy.hdiff``
* ``npbench.benchmarks.polybench.jacobi_1d.jacobi_1d_numpy.kernel``
* ``npbench.benchmarks.polybench.fdtd_2d.fdtd_2d_numpy.kernel``
* ``npbench.benchmarks.weather_stencils.vadv.vadv_numpy.vadv``
* ``npbench.benchmarks.cavity_flow.cavity_flow_numpy.cavity_flow``
* ``npbench.benchmarks.channel_flow.channel_flow_numpy.channel_flow``

and their ``initialize`` functions, runs them on seeded inputs, and writes

* ``cases.npz``     -- inputs and outputs of the small cases (exact arrays);
* ``manifest.json`` -- every case with its parameters, and for the larger
  preset cases SHA-256 digests of the inputs and outputs instead of arrays.

The tests under ``tests/`` compare the oracle and the CUDA kernels with these
files; none of them reads the reference at run time.
"""
import argparse
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def sha(a):
    a = np.ascontiguousarray(a)
    return hashlib.sha256(a.tobytes()).hexdigest()


def special_values(rng, shape, dtype):
    """U[0,1) sprinkled with signed zeros, negatives, tiny, huge, inf and nan."""
    a = rng.random(shape).astype(dtype)
    flat = a.reshape(-1)
    info = np.finfo(dtype)
    pool = np.array([0.0, -0.0, -0.75, 1.5, info.tiny, info.tiny * 2 ** -3, -info.tiny / 4,
                     info.max / 1.5, -info.max / 3, np.inf, -np.inf, np.nan, 1e-3, 3.0],
                    dtype=dtype)
    idx = rng.choice(flat.size, size=max(1, flat.size // 6), replace=False)
    flat[idx] = pool[rng.integers(0, pool.size, size=idx.size)]
    return a


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("NPBENCH_SRC"),
                    help="NPBench source tree (default: $NPBENCH_SRC)")
    args = ap.parse_args()
    if not args.ref:
        ap.error("give --ref DIR or set NPBENCH_SRC to an NPBench source tree")
    sys.dont_write_bytecode = True
    sys.path.insert(0, args.ref)
    from npbench.benchmarks.polybench.jacobi_2d import jacobi_2d_numpy, jacobi_2d
    from npbench.benchmarks.polybench.heat_3d import heat_3d_numpy, heat_3d
    from npbench.benchmarks.weather_stencils.hdiff import hdiff_numpy, hdiff
    from npbench.benchmarks.polybench.jacobi_1d import jacobi_1d_numpy, jacobi_1d
    from npbench.benchmarks.polybench.fdtd_2d import fdtd_2d_numpy, fdtd_2d
    from npbench.benchmarks.weather_stencils.vadv import vadv_numpy, vadv
    from npbench.benchmarks.cavity_flow import cavity_flow_numpy, cavity_flow
    from npbench.benchmarks.channel_flow import channel_flow_numpy, channel_flow

    arrays, cases = {}, []
    rng = np.random.default_rng(20211)

    def add_tsteps_case(bench, kern, name, tsteps, A, B, store=True, **meta):
        a, b = A.copy(), B.copy()
        kern(tsteps, a, b)
        case = dict(name=name, bench=bench, tsteps=int(tsteps), dtype=A.dtype.name,
                    shape=list(A.shape), **meta)
        if store:
            for k, v in (("A_in", A), ("B_in", B), ("A_out", a), ("B_out", b)):
                arrays[f"{name}/{k}"] = v
        else:
            case.update(sha_A_in=sha(A), sha_B_in=sha(B), sha_A_out=sha(a), sha_B_out=sha(b))
        cases.append(case)

    # Jacobi-2D: empty/ragged interiors, non-square, step counts 0..17, both dtypes.
    for dt in (np.float64, np.float32):
        for shape in [(2, 2), (2, 6), (3, 3), (4, 4), (5, 7), (9, 4), (33, 47), (64, 65)]:
            for T in ((0, 1, 2, 3, 17) if shape[0] * shape[1] < 100 else (2, 17)):
                A = rng.random(shape).astype(dt)
                B = rng.random(shape).astype(dt)
                add_tsteps_case("jacobi_2d", jacobi_2d_numpy.kernel,
                                f"jacobi_2d/{dt.__name__}/{shape[0]}x{shape[1]}/T{T}", T, A, B)
        A = special_values(rng, (23, 29), dt)
        B = special_values(rng, (23, 29), dt)
        add_tsteps_case("jacobi_2d", jacobi_2d_numpy.kernel,
                        f"jacobi_2d/{dt.__name__}/special/T4", 4, A, B, special=True)
        # The reference's own initializer at preset S (N=150, TSTEPS=50).
        A, B = jacobi_2d.initialize(150, dt)
        add_tsteps_case("jacobi_2d", jacobi_2d_numpy.kernel,
                        f"jacobi_2d/{dt.__name__}/presetS", 50, A, B, store=False,
                        init="reference", N=150)

    # Heat-3D.
    for dt in (np.float64, np.float32):
        for shape in [(2, 4, 4), (3, 3, 3), (4, 5, 6), (5, 3, 7), (9, 17, 33), (12, 12, 12)]:
            for T in ((0, 1, 2, 3, 17) if np.prod(shape) < 200 else (2, 17)):
                A = rng.random(shape).astype(dt)
                B = A.copy()
                add_tsteps_case("heat_3d", heat_3d_numpy.kernel,
                                f"heat_3d/{dt.__name__}/{'x'.join(map(str, shape))}/T{T}", T, A, B)
        A = special_values(rng, (7, 9, 11), dt)
        B = special_values(rng, (7, 9, 11), dt)
        add_tsteps_case("heat_3d", heat_3d_numpy.kernel,
                        f"heat_3d/{dt.__name__}/special/T3", 3, A, B, special=True)
        A, B = heat_3d.initialize(25, dt)
        add_tsteps_case("heat_3d", heat_3d_numpy.kernel,
                        f"heat_3d/{dt.__name__}/presetS", 25, A, B, store=False,
                        init="reference", N=25)

    # hdiff (float64 only).
    for (I, J, K) in [(1, 1, 1), (1, 3, 2), (4, 5, 3), (13, 7, 1), (8, 8, 5), (16, 9, 17)]:
        inf = rng.random((I + 4, J + 4, K))
        coeff = rng.random((I, J, K))
        out0 = rng.random((I, J, K))
        out = out0.copy()
        hdiff_numpy.hdiff(inf, out, coeff)
        name = f"hdiff/float64/{I}x{J}x{K}"
        arrays.update({f"{name}/in": inf, f"{name}/coeff": coeff, f"{name}/out_in": out0,
                       f"{name}/out": out})
        cases.append(dict(name=name, bench="hdiff", dtype="float64", shape=[I, J, K]))
    inf = special_values(rng, (10, 11, 6), np.float64)
    coeff = special_values(rng, (6, 7, 6), np.float64)
    out = np.zeros((6, 7, 6))
    with np.errstate(all="ignore"):
        hdiff_numpy.hdiff(inf, out, coeff)
    name = "hdiff/float64/special"
    arrays.update({f"{name}/in": inf, f"{name}/coeff": coeff, f"{name}/out_in": np.zeros_like(out),
                   f"{name}/out": out})
    cases.append(dict(name=name, bench="hdiff", dtype="float64", shape=[6, 7, 6], special=True))
    # Preset S with the reference initializer (default_rng(42)).
    inf, out, coeff = hdiff.initialize(64, 64, 60)
    o = out.copy()
    hdiff_numpy.hdiff(inf, o, coeff)
    cases.append(dict(name="hdiff/float64/presetS", bench="hdiff", dtype="float64",
                      shape=[64, 64, 60], init="reference", sha_in=sha(inf), sha_coeff=sha(coeff),
                      sha_out=sha(o)))

    # Jacobi-1D.
    for dt in (np.float64, np.float32):
        for n in (2, 3, 4, 17, 300):
            for T in ((0, 1, 2, 3, 17) if n < 100 else (2, 40)):
                A = rng.random(n).astype(dt)
                B = rng.random(n).astype(dt)
                add_tsteps_case("jacobi_1d", jacobi_1d_numpy.kernel, f"jacobi_1d/{dt.__name__}/{n}/T{T}",
                                T, A, B)
        A, B = special_values(rng, (41,), dt), special_values(rng, (41,), dt)
        add_tsteps_case("jacobi_1d", jacobi_1d_numpy.kernel, f"jacobi_1d/{dt.__name__}/special/T5", 5,
                        A, B, special=True)
        A, B = jacobi_1d.initialize(3200, dt)
        add_tsteps_case("jacobi_1d", jacobi_1d_numpy.kernel, f"jacobi_1d/{dt.__name__}/presetS", 800,
                        A, B, store=False, init="reference", N=3200)

    # FDTD-2D (TMAX steps over ex, ey, hz; _fict_ of length TMAX).
    def add_fdtd_case(name, tmax, ex, ey, hz, fict, store=True, **meta):
        e1, e2, h = ex.copy(), ey.copy(), hz.copy()
        fdtd_2d_numpy.kernel(tmax, e1, e2, h, fict)
        case = dict(name=name, bench="fdtd_2d", tsteps=int(tmax), dtype=ex.dtype.name,
                    shape=list(ex.shape), **meta)
        if store:
            for k, v in (("ex_in", ex), ("ey_in", ey), ("hz_in", hz), ("fict", fict),
                         ("ex_out", e1), ("ey_out", e2), ("hz_out", h)):
                arrays[f"{name}/{k}"] = v
        else:
            case.update(sha_ex_out=sha(e1), sha_ey_out=sha(e2), sha_hz_out=sha(h))
        cases.append(case)

    for dt in (np.float64, np.float32):
        for shape in [(1, 1), (2, 3), (5, 7), (20, 22), (33, 9)]:
            for T in (0, 1, 3, 10):
                ex, ey, hz = (rng.random(shape).astype(dt) for _ in range(3))
                fict = rng.random(max(T, 1)).astype(dt)
                add_fdtd_case(f"fdtd_2d/{dt.__name__}/{shape[0]}x{shape[1]}/T{T}", T, ex, ey, hz, fict)
        ex, ey, hz = (special_values(rng, (9, 11), dt) for _ in range(3))
        add_fdtd_case(f"fdtd_2d/{dt.__name__}/special/T4", 4, ex, ey, hz,
                      special_values(rng, (4,), dt), special=True)
        ex, ey, hz, fict = fdtd_2d.initialize(20, 200, 220, dt)
        add_fdtd_case(f"fdtd_2d/{dt.__name__}/presetS", 20, ex, ey, hz, fict, store=False,
                      init="reference", TMAX=20, NX=200, NY=220)

    # vadv (float64; K >= 2).  Its own generator, so the cases above keep their draws.
    vrng = np.random.default_rng(20212)

    def add_vadv_case(name, us, u, w, up, ut, dtr, store=True, **meta):
        out = us.copy()
        vadv_numpy.vadv(out, u, w, up, ut, dtr)
        case = dict(name=name, bench="vadv", dtype="float64", shape=list(us.shape),
                    dtr_stage=float(dtr), **meta)
        if store:
            for k, v in (("utens_stage_in", us), ("u_stage", u), ("wcon", w), ("u_pos", up),
                         ("utens", ut), ("utens_stage_out", out)):
                arrays[f"{name}/{k}"] = v
        else:
            case.update(sha_in=sha(us), sha_out=sha(out))
        cases.append(case)

    for (I, J, K) in [(1, 1, 2), (1, 1, 3), (2, 3, 2), (3, 2, 5), (0, 3, 4), (3, 0, 4),
                      (5, 4, 17), (7, 9, 33), (16, 8, 40)]:
        for dtr in (3.0 / 20.0, 0.7):
            us, u, up, ut = (vrng.random((I, J, K)) for _ in range(4))
            w = vrng.random((I + 1, J, K))
            add_vadv_case(f"vadv/float64/{I}x{J}x{K}/dtr{dtr:g}", us, u, w, up, ut, dtr)
    # Full special pool (NaN and inf spread along the columns).
    us, u, up, ut = (special_values(vrng, (6, 7, 9), np.float64) for _ in range(4))
    w = special_values(vrng, (7, 7, 9), np.float64)
    add_vadv_case("vadv/float64/special", us, u, w, up, ut, 0.15, special=True)
    # Finite edge values: signed zeros, subnormal and tiny wcon sums, exact cancellations,
    # negatives and repeated u levels (zero differences).
    us, u, up, ut = (vrng.random((5, 6, 12)) for _ in range(4))
    w = vrng.random((6, 6, 12))
    flat = w.reshape(-1)
    pool = np.array([0.0, -0.0, 5e-324, -2.5e-320, 2.0 ** -1021, 2.0 ** -1019, 2.0 ** -1018,
                     -0.5, 1e-300])
    idx = vrng.choice(flat.size, size=flat.size // 3, replace=False)
    flat[idx] = pool[vrng.integers(0, pool.size, size=idx.size)]
    w[1:4, :, 3] = -w[0:3, :, 3]          # w sums of exactly zero
    u[:, :, 5] = u[:, :, 4]               # zero differences
    u[:, ::2, 7] = -0.0
    u[:, 1::2, 6] = 0.0
    us[0, 0, :] = -us[0, 0, :]
    add_vadv_case("vadv/float64/edge", us, u, w, up, ut, 0.15, special=True)
    # Signed zeros through the whole solve: u constant along K (zero differences),
    # or alternating +0/-0; with u_pos = +0, utens = utens_stage = -0 and a
    # negative dtr_stage, the sign of each zero difference reaches the output
    # (a solver that takes -(previous product) for (-as)*(u[k-1] - u[k]) without
    # IEEE's rule for zero differences gets a third of these outputs wrong).
    for K in (8, 6):
        I, J = 3, 4
        us, u, up, ut = (vrng.random((I, J, K)) for _ in range(4))
        w = vrng.random((I + 1, J, K))
        u[0, :, :] = 0.5
        u[1, 0, :] = 0.0
        u[1, 1, :] = -0.0
        u[1, 2, :] = np.where(np.arange(K) % 2 == 0, 0.0, -0.0)
        u[1, 3, :] = np.where(np.arange(K) % 2 == 0, -0.0, 0.0)
        up[0:2] = 0.0
        ut[0:2] = -0.0
        us[0:2] = -0.0
        add_vadv_case(f"vadv/float64/zeros/K{K}", us, u, w, up, ut, -0.15, special=True)
    # Preset S with the reference initializer (default_rng(42)).
    dtr, us, u, w, up, ut = vadv.initialize(60, 60, 40)
    add_vadv_case("vadv/float64/presetS", us, u, w, up, ut, dtr, store=False, init="reference",
                  I=60, J=60, K=40)
    # K < 2: the reference raises IndexError (it reads level 1 unconditionally).
    for K in (0, 1):
        z = np.zeros((2, 3, K))
        try:
            vadv_numpy.vadv(z.copy(), z, np.zeros((3, 3, K)), z, z, 0.15)
            raised = None
        except Exception as e:  # noqa: BLE001 - record what the reference raises
            raised = type(e).__name__
        cases.append(dict(name=f"vadv/float64/K{K}", bench="vadv", dtype="float64",
                          shape=[2, 3, K], dtr_stage=0.15, raises=raised))

    # cavity_flow (float64): reference initialize (zeros) and random fields.
    crng = np.random.default_rng(20213)

    def add_cfd_case(name, ny, nx, nt, nit, u, v, p, rho=1.0, nu=0.1, store=True, **meta):
        _, _, _, dx, dy, dt = cavity_flow.initialize(ny, nx)
        a, b, c = u.copy(), v.copy(), p.copy()
        cavity_flow_numpy.cavity_flow(nx, ny, nt, nit, a, b, dt, dx, dy, c, rho, nu)
        case = dict(name=name, bench="cavity_flow", dtype="float64", shape=[ny, nx], nt=nt,
                    nit=nit, rho=rho, nu=nu, dx=dx, dy=dy, dt=dt, **meta)
        if store:
            for k, val in (("u_in", u), ("v_in", v), ("p_in", p), ("u_out", a), ("v_out", b),
                           ("p_out", c)):
                arrays[f"{name}/{k}"] = val
        else:
            case.update(sha_u=sha(a), sha_v=sha(b), sha_p=sha(c))
        cases.append(case)

    for (ny, nx, nt, nit) in [(2, 2, 2, 2), (2, 5, 3, 2), (5, 2, 3, 2), (3, 3, 2, 3), (5, 7, 3, 2),
                              (12, 9, 4, 3), (31, 33, 6, 5), (40, 17, 3, 4), (9, 70, 2, 1),
                              (6, 6, 0, 3), (6, 6, 2, 0)]:
        u0, v0, p0, _, _, _ = cavity_flow.initialize(ny, nx)
        add_cfd_case(f"cavity_flow/float64/{ny}x{nx}/nt{nt}/nit{nit}/init", ny, nx, nt, nit,
                     u0, v0, p0)
        u0, v0, p0 = (crng.random((ny, nx)) for _ in range(3))
        add_cfd_case(f"cavity_flow/float64/{ny}x{nx}/nt{nt}/nit{nit}/rand", ny, nx, nt, nit,
                     u0, v0, p0, rho=1.3, nu=0.07)
    u0, v0, p0 = (special_values(crng, (8, 9), np.float64) for _ in range(3))
    add_cfd_case("cavity_flow/float64/special", 8, 9, 3, 2, u0, v0, p0, special=True)
    u0, v0, p0, _, _, _ = cavity_flow.initialize(61, 61)
    add_cfd_case("cavity_flow/float64/presetS", 61, 61, 25, 5, u0, v0, p0, store=False,
                 init="reference")
    # ny or nx below 2: the reference's pressure boundary statements raise IndexError.
    for (ny, nx) in [(1, 5), (5, 1)]:
        u0, v0, p0 = (np.zeros((ny, nx)) for _ in range(3))
        try:
            cavity_flow_numpy.cavity_flow(nx, ny, 1, 1, u0, v0, 0.01, 0.5, 0.5, p0, 1.0, 0.1)
            raised = None
        except Exception as e:  # noqa: BLE001 - record what the reference raises
            raised = type(e).__name__
        cases.append(dict(name=f"cavity_flow/float64/{ny}x{nx}/raises", bench="cavity_flow",
                          dtype="float64", shape=[ny, nx], nt=1, nit=1, raises=raised))

    # channel_flow (float64): the step count is part of each case.
    hrng = np.random.default_rng(20214)

    def add_chan_case(name, ny, nx, nit, u, v, p, rho=1.0, nu=0.1, F=1.0, store=True, **meta):
        _, _, _, dx, dy, dt = channel_flow.initialize(ny, nx)
        a, b, c = u.copy(), v.copy(), p.copy()
        steps = channel_flow_numpy.channel_flow(nit, a, b, dt, dx, dy, c, rho, nu, F)
        case = dict(name=name, bench="channel_flow", dtype="float64", shape=[ny, nx], nit=nit,
                    rho=rho, nu=nu, F=F, dx=dx, dy=dy, dt=dt, steps=int(steps), **meta)
        if store:
            for k, val in (("u_in", u), ("v_in", v), ("p_in", p), ("u_out", a), ("v_out", b),
                           ("p_out", c)):
                arrays[f"{name}/{k}"] = val
        else:
            case.update(sha_u=sha(a), sha_v=sha(b), sha_p=sha(c))
        cases.append(case)

    for (ny, nx, nit) in [(2, 2, 1), (2, 5, 2), (3, 2, 2), (5, 7, 2), (12, 9, 3), (31, 33, 5),
                          (4, 40, 1), (9, 12, 0)]:
        u0, v0, p0, _, _, _ = channel_flow.initialize(ny, nx)
        add_chan_case(f"channel_flow/float64/{ny}x{nx}/nit{nit}/init", ny, nx, nit, u0, v0, p0)
    # random pressure, other physical constants
    u0, v0, _, _, _, _ = channel_flow.initialize(9, 12)
    add_chan_case("channel_flow/float64/9x12/nit3/randp", 9, 12, 3, u0, v0, hrng.random((9, 12)),
                  rho=1.2, nu=0.05, F=0.5)
    # two rows, negative sum(u): the first udiff is +inf, so a second step runs
    add_chan_case("channel_flow/float64/2x6/nit1/negu", 2, 6, 1, -hrng.random((2, 6)),
                  hrng.random((2, 6)), hrng.random((2, 6)))
    u0, v0, p0 = (special_values(hrng, (6, 8), np.float64) for _ in range(3))
    add_chan_case("channel_flow/float64/special", 6, 8, 2, u0, v0, p0, special=True)
    u0, v0, p0, _, _, _ = channel_flow.initialize(61, 61)
    add_chan_case("channel_flow/float64/presetS", 61, 61, 5, u0, v0, p0, store=False,
                  init="reference")
    for (ny, nx, nit) in [(5, 1, 0), (1, 5, 1)]:
        u0, v0, p0 = (np.zeros((ny, nx)) for _ in range(3))
        try:
            channel_flow_numpy.channel_flow(nit, u0, v0, 0.01, 0.5, 0.5, p0, 1.0, 0.1, 1.0)
            raised = None
        except Exception as e:  # noqa: BLE001 - record what the reference raises
            raised = type(e).__name__
        cases.append(dict(name=f"channel_flow/float64/{ny}x{nx}/raises", bench="channel_flow",
                          dtype="float64", shape=[ny, nx], nit=nit, raises=raised))

    np.savez_compressed(os.path.join(HERE, "cases.npz"), **arrays)
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump({"numpy": np.__version__, "seed": 20211, "cases": cases}, f, indent=1)
    print(f"{len(cases)} cases, {len(arrays)} arrays")


if __name__ == "__main__":
    with np.errstate(all="ignore"):
        main()
