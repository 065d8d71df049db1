"""Pin the CPU oracle (NumPy and C restatements) to the reference's golden vectors.

The golden vectors were produced by the reference's own NumPy kernels
(tests/golden/make_golden.py).  Both restatements must reproduce them bit for
bit, including signed zeros, infinities and NaN positions.
"""
import hashlib

import numpy as np
import pytest

from conftest import bits_equal, first_diff
from oracle import cref, stencils_np
from npbench_gb300 import workloads

ORACLES = {"numpy": stencils_np, "c": cref}


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _cases(golden, bench, stored=True):
    manifest, arrays = golden
    for c in manifest["cases"]:
        if c["bench"] != bench:
            continue
        if stored == ("init" not in c):
            yield c


@pytest.mark.parametrize("which", sorted(ORACLES))
@pytest.mark.parametrize("bench,fn", [("jacobi_2d", "jacobi_2d_kernel"),
                                      ("heat_3d", "heat_3d_kernel"),
                                      ("jacobi_1d", "jacobi_1d_kernel")])
def test_pingpong_golden(golden, which, bench, fn):
    _, arrays = golden
    kern = getattr(ORACLES[which], fn)
    n = 0
    with np.errstate(all="ignore"):
        for c in _cases(golden, bench):
            name = c["name"]
            a, b = arrays[f"{name}/A_in"].copy(), arrays[f"{name}/B_in"].copy()
            kern(c["tsteps"], a, b)
            assert bits_equal(a, arrays[f"{name}/A_out"]), (name, first_diff(a, arrays[f"{name}/A_out"]))
            assert bits_equal(b, arrays[f"{name}/B_out"]), (name, first_diff(b, arrays[f"{name}/B_out"]))
            n += 1
    assert n >= 20


@pytest.mark.parametrize("which", sorted(ORACLES))
def test_hdiff_golden(golden, which):
    _, arrays = golden
    n = 0
    with np.errstate(all="ignore"):
        for c in _cases(golden, "hdiff"):
            name = c["name"]
            out = arrays[f"{name}/out_in"].copy()
            ORACLES[which].hdiff(arrays[f"{name}/in"], out, arrays[f"{name}/coeff"])
            assert bits_equal(out, arrays[f"{name}/out"]), (name, first_diff(out, arrays[f"{name}/out"]))
            n += 1
    assert n >= 6


@pytest.mark.parametrize("which", sorted(ORACLES))
def test_fdtd_golden(golden, which):
    _, arrays = golden
    n = 0
    with np.errstate(all="ignore"):
        for c in _cases(golden, "fdtd_2d"):
            name = c["name"]
            ex, ey, hz = (arrays[f"{name}/{k}_in"].copy() for k in ("ex", "ey", "hz"))
            ORACLES[which].fdtd_2d_kernel(c["tsteps"], ex, ey, hz, arrays[f"{name}/fict"])
            for k, v in (("ex", ex), ("ey", ey), ("hz", hz)):
                assert bits_equal(v, arrays[f"{name}/{k}_out"]), (name, k)
            n += 1
    assert n >= 20


@pytest.mark.parametrize("which", sorted(ORACLES))
def test_vadv_golden(golden, which):
    _, arrays = golden
    n = 0
    with np.errstate(all="ignore"):
        for c in _cases(golden, "vadv"):
            name = c["name"]
            if "raises" in c:
                I, J, K = c["shape"]
                z = np.zeros((I, J, K))
                with pytest.raises(IndexError):
                    ORACLES[which].vadv(z.copy(), z, np.zeros((I + 1, J, K)), z, z, c["dtr_stage"])
                continue
            us = arrays[f"{name}/utens_stage_in"].copy()
            ORACLES[which].vadv(us, *(arrays[f"{name}/{k}"] for k in
                                      ("u_stage", "wcon", "u_pos", "utens")), c["dtr_stage"])
            exp = arrays[f"{name}/utens_stage_out"]
            assert bits_equal(us, exp), (name, first_diff(us, exp))
            n += 1
    assert n >= 20


def cfd_case_args(arrays, c, copy=True):
    """(nx, ny, nt, nit, u, v, dt, dx, dy, p, rho, nu) for a stored cavity_flow case."""
    name = c["name"]
    u, v, p = (arrays[f"{name}/{k}_in"] for k in ("u", "v", "p"))
    if copy:
        u, v, p = u.copy(), v.copy(), p.copy()
    ny, nx = c["shape"]
    return (nx, ny, c["nt"], c["nit"], u, v, c["dt"], c["dx"], c["dy"], p, c["rho"], c["nu"])


@pytest.mark.parametrize("which", sorted(ORACLES))
def test_cavity_flow_golden(golden, which):
    _, arrays = golden
    n = 0
    with np.errstate(all="ignore"):
        for c in _cases(golden, "cavity_flow"):
            name = c["name"]
            if "raises" in c:
                ny, nx = c["shape"]
                z = [np.zeros((ny, nx)) for _ in range(3)]
                with pytest.raises(IndexError):
                    ORACLES[which].cavity_flow(nx, ny, 1, 1, z[0], z[1], 0.01, 0.5, 0.5, z[2],
                                               1.0, 0.1)
                continue
            args = cfd_case_args(arrays, c)
            ORACLES[which].cavity_flow(*args)
            for k, got in (("u", args[4]), ("v", args[5]), ("p", args[9])):
                exp = arrays[f"{name}/{k}_out"]
                assert bits_equal(got, exp), (name, k, first_diff(got, exp))
            n += 1
    assert n >= 20


@pytest.mark.parametrize("which", sorted(ORACLES))
def test_channel_flow_golden(golden, which):
    _, arrays = golden
    n = 0
    with np.errstate(all="ignore"):
        for c in _cases(golden, "channel_flow"):
            name = c["name"]
            if "raises" in c:
                ny, nx = c["shape"]
                z = [np.zeros((ny, nx)) for _ in range(3)]
                with pytest.raises(IndexError):
                    ORACLES[which].channel_flow(c["nit"], z[0], z[1], 0.01, 0.5, 0.5, z[2], 1.0,
                                                0.1, 1.0)
                continue
            u, v, p = (arrays[f"{name}/{k}_in"].copy() for k in ("u", "v", "p"))
            steps = ORACLES[which].channel_flow(c["nit"], u, v, c["dt"], c["dx"], c["dy"], p,
                                                c["rho"], c["nu"], c["F"])
            assert steps == c["steps"], name
            for k, got in (("u", u), ("v", v), ("p", p)):
                exp = arrays[f"{name}/{k}_out"]
                assert bits_equal(got, exp), (name, k, first_diff(got, exp))
            n += 1
    assert n >= 10


def test_c_pairwise_sum_is_numpy_sum():
    """The C restatement of np.sum (+0.0 plus NumPy's pairwise summation)."""
    rng = np.random.default_rng(11)
    for n in list(range(0, 260)) + [1000, 4097, 8193, 10201, 40401]:
        a = rng.standard_normal(n) * np.exp(rng.standard_normal(n) * 6)
        assert cref.numpy_sum(a) == np.sum(a), n
    assert np.signbit(np.sum(np.full(9, -0.0))) == np.signbit(cref.numpy_sum(np.full(9, -0.0)))


@pytest.mark.parametrize("which", sorted(ORACLES))
def test_reference_initializer_presets(golden, which):
    """Preset S with the reference's own initializers, checked by SHA-256."""
    o = ORACLES[which]
    seen = 0
    for c in golden[0]["cases"]:
        if c.get("init") != "reference":
            continue
        dt = np.dtype(c["dtype"])
        if c["bench"] == "fdtd_2d":
            ex, ey, hz, fict = workloads.init_fdtd_2d(c["TMAX"], c["NX"], c["NY"], dt.type)
            o.fdtd_2d_kernel(c["tsteps"], ex, ey, hz, fict)
            assert (_sha(ex), _sha(ey), _sha(hz)) == (c["sha_ex_out"], c["sha_ey_out"],
                                                      c["sha_hz_out"]), c["name"]
            seen += 1
            continue
        if c["bench"] == "channel_flow":
            ny, nx = c["shape"]
            u, v, p, dx, dy, dt = workloads.init_channel_flow(ny, nx)
            assert (dx, dy, dt) == (c["dx"], c["dy"], c["dt"]), c["name"]
            steps = o.channel_flow(c["nit"], u, v, dt, dx, dy, p, c["rho"], c["nu"], c["F"])
            assert steps == c["steps"], c["name"]
            assert (_sha(u), _sha(v), _sha(p)) == (c["sha_u"], c["sha_v"], c["sha_p"]), c["name"]
            seen += 1
            continue
        if c["bench"] == "cavity_flow":
            ny, nx = c["shape"]
            u, v, p, dx, dy, dt = workloads.init_cavity_flow(ny, nx)
            assert (dx, dy, dt) == (c["dx"], c["dy"], c["dt"]), c["name"]
            o.cavity_flow(nx, ny, c["nt"], c["nit"], u, v, dt, dx, dy, p, c["rho"], c["nu"])
            assert (_sha(u), _sha(v), _sha(p)) == (c["sha_u"], c["sha_v"], c["sha_p"]), c["name"]
            seen += 1
            continue
        if c["bench"] == "vadv":
            dtr, us, u, w, up, ut = workloads.init_vadv(c["I"], c["J"], c["K"])
            assert _sha(us) == c["sha_in"] and dtr == c["dtr_stage"], c["name"]
            o.vadv(us, u, w, up, ut, dtr)
            assert _sha(us) == c["sha_out"], c["name"]
            seen += 1
            continue
        if c["bench"] == "jacobi_1d":
            A, B = workloads.init_jacobi_1d(c["N"], dt.type)
            kern = o.jacobi_1d_kernel
        elif c["bench"] == "jacobi_2d":
            A, B = workloads.init_jacobi_2d(c["N"], dt.type)
            kern = o.jacobi_2d_kernel
        elif c["bench"] == "heat_3d":
            A, B = workloads.init_heat_3d(c["N"], dt.type)
            kern = o.heat_3d_kernel
        else:
            I, J, K = c["shape"]
            inf, out, coeff = workloads.init_hdiff(I, J, K)
            assert _sha(inf) == c["sha_in"] and _sha(coeff) == c["sha_coeff"], c["name"]
            o.hdiff(inf, out, coeff)
            assert _sha(out) == c["sha_out"], c["name"]
            seen += 1
            continue
        assert _sha(A) == c["sha_A_in"] and _sha(B) == c["sha_B_in"], c["name"]
        kern(c["tsteps"], A, B)
        assert _sha(A) == c["sha_A_out"] and _sha(B) == c["sha_B_out"], c["name"]
        seen += 1
    assert seen == 12


def test_oracles_agree_on_random_nonsquare():
    """The two restatements agree with each other beyond the golden sizes."""
    rng = np.random.default_rng(7)
    for dt in (np.float64, np.float32):
        A = rng.random((61, 130)).astype(dt)
        B = rng.random((61, 130)).astype(dt)
        a1, b1, a2, b2 = A.copy(), B.copy(), A.copy(), B.copy()
        stencils_np.jacobi_2d_kernel(9, a1, b1)
        cref.jacobi_2d_kernel(9, a2, b2)
        assert bits_equal(a1, a2) and bits_equal(b1, b2)
        H = rng.random((19, 23, 41)).astype(dt)
        h1, g1, h2, g2 = H.copy(), H.copy(), H.copy(), H.copy()
        stencils_np.heat_3d_kernel(6, h1, g1)
        cref.heat_3d_kernel(6, h2, g2)
        assert bits_equal(h1, h2) and bits_equal(g1, g2)
    inf, out, co = workloads.uniform_hdiff(21, 34, 19, seed=3)
    o1, o2 = out.copy(), out.copy()
    stencils_np.hdiff(inf, o1, co)
    cref.hdiff(inf, o2, co)
    assert bits_equal(o1, o2)


def test_planted_mistake_is_caught(golden):
    """A one-ulp change in the oracle's output must fail the comparison."""
    _, arrays = golden
    name = "jacobi_2d/float64/33x47/T17"
    a, b = arrays[f"{name}/A_in"].copy(), arrays[f"{name}/B_in"].copy()
    stencils_np.jacobi_2d_kernel(17, a, b)
    a[5, 7] = np.nextafter(a[5, 7], 2.0)
    assert not bits_equal(a, arrays[f"{name}/A_out"])
