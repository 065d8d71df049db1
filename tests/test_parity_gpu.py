"""Parity of the CUDA stencils with the reference, on the GPU.

* every stored golden case (reference NumPy outputs) -- bit for bit;
* preset S with the reference initializers -- SHA-256 of the outputs;
* seeded U[0,1) grids at the full benchmark sizes (Jacobi-2D 1000^2 x 100
  steps, Heat-3D 256^3 x 100 steps in float64 and float32, hdiff and vadv
  256x256x160, Jacobi-1D and FDTD-2D paper presets) against the C oracle --
  bit for bit;
* host NumPy arrays through the same entry points (copy in, copy back).

Bit-exact means identical bit patterns, except that any NaN matches any NaN.
"""
import hashlib

import numpy as np
import pytest

from conftest import bits_equal, first_diff

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from npbench_gb300 import _lib, stencils, workloads  # noqa: E402
from oracle import cref  # noqa: E402

DEV = torch.device("cuda", 0)


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(DEV)


def _host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


KERNELS = {"jacobi_2d": stencils.jacobi_2d_kernel, "heat_3d": stencils.heat_3d_kernel,
           "jacobi_1d": stencils.jacobi_1d_kernel}
INITS = {"jacobi_2d": workloads.init_jacobi_2d, "heat_3d": workloads.init_heat_3d,
         "jacobi_1d": workloads.init_jacobi_1d}


@pytest.mark.parametrize("bench", ["jacobi_2d", "heat_3d", "jacobi_1d"])
def test_golden_pingpong_bit_exact(golden, bench):
    manifest, arrays = golden
    n = 0
    for c in manifest["cases"]:
        if c["bench"] != bench or "init" in c:
            continue
        name = c["name"]
        A, B = _dev(arrays[f"{name}/A_in"]), _dev(arrays[f"{name}/B_in"])
        KERNELS[bench](c["tsteps"], A, B)
        a, b = _host(A), _host(B)
        assert bits_equal(a, arrays[f"{name}/A_out"]), (name, first_diff(a, arrays[f"{name}/A_out"]))
        assert bits_equal(b, arrays[f"{name}/B_out"]), (name, first_diff(b, arrays[f"{name}/B_out"]))
        n += 1
    assert n >= 20


def test_golden_hdiff_bit_exact(golden):
    manifest, arrays = golden
    n = 0
    for c in manifest["cases"]:
        if c["bench"] != "hdiff" or "init" in c:
            continue
        name = c["name"]
        out = _dev(arrays[f"{name}/out_in"])
        stencils.hdiff(_dev(arrays[f"{name}/in"]), out, _dev(arrays[f"{name}/coeff"]))
        o = _host(out)
        assert bits_equal(o, arrays[f"{name}/out"]), (name, first_diff(o, arrays[f"{name}/out"]))
        n += 1
    assert n >= 6


def test_golden_fdtd_bit_exact(golden):
    manifest, arrays = golden
    n = 0
    for c in manifest["cases"]:
        if c["bench"] != "fdtd_2d" or "init" in c:
            continue
        name = c["name"]
        ex, ey, hz = (_dev(arrays[f"{name}/{k}_in"]) for k in ("ex", "ey", "hz"))
        stencils.fdtd_2d_kernel(c["tsteps"], ex, ey, hz, _dev(arrays[f"{name}/fict"]))
        for k, v in (("ex", ex), ("ey", ey), ("hz", hz)):
            assert bits_equal(_host(v), arrays[f"{name}/{k}_out"]), (name, k)
        n += 1
    assert n >= 20


def _vadv_args(arrays, name):
    return [_dev(arrays[f"{name}/{k}"]) for k in ("u_stage", "wcon", "u_pos", "utens")]


def test_golden_vadv_bit_exact(golden):
    manifest, arrays = golden
    n = 0
    for c in manifest["cases"]:
        if c["bench"] != "vadv" or "init" in c:
            continue
        name = c["name"]
        if "raises" in c:
            I, J, K = c["shape"]
            z = torch.zeros((I, J, K), dtype=torch.float64, device=DEV)
            with pytest.raises(IndexError):
                stencils.vadv(z.clone(), z, torch.zeros((I + 1, J, K), dtype=torch.float64,
                                                        device=DEV), z, z, c["dtr_stage"])
            continue
        us = _dev(arrays[f"{name}/utens_stage_in"])
        stencils.vadv(us, *_vadv_args(arrays, name), c["dtr_stage"])
        o, exp = _host(us), arrays[f"{name}/utens_stage_out"]
        assert bits_equal(o, exp), (name, first_diff(o, exp))
        n += 1
    assert n >= 20


def test_vadv_library_allocated_workspace(golden):
    """workspace = NULL: the call allocates and frees its workspace stream-ordered."""
    from npbench_gb300 import _lib
    _, arrays = golden
    name = "vadv/float64/16x8x40/dtr0.7"
    us = _dev(arrays[f"{name}/utens_stage_in"])
    u, w, up, ut = _vadv_args(arrays, name)
    lib = _lib.load()
    st = lib.npbgb_vadv(us.data_ptr(), u.data_ptr(), w.data_ptr(), up.data_ptr(), ut.data_ptr(),
                        0.7, 16, 8, 40, _lib.NPBGB_F64, None, 0,
                        torch.cuda.current_stream(DEV).cuda_stream)
    _lib.check(st, "vadv")
    assert bits_equal(_host(us), arrays[f"{name}/utens_stage_out"])


def test_vadv_paper_size_vs_oracle():
    rng = np.random.default_rng(17)
    I, J, K = 256, 256, 160
    us, u, up, ut = (rng.random((I, J, K)) for _ in range(4))
    w = rng.random((I + 1, J, K))
    d = _dev(us)
    stencils.vadv(d, _dev(u), _dev(w), _dev(up), _dev(ut), 3.0 / 20.0)
    cref.vadv(us, u, w, up, ut, 3.0 / 20.0)
    o = _host(d)
    assert bits_equal(o, us), first_diff(o, us)


@pytest.mark.parametrize("IJK", [(1, 1, 2), (3, 5, 2), (7, 3, 3), (65, 1, 9), (33, 31, 7),
                                 (2, 700, 5)])
def test_vadv_ragged_shapes(IJK):
    I, J, K = IJK
    rng = np.random.default_rng(I * 10000 + J * 100 + K)
    us, u, up, ut = (rng.random((I, J, K)) for _ in range(4))
    w = rng.random((I + 1, J, K))
    d = _dev(us)
    stencils.vadv(d, _dev(u), _dev(w), _dev(up), _dev(ut), 0.15)
    cref.vadv(us, u, w, up, ut, 0.15)
    assert bits_equal(_host(d), us), IJK


def _cfd_args(arrays, c):
    name = c["name"]
    u, v, p = (_dev(arrays[f"{name}/{k}_in"]) for k in ("u", "v", "p"))
    ny, nx = c["shape"]
    return (nx, ny, c["nt"], c["nit"], u, v, c["dt"], c["dx"], c["dy"], p, c["rho"], c["nu"])


def test_golden_cavity_flow_bit_exact(golden):
    manifest, arrays = golden
    n = 0
    for c in manifest["cases"]:
        if c["bench"] != "cavity_flow" or "init" in c:
            continue
        name = c["name"]
        if "raises" in c:
            ny, nx = c["shape"]
            z = [torch.zeros((ny, nx), dtype=torch.float64, device=DEV) for _ in range(3)]
            with pytest.raises(IndexError):
                stencils.cavity_flow(nx, ny, 1, 1, z[0], z[1], 0.01, 0.5, 0.5, z[2], 1.0, 0.1)
            continue
        args = _cfd_args(arrays, c)
        stencils.cavity_flow(*args)
        for k, t in (("u", args[4]), ("v", args[5]), ("p", args[9])):
            got, exp = _host(t), arrays[f"{name}/{k}_out"]
            assert bits_equal(got, exp), (name, k, first_diff(got, exp))
        n += 1
    assert n >= 20


@pytest.mark.parametrize("shape,nt,nit", [((101, 101), 700, 50), ((400, 37), 5, 7),
                                          ((3, 300), 4, 3), ((161, 5), 6, 9), ((4, 50), 5, 6),
                                          ((7, 2000), 3, 4), ((153, 11), 4, 5)])
def test_cavity_flow_vs_oracle(shape, nt, nit):
    """The paper preset (one persistent launch for 700 steps of 50 pressure
    iterations) and band splits with several rows per band, from random fields."""
    ny, nx = shape
    rng = np.random.default_rng(ny * 1000 + nx)
    u, v, p = (rng.random(shape) for _ in range(3))
    dx, dy, dt = 2 / (nx - 1), 2 / (ny - 1), .1 / ((nx - 1) * (ny - 1))
    dev = [_dev(x) for x in (u, v, p)]
    stencils.cavity_flow(nx, ny, nt, nit, dev[0], dev[1], dt, dx, dy, dev[2], 1.0, 0.1)
    cref.cavity_flow(nx, ny, nt, nit, u, v, dt, dx, dy, p, 1.0, 0.1)
    for d, h, k in zip(dev, (u, v, p), "uvp"):
        got = _host(d)
        assert bits_equal(got, h), (shape, k, first_diff(got, h))


def test_cavity_flow_library_allocated_workspace(golden):
    """workspace = NULL: the call allocates and frees its workspace stream-ordered."""
    from npbench_gb300 import _lib
    manifest, arrays = golden
    c = next(c for c in manifest["cases"] if c["name"] == "cavity_flow/float64/31x33/nt6/nit5/rand")
    nx, ny, nt, nit, u, v, dt, dx, dy, p, rho, nu = _cfd_args(arrays, c)
    lib = _lib.load()
    st = lib.npbgb_cavity_flow(u.data_ptr(), v.data_ptr(), p.data_ptr(), ny, nx, nt, nit, dt, dx,
                               dy, rho, nu, _lib.NPBGB_F64, None, 0,
                               torch.cuda.current_stream(DEV).cuda_stream)
    _lib.check(st, "cavity_flow")
    assert lib.npbgb_device_status(None) == _lib.NPBGB_OK
    for k, t in (("u", u), ("v", v), ("p", p)):
        assert bits_equal(_host(t), arrays[f"{c['name']}/{k}_out"]), k


def test_golden_channel_flow_bit_exact(golden):
    manifest, arrays = golden
    n = 0
    for c in manifest["cases"]:
        if c["bench"] != "channel_flow" or "init" in c:
            continue
        name = c["name"]
        if "raises" in c:
            ny, nx = c["shape"]
            z = [torch.zeros((ny, nx), dtype=torch.float64, device=DEV) for _ in range(3)]
            with pytest.raises(IndexError):
                stencils.channel_flow(c["nit"], z[0], z[1], 0.01, 0.5, 0.5, z[2], 1.0, 0.1, 1.0)
            continue
        u, v, p = (_dev(arrays[f"{name}/{k}_in"]) for k in ("u", "v", "p"))
        steps = stencils.channel_flow(c["nit"], u, v, c["dt"], c["dx"], c["dy"], p, c["rho"],
                                      c["nu"], c["F"])
        assert steps == c["steps"], (name, steps)
        for k, t in (("u", u), ("v", v), ("p", p)):
            got, exp = _host(t), arrays[f"{name}/{k}_out"]
            assert bits_equal(got, exp), (name, k, first_diff(got, exp))
        n += 1
    assert n >= 10


@pytest.mark.parametrize("shape,nit", [((101, 101), 50), ((400, 37), 3), ((161, 2), 4),
                                       ((5, 64), 6), ((40, 9), 7)])
def test_channel_flow_vs_oracle(shape, nit):
    """The paper preset (989 steps of 50 pressure iterations in one launch) and
    band splits with several rows per band, from the reference's initial state."""
    ny, nx = shape
    u, v, p, dx, dy, dt = workloads.init_channel_flow(ny, nx)
    dev = [_dev(x) for x in (u, v, p)]
    s_gpu = stencils.channel_flow(nit, dev[0], dev[1], dt, dx, dy, dev[2], 1.0, 0.1, 1.0)
    s_ref = cref.channel_flow(nit, u, v, dt, dx, dy, p, 1.0, 0.1, 1.0)
    assert s_gpu == s_ref
    for d, h, k in zip(dev, (u, v, p), "uvp"):
        got = _host(d)
        assert bits_equal(got, h), (shape, k, first_diff(got, h))


def test_channel_flow_step_cap():
    """max_steps bounds the loop: RuntimeError, with the state after that many steps."""
    u, v, p, dx, dy, dt = workloads.init_channel_flow(12, 9)
    dev = [_dev(x) for x in (u, v, p)]
    with pytest.raises(RuntimeError):
        stencils.channel_flow(3, dev[0], dev[1], dt, dx, dy, dev[2], 1.0, 0.1, 1.0, max_steps=17)
    from npbench_gb300 import _lib
    assert _lib.load().npbgb_device_status(None) == _lib.NPBGB_OK


@pytest.mark.parametrize("pdl", [0, 1])
def test_chained_launch_modes_bit_exact(pdl):
    """Programmatic dependent launch on or off: the same bits from every time loop."""
    from npbench_gb300 import _lib
    old = _lib.set_config(_lib.NPBGB_CFG_PDL, pdl)
    try:
        for dt in (np.float64, np.float32):
            A, B = workloads.uniform_pair((333, 517), dt, seed=21)
            dA, dB = _dev(A), _dev(B)
            stencils.jacobi_2d_kernel(23, dA, dB)
            cref.jacobi_2d_kernel(23, A, B)
            assert bits_equal(_host(dA), A) and bits_equal(_host(dB), B)
            H, G = workloads.uniform_heat((45, 66, 130), dt, seed=22)
            dH, dG = _dev(H), _dev(G)
            stencils.heat_3d_kernel(9, dH, dG)
            cref.heat_3d_kernel(9, H, G)
            assert bits_equal(_host(dH), H) and bits_equal(_host(dG), G)
            A, B = workloads.uniform_pair((20000,), dt, seed=23)
            dA, dB = _dev(A), _dev(B)
            stencils.jacobi_1d_kernel(70, dA, dB)
            cref.jacobi_1d_kernel(70, A, B)
            assert bits_equal(_host(dA), A) and bits_equal(_host(dB), B)
            ex, ey, hz, fict = workloads.init_fdtd_2d(40, 130, 170, dt)
            dev = [_dev(x) for x in (ex, ey, hz, fict)]
            stencils.fdtd_2d_kernel(40, *dev)
            cref.fdtd_2d_kernel(40, ex, ey, hz, fict)
            for d, h in zip(dev[:3], (ex, ey, hz)):
                assert bits_equal(_host(d), h)
    finally:
        _lib.set_config(_lib.NPBGB_CFG_PDL, old)


def test_reference_initializer_presets(golden):
    seen = 0
    for c in golden[0]["cases"]:
        if c.get("init") != "reference":
            continue
        if c["bench"] == "fdtd_2d":
            ex, ey, hz, fict = workloads.init_fdtd_2d(c["TMAX"], c["NX"], c["NY"],
                                                      np.dtype(c["dtype"]).type)
            dev = [_dev(x) for x in (ex, ey, hz, fict)]
            stencils.fdtd_2d_kernel(c["tsteps"], *dev)
            assert [_sha(_host(x)) for x in dev[:3]] == [c["sha_ex_out"], c["sha_ey_out"],
                                                         c["sha_hz_out"]], c["name"]
        elif c["bench"] == "hdiff":
            inf, out, coeff = workloads.init_hdiff(*c["shape"])
            o = _dev(out)
            stencils.hdiff(_dev(inf), o, _dev(coeff))
            assert _sha(_host(o)) == c["sha_out"], c["name"]
        elif c["bench"] == "channel_flow":
            ny, nx = c["shape"]
            u, v, p, dx, dy, dt = workloads.init_channel_flow(ny, nx)
            dev = [_dev(x) for x in (u, v, p)]
            steps = stencils.channel_flow(c["nit"], dev[0], dev[1], dt, dx, dy, dev[2], c["rho"],
                                          c["nu"], c["F"])
            assert steps == c["steps"], c["name"]
            assert [_sha(_host(x)) for x in dev] == [c["sha_u"], c["sha_v"], c["sha_p"]], c["name"]
        elif c["bench"] == "cavity_flow":
            ny, nx = c["shape"]
            u, v, p, dx, dy, dt = workloads.init_cavity_flow(ny, nx)
            dev = [_dev(x) for x in (u, v, p)]
            stencils.cavity_flow(nx, ny, c["nt"], c["nit"], dev[0], dev[1], dt, dx, dy, dev[2],
                                 c["rho"], c["nu"])
            assert [_sha(_host(x)) for x in dev] == [c["sha_u"], c["sha_v"], c["sha_p"]], c["name"]
        elif c["bench"] == "vadv":
            dtr, us, u, w, up, ut = workloads.init_vadv(c["I"], c["J"], c["K"])
            d = _dev(us)
            stencils.vadv(d, _dev(u), _dev(w), _dev(up), _dev(ut), dtr)
            assert _sha(_host(d)) == c["sha_out"], c["name"]
        else:
            A, B = INITS[c["bench"]](c["N"], np.dtype(c["dtype"]).type)
            dA, dB = _dev(A), _dev(B)
            KERNELS[c["bench"]](c["tsteps"], dA, dB)
            assert _sha(_host(dA)) == c["sha_A_out"], c["name"]
            assert _sha(_host(dB)) == c["sha_B_out"], c["name"]
        seen += 1
    assert seen == 12


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_jacobi_1d_paper_size_vs_oracle(dtype):
    A, B = workloads.uniform_pair((32000,), dtype, seed=15)
    dA, dB = _dev(A), _dev(B)
    stencils.jacobi_1d_kernel(4000, dA, dB)
    cref.jacobi_1d_kernel(4000, A, B)
    assert bits_equal(_host(dA), A) and bits_equal(_host(dB), B)
    # Sizes that select each segment width (128, 256, 512, 1024 points per CTA).
    for n, T in ((3, 5), (1026, 17), (2049, 34), (5000, 3), (50000, 40), (400000, 9)):
        A, B = workloads.uniform_pair((n,), dtype, seed=n)
        dA, dB = _dev(A), _dev(B)
        stencils.jacobi_1d_kernel(T, dA, dB)
        cref.jacobi_1d_kernel(T, A, B)
        assert bits_equal(_host(dA), A) and bits_equal(_host(dB), B), (n, T)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_fdtd_paper_size_vs_oracle(dtype):
    ex, ey, hz, fict = workloads.init_fdtd_2d(500, 1000, 1200, dtype)
    rng = np.random.default_rng(16)
    ex, ey, hz = (rng.random(ex.shape).astype(dtype) for _ in range(3))
    dev = [_dev(x) for x in (ex, ey, hz, fict)]
    stencils.fdtd_2d_kernel(500, *dev)
    cref.fdtd_2d_kernel(500, ex, ey, hz, fict)
    for d, h in zip(dev[:3], (ex, ey, hz)):
        assert bits_equal(_host(d), h), first_diff(_host(d), h)


def test_fdtd_rejects_short_fict():
    ex = torch.zeros((4, 5), dtype=torch.float64, device=DEV)
    with pytest.raises(IndexError):
        stencils.fdtd_2d_kernel(3, ex, ex.clone(), ex.clone(), torch.zeros(2, dtype=torch.float64,
                                                                             device=DEV))


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_jacobi_full_size_vs_oracle(dtype):
    A, B = workloads.uniform_pair((1000, 1000), dtype, seed=11)
    dA, dB = _dev(A), _dev(B)
    stencils.jacobi_2d_kernel(100, dA, dB)
    cref.jacobi_2d_kernel(100, A, B)
    assert bits_equal(_host(dA), A), first_diff(_host(dA), A)
    assert bits_equal(_host(dB), B)


@pytest.mark.parametrize("shape,tsteps", [((2800, 2800), 30), ((4096, 4096), 12), ((3000, 4098), 5)])
def test_jacobi_beyond_l2_vs_oracle(shape, tsteps):
    """Binary64 grids whose pair the L2 does not hold take each warp's TMA ring (the
    2800^2 paper preset through its shape class's setting, 4096^2 and 3000 x 4098 by the
    size rule): the oracle's bits, with the shipped tuning applied."""
    A, B = workloads.uniform_pair(shape, np.float64, seed=shape[1])
    dA, dB = _dev(A), _dev(B)
    stencils.jacobi_2d_kernel(tsteps, dA, dB)
    _lib.device_status()
    cref.jacobi_2d_kernel(tsteps, A, B)
    assert bits_equal(_host(dA), A), first_diff(_host(dA), A)
    assert bits_equal(_host(dB), B)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_heat_full_size_vs_oracle(dtype):
    A, B = workloads.uniform_heat((256, 256, 256), dtype, seed=12)
    dA, dB = _dev(A), _dev(B)
    stencils.heat_3d_kernel(100, dA, dB)
    cref.heat_3d_kernel(100, A, B)
    assert bits_equal(_host(dA), A), first_diff(_host(dA), A)
    assert bits_equal(_host(dB), B)


def test_hdiff_full_size_vs_oracle():
    inf, out, coeff = workloads.uniform_hdiff(256, 256, 160, seed=13)
    d = _dev(out)
    stencils.hdiff(_dev(inf), d, _dev(coeff))
    cref.hdiff(inf, out, coeff)
    assert bits_equal(_host(d), out), first_diff(_host(d), out)


def test_jacobi_large_grid_plain_adds():
    """Grids of 2^21 cells and more take the fixed-point path with plain integer
    additions (smaller ones issue them as multiply-adds): 1500^2 against the oracle."""
    for dtype in (np.float64, np.float32):
        A, B = workloads.uniform_pair((1500, 1500), dtype, seed=21)
        dA, dB = _dev(A), _dev(B)
        stencils.jacobi_2d_kernel(6, dA, dB)
        cref.jacobi_2d_kernel(6, A, B)
        assert bits_equal(_host(dA), A) and bits_equal(_host(dB), B), dtype


@pytest.mark.parametrize("shape", [(3, 3), (7, 300), (300, 7), (129, 257), (1000, 33)])
def test_jacobi_ragged_shapes(shape):
    for dtype in (np.float64, np.float32):
        A, B = workloads.uniform_pair(shape, dtype, seed=shape[0])
        dA, dB = _dev(A), _dev(B)
        stencils.jacobi_2d_kernel(7, dA, dB)
        cref.jacobi_2d_kernel(7, A, B)
        assert bits_equal(_host(dA), A) and bits_equal(_host(dB), B), (shape, dtype)


@pytest.mark.parametrize("shape", [(3, 3, 3), (3, 40, 70), (70, 3, 40), (33, 65, 3), (37, 45, 131)])
def test_heat_ragged_shapes(shape):
    for dtype in (np.float64, np.float32):
        A, B = workloads.uniform_heat(shape, dtype, seed=sum(shape))
        dA, dB = _dev(A), _dev(B)
        stencils.heat_3d_kernel(5, dA, dB)
        cref.heat_3d_kernel(5, A, B)
        assert bits_equal(_host(dA), A) and bits_equal(_host(dB), B), (shape, dtype)


@pytest.mark.parametrize("IJK", [(1, 1, 1), (3, 17, 2), (17, 3, 33), (9, 9, 64), (64, 64, 160),
                                 (130, 70, 31)])
def test_hdiff_ragged_shapes(IJK):
    inf, out, coeff = workloads.uniform_hdiff(*IJK, seed=sum(IJK))
    d = _dev(out)
    stencils.hdiff(_dev(inf), d, _dev(coeff))
    cref.hdiff(inf, out, coeff)
    assert bits_equal(_host(d), out), (IJK, first_diff(_host(d), out))


def _wide_range(shape, rng):
    """Doubles across the whole binary64 range: random exponents from the
    subnormals to 2^1023, random signs, signed zeros, repeated neighbours (exact
    zero differences) and a few infinities."""
    m = rng.random(shape) + 1.0
    e = rng.integers(-1074, 1024, size=shape)
    v = np.ldexp(m, e) * rng.choice([-1.0, 1.0], size=shape)
    v[rng.random(shape) < 0.08] = 0.0
    v[rng.random(shape) < 0.04] = -0.0
    rep = rng.random(shape) < 0.15
    v[1:][rep[1:]] = v[:-1][rep[1:]]
    v[rng.random(shape) < 0.005] = np.inf
    near = rng.random(shape) < 0.3  # keep many values where the integer path runs
    v[near] = np.ldexp(rng.random(shape) + 0.5, rng.integers(-8, 8, size=shape))[near]
    return v


@pytest.mark.parametrize("ctas,depth", [(1, 2), (1, 32), (2, 48), (4, 64), (8, 16)])
def test_jacobi_1d_launch_shapes_bit_exact(ctas, depth):
    """Every Jacobi-1D launch shape (segments per SM, half-sweeps per launch)
    leaves the oracle's bits, also for sweep counts that are not a multiple of
    the depth."""
    old = (_lib.set_config(_lib.NPBGB_CFG_JACOBI1D_CTAS, ctas),
           _lib.set_config(_lib.NPBGB_CFG_JACOBI1D_DEPTH, depth))
    try:
        for n, T in ((32000, 37), (5000, 50), (40, 9)):
            A, B = workloads.init_jacobi_1d(n, np.float64)
            dA, dB = _dev(A), _dev(B)
            stencils.jacobi_1d_kernel(T, dA, dB)
            cref.jacobi_1d_kernel(T, A, B)
            assert bits_equal(_host(dA), A) and bits_equal(_host(dB), B), (ctas, depth, n, T)
    finally:
        _lib.set_config(_lib.NPBGB_CFG_JACOBI1D_CTAS, old[0])
        _lib.set_config(_lib.NPBGB_CFG_JACOBI1D_DEPTH, old[1])


@pytest.mark.parametrize("mask", [0x000000, 0x00ff00, 0xffffff, 0x55aa55, 0x0f0f0f])
def test_hdiff_integer_pipe_masks_bit_exact(golden, mask):
    """Every NPBGB_CFG_HDIFF_EMU mask (which items use the integer-pipe binary64
    addition) leaves the oracle's bits, on the golden cases (special values
    included) and on inputs spanning the binary64 range."""
    manifest, arrays = golden
    old = _lib.set_config(_lib.NPBGB_CFG_HDIFF_EMU, mask)
    try:
        for c in manifest["cases"]:
            if c["bench"] != "hdiff" or "init" in c:
                continue
            name = c["name"]
            out = _dev(arrays[f"{name}/out_in"])
            stencils.hdiff(_dev(arrays[f"{name}/in"]), out, _dev(arrays[f"{name}/coeff"]))
            assert bits_equal(_host(out), arrays[f"{name}/out"]), (hex(mask), name)
        rng = np.random.default_rng(mask + 7)
        for IJK in [(9, 10, 40), (17, 33, 64)]:
            I, J, K = IJK
            inf = _wide_range((I + 4, J + 4, K), rng)
            coeff = _wide_range((I, J, K), rng)
            out = np.zeros((I, J, K))
            d = _dev(out)
            stencils.hdiff(_dev(inf), d, _dev(coeff))
            cref.hdiff(inf, out, coeff)
            assert bits_equal(_host(d), out), (hex(mask), IJK, first_diff(_host(d), out))
    finally:
        _lib.set_config(_lib.NPBGB_CFG_HDIFF_EMU, old)


def test_host_numpy_arrays_are_updated_in_place(golden):
    _, arrays = golden
    name = "jacobi_2d/float64/33x47/T17"
    a, b = arrays[f"{name}/A_in"].copy(), arrays[f"{name}/B_in"].copy()
    a_id, b_id = id(a), id(b)
    stencils.jacobi_2d_kernel(17, a, b)
    assert id(a) == a_id and id(b) == b_id
    assert bits_equal(a, arrays[f"{name}/A_out"]) and bits_equal(b, arrays[f"{name}/B_out"])
    # non-contiguous host views are handled like NumPy does
    big = np.zeros((12, 12, 12))
    big[::2, ::2, ::2] = np.random.default_rng(1).random((6, 6, 6))
    ref = big[::2, ::2, ::2].copy(), big[::2, ::2, ::2].copy()
    va = big[::2, ::2, ::2]
    vb = va.copy()
    stencils.heat_3d_kernel(4, va, vb)
    cref.heat_3d_kernel(4, *ref)
    assert bits_equal(big[::2, ::2, ::2], ref[0]) and bits_equal(vb, ref[1])


def test_noncontiguous_tensor_keeps_identity():
    A, B = workloads.uniform_pair((40, 60), np.float64, seed=2)
    big = torch.zeros((40, 120), dtype=torch.float64, device=DEV)
    big[:, ::2] = _dev(A)
    view = big[:, ::2]
    dB = _dev(B)
    stencils.jacobi_2d_kernel(6, view, dB)
    cref.jacobi_2d_kernel(6, A, B)
    assert bits_equal(_host(big[:, ::2]), A) and bits_equal(_host(dB), B)
    assert bits_equal(_host(big[:, 1::2]), np.zeros((40, 60)))


def test_cpu_tensor_is_rejected():
    with pytest.raises(ValueError):
        stencils.jacobi_2d_kernel(3, torch.zeros(5, 5, dtype=torch.float64),
                                  torch.zeros(5, 5, dtype=torch.float64))


def test_determinism_across_runs():
    A, B = workloads.uniform_heat((96, 80, 72), np.float64, seed=5)
    outs = []
    for _ in range(2):
        dA, dB = _dev(A), _dev(B)
        stencils.heat_3d_kernel(9, dA, dB)
        outs.append((_host(dA), _host(dB)))
    assert bits_equal(outs[0][0], outs[1][0]) and bits_equal(outs[0][1], outs[1][1])


def _mixed_range_field(shape, seed):
    """U[0,1) with patches outside the fixed-point range: negatives, tiny, >= 1, -0.0."""
    rng = np.random.default_rng(seed)
    a = rng.random(shape)
    flat = a.reshape(-1)
    idx = rng.choice(flat.size, size=flat.size // 50, replace=False)
    pool = np.array([-0.3, 1e-5, 2.5, -0.0, 0.0, 1.0, 3e-300, 0.999999999])
    flat[idx] = pool[rng.integers(0, pool.size, idx.size)]
    return a


@pytest.mark.parametrize("field", ["uniform", "mixed", "scaled"])
def test_heat_f64_integer_and_hardware_paths_agree(field):
    """The fixed-point binary64 path and the hardware path give the oracle's bits."""
    from npbench_gb300 import _lib
    shape = (70, 90, 100)
    if field == "uniform":
        A = workloads.uniform_heat(shape, np.float64, seed=21)[0]
    elif field == "mixed":
        A = _mixed_range_field(shape, 22)
    else:
        A = 3.0 * workloads.uniform_heat(shape, np.float64, seed=23)[0] - 1.0
    ref_a, ref_b = A.copy(), A.copy()
    cref.heat_3d_kernel(6, ref_a, ref_b)
    for emul in (1, 0):
        old = _lib.set_config(_lib.NPBGB_CFG_F64_EMULATION, emul)
        try:
            dA, dB = _dev(A), _dev(A)
            stencils.heat_3d_kernel(6, dA, dB)
            assert bits_equal(_host(dA), ref_a), (field, emul, first_diff(_host(dA), ref_a))
            assert bits_equal(_host(dB), ref_b), (field, emul)
        finally:
            _lib.set_config(_lib.NPBGB_CFG_F64_EMULATION, old)


@pytest.mark.parametrize("chunk", [1, 3, 8, 33, 500])
def test_heat_chunking_does_not_change_bits(chunk):
    from npbench_gb300 import _lib
    A = workloads.uniform_heat((41, 37, 70), np.float64, seed=chunk)[0]
    ref_a, ref_b = A.copy(), A.copy()
    cref.heat_3d_kernel(4, ref_a, ref_b)
    old = _lib.set_config(_lib.NPBGB_CFG_HEAT_CHUNK, chunk)
    try:
        for dt in (np.float64, np.float32):
            a = A.astype(dt)
            ra, rb = a.copy(), a.copy()
            cref.heat_3d_kernel(4, ra, rb)
            dA, dB = _dev(a), _dev(a)
            stencils.heat_3d_kernel(4, dA, dB)
            assert bits_equal(_host(dA), ra) and bits_equal(_host(dB), rb), (chunk, dt)
    finally:
        _lib.set_config(_lib.NPBGB_CFG_HEAT_CHUNK, old)


@pytest.mark.parametrize("tma", [1, 0])
@pytest.mark.parametrize("shape", [(256, 256, 256), (66, 130, 200), (9, 40, 34), (5, 37, 46)])
def test_heat_tma_and_plain_staging(tma, shape):
    """TMA staging (16-byte-aligned rows) and plain staging give the oracle's bits."""
    from npbench_gb300 import _lib
    old = _lib.set_config(_lib.NPBGB_CFG_HEAT_TMA, tma)
    try:
        for dtype in (np.float64, np.float32):
            A = _mixed_range_field(shape, 31).astype(dtype) if shape[0] < 100 else \
                workloads.uniform_heat(shape, dtype, seed=30)[0]
            ra, rb = A.copy(), A.copy()
            T = 3 if shape[0] == 256 else 7
            cref.heat_3d_kernel(T, ra, rb)
            dA, dB = _dev(A), _dev(A)
            stencils.heat_3d_kernel(T, dA, dB)
            _lib.device_status()
            assert bits_equal(_host(dA), ra), (tma, shape, dtype, first_diff(_host(dA), ra))
            assert bits_equal(_host(dB), rb), (tma, shape, dtype)
    finally:
        _lib.set_config(_lib.NPBGB_CFG_HEAT_TMA, old)


@pytest.mark.parametrize("field", ["uniform", "mixed", "scaled"])
def test_jacobi_f64_integer_and_hardware_paths_agree(field):
    from npbench_gb300 import _lib
    shape = (300, 517)
    if field == "uniform":
        A, B = workloads.uniform_pair(shape, np.float64, seed=41)
    elif field == "mixed":
        A, B = _mixed_range_field(shape, 42), _mixed_range_field(shape, 43)
    else:
        A, B = (4.0 * x - 2.0 for x in workloads.uniform_pair(shape, np.float64, seed=44))
    ra, rb = A.copy(), B.copy()
    cref.jacobi_2d_kernel(9, ra, rb)
    for emul in (1, 0):
        old = _lib.set_config(_lib.NPBGB_CFG_F64_EMULATION, emul)
        try:
            dA, dB = _dev(A), _dev(B)
            stencils.jacobi_2d_kernel(9, dA, dB)
            assert bits_equal(_host(dA), ra), (field, emul, first_diff(_host(dA), ra))
            assert bits_equal(_host(dB), rb), (field, emul)
        finally:
            _lib.set_config(_lib.NPBGB_CFG_F64_EMULATION, old)


@pytest.mark.parametrize("tma", [2, 0])
@pytest.mark.parametrize("shape", [(300, 518), (37, 46), (5, 8), (130, 4), (1000, 1000)])
def test_jacobi_tma_ring_and_plain_loads(tma, shape):
    """Each warp's TMA ring (forced on every grid whose rows are 16-byte multiples)
    and the plain-load strips give the oracle's bits: binary64 in fixed point and on
    hardware, with uniform and mixed-range fields, and binary32; odd widths fall back
    to the plain loads, chunks of 1 and 7 rows leave partial boxes."""
    from npbench_gb300 import autotune
    keys = (_lib.NPBGB_CFG_JACOBI_TMA, _lib.NPBGB_CFG_JACOBI_CHUNK)
    was = autotune.enabled()
    autotune.disable()
    try:
        for chunk in (0, 1, 7):
            old = [_lib.set_config(k, v) for k, v in zip(keys, (tma, chunk))]
            try:
                cases = [(np.float64, "uniform", 1), (np.float64, "mixed", 1),
                         (np.float64, "uniform", 0), (np.float32, "uniform", 1)]
                for dt, field, emul in cases:
                    A, B = (workloads.uniform_pair(shape, dt, seed=shape[0] + chunk)
                            if field == "uniform"
                            else (_mixed_range_field(shape, 90), _mixed_range_field(shape, 91)))
                    T = 4 if shape[0] == 1000 else 7
                    ra, rb = A.copy(), B.copy()
                    cref.jacobi_2d_kernel(T, ra, rb)
                    old_e = _lib.set_config(_lib.NPBGB_CFG_F64_EMULATION, emul)
                    try:
                        dA, dB = _dev(A), _dev(B)
                        stencils.jacobi_2d_kernel(T, dA, dB)
                        _lib.device_status()
                    finally:
                        _lib.set_config(_lib.NPBGB_CFG_F64_EMULATION, old_e)
                    assert bits_equal(_host(dA), ra), (tma, shape, chunk, dt, field, emul,
                                                       first_diff(_host(dA), ra))
                    assert bits_equal(_host(dB), rb), (tma, shape, chunk, dt, field, emul)
            finally:
                for k, v in zip(keys, old):
                    _lib.set_config(k, v)
    finally:
        if was:
            autotune.enable()


@pytest.mark.parametrize("chunk", [1, 5, 64, 4000])
def test_jacobi_chunking_does_not_change_bits(chunk):
    from npbench_gb300 import _lib
    old = _lib.set_config(_lib.NPBGB_CFG_JACOBI_CHUNK, chunk)
    try:
        for dt in (np.float64, np.float32):
            A, B = workloads.uniform_pair((123, 301), dt, seed=chunk)
            ra, rb = A.copy(), B.copy()
            cref.jacobi_2d_kernel(5, ra, rb)
            dA, dB = _dev(A), _dev(B)
            stencils.jacobi_2d_kernel(5, dA, dB)
            assert bits_equal(_host(dA), ra) and bits_equal(_host(dB), rb), (chunk, dt)
    finally:
        _lib.set_config(_lib.NPBGB_CFG_JACOBI_CHUNK, old)


def test_bounded_device_wait_reports_timeout_and_context_survives():
    """A wait that nothing completes gives up after its limit; the host reads the status."""
    from npbench_gb300 import _lib
    lib = _lib.load()
    _lib.device_status()  # clean slate
    st = torch.cuda.current_stream().cuda_stream
    assert lib.npbgb_selftest_wait_timeout(20_000_000, st) == _lib.NPBGB_OK  # 20 ms
    with pytest.raises(_lib.NpbgbError) as ei:
        _lib.device_status()
    assert ei.value.status == _lib.NPBGB_ERR_TIMEOUT
    _lib.device_status()  # cleared after being reported
    # the context is still usable
    A, B = workloads.uniform_pair((50, 60), np.float64, seed=1)
    dA, dB = _dev(A), _dev(B)
    stencils.jacobi_2d_kernel(3, dA, dB)
    cref.jacobi_2d_kernel(3, A, B)
    assert bits_equal(_host(dA), A)


@pytest.mark.parametrize("rows,cvt,hw,mad", [(1, 0, 0, 0), (2, 0, 0, 0), (2, 1, 0, 5), (4, 1, 3, 0),
                                             (2, 0, 4, 0), (4, 0, 32, 0), (2, 0, 7, 4),
                                             (2, 0, 7, 9), (1, 0, 3, 8), (4, 1, 8, 24)])
def test_heat_kernel_variants_bit_exact(rows, cvt, hw, mad):
    """Every heat3d variant (rows per thread, conversion path, hardware rows, fixed-point
    rows with their adds on the multiply-add pipe) gives the oracle's bits."""
    from npbench_gb300 import _lib
    keys = (_lib.NPBGB_CFG_HEAT_ROWS, _lib.NPBGB_CFG_F64_CVT, _lib.NPBGB_CFG_HEAT_HW_ROWS,
            _lib.NPBGB_CFG_HEAT_MAD_ROWS)
    old = [_lib.set_config(k, v) for k, v in zip(keys, (rows, cvt, hw, mad))]
    try:
        for dtype in (np.float64, np.float32):
            for field in ("uniform", "mixed"):
                shape = (34, 70, 100)
                A = (workloads.uniform_heat(shape, dtype, seed=rows)[0] if field == "uniform"
                     else _mixed_range_field(shape, 50 + rows).astype(dtype))
                ra, rb = A.copy(), A.copy()
                cref.heat_3d_kernel(5, ra, rb)
                dA, dB = _dev(A), _dev(A)
                stencils.heat_3d_kernel(5, dA, dB)
                _lib.device_status()
                assert bits_equal(_host(dA), ra), (rows, cvt, hw, mad, dtype, field,
                                                   first_diff(_host(dA), ra))
                assert bits_equal(_host(dB), rb)
    finally:
        for k, v in zip(keys, old):
            _lib.set_config(k, v)


@pytest.mark.parametrize("hw_warps", [0, 1, 3, 8])
def test_jacobi_hw_warp_mix_bit_exact(hw_warps):
    from npbench_gb300 import _lib
    old = _lib.set_config(_lib.NPBGB_CFG_JACOBI_HW_WARPS, hw_warps)
    try:
        for field in ("uniform", "mixed"):
            shape = (200, 1100)
            A, B = (workloads.uniform_pair(shape, np.float64, seed=hw_warps) if field == "uniform"
                    else (_mixed_range_field(shape, 60), _mixed_range_field(shape, 61)))
            ra, rb = A.copy(), B.copy()
            cref.jacobi_2d_kernel(6, ra, rb)
            dA, dB = _dev(A), _dev(B)
            stencils.jacobi_2d_kernel(6, dA, dB)
            assert bits_equal(_host(dA), ra) and bits_equal(_host(dB), rb), (hw_warps, field)
    finally:
        _lib.set_config(_lib.NPBGB_CFG_JACOBI_HW_WARPS, old)


@pytest.mark.parametrize("adds,mul", [(1, 0), (2, 1), (3, 1), (3, 2), (1, 2), (0, 2), (2, 0)])
@pytest.mark.parametrize("hw_warps", [0, 3, 8])
def test_jacobi_f64_add_and_product_forms_bit_exact(adds, mul, hw_warps):
    """Binary64 Jacobi-2D with each form of the fixed-point additions (integer adds,
    multiply-add 64-bit adds, rounding on the multiply-add pipe) and of the product by
    0.2 (hardware, integer for the fixed-point points, integer for every point), on
    uniform fields and on fields with negatives, -0.0, tiny, subnormal and >= 1 values."""
    from npbench_gb300 import _lib, autotune
    keys = (_lib.NPBGB_CFG_JACOBI_FX_ADDS, _lib.NPBGB_CFG_JACOBI_FX_MUL,
            _lib.NPBGB_CFG_JACOBI_HW_WARPS)
    old = [_lib.set_config(k, v) for k, v in zip(keys, (adds, mul, hw_warps))]
    was = autotune.enabled()
    autotune.disable()
    try:
        for field in ("uniform", "mixed"):
            for shape in ((200, 1100), (37, 45)):
                A, B = (workloads.uniform_pair(shape, np.float64, seed=adds + mul)
                        if field == "uniform"
                        else (_mixed_range_field(shape, 70 + adds), _mixed_range_field(shape, 80 + mul)))
                ra, rb = A.copy(), B.copy()
                cref.jacobi_2d_kernel(6, ra, rb)
                dA, dB = _dev(A), _dev(B)
                stencils.jacobi_2d_kernel(6, dA, dB)
                assert bits_equal(_host(dA), ra) and bits_equal(_host(dB), rb), (field, shape)
    finally:
        for k, v in zip(keys, old):
            _lib.set_config(k, v)
        if was:
            autotune.enable()


@pytest.mark.parametrize("bench,shape,tsteps", [("jacobi_2d", (1000, 1000), 10),
                                                ("jacobi_2d", (1000, 1000), 100),
                                                ("heat_3d", (256, 256, 256), 10),
                                                ("heat_3d", (256, 256, 256), 100)])
def test_fp32_form_error_against_fp64(bench, shape, tsteps):
    """The float32 form: max-abs and relative-L2 error against the float64 run (<= 1e-5)."""
    if bench == "jacobi_2d":
        A, B = workloads.uniform_pair(shape, np.float64, seed=70)
        kern = stencils.jacobi_2d_kernel
    else:
        A, B = workloads.uniform_heat(shape, np.float64, seed=71)
        kern = stencils.heat_3d_kernel
    d64 = (_dev(A), _dev(B))
    d32 = (_dev(A.astype(np.float32)), _dev(B.astype(np.float32)))
    kern(tsteps, *d64)
    kern(tsteps, *d32)
    ref = d64[0]
    diff = d32[0].double() - ref
    max_abs = float(diff.abs().max())
    rel_l2 = float(diff.norm() / ref.norm())
    print(f"\nfp32-vs-fp64 {bench} {shape} TSTEPS={tsteps}: max_abs={max_abs:.3e} rel_l2={rel_l2:.3e}")
    assert rel_l2 <= 1e-5 and max_abs < 1e-4


@pytest.mark.parametrize("shape", [(3, 3, 4), (4, 5, 8), (18, 34, 36), (40, 70, 68), (67, 33, 100),
                                   (128, 130, 132), (9, 300, 44)])
@pytest.mark.parametrize("tsteps", [4, 5, 6, 7, 12])
def test_heat_f32_two_steps_per_launch(shape, tsteps):
    """Binary32 Heat-3D with two half-sweeps per launch (temporal blocking) gives the
    oracle's bits, also when A and B start with different faces (B's faces are the
    odd steps' faces) and whatever the number of planes per CTA."""
    from npbench_gb300 import _lib
    rng = np.random.default_rng(sum(shape) + tsteps)
    A = rng.random(shape).astype(np.float32)
    B = rng.random(shape).astype(np.float32)  # distinct faces
    ra, rb = A.copy(), B.copy()
    cref.heat_3d_kernel(tsteps, ra, rb)
    old = (_lib.get_config(_lib.NPBGB_CFG_HEAT_TB), _lib.get_config(_lib.NPBGB_CFG_HEAT_TB_CHUNK))
    try:
        for tb, chunk in ((2, 0), (2, 1), (2, 5), (1, 0)):
            _lib.set_config(_lib.NPBGB_CFG_HEAT_TB, tb)
            _lib.set_config(_lib.NPBGB_CFG_HEAT_TB_CHUNK, chunk)
            dA, dB = _dev(A), _dev(B)
            stencils.heat_3d_kernel(tsteps, dA, dB)
            _lib.device_status()
            assert bits_equal(_host(dA), ra), (tb, chunk, first_diff(_host(dA), ra))
            assert bits_equal(_host(dB), rb), (tb, chunk, first_diff(_host(dB), rb))
    finally:
        _lib.set_config(_lib.NPBGB_CFG_HEAT_TB, old[0])
        _lib.set_config(_lib.NPBGB_CFG_HEAT_TB_CHUNK, old[1])


@pytest.mark.parametrize("n,tb", [(384, 2), (416, 0)])
def test_heat_f32_two_steps_full_size_out_of_l2(n, tb):
    """Binary32 grids beyond L2 against the oracle: 384^3 with the two-step kernel
    forced; 416^3 (275 MB per array) with the automatic choice (one step, 4-plane
    chunks) at each depth of the shared-memory plane ring."""
    from npbench_gb300 import _lib
    A0, B0 = workloads.uniform_heat((n, n, n), np.float32, seed=33)
    A, B = A0.copy(), B0.copy()
    cref.heat_3d_kernel(10, A, B)
    old = (_lib.set_config(_lib.NPBGB_CFG_HEAT_TB, tb),
           _lib.get_config(_lib.NPBGB_CFG_HEAT_STAGES))
    try:
        for stages in ((0,) if tb == 2 else (0, 4, 6, 8)):
            _lib.set_config(_lib.NPBGB_CFG_HEAT_STAGES, stages)
            dA, dB = _dev(A0), _dev(B0)
            stencils.heat_3d_kernel(10, dA, dB)
            _lib.device_status()
            assert bits_equal(_host(dA), A), (stages, first_diff(_host(dA), A))
            assert bits_equal(_host(dB), B), stages
            del dA, dB
    finally:
        _lib.set_config(_lib.NPBGB_CFG_HEAT_TB, old[0])
        _lib.set_config(_lib.NPBGB_CFG_HEAT_STAGES, old[1])


@pytest.mark.parametrize("stages", [4, 6, 8])
@pytest.mark.parametrize("chunk", [0, 1, 3, 4, 9])
def test_heat_f32_plane_ring_depths(stages, chunk):
    """The binary32 TMA kernel at each ring depth and plane chunk, ragged shapes, against
    the oracle."""
    from npbench_gb300 import _lib
    old = (_lib.get_config(_lib.NPBGB_CFG_HEAT_STAGES), _lib.get_config(_lib.NPBGB_CFG_HEAT_CHUNK))
    try:
        _lib.set_config(_lib.NPBGB_CFG_HEAT_STAGES, stages)
        _lib.set_config(_lib.NPBGB_CFG_HEAT_CHUNK, chunk)
        for shape in ((5, 6, 8), (37, 45, 68), (70, 33, 100)):
            A = workloads.uniform_heat(shape, np.float32, seed=stages + chunk)[0]
            ra, rb = A.copy(), A.copy()
            cref.heat_3d_kernel(7, ra, rb)
            dA, dB = _dev(A), _dev(A)
            stencils.heat_3d_kernel(7, dA, dB)
            _lib.device_status()
            assert bits_equal(_host(dA), ra), (shape, first_diff(_host(dA), ra))
            assert bits_equal(_host(dB), rb), shape
    finally:
        _lib.set_config(_lib.NPBGB_CFG_HEAT_STAGES, old[0])
        _lib.set_config(_lib.NPBGB_CFG_HEAT_CHUNK, old[1])


@pytest.mark.parametrize("shape", [(5, 5), (300, 7), (7, 300), (157, 1000), (1000, 1000),
                                   (1500, 900), (160, 2053)])
@pytest.mark.parametrize("tsteps", [2, 3, 9, 60])
def test_jacobi_bands_in_shared_memory(shape, tsteps):
    """The whole Jacobi-2D time loop in one launch, bands of rows resident in shared
    memory (on, with the warps per CTA by width and forced to 8 and 32), against the
    oracle, as the chained launches (the default) are, in both precisions; A and B
    start with different faces."""
    from npbench_gb300 import _lib
    old = (_lib.get_config(_lib.NPBGB_CFG_JACOBI_BANDS),
           _lib.get_config(_lib.NPBGB_CFG_JACOBI_BANDS_WARPS))
    try:
        for dtype in (np.float64, np.float32):
            A, B = workloads.uniform_pair(shape, dtype, seed=sum(shape) + tsteps)
            ra, rb = A.copy(), B.copy()
            cref.jacobi_2d_kernel(tsteps, ra, rb)
            for mode, warps in ((2, 0), (2, 8), (2, 32), (0, 0)):
                _lib.set_config(_lib.NPBGB_CFG_JACOBI_BANDS, mode)
                _lib.set_config(_lib.NPBGB_CFG_JACOBI_BANDS_WARPS, warps)
                dA, dB = _dev(A), _dev(B)
                stencils.jacobi_2d_kernel(tsteps, dA, dB)
                _lib.device_status()
                assert bits_equal(_host(dA), ra), (mode, warps, dtype, first_diff(_host(dA), ra))
                assert bits_equal(_host(dB), rb), (mode, warps, dtype, first_diff(_host(dB), rb))
    finally:
        _lib.set_config(_lib.NPBGB_CFG_JACOBI_BANDS, old[0])
        _lib.set_config(_lib.NPBGB_CFG_JACOBI_BANDS_WARPS, old[1])


def test_launch_counter_matches_the_paths_taken():
    """The library's launch counter: Jacobi-2D 1000^2 at TSTEPS=100 is 198 chained
    launches, or one with the bands in shared memory; a batch graph counts its kernels
    at each replay."""
    import torch
    from npbench_gb300 import _lib, autotune
    from npbench_gb300.batch import Batch
    was = autotune.enabled()
    autotune.disable()
    try:
        for dt, bands, want in ((np.float64, 0, 198), (np.float64, 2, 1), (np.float32, 0, 198)):
            old = _lib.set_config(_lib.NPBGB_CFG_JACOBI_BANDS, bands)
            A, B = workloads.uniform_pair((1000, 1000), dt, seed=5)
            dA, dB = _dev(A), _dev(B)
            torch.cuda.synchronize()
            n0 = _lib.launches()
            stencils.jacobi_2d_kernel(100, dA, dB)
            torch.cuda.synchronize()
            _lib.set_config(_lib.NPBGB_CFG_JACOBI_BANDS, old)
            assert _lib.launches() - n0 == want, (dt, bands)
    finally:
        if was:
            autotune.enable()
    grids = [_dev(x) for x in workloads.uniform_pair((100, 90), np.float64, seed=6)]
    with Batch([(grids[0], grids[1], 5)], mode="stepped") as b:
        b.launch(graph=True)
        torch.cuda.synchronize()
        n0 = _lib.launches()
        b.launch(graph=True)
        b.launch(graph=True)
        torch.cuda.synchronize()
        assert b.info()["ctas"] == 8  # stepped form: one launch per half-sweep
        assert _lib.launches() - n0 == 2 * 8
