"""GPU parity: the sm_103a drop-in against the oracle and the reference fixtures.

FP64 tolerance: relative L2 <= 1e-12 in vorticity (the bar for the plain FP64
path).  Everything here calls the product through its C-ABI / drop-in API.
"""
import numpy as np
import pytest

from conftest import golden, rel_l2, tg_vorticity, random_field

import oracle as O

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _gpu(nsgb, nx, ny, Re=100.0, prec=0):
    return nsgb.Solver(nx, ny, Re=Re, precision=prec).setup(ic=None)


def test_config1_tg32_compat_path(nsgb):
    g = golden("config1_tg32.npz")
    s = _gpu(nsgb, 32, 32)
    s.set_vorticity(tg_vorticity(32, 32))
    s.derivatives()
    s.d.dt = 1e-3
    s.advance(100)
    assert rel_l2(s.cplx("omega_hat"), g["omega_hat"]) <= TOL
    assert abs(s.d.t - float(g["t"])) <= 1e-15
    assert abs(s.energy() - float(g["energy"])) <= 1e-13 * abs(float(g["energy"]))
    assert abs(s.enstrophy() - float(g["enstrophy"])) <= 1e-13 * abs(float(g["enstrophy"]))
    assert rel_l2(s.real("u")[32 // 3], g["u_row"]) <= TOL
    assert rel_l2(s.real("v")[32 // 5], g["v_row"]) <= TOL
    assert rel_l2(s.real("omega")[32 // 7], g["omega_row"]) <= TOL


def test_config1_tg128_device_resident(nsgb):
    """Config 1 (128^2, FP64, nu = 0.01, dt = 1e-3, 1000 steps) through advance_n."""
    g = golden("config1_tg128.npz")
    s = _gpu(nsgb, 128, 128)
    s.set_vorticity(tg_vorticity(128, 128))
    s.derivatives()
    s.d.dt = 1e-3
    s.advance_n(1000)
    s.sync_host()
    assert rel_l2(s.cplx("omega_hat"), g["omega_hat"]) <= TOL
    assert rel_l2(s.cplx("psi_hat"), g["psi_hat"]) <= TOL
    assert abs(s.d.t - float(g["t"])) <= 1e-12
    # analytic decay omega(t) = omega0 exp(-2 nu t)
    w0 = np.fft.rfft2(tg_vorticity(128, 128)) / 128 ** 2
    assert rel_l2(s.cplx("omega_hat"), w0 * np.exp(-0.02 * s.d.t)) < 1e-9


def test_random_hv_sfd_reference_loop(nsgb):
    """dt = cfl(); advance_rk4() loop with hyperviscosity + SFD (the reference test loop)."""
    g = golden("random64_hv_sfd.npz")
    s = _gpu(nsgb, 64, 64, Re=1000.0)
    s.set_vorticity(g["omega0"])
    s.derivatives()
    s.set_hyperviscosity(enabled=1, coefficient=0.5, order=4, cutoff_ratio=0.5, sfd_enabled=1, sfd_strength=0.2,
                         sfd_timescale=0.3)
    w = np.ctypeslib.as_array(s.d.hyperviscosity_weights, shape=(64, 33))
    assert rel_l2(w, g["weights"]) <= 1e-14
    s.d.cfl_factor = 0.5
    dts = []
    for _ in range(len(g["dts"])):
        s.d.dt = s.cfl()
        dts.append(s.d.dt)
        s.advance(1)
    assert np.allclose(dts, g["dts"], rtol=1e-12, atol=0)
    assert rel_l2(s.cplx("omega_hat"), g["omega_hat"]) <= TOL
    assert rel_l2(s.cplx("sfd_hat"), g["sfd_hat"]) <= TOL


def test_random_hv_sfd_device_adaptive(nsgb):
    """Same run with the CFL dt computed on the device inside advance_n."""
    g = golden("random64_hv_sfd.npz")
    s = _gpu(nsgb, 64, 64, Re=1000.0)
    s.set_vorticity(g["omega0"])
    s.derivatives()
    s.set_hyperviscosity(enabled=1, coefficient=0.5, order=4, cutoff_ratio=0.5, sfd_enabled=1, sfd_strength=0.2,
                         sfd_timescale=0.3)
    s.d.cfl_factor = 0.5
    s.advance_n(len(g["dts"]), adaptive=True)
    s.sync_host()
    assert abs(s.d.t - float(g["t"])) <= 1e-12 * float(g["t"])
    assert rel_l2(s.cplx("omega_hat"), g["omega_hat"]) <= TOL


# ---- grids that are not powers of two (mixed-radix transforms; odd nx runs the
# full-length row transform).  The reference computes at any size; its
# benchmark's 192^2 case is config-1 physics for 150 steps
# (performance_benchmark.c:103).
HV_SFD = dict(enabled=1, coefficient=0.5, order=4, cutoff_ratio=0.5, sfd_enabled=1, sfd_strength=0.2,
              sfd_timescale=0.3)
HV_ONLY = dict(enabled=1, coefficient=0.3, order=8, cutoff_ratio=0.65)
NON_POW2 = [("random96x64_hv_sfd.npz", 96, 64, HV_SFD), ("random45x30_hv.npz", 45, 30, HV_ONLY)]


@pytest.mark.parametrize("device_resident", [False, True])
def test_config1_tg192_benchmark_grid(nsgb, device_resident):
    g = golden("config1_tg192.npz")
    s = _gpu(nsgb, 192, 192)
    s.set_vorticity(tg_vorticity(192, 192))
    s.derivatives()
    s.d.dt = 1e-3
    if device_resident:
        s.advance_n(150)
        s.sync_host()
    else:
        s.advance(150)
    assert rel_l2(s.cplx("omega_hat"), g["omega_hat"]) <= TOL
    assert abs(s.d.t - float(g["t"])) <= 1e-12
    assert abs(s.energy() - float(g["energy"])) <= 1e-13 * abs(float(g["energy"]))
    assert abs(s.enstrophy() - float(g["enstrophy"])) <= 1e-13 * abs(float(g["enstrophy"]))
    assert rel_l2(s.real("omega")[192 // 7], g["omega_row"]) <= TOL


@pytest.mark.parametrize("name,nx,ny,hv", NON_POW2)
def test_random_non_pow2_reference_loop(nsgb, name, nx, ny, hv):
    """dt = cfl(); advance_rk4() with hyperviscosity (and SFD) on a 96 x 64 grid
    (row transform 48 = 16 * 3) and a 45 x 30 grid (odd nx: 45 = 9 * 5)."""
    g = golden(name)
    s = _gpu(nsgb, nx, ny, Re=1000.0)
    s.set_vorticity(g["omega0"])
    s.derivatives()
    s.set_hyperviscosity(**hv)
    w = np.ctypeslib.as_array(s.d.hyperviscosity_weights, shape=(ny, nx // 2 + 1))
    assert rel_l2(w, g["weights"]) <= 1e-14
    s.d.cfl_factor = 0.5
    dts = []
    for _ in range(len(g["dts"])):
        s.d.dt = s.cfl()
        dts.append(s.d.dt)
        s.advance(1)
    assert np.allclose(dts, g["dts"], rtol=1e-12, atol=0)
    assert rel_l2(s.cplx("omega_hat"), g["omega_hat"]) <= TOL
    if hv.get("sfd_enabled"):
        assert rel_l2(s.cplx("sfd_hat"), g["sfd_hat"]) <= TOL


@pytest.mark.parametrize("name,nx,ny,hv", NON_POW2)
def test_random_non_pow2_device_adaptive(nsgb, name, nx, ny, hv):
    g = golden(name)
    s = _gpu(nsgb, nx, ny, Re=1000.0)
    s.set_vorticity(g["omega0"])
    s.derivatives()
    s.set_hyperviscosity(**hv)
    s.d.cfl_factor = 0.5
    s.advance_n(len(g["dts"]), adaptive=True)
    s.sync_host()
    assert abs(s.d.t - float(g["t"])) <= 1e-12 * float(g["t"])
    assert rel_l2(s.cplx("omega_hat"), g["omega_hat"]) <= TOL


@pytest.mark.parametrize("nx,ny", [(192, 192), (96, 64), (45, 30), (62, 31), (98, 21)])
def test_non_pow2_fp32_against_fp64_oracle(nsgb, port, nx, ny):
    """FP32 bulk on mixed-radix grids (a factor 31 and a factor 7 included) against
    the FP64 oracle after 5 steps: relative L2 <= 1e-5."""
    w = random_field(nx, ny, 12)
    gpu = _gpu(nsgb, nx, ny, Re=500.0, prec=nsgb.FP32)
    ora = O.Solver(port, nx, ny, Re=500.0).setup(ic=None)
    for x in (gpu, ora):
        x.set_vorticity(w)
        x.derivatives()
        x.d.dt = 2e-3
    gpu.advance_n(5)
    gpu.sync_host()
    ora.advance(5)
    assert rel_l2(gpu.cplx("omega_hat"), ora.cplx("omega_hat")) <= 1e-5


def test_nonlinear_terms_non_square(nsgb):
    g = golden("nonlinear_32x16.npz")
    s = _gpu(nsgb, 32, 16)
    s.cplx("omega_hat")[:] = g["omega_hat"]
    s.cplx("psi_hat")[:] = g["psi_hat"]
    s._f("compute_nonlinear_terms")(s.ptr)
    assert rel_l2(s.cplx("nonlinear_hat"), g["nonlinear_hat"]) <= TOL
    assert rel_l2(s.real("p"), g["jac"]) <= TOL


@pytest.mark.parametrize("nx,ny", [(8, 8), (32, 32), (64, 16), (16, 128), (256, 256), (192, 192), (96, 64), (45, 30),
                                   (12, 10), (62, 31), (98, 21), (9, 15)])
def test_transforms_match_oracle(nsgb, port, nx, ny):
    f = np.random.default_rng(nx + ny).standard_normal((ny, nx))
    s = _gpu(nsgb, nx, ny)
    o = O.Solver(port, nx, ny).setup(ic=None)
    for x in (s, o):
        x.real("p")[:] = f
        x._f("physical_to_spectral")(x.ptr, x.d.p, x.d.u_hat)
    assert rel_l2(s.cplx("u_hat"), o.cplx("u_hat")) <= 1e-14
    for x in (s, o):
        x._f("spectral_to_physical")(x.ptr, x.d.u_hat, x.d.v)
    assert rel_l2(s.real("v"), o.real("v")) <= 1e-14
    # the reference leaves the dealiased input in nonlinear_hat (spectral_transforms.c:27-30)
    assert np.array_equal(s.cplx("nonlinear_hat"), s.cplx("u_hat") * s.mask())
