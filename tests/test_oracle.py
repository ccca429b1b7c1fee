"""CPU tests of the oracle itself: pin it before trusting it.

* the FFTW-API shim against numpy's pocketfft (r2c/c2r, 2-D, odd/even sizes);
* the C restatement against the golden fixtures produced by the reference's own
  sources (tests/golden/make_golden.py), and bit-for-bit against the reference
  build when that build exists in this checkout;
* Philox4x64-10 against numpy.random.Philox;
* the reference test assertions that hold (and the ones the reference code
  itself cannot meet, documented here).
"""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import golden, rel_l2, tg_vorticity, random_field

import oracle as O


def _solver(port, nx, ny, Re=100.0):
    return O.Solver(port, nx, ny, Re=Re).setup(ic=None)


SHIM_SIZES_MIXED = [(12, 10), (192, 192), (96, 64), (45, 30), (98, 21), (62, 31)]


@pytest.mark.parametrize("nx,ny", [(32, 32), (64, 16), (128, 64), (8, 8)] + SHIM_SIZES_MIXED)
def test_shim_r2c_matches_numpy(port, nx, ny):
    s = _solver(port, nx, ny)
    f = np.random.default_rng(0).standard_normal((ny, nx))
    s.real("p")[:] = f
    s._f("physical_to_spectral")(s.ptr, s.d.p, s.d.u_hat)
    ref = np.fft.rfft2(f) / (nx * ny) * s.mask()
    assert np.abs(s.cplx("u_hat") - ref).max() <= 1e-14 * np.abs(ref).max()


@pytest.mark.parametrize("nx,ny", [(32, 32), (64, 16), (128, 64)] + SHIM_SIZES_MIXED)
def test_shim_c2r_matches_numpy(port, nx, ny):
    s = _solver(port, nx, ny)
    f = np.random.default_rng(1).standard_normal((ny, nx))
    fh = np.fft.rfft2(f) / (nx * ny) * s.mask()
    s.cplx("u_hat")[:] = fh
    s._f("spectral_to_physical")(s.ptr, s.d.u_hat, s.d.p)
    ref = np.fft.irfft2(fh, s=(ny, nx)) * (nx * ny)
    assert np.abs(s.real("p") - ref).max() <= 1e-14 * np.abs(ref).max()


def test_philox_matches_numpy():
    for key, ctr in [((7, 0), (5, 0, 0, 0)), ((123456789, 42), (2 ** 63, 9, 3, 1))]:
        bg = np.random.Philox(key=np.array(key, dtype=np.uint64), counter=np.array(ctr, dtype=np.uint64))
        expect = bg.random_raw(4)
        got = O.philox4x64([(ctr[0] + 1) % 2 ** 64, *ctr[1:]], key)
        assert np.array_equal(got, expect)


def test_config1_tg32_matches_reference_fixture(port):
    g = golden("config1_tg32.npz")
    s = _solver(port, 32, 32)
    s.set_vorticity(tg_vorticity(32, 32))
    s.derivatives()
    s.d.dt = 1e-3
    s.advance(100)
    assert rel_l2(s.cplx("omega_hat"), g["omega_hat"]) <= 1e-14
    assert abs(s.d.t - float(g["t"])) == 0.0
    assert abs(s.energy() - float(g["energy"])) <= 1e-15


def test_random_hv_sfd_matches_reference_fixture(port):
    g = golden("random64_hv_sfd.npz")
    s = _solver(port, 64, 64, Re=1000.0)
    s.set_vorticity(g["omega0"])
    s.derivatives()
    s.set_hyperviscosity(enabled=1, coefficient=0.5, order=4, cutoff_ratio=0.5, sfd_enabled=1, sfd_strength=0.2,
                         sfd_timescale=0.3)
    s.d.cfl_factor = 0.5
    dts = []
    for _ in range(len(g["dts"])):
        s.d.dt = s.cfl()
        dts.append(s.d.dt)
        s.advance(1)
    assert np.allclose(dts, g["dts"], rtol=1e-14, atol=0)
    assert rel_l2(s.cplx("omega_hat"), g["omega_hat"]) <= 1e-14
    assert rel_l2(s.cplx("sfd_hat"), g["sfd_hat"]) <= 1e-14


# grids that are not powers of two: the reference (FFTW) accepts any size; its
# benchmark runs config-1 physics at 192^2 (performance_benchmark.c:103)
HV_SFD = dict(enabled=1, coefficient=0.5, order=4, cutoff_ratio=0.5, sfd_enabled=1, sfd_strength=0.2,
              sfd_timescale=0.3)
HV_ONLY = dict(enabled=1, coefficient=0.3, order=8, cutoff_ratio=0.65)


def test_config1_tg192_matches_reference_fixture(port):
    g = golden("config1_tg192.npz")
    s = _solver(port, 192, 192)
    s.set_vorticity(tg_vorticity(192, 192))
    s.derivatives()
    s.d.dt = 1e-3
    s.advance(150)
    assert rel_l2(s.cplx("omega_hat"), g["omega_hat"]) <= 1e-14
    assert s.d.t == float(g["t"])
    assert abs(s.energy() - float(g["energy"])) <= 1e-15


@pytest.mark.parametrize("name,nx,ny,hv", [("random96x64_hv_sfd.npz", 96, 64, HV_SFD),
                                           ("random45x30_hv.npz", 45, 30, HV_ONLY)])
def test_random_non_pow2_matches_reference_fixture(port, name, nx, ny, hv):
    g = golden(name)
    s = _solver(port, nx, ny, Re=1000.0)
    s.set_vorticity(g["omega0"])
    s.derivatives()
    s.set_hyperviscosity(**hv)
    s.d.cfl_factor = 0.5
    for dt in g["dts"]:
        s.d.dt = s.cfl()
        assert s.d.dt == dt
        s.advance(1)
    assert rel_l2(s.cplx("omega_hat"), g["omega_hat"]) <= 1e-14


def test_nonlinear_matches_reference_fixture(port):
    g = golden("nonlinear_32x16.npz")
    s = _solver(port, 32, 16)
    s.cplx("omega_hat")[:] = g["omega_hat"]
    s.cplx("psi_hat")[:] = g["psi_hat"]
    s._f("compute_nonlinear_terms")(s.ptr)
    assert rel_l2(s.cplx("nonlinear_hat"), g["nonlinear_hat"]) <= 1e-14
    assert rel_l2(s.real("p"), g["jac"]) <= 1e-14


def test_forcing_matches_reference_fixture(port):
    g = golden("forcing_toy.npz")
    k2 = g["k2"].copy()
    for name, typ, tau, dt in (("white", 0, 0.5, 0.1), ("colored", 1, 0.2, 0.05)):
        cfg = O.ForcingConfig()
        port.nso_forcing_config_default(C.byref(cfg))
        cfg.kmin, cfg.kmax, cfg.energy_target, cfg.seed, cfg.type = 0.5, 2.5, 1.5, 42, typ
        cfg.correlation_time = tau
        st = O.ForcingState()
        assert port.nso_forcing_state_init(C.byref(st), C.byref(cfg), k2.ctypes.data_as(O._DP), 4, 4) == 0
        assert st.active_modes == int(g[name + "_active"])
        f = np.zeros(16, dtype=np.complex128)
        for step in range(3):
            port.nso_forcing_generate(C.byref(st), dt, k2.ctypes.data_as(O._DP),
                                      f.view(np.float64).ctypes.data_as(O._DP))
            assert np.array_equal(f, g[name][step])
            # the reference's own assertion (tests/test_solvers.c:278): sum |f|^2 == target
            assert abs(np.sum(np.abs(f) ** 2) - 1.5) < 1e-6
        assert st.rng_state == int(g[name + "_rng_state"])
        port.nso_forcing_state_free(C.byref(st))


def test_reference_test_assertions_on_oracle(port):
    """Assertions of the reference's tests/test_solvers.c:433-664 that its code meets."""
    s = O.Solver(port, 64, 64).setup(ic=None)
    assert s.d.nkx == 33 and s.d.nx == 64
    s = O.Solver(port, 32, 32).setup(ic=None)
    kx = np.ctypeslib.as_array(s.d.kx, shape=(s.d.nkx,))
    assert abs(kx[0]) < 1e-10 and abs(kx[1] - 1.0) < 1e-10
    assert s.k2()[0, 0] == 0.0 and s.mask()[0, 0] == 1
    # dealiasing zeroes all masked modes
    s.cplx("omega_hat")[:] = 1.0
    s._f("apply_dealiasing")(s.ptr, s.d.omega_hat)
    assert np.all(np.abs(s.cplx("omega_hat")[s.mask() == 0]) < 1e-15)
    # FFT roundtrip of sin x cos y
    x = np.arange(32) * 2 * np.pi / 32
    f = np.sin(x)[None, :] * np.cos(x)[:, None]
    s.real("omega")[:] = f
    s._f("physical_to_spectral")(s.ptr, s.d.omega, s.d.omega_hat)
    s._f("spectral_to_physical")(s.ptr, s.d.omega_hat, s.d.omega)
    assert np.abs(s.real("omega") - f).max() < 1e-10


def test_taylor_green_decay_on_oracle(port):
    """Analytic decay omega(t) = omega0 exp(-2 nu t) for k^2 = 2 (config 1 at 32^2)."""
    g = golden("config1_tg32.npz")
    n = 32
    w0 = np.fft.rfft2(tg_vorticity(n, n)) / n ** 2
    decay = np.exp(-2 * 0.01 * float(g["t"]))
    assert rel_l2(g["omega_hat"], w0 * decay) < 1e-9


@pytest.mark.skipif(not O.have_ref(), reason="reference build not present (bit-exact check runs where it is)")
@pytest.mark.parametrize("nx,ny", [(32, 32), (96, 64), (45, 30)])
def test_restatement_bit_exact_vs_reference_build(port, nx, ny):
    ref = O.load("ref")
    os.environ["OMP_NUM_THREADS"] = "1"
    w = random_field(nx, ny, 9)
    a = O.Solver(port, nx, ny, Re=800.0).setup(ic=None)
    b = O.Solver(ref, nx, ny, Re=800.0).setup(ic=None)
    for s in (a, b):
        s.set_vorticity(w)
        s.derivatives()
        s.set_hyperviscosity(enabled=1, coefficient=0.3, order=8, cutoff_ratio=0.65)
        s.d.cfl_factor = 0.4
        s.advance(10, adaptive=True)
    assert np.array_equal(a.cplx("omega_hat"), b.cplx("omega_hat"))
    assert np.array_equal(a.real("u"), b.real("u"))
    assert a.d.t == b.d.t
