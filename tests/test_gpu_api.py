"""The whole drop-in API on the GPU against the oracle, the reference fixtures
and the reference's own test assertions (tests/test_solvers.c:239-664)."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import golden, rel_l2, random_field, tg_vorticity

import oracle as O

pytestmark = pytest.mark.gpu


def _pair(nsgb, port, nx, ny, Re=100.0):
    return nsgb.Solver(nx, ny, Re=Re).setup(ic=None), O.Solver(port, nx, ny, Re=Re).setup(ic=None)


# ------------------------------------------------ reference test assertions
def test_reference_solver_tests(nsgb):
    s = nsgb.Solver(64, 64).setup(ic=None)
    assert s.d.nkx == 33 and s.d.nx == 64 and bool(s.d.u) and bool(s.d.omega_hat)
    s = nsgb.Solver(32, 32).setup(ic=None)
    kx = np.ctypeslib.as_array(s.d.kx, shape=(s.d.nkx,))
    assert abs(kx[0]) < 1e-10 and abs(kx[1] - 1.0) < 1e-10 and abs(s.k2()[0, 0]) < 1e-10 and s.mask()[0, 0] == 1
    assert s.d.forward_plan and s.d.backward_plan
    # FFT round trip of sin x cos y (test_solvers.c:473-511)
    x = np.arange(32) * 2 * np.pi / 32
    f = np.sin(x)[None, :] * np.cos(x)[:, None]
    s.real("omega")[:] = f
    s._f("physical_to_spectral")(s.ptr, s.d.omega, s.d.omega_hat)
    s._f("spectral_to_physical")(s.ptr, s.d.omega_hat, s.d.omega)
    assert np.abs(s.real("omega") - f).max() < 1e-10
    # dealiasing (:513-545)
    s.cplx("omega_hat")[:] = 1.0
    s._f("apply_dealiasing")(s.ptr, s.d.omega_hat)
    assert np.all(np.abs(s.cplx("omega_hat")[s.mask() == 0]) < 1e-15)
    # uniform vorticity gives zero velocity (:547-577)
    s.cplx("omega_hat")[:] = 0.0
    s.cplx("omega_hat")[0, 0] = 1.0
    s._f("compute_velocity_from_vorticity")(s.ptr)
    s._f("spectral_to_physical")(s.ptr, s.d.u_hat, s.d.u)
    s._f("spectral_to_physical")(s.ptr, s.d.v_hat, s.d.v)
    assert max(np.abs(s.real("u")).max(), np.abs(s.real("v")).max()) < 1e-10
    # energy / enstrophy of the Taylor-Green field (:579-614)
    t = nsgb.Solver(32, 32).setup(ic="tg")
    assert 0.0 < t.energy() < 1.0 and t.enstrophy() > 0.0


def test_reference_hyperviscosity_test(nsgb):
    """tests/test_solvers.c:616-664."""
    s = nsgb.Solver(32, 32).setup(ic=None)
    s.set_hyperviscosity(enabled=1, coefficient=0.05, order=4, cutoff_ratio=0.6, sfd_enabled=1, sfd_strength=0.3,
                         sfd_timescale=0.4)
    w = np.ctypeslib.as_array(s.d.hyperviscosity_weights, shape=(32, 17))
    assert abs(w[0, 0]) < 1e-12 and w[-1, -1] > 0.0
    s.cplx("rk1_hat")[:] = 0.0
    s.cplx("omega_hat")[:] = 1.0
    s.lib.ns_spectral_hyperviscosity_apply(s.ptr, s.d.rk1_hat, s.d.omega_hat)
    rhs = s.cplx("rk1_hat")
    assert abs(rhs[0, 0]) < 1e-8 and abs(rhs[-1, -1]) > 1e-3
    s.lib.ns_spectral_hyperviscosity_post_step(s.ptr, s.d.omega_hat, 0.1)
    assert abs(s.cplx("sfd_hat")[-1, -1]) > 0.0


# ------------------------------------------------------------ vs the oracle
@pytest.mark.parametrize("nx,ny", [(32, 32), (64, 16), (128, 256)])
def test_grids_and_taylor_green_match(nsgb, port, nx, ny):
    g, o = _pair(nsgb, port, nx, ny)
    for name, n in (("x", nx), ("y", ny), ("kx", nx // 2 + 1), ("ky", ny)):
        assert np.array_equal(np.ctypeslib.as_array(getattr(g.d, name), shape=(n,)),
                              np.ctypeslib.as_array(getattr(o.d, name), shape=(n,)))
    assert np.array_equal(g.k2(), o.k2()) and np.array_equal(g.mask(), o.mask())
    for s in (g, o):
        s._f("initialize_taylor_green")(s.ptr)
    for name in ("u", "v", "omega", "p"):
        assert np.allclose(g.real(name), o.real(name), rtol=0, atol=1e-14)
    for name in ("omega_hat", "u_hat", "v_hat"):
        assert rel_l2(g.cplx(name), o.cplx(name)) <= 1e-14


def test_analysis_matches(nsgb, port):
    g = golden("analysis64.npz")
    s = nsgb.Solver(64, 64, Re=500.0).setup(ic=None)
    s.set_vorticity(g["omega"])
    s.derivatives()
    assert abs(s.energy() - float(g["energy"])) <= 1e-13 * float(g["energy"])
    assert abs(s.enstrophy() - float(g["enstrophy"])) <= 1e-13 * float(g["enstrophy"])
    assert abs(s.cfl() - float(g["cfl"])) <= 1e-13 * float(g["cfl"])
    o = O.Solver(port, 64, 64, Re=500.0).setup(ic=None)
    o.set_vorticity(g["omega"])
    o.derivatives()
    frac = C.c_double()
    assert s.lib.ns_spectral_check_resolution(s.ptr) == port.nso_check_resolution(o.ptr, C.byref(frac))
    # shell spectrum sums and counts (spectral_analysis.c:103-142)
    h = s.lib.ns_spectral_gpu_handle(s.ptr)
    f = s.lib.ns_gpu_spectral_stats
    f.argtypes = [C.c_void_p] + [C.c_void_p] * 3 + [C.c_void_p] * 5
    nb = 32
    eg = np.zeros(nb)
    cg = np.zeros(nb, dtype=np.int32)
    mx = C.c_double()
    er = C.c_double()
    rf = C.c_double()
    assert f(h, s.d.omega_hat, s.d.u_hat, s.d.v_hat, C.addressof(rf), C.addressof(mx), C.addressof(er),
             eg.ctypes.data, cg.ctypes.data) == 0
    eo = np.zeros(nb)
    co = np.zeros(nb, dtype=np.int32)
    assert port.nso_spectrum(o.ptr, eo.ctypes.data_as(O._DP), co.ctypes.data_as(C.POINTER(C.c_int))) == nb
    # shells beyond the field's band hold only transform round-off: compare against the largest bin
    assert np.array_equal(cg, co) and np.allclose(eg, eo, rtol=1e-12, atol=1e-13 * eo.max())
    mxo = C.c_double()
    ero = C.c_double()
    port.nso_convergence_stats(o.ptr, C.byref(mxo), C.byref(ero))
    # the tail estimate of a smooth field is itself round-off: bound it on the field's scale
    assert abs(mx.value - mxo.value) <= 1e-15 * mxo.value
    assert abs(er.value - ero.value) <= 1e-13 * ero.value + 1e-15 * mxo.value
    assert abs(rf.value - frac.value) <= 1e-12 * frac.value + 1e-14


def test_first_step_uses_stored_psi_hat(nsgb, port):
    """Q1: without compute_derivatives, stage 1 uses the stored (zero) psi_hat, as the reference does."""
    w = random_field(32, 32, 4)
    g, o = _pair(nsgb, port, 32, 32, Re=300.0)
    for s in (g, o):
        s.set_vorticity(w)
        s.d.dt = 5e-3
        s.advance(3)
    assert rel_l2(g.cplx("omega_hat"), o.cplx("omega_hat")) <= 1e-12


def test_masked_out_modes_evolve_like_the_reference(nsgb, port):
    """A caller may write modes outside the 2/3 mask; the reference evolves them by the linear terms only."""
    rng = np.random.default_rng(8)
    wh = (rng.standard_normal((32, 17)) + 1j * rng.standard_normal((32, 17))) * 1e-2
    g, o = _pair(nsgb, port, 32, 32, Re=200.0)
    for s in (g, o):
        s.cplx("omega_hat")[:] = wh
        s.derivatives()
        s.set_hyperviscosity(enabled=1, coefficient=0.2, order=4, cutoff_ratio=0.5, sfd_enabled=1, sfd_strength=0.5,
                             sfd_timescale=0.2)
        s.d.dt = 2e-3
        s.advance(5)
    assert rel_l2(g.cplx("omega_hat"), o.cplx("omega_hat")) <= 1e-12
    assert rel_l2(g.cplx("sfd_hat"), o.cplx("sfd_hat")) <= 1e-12
    m = g.mask() == 0
    assert np.abs(g.cplx("omega_hat")[m]).max() > 0


def test_hyperviscosity_api_matches(nsgb, port):
    rng = np.random.default_rng(3)
    g, o = _pair(nsgb, port, 64, 32)
    st = rng.standard_normal((32, 33)) + 1j * rng.standard_normal((32, 33))
    rhs = rng.standard_normal((32, 33)) + 1j * rng.standard_normal((32, 33))
    for s in (g, o):
        s.set_hyperviscosity(enabled=1, coefficient=0.7, order=6, cutoff_ratio=0.3, sfd_enabled=1, sfd_strength=0.4,
                             sfd_timescale=0.25)
        s.cplx("omega_hat")[:] = st
        s.cplx("rk2_hat")[:] = rhs
        s.cplx("sfd_hat")[:] = 0.5 * st
        hv = s.lib._hv if hasattr(s.lib, "_hv") else "ns_spectral_hyperviscosity_"
        getattr(s.lib, hv + "apply")(s.ptr, s.d.rk2_hat, s.d.omega_hat)
        getattr(s.lib, hv + "post_step")(s.ptr, s.d.omega_hat, 0.05)
    assert rel_l2(g.cplx("rk2_hat"), o.cplx("rk2_hat")) <= 1e-14
    assert rel_l2(g.cplx("sfd_hat"), o.cplx("sfd_hat")) <= 1e-15
    assert g.d.hyperviscosity.kmax == o.d.hyperviscosity.kmax
    assert g.d.hyperviscosity.inv_bandwidth == o.d.hyperviscosity.inv_bandwidth


def test_derivatives_and_nonlinear_match(nsgb, port):
    w = random_field(64, 64, 12)
    g, o = _pair(nsgb, port, 64, 64)
    for s in (g, o):
        s.set_vorticity(w)
        s.derivatives()
    for name in ("psi_hat", "u_hat", "v_hat"):
        assert rel_l2(g.cplx(name), o.cplx(name)) <= 1e-14
    for name in ("u", "v", "omega"):
        assert rel_l2(g.real(name), o.real(name)) <= 1e-13
    assert np.array_equal(g.cplx("nonlinear_hat"), g.cplx("omega_hat") * g.mask())
    for s in (g, o):
        s._f("compute_nonlinear_terms")(s.ptr)
    assert rel_l2(g.cplx("nonlinear_hat"), o.cplx("nonlinear_hat")) <= 1e-13
    for name in ("u", "v", "psi", "omega", "p"):  # the reference's aliasing: psi_x, psi_y, omega_x, omega_y, J
        assert rel_l2(g.real(name), o.real(name)) <= 1e-13


def test_output_solution_writes_reference_format(nsgb, tmp_path):
    s = nsgb.Solver(16, 8).setup(ic="tg")
    s.derivatives()
    path = tmp_path / "sol.dat"
    s.lib.ns_spectral_output_solution(s.ptr, str(path).encode())
    lines = path.read_text().splitlines()
    assert lines[0] == "# Spectral Navier-Stokes Solution" and lines[1] == "# x y u v omega psi"
    rows = [l for l in lines[2:] if l.strip()]
    assert len(rows) == 16 * 8
    vals = np.array([[float(t) for t in r.split()] for r in rows])
    assert np.allclose(vals[:, 2], s.real("u").ravel(), atol=1e-7)
    assert np.allclose(vals[:, 5], s.real("psi").ravel(), atol=1e-7)


# ---------------------------------------------------------------- forcing
def test_forcing_api_matches_reference_stream(nsgb):
    g = golden("forcing_toy.npz")
    lib = nsgb.load()
    k2 = g["k2"].copy()
    for name, typ, tau, dt in (("white", 0, 0.5, 0.1), ("colored", 1, 0.2, 0.05)):
        cfg = nsgb.ForcingConfig()
        lib.ns_forcing_config_default(C.byref(cfg))
        cfg.kmin, cfg.kmax, cfg.energy_target, cfg.seed, cfg.type = 0.5, 2.5, 1.5, 42, typ
        cfg.correlation_time = tau
        st = nsgb.ForcingState()
        assert lib.ns_forcing_state_init(C.byref(st), C.byref(cfg), k2.ctypes.data_as(nsgb._DP), 4, 4) == 0
        assert st.active_modes == int(g[name + "_active"])
        f = np.zeros(16, dtype=np.complex128)
        for step in range(3):
            lib.ns_forcing_generate(C.byref(st), dt, k2.ctypes.data_as(nsgb._DP),
                                    f.view(np.float64).ctypes.data_as(nsgb._DP))
            assert rel_l2(f, g[name][step]) <= 1e-14
            assert abs(np.sum(np.abs(f) ** 2) - 1.5) < 1e-6  # tests/test_solvers.c:278
        assert st.rng_state == int(g[name + "_rng_state"]) and st.have_spare == 0
        lib.ns_forcing_state_free(C.byref(st))


def test_random_spectrum_and_forced_run_match_fixture(nsgb):
    g = golden("ext_random_forced64.npz")
    s = nsgb.Solver(64, 64, Re=1e4).setup(ic=None)
    s.random_spectrum(7, 4.0, 0.5)
    assert rel_l2(s.cplx("omega_hat"), g["ic_omega_hat"]) <= 1e-13
    e, z = s.diagnostics()
    assert abs(e - 0.5) <= 1e-13
    s.set_hyperviscosity(enabled=1, coefficient=2.0, order=4, cutoff_ratio=0.0)
    s.set_forcing(4.0, 6.0, 1e-3, 11)
    s.d.cfl_factor = 0.5
    s.advance_n(20, adaptive=True)
    s.sync_host()
    assert abs(s.d.t - float(g["forced_t"])) <= 1e-12 * float(g["forced_t"])
    assert rel_l2(s.cplx("omega_hat"), g["forced_omega_hat"]) <= 1e-12


# ------------------------------------------------------- failure detection
def test_nonfinite_state_is_reported_not_faulted(nsgb):
    """Fault injection on the host: a NaN written into the caller's state makes the
    diagnostics return SOLVER_DIVERGED; no device fault is involved."""
    s = nsgb.Solver(32, 32).setup(ic="tg")
    s.derivatives()
    s.cplx("omega_hat")[3, 2] = complex(np.nan, 0.0)
    e = C.c_double()
    z = C.c_double()
    st = s.lib.ns_spectral_gpu_diagnostics(s.ptr, C.byref(e), C.byref(z))
    assert st == 2  # SOLVER_DIVERGED
    # the instance stays usable afterwards
    s.cplx("omega_hat")[3, 2] = 0.0
    assert s.lib.ns_spectral_gpu_diagnostics(s.ptr, C.byref(e), C.byref(z)) == 0


def test_invalid_arguments_return_errors(nsgb):
    s = nsgb.Solver(32, 32).setup(ic=None)
    assert s.lib.ns_spectral_gpu_advance_n(s.ptr, -1, 0) == 4  # SOLVER_INVALID_PARAM
    assert s.lib.ns_spectral_gpu_set_forcing(s.ptr, 1, 6.0, 4.0, 1e-3, 1) == 4


# --------------------------------------------------- large-size properties
def test_2048_fp32_properties(nsgb):
    s = nsgb.Solver(2048, 2048, Re=1e5, precision=nsgb.FP32).setup(ic=None)
    s.random_spectrum(3, 8.0, 0.5)
    s.d.cfl_factor = 0.5
    s.advance_n(20, adaptive=True)
    s.sync_host()
    e_par, z_par = s.diagnostics()
    # Parseval: the physical-space reductions of the refreshed u, v, omega agree
    assert abs(s.energy() - e_par) <= 1e-5 * e_par
    assert abs(s.enstrophy() - z_par) <= 1e-5 * z_par
    # unforced, inviscid-range run: energy does not grow
    assert e_par <= 0.5 * (1 + 1e-5)
    # the velocity is divergence free in spectral space: kx u_hat + ky v_hat = 0
    kx = np.ctypeslib.as_array(s.d.kx, shape=(s.d.nkx,))[None, :]
    ky = np.ctypeslib.as_array(s.d.ky, shape=(s.d.nky,))[:, None]
    div = kx * s.cplx("u_hat") + ky * s.cplx("v_hat")
    assert np.abs(div).max() <= 1e-12 * np.abs(kx * s.cplx("u_hat")).max()


def test_host_step_rewrites_what_the_reference_rewrites(nsgb, port):
    """ns_spectral_advance_rk4 moves its arrays with ns_gpu_step_host: omega_hat and
    psi_hat come back as kept modes only when the call itself saw zeros outside the
    mask.  A caller that scribbled on psi_hat outside the mask and on u_hat, v_hat
    gets every array back as the reference writes it (psi_hat = -omega_hat/k^2 on
    all modes, spectral_core.c:17-31)."""
    n = 32
    w = random_field(n, n, 5)
    gpu = nsgb.Solver(n, n, Re=300.0).setup(ic=None)
    ora = O.Solver(port, n, n, Re=300.0).setup(ic=None)
    out = gpu.mask() == 0
    junk = np.random.default_rng(3).standard_normal(int(out.sum()))
    for x in (gpu, ora):
        x.set_vorticity(w)
        x.derivatives()
        x.d.dt = 1e-3
        x.cplx("psi_hat")[out] = junk
        x.cplx("u_hat")[:] = 7.0
        x.cplx("v_hat")[:] = -3.0
    gpu.advance(2)
    ora.advance(2)
    for name in ("omega_hat", "psi_hat", "u_hat", "v_hat"):
        assert rel_l2(gpu.cplx(name), ora.cplx(name)) <= 1e-12, name
    assert np.all(gpu.cplx("psi_hat")[out] == 0)
    for name in ("u", "v", "omega"):
        assert rel_l2(gpu.real(name), ora.real(name)) <= 1e-12, name
    assert gpu.d.t == ora.d.t


@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (1, 2e-6)])
def test_add_vorticity_device_then_advance(nsgb, prec, tol):
    """ns_gpu_add_vorticity_device adds the masked forward transform of a float
    field to the state and leaves the next step's fields ready: the spectrum
    matches numpy's rfft2 on the kept modes, and two steps from there match two
    steps of an instance that was given the same spectrum by upload."""
    torch = pytest.importorskip("torch")
    nx, ny = 64, 48
    g = nsgb.Gpu(nx, ny, 2 * np.pi, 2 * np.pi, prec)
    g.set_params(Re=500.0, dt=2e-3, adaptive_dt=0)
    g.random_spectrum(3, 4.0, 0.5)
    w0 = g.download(("omega_hat",))["omega_hat"]
    delta = np.random.default_rng(5).standard_normal((ny, nx)).astype(np.float32)
    d = torch.from_numpy(delta).cuda()
    g.check(g.lib.ns_gpu_add_vorticity_device(g.h, C.c_void_p(d.data_ptr())), "add_vorticity_device")
    w1 = g.download(("omega_hat",))["omega_hat"]
    kx_kept, ky_kept = g.dims()
    kyh = (ky_kept - 1) // 2
    rows = np.r_[0:kyh + 1, ny - kyh:ny]
    ref = np.fft.rfft2(delta.astype(np.float64)) / (nx * ny)
    kept = np.zeros(w0.shape, dtype=bool)
    kept[np.ix_(rows, np.arange(kx_kept))] = True
    assert rel_l2(w1[kept], (w0 + ref)[kept]) <= tol
    assert np.array_equal(w1[~kept], w0[~kept])
    h = nsgb.Gpu(nx, ny, 2 * np.pi, 2 * np.pi, prec)
    h.set_params(Re=500.0, dt=2e-3, adaptive_dt=0)
    h.upload(w1, dt=2e-3)  # the upload also sets the step's dt
    g.advance(2)
    h.advance(2)
    a = g.download(("omega_hat",))["omega_hat"]
    b = h.download(("omega_hat",))["omega_hat"]
    assert rel_l2(a, b) <= tol
    g.close()
    h.close()
