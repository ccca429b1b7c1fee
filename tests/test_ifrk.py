"""Integrating-factor RK4 (a scheme option with no reference counterpart).

CPU: the oracle's restatement (Lawson's IF-RK4 over the reference's stage
nonlinear term) is exact for Taylor-Green decay, fourth-order accurate, equal
to the reference RK4 when nothing is linear, and stable where explicit RK4 is
not.  GPU: the generic and the 2048-point stage kernels against that oracle in
FP64 at <= 1e-12 relative L2, with hyperviscosity, SFD, forcing and device CFL.
"""
import numpy as np
import pytest

from conftest import grid, rel_l2

import oracle as O

TOL = 1e-12


def _field(n, kind):
    X, Y = np.meshgrid(grid(n), grid(n))
    if kind == "tg":
        return 2.0 * np.sin(X) * np.sin(Y)
    return np.sin(X) * np.sin(2 * Y) + 0.5 * np.cos(3 * X + Y) + 0.3 * np.sin(5 * X - 2 * Y)


def _oracle(port, n, scheme, dt, steps, kind="r", Re=100.0, hv=None):
    s = O.Solver(port, n, n, Re=Re).setup(ic=None)
    s.set_vorticity(_field(n, kind))
    s.derivatives()
    if hv is not None:
        s.set_hyperviscosity(enabled=1, coefficient=hv, order=4, cutoff_ratio=0.0)
    s.d.dt = dt
    port.nso_ext_run_scheme(s.ptr, scheme, steps, 0, 0, 0.0, 0.0, 0.0, 0, 0)
    return s


def test_taylor_green_decay_is_exact_at_large_dt(port):
    """k^2 = 2 everywhere: the Jacobian vanishes and the decay is integrated exactly."""
    s = _oracle(port, 32, 1, 0.25, 8, kind="tg")
    exact = _field(32, "tg") * np.exp(-2.0 * s.d.t / 100.0)
    assert abs(s.d.t - 2.0) < 1e-14
    assert np.abs(s.real("omega") - exact).max() < 1e-14


def test_fourth_order_convergence(port):
    ref = _oracle(port, 32, 0, 1e-4, 2000)
    errs = []
    for dt in (2e-2, 1e-2, 5e-3):
        s = _oracle(port, 32, 1, dt, int(round(0.2 / dt)))
        errs.append(np.linalg.norm(s.cplx("omega_hat") - ref.cplx("omega_hat")))
    for e0, e1 in zip(errs, errs[1:]):
        assert 12.0 < e0 / e1 < 20.0, errs


def test_reduces_to_rk4_without_linear_terms(port):
    """Re -> infinity, no hyperviscosity: E = 1 and the two schemes coincide."""
    a = _oracle(port, 32, 0, 1e-2, 10, Re=1e300)
    b = _oracle(port, 32, 1, 1e-2, 10, Re=1e300)
    assert rel_l2(b.cplx("omega_hat"), a.cplx("omega_hat")) < 1e-14


def test_stable_where_explicit_rk4_is_not(port):
    """Hyperviscous decay rate x dt ~ 19 at the kept-band edge: beyond explicit RK4's
    real-axis limit (~2.79), so round-off there grows without bound under RK4."""
    dt, steps, c = 0.05, 40, 2000.0
    rk = _oracle(port, 32, 0, dt, steps, hv=c)
    ifr = _oracle(port, 32, 1, dt, steps, hv=c)
    w0 = np.abs(_field(32, "r")).max()
    assert not np.isfinite(rk.real("omega")).all() or np.abs(rk.real("omega")).max() > 1e3 * w0
    assert np.abs(ifr.real("omega")).max() <= 1.01 * w0


# ------------------------------------------------------------------- GPU
def _oracle_run(port, nx, ny, steps, sfd=False, Re=1e3, hv=2.0, seed=5):
    s = O.Solver(port, nx, ny, Re=Re).setup(ic=None)
    port.nso_ext_init_random_spectrum(s.ptr, seed, 4.0, 0.5)
    kw = dict(enabled=1, coefficient=hv, order=4, cutoff_ratio=0.0)
    if sfd:
        kw.update(sfd_enabled=1, sfd_strength=0.5, sfd_timescale=0.05)
    s.set_hyperviscosity(**kw)
    s.d.cfl_factor = 0.5
    port.nso_ext_run_scheme(s.ptr, 1, steps, 1, 1, 4.0, 6.0, 1e-3, 11, 0)
    return s


def _gpu_run(nsgb, nx, ny, steps, prec, sfd=False, Re=1e3, hv=2.0, seed=5, scheme=1):
    s = nsgb.Solver(nx, ny, Re=Re, precision=prec).setup(ic=None)
    s.set_forcing(4.0, 6.0, 1e-3, 11)
    s.set_scheme(scheme)
    s.d.cfl_factor = 0.5
    s.random_spectrum(seed, 4.0, 0.5)
    kw = dict(enabled=1, coefficient=hv, order=4, cutoff_ratio=0.0)
    if sfd:
        kw.update(sfd_enabled=1, sfd_strength=0.5, sfd_timescale=0.05)
    s.set_hyperviscosity(**kw)  # after the IC, as on the oracle side: _set seeds the SFD filter with omega_hat
    s.advance_n(steps, adaptive=True)
    s.sync_host()
    return s


@pytest.mark.gpu
@pytest.mark.parametrize("nx,ny,steps,sfd", [(64, 64, 12, False), (64, 64, 12, True), (128, 64, 8, True),
                                             (2048, 128, 4, False), (128, 2048, 4, True)])
def test_gpu_ifrk4_fp64_matches_oracle(nsgb, port, nx, ny, steps, sfd):
    o = _oracle_run(port, nx, ny, steps, sfd=sfd)
    g = _gpu_run(nsgb, nx, ny, steps, nsgb.FP64, sfd=sfd)
    assert abs(g.d.t - o.d.t) <= 1e-12 * o.d.t
    assert rel_l2(g.cplx("omega_hat"), o.cplx("omega_hat")) <= TOL
    assert rel_l2(g.real("omega"), o.real("omega")) <= TOL


@pytest.mark.gpu
def test_gpu_ifrk4_fp32_2048_tracks_fp64(nsgb):
    a = _gpu_run(nsgb, 2048, 2048, 5, nsgb.FP64)
    b = _gpu_run(nsgb, 2048, 2048, 5, nsgb.FP32)
    assert rel_l2(b.cplx("omega_hat"), a.cplx("omega_hat")) <= 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("nx,ny,scheme", [(128, 2048, 0), (128, 2048, 1), (2048, 2048, 0)])
def test_gpu_fp32_column_pass_with_sfd_tracks_fp64(nsgb, nx, ny, scheme):
    # the FP32 2048-point column pass with every term of its stage algebra on:
    # hyperviscosity, SFD relaxation and post-step, forcing (explicit RK4 and IF-RK4)
    a = _gpu_run(nsgb, nx, ny, 5, nsgb.FP64, sfd=True, scheme=scheme)
    b = _gpu_run(nsgb, nx, ny, 5, nsgb.FP32, sfd=True, scheme=scheme)
    assert rel_l2(b.cplx("omega_hat"), a.cplx("omega_hat")) <= 1e-5
    assert rel_l2(b.cplx("sfd_hat"), a.cplx("sfd_hat")) <= 1e-5
    assert abs(b.d.t - a.d.t) <= 1e-6 * a.d.t


@pytest.mark.gpu
def test_gpu_rejects_unknown_scheme(nsgb):
    s = nsgb.Solver(32, 32, Re=100.0).setup(ic=None)
    with pytest.raises(RuntimeError):
        s.set_scheme(2)
