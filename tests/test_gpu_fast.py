"""The 2048-point stage kernels (row pass for nx = 2048, column pass for ny = 2048).

FP64 runs of the benchmark physics (random-phase IC, hyperviscosity, Philox
forcing, device CFL dt) against the oracle restatement at <= 1e-12 relative L2,
at the full 2048^2 size and at non-square sizes where only one of the two fast
kernels is active; then the FP32 bulk path against FP64 at 2048^2.
"""
import numpy as np
import pytest

from conftest import rel_l2

import oracle as O

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _oracle_run(port, nx, ny, steps, Re=1e4, hv=2.0, seed=7):
    s = O.Solver(port, nx, ny, Re=Re).setup(ic=None)
    port.nso_ext_init_random_spectrum(s.ptr, seed, 4.0, 0.5)
    s.set_hyperviscosity(enabled=1, coefficient=hv, order=4, cutoff_ratio=0.0)
    s.d.cfl_factor = 0.5
    port.nso_ext_run(s.ptr, steps, 1, 1, 4.0, 6.0, 1e-3, 11, 0)
    return s


def _gpu_run(nsgb, nx, ny, steps, prec, Re=1e4, hv=2.0, seed=7):
    s = nsgb.Solver(nx, ny, Re=Re, precision=prec).setup(ic=None)
    s.set_hyperviscosity(enabled=1, coefficient=hv, order=4, cutoff_ratio=0.0)
    s.set_forcing(4.0, 6.0, 1e-3, 11)
    s.d.cfl_factor = 0.5
    s.random_spectrum(seed, 4.0, 0.5)
    s.advance_n(steps, adaptive=True)
    s.sync_host()
    return s


@pytest.mark.parametrize("nx,ny,steps", [(2048, 128, 6), (128, 2048, 6), (2048, 2048, 3)])
def test_fast_kernels_fp64_match_oracle(nsgb, port, nx, ny, steps):
    o = _oracle_run(port, nx, ny, steps)
    g = _gpu_run(nsgb, nx, ny, steps, nsgb.FP64)
    assert abs(g.d.t - o.d.t) <= 1e-12 * o.d.t
    assert rel_l2(g.cplx("omega_hat"), o.cplx("omega_hat")) <= TOL
    assert rel_l2(g.real("u"), o.real("u")) <= TOL
    assert rel_l2(g.real("omega"), o.real("omega")) <= TOL


@pytest.mark.parametrize("nx,ny,steps", [(2048, 2048, 10), (2048, 128, 10), (128, 2048, 10), (128, 4096, 10),
                                         (4096, 128, 10), (4096, 4096, 3)])
def test_fast_fp32_vs_fp64_2048(nsgb, nx, ny, steps):
    # the FP32 stage kernels (k_row_t / k_row_4k, k_col_q at 2048 and 4096; alone on the non-square grids) against FP64
    a = _gpu_run(nsgb, nx, ny, steps, nsgb.FP64)
    b = _gpu_run(nsgb, nx, ny, steps, nsgb.FP32)
    err = rel_l2(b.cplx("omega_hat"), a.cplx("omega_hat"))
    assert err <= 1e-5, err
    assert rel_l2(b.real("u"), a.real("u")) <= 1e-5
    assert abs(b.d.t - a.d.t) <= 1e-6 * a.d.t
    ea, za = a.diagnostics()
    eb, zb = b.diagnostics()
    assert abs(eb - ea) <= 1e-6 * ea
    assert abs(zb - za) <= 1e-5 * za
