"""Forcing noise keyed by the physical mode: a coarse step of M = 8 draws equals 8
fine steps of one draw each, on the same grid and across grids (spectral
truncation of a 64^2 run onto 32^2).  The runs start from rest with a forcing
amplitude so small that the Jacobian of the forced field (quadratic in it) is
below FP64 rounding of the linear forcing sum."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
L = 2 * math.pi


def _forced(nsgb, n, dt, m):
    g = nsgb.Gpu(n, n, L, L, nsgb.FP64)
    g.set_params(Re=1e30, adaptive_dt=0, dt=dt, forcing_enabled=1, forcing_kmin=2.0, forcing_kmax=6.0,
                 forcing_epsilon=1e-24, forcing_seed=42, forcing_substeps=m)
    g.upload(np.zeros((n, n // 2 + 1), dtype=np.complex128), t=0.0, dt=dt, step0=16)
    return g


def test_substeps_sum_the_fine_draws(nsgb):
    dt = 1e-3
    a = _forced(nsgb, 64, dt, 1)
    b = _forced(nsgb, 64, 8 * dt, 8)
    a.advance(8)
    b.advance(1)
    x = a.download(("omega_hat",))
    y = b.download(("omega_hat",))
    assert np.linalg.norm(x["omega_hat"]) > 0
    assert np.linalg.norm(x["omega_hat"] - y["omega_hat"]) <= 1e-9 * np.linalg.norm(x["omega_hat"])
    assert abs(x["t"] - y["t"]) <= 1e-15
    a.close()
    b.close()


def test_coarse_grid_draws_the_fine_grids_noise(nsgb):
    dt = 1e-3
    fine = _forced(nsgb, 64, dt, 1)
    coarse = _forced(nsgb, 32, 8 * dt, 8)
    fine.advance(8)
    coarse.advance(1)
    truth = nsgb.Gpu(32, 32, L, L, nsgb.FP64)
    truth.set_params(Re=1e30)
    fine.check(fine.lib.ns_gpu_filter_state(fine.h, truth.h), "filter_state")
    x = truth.download(("omega_hat",))["omega_hat"]
    y = coarse.download(("omega_hat",))["omega_hat"]
    assert np.linalg.norm(x) > 0
    assert np.linalg.norm(x - y) <= 1e-9 * np.linalg.norm(x)
    for g in (fine, coarse, truth):
        g.close()
