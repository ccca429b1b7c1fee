"""Device-side energy spectrum of the resident state (ns_gpu_energy_spectrum) against
the oracle's restatement of ns_spectral_analyze_spectrum's binning
(spectral_analysis.c:103-142, oracle nso_spectrum) on the same omega_hat."""
import ctypes as C

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,prec", [(64, 0), (128, 0), (256, 1)])
def test_energy_spectrum_matches_oracle_binning(nsgb, port, n, prec):
    g = nsgb.Gpu(n, n, precision=prec)
    g.set_params(Re=1000.0)
    wh = np.zeros((n, n // 2 + 1), dtype=np.complex128)
    g.check(g.lib.ns_gpu_random_spectrum_host(g.h, 11, 6.0, 0.5, wh.view(np.float64).ctypes.data_as(O._DP)),
            "random_spectrum_host")
    if prec == 1:  # the FP32 state holds the spectrum rounded to float
        wh = wh.astype(np.complex64).astype(np.complex128)
    es, em, ct = g.energy_spectrum()
    o = O.Solver(port, n, n, Re=1000.0).setup(ic=None)
    o.cplx("omega_hat")[:] = wh
    o._f("compute_velocity_from_vorticity")(o.ptr)
    nb = min(n // 2 + 1, n // 2)
    eo = np.zeros(nb)
    co = np.zeros(nb, dtype=np.int32)
    assert port.nso_spectrum(o.ptr, eo.ctypes.data_as(O._DP), co.ctypes.data_as(C.POINTER(C.c_int))) == nb
    assert np.array_equal(ct, co)
    tol = 1e-12 if prec == 0 else 1e-6
    assert np.allclose(es, eo, rtol=tol, atol=tol * eo.max())
    with np.errstate(invalid="ignore", divide="ignore"):
        mo = np.where(co > 0, eo / np.maximum(co, 1), 0.0)
    assert np.allclose(em, mo, rtol=tol, atol=tol * mo.max())
    # Parseval over the half plane: at most the state's energy
    assert es.sum() <= g.diagnostics()["energy"] * (1 + 1e-9)
    o.close()
    g.close()


def test_energy_spectrum_follows_the_run(nsgb):
    """E(k) of a forced, hyperviscous 256^2 run every few steps stays finite and its
    shell sums track the device energy: the reference bins the kx >= 0 half plane
    only, which holds half the energy plus half of the kx = 0 column's."""
    g = nsgb.Gpu(256, 256, precision=1)
    g.set_params(Re=1e4, cfl_factor=0.5, adaptive_dt=1, hv_enabled=1, hv_coefficient=50.0, hv_order=8,
                 hv_cutoff_ratio=0.0, forcing_enabled=1, forcing_kmin=4.0, forcing_kmax=6.0,
                 forcing_epsilon=1e-3, forcing_seed=5)
    g.random_spectrum(2, 4.0, 0.5)
    for _ in range(3):
        g.advance(5)
        es, em, ct = g.energy_spectrum()
        e = g.diagnostics()["energy"]
        assert np.isfinite(es).all() and 0.45 * e <= es.sum() <= 0.75 * e
    g.close()
