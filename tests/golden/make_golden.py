"""Generate the golden fixtures in tests/golden/ from the reference itself.

Every fixture whose path is a reference behaviour comes from ``oracle/_ref``:
the reference's own spectral sources compiled unmodified against the project
FFTW-API shim (``make -C oracle ref``, which needs the reference tree).  The
project-extension fixtures (random-phase IC, Philox forcing) come from the
oracle restatement, since the reference has no such functions.

    OMP_NUM_THREADS=1 python tests/golden/make_golden.py

Outputs are small .npz files; the GPU tests read them on machines without the
reference tree.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402


def grid(n, L=2 * np.pi):
    return np.arange(n) * L / n


def tg_vorticity(nx, ny):
    x, y = grid(nx), grid(ny)
    return 2.0 * np.sin(x)[None, :] * np.sin(y)[:, None]


def random_field(nx, ny, seed):
    rng = np.random.default_rng(seed)
    f = rng.standard_normal((ny, nx))
    # smooth it so the run is resolved: keep |k| <= min(nx,ny)/6
    fh = np.fft.rfft2(f)
    kx = np.fft.rfftfreq(nx, 1.0 / nx)[None, :]
    ky = np.fft.fftfreq(ny, 1.0 / ny)[:, None]
    fh[np.sqrt(kx ** 2 + ky ** 2) > min(nx, ny) / 6] = 0
    return np.fft.irfft2(fh, s=(ny, nx))


HV_SFD = dict(enabled=1, coefficient=0.5, order=4, cutoff_ratio=0.5, sfd_enabled=1, sfd_strength=0.2,
              sfd_timescale=0.3)
HV_ONLY = dict(enabled=1, coefficient=0.3, order=8, cutoff_ratio=0.65)


def config1(ref, n, steps):
    """Config 1: omega0 = 2 sin x sin y written into omega, physical_to_spectral,
    compute_derivatives (as performance_benchmark.c:63), nu = 0.01, dt = 1e-3."""
    s = O.Solver(ref, n, n, Re=100.0).setup(ic=None)
    s.set_vorticity(tg_vorticity(n, n))
    s.derivatives()
    s.d.dt = 1e-3
    s.advance(steps)
    out = dict(omega_hat=s.cplx("omega_hat").copy(), psi_hat=s.cplx("psi_hat").copy(),
               t=s.d.t, energy=s.energy(), enstrophy=s.enstrophy(),
               u_row=s.real("u")[n // 3].copy(), v_row=s.real("v")[n // 5].copy(),
               omega_row=s.real("omega")[n // 7].copy())
    s.close()
    return out


def config1_benchmark_case(ref, n, steps):
    """Config-1 physics on the reference benchmark's non-power-of-two grid
    (performance_benchmark.c:103 runs 192^2 for 150 steps): omega_hat, time,
    energy and enstrophy only (the spectrum of this run is a few modes plus
    round-off, so one array is the whole check)."""
    out = config1(ref, n, steps)
    return {k: out[k] for k in ("omega_hat", "t", "energy", "enstrophy", "omega_row")}


def random_hv(ref, n, steps, seed=1, ny=None, hv=None):
    ny = n if ny is None else ny
    s = O.Solver(ref, n, ny, Re=1000.0).setup(ic=None)
    w = random_field(n, ny, seed)
    s.set_vorticity(w)
    s.derivatives()
    s.set_hyperviscosity(**(hv or HV_SFD))
    s.d.cfl_factor = 0.5
    omega0 = w.copy()
    dts = []
    for _ in range(steps):
        s.d.dt = s.cfl()
        dts.append(s.d.dt)
        s.advance(1)
    out = dict(omega0=omega0, omega_hat=s.cplx("omega_hat").copy(), sfd_hat=s.cplx("sfd_hat").copy(), t=s.d.t,
               dts=np.array(dts), energy=s.energy(), enstrophy=s.enstrophy(),
               weights=np.ctypeslib.as_array(s.d.hyperviscosity_weights, shape=(s.d.nky, s.d.nkx)).copy())
    s.close()
    return out


def nonlinear(ref, nx, ny, seed=3):
    s = O.Solver(ref, nx, ny, Re=100.0).setup(ic=None)
    s.set_vorticity(random_field(nx, ny, seed))
    s._f("compute_velocity_from_vorticity")(s.ptr)
    wh, ph = s.cplx("omega_hat").copy(), s.cplx("psi_hat").copy()
    s._f("compute_nonlinear_terms")(s.ptr)
    out = dict(omega_hat=wh, psi_hat=ph, nonlinear_hat=s.cplx("nonlinear_hat").copy(), jac=s.real("p").copy())
    s.close()
    return out


def forcing_case(ref):
    """The reference's own forcing test input (tests/test_solvers.c:239-295): 4x4 toy k^2."""
    nkx = nky = 4
    k2 = np.array([[i * i + j * j for i in range(nkx)] for j in range(nky)], dtype=np.float64).ravel()
    out = {"k2": k2}
    fp = ref._fp
    for name, typ, tau, dt in (("white", 0, 0.5, 0.1), ("colored", 1, 0.2, 0.05)):
        cfg = O.ForcingConfig()
        getattr(ref, fp + "config_default")(C.byref(cfg))
        cfg.kmin, cfg.kmax, cfg.energy_target, cfg.seed, cfg.type = 0.5, 2.5, 1.5, 42, typ
        cfg.correlation_time = tau
        st = O.ForcingState()
        rc = getattr(ref, fp + "state_init")(C.byref(st), C.byref(cfg), k2.ctypes.data_as(O._DP), nkx, nky)
        assert rc == 0
        f = np.zeros(nkx * nky, dtype=np.complex128)
        seq = []
        for _ in range(3):
            getattr(ref, fp + "generate")(C.byref(st), dt, k2.ctypes.data_as(O._DP), f.view(np.float64).ctypes.data_as(O._DP))
            seq.append(f.copy())
        out[name] = np.array(seq)
        out[name + "_rng_state"] = np.uint64(st.rng_state)
        out[name + "_active"] = st.active_modes
        getattr(ref, fp + "state_free")(C.byref(st))
    return out


def analysis(ref, n=64, seed=5):
    s = O.Solver(ref, n, n, Re=500.0).setup(ic=None)
    s.set_vorticity(random_field(n, n, seed) * 3.0)
    s.derivatives()
    out = dict(omega=s.real("omega").copy(), energy=s.energy(), enstrophy=s.enstrophy(), cfl=s.cfl())
    s.close()
    return out


def ext_cases(port):
    out = {}
    s = O.Solver(port, 64, 64, Re=1e4).setup(ic=None)
    port.nso_ext_init_random_spectrum(s.ptr, 7, 4.0, 0.5)
    out["ic_omega_hat"] = s.cplx("omega_hat").copy()
    s.set_hyperviscosity(enabled=1, coefficient=2.0, order=4, cutoff_ratio=0.0)
    s.d.cfl_factor = 0.5
    port.nso_ext_run(s.ptr, 20, 1, 1, 4.0, 6.0, 1e-3, 11, 0)
    out["forced_omega_hat"] = s.cplx("omega_hat").copy()
    out["forced_t"] = s.d.t
    s.close()
    return out


def main():
    O.build(ref=True)
    ref = O.load("ref")
    port = O.load("port")
    np.savez_compressed(os.path.join(HERE, "config1_tg32.npz"), **config1(ref, 32, 100))
    np.savez_compressed(os.path.join(HERE, "config1_tg128.npz"), **config1(ref, 128, 1000))
    np.savez_compressed(os.path.join(HERE, "random64_hv_sfd.npz"), **random_hv(ref, 64, 20))
    # grids that are not powers of two (FFTW, and so the reference, takes any size)
    np.savez_compressed(os.path.join(HERE, "config1_tg192.npz"), **config1_benchmark_case(ref, 192, 150))
    np.savez_compressed(os.path.join(HERE, "random96x64_hv_sfd.npz"), **random_hv(ref, 96, 20, seed=2, ny=64))
    np.savez_compressed(os.path.join(HERE, "random45x30_hv.npz"), **random_hv(ref, 45, 10, seed=4, ny=30, hv=HV_ONLY))
    np.savez_compressed(os.path.join(HERE, "nonlinear_32x16.npz"), **nonlinear(ref, 32, 16))
    np.savez_compressed(os.path.join(HERE, "forcing_toy.npz"), **forcing_case(ref))
    np.savez_compressed(os.path.join(HERE, "analysis64.npz"), **analysis(ref))
    np.savez_compressed(os.path.join(HERE, "ext_random_forced64.npz"), **ext_cases(port))
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
