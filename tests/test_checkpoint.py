"""Checkpoint / resume (include/checkpoint.h): the reference's names
(src/common/checkpoint.c:266-360) in an .npz archive.

CPU tests drive the writer and reader on a host-only NSSpectralData (no device
instance attached) and read the file with numpy; the GPU test checks that a run
resumed from a checkpoint continues exactly as the uninterrupted run."""
import ctypes as C

import numpy as np
import pytest


def host_state(nsgb, nx, ny, seed):
    """NSSpectralData over numpy arrays, no device instance (gpu = NULL)."""
    rng = np.random.default_rng(seed)
    nkx, nky = nx // 2 + 1, ny
    arrs = {}
    d = nsgb.SpectralData()
    d.nx, d.ny, d.nkx, d.nky = nx, ny, nkx, nky
    d.Lx, d.Ly, d.Re, d.dt, d.t, d.cfl_factor = 6.0, 7.0, 123.0, 1e-3, 0.25, 0.4
    for name in ("u", "v", "p", "omega", "psi"):
        arrs[name] = rng.standard_normal((ny, nx))
        setattr(d, name, arrs[name].ctypes.data_as(C.POINTER(C.c_double)))
    for name in ("u_hat", "v_hat", "omega_hat", "psi_hat", "sfd_hat"):
        a = rng.standard_normal((nky, nkx)) + 1j * rng.standard_normal((nky, nkx))
        arrs[name] = a
        setattr(d, name, a.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)))
    d.hyperviscosity.enabled = 1
    d.hyperviscosity.coefficient = 0.5
    d.hyperviscosity.order = 6
    d.hyperviscosity.cutoff_ratio = 0.6
    d.hyperviscosity.sfd_strength = 0.1
    d.hyperviscosity.sfd_timescale = 2.0
    d.hyperviscosity.sfd_enabled = 1
    d.gpu = None
    return d, arrs


def test_npz_layout_matches_reference_names(nsgb, tmp_path):
    lib = nsgb.load(build=False)
    d, arrs = host_state(nsgb, 16, 8, 1)
    path = str(tmp_path / "ck.npz")
    assert lib.ns_checkpoint_write_spectral(path.encode(), C.byref(d)) == 0
    z = np.load(path)
    # attributes and datasets of checkpoint.c:272-297
    assert z["solver"].item() == b"spectral"
    assert float(z["time"]) == 0.25 and float(z["dt"]) == 1e-3 and float(z["Re"]) == 123.0
    assert int(z["nx"]) == 16 and int(z["ny"]) == 8 and float(z["Lx"]) == 6.0 and float(z["Ly"]) == 7.0
    for name in ("u", "v", "omega", "psi"):
        assert z[f"fields/{name}"].shape == (8, 16) and np.array_equal(z[f"fields/{name}"], arrs[name])
    for name in ("u_hat", "v_hat", "omega_hat", "psi_hat", "sfd_hat"):
        assert z[f"fields/{name}"].dtype == np.complex128 and np.array_equal(z[f"fields/{name}"], arrs[name])
    hv = z["hyperviscosity"]
    assert hv.shape == (10,) and hv[0] == 1 and hv[1] == 0.5 and hv[2] == 6 and hv[6] == 1
    assert float(z["cfl_factor"]) == 0.4


def test_read_restores_every_array_and_scalar(nsgb, tmp_path):
    lib = nsgb.load(build=False)
    a, arrs = host_state(nsgb, 32, 16, 2)
    path = str(tmp_path / "ck.npz")
    assert lib.ns_checkpoint_write_spectral(path.encode(), C.byref(a)) == 0
    b, brr = host_state(nsgb, 32, 16, 3)
    b.t = b.dt = b.Re = 0.0
    assert lib.ns_checkpoint_read_spectral(path.encode(), C.byref(b)) == 0
    for name in ("u", "v", "omega", "psi", "u_hat", "v_hat", "omega_hat", "psi_hat", "sfd_hat"):
        assert np.array_equal(brr[name], arrs[name]), name
    assert (b.t, b.dt, b.Re, b.Lx, b.Ly, b.cfl_factor) == (0.25, 1e-3, 123.0, 6.0, 7.0, 0.4)
    assert (b.hyperviscosity.order, b.hyperviscosity.sfd_enabled) == (6, 1)


def test_read_rejects_mismatched_grid_and_garbage(nsgb, tmp_path):
    lib = nsgb.load(build=False)
    a, _ = host_state(nsgb, 32, 16, 4)
    path = str(tmp_path / "ck.npz")
    assert lib.ns_checkpoint_write_spectral(path.encode(), C.byref(a)) == 0
    b, _ = host_state(nsgb, 16, 16, 5)
    assert lib.ns_checkpoint_read_spectral(path.encode(), C.byref(b)) == -1
    bad = tmp_path / "bad.npz"
    bad.write_bytes(b"not a zip file at all" * 10)
    assert lib.ns_checkpoint_read_spectral(str(bad).encode(), C.byref(a)) == -1
    assert lib.ns_checkpoint_read_spectral(str(tmp_path / "missing.npz").encode(), C.byref(a)) == -1


def test_failed_read_leaves_state_untouched(nsgb, tmp_path):
    """A file whose omega_hat entry is missing is refused before any array of the
    state is overwritten (u, v, omega, psi come earlier in the file)."""
    lib = nsgb.load(build=False)
    a, _ = host_state(nsgb, 32, 16, 6)
    path = tmp_path / "ck.npz"
    assert lib.ns_checkpoint_write_spectral(str(path).encode(), C.byref(a)) == 0
    bad = tmp_path / "no_omega_hat.npz"
    raw = path.read_bytes()
    assert raw.count(b"fields/omega_hat.npy") == 2  # local header + central directory
    bad.write_bytes(raw.replace(b"fields/omega_hat.npy", b"fields/omegX_hat.npy"))
    b, brr = host_state(nsgb, 32, 16, 7)
    before = {k: v.copy() for k, v in brr.items()}
    t0, dt0 = b.t, b.dt
    assert lib.ns_checkpoint_read_spectral(str(bad).encode(), C.byref(b)) == -1
    for name, v in before.items():
        assert np.array_equal(brr[name], v), name
    assert (b.t, b.dt) == (t0, dt0)


@pytest.mark.gpu
@pytest.mark.parametrize("device_resident", [False, True])
def test_resume_continues_exactly(nsgb, tmp_path, device_resident):
    """10 steps straight == 4 steps, checkpoint, fresh instance, read, 6 steps (FP64,
    hyperviscosity + SFD + forcing, adaptive dt)."""
    lib = nsgb.load(build=False)

    def make():
        s = nsgb.Solver(64, 64, Re=800.0).setup(ic=None)
        s.set_hyperviscosity(enabled=1, coefficient=2.0, order=4, cutoff_ratio=0.3, sfd_enabled=1,
                             sfd_strength=0.05, sfd_timescale=0.5)
        s.set_forcing(3.0, 5.0, 1e-3, 77)
        s.d.cfl_factor = 0.4
        return s

    def run(s, n):
        if device_resident:
            s.advance_n(n, adaptive=True)
        else:
            s.advance(n, adaptive=True)

    a = make()
    a.random_spectrum(9, 5.0, 0.5)
    run(a, 10)
    if device_resident:
        a.sync_host()
    ref = a.cplx("omega_hat").copy()
    t_ref = a.d.t

    b = make()
    b.random_spectrum(9, 5.0, 0.5)
    run(b, 4)
    path = str(tmp_path / "mid.npz")
    assert lib.ns_checkpoint_write_spectral(path.encode(), b.ptr) == 0
    b.close()
    c = make()
    c.set_forcing(1.0, 2.0, 5e-3, 1)  # overwritten by the checkpoint's forcing state
    assert lib.ns_checkpoint_read_spectral(path.encode(), c.ptr) == 0
    run(c, 6)
    if device_resident:
        c.sync_host()
    assert c.d.t == t_ref
    assert np.array_equal(c.cplx("omega_hat"), ref)
    a.close()
    c.close()
