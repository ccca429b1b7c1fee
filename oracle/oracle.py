"""ctypes access to the CPU oracle (test infrastructure only).

Two libraries share one calling convention:

* ``oracle/_build/libns_oracle.so`` -- the project's C restatement of the
  reference spectral step (``oracle/ns_oracle.c``), symbols ``nso_*``;
* ``oracle/_ref/libns_ref.so`` -- the reference's own spectral sources compiled
  unmodified against the project FFTW-API shim (built only where the reference
  tree exists), symbols ``ns_spectral_*``.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU legs import this
module; the GPU product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libns_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libns_ref.so")
# The reference tree is named by the environment (NS_REFERENCE_TREE); without
# it the Makefile's own default location is tried by its ``ref-if-present``
# target, and the reference build is skipped where no tree exists.
REF_TREE = os.environ.get("NS_REFERENCE_TREE") or None


def have_ref() -> bool:
    """True when the reference build (oracle/_ref/libns_ref.so) exists."""
    return os.path.exists(REF_SO)


class HVConfig(C.Structure):
    """NSSpectralHyperviscosityConfig (src/spectral/ns_spectral_solver.h:8-19)."""

    _fields_ = [
        ("enabled", C.c_int),
        ("coefficient", C.c_double),
        ("order", C.c_int),
        ("cutoff_ratio", C.c_double),
        ("sfd_strength", C.c_double),
        ("sfd_timescale", C.c_double),
        ("sfd_enabled", C.c_int),
        ("kmax", C.c_double),
        ("cutoff_wavenumber", C.c_double),
        ("inv_bandwidth", C.c_double),
    ]


_DP = C.POINTER(C.c_double)


class SpectralData(C.Structure):
    """NSSpectralData field order (src/spectral/ns_spectral_solver.h:22-68)."""

    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nkx", C.c_int), ("nky", C.c_int),
        ("Lx", C.c_double), ("Ly", C.c_double), ("Re", C.c_double),
        ("dt", C.c_double), ("t", C.c_double), ("cfl_factor", C.c_double),
        ("u", _DP), ("v", _DP), ("p", _DP), ("omega", _DP), ("psi", _DP),
        ("x", _DP), ("y", _DP),
        ("u_hat", _DP), ("v_hat", _DP), ("omega_hat", _DP), ("psi_hat", _DP),
        ("nonlinear_hat", _DP), ("rk1_hat", _DP), ("rk2_hat", _DP),
        ("rk3_hat", _DP), ("rk4_hat", _DP), ("omega_tmp_hat", _DP),
        ("kx", _DP), ("ky", _DP), ("k2", _DP),
        ("forward_plan", C.c_void_p), ("backward_plan", C.c_void_p),
        ("dealias_mask", C.POINTER(C.c_int)),
        ("hyperviscosity", HVConfig),
        ("hyperviscosity_weights", _DP),
        ("sfd_hat", _DP),
    ]


class ForcingConfig(C.Structure):
    """NSForcingConfig (src/common/forcing.h:12-19)."""

    _fields_ = [
        ("kmin", C.c_double), ("kmax", C.c_double), ("energy_target", C.c_double),
        ("correlation_time", C.c_double), ("seed", C.c_ulong), ("type", C.c_int),
    ]


class ForcingState(C.Structure):
    """NSForcingState (src/common/forcing.h:21-32)."""

    _fields_ = [
        ("config", ForcingConfig), ("nkx", C.c_int), ("nky", C.c_int),
        ("spectral_size", C.c_int), ("active_modes", C.c_int),
        ("weights", _DP), ("colored_state", _DP), ("have_spare", C.c_uint),
        ("spare_gaussian", C.c_double), ("rng_state", C.c_ulonglong),
    ]


def build(ref: bool = True) -> None:
    """Compile the restatement (and the reference build when its tree exists)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if not ref:
        return
    if REF_TREE:
        if os.path.isdir(REF_TREE):
            subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF_TREE}"], check=True)
    else:
        subprocess.run(["make", "-s", "-C", HERE, "ref-if-present"], check=True)


_LIBS: dict = {}


def load(kind: str = "port") -> C.CDLL:
    """Load ``port`` (restatement) or ``ref`` (reference sources) and set prototypes."""
    if kind in _LIBS:
        return _LIBS[kind]
    path = PORT_SO if kind == "port" else REF_SO
    if not os.path.exists(path):
        build(ref=(kind == "ref"))
    lib = C.CDLL(path)
    p = "nso_" if kind == "port" else "ns_spectral_"
    sp = C.POINTER(SpectralData)

    def proto(name, res, *args):
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = list(args)

    proto(p + "allocate", sp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double)
    proto(p + "free", None, sp)
    for name in ("initialize_grids", "initialize_fft_plans", "initialize_taylor_green",
                 "compute_derivatives", "compute_velocity_from_vorticity",
                 "compute_nonlinear_terms", "advance_rk4"):
        proto(p + name, None, sp)
    proto(p + "physical_to_spectral", None, sp, _DP, _DP)
    proto(p + "spectral_to_physical", None, sp, _DP, _DP)
    proto(p + "apply_dealiasing", None, sp, _DP)
    for name in ("compute_cfl_timestep", "compute_energy", "compute_enstrophy"):
        proto(p + name, C.c_double, sp)
    hv = "nso_hv_" if kind == "port" else "ns_spectral_hyperviscosity_"
    proto(hv + "default", None, C.POINTER(HVConfig))
    proto(hv + "set", None, sp, C.POINTER(HVConfig))
    proto(hv + "update_weights", None, sp)
    proto(hv + "apply", None, sp, _DP, _DP)
    proto(hv + "post_step", None, sp, _DP, C.c_double)
    fp = "nso_forcing_" if kind == "port" else "ns_forcing_"
    proto(fp + "config_default", None, C.POINTER(ForcingConfig))
    proto(fp + "state_init", C.c_int, C.POINTER(ForcingState), C.POINTER(ForcingConfig), _DP,
          C.c_int, C.c_int)
    proto(fp + "state_free", None, C.POINTER(ForcingState))
    proto(fp + "generate", None, C.POINTER(ForcingState), C.c_double, _DP, _DP)
    if kind == "port":
        proto("nso_check_resolution", C.c_int, sp, _DP)
        proto("nso_convergence_stats", None, sp, _DP, _DP)
        proto("nso_spectrum", C.c_int, sp, _DP, C.POINTER(C.c_int))
        proto("nso_ext_philox4x64", None, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
              C.POINTER(C.c_uint64))
        proto("nso_ext_init_random_spectrum", None, sp, C.c_uint64, C.c_double, C.c_double)
        proto("nso_ext_run", None, sp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
              C.c_double, C.c_uint64, C.c_uint64)
        proto("nso_ext_run_scheme", None, sp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
              C.c_double, C.c_uint64, C.c_uint64)
    else:
        proto("ns_spectral_check_resolution", C.c_int, sp)
    lib._prefix = p
    lib._hv = hv
    lib._fp = fp
    _LIBS[kind] = lib
    return lib


def _real(ptr, ny, nx) -> np.ndarray:
    return np.ctypeslib.as_array(ptr, shape=(ny, nx))


def _cplx(ptr, nky, nkx) -> np.ndarray:
    return np.ctypeslib.as_array(ptr, shape=(nky, nkx * 2)).view(np.complex128)


class Solver:
    """Drives one solver instance through the reference API of ``lib``.

    Array accessors return live numpy views of the C arrays (writes go through).
    """

    def __init__(self, lib: C.CDLL, nx: int, ny: int, Lx: float = 2 * np.pi,
                 Ly: float = 2 * np.pi, Re: float = 100.0):
        self.lib = lib
        self.p = lib._prefix
        self.ptr = getattr(lib, self.p + "allocate")(nx, ny, Lx, Ly, Re)
        if not self.ptr:
            raise MemoryError("allocate returned NULL")
        self.d = self.ptr.contents

    def _f(self, name):
        return getattr(self.lib, self.p + name)

    def close(self):
        if self.ptr:
            self._f("free")(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- setup -----------------------------------------------------------
    def setup(self, ic: str = "tg"):
        self._f("initialize_grids")(self.ptr)
        self._f("initialize_fft_plans")(self.ptr)
        if ic == "tg":
            self._f("initialize_taylor_green")(self.ptr)
        return self

    # --- arrays ------------------------------------------------------------
    def real(self, name):
        return _real(getattr(self.d, name), self.d.ny, self.d.nx)

    def cplx(self, name):
        return _cplx(getattr(self.d, name), self.d.nky, self.d.nkx)

    def k2(self):
        return np.ctypeslib.as_array(self.d.k2, shape=(self.d.nky, self.d.nkx))

    def mask(self):
        return np.ctypeslib.as_array(self.d.dealias_mask, shape=(self.d.nky, self.d.nkx))

    # --- operations --------------------------------------------------------
    def set_vorticity(self, omega: np.ndarray):
        """Write omega (physical) and transform it, as a caller of the API would."""
        self.real("omega")[:] = omega
        self._f("physical_to_spectral")(self.ptr, self.d.omega, self.d.omega_hat)

    def derivatives(self):
        self._f("compute_derivatives")(self.ptr)

    def advance(self, n: int = 1, adaptive: bool = False):
        for _ in range(n):
            if adaptive:
                self.d.dt = self._f("compute_cfl_timestep")(self.ptr)
            self._f("advance_rk4")(self.ptr)

    def energy(self):
        return self._f("compute_energy")(self.ptr)

    def enstrophy(self):
        return self._f("compute_enstrophy")(self.ptr)

    def cfl(self):
        return self._f("compute_cfl_timestep")(self.ptr)

    def set_hyperviscosity(self, **kw):
        cfg = HVConfig()
        getattr(self.lib, self.lib._hv + "default")(C.byref(cfg))
        for k, v in kw.items():
            setattr(cfg, k, v)
        getattr(self.lib, self.lib._hv + "set")(self.ptr, C.byref(cfg))


def philox4x64(counter, key) -> np.ndarray:
    lib = load("port")
    c = (C.c_uint64 * 4)(*counter)
    k = (C.c_uint64 * 2)(*key)
    o = (C.c_uint64 * 4)()
    lib.nso_ext_philox4x64(c, k, o)
    return np.array(list(o), dtype=np.uint64)
