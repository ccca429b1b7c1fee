"""Python binding (ctypes) of the GB300 drop-in solver library.

Mirrors the reference C API (src/spectral/ns_spectral_solver.h:71-113 of
DiogoRibeiro7/navier-stokes-solvers) and the C-ABI of include/ns_gpu.h, for
tests and benchmarks.  It loads ``libns_gb300.so`` from this directory and
raises if it is missing or no GPU is present: there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libns_gb300.so")

_DP = C.POINTER(C.c_double)


class HVConfig(C.Structure):
    """NSSpectralHyperviscosityConfig (src/spectral/ns_spectral_solver.h:8-19)."""

    _fields_ = [
        ("enabled", C.c_int), ("coefficient", C.c_double), ("order", C.c_int),
        ("cutoff_ratio", C.c_double), ("sfd_strength", C.c_double),
        ("sfd_timescale", C.c_double), ("sfd_enabled", C.c_int), ("kmax", C.c_double),
        ("cutoff_wavenumber", C.c_double), ("inv_bandwidth", C.c_double),
    ]


class SpectralData(C.Structure):
    """NSSpectralData: the reference field order plus the appended ``gpu`` pointer."""

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
        ("gpu", C.c_void_p),
    ]


class ForcingConfig(C.Structure):
    _fields_ = [
        ("kmin", C.c_double), ("kmax", C.c_double), ("energy_target", C.c_double),
        ("correlation_time", C.c_double), ("seed", C.c_ulong), ("type", C.c_int),
    ]


class ForcingState(C.Structure):
    _fields_ = [
        ("config", ForcingConfig), ("nkx", C.c_int), ("nky", C.c_int),
        ("spectral_size", C.c_int), ("active_modes", C.c_int),
        ("weights", _DP), ("colored_state", _DP), ("have_spare", C.c_uint),
        ("spare_gaussian", C.c_double), ("rng_state", C.c_ulonglong),
    ]


class GpuParams(C.Structure):
    """ns_gpu_params (include/ns_gpu.h)."""

    _fields_ = [
        ("Re", C.c_double), ("cfl_factor", C.c_double), ("adaptive_dt", C.c_int),
        ("dt", C.c_double), ("hv_enabled", C.c_int), ("hv_coefficient", C.c_double),
        ("hv_order", C.c_int), ("hv_cutoff_ratio", C.c_double), ("sfd_enabled", C.c_int),
        ("sfd_strength", C.c_double), ("sfd_timescale", C.c_double),
        ("forcing_enabled", C.c_int), ("forcing_kmin", C.c_double),
        ("forcing_kmax", C.c_double), ("forcing_epsilon", C.c_double),
        ("forcing_seed", C.c_uint64), ("scheme", C.c_int), ("forcing_substeps", C.c_int),
    ]


class EnsembleConfig(C.Structure):
    """ns_gpu_ensemble_config (include/ns_gpu.h)."""

    _fields_ = [("threads", C.c_int), ("row_radix", C.c_int), ("col_radix", C.c_int), ("cluster", C.c_int)]

    def as_tuple(self):
        return (self.threads, self.row_radix, self.col_radix, self.cluster)


class Tiling(C.Structure):
    """ns_gpu_tiling (include/ns_gpu.h)."""

    _fields_ = [("row_radix", C.c_int), ("col_radix", C.c_int), ("rows_per_cta", C.c_int),
                ("cols_per_cta", C.c_int), ("row_field_groups", C.c_int), ("col_field_groups", C.c_int),
                ("register_resident", C.c_int)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


FP64, FP32 = 0, 1
_LIB = None


def load(build: bool = True) -> C.CDLL:
    """Load libns_gb300.so (building it first when ``build`` and sources changed)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if build:
        import importlib.util
        spec = importlib.util.spec_from_file_location("ns_gb300_build", os.path.join(PKG, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with build.py (no CPU fallback exists)")
    lib = C.CDLL(LIB_PATH)
    sp = C.POINTER(SpectralData)
    vp = C.c_void_p

    def proto(name, res, *args):
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = list(args)

    proto("ns_spectral_allocate", sp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double)
    proto("ns_spectral_allocate_ex", sp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int)
    proto("ns_spectral_free", None, sp)
    for n in ("initialize_grids", "initialize_fft_plans", "initialize_taylor_green", "compute_derivatives",
              "compute_velocity_from_vorticity", "compute_nonlinear_terms", "advance_rk4", "analyze_spectrum",
              "hyperviscosity_update_weights"):
        proto("ns_spectral_" + n, None, sp)
    proto("ns_spectral_physical_to_spectral", None, sp, _DP, _DP)
    proto("ns_spectral_spectral_to_physical", None, sp, _DP, _DP)
    proto("ns_spectral_apply_dealiasing", None, sp, _DP)
    for n in ("compute_cfl_timestep", "compute_energy", "compute_enstrophy"):
        proto("ns_spectral_" + n, C.c_double, sp)
    proto("ns_spectral_check_resolution", C.c_int, sp)
    proto("ns_spectral_analyze_convergence", None, sp, C.c_int)
    proto("ns_spectral_hyperviscosity_default", None, C.POINTER(HVConfig))
    proto("ns_spectral_hyperviscosity_set", None, sp, C.POINTER(HVConfig))
    proto("ns_spectral_hyperviscosity_apply", None, sp, _DP, _DP)
    proto("ns_spectral_hyperviscosity_post_step", None, sp, _DP, C.c_double)
    proto("ns_spectral_output_solution", None, sp, C.c_char_p)
    proto("ns_spectral_gpu_advance_n", C.c_int, sp, C.c_int, C.c_int)
    proto("ns_spectral_gpu_sync_host", C.c_int, sp)
    proto("ns_spectral_gpu_set_forcing", C.c_int, sp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_ulonglong)
    proto("ns_spectral_gpu_set_scheme", C.c_int, sp, C.c_int)
    proto("ns_spectral_gpu_diagnostics", C.c_int, sp, _DP, _DP)
    proto("ns_spectral_initialize_random_spectrum", C.c_int, sp, C.c_ulonglong, C.c_double, C.c_double)
    proto("ns_spectral_gpu_last_error", C.c_char_p, sp)
    proto("ns_spectral_gpu_handle", vp, sp)
    proto("ns_checkpoint_write_spectral", C.c_int, C.c_char_p, sp)
    proto("ns_checkpoint_read_spectral", C.c_int, C.c_char_p, sp)
    proto("ns_forcing_config_default", None, C.POINTER(ForcingConfig))
    proto("ns_forcing_state_init", C.c_int, C.POINTER(ForcingState), C.POINTER(ForcingConfig), _DP, C.c_int, C.c_int)
    proto("ns_forcing_state_free", None, C.POINTER(ForcingState))
    proto("ns_forcing_generate", None, C.POINTER(ForcingState), C.c_double, _DP, _DP)
    # C-ABI
    proto("ns_gpu_create", C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.POINTER(vp))
    proto("ns_gpu_destroy", None, vp)
    proto("ns_gpu_last_error", C.c_char_p, vp)
    proto("ns_gpu_status_string", C.c_char_p, C.c_int)
    proto("ns_gpu_dims", C.c_int, vp, C.POINTER(C.c_int), C.POINTER(C.c_int))
    proto("ns_gpu_set_params", C.c_int, vp, C.POINTER(GpuParams))
    proto("ns_gpu_synchronize", C.c_int, vp)
    proto("ns_gpu_launch_count", C.c_uint64, vp)
    proto("ns_gpu_upload_state", C.c_int, vp, _DP, _DP, _DP, C.c_double, C.c_double, C.c_uint64)
    proto("ns_gpu_advance", C.c_int, vp, C.c_int)
    proto("ns_gpu_download_state", C.c_int, vp, _DP, _DP, _DP, _DP, _DP, _DP, _DP, _DP, _DP, _DP)
    proto("ns_gpu_diagnostics", C.c_int, vp, _DP, _DP, _DP, _DP)
    proto("ns_gpu_init_random_spectrum", C.c_int, vp, C.c_uint64, C.c_double, C.c_double)
    proto("ns_gpu_random_spectrum_host", C.c_int, vp, C.c_uint64, C.c_double, C.c_double, _DP)
    proto("ns_gpu_state_device_ptr", vp, vp)
    proto("ns_gpu_energy_spectrum", C.c_int, vp, C.c_int, _DP, _DP, C.POINTER(C.c_int))
    fp = C.POINTER(C.c_float)
    proto("ns_gpu_vorticity_device", C.c_int, vp, vp)
    proto("ns_gpu_add_vorticity_device", C.c_int, vp, vp)
    proto("ns_gpu_filter_state", C.c_int, vp, vp)
    proto("ns_ensemble_partition", C.c_int, C.c_int, C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_int), _DP)
    proto("ns_ensemble_member_cost", C.c_double, C.c_int)
    proto("ns_cnn_create", C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint64, C.POINTER(vp))
    proto("ns_cnn_destroy", None, vp)
    proto("ns_cnn_last_error", C.c_char_p, vp)
    proto("ns_cnn_param_count", C.c_int, vp, C.POINTER(C.c_size_t))
    proto("ns_cnn_launch_count", C.c_uint64, vp)
    proto("ns_cnn_get_params", C.c_int, vp, fp)
    proto("ns_cnn_set_params", C.c_int, vp, fp)
    proto("ns_cnn_set_normalization", C.c_int, vp, C.c_float, C.c_float, C.c_float)
    proto("ns_cnn_set_dataset", C.c_int, vp, fp, fp, C.c_int)
    proto("ns_cnn_loss_and_grads", C.c_int, vp, fp, fp, C.c_int, _DP, fp)
    proto("ns_cnn_forward_host", C.c_int, vp, fp, C.c_int, fp)
    proto("ns_cnn_train", C.c_int, vp, C.c_int, C.c_int, C.c_float, C.c_float, C.c_uint64, _DP)
    proto("ns_cnn_correct_step", C.c_int, vp, vp, C.c_int)
    proto("ns_cnn_set_tensor_cores", C.c_int, vp, C.c_int)
    proto("ns_cnn_time_hidden_layer", C.c_int, vp, C.c_int, C.c_int, _DP)
    proto("ns_cnn_time_hidden_layer_inference", C.c_int, vp, C.c_int, C.c_int, _DP)
    proto("ns_cnn_probe_wait_timeout", C.c_int, vp, C.c_longlong, C.POINTER(C.c_int))
    ecp = C.POINTER(EnsembleConfig)
    proto("ns_gpu_create_for_ensemble", C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, ecp, C.POINTER(vp))
    proto("ns_gpu_create_tiled", C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.POINTER(Tiling),
          C.POINTER(vp))
    proto("ns_gpu_get_tiling", C.c_int, vp, C.POINTER(Tiling))
    proto("ns_gpu_ensemble_create", C.c_int, C.c_int, C.POINTER(C.c_int), C.c_double, ecp, C.POINTER(vp))
    proto("ns_gpu_ensemble_destroy", None, vp)
    proto("ns_gpu_ensemble_member", vp, vp, C.c_int)
    proto("ns_gpu_ensemble_advance", C.c_int, vp, C.c_int)
    proto("ns_gpu_ensemble_synchronize", C.c_int, vp)
    proto("ns_gpu_ensemble_advance_timed", C.c_int, vp, C.c_int, C.c_int, _DP)
    proto("ns_gpu_ensemble_reconfigure", C.c_int, vp, ecp)
    proto("ns_gpu_ensemble_autotune", C.c_int, vp, C.c_int, C.c_char_p, ecp, _DP)
    proto("ns_gpu_ensemble_info", C.c_int, vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_size_t),
          C.POINTER(C.c_int), C.POINTER(C.c_uint64))
    proto("ns_gpu_ensemble_last_error", C.c_char_p, vp)
    _LIB = lib
    return lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_DP)


class Solver:
    """One drop-in solver instance driven through the reference API.

    The method names follow ``oracle/oracle.py``'s Solver so a test can run the
    same script against both.  Array accessors return live numpy views of the
    host arrays of the C struct.
    """

    def __init__(self, nx: int, ny: int, Lx: float = 2 * np.pi, Ly: float = 2 * np.pi, Re: float = 100.0,
                 precision: int = FP64):
        self.lib = load()
        self.ptr = self.lib.ns_spectral_allocate_ex(nx, ny, Lx, Ly, Re, precision)
        if not self.ptr:
            raise RuntimeError("ns_spectral_allocate returned NULL (no GPU, or invalid size)")
        self.d = self.ptr.contents

    def close(self):
        if getattr(self, "ptr", None):
            self.lib.ns_spectral_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _f(self, name):
        return getattr(self.lib, "ns_spectral_" + name)

    def setup(self, ic: str = "tg"):
        self._f("initialize_grids")(self.ptr)
        self._f("initialize_fft_plans")(self.ptr)
        if ic == "tg":
            self._f("initialize_taylor_green")(self.ptr)
        return self

    def real(self, name):
        return np.ctypeslib.as_array(getattr(self.d, name), shape=(self.d.ny, self.d.nx))

    def cplx(self, name):
        return np.ctypeslib.as_array(getattr(self.d, name), shape=(self.d.nky, self.d.nkx * 2)).view(np.complex128)

    def k2(self):
        return np.ctypeslib.as_array(self.d.k2, shape=(self.d.nky, self.d.nkx))

    def mask(self):
        return np.ctypeslib.as_array(self.d.dealias_mask, shape=(self.d.nky, self.d.nkx))

    def set_vorticity(self, omega: np.ndarray):
        self.real("omega")[:] = omega
        self._f("physical_to_spectral")(self.ptr, self.d.omega, self.d.omega_hat)

    def derivatives(self):
        self._f("compute_derivatives")(self.ptr)

    def advance(self, n: int = 1, adaptive: bool = False):
        for _ in range(n):
            if adaptive:
                self.d.dt = self._f("compute_cfl_timestep")(self.ptr)
            self._f("advance_rk4")(self.ptr)

    def advance_n(self, n: int, adaptive: bool = False):
        st = self._f("gpu_advance_n")(self.ptr, n, 1 if adaptive else 0)
        if st != 0:
            raise RuntimeError(f"gpu_advance_n failed ({st}): {self._f('gpu_last_error')(self.ptr)}")

    def sync_host(self):
        st = self._f("gpu_sync_host")(self.ptr)
        if st != 0:
            raise RuntimeError(f"gpu_sync_host failed ({st})")

    def set_forcing(self, kmin, kmax, epsilon, seed, enabled=True):
        st = self._f("gpu_set_forcing")(self.ptr, 1 if enabled else 0, kmin, kmax, epsilon, seed)
        if st != 0:
            raise RuntimeError(f"gpu_set_forcing failed ({st})")

    def set_scheme(self, scheme: int):
        """0: the reference RK4, 1: integrating-factor RK4."""
        st = self._f("gpu_set_scheme")(self.ptr, scheme)
        if st != 0:
            raise RuntimeError(f"gpu_set_scheme failed ({st})")

    def diagnostics(self):
        e = C.c_double()
        z = C.c_double()
        st = self._f("gpu_diagnostics")(self.ptr, C.byref(e), C.byref(z))
        if st != 0:
            raise RuntimeError(f"gpu_diagnostics failed ({st})")
        return e.value, z.value

    def random_spectrum(self, seed, k0, energy):
        st = self._f("initialize_random_spectrum")(self.ptr, seed, k0, energy)
        if st != 0:
            raise RuntimeError(f"initialize_random_spectrum failed ({st})")

    def energy(self):
        return self._f("compute_energy")(self.ptr)

    def enstrophy(self):
        return self._f("compute_enstrophy")(self.ptr)

    def cfl(self):
        return self._f("compute_cfl_timestep")(self.ptr)

    def set_hyperviscosity(self, **kw):
        cfg = HVConfig()
        self.lib.ns_spectral_hyperviscosity_default(C.byref(cfg))
        for k, v in kw.items():
            setattr(cfg, k, v)
        self.lib.ns_spectral_hyperviscosity_set(self.ptr, C.byref(cfg))

    def launches(self) -> int:
        return int(self.lib.ns_gpu_launch_count(self.lib.ns_spectral_gpu_handle(self.ptr)))


def ensemble_partition(sizes, nranks: int):
    """rank of every member (ns_ensemble_partition) and the summed cost per rank"""
    lib = load()
    n = (C.c_int * max(1, len(sizes)))(*sizes)
    out = (C.c_int * max(1, len(sizes)))()
    cost = (C.c_double * nranks)()
    st = lib.ns_ensemble_partition(len(sizes), n, nranks, out, cost)
    if st != 0:
        raise RuntimeError(f"ns_ensemble_partition failed: {lib.ns_gpu_status_string(st).decode()}")
    return [int(out[i]) for i in range(len(sizes))], [float(cost[r]) for r in range(nranks)]


class Gpu:
    """Direct use of the C-ABI (include/ns_gpu.h) with a device-resident state."""

    def __init__(self, nx: int, ny: int, Lx: float = 2 * np.pi, Ly: float = 2 * np.pi, precision: int = FP32,
                 ensemble_config: "EnsembleConfig | None" = None, handle=None, tiling: "dict | None" = None):
        self.lib = load()
        self.owned = handle is None
        if handle is None:
            h = C.c_void_p()
            if tiling is not None:
                t = Tiling(**tiling)
                st = self.lib.ns_gpu_create_tiled(nx, ny, Lx, Ly, precision, C.byref(t), C.byref(h))
            elif ensemble_config is None:
                st = self.lib.ns_gpu_create(nx, ny, Lx, Ly, precision, C.byref(h))
            else:
                st = self.lib.ns_gpu_create_for_ensemble(nx, ny, Lx, Ly, precision, C.byref(ensemble_config), C.byref(h))
            if st != 0:
                raise RuntimeError(f"ns_gpu_create failed: {self.lib.ns_gpu_status_string(st).decode()}")
        else:
            h = C.c_void_p(handle)
        self.h = h
        self.nx, self.ny = nx, ny
        self.nkx, self.nky = nx // 2 + 1, ny

    def check(self, st, what):
        if st != 0:
            raise RuntimeError(f"{what} failed ({st}): {self.lib.ns_gpu_last_error(self.h).decode()}")

    def close(self):
        if getattr(self, "h", None):
            if self.owned:
                self.lib.ns_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, **kw):
        p = GpuParams()
        p.Re, p.cfl_factor, p.dt = 1.0, 0.3, 0.01
        p.hv_order, p.hv_cutoff_ratio, p.sfd_timescale = 8, 0.65, 1.0
        for k, v in kw.items():
            setattr(p, k, v)
        self.check(self.lib.ns_gpu_set_params(self.h, C.byref(p)), "set_params")

    def upload(self, omega_hat: np.ndarray, psi_hat=None, sfd_hat=None, t=0.0, dt=0.01, step0=0):
        w = np.ascontiguousarray(omega_hat, dtype=np.complex128)
        p = None if psi_hat is None else np.ascontiguousarray(psi_hat, dtype=np.complex128)
        s = None if sfd_hat is None else np.ascontiguousarray(sfd_hat, dtype=np.complex128)
        self.check(self.lib.ns_gpu_upload_state(self.h, _ptr(w.view(np.float64)),
                                                None if p is None else _ptr(p.view(np.float64)),
                                                None if s is None else _ptr(s.view(np.float64)), t, dt, step0),
                   "upload_state")

    def random_spectrum(self, seed, k0, energy):
        self.check(self.lib.ns_gpu_init_random_spectrum(self.h, seed, k0, energy), "init_random_spectrum")

    def advance(self, n):
        self.check(self.lib.ns_gpu_advance(self.h, n), "advance")

    def sync(self):
        self.check(self.lib.ns_gpu_synchronize(self.h), "synchronize")

    def download(self, fields=("omega_hat",)):
        out = {}
        args = []
        for name in ("omega_hat", "psi_hat", "u_hat", "v_hat", "sfd_hat"):
            if name in fields:
                a = np.zeros((self.nky, self.nkx), dtype=np.complex128)
                out[name] = a
                args.append(_ptr(a.view(np.float64)))
            else:
                args.append(None)
        for name in ("u", "v", "omega"):
            if name in fields:
                a = np.zeros((self.ny, self.nx), dtype=np.float64)
                out[name] = a
                args.append(_ptr(a))
            else:
                args.append(None)
        t = C.c_double()
        dt = C.c_double()
        self.check(self.lib.ns_gpu_download_state(self.h, *args, C.byref(t), C.byref(dt)), "download_state")
        out["t"], out["dt"] = t.value, dt.value
        return out

    def diagnostics(self):
        e, z, t, dt = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        self.check(self.lib.ns_gpu_diagnostics(self.h, C.byref(e), C.byref(z), C.byref(t), C.byref(dt)),
                   "diagnostics")
        return {"energy": e.value, "enstrophy": z.value, "t": t.value, "dt": dt.value}

    def launches(self) -> int:
        return int(self.lib.ns_gpu_launch_count(self.h))

    def energy_spectrum(self, nbins: int | None = None):
        """Shell sums, per-shell means and mode counts (spectral_analysis.c:103-142)."""
        if nbins is None:
            nbins = min(self.nkx, self.nky // 2)
        es = np.zeros(nbins)
        em = np.zeros(nbins)
        ct = np.zeros(nbins, dtype=np.int32)
        self.check(self.lib.ns_gpu_energy_spectrum(self.h, nbins, _ptr(es), _ptr(em),
                                                   ct.ctypes.data_as(C.POINTER(C.c_int))), "energy_spectrum")
        return es, em, ct

    def dims(self):
        a, b = C.c_int(), C.c_int()
        self.lib.ns_gpu_dims(self.h, C.byref(a), C.byref(b))
        return a.value, b.value

    def tiling(self) -> dict:
        """The stage kernels' resolved tiling (ns_gpu_get_tiling)."""
        t = Tiling()
        self.check(self.lib.ns_gpu_get_tiling(self.h, C.byref(t)), "get_tiling")
        return t.as_dict()


class Ensemble:
    """Batched ensemble (ns_gpu_ensemble_*): members of mixed sizes advanced by one
    persistent launch replayed from a CUDA graph."""

    def __init__(self, sizes, L: float = 2 * np.pi, config=(128, 16, 16, 1)):
        self.lib = load()
        self.sizes = [int(n) for n in sizes]
        cfg = EnsembleConfig(*config)
        arr = (C.c_int * len(self.sizes))(*self.sizes)
        h = C.c_void_p()
        st = self.lib.ns_gpu_ensemble_create(len(self.sizes), arr, L, C.byref(cfg), C.byref(h))
        if st != 0:
            raise RuntimeError(f"ns_gpu_ensemble_create failed: {self.lib.ns_gpu_status_string(st).decode()}")
        self.h = h
        self.members = [Gpu(n, n, L, L, handle=self.lib.ns_gpu_ensemble_member(h, i)) for i, n in enumerate(self.sizes)]

    def check(self, st, what):
        if st != 0:
            raise RuntimeError(f"{what} failed ({st}): {self.lib.ns_gpu_ensemble_last_error(self.h).decode()}")

    def advance(self, n: int):
        self.check(self.lib.ns_gpu_ensemble_advance(self.h, n), "ensemble_advance")

    def sync(self):
        self.check(self.lib.ns_gpu_ensemble_synchronize(self.h), "ensemble_synchronize")

    def advance_timed(self, n: int, reps: int = 1) -> float:
        ms = C.c_double()
        self.check(self.lib.ns_gpu_ensemble_advance_timed(self.h, n, reps, C.byref(ms)), "ensemble_advance_timed")
        return ms.value

    def reconfigure(self, config):
        cfg = EnsembleConfig(*config)
        self.check(self.lib.ns_gpu_ensemble_reconfigure(self.h, C.byref(cfg)), "ensemble_reconfigure")

    def autotune(self, steps: int = 2, cache_path: str | None = None):
        best = EnsembleConfig()
        ms = C.c_double()
        self.check(self.lib.ns_gpu_ensemble_autotune(self.h, steps, cache_path.encode() if cache_path else None,
                                                     C.byref(best), C.byref(ms)), "ensemble_autotune")
        return best.as_tuple(), ms.value

    def info(self) -> dict:
        g, t, c = C.c_int(), C.c_int(), C.c_int()
        sm = C.c_size_t()
        ln = C.c_uint64()
        self.check(self.lib.ns_gpu_ensemble_info(self.h, C.byref(g), C.byref(t), C.byref(sm), C.byref(c), C.byref(ln)),
                   "ensemble_info")
        return {"grid": g.value, "threads": t.value, "smem": sm.value, "cluster": c.value, "launches": ln.value}

    def close(self):
        if getattr(self, "h", None):
            for m in self.members:
                m.h = None
            self.lib.ns_gpu_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class Corrector:
    """Learned coarse-grid corrector network (ns_cnn_*)."""

    def __init__(self, height: int, width: int, max_batch: int, seed: int = 1):
        self.lib = load()
        h = C.c_void_p()
        st = self.lib.ns_cnn_create(height, width, max_batch, seed, C.byref(h))
        if st != 0:
            raise RuntimeError(f"ns_cnn_create failed: {self.lib.ns_gpu_status_string(st).decode()}")
        self.h = h
        self.H, self.W = height, width
        n = C.c_size_t()
        self.lib.ns_cnn_param_count(h, C.byref(n))
        self.nparam = n.value

    def check(self, st, what):
        if st != 0:
            raise RuntimeError(f"{what} failed ({st}): {self.lib.ns_cnn_last_error(self.h).decode()}")

    def params(self) -> np.ndarray:
        p = np.zeros(self.nparam, dtype=np.float32)
        self.check(self.lib.ns_cnn_get_params(self.h, _fptr(p)), "get_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        self.check(self.lib.ns_cnn_set_params(self.h, _fptr(p)), "set_params")

    def set_normalization(self, s0, s1, so):
        self.check(self.lib.ns_cnn_set_normalization(self.h, s0, s1, so), "set_normalization")

    def set_dataset(self, inputs, targets):
        i = np.ascontiguousarray(inputs, dtype=np.float32)
        t = np.ascontiguousarray(targets, dtype=np.float32)
        self.check(self.lib.ns_cnn_set_dataset(self.h, _fptr(i), _fptr(t), i.shape[0]), "set_dataset")

    def loss_and_grads(self, inputs, targets):
        i = np.ascontiguousarray(inputs, dtype=np.float32)
        t = np.ascontiguousarray(targets, dtype=np.float32)
        g = np.zeros(self.nparam, dtype=np.float32)
        loss = C.c_double()
        self.check(self.lib.ns_cnn_loss_and_grads(self.h, _fptr(i), _fptr(t), i.shape[0], C.byref(loss), _fptr(g)),
                   "loss_and_grads")
        return loss.value, g

    def forward(self, inputs):
        i = np.ascontiguousarray(inputs, dtype=np.float32)
        out = np.zeros((i.shape[0], self.H, self.W), dtype=np.float32)
        self.check(self.lib.ns_cnn_forward_host(self.h, _fptr(i), i.shape[0], _fptr(out)), "forward")
        return out

    def train(self, iterations, batch, lr, weight_decay=0.0, seed=1):
        hist = np.zeros(iterations)
        self.check(self.lib.ns_cnn_train(self.h, iterations, batch, lr, weight_decay, seed, _ptr(hist)), "train")
        return hist

    def time_hidden_layer(self, batch: int, reps: int = 10) -> float:
        ms = C.c_double()
        self.check(self.lib.ns_cnn_time_hidden_layer(self.h, batch, reps, C.byref(ms)), "time_hidden_layer")
        return ms.value

    def time_hidden_layer_inference(self, batch: int, reps: int = 10) -> float:
        """The same layer on the inference path (BF16 activation out only)."""
        ms = C.c_double()
        self.check(self.lib.ns_cnn_time_hidden_layer_inference(self.h, batch, reps, C.byref(ms)),
                   "time_hidden_layer_inference")
        return ms.value

    def probe_wait_timeout(self, wait_cycles: int) -> int:
        """Failure-detection self-test: a tensor-core launch whose waits run out
        with no MMA issued; returns the kernel's error flag (1 = expiry recorded)."""
        out = C.c_int(-1)
        self.check(self.lib.ns_cnn_probe_wait_timeout(self.h, int(wait_cycles), C.byref(out)), "probe_wait_timeout")
        return out.value

    def set_tensor_cores(self, enable: bool):
        self.check(self.lib.ns_cnn_set_tensor_cores(self.h, 1 if enable else 0), "set_tensor_cores")

    def correct_step(self, gpu: "Gpu", n: int = 1):
        self.check(self.lib.ns_cnn_correct_step(self.h, gpu.h, n), "correct_step")

    def launches(self) -> int:
        return int(self.lib.ns_cnn_launch_count(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.lib.ns_cnn_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
