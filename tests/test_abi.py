"""CPU checks of the C-ABI library: it loads without a GPU, exports every
function the headers in include/ declare, and fails loudly (no CPU fallback)
when no CUDA device is present."""
import ctypes as C
import glob
import os
import re

import pytest

from conftest import ROOT


def _declared_functions():
    names = {}
    for h in sorted(glob.glob(os.path.join(ROOT, "include", "*.h"))):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        txt = re.sub(r"//[^\n]*", "", txt)
        txt = re.sub(r"#[^\n]*", "", txt)
        for m in re.finditer(r"\b([A-Za-z_][\w]*)\s*\(([^;{}]*)\)\s*;", txt):
            name = m.group(1)
            if name.startswith(("ns_", "NS_")):
                names[name] = os.path.basename(h)
    return names


def test_headers_declare_the_reference_api():
    names = _declared_functions()
    reference_api = [
        "ns_spectral_allocate", "ns_spectral_free", "ns_spectral_initialize_grids", "ns_spectral_initialize_fft_plans",
        "ns_spectral_initialize_taylor_green", "ns_spectral_physical_to_spectral", "ns_spectral_spectral_to_physical",
        "ns_spectral_apply_dealiasing", "ns_spectral_compute_derivatives", "ns_spectral_compute_velocity_from_vorticity",
        "ns_spectral_compute_nonlinear_terms", "ns_spectral_advance_rk4", "ns_spectral_compute_cfl_timestep",
        "ns_spectral_compute_energy", "ns_spectral_compute_enstrophy", "ns_spectral_analyze_convergence",
        "ns_spectral_analyze_spectrum", "ns_spectral_check_resolution", "ns_spectral_hyperviscosity_default",
        "ns_spectral_hyperviscosity_set", "ns_spectral_hyperviscosity_update_weights",
        "ns_spectral_hyperviscosity_apply", "ns_spectral_hyperviscosity_post_step", "ns_spectral_output_solution",
        "ns_forcing_config_default", "ns_forcing_state_init", "ns_forcing_state_free", "ns_forcing_generate",
        "ns_config_init", "ns_config_free", "ns_config_set", "ns_config_get_string", "ns_config_get_int",
        "ns_config_get_double", "ns_config_get_bool", "ns_config_has_key", "ns_config_load_files",
        "ns_config_validate",
    ]
    missing = [n for n in reference_api if n not in names]
    assert not missing, missing


def test_library_exports_every_declared_symbol(nsgb):
    lib = C.CDLL(nsgb.LIB_PATH)
    missing = []
    for name, header in _declared_functions().items():
        try:
            getattr(lib, name)
        except AttributeError:
            missing.append(f"{header}:{name}")
    assert not missing, missing


def test_no_cpu_fallback_without_gpu(nsgb):
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:  # pragma: no cover
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present: this checks the no-GPU failure path")
    lib = nsgb.load()
    h = C.c_void_p()
    st = lib.ns_gpu_create(64, 64, 1.0, 1.0, 0, C.byref(h))
    assert st == 2  # NS_GPU_ERR_NO_DEVICE
    assert not h.value
    assert not lib.ns_spectral_allocate(64, 64, 1.0, 1.0, 100.0)
    with pytest.raises(RuntimeError):
        nsgb.Solver(64, 64)


def test_non_pow2_sizes_accepted(nsgb):
    """Sizes the reference's FFTW takes (192^2, 96 x 64, odd 45 x 30, a factor 31)
    pass validation and reach the device check (here: no device)."""
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a GPU is present: this checks validation on a host without one")
    except ImportError:
        pass
    lib = nsgb.load()
    h = C.c_void_p()
    for nx, ny in [(192, 192), (96, 64), (45, 30), (62, 31), (4095, 8), (8, 3000)]:
        assert lib.ns_gpu_create(nx, ny, 1.0, 1.0, 0, C.byref(h)) == 2  # NS_GPU_ERR_NO_DEVICE, not INVALID


def test_invalid_sizes_rejected_before_any_device_call(nsgb):
    lib = nsgb.load()
    h = C.c_void_p()
    # out of [8, 4096], or a transform length with a prime factor above 31
    # (74: row length 37; 37 and 2 * 41 * 3: column lengths)
    for nx, ny in [(64, 4), (8192, 64), (0, 64), (74, 64), (64, 37), (64, 246)]:
        assert lib.ns_gpu_create(nx, ny, 1.0, 1.0, 0, C.byref(h)) == 1  # NS_GPU_ERR_INVALID
    assert lib.ns_gpu_create(64, 64, 1.0, 1.0, 7, C.byref(h)) == 1


def test_invalid_tilings_rejected_before_any_device_call(nsgb):
    """ns_gpu_create_tiled checks the tiling's own fields before it looks for a
    device: radix other than 4 / 16, blocks that are not powers of two, field
    group switches outside -1..1."""
    lib = nsgb.load()
    h = C.c_void_p()
    bad = [dict(row_radix=8), dict(col_radix=2), dict(rows_per_cta=3), dict(cols_per_cta=128),
           dict(row_field_groups=2), dict(col_field_groups=-2), dict(rows_per_cta=-4)]
    for kw in bad:
        t = nsgb.Tiling(**kw)
        assert lib.ns_gpu_create_tiled(256, 256, 1.0, 1.0, 1, C.byref(t), C.byref(h)) == 1, kw
    try:
        import torch

        if torch.cuda.is_available():
            return
    except ImportError:
        pass
    t = nsgb.Tiling(row_radix=16, col_radix=4, rows_per_cta=1, cols_per_cta=2, row_field_groups=1, col_field_groups=1)
    assert lib.ns_gpu_create_tiled(256, 256, 1.0, 1.0, 1, C.byref(t), C.byref(h)) == 2  # valid: no device here
