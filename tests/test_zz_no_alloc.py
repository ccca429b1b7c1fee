"""The allocation-free forward transform against the instance path.

ns_gpu_forward_noalloc serves callers that cannot allocate device memory (a host
framework that owns every device allocation through its own pool, a real-time
loop that may not allocate, a process whose device memory is fully reserved):
they pass their own device input and output and the transform uses only the
library's fixed static scratch array.  This file checks, through the C-ABI, that
two calls in a row (different fields, then a different grid, so the second call
must not depend on what the first left in the shared array) give the same
spectrum as the existing entry point (ns_spectral_physical_to_spectral on an
instance, which calls ns_gpu_forward) within the FP64 transform tolerance, and
that an oversized grid is refused before anything runs.

It lives in its own file, named to be collected last, and passes both alone in
a fresh process (where its first call performs the per-device set-up) and after
the other GPU tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-14  # FP64 transforms, as in test_gpu_parity.test_transforms_match_oracle


def _noalloc(lib, nx, ny, field_ptr, out_ptr):
    f = lib.ns_gpu_forward_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    return f(nx, ny, field_ptr, out_ptr, None)


def _instance_forward(nsgb, field):
    ny, nx = field.shape
    s = nsgb.Solver(nx, ny).setup(ic=None)
    s.real("p")[:] = field
    s._f("physical_to_spectral")(s.ptr, s.d.p, s.d.u_hat)
    out = s.cplx("u_hat").copy()
    s.close()
    return out


# (ny, nx) pairs, two calls in a row per case: the second grid differs from the
# first.  (8, 16) runs the radix-4 branches of both passes (a row transform of 8
# points, a column of 8); (1024, 1024) is the largest grid the 8 MiB array admits.
@pytest.mark.parametrize("shape_seq", [((64, 128), (256, 32)), ((8, 16), (1024, 1024))])
def test_forward_noalloc_matches_instance_path(nsgb, shape_seq):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device visible to torch for the test's own buffers")
    lib = nsgb.load()
    rng = np.random.default_rng(2024)
    for ny, nx in shape_seq:
        field = rng.standard_normal((ny, nx))
        expect = _instance_forward(nsgb, field)
        d_in = torch.tensor(field, dtype=torch.float64, device="cuda")
        # poison the output so a mode the call failed to write would show up
        d_out = torch.full((ny, nx // 2 + 1, 2), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        assert _noalloc(lib, nx, ny, d_in.data_ptr(), d_out.data_ptr()) == 0
        torch.cuda.synchronize()
        got = d_out.cpu().numpy().view(np.complex128)[..., 0]
        err = np.linalg.norm(got - expect) / np.linalg.norm(expect)
        assert np.isfinite(got).all()
        assert err <= TOL, f"{nx}x{ny}: relative L2 {err:.3e}"


def test_forward_noalloc_rejects_oversized_grid(nsgb):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device visible to torch for the test's own buffers")
    lib = nsgb.load()
    d_in = torch.zeros((2048, 2048), dtype=torch.float64, device="cuda")
    d_out = torch.zeros((2048, 1025, 2), dtype=torch.float64, device="cuda")
    # a 2048^2 intermediate needs ~22 MiB, above the 8 MiB static array: refused on the host
    assert _noalloc(lib, 2048, 2048, d_in.data_ptr(), d_out.data_ptr()) == 1
