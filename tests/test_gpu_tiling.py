"""Stage-kernel tilings (ns_gpu_create_tiled): a thread group per field in the
row and column passes runs every transform with the same arithmetic as one
group per row / column block, so the states agree bit for bit; the automatic
tiling of every size matches the FP64 oracle elsewhere (test_gpu_parity.py)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(nsgb, n, ny, prec, tiling, steps=6, physical=False):
    g = nsgb.Gpu(n, ny, 2 * np.pi, 2 * np.pi, prec, tiling=tiling)
    g.set_params(Re=2000.0, cfl_factor=0.4, adaptive_dt=1, hv_enabled=1, hv_coefficient=1e-6, hv_order=4,
                 hv_cutoff_ratio=0.0, forcing_enabled=1, forcing_kmin=2.0, forcing_kmax=4.0, forcing_epsilon=1e-3,
                 forcing_seed=11)
    g.random_spectrum(5, 4.0, 0.5)
    g.advance(steps)
    if physical:
        d = g.download(("omega_hat", "u", "v", "omega"))
        out = np.concatenate([d["omega_hat"].view(np.float64).ravel()] + [d[k].ravel() for k in ("u", "v", "omega")])
    else:
        out = g.download(("omega_hat",))["omega_hat"]
    t = g.tiling()
    g.close()
    return out, t


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("n,ny,er,ec", [(256, 256, 4, 4), (1024, 512, 16, 16), (512, 256, 4, 4), (256, 128, 4, 4)])
def test_field_groups_bit_identical(nsgb, prec, n, ny, er, ec):
    base = dict(row_radix=er, col_radix=ec)
    a, ta = _run(nsgb, n, ny, prec, dict(base, row_field_groups=-1, col_field_groups=-1))
    b, tb = _run(nsgb, n, ny, prec, dict(base, row_field_groups=1, col_field_groups=1))
    assert ta["row_field_groups"] == -1 and tb["row_field_groups"] == 1 and tb["col_field_groups"] == 1
    assert np.isfinite(a).all()
    assert np.array_equal(a, b)


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("n,rpc", [(32, 1), (64, 1), (64, 2), (128, 1), (128, 4)])
def test_field_groups_narrower_than_a_warp(nsgb, prec, n, rpc):
    """Row transforms of 4, 8 and 16 threads (radix 4 at 32^2 .. 128^2): the four
    groups of a row share warps, every group transforms its own copy of the
    product and stores a quarter of it; column groups of 8 or 16 threads take 4 or
    2 columns each.  The velocity download runs the three-field row pass (three
    groups per row)."""
    base = dict(row_radix=4, col_radix=4, rows_per_cta=rpc)
    a, _ = _run(nsgb, n, n, prec, dict(base, row_field_groups=-1, col_field_groups=-1), physical=True)
    b, tb = _run(nsgb, n, n, prec, dict(base, row_field_groups=1, col_field_groups=1), physical=True)
    assert tb["row_field_groups"] == 1 and tb["col_field_groups"] == 1 and tb["rows_per_cta"] == rpc
    assert tb["cols_per_cta"] * (n // 4) % 32 == 0
    assert np.isfinite(a).all()
    assert np.array_equal(a, b)


def test_field_groups_with_named_barriers(nsgb):
    """Transforms of 64 threads (two warps per field group: named barriers per
    group instead of warp barriers), rows of 2048 points with radix 16."""
    base = dict(row_radix=16, col_radix=16)
    a, _ = _run(nsgb, 2048, 1024, 1, dict(base, row_field_groups=-1, col_field_groups=-1), steps=3)
    b, tb = _run(nsgb, 2048, 1024, 1, dict(base, row_field_groups=1, col_field_groups=1, rows_per_cta=1), steps=3)
    assert tb["row_field_groups"] == 1 and tb["register_resident"] == 0
    assert np.array_equal(a, b)


def test_automatic_tiling_reported(nsgb):
    g = nsgb.Gpu(2048, 2048, precision=1)
    assert g.tiling()["register_resident"] == 3
    g.close()
    g = nsgb.Gpu(256, 256, precision=1)
    t = g.tiling()
    assert t["row_radix"] in (4, 16) and t["rows_per_cta"] >= 1 and t["register_resident"] == 0
    g.close()
    with pytest.raises(RuntimeError):
        # four groups of 64 threads per row at 4 rows per CTA: 1024 threads
        nsgb.Gpu(1024, 1024, precision=1, tiling=dict(row_radix=4, rows_per_cta=4, row_field_groups=1))


@pytest.mark.parametrize("prec", [0, 1])
def test_field_groups_mixed_radix_bit_identical(nsgb, prec):
    """Lengths that are not powers of two (192 x 96: row transform 96 = 2^5 x 3,
    column 96): the mixed-radix bodies with a group per field, each group with its
    own scratch sequence, against one group per row / column block."""
    a, _ = _run(nsgb, 192, 96, prec, dict(row_field_groups=-1, col_field_groups=-1))
    b, tb = _run(nsgb, 192, 96, prec, dict(row_field_groups=1, col_field_groups=1))
    assert tb["row_radix"] == 0 and tb["row_field_groups"] == 1 and tb["col_field_groups"] == 1
    assert np.isfinite(a).all()
    assert np.array_equal(a, b)
