"""Batched ensembles (ns_gpu_ensemble_*): one persistent launch advances members of
mixed sizes; every member must match the same member advanced alone through the
single-instance path with the same kernel tiling (ns_gpu_create_for_ensemble),
for plain and cluster-shared members.  The two paths run the same stage bodies
inlined into different kernels, where the compiler may fuse different
multiply-adds, so the bar is FP32 rounding (relative L2 <= 2e-6 after 6 steps),
not bit equality; replays of the same ensemble kernel are compared bit for bit.
The single-instance path is itself parity-tested against the oracle
(test_gpu_parity.py, test_gpu_api.py).
"""
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

L = 2 * math.pi


def hv_coefficient(n: int, cfl: float = 0.5) -> float:
    """nu_h |k|^4 in the reference ramp form (cutoff 0, order 4) with damping O(1) per step at 2/3 kmax."""
    kmax = math.hypot(n / 2, n / 2)
    dt_ref = cfl * (2 * math.pi / n) / 3.0
    kd = 2.0 / 3.0 * kmax
    return kmax ** 4 / (kd ** 4 * dt_ref)


def member_params(n: int, seed: int) -> dict:
    return dict(Re=1e4, cfl_factor=0.5, adaptive_dt=1, dt=1e-3, hv_enabled=1, hv_coefficient=hv_coefficient(n),
                hv_order=4, hv_cutoff_ratio=0.0, forcing_enabled=1, forcing_kmin=4.0, forcing_kmax=6.0,
                forcing_epsilon=1e-3, forcing_seed=1000 + seed)


def setup_member(g, n: int, seed: int):
    g.set_params(**member_params(n, seed))
    g.random_spectrum(seed, 4.0, 0.5)


def run_alone(nsgb, n: int, seed: int, steps: int, config):
    g = nsgb.Gpu(n, n, L, L, nsgb.FP32, ensemble_config=nsgb.EnsembleConfig(*config))
    setup_member(g, n, seed)
    g.advance(steps)
    out = g.download(("omega_hat",))
    g.close()
    return out


@pytest.mark.parametrize("config", [(128, 16, 16, 1), (128, 16, 16, 2), (256, 4, 16, 4)])
def test_members_equal_their_own_sequential_runs(nsgb, config):
    sizes = [64, 64, 128, 64, 256, 128, 64]
    steps = 6
    ens = nsgb.Ensemble(sizes, L, config=config)
    for i, (m, n) in enumerate(zip(ens.members, sizes)):
        setup_member(m, n, 17 + i)
    ens.advance(steps - 2)
    ens.advance(2)  # a second launch (new graph) continues from the first
    ens.sync()
    info = ens.info()
    assert info["launches"] == 2 and info["cluster"] == config[3]
    for i, (m, n) in enumerate(zip(ens.members, sizes)):
        got = m.download(("omega_hat",))
        ref = run_alone(nsgb, n, 17 + i, steps, config)
        assert abs(got["t"] - ref["t"]) <= 1e-6 * ref["t"], (i, n, got["t"], ref["t"])
        err = float(np.linalg.norm(got["omega_hat"] - ref["omega_hat"]) / np.linalg.norm(ref["omega_hat"]))
        assert err <= 2e-6, (i, n, err)
        assert np.isfinite(got["omega_hat"]).all()
    ens.close()


def test_graph_replay_matches_separate_launches(nsgb):
    """The same number of steps as 3 x 2 (one graph replayed) and 1 x 6 launches."""
    sizes = [64, 128, 64]
    cfg = (128, 16, 16, 1)
    a = nsgb.Ensemble(sizes, L, config=cfg)
    b = nsgb.Ensemble(sizes, L, config=cfg)
    for e in (a, b):
        for i, (m, n) in enumerate(zip(e.members, sizes)):
            setup_member(m, n, 5 + i)
    for _ in range(3):
        a.advance(2)
    b.advance(6)
    for ma, mb in zip(a.members, b.members):
        x = ma.download(("omega_hat",))["omega_hat"]
        y = mb.download(("omega_hat",))["omega_hat"]
        assert np.array_equal(x, y)
    a.close()
    b.close()


def test_ensemble_energy_budget_and_forcing(nsgb):
    """Forced, hyperviscous members stay finite and near the initial energy over a short horizon."""
    sizes = [64] * 8 + [128] * 4
    ens = nsgb.Ensemble(sizes, L, config=(128, 16, 16, 1))
    for i, (m, n) in enumerate(zip(ens.members, sizes)):
        setup_member(m, n, 100 + i)
    ens.advance(20)
    for m in ens.members:
        d = m.diagnostics()
        assert np.isfinite(d["energy"]) and 0.3 < d["energy"] < 0.7, d
        assert d["t"] > 0
    ens.close()


def test_autotune_picks_a_valid_tiling_and_caches_it(nsgb, tmp_path):
    sizes = [64, 128, 32, 64]
    ens = nsgb.Ensemble(sizes, L, config=(128, 4, 4, 1))
    for i, (m, n) in enumerate(zip(ens.members, sizes)):
        setup_member(m, n, 3 + i)
    cache = str(tmp_path / "tune.jsonl")
    best, ms = ens.autotune(steps=1, cache_path=cache)
    assert ms > 0 and best[0] % 32 == 0 and best[1] in (4, 16) and best[2] in (4, 16) and best[3] in (1, 2, 4, 8)
    assert os.path.exists(cache) and "row_radix" in open(cache).read()
    best2, ms2 = ens.autotune(steps=1, cache_path=cache)  # cache hit: same answer, no timing
    assert best2 == best and ms2 == pytest.approx(ms, rel=1e-5)
    ens.advance(2)
    ens.sync()
    ens.close()


def test_invalid_configurations_are_rejected(nsgb):
    with pytest.raises(RuntimeError):
        nsgb.Ensemble([64, 100], L)  # not a power of two
    with pytest.raises(RuntimeError):
        nsgb.Ensemble([64], L, config=(512, 16, 16, 1))  # 16-value transforms cap a CTA at 256 threads
    with pytest.raises(RuntimeError):
        nsgb.Ensemble([32], L, config=(128, 16, 16, 1))  # a 32^2 row block would need 128 rows


def test_config3_members_against_the_fp64_oracle(nsgb, port):
    """One member of each config-3 size (64^2, 128^2, 256^2), FP32 inside the
    persistent ensemble kernel, against the FP64 oracle at its own size: same
    random-phase initial spectrum (k0 = 4), hyperviscosity p = 2, Philox forcing
    on 4 <= |k| <= 6 with the member's own seed, CFL 0.5 adaptive dt; relative L2
    of the vorticity spectrum <= 1e-5 after 10 steps."""
    import oracle as O

    sizes = [64, 128, 256]
    steps = 10
    ens = nsgb.Ensemble(sizes, L, config=(256, 4, 4, 4))
    for i, (m, n) in enumerate(zip(ens.members, sizes)):
        setup_member(m, n, 40 + i)
    ens.advance(steps)
    ens.sync()
    for i, (m, n) in enumerate(zip(ens.members, sizes)):
        p = member_params(n, 40 + i)
        o = O.Solver(port, n, n, Re=p["Re"]).setup(ic=None)
        port.nso_ext_init_random_spectrum(o.ptr, 40 + i, 4.0, 0.5)
        o.set_hyperviscosity(enabled=1, coefficient=p["hv_coefficient"], order=4, cutoff_ratio=0.0)
        o.d.cfl_factor = p["cfl_factor"]
        port.nso_ext_run(o.ptr, steps, 1, 1, p["forcing_kmin"], p["forcing_kmax"], p["forcing_epsilon"],
                         p["forcing_seed"], 0)
        got = m.download(("omega_hat",))
        ref = o.cplx("omega_hat")
        err = float(np.linalg.norm(got["omega_hat"] - ref) / np.linalg.norm(ref))
        assert err <= 1e-5, (n, err)
        assert abs(got["t"] - o.d.t) <= 1e-6 * o.d.t, (n, got["t"], o.d.t)
        o.close()
    ens.close()
