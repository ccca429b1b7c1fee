"""Learned coarse-grid corrector: training data from this solver, training with the
library's own kernels (ns_cnn_*), evaluation against the filtered fine solution.

No reference counterpart.  The fine solver runs at FINE^2, its state is spectrally
truncated to COARSE^2 (ns_gpu_filter_state) every RATIO fine steps, and the
network learns the difference between the filtered fine state and one plain
coarse step of RATIO x the fine time step:

    input   (omega_c(t), omega_plain(t + D) - omega_c(t))     omega_c = filtered fine
    target  omega_c(t + D) - omega_plain(t + D)

Applied online, every coarse step is a plain RK4 step followed by
omega += CNN(...) (ns_cnn_correct_step); the plain fine solver is the judge of
its error.  All numerics run in the library (ns_gpu_*, ns_cnn_*); this module
only sequences the calls and keeps host copies of the samples.
"""
from __future__ import annotations

import math
import time

import numpy as np

import nsgb

L = 2 * math.pi


def hv_coefficient(n: int, cfl: float = 0.5) -> float:
    """nu_h |k|^4 in the reference ramp form (cutoff 0, order 4): damping O(1) per
    CFL-limited step at 2/3 of the grid's largest wavenumber."""
    kmax = math.hypot(n / 2, n / 2)
    dt_ref = cfl * (2 * math.pi / n) / 3.0
    kd = 2.0 / 3.0 * kmax
    return kmax ** 4 / (kd ** 4 * dt_ref)


def params(n: int, dt: float, Re: float = 1e5, forcing_seed: int | None = None, epsilon: float = 1e-3,
           substeps: int = 1, hv_order: int = 4) -> dict:
    """Config-2 physics on an n^2 grid with a fixed dt.  With forcing, a coarse
    instance takes `substeps` forcing draws per step: the forcing noise is keyed
    by the physical mode and the fine step, so a coarse step of `substeps` fine
    steps receives the fine run's forcing exactly (ns_gpu_params.forcing_substeps)."""
    kmax = math.hypot(n / 2, n / 2)
    dt_ref = 0.5 * (2 * math.pi / n) / 3.0
    c = kmax ** hv_order / ((2.0 / 3.0 * kmax) ** hv_order * dt_ref)  # damping O(1) per step at 2/3 kmax
    p = dict(Re=Re, cfl_factor=0.5, adaptive_dt=0, dt=dt, hv_enabled=1, hv_coefficient=c, hv_order=hv_order,
             hv_cutoff_ratio=0.0)
    if forcing_seed is not None:
        p.update(forcing_enabled=1, forcing_kmin=4.0, forcing_kmax=6.0, forcing_epsilon=epsilon,
                 forcing_seed=forcing_seed, forcing_substeps=substeps)
    return p


def _omega(g: "nsgb.Gpu") -> np.ndarray:
    return g.download(("omega",))["omega"].astype(np.float32)


def _filter(fine: "nsgb.Gpu", coarse: "nsgb.Gpu"):
    fine.check(fine.lib.ns_gpu_filter_state(fine.h, coarse.h), "filter_state")


def fine_dt(fine_n: int, seed: int, k0: float, cfl: float = 0.4) -> float:
    """Fixed fine time step: the reference CFL rule at the initial state, factor cfl."""
    g = nsgb.Gpu(fine_n, fine_n, L, L, nsgb.FP32)
    g.set_params(**dict(params(fine_n, 1e-4), adaptive_dt=1, cfl_factor=cfl))
    g.random_spectrum(seed, k0, 0.5)
    g.advance(1)
    dt = g.diagnostics()["dt"]
    g.close()
    return dt


def generate(seeds, fine_n=1024, coarse_n=256, ratio=8, spinup=200, snapshots=32, k0=8.0, dt_f=None,
             forcing=False, hv_order=4):
    """Samples (inputs [N][2][c][c], targets [N][c][c]) from seeded fine runs."""
    if dt_f is None:
        dt_f = fine_dt(fine_n, seeds[0], k0)
    fine = nsgb.Gpu(fine_n, fine_n, L, L, nsgb.FP32)
    coarse = nsgb.Gpu(coarse_n, coarse_n, L, L, nsgb.FP32)
    xs, ts = [], []
    for seed in seeds:
        fseed = (1000 + seed) if forcing else None
        fine.set_params(**params(fine_n, dt_f, forcing_seed=fseed, hv_order=hv_order))
        coarse.set_params(**params(coarse_n, ratio * dt_f, forcing_seed=fseed, substeps=ratio, hv_order=hv_order))
        fine.random_spectrum(seed, k0, 0.5)
        fine.advance(spinup)
        for _ in range(snapshots):
            _filter(fine, coarse)
            w0 = _omega(coarse)
            coarse.advance(1)
            wp = _omega(coarse)
            fine.advance(ratio)
            _filter(fine, coarse)
            wt = _omega(coarse)
            xs.append(np.stack([w0, wp - w0]))
            ts.append(wt - wp)
    fine.close()
    coarse.close()
    return np.asarray(xs, dtype=np.float32), np.asarray(ts, dtype=np.float32), dt_f


def normalisation(inputs: np.ndarray, targets: np.ndarray):
    """Per-channel scales that make inputs and targets of unit RMS."""
    s0 = 1.0 / max(float(np.sqrt(np.mean(inputs[:, 0] ** 2))), 1e-30)
    s1 = 1.0 / max(float(np.sqrt(np.mean(inputs[:, 1] ** 2))), 1e-30)
    so = 1.0 / max(float(np.sqrt(np.mean(targets ** 2))), 1e-30)
    return s0, s1, so


def rel_l2(a, b) -> float:
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def evaluate(net: "nsgb.Corrector", seeds, horizon, fine_n=1024, coarse_n=256, ratio=8, spinup=200, k0=8.0,
             dt_f=None, forcing=False, every=1):
    """Relative L2 of plain and corrected coarse runs against the filtered fine run
    over `horizon` coarse steps, energy-spectrum error at the end, and wall times."""
    if dt_f is None:
        dt_f = fine_dt(fine_n, seeds[0], k0)
    fine = nsgb.Gpu(fine_n, fine_n, L, L, nsgb.FP32)
    plain = nsgb.Gpu(coarse_n, coarse_n, L, L, nsgb.FP32)
    learned = nsgb.Gpu(coarse_n, coarse_n, L, L, nsgb.FP32)
    out = []
    for seed in seeds:
        fseed = (1000 + seed) if forcing else None
        fine.set_params(**params(fine_n, dt_f, forcing_seed=fseed))
        for g in (plain, learned):
            g.set_params(**params(coarse_n, ratio * dt_f, forcing_seed=fseed, substeps=ratio))
        fine.random_spectrum(seed, k0, 0.5)
        fine.advance(spinup)
        _filter(fine, plain)
        _filter(fine, learned)
        errs_p, errs_l = [], []
        t_fine = t_plain = t_learned = 0.0
        done = 0
        while done < horizon:
            k = min(every, horizon - done)
            # each solver runs k coarse steps' worth as one asynchronous call sequence
            for g in (fine, plain, learned):
                g.sync()
            t0 = time.perf_counter()
            fine.advance(ratio * k)
            fine.sync()
            t_fine += time.perf_counter() - t0
            t0 = time.perf_counter()
            plain.advance(k)
            plain.sync()
            t_plain += time.perf_counter() - t0
            t0 = time.perf_counter()
            net.correct_step(learned, k)
            learned.sync()
            t_learned += time.perf_counter() - t0
            done += k
            truth = nsgb.Gpu(coarse_n, coarse_n, L, L, nsgb.FP32)
            truth.set_params(**params(coarse_n, ratio * dt_f))
            _filter(fine, truth)
            wt = _omega(truth)
            et = truth.energy_spectrum()[1]
            truth.close()
            errs_p.append(rel_l2(_omega(plain), wt))
            errs_l.append(rel_l2(_omega(learned), wt))
        ep = plain.energy_spectrum()[1]
        el = learned.energy_spectrum()[1]
        band = slice(1, coarse_n // 3)
        spec = lambda e: float(np.mean(np.abs(np.log(np.maximum(e[band], 1e-300) / np.maximum(et[band], 1e-300)))))
        out.append({"seed": int(seed), "rel_l2_plain": errs_p, "rel_l2_learned": errs_l,
                    "log_spectrum_error_plain": spec(ep), "log_spectrum_error_learned": spec(el),
                    "wall_s_fine": t_fine, "wall_s_plain": t_plain, "wall_s_learned": t_learned})
    fine.close()
    plain.close()
    learned.close()
    return out, dt_f


def main(argv=None):
    """Config-4 experiment: generate, train, evaluate; one JSON document on stdout."""
    import argparse
    import json

    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--fine", type=int, default=1024)
    ap.add_argument("--coarse", type=int, default=256)
    ap.add_argument("--ratio", type=int, default=8)
    ap.add_argument("--train-seeds", type=int, default=64)
    ap.add_argument("--snapshots", type=int, default=32)
    ap.add_argument("--spinup", type=int, default=200)
    ap.add_argument("--iters", type=int, default=20000)
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--weight-decay", type=float, default=1e-4)
    ap.add_argument("--eval-seeds", type=int, default=16)
    ap.add_argument("--horizon", type=int, default=2000)
    ap.add_argument("--every", type=int, default=50)
    ap.add_argument("--forcing", action="store_true", help="forced runs (shells 4-6, eps 1e-3)")
    ap.add_argument("--save", default=None, help="write the trained parameters (.npy)")
    a = ap.parse_args(argv)
    t0 = time.time()
    x, t, dt_f = generate(list(range(a.train_seeds)), a.fine, a.coarse, a.ratio, a.spinup, a.snapshots,
                          forcing=a.forcing)
    t_gen = time.time() - t0
    s0, s1, so = normalisation(x, t)
    net = nsgb.Corrector(a.coarse, a.coarse, max_batch=a.batch, seed=1)
    net.set_normalization(s0, s1, so)
    net.set_dataset(x, t)
    t0 = time.time()
    hist = net.train(a.iters, a.batch, a.lr, a.weight_decay, seed=7)
    t_train = time.time() - t0
    if a.save:
        np.save(a.save, net.params())
    eval_seeds = list(range(10000, 10000 + a.eval_seeds))
    res, _ = evaluate(net, eval_seeds, a.horizon, a.fine, a.coarse, a.ratio, a.spinup, dt_f=dt_f,
                      forcing=a.forcing, every=a.every)
    mean = lambda key, i: float(np.mean([r[key][i] for r in res]))
    n_eval = len(res[0]["rel_l2_plain"])
    summary = {
        "config": {"fine": a.fine, "coarse": a.coarse, "ratio": a.ratio, "train_seeds": a.train_seeds,
                   "samples": int(x.shape[0]), "iters": a.iters, "batch": a.batch, "horizon": a.horizon,
                   "eval_seeds": a.eval_seeds, "forcing": a.forcing, "dt_fine": dt_f},
        "seconds": {"generate": t_gen, "train": t_train},
        "loss": {"first": float(hist[:10].mean()), "last": float(hist[-100:].mean())},
        "rel_l2_vs_filtered_fine": {
            "coarse_steps": [min((i + 1) * a.every, a.horizon) for i in range(n_eval)],
            "plain": [mean("rel_l2_plain", i) for i in range(n_eval)],
            "learned": [mean("rel_l2_learned", i) for i in range(n_eval)]},
        "log_spectrum_error_end": {"plain": float(np.mean([r["log_spectrum_error_plain"] for r in res])),
                                   "learned": float(np.mean([r["log_spectrum_error_learned"] for r in res]))},
        "wall_s_per_coarse_step": {k: float(np.sum([r[f"wall_s_{k}"] for r in res]) / (a.horizon * len(res)))
                                   for k in ("fine", "plain", "learned")},
        "network_launches": net.launches(),
    }
    net.close()
    print(json.dumps(summary))
    return 0




def ensemble_spectrum_comparison(net: "nsgb.Corrector", fine_n: int, coarse_n: int, ratio: int, members: int,
                                 fine_steps: int, spectrum_every: int, dt_f: float, k0: float = 8.0, seed: int = 0,
                                 hv_order: int = 4, forcing: bool = True):
    """Config-5 comparison: time-averaged energy spectrum of one fine run (spectrum
    every `spectrum_every` fine steps) against that of an ensemble of `members`
    learned-corrected coarse runs of the same statistics (own seeds, same forcing
    parameters), and of the plain coarse ensemble; wall time of each."""
    def prm(n, dt, fseed, sub):
        return params(n, dt, forcing_seed=fseed if forcing else None, substeps=sub, hv_order=hv_order)

    fine = nsgb.Gpu(fine_n, fine_n, L, L, nsgb.FP32)
    fine.set_params(**prm(fine_n, dt_f, 5000 + seed, 1))
    fine.random_spectrum(seed, k0, 0.5)
    nb = coarse_n // 2
    e_fine = np.zeros(nb)
    t0 = time.perf_counter()
    nspec = 0
    for _ in range(fine_steps // spectrum_every):
        fine.advance(spectrum_every)
        e_fine += fine.energy_spectrum(nb)[1]
        nspec += 1
    fine.sync()
    t_fine = time.perf_counter() - t0
    e_fine /= max(nspec, 1)
    fine.close()

    coarse_steps = fine_steps // ratio
    every_c = max(1, spectrum_every // ratio)
    out = {}
    for mode in ("plain", "learned"):
        acc = np.zeros(nb)
        cnt = 0
        t_run = 0.0
        g = nsgb.Gpu(coarse_n, coarse_n, L, L, nsgb.FP32)
        for m in range(members):
            g.set_params(**prm(coarse_n, ratio * dt_f, 7000 + m, ratio))
            g.random_spectrum(100 + m, k0, 0.5)
            g.sync()
            t0 = time.perf_counter()
            for _ in range(coarse_steps // every_c):
                if mode == "plain":
                    g.advance(every_c)
                else:
                    net.correct_step(g, every_c)
                acc += g.energy_spectrum(nb)[1]
                cnt += 1
            g.sync()
            t_run += time.perf_counter() - t0
        g.close()
        acc /= max(cnt, 1)
        band = slice(1, coarse_n // 3)
        err = float(np.mean(np.abs(np.log(np.maximum(acc[band], 1e-300) / np.maximum(e_fine[band], 1e-300)))))
        out[mode] = {"log_spectrum_error": err, "wall_s": t_run, "spectrum": acc.tolist()}
    return {"fine": {"n": fine_n, "steps": fine_steps, "wall_s": t_fine, "spectrum": e_fine.tolist()},
            "coarse": {"n": coarse_n, "members": members, "steps_per_member": coarse_steps}, **out}


def config5(argv=None):
    """Train a fine -> coarse corrector (default 4096^2 -> 512^2) and compare the
    time-averaged E(k) of the fine run with learned and plain coarse ensembles."""
    import argparse
    import json

    ap = argparse.ArgumentParser()
    ap.add_argument("--fine", type=int, default=4096)
    ap.add_argument("--coarse", type=int, default=512)
    ap.add_argument("--ratio", type=int, default=8)
    ap.add_argument("--train-seeds", type=int, default=8)
    ap.add_argument("--snapshots", type=int, default=16)
    ap.add_argument("--iters", type=int, default=1000)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--members", type=int, default=64)
    ap.add_argument("--fine-steps", type=int, default=10000)
    ap.add_argument("--spectrum-every", type=int, default=100)
    ap.add_argument("--hv-order", type=int, default=8, help="hyperviscosity order (p = 4 -> 8)")
    ap.add_argument("--spinup", type=int, default=3000,
                    help="fine steps before the training snapshots: the cascade must have reached the coarse "
                         "cutoff, or the plain coarse step is already exact and the targets are round-off")
    a = ap.parse_args(argv)
    t0 = time.time()
    x, t, dt_f = generate(list(range(a.train_seeds)), a.fine, a.coarse, a.ratio, a.spinup, a.snapshots, forcing=True,
                          hv_order=a.hv_order)
    t_gen = time.time() - t0
    s0, s1, so = normalisation(x, t)
    net = nsgb.Corrector(a.coarse, a.coarse, max_batch=a.batch, seed=1)
    net.set_normalization(s0, s1, so)
    net.set_dataset(x, t)
    t0 = time.time()
    hist = net.train(a.iters, a.batch, 1e-3, 1e-4, seed=11)
    t_train = time.time() - t0
    res = ensemble_spectrum_comparison(net, a.fine, a.coarse, a.ratio, a.members, a.fine_steps, a.spectrum_every,
                                       dt_f, hv_order=a.hv_order)
    net.close()
    res["training"] = {"samples": int(x.shape[0]), "iters": a.iters, "batch": a.batch, "spinup": a.spinup,
                       "target_rms_over_input_rms": float(np.sqrt(np.mean(t ** 2)) / np.sqrt(np.mean(x[:, 0] ** 2))),
                       "generate_s": t_gen,
                       "train_s": t_train, "loss_first": float(hist[:10].mean()), "loss_last": float(hist[-50:].mean())}
    res["dt_fine"] = dt_f
    print(json.dumps(res))
    return 0


def step_timing(argv=None):
    """Wall time of the learned-corrected coarse step (plain RK4 step + network +
    correction) against the plain step, on an untrained network (the time does not
    depend on the weights): `warmup` corrected steps, then `steps` timed ones.  The
    launch sequence a profiler captures for the corrected step."""
    import argparse
    import json

    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--ratio", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--steps", type=int, default=3)
    a = ap.parse_args(argv)
    dt = a.ratio * 7.5e-4
    g = nsgb.Gpu(a.n, a.n, 2 * np.pi, 2 * np.pi, nsgb.FP32)
    g.set_params(**params(a.n, dt, forcing_seed=1000, substeps=a.ratio))
    g.random_spectrum(3, 8.0, 0.5)
    net = nsgb.Corrector(a.n, a.n, max_batch=1, seed=1)
    net.set_normalization(1.0, 1.0, 1.0)
    net.correct_step(g, a.warmup)
    g.sync()
    t0 = time.perf_counter()
    net.correct_step(g, a.steps)
    g.sync()
    t1 = time.perf_counter()
    g.advance(a.steps)
    g.sync()
    t2 = time.perf_counter()
    print(json.dumps({"n": a.n, "steps": a.steps, "learned_ms_per_step": (t1 - t0) / a.steps * 1e3,
                      "plain_ms_per_step": (t2 - t1) / a.steps * 1e3}))
    net.close()
    g.close()
    return 0


if __name__ == "__main__":
    import sys

    if len(sys.argv) > 1 and sys.argv[1] == "config5":
        raise SystemExit(config5(sys.argv[2:]))
    if len(sys.argv) > 1 and sys.argv[1] == "step-timing":
        raise SystemExit(step_timing(sys.argv[2:]))
    raise SystemExit(main())
