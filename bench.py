#!/usr/bin/env python3
"""Benchmark of the GB300 pseudospectral step (one JSON line on stdout).

Workload (the headline 2048^2 configuration): 2-D incompressible Navier-Stokes,
vorticity-streamfunction, doubly periodic [0, 2pi]^2, 2048 x 2048, FP32 bulk
arithmetic, classical RK4 with 2/3 dealiasing, nu = 1e-5, ramp hyperviscosity
with order 4 (nu_h k^4 form) scaled so the damping at 2/3 kmax is O(1) per
step, white-in-time Philox forcing on shells 4 <= |k| <= 6 at injection rate
1e-3, adaptive dt at CFL 0.5, seeded random-phase initial vorticity with
E(k) ~ k^4 exp(-(k/8)^2) and E = 0.5.  Synthetic data, no files.

  value   grid-pt*steps/s of the device-resident step (C-ABI ns_gpu_advance),
          K steps timed with CUDA events on the library stream, a 256 MiB L2
          flush between steps outside the timed events (the step's working set
          is below the 129 MB L2).
  e2e     the same metric through the reference-facing drop-in API with host
          arrays: per step ns_spectral_compute_cfl_timestep + ns_spectral_advance_rk4
          (the reference's own loop), every host<->device copy inside the timing.
  roofline  the dominant kernel's algorithmic HBM bytes per launch over its mean
          CUDA-event duration, against MEASURED_PEAKS.json hbm_gbs.
  cpu_baseline  the CPU oracle (C restatement of the reference step, FP64,
          OpenMP over all host cores) on a bounded sample of the same workload.

--impl reference times that CPU implementation alone (rank 0).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "navier-stokes-solvers_gb300"))

N = 2048
RE = 1.0e5
K0 = 8.0
E0 = 0.5
CFL = 0.5
F_KMIN, F_KMAX, F_EPS, F_SEED = 4.0, 6.0, 1.0e-3, 20251203
IC_SEED = 1
FLUSH_BYTES = 256 << 20
METRIC = "grid-pt*steps/s at 2048^2 (1 GB300)"
UNIT = "grid-pt*steps/s"


def hv_coefficient(n: int) -> float:
    """Reference HV form w = c (|k|/kmax)^4 (cutoff_ratio 0, order 4) equals nu_h |k|^4
    with c = nu_h kmax^4; nu_h makes w(2/3 kmax) * dt_ref = 1 with dt_ref = CFL dx / 3."""
    kmax = math.hypot(n / 2, n / 2)
    dt_ref = CFL * (2 * math.pi / n) / 3.0
    kd = 2.0 / 3.0 * kmax
    nu_h = 1.0 / (kd ** 4 * dt_ref)
    return nu_h * kmax ** 4


def workload_config(n: int) -> dict:
    return {
        "workload": f"forced 2-D turbulence {n}^2, RK4 + 2/3 dealiasing, hyperviscosity p=2, "
                    f"Philox forcing |k| in [4,6] eps=1e-3, adaptive CFL 0.5",
        "nx": n, "ny": n, "Re": RE, "hv_order": 4, "hv_coefficient": hv_coefficient(n),
        "forcing": {"kmin": F_KMIN, "kmax": F_KMAX, "epsilon": F_EPS},
        "ic": {"spectrum": "k^4 exp(-(k/8)^2)", "energy": E0, "seed": IC_SEED},
        "l2": "256 MiB flush between timed steps (step working set < L2)",
    }


def gpu_params(nsgb_mod, n: int, adaptive: int = 1) -> dict:
    return dict(Re=RE, cfl_factor=CFL, adaptive_dt=adaptive, dt=1e-4, hv_enabled=1,
                hv_coefficient=hv_coefficient(n), hv_order=4, hv_cutoff_ratio=0.0,
                forcing_enabled=1, forcing_kmin=F_KMIN, forcing_kmax=F_KMAX, forcing_epsilon=F_EPS,
                forcing_seed=F_SEED)


# --------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int = 0):
        self.gpu_index = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.gpu_index), "-f", self.path],
                stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sms, maxes, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            with open(self.path) as f:
                for line in f:
                    parts = [p.strip() for p in line.split(",")]
                    if len(parts) < 9:
                        continue
                    try:
                        sms.append(float(parts[1]))
                        maxes.append(float(parts[2]))
                    except ValueError:
                        continue
                    for name, val in zip(names, parts[5:9]):
                        if val.lower().startswith("active"):
                            reasons.add(name)
        except OSError:
            pass
        finally:
            if self.path and os.path.exists(self.path):
                os.unlink(self.path)
        if not sms:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sms), "sm_max_mhz": max(maxes), "reasons": sorted(reasons),
                "samples": len(sms)}


# ----------------------------------------------------------------- peaks
def hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic(kind: str, n: int, prec: str):
    """DRAM bytes per launch of a kernel from the committed ncu summary, if recorded."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    try:
        with open(p) as f:
            for line in f:
                if line.startswith("#") or not line.strip():
                    continue
                kv = dict(tok.split("=", 1) for tok in line.split() if "=" in tok)
                if kv.get("kernel") == kind and int(kv.get("n", 0)) == n and kv.get("prec") == prec:
                    return float(kv["dram_bytes_per_launch"])
    except (OSError, ValueError, KeyError):
        pass
    return None


# the FP32 stage kernels at 2048^2: x-pass (row) and y-pass (column)
STAGE_KERNELS = {"row": "k_row_t", "col": "k_col_q"}


def model_bytes(n: int, elem: int):
    """Algorithmic HBM bytes per launch: row kernel 5A, column kernel 5A + 11C/4
    (A = Kx*ny, C = Kx*Ky complex values; 40A + 11C per RK4 step)."""
    nkx = n // 2 + 1
    kx = (2 * nkx) // 3 + 1
    ky = 2 * ((2 * n) // 6) + 1
    A, Cc = kx * n, kx * ky
    return {"row": 5 * A * elem, "col": (5 * A + 11 * Cc / 4) * elem, "step": (40 * A + 11 * Cc) * elem}


# ------------------------------------------------------- FP64 and horizon legs
def fp64_leg(n: int, steps: int, warmup: int = 3) -> dict:
    """The same 2048^2 workload on the FP64 path (every operation in double, the
    precision of the reference's own solver), timed like the headline: CUDA events
    per step on the library stream with the L2 flush between steps."""
    import ctypes as C

    import nsgb

    g = nsgb.Gpu(n, n, precision=nsgb.FP64)
    g.set_params(**gpu_params(nsgb, n))
    g.random_spectrum(IC_SEED, K0, E0)
    g.advance(warmup)
    g.sync()
    total = C.c_double()
    g.check(g.lib.ns_gpu_advance_timed(g.h, steps, C.c_size_t(FLUSH_BYTES), C.byref(total), None), "advance_timed")
    g.close()
    ms = total.value / steps
    mb = model_bytes(n, 16)
    return {"workload": f"{n}^2, the headline workload in FP64", "dtype": "f64", "steps": steps,
            "ms_per_step": ms, "value": n * n / (ms * 1e-3), "unit": UNIT,
            "step_model_bytes": mb["step"], "step_GBps": mb["step"] / (ms * 1e-3) / 1e9}


def horizon_leg(n: int, steps: int, every: int) -> dict:
    """FP32 bulk against the FP64 path over the full config-2 horizon: the same
    initial spectrum, forcing stream and adaptive-dt rule, sampled every `every`
    steps (relative L2 of the vorticity spectrum, energy and enstrophy error).
    The two runs choose their own dt from their own velocity, so their times are
    reported beside the errors."""
    import nsgb
    import numpy as np

    g64 = nsgb.Gpu(n, n, precision=nsgb.FP64)
    g32 = nsgb.Gpu(n, n, precision=nsgb.FP32)
    for x in (g64, g32):
        x.set_params(**gpu_params(nsgb, n))
        x.random_spectrum(IC_SEED, K0, E0)
    samples = []
    t0 = time.perf_counter()
    done = 0
    while done < steps:
        k = min(every, steps - done)
        g64.advance(k)
        g32.advance(k)
        done += k
        a = g32.download(("omega_hat",))["omega_hat"]
        b = g64.download(("omega_hat",))["omega_hat"]
        d32, d64 = g32.diagnostics(), g64.diagnostics()
        samples.append({"step": done, "rel_l2_vorticity": float(np.linalg.norm(a - b) / np.linalg.norm(b)),
                        "energy_rel_err": abs(d32["energy"] - d64["energy"]) / abs(d64["energy"]),
                        "enstrophy_rel_err": abs(d32["enstrophy"] - d64["enstrophy"]) / abs(d64["enstrophy"]),
                        "t_fp32": d32["t"], "t_fp64": d64["t"], "energy_fp64": d64["energy"],
                        "enstrophy_fp64": d64["enstrophy"]})
    g64.close()
    g32.close()
    return {"workload": f"{n}^2 config-2 physics, FP32 bulk vs FP64, {steps} steps", "every": every,
            "samples": samples, "wall_s": time.perf_counter() - t0}


# ------------------------------------------------------------ ensemble leg
ENS_MIX = ((64, 128), (128, 96), (256, 32))   # (side, members): 4,194,304 points = 2048^2
ENS_K0 = 4.0


def ensemble_member_params(n: int, seed: int) -> dict:
    return dict(Re=RE, cfl_factor=CFL, adaptive_dt=1, dt=1e-4, hv_enabled=1, hv_coefficient=hv_coefficient(n),
                hv_order=4, hv_cutoff_ratio=0.0, forcing_enabled=1, forcing_kmin=F_KMIN, forcing_kmax=F_KMAX,
                forcing_epsilon=F_EPS, forcing_seed=F_SEED + 7919 * seed)


def ensemble_leg(steps: int, seq_steps: int = 10, tiling=None, ws: int = 1, rank: int = 0) -> dict:
    """Config-3 ensemble: one persistent launch (CUDA graph) per `steps` steps versus
    every member advanced alone, one member after another, with the same tiling.
    tiling (threads, row radix, column radix, cluster) skips the autotuner, so the
    first ensemble launch is the untimed warm-up of that tiling (ncu captures).
    With ws > 1 ranks, each rank runs the members ns_ensemble_partition gives it
    (member seeds stay the global member index) and the value is all members'
    points over the slowest rank's time."""
    import nsgb

    all_sizes = [n for n, cnt in ENS_MIX for _ in range(cnt)]
    rank_of, rank_cost = nsgb.ensemble_partition(all_sizes, ws)
    mine = [i for i in range(len(all_sizes)) if rank_of[i] == rank]
    sizes = [all_sizes[i] for i in mine]
    ens = nsgb.Ensemble(sizes, 2 * math.pi, config=tuple(tiling) if tiling else (128, 16, 16, 1))
    cache = os.path.join(ROOT, "navier-stokes-solvers_gb300", "_build", "ensemble_tune.jsonl")
    os.makedirs(os.path.dirname(cache), exist_ok=True)
    for i, m, n in zip(mine, ens.members, sizes):
        m.set_params(**ensemble_member_params(n, i))
        m.random_spectrum(IC_SEED + i, ENS_K0, E0)
    if tiling:
        best, tune_ms = tuple(tiling), None
    else:
        best, tune_ms = ens.autotune(steps=2, cache_path=cache)
        for i, m in zip(mine, ens.members):  # tuning advanced the members: restart
            m.random_spectrum(IC_SEED + i, ENS_K0, E0)
    ens.advance(3)
    barrier(ws)
    ms = reduce_max(ens.advance_timed(steps, 1), ws)
    points = sum(n * n for n in all_sizes)
    energies = [m.diagnostics()["energy"] for m in ens.members]
    info = ens.info()
    ens.close()
    if ws > 1:
        value = points * steps / (ms * 1e-3)
        return {"workload": "config-3 ensemble over ranks (256 members: 128 x 64^2, 96 x 128^2, 32 x 256^2)",
                "metric": "aggregate grid-pt*steps/s", "value": value, "steps": steps, "ms_per_step": ms / steps,
                "ranks": ws, "members_on_rank0": len(mine), "partition": "ns_ensemble_partition (LPT on n^2 log n^2)",
                "rank_cost": rank_cost, "scaling": "strong (fixed member set split over ranks)"}

    # the same members one after another through the single-instance path
    cfg = nsgb.EnsembleConfig(*best)
    seq = []
    for i, n in enumerate(sizes):
        g = nsgb.Gpu(n, n, 2 * math.pi, 2 * math.pi, nsgb.FP32, ensemble_config=cfg)
        g.set_params(**ensemble_member_params(n, i))
        g.random_spectrum(IC_SEED + i, ENS_K0, E0)
        g.advance(2)
        g.sync()
        seq.append(g)
    t0 = time.perf_counter()
    for g in seq:
        g.advance(seq_steps)
        g.sync()
    seq_s = time.perf_counter() - t0
    for g in seq:
        g.close()
    value = points * steps / (ms * 1e-3)
    seq_value = points * seq_steps / seq_s
    return {"workload": "ensemble of 256 members: 128 x 64^2, 96 x 128^2, 32 x 256^2 (4,194,304 points), FP32, "
                        "RK4 + hyperviscosity p=2, own seeds for the k0=4 initial spectrum and the forcing, "
                        "per-member adaptive dt at CFL 0.5",
            "metric": "aggregate grid-pt*steps/s", "value": value, "steps": steps, "ms_per_step": ms / steps,
            "launches_per_advance": 1, "graph": True, "tiling": {"threads": best[0], "row_radix": best[1],
                                                                   "col_radix": best[2], "cluster": best[3]},
            "grid": info["grid"], "smem_bytes": info["smem"], "autotune_ms_per_step": tune_ms,
            "sequential": {"value": seq_value, "steps_per_member": seq_steps,
                           "how": "each member alone (ns_gpu_advance, same tiling), one after another, host-synchronised"},
            "speedup_vs_sequential": value / seq_value,
            "energy_min_max": [min(energies), max(energies)],
            "l2": "members stay resident in L2 (state ~ 2048^2 single field); no flush inside the persistent launch"}


# ----------------------------------------------------- corrector / config-5 legs
def corrector_leg(steps: int = 20, batch: int = 32) -> dict:
    """Wall time of the learned-corrected 256^2 step against the 8 fine 1024^2 steps it
    replaces (timing does not depend on the weights), and the tensor-core roofline of
    the network's dominant kernel (one 64 -> 64 hidden layer on a training batch)."""
    import nsgb
    import corrector as CR

    fine_n, coarse_n, ratio = 1024, 256, 8
    dt_f = CR.fine_dt(fine_n, IC_SEED, K0)
    fine = nsgb.Gpu(fine_n, fine_n, 2 * math.pi, 2 * math.pi, nsgb.FP32)
    plain = nsgb.Gpu(coarse_n, coarse_n, 2 * math.pi, 2 * math.pi, nsgb.FP32)
    learned = nsgb.Gpu(coarse_n, coarse_n, 2 * math.pi, 2 * math.pi, nsgb.FP32)
    fine.set_params(**CR.params(fine_n, dt_f, forcing_seed=F_SEED))
    for g in (plain, learned):
        g.set_params(**CR.params(coarse_n, ratio * dt_f, forcing_seed=F_SEED, substeps=ratio))
    fine.random_spectrum(IC_SEED, K0, E0)
    fine.advance(2)
    for g in (plain, learned):
        fine.check(fine.lib.ns_gpu_filter_state(fine.h, g.h), "filter_state")
    net = nsgb.Corrector(coarse_n, coarse_n, max_batch=batch, seed=1)
    fine.advance(ratio)
    plain.advance(1)
    net.correct_step(learned, 1)
    for g in (fine, plain, learned):
        g.sync()

    def wall(fn):
        t0 = time.perf_counter()
        fn()
        return time.perf_counter() - t0

    t_fine = wall(lambda: (fine.advance(ratio * steps), fine.sync()))
    t_plain = wall(lambda: (plain.advance(steps), plain.sync()))
    t_learned = wall(lambda: (net.correct_step(learned, steps), learned.sync()))
    ms_inf = net.time_hidden_layer_inference(batch, 10)
    ms_tc = net.time_hidden_layer(batch, 10)
    net.set_tensor_cores(False)
    ms_simt = net.time_hidden_layer(batch, 2)
    net.set_tensor_cores(True)
    npx = batch * coarse_n * coarse_n
    flops = 2.0 * npx * 64 * 576
    tflops = flops / (ms_inf * 1e-3) / 1e12
    tflops_train = flops / (ms_tc * 1e-3) / 1e12
    # training-path layer: BF16 input read, FP32 pre-activation + FP32 activation + BF16 activation written
    train_bytes = npx * 64 * (2 + 4 + 4 + 2)
    peak = None
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        peak, hbm_peak = float(pk["bf16_tflops"]), float(pk["hbm_gbs"])
        peak_src = "measured"
    except (OSError, KeyError, ValueError):
        peak, hbm_peak, peak_src = 1900.0, 6800.0, "fallback"
    for x in (fine, plain, learned):
        x.close()
    net.close()
    return {"workload": "learned-corrected 256^2 step (plain RK4 + CNN) vs 8 steps of 1024^2 (config-2 physics, "
                        "matched forcing)", "steps": steps,
            "ms_per_coarse_step": {"fine_1024_x8": t_fine / steps * 1e3, "plain_256": t_plain / steps * 1e3,
                                   "learned_256": t_learned / steps * 1e3},
            "wall_ratio_fine_over_learned": t_fine / t_learned,
            "tensor_roofline": {"kernel": "k_conv_tc (64->64 3x3, tcgen05 BF16 -> FP32 TMEM)", "bound": "tensor",
                                "path": "inference: BF16 activation in and out (the layer the corrected step runs)",
                                "batch": batch, "flops_per_launch": flops, "mean_launch_ms": ms_inf,
                                "achieved": tflops, "peak": peak, "unit": "TFLOP/s", "frac": tflops / peak,
                                "peak_source": peak_src},
            "tensor_roofline_training": {"path": "training: FP32 pre-activation and activation plus the BF16 "
                                                 "activation written (the backward pass reads them)",
                                         "batch": batch, "mean_launch_ms": ms_tc, "achieved_tflops": tflops_train,
                                         "frac_tensor": tflops_train / peak, "hbm_bytes_per_launch": train_bytes,
                                         "achieved_GBps": train_bytes / (ms_tc * 1e-3) / 1e9,
                                         "frac_hbm": train_bytes / (ms_tc * 1e-3) / 1e9 / hbm_peak},
            "simt_same_layer_ms": ms_simt,
            "accuracy": "not measured in this leg: the trained network's error against the filtered 1024^2 run "
                        "comes from navier-stokes-solvers_gb300/corrector.py on held-out seeds"}


def config5_leg(steps: int = 10) -> dict:
    """4096^2 forced run (FP32 bulk, p=4 hyperviscosity, CFL 0.4) on the 4096-point row
    (k_row_4k) and column (k_col_q) passes, with the energy spectrum of the device state."""
    import nsgb

    n = 4096
    g = nsgb.Gpu(n, n, 2 * math.pi, 2 * math.pi, nsgb.FP32)
    kmax = math.hypot(n / 2, n / 2)
    dt_ref = 0.4 * (2 * math.pi / n) / 3.0
    c8 = kmax ** 8 / ((2.0 / 3.0 * kmax) ** 8 * dt_ref)
    g.set_params(Re=RE, cfl_factor=0.4, adaptive_dt=1, dt=1e-4, hv_enabled=1, hv_coefficient=c8, hv_order=8,
                 hv_cutoff_ratio=0.0, forcing_enabled=1, forcing_kmin=F_KMIN, forcing_kmax=F_KMAX,
                 forcing_epsilon=F_EPS, forcing_seed=F_SEED)
    g.random_spectrum(IC_SEED, K0, E0)
    g.advance(3)
    import ctypes as C

    total = C.c_double()
    g.check(g.lib.ns_gpu_advance_timed(g.h, steps, C.c_size_t(0), C.byref(total), None), "advance_timed")
    t0 = time.perf_counter()
    es, em, ct = g.energy_spectrum()
    t_spec = time.perf_counter() - t0
    d = g.diagnostics()
    g.close()
    return {"workload": "forced 4096^2, FP32, RK4, hyperviscosity p=4 (order 8), CFL 0.4, stage kernels k_row_4k / k_col_q",
            "value": n * n * steps / (total.value * 1e-3), "unit": UNIT, "ms_per_step": total.value / steps,
            "spectrum_ms": t_spec * 1e3, "spectrum_bins": int(len(es)), "energy": d["energy"],
            "l2": "working set above L2; no flush"}


# ------------------------------------------------------------ CPU legs
def cpu_sample(n: int, budget_s: float, max_steps: int):
    """Time the oracle restatement (FP64, OpenMP) on the workload for up to budget_s."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build(ref=False)
    lib = O.load("port")
    s = O.Solver(lib, n, n, Re=RE).setup(ic=None)
    lib.nso_ext_init_random_spectrum(s.ptr, IC_SEED, K0, E0)
    s.set_hyperviscosity(enabled=1, coefficient=hv_coefficient(n), order=4, cutoff_ratio=0.0)
    s.d.cfl_factor = CFL
    t0 = time.perf_counter()
    steps = 0
    while steps < max_steps:
        lib.nso_ext_run(s.ptr, 1, 1, 1, F_KMIN, F_KMAX, F_EPS, F_SEED, steps)
        steps += 1
        if time.perf_counter() - t0 > budget_s:
            break
    el = time.perf_counter() - t0
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": n * n * steps / el, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{steps} RK4 step(s) of the {n}^2 workload in FP64 on the oracle restatement "
                      f"(project FFT shim, not FFTW), {el:.1f} s"}


# ---------------------------------------------------------------- main
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def reduce_max(x: float, ws: int):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_value(n: int, steps: int, ws: int, ms_total: float) -> float:
    """Whole-job grid-pt*steps/s: every replica's points over the slowest rank's time."""
    return n * n * steps * ws / (ms_total * 1e-3)


def barrier(ws: int):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def run_reference(args, ws, rank):
    if rank != 0:
        return 0
    budget = float(os.environ.get("NS_BENCH_REF_BUDGET_S", "90"))
    cb = cpu_sample(N, budget, max(1, args.steps))
    line = {
        "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": N * N / cb["value"] * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(N), "impl": "reference",
        "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--kernels-only", action="store_true",
                    help="only warmup + timed steps (a short launch sequence for ncu captures); prints no JSON")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--ensemble-steps", type=int, default=100, help="steps of the timed ensemble launch (0: skip)")
    ap.add_argument("--ensemble-only", action="store_true", help="run only the ensemble leg and print its JSON")
    ap.add_argument("--ensemble-tiling", default="",
                    help="threads,row_radix,col_radix,cluster for the ensemble leg instead of the autotuner")
    ap.add_argument("--no-extra", action="store_true", help="skip the corrector and 4096^2 legs")
    ap.add_argument("--fp64-steps", type=int, default=20, help="timed steps of the FP64 leg (0: skip)")
    ap.add_argument("--horizon-steps", type=int, default=5000,
                    help="steps of the FP32-vs-FP64 horizon comparison (config 2: 5000; 0: skip)")
    ap.add_argument("--horizon-every", type=int, default=500)
    ap.add_argument("--extra-only", action="store_true", help="run only the corrector and 4096^2 legs")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    ws, rank, local = dist_env()
    if ws > 1:
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local))
        import torch.distributed as dist

        dist.init_process_group("gloo")
    if args.impl == "reference":
        rc = run_reference(args, ws, rank)
        if ws > 1:
            import torch.distributed as dist

            dist.destroy_process_group()
        return rc

    import numpy as np
    import nsgb

    ens_tiling = tuple(int(x) for x in args.ensemble_tiling.split(",")) if args.ensemble_tiling else None
    if args.ensemble_only:
        print(json.dumps(ensemble_leg(max(1, args.ensemble_steps), tiling=ens_tiling)), flush=True)
        return 0
    if args.extra_only:
        print(json.dumps({"corrector": corrector_leg(), "config5_4096": config5_leg()}), flush=True)
        return 0

    n = args.n
    prec = nsgb.FP32 if args.precision == "fp32" else nsgb.FP64
    g = nsgb.Gpu(n, n, precision=prec)
    g.set_params(**gpu_params(nsgb, n))
    g.random_spectrum(IC_SEED, K0, E0)
    g.advance(args.warmup)
    g.sync()
    if args.kernels_only:
        g.advance(args.steps)
        g.sync()
        d = g.diagnostics()
        print(f"kernels-only: {n}^2 {args.precision} {args.steps} steps, E={d['energy']:.6e}", file=sys.stderr)
        g.close()
        return 0

    barrier(ws)
    launches0 = g.launches()
    import ctypes as C

    total = C.c_double()
    with ClockSampler(0) as clk:
        t_wall0 = time.perf_counter()
        g.check(g.lib.ns_gpu_advance_timed(g.h, args.steps, C.c_size_t(FLUSH_BYTES), C.byref(total), None),
                "advance_timed")
        t_wall = time.perf_counter() - t_wall0
    clocks = clk.summary()
    launches = g.launches() - launches0
    ms_total = reduce_max(total.value, ws)
    barrier(ws)
    diag = g.diagnostics()
    value = aggregate_value(n, args.steps, ws, ms_total)

    # per-kernel CUDA-event timing for the roofline (separate pass, same flush)
    prof_steps = min(args.steps, 50)
    kms = (C.c_double * 2)()
    kcnt = (C.c_int * 2)()
    g.check(g.lib.ns_gpu_profile_kernels(g.h, prof_steps, C.c_size_t(FLUSH_BYTES), kms, kcnt), "profile_kernels")
    mb = model_bytes(n, 8)
    row_ms, col_ms = kms[0] / max(kcnt[0], 1), kms[1] / max(kcnt[1], 1)
    dom = "row" if kms[0] >= kms[1] else "col"
    dom_ms = row_ms if dom == "row" else col_ms
    peak, peak_src = hbm_peak()
    achieved = mb[dom] / (dom_ms * 1e-3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": ncu_traffic(dom, n, "fp32"), "kernel": f"{STAGE_KERNELS[dom]} (FP32, {n}^2)",
                "peak_source": peak_src,
                "algorithmic_bytes_per_launch": mb[dom], "mean_launch_ms": dom_ms,
                "kernels": {"row": {"mean_ms": row_ms, "launches": kcnt[0], "bytes": mb["row"],
                                    "GBps": mb["row"] / (row_ms * 1e-3) / 1e9},
                            "col": {"mean_ms": col_ms, "launches": kcnt[1], "bytes": mb["col"],
                                    "GBps": mb["col"] / (col_ms * 1e-3) / 1e9}},
                "step_model_bytes": mb["step"],
                "step_GBps": mb["step"] / (ms_total / args.steps * 1e-3) / 1e9}

    # FP32 bulk vs FP64 on the device, same IC and forcing, short horizon
    cmp_steps = 20
    g64 = nsgb.Gpu(n, n, precision=nsgb.FP64)
    g32 = nsgb.Gpu(n, n, precision=nsgb.FP32)
    for x in (g64, g32):
        x.set_params(**gpu_params(nsgb, n))
        x.random_spectrum(IC_SEED, K0, E0)
        x.advance(cmp_steps)
    a = g32.download(("omega_hat",))
    b = g64.download(("omega_hat",))
    d32, d64 = g32.diagnostics(), g64.diagnostics()
    fp32_cmp = {"steps": cmp_steps,
                "rel_l2_vorticity": float(np.linalg.norm(a["omega_hat"] - b["omega_hat"]) / np.linalg.norm(b["omega_hat"])),
                "energy_rel_err": abs(d32["energy"] - d64["energy"]) / abs(d64["energy"]),
                "enstrophy_rel_err": abs(d32["enstrophy"] - d64["enstrophy"]) / abs(d64["enstrophy"]),
                "t_fp32": d32["t"], "t_fp64": d64["t"]}
    g64.close()
    g32.close()

    # end to end through the drop-in reference API (host arrays, copies inside the timing)
    e2e = None
    if not args.no_e2e:
        s = nsgb.Solver(n, n, Re=RE, precision=nsgb.FP32).setup(ic=None)
        s.set_hyperviscosity(enabled=1, coefficient=hv_coefficient(n), order=4, cutoff_ratio=0.0)
        s.set_forcing(F_KMIN, F_KMAX, F_EPS, F_SEED)
        s.d.cfl_factor = CFL
        s.random_spectrum(IC_SEED, K0, E0)
        s.advance(2, adaptive=True)
        e_steps = max(3, min(args.steps, 20))
        t0 = time.perf_counter()
        s.advance(e_steps, adaptive=True)
        el = time.perf_counter() - t0
        nr, nc = n * n * 8, (n // 2 + 1) * n * 16
        kx_kept, ky_kept = (2 * (n // 2 + 1)) // 3 + 1, 2 * ((2 * n) // 6) + 1
        kept = kx_kept * ky_kept * 16
        # in: u, v (CFL) and omega_hat, psi_hat; out: u_hat, v_hat, u, v, omega in full
        # and the kept modes of omega_hat, psi_hat (their masked modes were zero on
        # entry and stay zero, so the step leaves them in place)
        e2e = {"value": n * n * e_steps / el, "unit": UNIT, "steps": e_steps,
               "h2d_bytes_per_step": 2 * nr + 2 * nc, "d2h_bytes_per_step": 2 * kept + 2 * nc + 3 * nr,
               "path": "ns_spectral_compute_cfl_timestep + ns_spectral_advance_rk4 per step (FP32 instance; "
                       "copies overlapped on two streams by ns_gpu_step_host)"}
        s.close()

    # the ensemble members are split over the ranks (ns_ensemble_partition); the
    # other secondary workloads run once, on rank 0 (replicas add nothing to them)
    ens = corr = c5 = f64 = horizon = None
    if args.ensemble_steps > 0:
        ens = ensemble_leg(args.ensemble_steps, tiling=ens_tiling, ws=ws, rank=rank)
    if rank == 0:
        if args.fp64_steps > 0:
            f64 = fp64_leg(n, args.fp64_steps)
        if args.horizon_steps > 0:
            horizon = horizon_leg(n, args.horizon_steps, max(1, args.horizon_every))
        if not args.no_extra:
            corr = corrector_leg()
            c5 = config5_leg()

    cpu = None
    if not args.no_cpu and rank == 0 and ws == 1:
        cpu = cpu_sample(n, float(os.environ.get("NS_BENCH_CPU_BUDGET_S", "15")), 20)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_total / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic", "config": workload_config(n),
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
        "gpu_launches": launches, "wall_s_timed_region": t_wall,
        "fp32_vs_fp64": fp32_cmp,
        "fp64": f64,
        "fp32_vs_fp64_horizon": horizon,
        "ensemble": ens,
        "corrector": corr,
        "config5_4096": c5,
        "diagnostics": {"energy": diag["energy"], "enstrophy": diag["enstrophy"], "t": diag["t"], "dt": diag["dt"]},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    g.close()
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
