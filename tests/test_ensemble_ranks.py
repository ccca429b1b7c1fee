"""Ensemble members over ranks: the partition (ns_ensemble_partition) and a
world_size-2 gloo run on CPU.

Members are independent solvers, so a multi-GPU ensemble gives each rank the
members the partition assigns it and gathers only the per-member diagnostics.
Here each rank advances its members through the CPU oracle (the restatement of
the reference step plus the forcing / random-spectrum extensions), and the
gathered diagnostics must equal a one-rank run of all members bit for bit.
"""
import math
import os
import socket
import sys

import pytest

from conftest import ROOT

SIZES = [16] * 6 + [32] * 4 + [64] * 2
STEPS = 4


def _hv(n):
    kmax = math.hypot(n / 2, n / 2)
    dt_ref = 0.5 * (2 * math.pi / n) / 3.0
    return kmax ** 4 / ((2.0 / 3.0 * kmax) ** 4 * dt_ref)


def run_members(port, members):
    """energy, enstrophy, time and the vorticity spectrum's checksum per member"""
    import numpy as np

    import oracle as O

    out = {}
    for m in members:
        n = SIZES[m]
        s = O.Solver(port, n, n, Re=1e4).setup(ic=None)
        port.nso_ext_init_random_spectrum(s.ptr, 100 + m, 2.0, 0.5)
        s.set_hyperviscosity(enabled=1, coefficient=_hv(n), order=4, cutoff_ratio=0.0)
        s.d.cfl_factor = 0.5
        port.nso_ext_run(s.ptr, STEPS, 1, 1, 1.0, 3.0, 1e-3, 7919 * m + 11, 0)
        w = s.cplx("omega_hat")
        out[m] = (s.energy(), s.enstrophy(), s.d.t, float(np.abs(w).sum()), float(np.real(w).sum()))
        s.close()
    return out


def _free_port():
    sk = socket.socket()
    sk.bind(("127.0.0.1", 0))
    p = sk.getsockname()[1]
    sk.close()
    return p


def _rank(rank, world, port_no, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port_no), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, os.path.join(ROOT, "navier-stokes-solvers_gb300"))
    import torch.distributed as dist

    import nsgb
    import oracle as O

    nsgb.load(build=False)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    rank_of, _ = nsgb.ensemble_partition(SIZES, world)
    mine = [m for m in range(len(SIZES)) if rank_of[m] == rank]
    local = run_members(O.load("port"), mine)
    gathered = [None] * world
    dist.all_gather_object(gathered, local)
    merged = {}
    for part in gathered:
        merged.update(part)
    q.put((rank, mine, merged))
    dist.destroy_process_group()


def test_partition_is_lpt_and_complete(nsgb):
    rank_of, cost = nsgb.ensemble_partition(SIZES, 3)
    assert sorted(set(rank_of)) == [0, 1, 2]
    lib = nsgb.load()
    total = sum(lib.ns_ensemble_member_cost(n) for n in SIZES)
    assert abs(sum(cost) - total) <= 1e-9 * total
    # the two 64^2 members (the largest) open two ranks; LPT stays within 4/3 of
    # the lower bound max(total / ranks, largest member)
    assert rank_of[10] != rank_of[11]
    bound = max(total / 3, lib.ns_ensemble_member_cost(64))
    assert max(cost) <= 4.0 / 3.0 * bound
    # deterministic, and one rank takes everything
    assert nsgb.ensemble_partition(SIZES, 3)[0] == rank_of
    assert nsgb.ensemble_partition(SIZES, 1)[0] == [0] * len(SIZES)
    with pytest.raises(RuntimeError):
        nsgb.ensemble_partition([16, 1], 2)


def test_two_ranks_gather_equals_one_rank(nsgb, port):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port_no = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port_no, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    mine0, mine1 = res[0][1], res[1][1]
    assert sorted(mine0 + mine1) == list(range(len(SIZES))) and not set(mine0) & set(mine1)
    assert res[0][2] == res[1][2]  # every rank holds the full gathered table
    single = run_members(port, range(len(SIZES)))
    assert res[0][2] == single
