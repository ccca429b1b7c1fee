"""bench.py's multi-rank path on CPU: world_size-2 gloo ranks.

The single-field step does not shard (one all-to-all transpose per 2-D FFT),
so N GPUs run N independent replicas (weak scaling, no data-path collective);
the only cross-rank operations are the barrier and the max-over-ranks of the
timed region, which these ranks exercise through bench.py's own helpers.
"""
import os
import socket
import sys

import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    ws, r, local = bench.dist_env()
    local_ms = 10.0 + 5.0 * rank          # ranks finish at different times
    bench.barrier(ws)
    ms = bench.reduce_max(local_ms, ws)
    value = bench.aggregate_value(n=64, steps=3, ws=ws, ms_total=ms)
    q.put((r, ws, local, ms, value))
    dist.destroy_process_group()


def test_two_rank_replicas_take_the_max_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    assert all(o[1] == 2 for o in out)
    assert all(o[3] == 15.0 for o in out)  # max over ranks, identical on every rank
    # whole-job throughput: both replicas' points over the slowest rank's time
    assert all(abs(o[4] - 64 * 64 * 3 * 2 / 15e-3) < 1e-6 * o[4] for o in out)


def test_single_rank_helpers_are_identity():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.reduce_max(3.25, 1) == 3.25
    bench.barrier(1)
    assert bench.aggregate_value(n=2048, steps=10, ws=1, ms_total=5.0) == 2048 * 2048 * 10 / 5e-3
