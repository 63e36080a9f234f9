"""Several-GPU runs are independent replicas (one process per GPU, no data exchanged): the
ranks meet at a barrier before the timed region and report the whole-job throughput against
the slowest rank's time.  The coordination runs here as two gloo ranks on the CPU, with
different per-rank times."""
import os
import socket

import pytest

from hos_gb300 import replicas


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ws, r, local = replicas.env()
    replicas.barrier(ws)
    t = 1.0 + 0.5 * r                        # rank 1 is the slow one
    tmax = replicas.max_over_ranks(t, ws)
    rate = replicas.aggregate_rate(ws, 1000.0, tmax)
    q.put((r, local, ws, tmax, rate))
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[0] for g in got] == [0, 1] and [g[1] for g in got] == [0, 1]
    for _, _, ws, tmax, rate in got:
        assert ws == 2 and tmax == 1.5 and rate == pytest.approx(2 * 1000.0 / 1.5)


def test_single_rank_needs_no_process_group():
    assert replicas.max_over_ranks(2.5, 1) == 2.5
    replicas.barrier(1)
    assert replicas.aggregate_rate(1, 10.0, 2.0) == 5.0
