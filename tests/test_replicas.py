"""The multi-GPU form of the benchmark is independent replicas (the path does
not shard); its host logic -- the barrier, the max-over-ranks time and the
whole-job rate -- runs here as two gloo ranks on the CPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import torch.distributed as td
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    td.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    bench.barrier(world)
    secs = 1.0 + rank  # the second rank is the slower one
    out.put((rank, bench.max_over_ranks(secs, world), bench.replica_rate(100.0, secs, world)))
    bench.barrier(world)
    td.destroy_process_group()


def test_two_gloo_ranks_report_the_slowest_time():
    import torch.multiprocessing as tmp
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert [g[1] for g in got] == [2.0, 2.0]          # max over ranks
    assert [g[2] for g in got] == [100.0, 100.0]      # 2 ranks x 100 units / 2 s
