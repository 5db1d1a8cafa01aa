"""The multi-GPU form of the benchmark is independent replicas: every rank
runs the whole workload, the job's time is the slowest rank's, and the value
is all ranks' units over that time.  Exercised here with two gloo ranks on
the CPU (the reduction and the formula; no GPU)."""
import os
import socket

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(ws), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    got_ws, got_rank, got_local = bench.dist_env()
    seconds = 1.0 + rank                      # rank 1 is the slow one
    slowest = bench.max_over_ranks(seconds, got_ws)
    value = bench.replica_value(4, got_ws, slowest)
    dist.barrier()
    dist.destroy_process_group()
    out.put((got_rank, got_local, got_ws, slowest, value))


def test_two_gloo_replicas_report_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1] and [r[1] for r in res] == [0, 1]
    for _, _, ws, slowest, value in res:
        assert ws == 2 and slowest == 2.0
        assert value == pytest.approx(4 * 2 / 2.0)


def test_single_process_needs_no_group():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.replica_value(4, 1, 0.5) == 8.0
