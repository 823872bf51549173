"""Multi-process (replica) logic of bench.py on CPU with the gloo backend,
world size 2: slowest-rank timing, whole-job rate, disjoint path ranges."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = bench.max_over_ranks(1.5 if rank == 0 else 2.5)
        q.put((rank, t, bench.rank_path0(rank, 1000)))
    finally:
        dist.destroy_process_group()


def test_replica_timing_and_ranges_world2():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert [r[1] for r in res] == [2.5, 2.5]            # both see the slowest rank
    assert [r[2] for r in res] == [0, 1000]             # disjoint path ranges


def test_whole_job_rate_and_single_process_identity():
    import bench
    assert bench.whole_job_rate(1000, 10, 2, 2.0) == pytest.approx(10000.0)
    assert bench.max_over_ranks(3.25) == 3.25          # not distributed: identity
