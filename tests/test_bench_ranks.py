"""bench.py's multi-rank bookkeeping on CPU: two gloo ranks on 127.0.0.1 take
the slowest rank's time, report the whole job's DOF-steps/s and give the
ensemble workload different instances per rank (the replica workloads the
same ones).  No GPU: the kernels run per rank and never wait on each other."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(dist, 10.0 * (rank + 1), device="cpu")
        out.put((rank, ms, bench.job_value(world, 1000, 50, ms),
                 [bench.rank_seed(rank, "config3", b) for b in range(2)],
                 [bench.rank_seed(rank, "config2", b) for b in range(2)]))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, ms0, v0, s3_0, s2_0), (r1, ms1, v1, s3_1, s2_1) = res
    assert ms0 == ms1 == 20.0
    assert v0 == v1 == 2 * 1000 * 50 / 0.020
    assert set(s3_0).isdisjoint(s3_1)          # ensembles shard: other columns per rank
    assert s2_0 == s2_1                        # single mesh: replicas
