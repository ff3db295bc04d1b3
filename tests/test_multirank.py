"""The N>1 bench path on the host: every rank steps its own replica of the
workload (no data-path collective); the job time is the slowest rank's (one
all-reduce MAX over gloo here, NCCL on GPUs) and the whole-job rate counts all
ranks' cells."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, results):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = 100.0 + 25.0 * rank  # rank 1 is the slowest
    out = bench.max_over_ranks(ms, "cpu")
    results[rank] = (out, bench.whole_job_rate(1000, world, 4, out))
    dist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    world = 2
    with mp.Manager() as m:
        results = m.dict()
        mp.spawn(_rank, args=(world, _free_port(), results), nprocs=world, join=True)
        res = dict(results)
    assert res[0][0] == res[1][0] == 125.0
    assert res[0][1] == pytest.approx(1000 * 2 * 4 / 0.125)
