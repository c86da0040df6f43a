"""The N-GPU bookkeeping of bench.py on CPU: two gloo ranks (replicas only,
no data-path collective) reduce their per-step times to the maximum, and the
whole-job value is that maximum divided by the number of replicas."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local = [100.0 + 50.0 * rank, 7.0 - rank]
        m = bench.max_over_ranks(local, world, device="cpu")
        out[rank] = (m, bench.whole_job_value(m[0], world))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_replicas_reduce_to_the_slowest_rank():
    world, port = 2, _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        m, value = res[rank]
        assert m == [150.0, 7.0]
        assert value == pytest.approx(75.0)


def test_one_rank_is_the_identity():
    import bench
    assert bench.max_over_ranks([3.0, 4.0], 1) == [3.0, 4.0]
    assert bench.whole_job_value(832.0, 1) == 832.0
