"""The multi-rank host logic of bench.py on two gloo ranks (CPU): each rank
draws its own workload (weak scaling, per-rank seed), the timings are reduced
to the slowest rank's on every rank, and the job's rate counts every rank's
units.  The data path has no collective; only this reduction and the
barriers around the timed region cross ranks."""
import os
import socket
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        assert bench.dist_env() == (world, rank, rank)
        # per-rank timings: the slowest rank's value must come back everywhere
        mine = [1.0 + rank, 5.0 - 2.0 * rank, 0.25 * (rank + 1)]
        red = bench.max_over_ranks(mine, torch.device("cpu"))
        dist.barrier()
        # per-rank proposals (the seed scheme of the workload generator)
        rng = np.random.default_rng(1 + 1000 * rank)
        draw = rng.standard_normal(4)
        out[rank] = (red.tolist(), draw.tolist())
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_to_the_slowest_and_draw_their_own_data():
    world = 2
    manager = mp.Manager()
    out = manager.dict()
    mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    (red0, d0), (red1, d1) = out[0], out[1]
    assert red0 == red1 == [2.0, 5.0, 0.5]
    assert d0 != d1
    sys.path.insert(0, ROOT)
    import bench

    # 10 steps of 3072 proposals on each of 2 ranks in 0.5 s of the slowest rank
    assert bench.job_rate(10, 3072, world, 0.5) == 10 * 3072 * 2 / 0.5
