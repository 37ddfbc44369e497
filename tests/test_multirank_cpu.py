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


def _shard_worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import Port

    from glass_gb300 import shard
    from glass_gb300 import workloads as wl

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        port_ = Port()
        bank, seg, props, tx = _shared_workload(port_)
        sub, idx = shard.shard_bank(bank, rank, world)
        pos, local = shard.shard_proposals(seg, idx)
        rA, rE = sub.interleaved()
        dl, ty, hh = port_.dlogl_batch(wl.T_YEAR, sub.NFFT, sub.qmin, np.ascontiguousarray(rA),
                                       np.ascontiguousarray(rE), np.ascontiguousarray(sub.invCA),
                                       np.ascontiguousarray(sub.invCE), local, props[pos], tx[pos], nthreads=1)
        # the ranks' results meet only for this check (the data path has no collective)
        mine = torch.full((len(seg),), float("nan"), dtype=torch.float64)
        mine[torch.from_numpy(pos)] = torch.from_numpy(np.asarray(dl))
        owner = torch.zeros(len(seg), dtype=torch.int64)
        owner[torch.from_numpy(pos)] = 1
        gathered = [torch.empty_like(mine) for _ in range(world)]
        owners = [torch.empty_like(owner) for _ in range(world)]
        dist.all_gather(gathered, mine)
        dist.all_gather(owners, owner)
        out[rank] = (idx.tolist(), [g.tolist() for g in gathered], [o.tolist() for o in owners])
    finally:
        dist.destroy_process_group()


def _shared_workload(port_):
    from glass_gb300 import workloads as wl

    rng = np.random.default_rng(17)
    T = wl.T_YEAR

    def wf(p):
        al = port_.alignment(T, 256, 0, p)
        h = port_.waveform(p, int(al[0]), T)
        return int(al[0]), h[3], h[4]

    bank, inj, _, _, _ = wl.tempered_bank(rng, wf, nseg=6, NFFT=256, nchain=6, ntemp=1, f_range=(2e-3, 4e-3))
    seg = rng.integers(0, 6, 40).astype(np.int32)
    props = np.array([wl.gaussian_jumps(rng, inj[s], wl.jump_scales(inj[s], 20.0), 1)[0] for s in seg])
    tx = rng.normal(0, 1, len(seg))
    return bank, seg, props, tx


def test_two_gloo_ranks_evaluate_disjoint_halves_of_a_segment_bank(port):
    """Two ranks take disjoint contiguous halves of one segment bank and the
    proposals on them; every proposal is evaluated by exactly one rank, and
    the union equals the single-process evaluation of the whole bank."""
    world = 2
    manager = mp.Manager()
    out = manager.dict()
    mp.spawn(_shard_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    idx0, g0, o0 = out[0]
    idx1, _, _ = out[1]
    assert set(idx0).isdisjoint(idx1) and sorted(idx0 + idx1) == list(range(6))
    owners = np.array(o0)
    assert (owners.sum(axis=0) == 1).all()  # every proposal on exactly one rank
    got = np.where(owners[0] == 1, np.array(g0[0]), np.array(g0[1]))
    from glass_gb300 import workloads as wl

    bank, seg, props, tx = _shared_workload(port)
    rA, rE = bank.interleaved()
    ref = port.dlogl_batch(wl.T_YEAR, bank.NFFT, bank.qmin, np.ascontiguousarray(rA), np.ascontiguousarray(rE),
                           np.ascontiguousarray(bank.invCA), np.ascontiguousarray(bank.invCE), seg, props, tx,
                           nthreads=1)[0]
    np.testing.assert_array_equal(got, np.asarray(ref))
