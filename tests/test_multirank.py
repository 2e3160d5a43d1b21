"""The N > 1 path on CPU with gloo, world size 2.

* bench.py's weak-scaling helpers: each rank burns its own seeded shard (distinct seeds, no
  collective on the data path) and the job's step time is the maximum over ranks.
* Strong scaling of one particle set: each rank burns a contiguous range, first of equal
  counts, then the range that sharding.partition gives it (cost-balanced on the first burn's
  Newton iterations, which the ranks exchange on the host), here with the oracle standing in
  for the GPU burn; the concatenated results equal a single-rank burn of the whole set bit for
  bit, because particles are independent."""
import os
import socket

import numpy as np
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    import workloads
    w = workloads.make("c2", P=64, seed=bench.shard_seed(rank))
    out[rank] = (bench.max_over_ranks(1.0 + 2.0 * rank, world), float(w["T"].sum()))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_shard_and_max():
    world, port = 2, _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 3.0  # max over ranks, seen by both
    assert not np.isclose(res[0][1], res[1][1])  # different shards


P_STRONG = 96


def _clustered():
    import workloads
    w = workloads.make("c2", P=P_STRONG, seed=21)
    order = np.argsort(w["T"])  # hot particles together, as in SPH data
    return dict(w, Y=w["Y"][:, order], T=w["T"][order], rho=w["rho"][order], dt=w["dt"][order])


def _strong_rank(rank, world, port, out):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    import sharding
    o = bench._oracle()[0]
    w = _clustered()
    eq = [(k * P_STRONG // world, (k + 1) * P_STRONG // world) for k in range(world)]
    a, b = eq[rank]
    _, _, first = bench.cpu_burn(o, w, slice(a, b), threads=1)
    its = [torch.zeros(e - s, dtype=torch.int32) for s, e in eq]
    dist.all_gather(its, torch.from_numpy(first[5].astype(np.int32)))
    ranges = sharding.partition(sharding.cost_estimate(prev_iterations=torch.cat(its).numpy()), world)
    # the next burn runs on the cost-balanced ranges (here again from the initial state)
    a, b = ranges[rank]
    _, _, second = bench.cpu_burn(o, w, slice(a, b), threads=1)
    out[rank] = (ranges, eq, first, second)
    dist.barrier()
    dist.destroy_process_group()


def test_strong_scaling_partition_equals_single_rank():
    import bench
    import sharding
    world, port = 2, _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_strong_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    ranges = res[0][0]
    assert ranges == res[1][0]  # every rank computed the same partition
    assert ranges[0][0] == 0 and ranges[-1][1] == P_STRONG and ranges[0][1] == ranges[1][0]
    o = bench._oracle()[0]
    _, _, whole = bench.cpu_burn(o, _clustered(), slice(0, P_STRONG), threads=2)
    for piece in (2, 3):  # equal-count ranges, then the cost-balanced ones
        for i in range(6):
            joined = np.concatenate([res[r][piece][i] for r in range(world)], axis=-1)
            assert np.array_equal(joined, whole[i]), (piece, i)
    cost = sharding.cost_estimate(prev_iterations=whole[5])
    assert sharding.imbalance(cost, ranges) <= sharding.imbalance(cost, res[0][1]) + 1e-12
