"""The N > 1 path of bench.py on CPU with gloo, world size 2: each rank burns its own shard
(distinct seeds, no collective on the data path) and the job's step time is the maximum
over ranks."""
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
