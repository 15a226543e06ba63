"""Multi-rank path of bench.py on CPU (gloo, world size 2): every rank builds
its own shard of instances (weak scaling, no data-path collective), timings
reduce by max over ranks and work by sum.  The GPU step itself runs per rank
unchanged; only this host logic differs between one and several GPUs."""

import os
import socket

import numpy as np
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parents[1]
    sys.path.insert(0, str(root / "gorilla-physics_gb300"))
    sys.path.insert(0, str(root))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    import bench
    from gpb import Model

    dist.init_process_group("gloo", rank=rank, world_size=world)
    M, q0, v0, _ = Model.from_config(1, 64, seed=bench.shard_seed(2026, rank))
    t_max = bench.all_reduce(1.5 + rank, "max", world, "cpu")
    n_sum = bench.all_reduce(float(M.n), "sum", world, "cpu")
    dist.barrier()
    dist.destroy_process_group()
    out[rank] = (t_max, n_sum, float(q0.sum()), int(M.joint_offset[-1]))


def test_two_rank_shards_and_reductions(built):
    world = 2
    port = _free_port()
    with mp.Manager() as man:
        out = man.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 2.5          # max over ranks
    assert res[0][1] == res[1][1] == 128.0        # instances summed over ranks
    assert res[0][2] != res[1][2] or res[0][3] != res[1][3]  # different shards


def test_single_rank_reductions_are_identity():
    import bench

    assert bench.all_reduce(3.25, "max", 1, "cpu") == 3.25
    assert bench.shard_seed(7, 0) == 7 and bench.shard_seed(7, 3) == 3007
