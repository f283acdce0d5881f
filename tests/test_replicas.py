"""The multi-GPU path is replicas only: each rank evaluates its own instance range, the
slowest rank's time is the job's. These run two gloo ranks on the CPU (no GPU): the shards
cover the instances exactly, results gathered from the ranks equal a single evaluation of all
instances (the oracle stands in for each rank's device sweep), and the time reduction takes
the maximum."""
import os
import socket

import numpy as np
import pytest

from casadi_gb300 import replicas as RP

torch = pytest.importorskip("torch")


def test_instance_ranges_cover_exactly():
    for n in (0, 1, 7, 1000, 1 << 20):
        for world in (1, 2, 3, 8):
            rs = [RP.instance_range(n, r, world) for r in range(world)]
            assert rs[0][0] == 0 and rs[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(rs, rs[1:]))
            sizes = [b - a for a, b in rs]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        RP.instance_range(10, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, n, out):
    import torch.distributed as dist
    import oracle as O
    from casadi_gb300 import workloads as W
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        f = W.cartpole_step()
        args = W.cartpole_inputs(n, steps=1, seed=4)
        mine = RP.shard(args, rank, world)
        res = O.eval(f.tape, mine, mine[0].shape[-1])[0]
        parts = [None] * world
        dist.all_gather_object(parts, res)
        slowest = RP.max_over_ranks(10.0 + rank)
        if rank == 0:
            np.save(out, np.concatenate(parts, axis=-1))
            with open(out + ".max", "w") as fh:
                fh.write(repr(slowest))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_match_one_evaluation(tmp_path):
    import torch.multiprocessing as mp
    import oracle as O
    from casadi_gb300 import workloads as W
    n, world = 1001, 2
    out = str(tmp_path / "res.npy")
    mp.start_processes(_rank_main, args=(world, _free_port(), n, out), nprocs=world,
                       start_method="spawn", join=True)
    got = np.load(out)
    f = W.cartpole_step()
    want = O.eval(f.tape, W.cartpole_inputs(n, steps=1, seed=4), n)[0]
    assert np.array_equal(got, want)
    assert float(open(out + ".max").read()) == 11.0
