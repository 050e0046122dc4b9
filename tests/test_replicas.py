"""Replica runs on the CPU: two gloo ranks each render their own seeded frame with the oracle
and aggregate units / time the way bench.py does under torchrun (sum of the ranks' fragments
over the slowest rank's time), with no collective on the data path."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from lucid_gb300 import replicas, scenes
    from oracle import binding as oracle
    sc = scenes.small_scene(96, 64, 500, seed=replicas.rank_seed(1, rank))
    frags = oracle.run(sc)["num_fragments"]
    local_ms = 10.0 * (rank + 1)
    rate, max_ms, units = replicas.aggregate(local_ms, frags, dist)
    out[rank] = (frags, rate, max_ms, units)
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_aggregate():
    from lucid_gb300 import replicas, scenes
    from oracle import binding as oracle
    oracle.lib()  # build the oracle before the ranks start
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.start_processes(_rank_main, args=(world, _free_port(), out), nprocs=world, start_method="spawn")
        res = dict(out)
    frags = [res[r][0] for r in range(world)]
    assert frags[0] != frags[1], "ranks must render different seeded frames"
    for r in range(world):
        _, rate, max_ms, units = res[r]
        assert max_ms == 20.0 and units == sum(frags)
        assert rate == pytest.approx(sum(frags) / 0.020)
    # one process: the local numbers
    single = scenes.small_scene(96, 64, 500, seed=replicas.rank_seed(1, 0))
    f0 = oracle.run(single)["num_fragments"]
    assert f0 == frags[0]
    assert replicas.aggregate(5.0, f0) == (f0 / 0.005, 5.0, float(f0))
