"""The multi-GPU layout is replicas only: every rank runs its own replicas
with its own seeds and the job's time is the slowest rank's.  This checks
that host logic with two gloo ranks on the CPU: disjoint seeds across
ranks, the max-over-ranks reduction bench.py uses, and that a replica's
trajectory (oracle) depends on its seed alone, not on the rank layout."""
import os
import socket

import numpy as np
import torch.distributed as dist
import torch.multiprocessing as mp

import bench
from oracle import oracle as O


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    wl = bench.make_workload(8, rank=rank)
    seeds = wl["seeds"].tolist()
    all_seeds = [None] * world
    dist.all_gather_object(all_seeds, seeds)
    slowest = bench.max_over_ranks(float(rank + 1) * 0.5, world)
    # replica 3 of this rank, a few hundred trials on an 8^3 bcc lattice
    mod = O.OracleModel("bcc", 4, 4, 4, wl["V"])
    r = O.OracleRng(int(seeds[3]))
    cfg, _ = mod.initial_setup(r, wl["conc"])
    acc, _ = mod.mc_run(cfg, r, 1.0 / (float(wl["T"][3]) * bench.K_B_IN_RY), 500)
    q.put((rank, all_seeds, slowest, acc, mod.total_energy(cfg)))
    dist.destroy_process_group()


def test_two_ranks_shard_replicas_without_collectives_on_the_data_path():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    seeds0, seeds1 = out[0][1][0], out[0][1][1]
    assert not set(seeds0) & set(seeds1)
    assert all(o[2] == 1.0 for o in out)          # both ranks see the slowest rank's time
    # the same replica run in one process gives the same trajectory
    for rank, _, _, acc, e in out:
        wl = bench.make_workload(8, rank=rank)
        mod = O.OracleModel("bcc", 4, 4, 4, wl["V"])
        r = O.OracleRng(int(wl["seeds"][3]))
        cfg, _ = mod.initial_setup(r, wl["conc"])
        a, _ = mod.mc_run(cfg, r, 1.0 / (float(wl["T"][3]) * bench.K_B_IN_RY), 500)
        assert a == acc and mod.total_energy(cfg) == e
