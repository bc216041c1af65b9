"""The multi-rank bench path on the CPU: two gloo ranks take disjoint shards
of the seeded workload and agree on the max-over-ranks time, with no other
exchange (the DCS path has none)."""
import os
import socket

import numpy as np
import torch.distributed as tdist
import torch.multiprocessing as mp

import bench
import oracle
from noa_gb300.elements import MUON_MASS, STANDARD_ROCK
from noa_gb300.workload import kinetic_recoil


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, n, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    K, q = kinetic_recoil(n, offset=bench.shard_offset(rank, n))
    d = oracle.dcs(1, K, q, STANDARD_ROCK, MUON_MASS, threads=1)
    slowest = bench.reduce_max(float(rank + 1) * 0.5, world)
    out[rank] = (K[0], float(d.sum()), slowest)
    tdist.barrier()
    tdist.destroy_process_group()


def test_two_gloo_ranks_shard_and_reduce():
    n, world = 2000, 2
    with mp.get_context("spawn").Manager() as m:  # no fork of a multi-threaded process
        out = m.dict()
        mp.spawn(_rank, args=(world, _free_port(), n, out), nprocs=world, join=True)
        res = dict(out)
    K_all, q_all = kinetic_recoil(world * n)
    for r in range(world):
        k0, s, slowest = res[r]
        assert k0 == K_all[r * n]                       # disjoint consecutive shards
        ref = oracle.dcs(1, K_all[r * n:(r + 1) * n], q_all[r * n:(r + 1) * n], STANDARD_ROCK, MUON_MASS)
        assert s == float(ref.sum())
        assert slowest == 1.0                           # max over ranks of (rank + 1) / 2
