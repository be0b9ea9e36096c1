"""Replica sharding over world_size 2 with the gloo backend (CPU): every
lattice point is owned by exactly one rank, and each rank's oracle values
gathered at the end equal the single-process values."""
import os

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from alps_gb300.sharding import shard_range


def test_shard_range_partitions():
    for n in [0, 1, 7, 512 * 512]:
        for world in [1, 2, 3, 8]:
            spans = [shard_range(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            for (a, b), (c, d) in zip(spans, spans[1:]):
                assert b == c
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import torch
    from alps_gb300 import workloads
    from oracle import pyoracle as po
    w = workloads.proton_electron(12, 24, 1.0, 0.3, 1e-8)
    system, species = workloads.build(w, po.generate_f0)
    P = po.OraclePlasma(system, species)
    P.set_k(1.0, 0.3)
    oms = np.linspace(0.2, 1.4, 10) - 0.05j
    lo, hi = shard_range(len(oms), rank, world)
    mine = P.disp_batch(oms[lo:hi])
    t = torch.zeros(len(oms), 2, dtype=torch.float64)
    t[lo:hi, 0] = torch.from_numpy(mine.real.copy())
    t[lo:hi, 1] = torch.from_numpy(mine.imag.copy())
    dist.all_reduce(t)  # each slot is written by exactly one rank
    if rank == 0:
        ref = P.disp_batch(oms)
        out.put(bool(np.array_equal(t[:, 0].numpy() + 1j * t[:, 1].numpy(), ref)))
    dist.destroy_process_group()


def test_gloo_two_rank_replicas():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert q.get(timeout=5) is True
