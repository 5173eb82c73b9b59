"""Multi-rank path on CPU: source sharding and the kernel sum over ranks (gloo, world size 2)."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from sparc_flows_gb300.distributed import shard, sum_kernels


def test_shard_covers_every_source_once():
    for n in (0, 1, 5, 32, 33):
        for world in (1, 2, 3, 8):
            parts = [shard(list(range(n)), r, world) for r in range(world)]
            assert sum(parts, []) == list(range(n))
            sizes = [len(p) for p in parts]
            assert max(sizes) - min(sizes) <= 1


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sources = list(range(5))
        mine = shard(sources, rank, world)
        # per-source "kernels": a field that identifies the source, summed over this rank's share
        ker = {"kernel_psi": torch.zeros(3, 4, dtype=torch.float64),
               "kernel_c": torch.zeros(3, 4, dtype=torch.float64)}
        for s in mine:
            ker["kernel_psi"] += (s + 1) * torch.ones(3, 4, dtype=torch.float64)
            ker["kernel_c"] += torch.full((3, 4), 10.0 ** s, dtype=torch.float64)
        tot = sum_kernels(ker)
        out[rank] = (mine, tot["kernel_psi"].numpy().copy(), tot["kernel_c"].numpy().copy())
    finally:
        dist.destroy_process_group()


def test_kernel_sum_over_two_gloo_ranks():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, _free_port(), out), nprocs=world, start_method="spawn")
    seen = sorted(sum((out[r][0] for r in range(world)), []))
    assert seen == list(range(5))
    for r in range(world):
        assert np.allclose(out[r][1], 15.0)            # 1 + 2 + 3 + 4 + 5
        assert np.allclose(out[r][2], 11111.0)         # 1 + 10 + 100 + 1000 + 10000


def test_sum_kernels_without_process_group_is_identity():
    k = {"hessian": torch.arange(6, dtype=torch.float64).reshape(2, 3)}
    assert sum_kernels(k) is k
