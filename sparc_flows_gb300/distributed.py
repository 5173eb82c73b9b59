"""Multi-GPU layout of the batched solves: independent sources sharded across ranks.

Sources (and line-search variants) are independent solves, one ``sparc`` process each in the
reference (full.py:85-93, linesearch.py:39-56); the only cross-source operation is the kernel
sum over sources before the gradient post-processing (grad.py:188-196).  Each rank here runs
its own batch on its own GPU with no collective on the data path, and the kernel sum is one
all-reduce of the (nz, nx) FP64 kernels at the end (NCCL between GPUs, gloo on hosts).
"""
from __future__ import annotations

import torch
import torch.distributed as dist


def shard(items: list, rank: int, world: int) -> list:
    """Contiguous share of ``items`` for ``rank`` of ``world``; sizes differ by at most one and
    every item lands on exactly one rank."""
    n = len(items)
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    hi = lo + base + (1 if rank < extra else 0)
    return items[lo:hi]


def sum_kernels(kernels: dict, group=None) -> dict:
    """Sum each kernel over all ranks (grad.py:188-196: the kernel of every source added up).
    ``kernels`` maps names to tensors already summed over this rank's sources; the result holds
    the same names summed over all sources of all ranks.  A no-op without a process group."""
    if not (dist.is_available() and dist.is_initialized()):
        return kernels
    out = {}
    for name in sorted(kernels):
        t = kernels[name].detach().clone().contiguous()
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        out[name] = t
    return out
