"""Multi-rank host logic of the shot loop (one process per GPU).

The reference distributes the shots over MPI ranks (init_MPIshot.c:19-30),
runs each rank's shots, and sums the ranks' gradients and misfits afterwards
(sum_grad_MPI.c:34-36, grad_obj.c:60).  One GB300 holds a whole batch, so
bench.py runs independent replicas; these helpers are the same steps for a
caller that shards one batch over several GPUs with torch.distributed (NCCL
on GPUs, gloo on CPUs).  The sums are taken in FP64, where the reference
reduces the gradient in float.
"""
from __future__ import annotations

import numpy as np


def shot_range(nshots: int, nranks: int, rank: int) -> tuple[int, int]:
    """0-based [first, last) of `rank`'s shots: contiguous blocks, the first
    nshots % nranks ranks one shot longer (init_MPIshot.c:19-30)."""
    if nranks < 1 or not 0 <= rank < nranks or nshots < 0:
        raise ValueError("bad shot partition arguments")
    q, r = divmod(nshots, nranks)
    first = q * rank + min(rank, r)
    return first, first + q + (1 if rank < r else 0)


def allreduce_gradient(grad, l2: float, dist, device: str = "cpu"):
    """Sum over the ranks of their partial gradients and misfits (FP64);
    returns (gradient as float64 array, misfit)."""
    import torch

    g = torch.as_tensor(np.ascontiguousarray(grad, dtype=np.float64)).to(device)
    m = torch.tensor([float(l2)], dtype=torch.float64, device=device)
    dist.all_reduce(g)
    dist.all_reduce(m)
    return g.cpu().numpy(), float(m.item())


def max_over_ranks(value: float, dist, device: str = "cpu") -> float:
    """The largest `value` over the ranks (a step time measured per rank)."""
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
