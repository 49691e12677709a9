"""Shot sharding across ranks: one GPU per rank, one all-reduce per gradient.

Shots are independent, so the batched forward shards by contiguous shot ranges
with no communication. The FWI gradient and misfit are sums over shots: each
rank computes its shard's float64 sums and one all-reduce (SUM) completes them.
The reduction is written against ``torch.distributed`` and is exercised on CPU
ranks with the gloo backend.
"""

from __future__ import annotations

import numpy as np
import torch


def shard_range(n_items: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous [begin, end) of ``n_items`` for ``rank``; sizes differ by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must lie in [0, world)")
    base, extra = divmod(int(n_items), int(world))
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def shard_sources(sources, rank: int, world: int):
    """This rank's contiguous slice of the transmitter list."""
    sources = np.asarray(sources)
    b, e = shard_range(len(sources), rank, world)
    return sources[b:e]


def allreduce_misfit_and_gradient(misfit, gradient, group=None):
    """Sum a float64 misfit and gradient over ranks (in place on ``gradient``).

    ``misfit`` is a float or a 1-element tensor; ``gradient`` a float64 tensor on
    the backend's device. Returns (misfit float, gradient tensor).
    """
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(misfit), gradient
    if gradient.dtype != torch.float64:
        raise ValueError("gradient must be float64")
    packed = torch.cat([gradient.reshape(-1),
                        torch.as_tensor([float(misfit)], dtype=torch.float64, device=gradient.device)])
    dist.all_reduce(packed, op=dist.ReduceOp.SUM, group=group)
    gradient.copy_(packed[:-1].reshape(gradient.shape))
    return float(packed[-1].item()), gradient


def sharded_misfit_and_grad(problem, m, group=None):
    """Distributed ``misfit_and_grad``: every rank images its shot shard, one all-reduce sums.

    ``problem`` is a ``TorchLeastSquaresFWI``; all ranks must pass the same m and
    sample the same sources (same ``shot_seed``).
    """
    import torch.distributed as dist
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    m = problem.project(m)
    sources = problem._sample_sources()
    mine = shard_sources(sources, rank, world)
    if len(mine):
        value, g_c2 = problem.gradient_c2(m, mine)
    else:
        value, g_c2 = 0.0, np.zeros(problem.model.shape)
    g = torch.as_tensor(g_c2, dtype=torch.float64, device=problem.model.device)
    value, g = allreduce_misfit_and_gradient(value, g, group)
    regularization, g_reg = problem.regularization(m)
    gradient = -g.cpu().numpy() / (m * m) + g_reg
    gradient[~problem.mask] = 0.0
    return value + regularization, gradient
