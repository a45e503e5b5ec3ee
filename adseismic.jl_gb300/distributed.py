"""Shot-parallel FWI over several GPUs (one process per GPU).

The reference assigns shots round-robin to GPUs (src/Utils.jl:317-331:
shot k goes to GPU k mod n_gpu) and sums the per-GPU losses and gradients.
Here each rank owns its shard, runs its own plan, and the per-iteration
exchange is one sum all-reduce of the FP64 gradient and loss.
"""
from __future__ import annotations

import torch


def shard_shots(shots, rank: int, world: int):
    """Round-robin shard: the shots with index k % world == rank (Utils.jl:317)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"invalid rank {rank} of {world}")
    return [s for k, s in enumerate(shots) if k % world == rank]


def allreduce_loss_grad(loss: torch.Tensor, grad: torch.Tensor, group=None):
    """Sum loss and gradient over all ranks (in place, returns them)."""
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size(group) == 1:
        return loss, grad
    buf = torch.cat([loss.reshape(1).to(grad.dtype), grad.reshape(-1)])
    dist.all_reduce(buf, op=dist.ReduceOp.SUM, group=group)
    loss.copy_(buf[0].to(loss.dtype).reshape(loss.shape))
    grad.copy_(buf[1:].view_as(grad))
    return loss, grad
