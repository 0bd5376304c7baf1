"""Shot sharding across ranks and the one exchange of the path: the sum of
the per-rank gradients (seistorch_dist.py:123 gets it from DDP hooks,
fwi.py:365 from an MPI allreduce).  Shots are independent, so each rank runs
its own shots through the native loop and only the float32 model gradient
travels."""
import torch
import torch.distributed as dist


def shard_shots(shots, rank, world):
    """Contiguous share of ``shots`` for ``rank`` (sizes differ by at most one)."""
    shots = list(shots)
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    n = len(shots)
    lo = rank * n // world
    hi = (rank + 1) * n // world
    return shots[lo:hi]


def allreduce_gradient(grad, group=None):
    """Sum a model gradient over the ranks in place; returns it."""
    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(grad, op=dist.ReduceOp.SUM, group=group)
    return grad


def reduce_loss(loss, group=None):
    """Sum a scalar misfit over the ranks (a 0-d tensor); returns it."""
    t = torch.as_tensor(loss, dtype=torch.float64).reshape(1).clone()
    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t[0]
