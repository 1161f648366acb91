"""Group-sharded SIRT over several processes: the reduce_df step.

Within one SIRT iteration the emitter groups are independent: each group's
forward solve, residual, adjoint and correlation need only the current field.
The reference exploits this on one GPU by running P of its M groups per pass
(sirt-mimo-norm-mem.cu:429-458).  Here the groups are split over ranks (one
process per GPU): rank r owns the contiguous range group_range(G, r, world),
runs the passes of that range (tomo_gradient_groups_device), and then every
rank needs every group's correlation for the update rule.

reduce_df completes a group-major correlation array [G, ...] of which this
rank filled its own rows by broadcasting each rank's rows from their owner.
No arithmetic happens in the exchange, so every rank ends with the array a
single process would have computed, bit for bit, and the update rule
(tomo_update_device: classic, scaled, normalised, weighted, averaged) gives
the same field on every rank as the unsharded iteration.  The exchange moves
G * nx * ny floats per iteration (32 MB for 32 groups of 512 x 512); summing
partial directions instead would move 2 * nx * ny floats for the normalised
rule but makes the field depend on the number of ranks.  ART updates the
field after every group, so it does not shard: its ranks run replicas.

The functions take torch tensors and a torch.distributed process group, so
the same code runs on GPUs with NCCL and on the CPU with gloo (the tests).
"""
from __future__ import annotations


def group_range(G: int, rank: int, world: int) -> tuple[int, int]:
    """(g0, ng): the contiguous groups rank owns; the first G % world ranks get one more."""
    if not (0 <= rank < world) or G < world:
        raise ValueError(f"cannot split {G} groups over {world} ranks (rank {rank})")
    base, extra = divmod(G, world)
    g0 = rank * base + min(rank, extra)
    return g0, base + (1 if rank < extra else 0)


def reduce_df(corr, group=None):
    """Completes corr ([G, ...], contiguous) in place: each rank's rows group_range(G, r, world)
    are broadcast from rank r to all ranks.  Returns corr."""
    import torch.distributed as dist

    world = dist.get_world_size(group)
    G = corr.shape[0]
    for r in range(world):
        g0, ng = group_range(G, r, world)
        src = dist.get_global_rank(group, r) if group is not None else r
        dist.broadcast(corr[g0:g0 + ng], src=src, group=group)
    return corr


def reduce_resid(r2: float, group=None, device=None) -> float:
    """Sum over ranks of each rank's squared record residual (FP64)."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([r2], dtype=torch.float64, device=device)
    dist.all_reduce(t, group=group)
    return float(t.item())


def sharded_iterate(ctx, method, sched, it, d_f, corr, d_ftrue=None, group=None):
    """One group-sharded SIRT iteration on this rank's context.

    d_f (torch tensor [ny, nx] on the context's GPU) is the field, the same on every rank, and is
    updated in place; corr is a [G, ny, nx] float32 tensor on that GPU used as the exchange
    buffer.  Returns (stats of the update, the squared residual summed over ranks)."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    G = ctx.G
    g0, ng = group_range(G, rank, world)
    r2 = ctx.gradient_groups_device(d_f.data_ptr(), g0, ng)
    ctx.get_correlations_device(g0, ng, corr[g0].data_ptr())
    ctx.synchronize()
    reduce_df(corr, group)
    torch.cuda.synchronize(corr.device)
    ctx.set_correlations_device(0, G, corr.data_ptr())
    st = ctx.update_device(method, sched, it, d_f.data_ptr(), 0 if d_ftrue is None else d_ftrue.data_ptr())
    return st, reduce_resid(r2, group, corr.device)
