"""One x on several GPUs: one process per GPU sweeps a contiguous shard of the
segment plan of D / S2_hard (pcg_D_shard), then the shards' per-level
partials are exchanged once and combined in shard order.

The exchange is the only collective: per level b the shards need the
survivor counts of all earlier shards (an exclusive scan of vectors of
pi(x_star) + 1 integers, 27 k at x = 1e22).  Every rank gathers all shards'
(acc, msum, csum) and evaluates

    D = sum_s ( sum_b acc_s[b] + msum_s[b] * sum_{s' < s} csum_s'[b] )

(pcg_shard_combine), so every rank ends with the same exact result.  The
reference splits [0, x/z) into chunks inside one process and obtains the
same offsets from its phi_vector (src/gourdon/D.cpp:382-421).

    import torch.distributed as dist
    dist.init_process_group("nccl")          # or "gloo"
    d = D_distributed(x, y, z, k)            # same value on every rank
"""
import primecount_gb300 as pcg


def combine_distributed(part, group=None):
    """All-gather this rank's ShardPart and combine all shards in rank order."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    gathered = [None] * world
    dist.all_gather_object(gathered, (part.acc, part.msum, part.csum), group=group)
    return pcg.shard_combine([pcg.ShardPart(a, m, c) for a, m, c in gathered])


def D_distributed(x, y, z, k, group=None, ctx=None, stream=None):
    """D(x, y, z, k) with this rank sweeping shard `rank` of `world`."""
    import torch.distributed as dist
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    part = pcg.D_shard(x, y, z, k, rank, world, ctx=ctx, stream=stream)
    return combine_distributed(part, group)


def S2_hard_distributed(x, y, z, c, group=None, ctx=None, stream=None):
    """S2_hard(x, y, z, c) with this rank sweeping shard `rank` of `world`."""
    import torch.distributed as dist
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    part = pcg.S2_hard_shard(x, y, z, c, rank, world, ctx=ctx, stream=stream)
    return combine_distributed(part, group)
