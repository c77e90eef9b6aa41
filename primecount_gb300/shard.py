"""One x on several GPUs: one process per GPU sweeps a contiguous shard of the
segment plan of D / S2_hard (pcg_D_shard), then the shards' per-level
partials are exchanged once and combined in shard order.

The exchange is the only collective: per level b the shards need the
survivor counts of all earlier shards (an exclusive scan of vectors of
pi(x_star) + 1 integers, 27 k at x = 1e22).  Every rank gathers all shards'
(acc, msum, csum) in one all_gather_into_tensor of int64 words and evaluates

    D = sum_s ( sum_b acc_s[b] + msum_s[b] * sum_{s' < s} csum_s'[b] )

(pcg_shard_combine), so every rank ends with the same exact result.  The
reference splits [0, x/z) into chunks inside one process and obtains the
same offsets from its phi_vector (src/gourdon/D.cpp:382-421).

    import torch.distributed as dist
    dist.init_process_group("nccl")          # or "gloo"
    d = D_distributed(x, y, z, k)            # same value on every rank
"""
import primecount_gb300 as pcg


def _i64(v):
    """v mod 2^64 as a signed 64-bit value."""
    v &= (1 << 64) - 1
    return v - (1 << 64) if v >= 1 << 63 else v


def combine_distributed(part, group=None):
    """All-gather this rank's ShardPart as one int64 tensor of 4 cols values
    (acc low and high words, msum, csum; cols is the same on every rank) and
    combine all shards in rank order.  With NCCL the tensor lives on the
    current CUDA device, with gloo on the host."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    cols = len(part.acc)
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend(group) == "nccl" else torch.device("cpu")
    mine = torch.tensor([_i64(a) for a in part.acc] + [_i64(a >> 64) for a in part.acc] +
                        [_i64(m) for m in part.msum] + [_i64(c) for c in part.csum], dtype=torch.int64, device=dev)
    allp = torch.empty(world * 4 * cols, dtype=torch.int64, device=dev)
    dist.all_gather_into_tensor(allp, mine, group=group)
    v = allp.view(world, 4, cols).cpu().tolist()
    parts = []
    for r in range(world):
        lo, hi, ms, cs = v[r]
        acc = [(h << 64) | (l & ((1 << 64) - 1)) for l, h in zip(lo, hi)]
        parts.append(pcg.ShardPart(acc, ms, cs))
    return pcg.shard_combine(parts)


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
