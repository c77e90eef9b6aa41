"""One x over several ranks: shard partials and their exchange + combine.

CPU (no GPU): the oracle computes each shard's partials (ora_D_partial, the
decomposition pcg_D_shard uses); the product's combine (pcg_shard_combine,
and primecount_gb300.shard.combine_distributed over a 2-rank gloo group)
must reproduce the reference's D goldens.  GPU: pcg_D_shard / pcg_S2_hard_shard
partials for 1, 2 and 3 shards combine to the golden values.
"""
import os
import socket

import pytest

import multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def shard_bounds(limit, n):
    """n contiguous ranges of [0, limit) starting at multiples of 240."""
    cuts = [0] + [(limit * i // n) // 240 * 240 for i in range(1, n)] + [limit]
    return [(cuts[i], cuts[i + 1]) for i in range(n)]


def oracle_parts(ora, x, y, z, k, n):
    limit = x // z
    ncols = 1 << 16
    parts = []
    for lo, hi in shard_bounds(limit, n):
        s, ms, cs = ora.D_partial(x, y, z, k, lo, hi, ncols)
        parts.append((s, ms, cs))
    return parts


def to_part(pcg, s, ms, cs):
    # the leaf sum of the shard goes to level 0, as pcg_D_shard reports it
    acc = [s] + [0] * (len(ms) - 1)
    return pcg.ShardPart(acc, ms, cs)


def _trim(ms, cs):
    n = max([i + 1 for i, (a, b) in enumerate(zip(ms, cs)) if a or b] or [1])
    return ms[:n], cs[:n]


@pytest.mark.parametrize("n", [1, 2, 3, 5])
def test_oracle_shards_combine(ora, pcg, golden, n):
    rows = [r for r in golden["D_tuples"] if r[0] <= 10 ** 12][::7][:6]
    assert rows
    for x, y, z, k, want in rows:
        parts = []
        for s, ms, cs in oracle_parts(ora, x, y, z, k, n):
            ms, cs = _trim(ms, cs)
            parts.append((s, ms, cs))
        cols = max(len(m) for _, m, _ in parts)
        objs = [to_part(pcg, s, ms + [0] * (cols - len(ms)), cs + [0] * (cols - len(cs))) for s, ms, cs in parts]
        assert pcg.shard_combine(objs) == want, (x, y, z, k, n)


def test_combine_order_matters(ora, pcg, golden):
    """The offsets come from earlier shards only: reversing the shards breaks
    the result (a planted mistake in the order, on the CPU)."""
    x, y, z, k, want = [r for r in golden["D_tuples"] if 10 ** 10 <= r[0] <= 10 ** 12][0]
    parts = [to_part(pcg, s, *_trim(ms, cs)) for s, ms, cs in oracle_parts(ora, x, y, z, k, 2)]
    cols = max(len(p.msum) for p in parts)
    for p in parts:
        p.acc += [0] * (cols - len(p.acc))
        p.msum += [0] * (cols - len(p.msum))
        p.csum += [0] * (cols - len(p.csum))
    assert pcg.shard_combine(parts) == want
    assert pcg.shard_combine(parts[::-1]) != want


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, x, y, z, k, q):
    import sys
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import torch.distributed as dist
    import oracle as ora
    import primecount_gb300 as pcg
    from primecount_gb300.shard import combine_distributed
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        lo, hi = shard_bounds(x // z, world)[rank]
        s, ms, cs = ora.D_partial(x, y, z, k, lo, hi, 1 << 12)
        part = to_part(pcg, s, ms, cs)
        q.put((rank, combine_distributed(part)))
    finally:
        dist.destroy_process_group()


def test_gloo_two_ranks(ora, pcg, golden):
    """world_size 2 over gloo on the CPU: each rank holds one shard's
    partials, all-gathers them and combines; both ranks get the golden D."""
    x, y, z, k, want = [r for r in golden["D_tuples"] if 10 ** 11 <= r[0] <= 10 ** 13][0]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, x, y, z, k, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = {}
    for _ in range(2):
        r, v = q.get(timeout=180)
        res[r] = v
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == {0: want, 1: want}


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 2, 3])
def test_gpu_D_shards(pcg, golden, n):
    for xs in ("100000000000000", "1000000000000000000"):
        g = golden["D_default"].get(xs)
        if g is None:
            continue
        x = int(xs)
        parts = [pcg.D_shard(x, g["y"], g["z"], g["k"], s, n) for s in range(n)]
        assert pcg.shard_combine(parts) == g["D"], (x, n)
    for x, y, z, k, want in golden["D_tuples"][::10]:
        parts = [pcg.D_shard(x, y, z, k, s, n) for s in range(n)]
        assert pcg.shard_combine(parts) == want, (x, y, z, k, n)


@pytest.mark.gpu
def test_gpu_S2_hard_shards(pcg, golden):
    for x, y, z, c, want in golden["S2_hard_tuples"][::8]:
        for n in (2, 3):
            parts = [pcg.S2_hard_shard(x, y, z, c, s, n) for s in range(n)]
            assert pcg.shard_combine(parts) == want, (x, y, z, c, n)


@pytest.mark.gpu
def test_gpu_more_shards_than_segments(pcg, golden):
    """64 shards of a small x: most shards hold no segment at all."""
    x, y, z, k, want = [r for r in golden["D_tuples"] if 10 ** 9 <= r[0] <= 10 ** 11][0]
    parts = [pcg.D_shard(x, y, z, k, s, 64) for s in range(64)]
    assert pcg.shard_combine(parts) == want
