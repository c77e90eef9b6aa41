"""Autotuner: the chosen configuration is one of the candidates, is used by
later calls on the context, and results stay exact."""
import pytest

pytestmark = pytest.mark.gpu


def test_autotune_then_exact(pcg, golden):
    ctx = pcg.Context(10 ** 17)
    best = pcg.autotune(10 ** 16, ctx=ctx)
    assert best["cta_threads"] in (128, 256, 512)
    assert best["segment_words"] in (4096, 6144, 8192, 16384)
    assert best["ms"] > 0
    g = golden["D_default"]["10000000000000000"]
    assert pcg.D(10 ** 16, g["y"], g["z"], g["k"], ctx=ctx) == g["D"]
    assert pcg.pi(10 ** 16, ctx=ctx) == golden["pi_pow10"][str(10 ** 16)]
    st = ctx.last_stats()
    ctx.close()


def test_autotune_needs_context(pcg):
    with pytest.raises(pcg.PrimecountError):
        pcg.autotune(10 ** 12, ctx=None)
