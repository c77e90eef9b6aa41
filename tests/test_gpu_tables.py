"""GPU: the device-built tables, read back entry by entry, against the oracle's
restatement of the reference's table builders (the reference checks its
tables the same way: test/gourdon/FactorTableD.cpp:37-171,
test/lmo/FactorTable.cpp, test/PiTable.cpp)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _primes_upto(n):
    s = np.ones(n + 1, dtype=bool)
    s[:2] = False
    for p in range(2, int(n ** 0.5) + 1):
        if s[p]:
            s[p * p::p] = False
    return np.nonzero(s)[0]


@pytest.mark.parametrize("x,y,z,k", [(10 ** 14, 660067, 660067, 8),     # the reference's default y = z
                                     (10 ** 12, 10000, 30000, 6)])      # y < z: the mpf <= y filter
def test_factor_table_d_entries(pcg, ora, x, y, z, k):
    ctx = pcg.Context(0)
    try:
        pcg.D(x, y, z, k, ctx=ctx)
        n, eb, lim = ctx.table_info("factor_d")
        assert (eb, lim) == (2, z)
        got = ctx.read_table("factor_d")
        want = np.array(ora.factor_table_d16(y, z), dtype=np.uint16)
        assert n == len(want)
        bad = np.nonzero(got != want)[0]
        assert bad.size == 0, (bad[:5], got[bad[:5]], want[bad[:5]])
    finally:
        ctx.close()


def test_factor_table_dr_entries(pcg, ora):
    ctx = pcg.Context(0)
    try:
        x = 10 ** 13
        d = pcg.dr_params(x)
        pcg.S2_hard(x, d["y"], d["z"], d["c"], ctx=ctx)
        n, eb, lim = ctx.table_info("factor_dr")
        assert lim == d["y"] and eb == 2
        got = ctx.read_table("factor_dr")
        want = np.array(ora.factor_table_dr16(d["y"]), dtype=np.uint16)
        assert n == len(want)
        assert np.array_equal(got, want)
    finally:
        ctx.close()


def test_pi_table_and_primes(pcg, ora):
    ctx = pcg.Context(10 ** 15)
    try:
        n, eb, lim = ctx.table_info("pi")
        assert eb == 8 and lim >= pcg.gourdon_params(10 ** 15)["y"]
        got = ctx.read_table("pi")
        want = np.array(ora.pi_table(lim), dtype=np.uint64)
        assert np.array_equal(got, want)
        primes = ctx.read_table("primes")
        ref = _primes_upto(lim)
        assert primes[0] == 0 and len(primes) == len(ref) + 1
        assert np.array_equal(primes[1:].astype(np.int64), ref)
    finally:
        ctx.close()


def test_factor_table_d_32bit_entries(pcg, ora, golden):
    """The reference's D() switches to 32-bit FactorTableD entries above
    z = 149 060 082 888 (src/gourdon/D.cpp:477-499), a size no practical
    input reaches; PCG_FACTOR_D_U32=1 forces that table and the 32-bit sweep
    on small cases.  Entries equal the 16-bit ones but for T_MAX (primes)
    and T_MAX - 1 (the number 1)."""
    os.environ["PCG_FACTOR_D_U32"] = "1"
    try:
        ctx = pcg.Context(0)
        x = 10 ** 14
        p = pcg.gourdon_params(x)
        assert pcg.D(x, p["y"], p["z"], p["k"], ctx=ctx) == 2876480095175
        n, eb, lim = ctx.table_info("factor_d")
        assert eb == 4
        got = ctx.read_table("factor_d")
        w16 = np.array(ora.factor_table_d16(p["y"], p["z"]), dtype=np.uint32)
        want = np.where(w16 == 0xFFFF, np.uint32(0xFFFFFFFF), np.where(w16 == 0xFFFE, np.uint32(0xFFFFFFFE), w16))
        assert np.array_equal(got, want)
        for x, y, z, k, res in golden["D_tuples"][-12:]:
            assert pcg.D(x, y, z, k, ctx=ctx) == res, (x, y, z, k)
        for xs in ("1000000000000000", "100000000000000000"):
            row = golden["D_default"][xs]
            assert pcg.D(int(xs), row["y"], row["z"], row["k"], ctx=ctx) == row["D"], xs
        ctx.close()
    finally:
        del os.environ["PCG_FACTOR_D_U32"]
