"""CPU: the oracle (test infrastructure) against the reference's golden vectors.

Pins the restatement in oracle/pcg_oracle.c to the reference's own
known-answer tables (test/gourdon/D.cpp, test/deleglise-rivat/
S2_hard_alpha.cpp) and to fixtures produced by the reference binary.
"""
import pytest


def test_D_reference_tuples(golden, ora):
    for x, y, z, k, res in golden["D_tuples"]:
        assert ora.D(x, y, z, k)[0] == res, (x, y, z, k)


def test_D_reference_tuples_chunked(golden, ora):
    # multi-chunk mode (phi offsets from a counting pass) gives the same sums
    for x, y, z, k, res in golden["D_tuples"]:
        assert ora.D(x, y, z, k, threads=4)[0] == res, (x, y, z, k)


def test_S2_hard_reference_tuples(golden, ora):
    for x, y, z, c, res in golden["S2_hard_tuples"]:
        assert ora.S2_hard(x, y, z, c)[0] == res, (x, y, z, c)
        assert ora.S2_hard(x, y, z, c, threads=3)[0] == res, (x, y, z, c)


def test_D_random_fixture(golden, ora):
    for x, y, z, k, res in golden["D_random"]:
        if x <= 10 ** 13:
            assert ora.D(x, y, z, k, threads=4)[0] == res, x


def test_S2_hard_random_fixture(golden, ora):
    for x, y, z, c, res in golden["S2_hard_random"]:
        if x <= 10 ** 13:
            assert ora.S2_hard(x, y, z, c, threads=4)[0] == res, x


def test_D_default_1e14_leaf_count(golden, ora):
    # leaf count of the instrumented reference at 1e14: 8 384 338 (917 691 two-prime)
    v, st = ora.D(10 ** 14, 660067, 660067, 8, threads=8)
    assert v == 2876480095175
    assert st["leaves"] == 8384338
    assert st["two_prime_leaves"] == 917691
    assert st["indices_scanned"] == 15544234


def test_params_match_reference(golden, ora):
    for xs, row in golden["D_default"].items():
        p = ora.gourdon_params(int(xs))
        assert (p["y"], p["z"], p["k"]) == (row["y"], row["z"], row["k"]), xs
    for xs, row in golden["S2_hard_default"].items():
        p = ora.dr_params(int(xs))
        assert (p["y"], p["z"], p["c"]) == (row["y"], row["z"], row["c"]), xs
    for x, y, z, k, _ in golden["D_random"]:
        p = ora.gourdon_params(x)
        assert (p["y"], p["z"], p["k"]) == (y, z, k), x


def _mobius_lpf_mpf(n):
    f, m, primes = n, 1, []
    p = 2
    while p * p <= f:
        if f % p == 0:
            e = 0
            while f % p == 0:
                f //= p
                e += 1
            primes.append((p, e))
        p += 1
    if f > 1:
        primes.append((f, 1))
    if any(e > 1 for _, e in primes):
        return 0, primes[0][0] if primes else 1, primes[-1][0] if primes else 1
    mu = -1 if len(primes) % 2 else 1
    return mu, (primes[0][0] if primes else 1), (primes[-1][0] if primes else 1)


def test_factor_table_d_semantics(ora):
    # FactorTableD entry semantics (src/gourdon/FactorTableD.hpp:20-39),
    # checked against trial division like test/gourdon/FactorTableD.cpp:37-171
    y, z = 500, 3000
    t = ora.factor_table_d16(y, z)
    primes = [p for p in range(2, z + 1) if all(p % q for q in range(2, int(p ** 0.5) + 1))]
    pi = {p: i + 1 for i, p in enumerate(primes)}
    for i, v in enumerate(t):
        n = 2310 * (i // 480) + [r for r in range(2310) if all(r % q for q in (2, 3, 5, 7, 11))][i % 480]
        if n > z:
            break
        mu, lpf, mpf = _mobius_lpf_mpf(n)
        if n == 1:
            assert v == 0xFFFE
        elif mu == 0 or mpf > y:
            assert v == 0, n
        elif lpf == n:
            assert v == 0xFFFF, n
        else:
            assert v == 2 * pi[lpf] + (1 if mu == -1 else 0), n


def test_pi_table(ora):
    t = ora.pi_table(5000)
    import bisect
    primes = [p for p in range(2, 5241) if all(p % q for q in range(2, int(p ** 0.5) + 1))]
    for x in range(0, 5000, 7):
        cnt = t[2 * (x // 240)]
        bits = t[2 * (x // 240) + 1]
        r = x % 240
        mask = 0
        for j in range(64):
            if 30 * (j // 8) + [1, 7, 11, 13, 17, 19, 23, 29][j % 8] <= r:
                mask |= 1 << j
        got = cnt + bin(bits & mask).count("1") if x >= 6 else [0, 0, 1, 2, 2, 3][x]
        assert got == bisect.bisect_right(primes, x), x


def test_phi_oracle(golden, ora):
    for x, a, res in golden["phi_random"]:
        if x <= 10 ** 7:
            assert ora.phi(x, a) == res, (x, a)


def test_deleglise_rivat_fixture_consistent(golden, ora):
    # the reference's Deleglise-Rivat terms add up to its pi(x) with pi(y) from the
    # oracle's sieve, and its y, z, c are the oracle's parameters (x up to 1e16 here)
    rows = [r for r in golden["dr_parts"] if r["x"] <= 10 ** 16]
    assert len(rows) >= 8
    for r in rows:
        p = ora.dr_params(r["x"])
        assert (p["y"], p["z"], p["c"]) == (r["y"], r["z"], r["c"]), r["x"]
        pi_y = ora.pi_sieve(r["y"])
        assert pi_y + r["S1"] + r["S2_trivial"] + r["S2_easy"] + r["S2_hard"] - 1 - r["P2"] == r["pi"], r["x"]
        if r["x"] <= 10 ** 13:
            assert ora.S2_hard(r["x"], r["y"], r["z"], r["c"], threads=4)[0] == r["S2_hard"], r["x"]
