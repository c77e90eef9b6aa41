"""The oracle's S2_hard against its definition, summed directly (the
brute-force check of the reference's test/deleglise-rivat/S2_hard.cpp:46-92):
with y = floor(x^(1/3)), z = x // y and c = PhiTiny's c(y),

    S2_hard(x, y, z, c) = sum over c < b < pi(y), y // p_b < m <= y, lpf(m) > p_b
                          of -mu(m) * phi(x // (p_b m), b - 1).

CPU only: the sums are plain Python, phi by Legendre's recursion."""
import functools
import random

import pytest


def icbrt(x):
    r = int(round(x ** (1.0 / 3)))
    while r * r * r > x:
        r -= 1
    while (r + 1) ** 3 <= x:
        r += 1
    return r


def get_c(y):
    # PhiTiny::get_c (PhiTiny.hpp:47-63): pi(y) capped at 8
    pi20 = [0, 0, 1, 2, 2, 3, 3, 4, 4, 4, 4, 5, 5, 6, 6, 6, 6, 7, 7, 8]
    return pi20[y] if 0 <= y < 20 else 8


def small_tables(y):
    """primes (1-indexed, primes[0] = 0), least prime factor and Moebius mu up to y."""
    lpf = [0] * (y + 1)
    for i in range(2, y + 1):
        if lpf[i] == 0:
            for j in range(i, y + 1, i):
                if lpf[j] == 0:
                    lpf[j] = i
    mu = [0] * (y + 1)
    if y >= 1:
        mu[1] = 1
        lpf[1] = y + 1          # 1 has no prime factor: lpf(1) > every p_b
    for n in range(2, y + 1):
        p = lpf[n]
        q = n // p
        mu[n] = 0 if q % p == 0 else -mu[q]
    primes = [0] + [n for n in range(2, y + 1) if lpf[n] == n]
    return primes, lpf, mu


def s2_hard_bruteforce(x):
    y = icbrt(x)
    primes, lpf, mu = small_tables(y)
    pi_y = len(primes) - 1
    c = get_c(y)

    @functools.lru_cache(maxsize=None)
    def phi(n, a):
        if a == 0 or n == 0:
            return n
        return phi(n, a - 1) - phi(n // primes[a], a - 1)

    s2 = 0
    for b in range(c + 1, pi_y):
        p = primes[b]
        for m in range(y // p + 1, y + 1):
            if lpf[m] > p:
                s2 -= mu[m] * phi(x // (p * m), b - 1)
    return s2, y, x // y, c


@pytest.mark.parametrize("xs", [list(range(1, 30000, 37)), [29999, 27000, 26999, 8000, 7999, 1000, 999]])
def test_oracle_S2_hard_small_x(ora, xs):
    for x in xs:
        want, y, z, c = s2_hard_bruteforce(x)
        got, _ = ora.S2_hard(x, y, z, c)
        assert got == want, (x, y, z, c)


def test_oracle_S2_hard_random_x(ora):
    rng = random.Random(20261203)
    for _ in range(60):
        x = rng.randint(1, 10 ** 7)
        want, y, z, c = s2_hard_bruteforce(x)
        got, _ = ora.S2_hard(x, y, z, c)
        assert got == want, (x, y, z, c)
