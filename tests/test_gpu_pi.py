"""GPU parity: pi(x) and phi(x, a) through the C ABI against the reference's
published values, fixtures made by the reference binary, and the oracle."""
import pytest

pytestmark = pytest.mark.gpu


def test_pi_powers_of_ten(pcg, golden):
    # README.md:163-277 of the reference: pi(10^n)
    for xs, v in golden["pi_pow10"].items():
        x = int(xs)
        if x <= 10 ** 19:
            assert pcg.pi(x) == v, xs


def test_pi_random_fixture(pcg, golden):
    for x, v in golden["pi_random"]:
        assert pcg.pi(x) == v, x


def test_gourdon_terms_match_reference(pcg, golden):
    # each term against the reference's --AC, --B, --D, --Phi0, --Sigma
    rows = golden.get("gourdon_parts", [])
    if not rows:
        pytest.skip("fixture has no gourdon_parts yet")
    for row in rows:
        x = row["x"]
        if x <= 10 ** 10:
            continue
        t = pcg.pi_terms(x)
        for k in ("AC", "B", "D", "Phi0", "Sigma", "pi"):
            assert t[k] == row[k], (x, k, t[k], row[k])


def test_pi_small_x_against_oracle(pcg, ora):
    xs = list(range(-5, 2000, 3)) + [30719, 65536, 10 ** 6 + 3]
    got = pcg.pi_batch(xs)
    for x, v in zip(xs, got):
        assert v == (ora.pi_sieve(x) if x >= 2 else 0), x


def test_pi_c_api(pcg):
    L = pcg.load()
    assert L.primecount_pi(10 ** 12) == 37607912018
    r = L.primecount_pi_128(pcg.to_i128(10 ** 11))
    assert pcg.from_i128(r) == 4118054813
    assert L.primecount_version() == b"8.7"


def test_phi_api_golden(pcg, golden):
    for x, a, v in golden["phi_api"]:
        assert pcg.phi(x, a) == v


def test_phi_random_fixture(pcg, golden):
    for x, a, v in golden["phi_random"]:
        assert pcg.phi(x, a) == v, (x, a)


def test_phi_edge_cases(pcg, ora):
    for x, a in [(0, 5), (-3, 2), (100, 0), (100, -1), (100, 60), (1000, 1), (1000, 8), (10 ** 6, 3),
                 (10 ** 6, 168), (10 ** 6, 169), (10 ** 6, 78498), (10 ** 6, 78499), (10 ** 7, 30), (10 ** 7, 447)]:
        want = ora.phi(x, a) if x >= 1 else 0
        assert pcg.phi(x, a) == want, (x, a)


def test_phi_all_regimes_against_oracle(pcg, ora):
    # a <= 8, small a (special leaves), p_a >= x^(1/4) (P2 + P3), a > pi(sqrt x)
    import random
    rng = random.Random(11)
    for _ in range(30):
        x = int(10 ** rng.uniform(6, 9))
        a = rng.choice([rng.randint(1, 8), rng.randint(9, 40), rng.randint(40, 1200)])
        assert pcg.phi(x, a) == ora.phi(x, a), (x, a)


def test_phi_special_leaves_beyond_sqrt_y(pcg, ora):
    # the special-leaf regime (8 < a, p_{a+1}^4 <= x) where p_a^2 exceeds the leaf
    # bound y: the levels with p_b^2 > y need m > p_b besides m > y / p_b
    # (43463692470, 78) is query 3976 of the seeded phi batch
    for x, a in [(3 * 10 ** 8, 30), (10 ** 9, 30), (2 * 10 ** 9, 30), (8 * 10 ** 9, 60), (10 ** 10, 60),
                 (43463692470, 78), (30000000000, 78)]:
        assert pcg.phi(x, a) == ora.phi(x, a), (x, a)


@pytest.mark.gpu
def test_pi_other_alpha(pcg, golden):
    """pi(x) does not depend on Gourdon's y and z: other alpha_y / alpha_z (the
    reference's --alpha-y / --alpha-z) give the same counts."""
    for n in (12, 15, 18):
        x = 10 ** n
        want = golden["pi_pow10"][str(x)]
        for ay, az in ((0, 2.0), (0, 3.5), (1.5, 1.0), (4.0, 1.5)):
            assert pcg.pi(x, alpha_y=ay, alpha_z=az) == want, (x, ay, az)


def test_pi_int128_configs(pcg, golden):
    # the 128-bit path end to end: x = 1e20, 1e21, 1e22 > 2^64, against the
    # reference's published pi(10^n) (README.md:253-277)
    for n in (20, 21, 22):
        x = 10 ** n
        assert pcg.pi(x) == golden["pi_pow10"][str(x)], n


def test_pi_terms_in_sequence(pcg, golden):
    # PCG_PI_OVERLAP=0 runs D and the other terms one after the other instead of
    # side by side on two streams: same values (read once per process, hence a child)
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    xs = [10 ** 15, 10 ** 17, 123456789012345678]
    code = ("import sys; sys.path.insert(0, %r); import primecount_gb300 as p; "
            "print(' '.join(str(p.pi(x)) for x in %r))" % (root, xs))
    env = dict(os.environ, PCG_PI_OVERLAP="0")
    out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    assert out.stdout.split() == [str(pcg.pi(x)) for x in xs]
    assert int(out.stdout.split()[0]) == golden["pi_pow10"][str(10 ** 15)]


def test_deleglise_rivat_terms_match_reference(pcg, golden):
    # the reference's --S1, --S2-trivial, --S2-easy, --S2-hard, --P2 and -d at
    # 25 x from 1e11 to 1e19 (fixtures of tests/golden/gen_golden.py)
    for row in golden["dr_parts"]:
        x = row["x"]
        t = pcg.pi_dr_terms(x)
        for k in ("S1", "S2_trivial", "S2_easy", "S2_hard", "P2", "pi"):
            assert t[k] == row[k], (x, k, t[k], row[k])
        assert t["pi"] == t["pi_y"] + t["S1"] + t["S2_trivial"] + t["S2_easy"] + t["S2_hard"] - 1 - t["P2"]
        assert pcg.dr_params(x)["y"] == row["y"]


def test_deleglise_rivat_powers_of_ten(pcg, golden):
    # README.md:163-277 of the reference: pi(10^n) by the second formula
    for xs, v in golden["pi_pow10"].items():
        x = int(xs)
        if x <= 10 ** 20:
            assert pcg.pi_deleglise_rivat(x) == v, x
    assert pcg.pi_deleglise_rivat(1) == 0 and pcg.pi_deleglise_rivat(10 ** 6) == 78498
