"""Serving loop host logic on the CPU: admission by the latency budget (load
shedding), refusal above the admitted x, and the plain comparator's rule, with
a fake compute call in place of the GPU (no device work)."""
import time

import pytest

from primecount_gb300 import serve as sv
import primecount_gb300 as pcg


def fake_compute(ctx, kind, x, a):
    time.sleep(min(0.05, sv.est_seconds(kind, x, a) / 50.0))
    return (kind, x, a)


def make(n, rate, seed=7):
    # a stream without the engine: pi_of stands in for pi(sqrt x)
    return sv.make_stream(seed, rate, n / rate, pi_range=(8, 20), pi_of=lambda v: [max(1, int(t ** 0.5)) for t in v])


def test_est_seconds_monotone():
    xs = [10 ** e for e in range(8, 21)]
    e = [sv.est_seconds("pi", x) for x in xs]
    assert all(a < b for a, b in zip(e, e[1:]))
    assert 2.0 < sv.est_seconds("pi", 10 ** 20) < 6.0
    assert sv.est_seconds("phi", 10 ** 8, 10) < 0.01


def test_budget_sheds_and_bounds_backlog():
    stream = make(300, 600.0)
    r = sv.run_served(stream, workers=4, max_x=10 ** 20, drain_s=5.0, latency_budget=2.0, compute=fake_compute)
    assert r["submitted"] == len(stream)
    assert r["shed_by_budget"] > 0
    assert r["admitted"] + r["shed_by_budget"] + r["refused_above_max_x"] == r["submitted"]
    assert r["completed"] + r["cancelled_at_deadline"] <= r["admitted"]
    assert r["completed"] > 0


def test_no_budget_admits_everything():
    stream = make(60, 300.0)
    r = sv.run_served(stream, workers=2, max_x=10 ** 20, drain_s=5.0, latency_budget=None, compute=fake_compute)
    assert r["shed_by_budget"] == 0 and r["admitted"] == len(stream)


def test_refusal_above_max_x():
    srv = sv.Server(max_x=10 ** 10, workers=1, compute=fake_compute)
    r = srv.submit("pi", 10 ** 12)
    with pytest.raises(pcg.PrimecountError) as e:
        r.future.result(timeout=5)
    assert e.value.status == 2
    ok = srv.submit("pi", 10 ** 9)
    assert ok.future.result(timeout=5) == ("pi", 10 ** 9, None)
    srv.close()


def test_plain_comparator_same_rule():
    stream = make(200, 600.0)
    r = sv.run_plain(stream, drain_s=3.0, latency_budget=2.0, compute=fake_compute)
    assert r["shed_by_budget"] > 0 and r["completed"] > 0
