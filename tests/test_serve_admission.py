"""Serving loop host logic on the CPU: admission by device memory (requests
wait for the memory of finished ones; a request above the budget is refused),
the latency budget with its fitted cost model (load shedding), refusal above
the admitted x, and the plain comparator's rule, with fake compute and memory
calls in place of the GPU (no device work)."""
import threading
import time

import pytest

from primecount_gb300 import serve as sv
import primecount_gb300 as pcg


def fake_seconds(kind, x, a=None):
    return 0.0005 + (0.01 if kind == "pi" else 0.004) * (x / 1e20) ** 0.3


def fake_compute(ctx, kind, x, a):
    time.sleep(fake_seconds(kind, x, a))
    return (kind, x, a)


def fake_bytes(kind, x, a):
    return int(x).bit_length() * 1000


def make(n, rate, seed=7):
    # a stream without the engine: pi_of stands in for pi(sqrt x)
    return sv.make_stream(seed, rate, n / rate, pi_range=(8, 20), pi_of=lambda v: [max(1, int(t ** 0.5)) for t in v])


def test_cost_model_interpolates_and_learns():
    m = sv.CostModel()
    for e in (10, 14, 18):
        m.observe("pi", 10 ** e, 1e-3 * 10 ** ((e - 10) / 2), weight=1.0)
    e = [m.est("pi", 10 ** k) for k in range(10, 21)]
    assert all(a < b for a, b in zip(e, e[1:]))
    assert abs(m.est("pi", 10 ** 14) / 1e-1 - 1) < 0.05
    assert 1e-2 < m.est("pi", 10 ** 12) < 1e-1          # between the measured decades
    assert m.est("pi", 10 ** 20) > m.est("pi", 10 ** 18)  # extrapolated
    for _ in range(50):
        m.observe("pi", 10 ** 14, 0.5)
    assert abs(m.est("pi", 10 ** 14) - 0.5) < 0.01       # completed requests move the figure


def test_server_calibrates_at_start():
    srv = sv.Server(max_x=10 ** 16, workers=1, compute=fake_compute)
    try:
        assert set(srv.cost.t["pi"]) >= {8, 10, 12, 14, 16}
        assert set(srv.cost.t["phi"]) >= {8, 12, 16}
    finally:
        srv.close()


def test_memory_admission_waits_and_refuses():
    # a budget of 3 requests' memory: never more than that on the "GPU" at once
    need = 200_000
    seen = []
    lock = threading.Lock()
    live = [0]

    def compute(ctx, kind, x, a):
        with lock:
            live[0] += 1
            seen.append(live[0])
        time.sleep(0.01)
        with lock:
            live[0] -= 1
        return x

    srv = sv.Server(max_x=10 ** 20, workers=6, mem_budget=3 * need, compute=compute,
                    bytes_of=lambda k, x, a: need if x < 10 ** 19 else 10 * need, calibrate=False)
    try:
        rs = [srv.submit("pi", 10 ** 12 + i) for i in range(30)]
        big = srv.submit("pi", 10 ** 19)
        for r in rs:
            assert r.future.result(timeout=10) == r.x
        with pytest.raises(pcg.PrimecountError) as e:
            big.future.result(timeout=5)
        assert e.value.status == sv.PCG_ENOMEM
        assert max(seen) <= 3
        assert srv.peak_inflight <= 3 * need
        assert srv.waited_for_memory > 0
        assert srv.refused_memory == 1
    finally:
        srv.close()


def test_budget_sheds_and_bounds_backlog():
    stream = make(600, 4000.0)          # several times what two workers finish
    r = sv.run_served(stream, workers=2, max_x=10 ** 20, drain_s=5.0, latency_budget=0.03, compute=fake_compute,
                      bytes_of=fake_bytes)
    assert r["submitted"] == len(stream)
    assert r["shed_by_budget"] > 0
    assert r["admitted"] + r["shed_by_budget"] + r["refused_above_max_x"] + r["refused_above_memory"] == r["submitted"]
    assert r["completed"] + r["cancelled_at_deadline"] <= r["admitted"]
    assert r["completed"] > 0


def test_no_budget_admits_everything():
    stream = make(60, 300.0)
    r = sv.run_served(stream, workers=2, max_x=10 ** 20, drain_s=5.0, latency_budget=None, compute=fake_compute)
    assert r["shed_by_budget"] == 0 and r["admitted"] == len(stream)


def test_refusal_above_max_x():
    srv = sv.Server(max_x=10 ** 10, workers=1, compute=fake_compute, calibrate=False)
    r = srv.submit("pi", 10 ** 12)
    with pytest.raises(pcg.PrimecountError) as e:
        r.future.result(timeout=5)
    assert e.value.status == 2
    ok = srv.submit("pi", 10 ** 9)
    assert ok.future.result(timeout=5) == ("pi", 10 ** 9, None)
    srv.close()


def test_plain_comparator_same_rule():
    stream = make(400, 4000.0)
    m = sv.CostModel()
    for e in (8, 12, 16, 20):
        m.observe("pi", 10 ** e, fake_seconds("pi", 10 ** e), weight=1.0)
        m.observe("phi", 10 ** e, fake_seconds("phi", 10 ** e), weight=1.0)
    r = sv.run_plain(stream, drain_s=3.0, latency_budget=0.01, compute=fake_compute, cost=m)
    assert r["shed_by_budget"] > 0 and r["completed"] > 0
