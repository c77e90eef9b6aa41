"""GPU: batched and served pi / phi queries give exactly the results of the
same queries computed alone, and the reference's fixture values."""
import random

import pytest

pytestmark = pytest.mark.gpu


def test_pi_batch_matches_fixture_and_single(pcg, golden):
    rows = golden["pi_random"][:60]
    xs = [x for x, _ in rows] + [10 ** 10, 10 ** 11, 7, 0, -4, 2 ** 40]
    got = pcg.pi_batch(xs)
    for (x, v), g in zip(rows, got):
        assert g == v, x
    alone = [pcg.pi(x) for x in xs[len(rows):]]
    assert got[len(rows):] == alone


def test_seeded_batch_against_the_reference(pcg):
    """Config 4's seeded batch (tests/golden/batch_4096.json, answers from the
    reference binary): every 8th query of each kind through the batch forms."""
    import json
    import os
    p = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "batch_4096.json")
    d = json.load(open(p))
    idx = [i for i in range(0, d["n"], 8) if d["pi"][i] is not None]
    assert len(idx) >= 256
    got = pcg.pi_batch([int(d["pi_x"][i]) for i in idx])
    assert got == [int(d["pi"][i]) for i in idx]
    idx = [i for i in range(0, d["n"], 8) if d["phi"][i] is not None]
    if idx:
        got = pcg.phi_batch([int(d["phi_x"][i]) for i in idx], [d["phi_a"][i] for i in idx])
        assert got == [int(d["phi"][i]) for i in idx]


def test_phi_batch_matches_fixture(pcg, golden):
    rows = golden["phi_random"]
    got = pcg.phi_batch([r[0] for r in rows], [r[1] for r in rows])
    assert got == [r[2] for r in rows]


def test_served_results_equal_alone(pcg, golden):
    from primecount_gb300.serve import Server
    rng = random.Random(5)
    reqs = [("pi", x, None) for x, _ in golden["pi_random"][:40]]
    reqs += [("phi", x, a) for x, a, _ in golden["phi_random"][:40]]
    rng.shuffle(reqs)
    alone = {}
    for k, x, a in reqs:
        alone[(k, x, a)] = pcg.pi(x) if k == "pi" else pcg.phi(x, a)
    srv = Server(max_x=10 ** 17, workers=4)
    try:
        futs = [(k, x, a, srv.submit(k, x, a)) for k, x, a in reqs]
        for k, x, a, r in futs:
            assert r.future.result(timeout=600) == alone[(k, x, a)], (k, x, a)
    finally:
        srv.close()


def test_server_refuses_above_max_and_cancels(pcg):
    from primecount_gb300.serve import Server
    srv = Server(max_x=10 ** 12, workers=1)
    try:
        r = srv.submit("pi", 10 ** 13)
        with pytest.raises(pcg.PrimecountError) as e:
            r.future.result(timeout=5)
        assert e.value.status == 2
        rs = [srv.submit("pi", 10 ** 12) for _ in range(50)]
        n = srv.cancel_pending()
        done = [q for q in rs if q.future.done()]
        assert n + len([q for q in done if not q.future.exception()]) <= 50
        for q in rs:
            if q.future.done() and q.future.exception():
                assert q.future.exception().status == 7
    finally:
        srv.close()


def test_threads_sharing_the_default_context(pcg, golden):
    # calls on one context run one at a time: threads calling through the
    # default context concurrently get the values of calls made alone
    import threading
    pows = {int(k): v for k, v in golden["pi_pow10"].items() if 10 ** 11 <= int(k) <= 10 ** 15}
    xs = sorted(pows) * 3
    got = {}
    errs = []

    def work(i, x):
        try:
            got[i] = pcg.pi(x) if i % 2 == 0 else pcg.D_default(x)
        except Exception as e:  # reported below
            errs.append(e)

    th = [threading.Thread(target=work, args=(i, x)) for i, x in enumerate(xs)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errs, errs
    for i, x in enumerate(xs):
        want = pows[x] if i % 2 == 0 else pcg.D_default(x)
        assert got[i] == want, (i, x)
