"""Serving loop for pi(x) and phi(x, a) queries on one GPU.

A Server keeps `workers` device contexts whose primes, PiTable and
FactorTable are sized for the largest admitted x and stay resident.  Requests
wait in one queue; every worker takes the next request as soon as it is free,
so requests that arrive while others are on the GPU are admitted as slots free
up and their launches overlap on the device (continuous batching).  Results
are exactly those of a call made alone: the workers share no mutable state.

Admission.  A request is refused at submission when its x exceeds the
admitted maximum (its tables would not fit the resident state), and, when a
latency budget is set, when the GPU-seconds already admitted but not finished
plus its own estimate exceed the budget (load shedding: under overload the
admitted requests keep a bounded latency instead of all of them waiting
behind an unbounded queue).  The estimate is a cost model of the engine on
one GB300 (`est_seconds`).

The plain comparator runs the same arrivals one request at a time with the
tables built inside every call (a fresh context per request), under the same
admission rule.

    python -m primecount_gb300.serve --rate 2000 --seconds 60 --plain   # config of record
"""
import argparse
import collections
import concurrent.futures as cf
import json
import math
import random
import threading
import time

import primecount_gb300 as pcg

PCG_EAGAIN = 9   # refused: the admitted backlog would exceed the latency budget


def est_seconds(kind, x, a=None):
    """GPU-seconds of one query on one GB300 with resident tables (measured:
    pi(1e16) 0.02 s, pi(1e18) 0.17 s, pi(1e20) 3.0 s; phi(x <= 1e16, a) a few ms)."""
    x = max(int(x), 2)
    if kind == "pi":
        return 0.004 + 3.0 * (x / 1e20) ** 0.6
    return 0.002 + 0.05 * (x / 1e16) ** 0.5


class Request:
    __slots__ = ("kind", "x", "a", "t_arrival", "t_done", "future", "est")

    def __init__(self, kind, x, a=None):
        self.kind, self.x, self.a = kind, x, a
        self.t_arrival = time.perf_counter()
        self.t_done = None
        self.future = cf.Future()
        self.est = est_seconds(kind, x, a)


def _compute_pcg(ctx, kind, x, a):
    return pcg.pi(x, ctx=ctx) if kind == "pi" else pcg.phi(x, a, ctx=ctx)


class Server:
    def __init__(self, max_x=10 ** 20, workers=4, mem_budget=0, latency_budget=None, compute=None):
        self.max_x = int(max_x)
        self.budget = latency_budget
        self.compute = compute or _compute_pcg
        self.ctx = [pcg.Context(self.max_x, mem_budget) if compute is None else None for _ in range(workers)]
        self.q = collections.deque()
        self.cv = threading.Condition()
        self.stop = False
        self.admitted = 0
        self.refused = 0              # above the admitted x
        self.shed = 0                 # refused by the latency budget
        self.backlog = 0.0            # estimated GPU-seconds admitted, not finished
        self.threads = [threading.Thread(target=self._work, args=(c,), daemon=True) for c in self.ctx]
        for t in self.threads:
            t.start()

    def device_bytes(self):
        return sum(c.device_bytes() for c in self.ctx if c is not None)

    def submit(self, kind, x, a=None):
        r = Request(kind, int(x), None if a is None else int(a))
        if r.x > self.max_x:
            self.refused += 1
            r.future.set_exception(pcg.PrimecountError(2, "x above the admitted maximum %d" % self.max_x))
            return r
        with self.cv:
            cost = r.est
            if self.budget is not None and self.backlog + cost > self.budget and self.backlog > 0:
                self.shed += 1
                r.future.set_exception(pcg.PrimecountError(PCG_EAGAIN, "overloaded: %.2f s of admitted work"
                                                           % self.backlog))
                return r
            r.est = cost
            self.backlog += cost
            self.admitted += 1
            self.q.append(r)
            self.cv.notify()
        return r

    def _work(self, ctx):
        while True:
            with self.cv:
                while not self.q and not self.stop:
                    self.cv.wait()
                if self.stop and not self.q:
                    return
                r = self.q.popleft()
            try:
                v = self.compute(ctx, r.kind, r.x, r.a)
                r.t_done = time.perf_counter()
                r.future.set_result(v)
            except Exception as e:  # reported through the future
                r.t_done = time.perf_counter()
                r.future.set_exception(e)
            with self.cv:
                self.backlog = max(0.0, self.backlog - r.est)

    def cancel_pending(self):
        """Drop the queued requests (they fail with PCG_ECANCELLED)."""
        with self.cv:
            n = len(self.q)
            while self.q:
                r = self.q.popleft()
                self.backlog = max(0.0, self.backlog - r.est)
                r.future.set_exception(pcg.PrimecountError(7, "cancelled"))
        return n

    def close(self):
        with self.cv:
            self.stop = True
            self.cv.notify_all()
        for t in self.threads:
            t.join()
        for c in self.ctx:
            if c is not None:
                c.close()


def pi_upper(x):
    """Upper bound of pi(x) for drawing a in [1, pi(sqrt x)] without a query."""
    if x < 17:
        return 6
    return int(1.25506 * x / math.log(x)) + 1


def make_stream(seed, rate, seconds, pi_range=(8, 20), phi_range=(8, 16), pi_frac=0.5, pi_of=None):
    """Poisson arrivals of mixed pi / phi requests from a seeded generator.
    a is uniform in [1, pi(sqrt x)] (pi computed for the small sqrt(x) by the
    engine itself, or by pi_of)."""
    rng = random.Random(seed)
    t = 0.0
    out = []
    while True:
        t += rng.expovariate(rate)
        if t >= seconds:
            break
        if rng.random() < pi_frac:
            out.append((t, "pi", int(10 ** rng.uniform(*pi_range)), None))
        else:
            x = int(10 ** rng.uniform(*phi_range))
            out.append((t, "phi", x, rng.random()))
    # resolve a = U{1, pi(sqrt x)} with exact pi(sqrt x)
    sq = sorted({int(math.isqrt(x)) for _, k, x, _ in out if k == "phi"})
    if sq:
        pis = dict(zip(sq, pi_of(sq) if pi_of else pcg.pi_batch(sq)))
    else:
        pis = {}
    res = []
    for t, k, x, u in out:
        if k == "phi":
            n = max(1, pis[math.isqrt(x)])
            res.append((t, k, x, 1 + int(u * n)))
        else:
            res.append((t, k, x, None))
    return res


def percentile(v, q):
    if not v:
        return None
    v = sorted(v)
    i = min(len(v) - 1, max(0, int(round(q * (len(v) - 1)))))
    return v[i]


def run_served(stream, workers=4, max_x=10 ** 20, drain_s=30.0, latency_budget=None, compute=None):
    srv = Server(max_x=max_x, workers=workers, latency_budget=latency_budget, compute=compute)
    t0 = time.perf_counter()
    reqs = []
    for (t, k, x, a) in stream:
        now = time.perf_counter() - t0
        if t > now:
            time.sleep(t - now)
        reqs.append(srv.submit(k, x, a))
    t_end_arrivals = time.perf_counter()
    deadline = t_end_arrivals + drain_s
    for r in reqs:
        rem = deadline - time.perf_counter()
        if rem <= 0:
            break
        try:
            r.future.result(timeout=rem)
        except Exception:
            pass
    cancelled = srv.cancel_pending()
    t_stop = time.perf_counter()
    srv.close()
    ok = [r for r in reqs if r.future.done() and not r.future.exception()]
    lat = [r.t_done - r.t_arrival for r in ok]
    return {"completed": len(ok), "submitted": len(reqs), "admitted": srv.admitted,
            "shed_by_budget": srv.shed, "refused_above_max_x": srv.refused,
            "cancelled_at_deadline": cancelled, "wall_s": t_stop - t0, "qps": len(ok) / (t_stop - t0),
            "p50_s": percentile(lat, 0.5), "p99_s": percentile(lat, 0.99),
            "results": {id(r): r.future.result() for r in ok}}


def run_plain(stream, drain_s=30.0, latency_budget=None, compute=None):
    """One request at a time, tables built inside every call; the same
    admission rule (budget on the estimated GPU-seconds waiting)."""
    t0 = time.perf_counter()
    lat = []
    n = shed = 0
    pending = collections.deque()
    backlog = 0.0
    i = 0
    limit = (stream[-1][0] if stream else 0) + drain_s
    while i < len(stream) or pending:
        now = time.perf_counter() - t0
        while i < len(stream) and stream[i][0] <= now:
            t, k, x, a = stream[i]
            e = est_seconds(k, x, a)
            if latency_budget is not None and backlog + e > latency_budget and backlog > 0:
                shed += 1
            else:
                pending.append((t, k, x, a, e))
                backlog += e
            i += 1
        if not pending:
            time.sleep(max(0.0, stream[i][0] - now))
            continue
        if now > limit:
            break
        t, k, x, a, e = pending.popleft()
        if compute is None:
            c = pcg.Context(0)
            v = _compute_pcg(c, k, x, a)
            c.close()
        else:
            compute(None, k, x, a)
        backlog = max(0.0, backlog - e)
        lat.append(time.perf_counter() - t0 - t)
        n += 1
    wall = time.perf_counter() - t0
    return {"completed": n, "submitted": len(stream), "shed_by_budget": shed, "wall_s": wall, "qps": n / wall,
            "p50_s": percentile(lat, 0.5), "p99_s": percentile(lat, 0.99)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--rate", type=float, default=2000)
    ap.add_argument("--seconds", type=float, default=60)
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--workers", type=int, default=8)
    ap.add_argument("--max-x", default="1e20")
    ap.add_argument("--pi-max-exp", type=float, default=20)
    ap.add_argument("--drain", type=float, default=30)
    ap.add_argument("--budget", type=float, default=2.0,
                    help="latency budget in estimated GPU-seconds of admitted work (0 = admit everything)")
    ap.add_argument("--plain", action="store_true")
    a = ap.parse_args()
    budget = a.budget if a.budget > 0 else None
    stream = make_stream(a.seed, a.rate, a.seconds, pi_range=(8, a.pi_max_exp))
    out = {"config": {"rate": a.rate, "seconds": a.seconds, "seed": a.seed, "workers": a.workers,
                      "pi_x": "10^U(8,%g)" % a.pi_max_exp, "phi_x": "10^U(8,16)", "requests": len(stream),
                      "latency_budget_s": budget}}
    r = run_served(stream, workers=a.workers, max_x=int(float(a.max_x)), drain_s=a.drain, latency_budget=budget)
    r.pop("results")
    out["served"] = r
    if a.plain:
        out["plain"] = run_plain(stream, drain_s=a.drain, latency_budget=budget)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
