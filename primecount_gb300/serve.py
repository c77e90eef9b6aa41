"""Serving loop for pi(x) and phi(x, a) queries on one GPU.

A Server keeps `workers` device contexts whose primes, PiTable and
FactorTable are sized for the largest admitted x and stay resident.  Requests
wait in one queue; every worker takes the next request as soon as it is free
and the request's device memory fits, so requests that arrive while others
are on the GPU are admitted as slots and memory free up, and their launches
overlap on the device (continuous batching).  Results are exactly those of a
call made alone: the workers share no mutable state.

Admission.
* Table memory: a request whose x exceeds the admitted maximum is refused at
  submission (PCG_ERANGE): its tables would not fit the resident state.
* Working memory: every request needs device memory beyond the resident
  tables -- the sweep's count and sign rows, the prime sieve's buffers, the
  formulas' temporaries -- which the engine states before the call
  (pcg_query_device_bytes).  The requests on the GPU together stay within the
  server's memory budget: a request larger than the budget is refused
  (PCG_ENOMEM); otherwise the head of the queue waits until the memory of
  finished requests is free.  A worker whose context keeps more working
  memory than its share of the budget after a request releases it
  (pcg_ctx_trim), so the memory held between requests stays within the
  budget too.
* Latency (optional): with a latency budget, a request is shed at submission
  when the GPU-seconds already admitted but not finished, plus its own, exceed
  it (load shedding: under overload the admitted requests keep a bounded
  latency instead of all of them waiting behind an unbounded queue).  The
  GPU-seconds come from a cost model fitted at start-up: the server times
  pi(10^e) and phi(10^e, a) on its own contexts, interpolates between the
  decades and refines each decade with the times of completed requests.

The plain comparator runs the same arrivals one request at a time with the
tables built inside every call (a fresh context per request), under the same
latency rule.

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
PCG_ENOMEM = 3


class CostModel:
    """GPU-seconds of one query by kind and decade of x (the decade of 10^d
    holds the x nearest to 10^d on a log scale): measured decades (start-up
    calibration, then an exponential average of completed requests) with
    log-linear interpolation between them and extrapolation beyond."""

    def __init__(self):
        self.t = {"pi": {}, "phi": {}}
        self.lock = threading.Lock()

    def observe(self, kind, x, seconds, weight=0.2):
        d = int(round(math.log10(max(int(x), 2))))   # the decade centred on 10^d
        with self.lock:
            old = self.t[kind].get(d)
            self.t[kind][d] = seconds if old is None else (1 - weight) * old + weight * seconds

    def est(self, kind, x, a=None):
        lx = math.log10(max(int(x), 2))
        with self.lock:
            pts = sorted(self.t[kind].items())
        if not pts:
            return 1e-3
        if len(pts) == 1:
            return max(pts[0][1], 1e-4)
        lo = [p for p in pts if p[0] <= lx]
        hi = [p for p in pts if p[0] > lx]
        if lo and hi:
            (d0, t0), (d1, t1) = lo[-1], hi[0]
        elif hi:
            (d0, t0), (d1, t1) = hi[0], hi[1]
        else:
            (d0, t0), (d1, t1) = lo[-2], lo[-1]
        l0, l1 = math.log(max(t0, 1e-5)), math.log(max(t1, 1e-5))
        f = (lx - d0) / (d1 - d0)
        return max(math.exp(l0 + f * (l1 - l0)), 1e-5)


class Request:
    __slots__ = ("kind", "x", "a", "t_arrival", "t_done", "future", "est", "need", "waited")

    def __init__(self, kind, x, a=None):
        self.kind, self.x, self.a = kind, x, a
        self.t_arrival = time.perf_counter()
        self.t_done = None
        self.future = cf.Future()
        self.est = 0.0
        self.need = 0
        self.waited = False


def _compute_pcg(ctx, kind, x, a):
    return pcg.pi(x, ctx=ctx) if kind == "pi" else pcg.phi(x, a, ctx=ctx)


class Server:
    """Serving loop over `workers` contexts (see the module docstring).

    mem_budget: device bytes for the working memory of the requests on the
    GPU (0: 45% of the device's free memory once the resident tables are
    built).  latency_budget: GPU-seconds of admitted, unfinished work above
    which requests are shed (None: none are).  compute / bytes_of stand in for
    the engine in host-only tests."""

    def __init__(self, max_x=10 ** 20, workers=4, mem_budget=0, latency_budget=None, compute=None,
                 bytes_of=None, calibrate=True):
        self.max_x = int(max_x)
        self.budget = latency_budget
        self.compute = compute or _compute_pcg
        real = compute is None
        self.ctx = [pcg.Context(self.max_x, 0) if real else None for _ in range(workers)]
        if bytes_of is None:
            bytes_of = (lambda k, x, a: pcg.query_device_bytes(k, x, a or 0, ctx=self.ctx[0])) if real \
                else (lambda k, x, a: 0)
        self.bytes_of = bytes_of
        if mem_budget:
            self.mem_budget = int(mem_budget)
        elif real:
            self.mem_budget = int(0.45 * pcg.device_memory()[0])
        else:
            self.mem_budget = 1 << 60
        self.share = self.mem_budget // max(1, workers)
        self.cost = CostModel()
        if calibrate:
            self._calibrate()
        self.q = collections.deque()
        self.cv = threading.Condition()
        self.stop = False
        self.admitted = 0
        self.refused = 0              # above the admitted x
        self.refused_memory = 0       # larger than the memory budget
        self.shed = 0                 # refused by the latency budget
        self.waited_for_memory = 0    # requests that waited at the head for memory
        self.backlog = 0.0            # estimated GPU-seconds admitted, not finished
        self.inflight = 0             # device bytes of the requests on the GPU
        self.peak_inflight = 0
        self.trims = 0
        self.threads = [threading.Thread(target=self._work, args=(c,), daemon=True) for c in self.ctx]
        for t in self.threads:
            t.start()

    def _calibrate(self):
        """Time pi(10^e) and phi(10^e, a) on the workers' first context."""
        ctx = self.ctx[0]
        top = int(math.floor(math.log10(max(self.max_x, 10))))
        for e in sorted(set(list(range(8, top + 1, 2)) + [top])):
            x = 10 ** e
            t0 = time.perf_counter()
            self.compute(ctx, "pi", x, None)
            self.cost.observe("pi", x, time.perf_counter() - t0, weight=1.0)
        for e in (8, 10, 12, 14, 16):
            x = 10 ** e
            a = max(9, int(math.isqrt(x) / (2 * math.log(math.isqrt(x)))))
            t0 = time.perf_counter()
            self.compute(ctx, "phi", x, a)
            self.cost.observe("phi", x, time.perf_counter() - t0, weight=1.0)

    def device_bytes(self):
        return sum(c.device_bytes() for c in self.ctx if c is not None)

    def submit(self, kind, x, a=None):
        r = Request(kind, int(x), None if a is None else int(a))
        if r.x > self.max_x:
            self.refused += 1
            r.future.set_exception(pcg.PrimecountError(2, "x above the admitted maximum %d" % self.max_x))
            return r
        r.need = int(self.bytes_of(kind, r.x, r.a))
        if r.need > self.mem_budget:
            self.refused_memory += 1
            r.future.set_exception(pcg.PrimecountError(PCG_ENOMEM, "needs %d device bytes, budget %d"
                                                       % (r.need, self.mem_budget)))
            return r
        r.est = self.cost.est(kind, r.x, r.a)
        with self.cv:
            if self.budget is not None and self.backlog + r.est > self.budget and self.backlog > 0:
                self.shed += 1
                r.future.set_exception(pcg.PrimecountError(PCG_EAGAIN, "overloaded: %.2f s of admitted work"
                                                           % self.backlog))
                return r
            self.backlog += r.est
            self.admitted += 1
            self.q.append(r)
            self.cv.notify()
        return r

    def _work(self, ctx):
        while True:
            with self.cv:
                while not self.stop and (not self.q or self.inflight + self.q[0].need > self.mem_budget):
                    if self.q:
                        self.q[0].waited = True     # at the head, its memory not free yet
                    self.cv.wait()
                if self.stop and not self.q:
                    return
                if self.inflight + self.q[0].need > self.mem_budget:
                    continue
                r = self.q.popleft()
                self.inflight += r.need
                self.peak_inflight = max(self.peak_inflight, self.inflight)
                if r.waited:
                    self.waited_for_memory += 1
            t0 = time.perf_counter()
            try:
                v = self.compute(ctx, r.kind, r.x, r.a)
                r.t_done = time.perf_counter()
                self.cost.observe(r.kind, r.x, r.t_done - t0)
                r.future.set_result(v)
            except Exception as e:  # reported through the future
                r.t_done = time.perf_counter()
                r.future.set_exception(e)
            if ctx is not None and r.need > self.share:
                # keep this worker's idle working memory within its share
                try:
                    ctx.trim()
                    self.trims += 1
                except pcg.PrimecountError:
                    pass
            with self.cv:
                self.backlog = max(0.0, self.backlog - r.est)
                self.inflight -= r.need
                self.cv.notify_all()

    def cancel_pending(self):
        """Drop the queued requests (they fail with PCG_ECANCELLED)."""
        with self.cv:
            n = len(self.q)
            while self.q:
                r = self.q.popleft()
                self.backlog = max(0.0, self.backlog - r.est)
                r.future.set_exception(pcg.PrimecountError(7, "cancelled"))
            self.cv.notify_all()
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


def run_served(stream, workers=4, max_x=10 ** 20, drain_s=30.0, latency_budget=None, compute=None,
               bytes_of=None, mem_budget=0, calibrate=True):
    srv = Server(max_x=max_x, workers=workers, latency_budget=latency_budget, compute=compute,
                 bytes_of=bytes_of, mem_budget=mem_budget, calibrate=calibrate)
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
            "refused_above_memory": srv.refused_memory, "waited_for_memory": srv.waited_for_memory,
            "mem_budget_bytes": srv.mem_budget, "peak_inflight_bytes": srv.peak_inflight, "trims": srv.trims,
            "cancelled_at_deadline": cancelled, "wall_s": t_stop - t0, "qps": len(ok) / (t_stop - t0),
            "p50_s": percentile(lat, 0.5), "p99_s": percentile(lat, 0.99),
            "cost_model": {k: {str(d): round(v, 6) for d, v in sorted(m.items())} for k, m in srv.cost.t.items()},
            "results": {id(r): r.future.result() for r in ok},
            "requests": [(r.kind, r.x, r.a, r.future.result()) for r in ok]}


def run_plain(stream, drain_s=30.0, latency_budget=None, compute=None, cost=None):
    """One request at a time, tables built inside every call; the same
    latency rule (budget on the estimated GPU-seconds waiting, the served
    run's fitted cost model when given)."""
    cost = cost or CostModel()
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
            e = cost.est(k, x, a)
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
            _compute_pcg(c, k, x, a)
            c.close()
        else:
            compute(None, k, x, a)
        backlog = max(0.0, backlog - e)
        lat.append(time.perf_counter() - t0 - t)
        n += 1
    wall = time.perf_counter() - t0
    return {"completed": n, "submitted": len(stream), "shed_by_budget": shed, "wall_s": wall, "qps": n / wall,
            "p50_s": percentile(lat, 0.5), "p99_s": percentile(lat, 0.99)}


def cost_from(table):
    """A CostModel holding the decade figures of a served run's report."""
    m = CostModel()
    for k, v in table.items():
        for d, t in v.items():
            m.t[k][int(d)] = t
    return m


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
    ap.add_argument("--mem-budget", type=float, default=0, help="device bytes for working memory (0 = auto)")
    ap.add_argument("--plain", action="store_true")
    a = ap.parse_args()
    budget = a.budget if a.budget > 0 else None
    stream = make_stream(a.seed, a.rate, a.seconds, pi_range=(8, a.pi_max_exp))
    out = {"config": {"rate": a.rate, "seconds": a.seconds, "seed": a.seed, "workers": a.workers,
                      "pi_x": "10^U(8,%g)" % a.pi_max_exp, "phi_x": "10^U(8,16)", "requests": len(stream),
                      "latency_budget_s": budget}}
    r = run_served(stream, workers=a.workers, max_x=int(float(a.max_x)), drain_s=a.drain, latency_budget=budget,
                   mem_budget=int(a.mem_budget))
    r.pop("results")
    r.pop("requests")
    out["served"] = r
    if a.plain:
        out["plain"] = run_plain(stream, drain_s=a.drain, latency_budget=budget, cost=cost_from(r["cost_model"]))
    print(json.dumps(out))


if __name__ == "__main__":
    main()
