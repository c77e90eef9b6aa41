#!/usr/bin/env python3
"""Headline benchmark: Gourdon's D(1e20) (the hard special leaves of
pi(1e20)) on one GB300, in hard-leaves/s.

One step = one D(x, y, z, k) evaluation at x = 1e20 with the reference's
default parameters (y = z = 245535363, k = 8): the full sieve of [0, x/z)
and all 22 178 370 075 hard leaves.

value        device-timed (CUDA events on the launching stream), tables
             resident in HBM, L2 flushed between steps.
e2e          the C-ABI call pcg_D on a fresh context: table construction,
             host->device parameter copies, the sweep and the device->host
             result copy, host wall clock.
roofline     the sieve/leaf kernel (k_sweep) against the measured HBM copy
             peak, with the algorithmic bytes of the hot-path table: 2 B per
             FactorTable entry read, 4 B per two-prime leaf (its prime),
             16 B per (segment, b) step (PiTable word of the level bounds),
             over its CUDA-event launch time; the 8 B reciprocal per leaf is
             implementation traffic, reported apart.  traffic = DRAM bytes
             per launch, scaled from the committed ncu capture of a smaller
             D by the algorithmic bytes.  int_ops: algorithmic integer and
             shared-memory operations (per leaf one division and one prefix
             query of a counter load and up to 8 popcounts; per cross-off
             one shared-memory read-modify-write) against the SMs' lane
             issue rate.
cpu_baseline the reference's own D() (its CLI --D, OpenMP on all host
             threads, built from its sources by oracle/ref.mk with its
             run-time SIMD dispatch) timed once on the whole workload; the
             oracle's restatement on a sample when the reference build is
             missing (kind "port").

--impl reference: the reference's own D(1e20) on all host threads, one
             whole evaluation per timed step (the warm-up steps run D at
             x / 1000); this arm imports nothing of primecount_gb300.
--gpus N > 1 (torchrun, NCCL): one D(1e20) over N GPUs -- rank r sweeps
             shard r of the segment plan (pcg_D_shard), then one all-gather
             of the per-level partials and the exact combine on every rank
             (strong scaling: the total work is fixed).
"""
import argparse
import json
import os
import platform
import re
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

X = 10 ** 20
WORKLOAD = "D(1e20) hard special leaves, Gourdon default parameters (y=z=245535363, k=8)"
METRIC = "pi(1e20) sec & hard-leaves/s on 1 GB300"
UNIT = "hard-leaves/s"
TOTAL_LEAVES_1E20 = 22178370075
# hard leaves of D(x) at the reference's default parameters (deterministic;
# the engine's and the oracle's counts agree)
LEAVES = {10 ** 14: 8384338, 10 ** 16: 111012964, 10 ** 18: 1524253981, 10 ** 20: TOTAL_LEAVES_1E20}
REF_BIN = os.path.join(ROOT, "oracle", "_ref", platform.machine(), "primecount")


def clocks_sampler(stop, out):
    cmd = ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
           "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
           "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
           "--format=csv,noheader,nounits", "-lms", "200"]
    try:
        p = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
    except Exception:
        return
    while not stop.is_set():
        line = p.stdout.readline()
        if not line:
            break
        out.append(line.strip())
    p.terminate()


def summarize_clocks(rows, dev):
    sm, mx, reasons = [], 0, set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for r in rows:
        f = [t.strip() for t in r.split(",")]
        if len(f) < 9 or f[0] != str(dev):
            continue
        try:
            sm.append(float(f[1]))
            mx = max(mx, float(f[2]))
        except ValueError:
            continue
        for n, v in zip(names, f[5:9]):
            if v.lower().startswith("active"):
                reasons.add(n)
    sm.sort()
    return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx or None,
            "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs"), "measured"
    return 6800.0, "fallback"


def profile_traffic():
    """DRAM bytes per k_sweep launch of D(1e20), from the committed summary of
    an ncu capture of every k_sweep launch of one D(1e20) (its line
    `dram_bytes_per_launch: N`), if present."""
    p = os.path.join(ROOT, "profiles", "k_sweep_traffic_D1e20.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.strip().startswith("dram_bytes_per_launch:"):
            try:
                return {"bytes": float(line.split(":", 1)[1].strip().split()[0]),
                        "source": "profiles/k_sweep_traffic_D1e20.md"}
            except ValueError:
                return None
    return None


def profile_issue():
    """Issue-slot use of k_sweep (ncu smsp__issue_active, % of peak) in a dense
    and a sparse wave of D(1e18), from the committed capture summary: the
    kernel is bound by integer issue and the per-level chain, not by HBM."""
    p = os.path.join(ROOT, "profiles", "k_sweep_D1e18.md")
    try:
        for line in open(p):
            if "smsp__issue_active" in line:
                cells = [c.strip() for c in line.strip().strip("|").split("|")]
                return {"dense_wave_pct": float(cells[1].split()[0]), "sparse_wave_pct": float(cells[2].split()[0]),
                        "source": "profiles/k_sweep_D1e18.md"}
    except (OSError, ValueError, IndexError):
        return None
    return None


def ref_D(x, threads):
    """(D(x), seconds) from the reference's own CLI: `primecount x --D -t N
    --time` (src/app/main.cpp:205-246, 569-570), the time being the
    reference's get_time() around its D()."""
    out = subprocess.run([REF_BIN, str(x), "--D", "-t%d" % threads, "--time"], check=True, capture_output=True,
                         text=True).stdout
    val = int(out.strip().splitlines()[0])
    secs = float(re.search(r"Seconds:\s*([0-9.]+)", out).group(1))
    return val, secs


def ref_build_flags():
    p = os.path.join(os.path.dirname(REF_BIN), "build_flags.txt")
    try:
        return open(p).read().strip()
    except OSError:
        return None


def cpu_baseline(p, threads, target_s=12.0):
    """The reference's own D(x) over the whole workload on all host threads
    (kind "reference"), or, without the reference build, the oracle's
    restatement of its chunk loop on a sample of the interval (kind "port")."""
    why = "the reference's build is missing"
    if os.access(REF_BIN, os.X_OK) and X in LEAVES:
        try:
            val, secs = ref_D(X, threads)
            return {"value": LEAVES[X] / secs, "unit": UNIT, "cores": threads, "kind": "reference",
                    "sample": "the whole D(%s) (%d hard leaves) by the reference's own --D on %d threads: %.2f s, "
                              "result %d" % (args_x_str(), LEAVES[X], threads, secs, val),
                    "seconds": secs, "build": ref_build_flags()}
        except (subprocess.CalledProcessError, OSError, AttributeError, ValueError) as e:
            why = "the reference's build failed to run: %s" % str(e)[:200]
    r = port_sample(p, threads, target_s)
    r["why_port"] = why
    return r


def args_x_str():
    return "%.0e" % X if X >= 10 ** 6 else str(X)


def port_sample(p, threads, target_s=12.0):
    """Oracle restatement of the reference's chunk loop, timed on a sample of
    D(x): nchunks sub-intervals starting at c / nchunks of [0, x/z), all
    host threads.  The rate is the sample's leaves over its wall time; the
    sample fraction grows until it takes about target_s."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.load()
    nchunks = max(64, 4 * threads)
    frac = 1e-4
    leaves, secs = oracle.D_sample(X, p["y"], p["z"], p["k"], nchunks, frac, threads)
    while secs < target_s * 2 / 3 and frac < 0.05:
        step = min(10.0, 0.8 * target_s / max(secs, 1e-3)) if secs < 0.3 else \
            max(1.1, min(2.0, (target_s / secs) ** 0.25))
        frac = min(0.05, frac * step)
        leaves, secs = oracle.D_sample(X, p["y"], p["z"], p["k"], nchunks, frac, threads)
    return {"value": leaves / secs, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "oracle chunk loop (the reference's build is missing) on %d sub-intervals starting at "
                      "c/%d of [0, x/z), together %.4g of the interval: %d leaves in %.1f s wall on %d threads"
                      % (nchunks, nchunks, frac, leaves, secs, threads)}


BATCH_FIXTURE = os.path.join(ROOT, "tests", "golden", "batch_4096.json")


def batch_workload(n, pcg):
    """The seeded batch (4096 pi(x), x = floor(10^U(10,18)); 4096 phi(x, a),
    x = floor(10^U(8,16)), a = 1 + floor(u pi(floor(sqrt x))); seed 20261203)
    with the reference's answers, from the committed fixture
    (tests/golden/gen_batch.py); without it, the same generator and no
    reference answers."""
    import math
    if os.path.exists(BATCH_FIXTURE):
        d = json.load(open(BATCH_FIXTURE))
        if d.get("n", 0) >= n:
            xs = [int(v) for v in d["pi_x"][:n]]
            px = [int(v) for v in d["phi_x"][:n]]
            us = d["phi_u"][:n]
            pa = d["phi_a"][:n]
            if any(a is None for a in pa):
                # a = 1 + floor(u pi(floor(sqrt x))) where the fixture has no answer yet
                pis = pcg.pi_batch([math.isqrt(x) for x in px])
                pa = [a if a is not None else 1 + int(u * max(1, p)) for a, u, p in zip(pa, us, pis)]
            return (xs, [None if v is None else int(v) for v in d["pi"][:n]], px, [int(a) for a in pa],
                    [None if v is None else int(v) for v in d["phi"][:n]], "tests/golden/batch_4096.json")
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import gen_batch
    xs, px, us = gen_batch.inputs(n)
    pis = pcg.pi_batch([math.isqrt(x) for x in px])
    pa = [1 + int(u * max(1, p)) for u, p in zip(us, pis)]
    return xs, [None] * n, px, pa, [None] * n, "generated (no fixture)"


def run_batch(args, pcg):
    import torch
    n = args.batch
    xs, want_pi, px, pa, want_phi, src = batch_workload(n, pcg)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r_pi = pcg.pi_batch(xs)
    t1 = time.perf_counter()
    r_phi = pcg.phi_batch(px, pa)
    t2 = time.perf_counter()
    checked = [(g, w) for g, w in zip(r_pi + r_phi, want_pi + want_phi) if w is not None]
    bad = sum(1 for g, w in checked if g != w)
    if bad:
        raise SystemExit("batch: %d answers differ from the reference fixture" % bad)
    # plain: one query per call, tables built inside (fresh context), on a
    # sample stratified by decade of x (the time of a query grows steeply
    # with x, so an unstratified sample of a few dozen queries misses the
    # largest ones): per decade the mean time of its sampled queries times
    # its number of queries estimates the whole batch's plain time
    import math
    per = max(1, args.plain_sample // 8)

    def plain(kind, xs_, fn, want):
        dec = {}
        for i, x in enumerate(xs_):
            dec.setdefault(int(math.log10(max(x, 1))), []).append(i)
        est, times = 0.0, []
        for d, idx in sorted(dec.items()):
            pick = [idx[(j * len(idx)) // per] for j in range(min(per, len(idx)))]
            ts = []
            for i in pick:
                c = pcg.Context(0)
                a0 = time.perf_counter()
                v = fn(i, c)
                ts.append(time.perf_counter() - a0)
                c.close()
                if v != want[i]:
                    raise SystemExit("batch: the plain answer differs from the batched one (%s, %d)" % (kind, i))
            times += ts
            est += len(idx) * sum(ts) / len(ts)
        return est, sorted(times)

    est_pi, plain_pi = plain("pi", xs, lambda i, c: pcg.pi(xs[i], ctx=c), r_pi)
    est_phi, plain_phi = plain("phi", px, lambda i, c: pcg.phi(px[i], pa[i], ctx=c), r_phi)

    def p99(v):
        return v[min(len(v) - 1, int(round(0.99 * (len(v) - 1))))] if v else None
    return {"queries": {"pi": n, "phi": n}, "seed": 20261203, "inputs": src,
            "engine": {"pi_qps": n / (t1 - t0), "phi_qps": n / (t2 - t1), "all_qps": 2 * n / (t2 - t0),
                       "seconds": t2 - t0, "pi_seconds": t1 - t0, "phi_seconds": t2 - t1,
                       "latency_note": "one call per kind: every query of a call completes when the call returns "
                                       "(p99 latency = the call's wall time)"},
            "plain_sample": {"queries_per_kind": len(plain_pi), "per_decade": per,
                             "pi_qps": n / est_pi, "phi_qps": n / est_phi,
                             "pi_seconds_est": est_pi, "phi_seconds_est": est_phi,
                             "all_qps": 2 * n / (est_pi + est_phi),
                             "pi_p99_of_sample_s": p99(plain_pi), "phi_p99_of_sample_s": p99(plain_phi),
                             "note": "the same batch one query per call (fresh context): per decade of x the mean "
                                     "time of an evenly spread sample times the decade's number of queries"},
            "checks": {"reference_answers_checked": len(checked), "mismatches": bad,
                       "plain_equal_batched": True}}


def run_reference(args, rank):
    """The reference's own D(x) (its CLI, OpenMP on all host threads): one
    whole evaluation per timed step.  Nothing of primecount_gb300 is
    imported: the reference's defaults give y, z, k itself."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    base = {"impl": "reference", "metric": METRIC, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int64/int128", "data": "synthetic (scalar x)",
            "config": {"workload": WORKLOAD if X == 10 ** 20 else "D(%s)" % args.x, "x": args.x,
                       "l2": "n/a (CPU)"}}
    why = None
    if not os.access(REF_BIN, os.X_OK) or X not in LEAVES:
        why = "the reference's build is missing"
    else:
        try:
            for _ in range(max(1, args.warmup)):
                ref_D(X // 1000, threads)
        except (subprocess.CalledProcessError, OSError, AttributeError, ValueError) as e:
            why = "the reference's build failed to run: %s" % str(e)[:200]
    if why:
        # the reference did not build on this host: the oracle's restatement
        p = None
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        oracle.load()
        p = oracle.gourdon_params(X)
        vals, t0 = [], time.time()
        for _ in range(args.steps):
            cb = port_sample(p, threads, target_s=8.0)
            vals.append(cb["value"])
        v = sum(vals) / len(vals)
        line = dict(base, value=v, ms_per_step=1000 * (time.time() - t0) / max(args.steps, 1),
                    cpu_baseline={"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                                  "sample": cb["sample"], "why_port": why},
                    e2e={"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0})
        print(json.dumps(line), flush=True)
        return
    secs, wall, val = [], [], None
    for _ in range(args.steps):
        t0 = time.perf_counter()
        val, s_ = ref_D(X, threads)
        wall.append(time.perf_counter() - t0)
        secs.append(s_)
    ms = 1000.0 * sum(secs) / len(secs)
    v = LEAVES[X] / (ms / 1000.0)
    line = dict(base, value=v, ms_per_step=ms, result=str(val),
                cpu_baseline={"value": v, "unit": UNIT, "cores": threads, "kind": "reference",
                              "sample": "the whole D(%s) per step (%d hard leaves) by the reference's own --D "
                                        "on %d threads; warm-up steps (at least one) D(x/1000)"
                                        % (args.x, LEAVES[X], threads),
                              "build": ref_build_flags(), "step_seconds": secs,
                              "step_wall_seconds": wall},
                e2e={"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0})
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--x", default="1e20", help="smaller x for profiling runs (the headline is 1e20)")
    ap.add_argument("--pi-steps", type=int, default=3, help="pi(x) end-to-end repetitions (the median is reported)")
    ap.add_argument("--batch", type=int, default=4096,
                    help="queries per kind of the batched workload (4096 = the full config; 0 = skip)")
    ap.add_argument("--plain-sample", type=int, default=32, help="queries per kind timed in the plain form")
    ap.add_argument("--serve-seconds", type=float, default=60, help="serving stream length (0 = skip)")
    ap.add_argument("--serve-drain", type=float, default=10, help="seconds to finish admitted requests")
    ap.add_argument("--serve-budget", type=float, default=2.0,
                    help="serving latency budget in estimated GPU-seconds (0 = admit everything)")
    args = ap.parse_args()
    global X
    X = int(float(args.x)) if "e" in args.x else int(args.x)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        run_reference(args, rank)
        return

    import torch
    import primecount_gb300 as pcg

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()

    p = pcg.gourdon_params(X)
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    ctx = pcg.Context(0)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    if world > 1:
        # one D(x) over the N GPUs: this rank sweeps shard `rank` of the
        # segment plan, then one all-gather of the per-level partials
        from primecount_gb300.shard import combine_distributed

        def step(c=None, s=None):
            part = pcg.D_shard(X, p["y"], p["z"], p["k"], rank, world, ctx=c or ctx, stream=s)
            return combine_distributed(part)
    else:
        def step(c=None, s=None):
            return pcg.D(X, p["y"], p["z"], p["k"], ctx=c or ctx, stream=s)

    for _ in range(max(args.warmup, 1)):
        v = step(s=sptr)
    stats0 = ctx.last_stats()

    rows = []
    stop = threading.Event()
    th = threading.Thread(target=clocks_sampler, args=(stop, rows), daemon=True)
    th.start()
    time.sleep(0.5)

    barrier()
    torch.cuda.synchronize()
    evs = []
    kernel_ms = 0.0
    launches = 0
    t0 = time.time()
    for i in range(args.steps):
        flush.fill_(i & 0xFF)
        s_ev = torch.cuda.Event(enable_timing=True)
        e_ev = torch.cuda.Event(enable_timing=True)
        s_ev.record(stream)
        v = step(s=sptr)
        e_ev.record(stream)
        evs.append((s_ev, e_ev))
        st = ctx.last_stats()
        kernel_ms += st["sweep_kernel_ms"]
        launches += st["sweep_launches"]
    torch.cuda.synchronize()
    barrier()
    wall = time.time() - t0
    stop.set()
    th.join(timeout=2)
    dev_ms = [a.elapsed_time(b) for a, b in evs]
    ms_step = sum(dev_ms) / len(dev_ms)
    if dist is not None:
        t = torch.tensor([ms_step], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_step = float(t.item())
    leaves = st["leaves"]
    if dist is not None:
        t = torch.tensor([leaves], dtype=torch.int64, device="cuda")
        dist.all_reduce(t)
        leaves = int(t.item())
    value = leaves / (ms_step / 1000.0)

    # e2e: the C-ABI call on a fresh context (tables built inside the call)
    e2e_t, h2d, d2h = [], 0, 0
    for _ in range(args.e2e_steps):
        c2 = pcg.Context(0)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        v2 = step(c=c2)
        e2e_t.append(time.perf_counter() - t1)
        s2 = c2.last_stats()
        h2d, d2h = s2["h2d_bytes"], s2["d2h_bytes"]
        c2.close()
        assert v2 == v
    e2e_s = sum(e2e_t) / len(e2e_t) if e2e_t else float("nan")

    # pi(x) end to end through the C ABI (pcg_pi, fresh context: every table
    # built inside the call), with the time of each Gourdon term
    pi_line = None
    if args.pi_steps > 0 and rank == 0:
        ts = []
        for _ in range(args.pi_steps):
            c3 = pcg.Context(0)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            pv = pcg.pi(X, ctx=c3)
            ts.append(time.perf_counter() - t1)
            s3 = c3.last_stats()
            c3.close()
        pi_line = {"x": args.x, "pi": str(pv), "seconds": sorted(ts)[len(ts) // 2], "seconds_min": min(ts),
                   "seconds_all": ts,
                   "terms_ms": {"D": s3["d_ms"], "AC": s3["ac_ms"], "B": s3["b_ms"], "Phi0": s3["phi0_ms"],
                                "Sigma": s3["sigma_ms"], "tables": s3["table_ms"]},
                   "terms_note": "a new context per call (tables built inside it); D runs beside A+C, B, Phi0 "
                                 "and Sigma, so the term times are wall times of the two host threads"}

    batch = run_batch(args, pcg) if args.batch > 0 and rank == 0 else None
    serve = None
    if args.serve_seconds > 0 and rank == 0:
        from primecount_gb300 import serve as sv
        stream = sv.make_stream(20261203, 2000, args.serve_seconds)
        budget = args.serve_budget if args.serve_budget > 0 else None
        r = sv.run_served(stream, workers=8, max_x=10 ** 20, drain_s=args.serve_drain, latency_budget=budget)
        r.pop("results")
        served_answers = r.pop("requests")
        plain = sv.run_plain(stream, drain_s=args.serve_drain, latency_budget=budget,
                             cost=sv.cost_from(r["cost_model"]))
        # every served answer against the same query computed alone (an evenly spread sample)
        step = max(1, len(served_answers) // 64)
        sample = served_answers[::step]
        alone_ok = all((pcg.pi(x) if k == "pi" else pcg.phi(x, a)) == v for k, x, a, v in sample)
        if not alone_ok:
            raise SystemExit("serve: an answer in the mix differs from the same query alone")
        serve = {"served": r, "plain": plain,
                 "checks": {"served_equal_alone_sample": len(sample)},
                 "config": {"rate": 2000, "seconds": args.serve_seconds, "seed": 20261203,
                            "pi_x": "10^U(8,20)", "phi_x": "10^U(8,16)", "requests": len(stream),
                            "latency_budget_s": budget, "workers": 8, "drain_s": args.serve_drain}}

    if rank != 0:
        return
    peak, peak_kind = measured_peaks()
    # algorithmic bytes of the hot-path table: 2 B per FactorTableD entry
    # read, 4 B per two-prime leaf (its prime), 16 B per (segment, level)
    # step (PiTable word of the level bounds); the 8 B reciprocal of m (or of
    # the prime) per leaf is this implementation's own traffic
    alg_bytes = 2 * st["factor_entries"] + 4 * st["two_prime_leaves"] + 16 * st["levels"]
    impl_bytes = 8 * st["leaves"]
    k_ms_call = kernel_ms / args.steps
    launches_call = launches / args.steps
    launch_s = k_ms_call / launches_call / 1000.0
    achieved = alg_bytes / launches_call / launch_s / 1e9
    tr = profile_traffic()
    traffic = tr["bytes"] if tr and X == 10 ** 20 else None
    # algorithmic integer / shared-memory operations: per leaf one division
    # and one prefix query (a counter load and up to 8 popcounts), per
    # cross-off multiple one shared-memory read-modify-write; against the
    # lane issue rate of the SMs (SMs x 128 lanes x SM clock)
    clk = summarize_clocks(rows, torch.cuda.current_device())
    sm_mhz = clk["sm_mhz"] or 2070.0
    nsm = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    ops = 10 * st["leaves"] + st["crossoff_multiples"]
    ops_peak = nsm * 128 * sm_mhz * 1e6
    ops_achieved = ops / launches_call / launch_s
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
            "kernel": "k_sweep", "alg_bytes_per_launch": alg_bytes / launches_call,
            "impl_bytes_per_launch": impl_bytes / launches_call,
            "impl_achieved_gbs": (alg_bytes + impl_bytes) / launches_call / launch_s / 1e9,
            "traffic_source": tr["source"] if tr else None,
            "launch_ms": k_ms_call / launches_call, "launches_per_step": launches_call,
            "int_ops": {"ops_per_launch": ops / launches_call, "ops_per_leaf": ops / max(st["leaves"], 1),
                        "crossoff_multiples_per_step": st["crossoff_multiples"],
                        "achieved_gops": ops_achieved / 1e9, "peak_gops": ops_peak / 1e9,
                        "frac": ops_achieved / ops_peak,
                        "peak": "%d SMs x 128 lanes x %.0f MHz (lane issue rate)" % (nsm, sm_mhz)},
            "issue_active": profile_issue()}
    cpu = None
    if not args.no_cpu and X == 10 ** 20:
        cpu = cpu_baseline(p, os.cpu_count() or 1)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "strong",
            "vs_baseline": None, "dtype": "int64/int128", "data": "synthetic (scalar x)",
            "config": {"workload": WORKLOAD if X == 10 ** 20 else "D(%s)" % args.x, "x": args.x, "y": p["y"], "z": p["z"], "k": p["k"],
                       "l2": "flushed between steps (256 MiB write)", "parallelism": ("%d shards of the segment plan, one all-gather" % world) if world > 1 else "1 GPU",
                       "segment_words": st["segment_words"], "ctas_per_sm": st["ctas_per_sm"]},
            "result": str(v), "leaves_per_step": leaves,
            "e2e": {"value": leaves / e2e_s, "unit": UNIT, "seconds": e2e_s,
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "pi_e2e": pi_line,
            "batch": batch,
            "serve": serve,
            "gpu_launches": int(st["kernel_launches"]) * args.steps,
            "roofline": roof, "cpu_baseline": cpu,
            "clocks": clk,
            "wall_s": wall}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
