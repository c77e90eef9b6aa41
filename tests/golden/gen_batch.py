#!/usr/bin/env python3
"""Generate tests/golden/batch_4096.json: the seeded batched-query workload
(4096 pi(x) with x = floor(10^U(10,18)) and 4096 phi(x, a) with
x = floor(10^U(8,16)), a = 1 + floor(u * pi(floor(sqrt x))), u = U(0,1);
Python's random.Random(20261203)) together with the answers of the reference
binary (oracle/_ref/<cpu arch>/primecount, built from the reference's sources
by oracle/ref.mk): `primecount x` and `primecount --phi x a`.

The inputs are stored as integers, so every host reads the same queries.
Existing answers are kept (the file is written as answers arrive), so an
interrupted run resumes.

Usage:  python tests/golden/gen_batch.py [--n 4096] [--jobs 4] [--threads 2]
"""
import argparse
import concurrent.futures as cf
import json
import math
import os
import platform
import random
import subprocess
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "batch_4096.json")
BIN = os.path.join(ROOT, "oracle", "_ref", platform.machine(), "primecount")
SEED = 20261203


def inputs(n):
    """The seeded queries: pi xs, phi xs and the uniform draws for a."""
    rng = random.Random(SEED)
    xs = [int(10 ** rng.uniform(10, 18)) for _ in range(n)]
    px = [int(10 ** rng.uniform(8, 16)) for _ in range(n)]
    us = [rng.random() for _ in range(n)]
    return xs, px, us


def ref(args, threads):
    out = subprocess.run([BIN] + [str(a) for a in args] + ["-t%d" % threads], check=True, capture_output=True,
                         text=True).stdout
    return int(out.strip().splitlines()[-1])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=4096)
    ap.add_argument("--jobs", type=int, default=4)
    ap.add_argument("--threads", type=int, default=2)
    a = ap.parse_args()
    data = json.load(open(OUT)) if os.path.exists(OUT) else {}
    xs, px, us = inputs(a.n)
    if data.get("pi_x") != [str(v) for v in xs] or data.get("phi_x") != [str(v) for v in px]:
        data = {"seed": SEED, "n": a.n,
                "source": "kimwalisch/primecount 8.7 binary built by oracle/ref.mk: primecount x, primecount --phi x a",
                "pi_x": [str(v) for v in xs], "phi_x": [str(v) for v in px], "phi_u": us,
                "pi": [None] * a.n, "pi_sqrt": [None] * a.n, "phi_a": [None] * a.n, "phi": [None] * a.n}
    lock = threading.Lock()

    def save():
        tmp = OUT + ".tmp"
        json.dump(data, open(tmp, "w"), separators=(",", ":"))
        os.replace(tmp, OUT)

    def job(kind, i):
        if kind == "pi":
            v = ref([xs[i]], a.threads)
            with lock:
                data["pi"][i] = str(v)
        else:
            x = px[i]
            ps = ref([math.isqrt(x)], a.threads)
            aa = 1 + int(us[i] * max(1, ps))
            v = ref(["--phi", x, aa], a.threads)
            with lock:
                data["pi_sqrt"][i] = ps
                data["phi_a"][i] = aa
                data["phi"][i] = str(v)

    todo = [("pi", i) for i in range(a.n) if data["pi"][i] is None]
    todo += [("phi", i) for i in range(a.n) if data["phi"][i] is None]
    # the pi queries first, each kind largest first, so that the pool ends on
    # small queries
    todo.sort(key=lambda t: (t[0] != "pi", -(xs[t[1]] if t[0] == "pi" else px[t[1]])))
    done = 0
    with cf.ThreadPoolExecutor(max_workers=a.jobs) as ex:
        for _ in cf.as_completed([ex.submit(job, k, i) for k, i in todo]):
            done += 1
            if done % 64 == 0:
                with lock:
                    save()
                print("done", done, "of", len(todo), flush=True)
    save()
    print("wrote", OUT)


if __name__ == "__main__":
    main()
