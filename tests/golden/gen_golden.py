#!/usr/bin/env python3
"""Generate the golden fixtures in tests/golden/ from the reference.

Sources (all read here, at generation time only; nothing at test time reads
the reference):

* the reference's own known-answer tables, read as text:
  - test/gourdon/D.cpp:36-89            (51 D(x, y, z, k) tuples)
  - test/deleglise-rivat/S2_hard_alpha.cpp:36-73 (35 S2_hard tuples)
  - README.md:163-277                   (pi(10^n), n = 10..22)
  - test/api/api.cpp:112-116            (phi(1e12, 78498))
  - test/gourdon/pi_gourdon.cpp:94-106  (pi(1e11), pi(1e12))
* the reference binary compiled from its sources by oracle/ref.mk
  (oracle/_ref/<cpu arch>/primecount), run for D, S2_hard, pi and phi at further
  inputs.  Parameters (y, z, k / c) are read from its --status output.

Usage:  python tests/golden/gen_golden.py [--ref <primecount source tree>] [--big]
--ref defaults to the environment variable PCG_REFERENCE.  --big adds the
multi-minute inputs (D at 1e19..1e22, S2_hard at 1e19..1e20).
Existing entries in the fixture are kept, so expensive values are computed
once.
"""
import argparse
import json
import os
import platform
import random
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "hard_leaves.json")
BIN = os.path.join(ROOT, "oracle", "_ref", platform.machine(), "primecount")


def tuples(path):
    s = open(path).read()
    pat = r"\{\s*(\d+)LL,\s*(\d+),\s*(\d+),\s*(\d+),\s*(-?\d+)LL\s*\}"
    return [[int(t) for t in m] for m in re.findall(pat, s)]


def readme_pi(path):
    s = open(path).read()
    rows = re.findall(r"<td>10<sup>(\d+)</sup></td>\s*<td>([\d,]+)</td>", s)
    return {int(n): int(v.replace(",", "")) for n, v in rows}


def run(args, threads=8):
    out = subprocess.run([BIN] + [str(a) for a in args] + ["-t%d" % threads],
                         check=True, capture_output=True, text=True).stdout
    return out


def run_status(x, opt):
    """Run `primecount x opt -s`; return (result, vars dict)."""
    out = run([x, opt, "-s"])
    out = re.sub(r"\x1b\[K|\r", "\n", out)
    vars_ = {}
    for key in ("x", "y", "z", "k", "c", "alpha", "alpha_y", "alpha_z", "x_star"):
        m = re.search(r"^%s = ([-\d.]+)$" % key, out, re.M)
        if m:
            vars_[key] = m.group(1)
    lines = [l for l in out.splitlines() if l.strip()]
    res = int(lines[-1]) if re.fullmatch(r"-?\d+", lines[-1].strip()) else None
    if res is None:
        m = re.findall(r"^(?:D|S2_hard|A \+ C|B|Phi0|Sigma|S1|S2_trivial|S2_easy|P2) = (-?\d+)$", out, re.M)
        res = int(m[-1])
    return res, vars_


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("PCG_REFERENCE"))
    ap.add_argument("--big", action="store_true")
    a = ap.parse_args()
    ref = a.ref
    if not ref:
        sys.exit("pass --ref <primecount source tree> or set PCG_REFERENCE")

    data = {}
    if os.path.exists(OUT):
        data = json.load(open(OUT))

    data["source"] = ("kimwalisch/primecount 8.7: test tables read as text, "
                      "further values from the reference binary built by oracle/ref.mk")
    data["D_tuples"] = tuples(os.path.join(ref, "test/gourdon/D.cpp"))
    data["S2_hard_tuples"] = tuples(os.path.join(ref, "test/deleglise-rivat/S2_hard_alpha.cpp"))
    pis = readme_pi(os.path.join(ref, "README.md"))
    pis[11] = 4118054813
    pis[12] = 37607912018
    data["pi_pow10"] = {str(10 ** n): v for n, v in sorted(pis.items())}
    data["phi_api"] = [[10 ** 12, 78498, 37607833521]]

    have_bin = os.path.exists(BIN)
    if not have_bin:
        print("reference binary missing: build it with make -f oracle/ref.mk", file=sys.stderr)
        json.dump(data, open(OUT, "w"), indent=1)
        return

    # D and S2_hard at default parameters, x = 10^15 .. 10^18 (and --big: beyond)
    dx = data.setdefault("D_default", {})
    sx = data.setdefault("S2_hard_default", {})
    exps = [15, 16, 17, 18]
    if a.big:
        exps += [19, 20, 21, 22]
    for e in exps:
        x = 10 ** e
        if str(x) not in dx:
            r, v = run_status(x, "--D")
            dx[str(x)] = {"y": int(v["y"]), "z": int(v["z"]), "k": int(v["k"]), "D": r}
            print("D", x, dx[str(x)], flush=True)
        if str(x) not in sx and e <= (20 if a.big else 18):
            r, v = run_status(x, "--S2-hard")
            sx[str(x)] = {"y": int(v["y"]), "z": int(v["z"]), "c": int(v["c"]), "S2_hard": r}
            print("S2_hard", x, sx[str(x)], flush=True)
        json.dump(data, open(OUT, "w"), indent=1)

    # D at seeded random x in [1e6, 1e15] with default parameters
    if "D_random" not in data:
        rng = random.Random(20261203)
        rows = []
        for _ in range(60):
            x = int(10 ** rng.uniform(6, 15))
            r, v = run_status(x, "--D")
            rows.append([x, int(v["y"]), int(v["z"]), int(v["k"]), r])
        data["D_random"] = rows
    if "S2_hard_random" not in data:
        rng = random.Random(20261204)
        rows = []
        for _ in range(60):
            x = int(10 ** rng.uniform(6, 15))
            r, v = run_status(x, "--S2-hard")
            rows.append([x, int(v["y"]), int(v["z"]), int(v["c"]), r])
        data["S2_hard_random"] = rows

    # pi(x) at seeded random x in [1e8, 1e17]
    if "pi_random" not in data:
        rng = random.Random(20261205)
        rows = []
        for _ in range(120):
            x = int(10 ** rng.uniform(8, 17))
            rows.append([x, int(run([x]).strip().splitlines()[-1])])
        data["pi_random"] = rows

    # phi(x, a) at seeded random (x, a): x log-uniform in [1e4, 1e12]
    if "phi_random" not in data:
        rng = random.Random(20261206)
        rows = []
        for _ in range(120):
            x = int(10 ** rng.uniform(4, 12))
            sq = int(x ** 0.5)
            pis_q = int(run([sq]).strip().splitlines()[-1])
            a_ = rng.randint(1, max(1, pis_q))
            rows.append([x, a_, int(run(["--phi", x, a_]).strip().splitlines()[-1])])
        data["phi_random"] = rows

    # Gourdon's other terms, to pin pi(x) term by term (--AC, --B, --Phi0,
    # --Sigma print the reference's own value of each formula)
    if "gourdon_parts" not in data:
        rng = random.Random(20261207)
        xs = [10 ** e for e in range(8, 19)] + [int(10 ** rng.uniform(8, 17)) for _ in range(24)]
        rows = []
        for x in xs:
            row = {"x": x}
            for opt, key in (("--AC", "AC"), ("--B", "B"), ("--Phi0", "Phi0"), ("--Sigma", "Sigma")):
                r, v = run_status(x, opt)
                row[key] = r
                row.update({"y": int(v["y"]), "z": int(v["z"]), "k": int(v["k"])} if "z" in v else {"y": int(v["y"])})
            row["D"] = run_status(x, "--D")[0]
            row["pi"] = int(run([x]).strip().splitlines()[-1])
            rows.append(row)
            print("parts", row, flush=True)
        data["gourdon_parts"] = rows

    # the Deleglise-Rivat terms (--S1, --S2-trivial, --S2-easy, --S2-hard, --P2)
    # and its pi(x) (-d), to pin the device form of that formula term by term
    if "dr_parts" not in data:
        rng = random.Random(20261204)
        xs = [10 ** e for e in range(11, 20)] + [int(10 ** rng.uniform(11, 18)) for _ in range(16)]
        rows = []
        for x in xs:
            row = {"x": x}
            for opt, key in (("--S1", "S1"), ("--S2-trivial", "S2_trivial"), ("--S2-easy", "S2_easy"),
                             ("--S2-hard", "S2_hard"), ("--P2", "P2")):
                r, v = run_status(x, opt)
                row[key] = r
                if "c" in v:
                    row.update({"y": int(v["y"]), "z": int(v["z"]), "c": int(v["c"])})
            row["pi"] = int(run([x, "-d"]).strip().splitlines()[-1])
            rows.append(row)
            print("dr", row, flush=True)
        data["dr_parts"] = rows

    json.dump(data, open(OUT, "w"), indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
