"""Command-line front end mirroring the reference's `primecount` program
(src/app/main.cpp, src/app/CmdOptions.cpp) for the options this engine
serves:

    python -m primecount_gb300 1e20                  pi(x) by Gourdon's algorithm
    python -m primecount_gb300 1e20 --D              D(x) with the default y, z, k
    python -m primecount_gb300 1e18 --S2-hard        S2_hard(x) with the default y, z, c
    python -m primecount_gb300 1e20 --AC | --B | --Phi0 | --Sigma
    python -m primecount_gb300 1e20 -d               pi(x) by the Deleglise-Rivat algorithm
    python -m primecount_gb300 1e20 --S1 | --S2-trivial | --S2-easy | --P2
    python -m primecount_gb300 1e12 78498 --phi      phi(x, a)
    options: -s / --status (print the parameters), --time, -t / --threads N,
             --alpha-y=A, --alpha-z=A (Gourdon's y = A x^(1/3), z = A y for pi(x))

Numbers are integer expressions as the reference's calculator accepts them:
1e20, 10^20, 2^64-1, 10**18 + 7 (integers only).  The result is printed on
the last line, alone, as the reference prints it.
"""
import ast
import re
import sys
import time

import primecount_gb300 as pcg


def parse_number(s):
    """Exact integer value of an expression such as 1e20, 10^18, 2**64-1."""
    t = s.strip().replace("^", "**")
    t = re.sub(r"(\d+)[eE](\d+)", r"(\1*10**\2)", t)
    node = ast.parse(t, mode="eval").body

    def ev(n):
        if isinstance(n, ast.Constant) and isinstance(n.value, int):
            return n.value
        if isinstance(n, ast.UnaryOp) and isinstance(n.op, (ast.USub, ast.UAdd)):
            v = ev(n.operand)
            return -v if isinstance(n.op, ast.USub) else v
        if isinstance(n, ast.BinOp):
            a, b = ev(n.left), ev(n.right)
            if isinstance(n.op, ast.Add):
                return a + b
            if isinstance(n.op, ast.Sub):
                return a - b
            if isinstance(n.op, ast.Mult):
                return a * b
            if isinstance(n.op, ast.FloorDiv) or isinstance(n.op, ast.Div):
                return a // b
            if isinstance(n.op, ast.Pow) and 0 <= b <= 256:
                return a ** b
        raise ValueError("invalid number: %s" % s)

    return ev(node)


OPTIONS = {"--D": "D", "-D": "D", "--S2-hard": "S2_hard", "--AC": "AC", "--B": "B", "-B": "B",
           "--Phi0": "Phi0", "--Sigma": "Sigma", "--phi": "phi", "-g": "pi", "--gourdon": "pi",
           "-d": "dr", "--deleglise-rivat": "dr", "--S1": "S1", "--S2-trivial": "S2_trivial",
           "--S2-easy": "S2_easy", "--P2": "P2"}
DR_TERMS = ("S1", "S2_trivial", "S2_easy", "P2")


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    numbers, option, status, timing, threads = [], "pi", False, False, 0
    alpha_y = alpha_z = 0.0
    i = 0
    while i < len(argv):
        a = argv[i]
        if a in OPTIONS:
            option = OPTIONS[a]
        elif a in ("-s", "--status"):
            status = True
        elif a == "--time":
            timing = True
        elif a in ("-t", "--threads"):
            i += 1
            threads = int(argv[i])
        elif a.startswith("--threads="):
            threads = int(a.split("=", 1)[1])
        elif a.startswith("--alpha-y="):
            alpha_y = float(a.split("=", 1)[1])
        elif a.startswith("--alpha-z="):
            alpha_z = float(a.split("=", 1)[1])
        elif a in ("-h", "--help"):
            print(__doc__)
            return 0
        else:
            numbers.append(parse_number(a))
        i += 1
    if option == "phi":
        if len(numbers) != 2:
            raise pcg.PrimecountError(1, "option --phi requires 2 numbers")
    elif len(numbers) != 1:
        raise pcg.PrimecountError(1, "missing x number" if not numbers else
                                  "expected 1 input number, but found %d" % len(numbers))
    x = numbers[0]
    t0 = time.perf_counter()
    if option == "D":
        p = pcg.gourdon_params(x)
        if status:
            print("x = %d\ny = %d\nz = %d\nk = %d\nx_star = %d" % (x, p["y"], p["z"], p["k"], p["x_star"]))
        r = pcg.D(x, p["y"], p["z"], p["k"], threads=threads)
    elif option == "S2_hard":
        p = pcg.dr_params(x)
        if status:
            print("x = %d\ny = %d\nz = %d\nc = %d" % (x, p["y"], p["z"], p["c"]))
        r = pcg.S2_hard(x, p["y"], p["z"], p["c"], threads=threads)
    elif option == "phi":
        r = pcg.phi(x, numbers[1], threads=threads)
    elif option == "pi":
        if status and x > 10 ** 10:
            p = pcg.gourdon_params(x)
            print("x = %d\ny = %d\nz = %d\nk = %d\nx_star = %d" % (x, p["y"], p["z"], p["k"], p["x_star"]))
        r = pcg.pi(x, threads=threads, alpha_y=alpha_y, alpha_z=alpha_z)
    elif option == "dr":
        if status and x > 10 ** 10:
            p = pcg.dr_params(x)
            print("x = %d\ny = %d\nz = %d\nc = %d" % (x, p["y"], p["z"], p["c"]))
        r = pcg.pi_deleglise_rivat(x, threads=threads)
    elif option in DR_TERMS:
        if x <= 10 ** 10:
            raise pcg.PrimecountError(1, "--%s: the formula terms are computed for x > 1e10" % option.replace("_", "-"))
        if status:
            p = pcg.dr_params(x)
            print("x = %d\ny = %d\nz = %d\nc = %d" % (x, p["y"], p["z"], p["c"]))
        r = pcg.pi_dr_terms(x)[option]
    else:
        if x <= 10 ** 10:
            raise pcg.PrimecountError(1, "--%s: the formula terms are computed for x > 1e10" % option)
        if status:
            p = pcg.gourdon_params(x)
            print("x = %d\ny = %d\nz = %d\nk = %d\nx_star = %d" % (x, p["y"], p["z"], p["k"], p["x_star"]))
        r = pcg.pi_terms(x, alpha_y=alpha_y, alpha_z=alpha_z)[option]
    dt = time.perf_counter() - t0
    if status:
        st = pcg.last_stats()
        print("Status: leaves = %d, segments = %d, kernel launches = %d" %
              (st["leaves"], st["segments"], st["kernel_launches"]))
    print(r)
    if timing:
        print("Seconds: %.3f" % dt)
    return 0


if __name__ == "__main__":
    try:
        sys.exit(main())
    except pcg.PrimecountError as e:
        print("Error: %s" % e, file=sys.stderr)
        sys.exit(1)
