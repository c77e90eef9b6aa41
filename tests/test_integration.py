"""The drop-in on the reference's side: primecount's own test programs for
the hard leaves (test/gourdon/D.cpp, test/deleglise-rivat/S2_hard_alpha.cpp,
test/gourdon/pi_gourdon.cpp) built against the reference's headers and
library with D() and S2_hard() replaced by primecount_gb300/integration/
hard_leaves_gpu.cpp, which calls libpcgpu (oracle/ref.mk, target itest).

CPU: the programs build, and pass on the reference's own bodies (the stub's
fallback when no GPU is present).  GPU: they pass with PCG_REQUIRE=1, every
D / S2_hard call computed by the engine."""
import os
import platform
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ITEST = os.path.join(ROOT, "oracle", "_ref", platform.machine(), "itest")


def build_itest(pcg):
    import __graft_entry__ as g
    ref = g.reference_tree()
    if ref is None:
        pytest.skip("no primecount source tree (PCG_REFERENCE or the staged oracle/_ref/src)")
    if not os.path.isfile(os.path.join(ref, "test", "gourdon", "D.cpp")):
        pytest.skip("the source tree has no test programs")
    r = subprocess.run(["make", "-f", os.path.join(ROOT, "oracle", "ref.mk"), "REF=" + ref, "PCGPU=" + ROOT,
                        "OUT=" + os.path.dirname(ITEST), "itest", "-j%d" % max(2, min(16, os.cpu_count() or 2))],
                       cwd=ROOT, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def run(prog, env_extra, timeout=900):
    env = dict(os.environ, **env_extra)
    r = subprocess.run([os.path.join(ITEST, prog)], capture_output=True, text=True, env=env, timeout=timeout)
    assert r.returncode == 0, (prog, r.stdout[-2000:], r.stderr[-2000:])
    assert "All tests passed successfully!" in r.stdout
    return r.stdout


def test_reference_D_program_builds_and_falls_back(pcg):
    build_itest(pcg)
    out = run("test_D", {"PCG_DISABLE": "1"})
    assert out.count("OK") >= 100                  # 51 tuples, 64- and 128-bit


@pytest.mark.gpu
def test_reference_programs_on_the_gpu(pcg):
    build_itest(pcg)
    env = {"PCG_REQUIRE": "1"}
    assert run("test_D", env).count("OK") >= 100
    run("test_S2_hard_alpha", env)
    run("test_pi_gourdon", env)
