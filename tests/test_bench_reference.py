"""bench.py's reference arm on the CPU: it times the reference's own D(x)
(its CLI built by oracle/ref.mk) and imports nothing of primecount_gb300, so
that no code of this engine runs in the arm the engine is compared with."""
import json
import os
import platform
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_BIN = os.path.join(ROOT, "oracle", "_ref", platform.machine(), "primecount")


@pytest.mark.skipif(not os.access(REF_BIN, os.X_OK), reason="the reference is not built on this host")
def test_reference_arm_runs_the_reference_without_the_engine():
    # primecount_gb300 made unimportable: the arm must not need it
    code = ("import sys, runpy; sys.modules['primecount_gb300'] = None; "
            "sys.argv = ['bench.py', '--impl', 'reference', '--x', '1e14', '--steps', '1', '--warmup', '1']; "
            "runpy.run_path(%r, run_name='__main__')" % os.path.join(ROOT, "bench.py"))
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["cpu_baseline"]["kind"] == "reference"
    assert line["result"] == "2876480095175"          # the reference's D(1e14) at its default parameters
    assert line["value"] > 0 and line["e2e"]["h2d_bytes_per_step"] == 0
