"""CPU: the C-ABI library loads, exports every symbol of include/pcgpu.h,
and fails loudly (no CPU fallback) when no GPU is present."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    src = open(os.path.join(ROOT, "include", "pcgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b((?:pcg|primecount)_[A-Za-z0-9_]+)\s*\(", src)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = header_symbols()
    for n in ("pcg_D", "pcg_S2_hard", "pcg_pi", "pcg_phi", "pcg_pi_batch", "pcg_phi_batch",
              "pcg_ctx_create", "pcg_ctx_destroy", "pcg_last_error", "primecount_pi"):
        assert n in names


def test_library_exports_every_symbol(pcg):
    out = subprocess.run(["nm", "-D", "--defined-only", pcg.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(l.split()[-1] for l in out.splitlines() if " T " in l)
    missing = [n for n in header_symbols() if n not in exported]
    assert not missing, missing
    L = ctypes.CDLL(pcg.LIB_PATH)
    for n in header_symbols():
        assert hasattr(L, n)


def test_library_links_no_oracle(pcg):
    out = subprocess.run(["nm", "-D", pcg.LIB_PATH], capture_output=True, text=True).stdout
    assert "ora_" not in out
    ldd = subprocess.run(["ldd", pcg.LIB_PATH], capture_output=True, text=True).stdout
    assert "liboracle" not in ldd


def test_params_host_logic(pcg, golden):
    # y, z, k selection is host logic (src/util.cpp:276-386) and needs no GPU
    for xs, row in golden["D_default"].items():
        p = pcg.gourdon_params(int(xs))
        assert (p["y"], p["z"], p["k"]) == (row["y"], row["z"], row["k"])
    for x, y, z, k, _ in golden["D_random"]:
        p = pcg.gourdon_params(x)
        assert (p["y"], p["z"], p["k"]) == (y, z, k), x
    for xs, row in golden["S2_hard_default"].items():
        p = pcg.dr_params(int(xs))
        assert (p["y"], p["z"], p["c"]) == (row["y"], row["z"], row["c"])
    for x, y, z, c, _ in golden["S2_hard_random"]:
        p = pcg.dr_params(x)
        assert (p["y"], p["z"], p["c"]) == (y, z, c), x


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-GPU error path")
def test_no_gpu_fails_loudly(pcg):
    with pytest.raises(pcg.PrimecountError) as e:
        pcg.D(10 ** 12, 10001, 10001, 8)
    assert e.value.status == 5  # PCG_ENODEV
    assert pcg.load().primecount_pi(10 ** 12) == -1


def test_invalid_arguments_rejected_before_launch(pcg):
    # negative x, y < 1: rejected on the host, status EINVAL (no device work)
    with pytest.raises(pcg.PrimecountError) as e:
        pcg.gourdon_params(-5)
    assert e.value.status == 1
