"""GPU: the allocation-free entry point pcg_D_noalloc against pcg_D.

pcg_D_noalloc serves callers that cannot allocate device memory at the
moment they need D(x, y, z, k): a serving request path that must not touch
the allocator, or a process whose device memory belongs to another
framework's pool.  It reads the tables of a context built beforehand (set-up
time, when allocating is allowed) and keeps all of its working memory in one
static device array inside libpcgpu.so.

This file sorts last so that, if it fails, a run stopping at the first
failure has already run every other test.  It needs nothing from the other
tests and passes alone in a fresh process.
"""
import ctypes
import os

import pytest

pytestmark = pytest.mark.gpu


def _bind(pcg):
    L = pcg.load()
    L.pcg_D_noalloc.argtypes = [ctypes.c_void_p, pcg.I128, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                ctypes.c_void_p, ctypes.POINTER(pcg.I128)]
    L.pcg_D_noalloc.restype = ctypes.c_int
    return L


def _cudart():
    """The CUDA runtime, for cudaMemGetInfo (free device memory is a property
    of the device, whichever runtime copy asks)."""
    import glob
    cands = ["libcudart.so", "libcudart.so.13", "libcudart.so.12"]
    cands += sorted(glob.glob("/usr/local/cuda/lib64/libcudart.so*"))
    try:
        import torch
        cands += sorted(glob.glob(os.path.join(os.path.dirname(torch.__file__), "lib", "libcudart*.so*")))
    except Exception:
        pass
    for c in cands:
        try:
            lib = ctypes.CDLL(c)
            lib.cudaMemGetInfo.argtypes = [ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)]
            return lib
        except OSError:
            continue
    return None


def _free_device_bytes(rt):
    free, total = ctypes.c_size_t(), ctypes.c_size_t()
    assert rt.cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total)) == 0
    return free.value


def test_noalloc_matches_pcg_D_on_two_calls(pcg):
    L = _bind(pcg)
    ctx = pcg.Context(10 ** 17)          # resident tables: built here, allocation allowed
    try:
        for x in (10 ** 12, 10 ** 14, 1234567890123456, 10 ** 17):
            p = pcg.gourdon_params(x)
            want = pcg.D(x, p["y"], p["z"], p["k"])          # the existing entry point
            for _ in range(2):                                 # two calls in a row share the scratch
                out = pcg.I128()
                st = L.pcg_D_noalloc(ctx._h, pcg.to_i128(x), p["y"], p["z"], p["k"], None, ctypes.byref(out))
                assert st == 0, L.pcg_last_error(ctx._h)
                assert pcg.from_i128(out) == want, x           # integers: bit-exact
    finally:
        ctx.close()


def test_noalloc_allocates_no_device_memory(pcg):
    L = _bind(pcg)
    rt = _cudart()
    if rt is None:
        pytest.skip("no CUDA runtime library to read the free device memory with")
    ctx = pcg.Context(10 ** 16)
    try:
        x = 10 ** 16
        p = pcg.gourdon_params(x)
        out = pcg.I128()
        # the first call on the device resolves the scratch address (and may
        # load the module); the second one is measured
        assert L.pcg_D_noalloc(ctx._h, pcg.to_i128(x), p["y"], p["z"], p["k"], None, ctypes.byref(out)) == 0
        before = _free_device_bytes(rt)
        out2 = pcg.I128()
        assert L.pcg_D_noalloc(ctx._h, pcg.to_i128(x), p["y"], p["z"], p["k"], None, ctypes.byref(out2)) == 0
        after = _free_device_bytes(rt)
        assert pcg.from_i128(out2) == pcg.from_i128(out) == 257656447322004
        assert abs(before - after) < (1 << 20)
    finally:
        ctx.close()


def test_noalloc_rejects_uncovered_tables(pcg):
    L = _bind(pcg)
    ctx = pcg.Context(10 ** 12)
    try:
        x = 10 ** 16
        p = pcg.gourdon_params(x)
        out = pcg.I128()
        st = L.pcg_D_noalloc(ctx._h, pcg.to_i128(x), p["y"], p["z"], p["k"], None, ctypes.byref(out))
        assert st == 2  # PCG_ERANGE: the context's tables do not cover y, z
        assert b"do not cover" in L.pcg_last_error(ctx._h)
    finally:
        ctx.close()
