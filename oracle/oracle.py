"""ctypes binding of the CPU oracle (oracle/pcg_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg as the checker.  The product (libpcgpu.so,
primecount_gb300) never imports it.
"""
import ctypes
import os
import subprocess
import shutil

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")


class Stats(ctypes.Structure):
    _fields_ = [("leaves", ctypes.c_int64), ("two_prime_leaves", ctypes.c_int64),
                ("indices_scanned", ctypes.c_int64)]


_lib = None


def build():
    cc = shutil.which("gcc") or shutil.which("cc")
    tmp = LIB + ".tmp"
    subprocess.run([cc, "-O2", "-fopenmp", "-shared", "-fPIC", os.path.join(HERE, "pcg_oracle.c"),
                    "-o", tmp, "-lm"], check=True)
    os.replace(tmp, LIB)


def load():
    global _lib
    if _lib is None:
        src = os.path.join(HERE, "pcg_oracle.c")
        if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
            build()
        L = ctypes.CDLL(LIB)
        i64, u64 = ctypes.c_int64, ctypes.c_uint64
        for fn in (L.ora_D, L.ora_S2_hard):
            fn.argtypes = [u64, i64, i64, i64, i64, ctypes.c_int, ctypes.POINTER(u64), ctypes.POINTER(i64),
                           ctypes.POINTER(Stats)]
            fn.restype = ctypes.c_int
        L.ora_D_sample.argtypes = [u64, i64, i64, i64, i64, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                   ctypes.POINTER(i64), ctypes.POINTER(ctypes.c_double)]
        L.ora_D_sample.restype = ctypes.c_int
        L.ora_D_partial.argtypes = [u64, i64, i64, i64, i64, i64, i64, ctypes.POINTER(u64), ctypes.POINTER(i64),
                                    ctypes.POINTER(i64), ctypes.POINTER(i64), i64]
        L.ora_D_partial.restype = ctypes.c_int
        L.ora_phi.argtypes = [i64, i64]
        L.ora_phi.restype = i64
        L.ora_pi_sieve.argtypes = [i64]
        L.ora_pi_sieve.restype = i64
        L.ora_factor_size.argtypes = [i64]
        L.ora_factor_size.restype = i64
        L.ora_factor_table_d16.argtypes = [i64, i64, ctypes.POINTER(ctypes.c_uint16)]
        L.ora_factor_table_dr16.argtypes = [i64, ctypes.POINTER(ctypes.c_uint16)]
        L.ora_pi_table.argtypes = [i64, ctypes.POINTER(u64)]
        L.ora_gourdon_params.argtypes = [u64, i64, ctypes.c_double, ctypes.c_double] + [ctypes.POINTER(i64)] * 4
        L.ora_gourdon_params.restype = None
        L.ora_dr_params.argtypes = [u64, i64, ctypes.c_double] + [ctypes.POINTER(i64)] * 3
        L.ora_dr_params.restype = None
        _lib = L
    return _lib


def _hard(fn, x, y, z, k, threads):
    lo, hi, st = ctypes.c_uint64(), ctypes.c_int64(), Stats()
    rc = fn(x & 0xFFFFFFFFFFFFFFFF, x >> 64, y, z, k, threads, ctypes.byref(lo), ctypes.byref(hi), ctypes.byref(st))
    if rc != 0:
        raise ValueError("oracle rejected the arguments (%d)" % rc)
    return (hi.value << 64) | lo.value, {"leaves": st.leaves, "two_prime_leaves": st.two_prime_leaves,
                                         "indices_scanned": st.indices_scanned}


def D(x, y, z, k, threads=1):
    """(D(x, y, z, k), work counters) -- restatement of src/gourdon/D.cpp."""
    return _hard(load().ora_D, x, y, z, k, threads)


def S2_hard(x, y, z, c, threads=1):
    """(S2_hard(x, y, z, c), work counters) -- restatement of S2_hard.cpp."""
    return _hard(load().ora_S2_hard, x, y, z, c, threads)


def D_sample(x, y, z, k, nchunks, fraction, threads):
    """(leaves, seconds) of the reference's chunk loop on a sample of D's interval."""
    leaves, secs = ctypes.c_int64(), ctypes.c_double()
    load().ora_D_sample(x & 0xFFFFFFFFFFFFFFFF, x >> 64, y, z, k, nchunks, fraction, threads,
                        ctypes.byref(leaves), ctypes.byref(secs))
    return leaves.value, secs.value


def D_partial(x, y, z, k, lo, hi, ncols):
    """(leaf sum, msum, csum) of the shard [lo, hi) of D with phi offsets
    counted from lo (the per-shard partials of the multi-GPU split)."""
    lo_, hi_ = ctypes.c_uint64(), ctypes.c_int64()
    ms = (ctypes.c_int64 * ncols)()
    cs = (ctypes.c_int64 * ncols)()
    rc = load().ora_D_partial(x & 0xFFFFFFFFFFFFFFFF, x >> 64, y, z, k, lo, hi, ctypes.byref(lo_),
                              ctypes.byref(hi_), ms, cs, ncols)
    if rc != 0:
        raise ValueError("oracle rejected the arguments (%d)" % rc)
    s = (hi_.value << 64) | lo_.value
    if s >= 1 << 127:
        s -= 1 << 128
    return s, list(ms), list(cs)


def phi(x, a):
    return load().ora_phi(x, a)


def pi_sieve(x):
    return load().ora_pi_sieve(x)


def factor_table_d16(y, z):
    n = load().ora_factor_size(z)
    buf = (ctypes.c_uint16 * n)()
    if load().ora_factor_table_d16(y, z, buf) != 0:
        raise ValueError("z too large")
    return list(buf)


def factor_table_dr16(y):
    n = load().ora_factor_size(y)
    buf = (ctypes.c_uint16 * n)()
    load().ora_factor_table_dr16(y, buf)
    return list(buf)


def pi_table(max_x):
    n = 2 * (max_x // 240 + 1)
    buf = (ctypes.c_uint64 * n)()
    load().ora_pi_table(max_x, buf)
    return list(buf)


def gourdon_params(x):
    y, z, k, xs = (ctypes.c_int64() for _ in range(4))
    load().ora_gourdon_params(x & 0xFFFFFFFFFFFFFFFF, x >> 64, -1.0, -1.0, ctypes.byref(y), ctypes.byref(z),
                              ctypes.byref(k), ctypes.byref(xs))
    return {"y": y.value, "z": z.value, "k": k.value, "x_star": xs.value}


def dr_params(x):
    y, z, c = (ctypes.c_int64() for _ in range(3))
    load().ora_dr_params(x & 0xFFFFFFFFFFFFFFFF, x >> 64, -1.0, ctypes.byref(y), ctypes.byref(z), ctypes.byref(c))
    return {"y": y.value, "z": z.value, "c": c.value}
