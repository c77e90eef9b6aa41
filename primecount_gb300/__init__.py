"""primecount_gb300 -- Python mirror of the GB300 hard-special-leaf engine.

The compute lives in libpcgpu.so (CUDA, sm_103a) behind the C ABI of
include/pcgpu.h; this module binds it with ctypes and mirrors the
reference's interface (kimwalisch/primecount 8.7, include/primecount.hpp and
the internal formula functions of include/gourdon.hpp / include/S.hpp):

    pi(x), phi(x, a)                      primecount::pi / primecount::phi
    D(x, y, z, k), S2_hard(x, y, z, c)    internal formula functions
    D_default(x), S2_hard_default(x)      the --D / --S2-hard CLI options
    pi_batch(xs), phi_batch(xs, as)       many queries per call (new)
    Context(max_x)                        device-resident tables (new)

Errors raise PrimecountError (the reference's primecount_error).  There is
no CPU fallback: without the CUDA library or a GPU every call raises.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libpcgpu.so")

PCG_OK = 0
STATUS = {0: "PCG_OK", 1: "PCG_EINVAL", 2: "PCG_ERANGE", 3: "PCG_ENOMEM", 4: "PCG_ECUDA",
          5: "PCG_ENODEV", 6: "PCG_ETIMEOUT", 7: "PCG_ECANCELLED", 8: "PCG_EINTERNAL",
          9: "PCG_EAGAIN"}   # 9: refused by the serving loop's latency budget (no C status)


class PrimecountError(RuntimeError):
    """Mirror of the reference's primecount_error; .status holds the pcg_status."""

    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS.get(status, status), msg))
        self.status = status


class I128(ctypes.Structure):
    _fields_ = [("lo", ctypes.c_uint64), ("hi", ctypes.c_int64)]


class Opts(ctypes.Structure):
    _fields_ = [("ctx", ctypes.c_void_p), ("stream", ctypes.c_void_p), ("threads", ctypes.c_int),
                ("print", ctypes.c_int), ("segment_words", ctypes.c_int), ("ctas_per_sm", ctypes.c_int),
                ("cta_threads", ctypes.c_int), ("alpha_y", ctypes.c_double), ("alpha_z", ctypes.c_double),
                ("checkpoint", ctypes.c_char_p), ("checkpoint_interval", ctypes.c_double),
                ("stop_after_waves", ctypes.c_int)]


class Tuning(ctypes.Structure):
    _fields_ = [("segment_words", ctypes.c_int), ("ctas_per_sm", ctypes.c_int), ("cta_threads", ctypes.c_int),
                ("group", ctypes.c_int), ("ms", ctypes.c_double)]


class Stats(ctypes.Structure):
    _fields_ = [("leaves", ctypes.c_uint64), ("two_prime_leaves", ctypes.c_uint64),
                ("segments", ctypes.c_uint64), ("levels", ctypes.c_uint64),
                ("factor_entries", ctypes.c_uint64), ("kernel_launches", ctypes.c_uint64),
                ("table_ms", ctypes.c_double), ("sweep_ms", ctypes.c_double),
                ("combine_ms", ctypes.c_double), ("total_ms", ctypes.c_double),
                ("sweep_kernel_ms", ctypes.c_double), ("sweep_launches", ctypes.c_uint64),
                ("h2d_bytes", ctypes.c_uint64), ("d2h_bytes", ctypes.c_uint64),
                ("segment_words", ctypes.c_int), ("ctas_per_sm", ctypes.c_int),
                ("threads_per_cta", ctypes.c_int), ("ac_ms", ctypes.c_double), ("b_ms", ctypes.c_double),
                ("phi0_ms", ctypes.c_double), ("sigma_ms", ctypes.c_double), ("d_ms", ctypes.c_double),
                ("crossoff_multiples", ctypes.c_uint64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def to_i128(v):
    v = int(v)
    return I128(v & 0xFFFFFFFFFFFFFFFF, v >> 64)


def from_i128(r):
    return (int(r.hi) << 64) | int(r.lo)


_lib = None


def load(path=None):
    """Load libpcgpu.so (raises PrimecountError if it was not built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise PrimecountError(5, "libpcgpu.so not built (python -m primecount_gb300.build): %s" % p)
    L = ctypes.CDLL(p)
    c_i64, c_p = ctypes.c_int64, ctypes.POINTER
    L.pcg_D.argtypes = [I128, c_i64, c_i64, c_i64, c_p(Opts), c_p(I128)]
    L.pcg_S2_hard.argtypes = [I128, c_i64, c_i64, c_i64, c_p(Opts), c_p(I128)]
    L.pcg_D_default.argtypes = [I128, c_p(Opts), c_p(I128), c_p(c_i64), c_p(c_i64), c_p(c_i64)]
    L.pcg_S2_hard_default.argtypes = [I128, c_p(Opts), c_p(I128), c_p(c_i64), c_p(c_i64), c_p(c_i64)]
    L.pcg_gourdon_params.argtypes = [I128, c_p(c_i64), c_p(c_i64), c_p(c_i64), c_p(c_i64)]
    L.pcg_dr_params.argtypes = [I128, c_p(c_i64), c_p(c_i64), c_p(c_i64)]
    L.pcg_pi.argtypes = [I128, c_p(Opts), c_p(I128)]
    L.pcg_phi.argtypes = [c_i64, c_i64, c_p(Opts), c_p(c_i64)]
    L.pcg_pi_terms.argtypes = [I128, c_p(Opts), c_p(I128)]
    L.pcg_pi_terms.restype = ctypes.c_int
    L.pcg_pi_deleglise_rivat.argtypes = [I128, c_p(Opts), c_p(I128)]
    L.pcg_pi_deleglise_rivat.restype = ctypes.c_int
    L.pcg_pi_dr_terms.argtypes = [I128, c_p(Opts), c_p(I128)]
    L.pcg_pi_dr_terms.restype = ctypes.c_int
    L.pcg_pi_batch.argtypes = [c_p(I128), ctypes.c_size_t, c_p(I128), c_p(Opts)]
    L.pcg_phi_batch.argtypes = [c_p(c_i64), c_p(c_i64), ctypes.c_size_t, c_p(c_i64), c_p(Opts)]
    L.pcg_ctx_create.argtypes = [I128, ctypes.c_uint64, c_p(ctypes.c_void_p)]
    L.pcg_ctx_destroy.argtypes = [ctypes.c_void_p]
    L.pcg_ctx_destroy.restype = None
    L.pcg_last_error.argtypes = [ctypes.c_void_p]
    L.pcg_last_error.restype = ctypes.c_char_p
    L.pcg_last_stats.argtypes = [ctypes.c_void_p, c_p(Stats)]
    L.pcg_ctx_device_bytes.argtypes = [ctypes.c_void_p]
    L.pcg_ctx_device_bytes.restype = ctypes.c_uint64
    L.primecount_pi.argtypes = [c_i64]
    L.primecount_pi.restype = c_i64
    L.primecount_pi_128.argtypes = [I128]
    L.primecount_pi_128.restype = I128
    L.primecount_phi.argtypes = [c_i64, c_i64]
    L.primecount_phi.restype = c_i64
    L.primecount_version.restype = ctypes.c_char_p
    shard_args = [I128, c_i64, c_i64, c_i64, ctypes.c_int, ctypes.c_int, c_p(Opts), c_p(I128), c_p(c_i64),
                  c_p(c_i64), c_i64, c_p(c_i64)]
    L.pcg_D_shard.argtypes = shard_args
    L.pcg_S2_hard_shard.argtypes = shard_args
    L.pcg_shard_combine.argtypes = [ctypes.c_int, c_i64, c_p(I128), c_p(c_i64), c_p(c_i64), c_p(I128)]
    L.pcg_ctx_read_table.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64,
                                     ctypes.c_void_p, c_p(ctypes.c_uint64), c_p(ctypes.c_int), c_p(c_i64)]
    L.pcg_ctx_read_table.restype = ctypes.c_int
    L.pcg_query_device_bytes.argtypes = [ctypes.c_void_p, ctypes.c_int, I128, c_i64, c_p(ctypes.c_uint64)]
    L.pcg_query_device_bytes.restype = ctypes.c_int
    L.pcg_ctx_trim.argtypes = [ctypes.c_void_p, c_p(ctypes.c_uint64)]
    L.pcg_ctx_trim.restype = ctypes.c_int
    L.pcg_device_memory.argtypes = [c_p(ctypes.c_uint64), c_p(ctypes.c_uint64)]
    L.pcg_device_memory.restype = ctypes.c_int
    L.pcg_autotune.argtypes = [I128, c_p(Opts), c_p(Tuning)]
    L.pcg_autotune.restype = ctypes.c_int
    for name in ("pcg_D", "pcg_S2_hard", "pcg_D_default", "pcg_S2_hard_default", "pcg_gourdon_params",
                 "pcg_dr_params", "pcg_pi", "pcg_phi", "pcg_pi_batch", "pcg_phi_batch", "pcg_ctx_create",
                 "pcg_last_stats", "pcg_D_shard", "pcg_S2_hard_shard", "pcg_shard_combine"):
        getattr(L, name).restype = ctypes.c_int
    if path is None:
        _lib = L
    return L


def _check(st, ctx=None):
    if st != PCG_OK:
        L = load()
        msg = L.pcg_last_error(ctx._h if ctx is not None else None)
        raise PrimecountError(st, (msg or b"").decode())


class Context:
    """Device-resident primes / PiTable / FactorTable sized for x <= max_x."""

    def __init__(self, max_x=0, mem_budget=0):
        L = load()
        h = ctypes.c_void_p()
        st = L.pcg_ctx_create(to_i128(max_x), int(mem_budget), ctypes.byref(h))
        if st != PCG_OK:
            raise PrimecountError(st, (L.pcg_last_error(None) or b"").decode())
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            load().pcg_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def device_bytes(self):
        return int(load().pcg_ctx_device_bytes(self._h))

    def last_stats(self):
        s = Stats()
        _check(load().pcg_last_stats(self._h, ctypes.byref(s)), self)
        return s.as_dict()

    def trim(self):
        """Free the per-call working memory kept between calls (pcg_ctx_trim);
        the resident tables stay.  Returns the bytes released."""
        f = ctypes.c_uint64()
        _check(load().pcg_ctx_trim(self._h, ctypes.byref(f)), self)
        return f.value

    TABLES = {"primes": 0, "pi": 1, "factor_d": 2, "factor_dr": 3}

    def table_info(self, name):
        """(entries, entry bytes, largest number covered) of a resident table."""
        n, eb, lim = ctypes.c_uint64(), ctypes.c_int(), ctypes.c_int64()
        _check(load().pcg_ctx_read_table(self._h, self.TABLES[name], 0, 0, None, ctypes.byref(n), ctypes.byref(eb),
                                         ctypes.byref(lim)), self)
        return n.value, eb.value, lim.value

    def read_table(self, name, first=0, count=None):
        """Entries [first, first + count) of a resident table as a numpy array
        (pcg_ctx_read_table): "primes", "pi", "factor_d" or "factor_dr"."""
        import numpy as np
        n, eb, _ = self.table_info(name)
        if count is None:
            count = n - first
        arr = np.empty(count, dtype={2: np.uint16, 4: np.uint32, 8: np.uint64}[eb])
        if count:
            _check(load().pcg_ctx_read_table(self._h, self.TABLES[name], first, count, arr.ctypes.data_as(ctypes.c_void_p),
                                             None, None, None), self)
        return arr


def _opts(ctx=None, stream=None, threads=0, print_=False, segment_words=0, ctas_per_sm=0, cta_threads=0,
          alpha_y=0.0, alpha_z=0.0, checkpoint=None, checkpoint_interval=0.0, stop_after_waves=0):
    o = Opts()
    o.alpha_y = alpha_y
    o.alpha_z = alpha_z
    o.checkpoint = os.fsencode(checkpoint) if checkpoint else None
    o.checkpoint_interval = checkpoint_interval
    o.stop_after_waves = stop_after_waves
    o.ctx = ctx._h if ctx is not None else None
    o.stream = stream
    o.threads = threads
    o.print = 1 if print_ else 0
    o.segment_words = segment_words
    o.ctas_per_sm = ctas_per_sm
    o.cta_threads = cta_threads
    return o


def last_stats(ctx=None):
    s = Stats()
    _check(load().pcg_last_stats(ctx._h if ctx is not None else None, ctypes.byref(s)), ctx)
    return s.as_dict()


def D(x, y, z, k, threads=0, print=False, ctx=None, stream=None, segment_words=0, ctas_per_sm=0, cta_threads=0,
      checkpoint=None, checkpoint_interval=0.0, stop_after_waves=0):
    """Gourdon's D(x, y, z, k): the hard special leaves (src/gourdon/D.cpp).
    checkpoint: file to resume from / save to (see pcg_opts in pcgpu.h)."""
    out = I128()
    o = _opts(ctx, stream, threads, print, segment_words, ctas_per_sm, cta_threads,
              checkpoint=checkpoint, checkpoint_interval=checkpoint_interval, stop_after_waves=stop_after_waves)
    _check(load().pcg_D(to_i128(x), int(y), int(z), int(k), ctypes.byref(o), ctypes.byref(out)), ctx)
    return from_i128(out)


def S2_hard(x, y, z, c, threads=0, print=False, ctx=None, stream=None, segment_words=0, ctas_per_sm=0,
            cta_threads=0, checkpoint=None, checkpoint_interval=0.0, stop_after_waves=0):
    """Deleglise-Rivat's S2_hard(x, y, z, c) (src/deleglise-rivat/S2_hard.cpp)."""
    out = I128()
    o = _opts(ctx, stream, threads, print, segment_words, ctas_per_sm, cta_threads,
              checkpoint=checkpoint, checkpoint_interval=checkpoint_interval, stop_after_waves=stop_after_waves)
    _check(load().pcg_S2_hard(to_i128(x), int(y), int(z), int(c), ctypes.byref(o), ctypes.byref(out)), ctx)
    return from_i128(out)


def gourdon_params(x):
    y, z, k, xs = (ctypes.c_int64() for _ in range(4))
    _check(load().pcg_gourdon_params(to_i128(x), ctypes.byref(y), ctypes.byref(z), ctypes.byref(k),
                                     ctypes.byref(xs)))
    return {"y": y.value, "z": z.value, "k": k.value, "x_star": xs.value}


def dr_params(x):
    y, z, c = (ctypes.c_int64() for _ in range(3))
    _check(load().pcg_dr_params(to_i128(x), ctypes.byref(y), ctypes.byref(z), ctypes.byref(c)))
    return {"y": y.value, "z": z.value, "c": c.value}


def D_default(x, **kw):
    """D(x) with the reference's default y, z, k (the --D option)."""
    p = gourdon_params(x)
    return D(x, p["y"], p["z"], p["k"], **kw)


def S2_hard_default(x, **kw):
    """S2_hard(x) with the reference's default y, z, c (the --S2-hard option)."""
    p = dr_params(x)
    return S2_hard(x, p["y"], p["z"], p["c"], **kw)


def pi(x, threads=0, print=False, ctx=None, stream=None, alpha_y=0.0, alpha_z=0.0):
    """Number of primes <= x (primecount::pi); alpha_y / alpha_z tune
    Gourdon's y and z (the reference's --alpha-y / --alpha-z)."""
    out = I128()
    o = _opts(ctx, stream, threads, print, alpha_y=alpha_y, alpha_z=alpha_z)
    _check(load().pcg_pi(to_i128(x), ctypes.byref(o), ctypes.byref(out)), ctx)
    return from_i128(out)


def pi_terms(x, ctx=None, stream=None, alpha_y=0.0, alpha_z=0.0):
    """The terms of Gourdon's formula for x > 1e10 (the reference's --AC, --B,
    --D, --Phi0, --Sigma options): dict with AC, B, D, Phi0, Sigma and pi."""
    out = (I128 * 6)()
    o = _opts(ctx, stream, alpha_y=alpha_y, alpha_z=alpha_z)
    _check(load().pcg_pi_terms(to_i128(x), ctypes.byref(o), out), ctx)
    v = [from_i128(t) for t in out]
    return dict(zip(("AC", "B", "D", "Phi0", "Sigma", "pi"), v))


def pi_deleglise_rivat(x, threads=0, print=False, ctx=None, stream=None):
    """Number of primes <= x by the Deleglise-Rivat formula (the reference's
    pi_deleglise_rivat, option -d): S2_hard on the engine, the other terms on
    the device as well."""
    out = I128()
    o = _opts(ctx, stream, threads, print)
    _check(load().pcg_pi_deleglise_rivat(to_i128(x), ctypes.byref(o), ctypes.byref(out)), ctx)
    return from_i128(out)


def pi_dr_terms(x, ctx=None, stream=None):
    """The terms of the Deleglise-Rivat formula for x > 1e10 (the reference's
    --S1, --S2-trivial, --S2-easy, --S2-hard, --P2 options): dict with S1,
    S2_trivial, S2_easy, S2_hard, P2, pi_y and pi."""
    out = (I128 * 7)()
    o = _opts(ctx, stream)
    _check(load().pcg_pi_dr_terms(to_i128(x), ctypes.byref(o), out), ctx)
    v = [from_i128(t) for t in out]
    return dict(zip(("S1", "S2_trivial", "S2_easy", "S2_hard", "P2", "pi_y", "pi"), v))


def phi(x, a, threads=0, ctx=None, stream=None):
    """Partial sieve function phi(x, a) (primecount::phi)."""
    out = ctypes.c_int64()
    o = _opts(ctx, stream, threads)
    _check(load().pcg_phi(int(x), int(a), ctypes.byref(o), ctypes.byref(out)), ctx)
    return out.value


def pi_batch(xs, ctx=None, stream=None):
    n = len(xs)
    arr = (I128 * n)(*[to_i128(v) for v in xs])
    out = (I128 * n)()
    o = _opts(ctx, stream)
    _check(load().pcg_pi_batch(arr, n, out, ctypes.byref(o)), ctx)
    return [from_i128(v) for v in out]


def phi_batch(xs, as_, ctx=None, stream=None):
    n = len(xs)
    ax = (ctypes.c_int64 * n)(*[int(v) for v in xs])
    aa = (ctypes.c_int64 * n)(*[int(v) for v in as_])
    out = (ctypes.c_int64 * n)()
    o = _opts(ctx, stream)
    _check(load().pcg_phi_batch(ax, aa, n, out, ctypes.byref(o)), ctx)
    return list(out)


def query_device_bytes(kind, x, a=0, ctx=None):
    """Device working memory of one pi(x) ("pi") or phi(x, a) ("phi") call
    beyond the resident tables of ctx (pcg_query_device_bytes)."""
    b = ctypes.c_uint64()
    _check(load().pcg_query_device_bytes(ctx._h if ctx is not None else None, 0 if kind == "pi" else 1,
                                         to_i128(x), int(a or 0), ctypes.byref(b)), ctx)
    return b.value


def device_memory():
    """(free, total) bytes of the current CUDA device (pcg_device_memory)."""
    f, t = ctypes.c_uint64(), ctypes.c_uint64()
    _check(load().pcg_device_memory(ctypes.byref(f), ctypes.byref(t)))
    return f.value, t.value


# ---------------------------------------------------------------- shards
class ShardPart:
    """Per-level partials of one shard: acc (int), msum, csum (lists of int)."""

    __slots__ = ("acc", "msum", "csum")

    def __init__(self, acc, msum, csum):
        self.acc, self.msum, self.csum = list(acc), list(msum), list(csum)


def _shard(fn, x, y, z, k, shard, nshards, ctx=None, stream=None, cap=1 << 16):
    cols = ctypes.c_int64()
    while True:
        acc = (I128 * cap)()
        ms = (ctypes.c_int64 * cap)()
        cs = (ctypes.c_int64 * cap)()
        o = _opts(ctx, stream)
        st = fn(to_i128(x), int(y), int(z), int(k), int(shard), int(nshards), ctypes.byref(o), acc, ms, cs,
                cap, ctypes.byref(cols))
        if st == 2 and cols.value > cap:
            cap = cols.value
            continue
        _check(st, ctx)
        n = cols.value
        return ShardPart([from_i128(acc[i]) for i in range(n)], ms[:n], cs[:n])


def D_shard(x, y, z, k, shard, nshards, ctx=None, stream=None):
    """Shard `shard` of `nshards` of D(x, y, z, k) (pcg_D_shard)."""
    return _shard(load().pcg_D_shard, x, y, z, k, shard, nshards, ctx, stream)


def S2_hard_shard(x, y, z, c, shard, nshards, ctx=None, stream=None):
    """Shard `shard` of `nshards` of S2_hard(x, y, z, c) (pcg_S2_hard_shard)."""
    return _shard(load().pcg_S2_hard_shard, x, y, z, c, shard, nshards, ctx, stream)


def shard_combine(parts):
    """The result from the partials of all shards, in shard order
    (pcg_shard_combine; host arithmetic, no GPU needed)."""
    n = len(parts)
    cols = max((len(p.acc) for p in parts), default=0)
    acc = (I128 * max(1, n * cols))()
    ms = (ctypes.c_int64 * max(1, n * cols))()
    cs = (ctypes.c_int64 * max(1, n * cols))()
    for s_, p in enumerate(parts):
        for b in range(len(p.acc)):
            acc[s_ * cols + b] = to_i128(p.acc[b])
            ms[s_ * cols + b] = p.msum[b]
            cs[s_ * cols + b] = p.csum[b]
    out = I128()
    _check(load().pcg_shard_combine(n, cols, acc, ms, cs, ctypes.byref(out)))
    return from_i128(out)


def autotune(x, ctx):
    """Time the sweep configurations on D(x) and keep the fastest in ctx for
    x's decade (pcg_autotune); returns the choice as a dict."""
    t = Tuning()
    o = _opts(ctx, None)
    _check(load().pcg_autotune(to_i128(x), ctypes.byref(o), ctypes.byref(t)), ctx)
    return {k: getattr(t, k) for k, _ in t._fields_}
