// api.cpp -- extern "C" boundary of libpcgpu and its host logic.
//
// Entry points mirror the reference's interfaces for the hard-leaf path
// (see include/pcgpu.h for the file:line of each).  Errors never cross the
// boundary as exceptions: every entry point returns a pcg_status and keeps
// the message for pcg_last_error(), the way the reference's C API catches
// primecount_error and prints it (src/api_c.cpp:19-30).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <chrono>
#include <mutex>
#include <thread>
#include <algorithm>

#include "pcg_internal.hpp"


namespace pcg {

// ---------------------------------------------------------------- errors
struct Failure {
  pcg_status status;
  std::string msg;
};

void fail(pcg_status s, const std::string& msg) { throw Failure{s, msg}; }

void cuda_check(cudaError_t e, const char* what)
{
  if (e == cudaSuccess) return;
  cudaGetLastError();
  pcg_status s = (e == cudaErrorMemoryAllocation) ? PCG_ENOMEM
               : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? PCG_ENODEV : PCG_ECUDA;
  fail(s, std::string(what) + ": " + cudaGetErrorString(e));
}

static thread_local std::string tl_error;

// ---------------------------------------------------------------- integer math
int64_t iroot(u128 x, int n)
{
  if (x == 0) return 0;
  auto ipow = [](u128 r, int e) { u128 p = 1; for (int i = 0; i < e; i++) p *= r; return p; };
  int64_t r = (int64_t) std::pow((double) x, 1.0 / n);
  if (n == 2) r = (int64_t) std::sqrt((double) x);
  if (n == 3) r = (int64_t) std::cbrt((double) x);
  if (r < 0) r = 0;
  for (; r > 0; r--)
    if (ipow((u128) r, n - 1) <= x / (u128) r) break;
  while (ipow((u128) (r + 1), n - 1) <= x / (u128) (r + 1)) r++;
  return r;
}

std::string to_string(i128 v)
{
  if (v == 0) return "0";
  bool neg = v < 0;
  u128 u = neg ? (u128) (-(v + 1)) + 1 : (u128) v;
  std::string s;
  while (u) { s.push_back((char) ('0' + (int) (u % 10))); u /= 10; }
  if (neg) s.push_back('-');
  std::reverse(s.begin(), s.end());
  return s;
}

Wheel2310::Wheel2310()
{
  int n = 0, last = -1;
  for (int r = 0; r < 2310; r++) {
    if (r % 2 && r % 3 && r % 5 && r % 7 && r % 11) { coprime[n] = (uint16_t) r; last = n; n++; }
    index[r] = (int16_t) last;
  }
}

const Wheel2310& wheel2310()
{
  static const Wheel2310 w;
  return w;
}

// ---------------------------------------------------------------- parameters
// Same formulas as the reference so that y, z, k are identical:
// get_alpha_gourdon (src/util.cpp:276-349) and pi_gourdon_64/128
// (src/gourdon/pi_gourdon.cpp:44-62).  The polynomial coefficients are the
// reference's empirical tuning constants.
static double in_between(double lo, double x, double hi) { return x < lo ? lo : (x > hi ? hi : x); }
static double truncate3(double n) { return (double) ((int64_t) (n * 1000)) / 1000.0; }

int64_t get_c(int64_t y)
{
  static const int64_t pi20[20] = {0, 0, 1, 2, 2, 3, 3, 4, 4, 4, 4, 5, 5, 6, 6, 6, 6, 7, 7, 8};
  return (y >= 0 && y < 20) ? pi20[y] : 8;
}

int64_t x_star_gourdon(u128 x, int64_t y)
{
  y = std::max<int64_t>(y, 1);
  u128 yy = (u128) y * (u128) y;
  u128 x_div_yy = (x + yy - 1) / yy;
  int64_t r4 = iroot(x, 4);
  int64_t xs = (u128) r4 > x_div_yy ? r4 : (int64_t) x_div_yy;
  int64_t sqrt_xy = isqrt(x / (u128) y);
  xs = std::min(xs, y);
  xs = std::min(xs, sqrt_xy);
  return std::max<int64_t>(xs, 1);
}

GourdonParams gourdon_params(u128 x) { return gourdon_params(x, 0, 0); }

GourdonParams gourdon_params(u128 x, double user_alpha_y, double user_alpha_z)
{
  double x16 = (double) iroot(x, 6);
  double logx = std::log((double) x);
  double alpha_yz;
  if (x <= (u128) 100000000000ull)
    alpha_yz = 0.078173 * logx + 1;
  else {
    const double a = 0.007888745747017503, b = -0.7610431057184933;
    const double c = 25.74106177417062, d = -288.9823576050215;
    alpha_yz = a * logx * logx * logx + b * logx * logx + c * logx + d;
  }
  double alpha_z = in_between(1, alpha_yz / 5, 1.0);
  double alpha_y = alpha_yz / alpha_z;
  if (user_alpha_y > 0) alpha_y = user_alpha_y;
  if (user_alpha_z > 0) alpha_z = user_alpha_z;
  alpha_y = in_between(1, alpha_y, x16);
  alpha_y = truncate3(alpha_y);
  alpha_z = truncate3(alpha_z);
  alpha_y = in_between(1, alpha_y, x16);
  double max_alpha_z = std::max(1.0, x16 / alpha_y);
  alpha_z = in_between(1, alpha_z, max_alpha_z);

  int64_t x13 = iroot(x, 3);
  int64_t sqrtx = isqrt(x);
  int64_t y = (int64_t) (x13 * alpha_y);
  y = std::max(y, x13 + 1);
  y = std::min(y, sqrtx - 1);
  y = std::max<int64_t>(y, 1);
  int64_t k = get_c(iroot(x, 4));
  int64_t z = (int64_t) (y * alpha_z);
  z = std::max(z, y);
  z = std::min(z, sqrtx - 1);
  z = std::max<int64_t>(z, 1);
  GourdonParams p;
  p.y = y;
  p.z = z;
  p.k = k;
  p.x_star = x_star_gourdon(x, y);
  return p;
}

DrParams dr_params(u128 x)
{
  double x16 = (double) iroot(x, 6);
  double logx = std::log((double) x);
  double alpha;
  if (x <= (u128) 1000000000ull)
    alpha = 0.078173 * logx + 1;
  else
    alpha = 0.00148918 * logx * logx * logx - 0.0691909 * logx * logx + 1.00165 * logx + 0.372253;
  alpha = in_between(1, alpha, x16);
  alpha = truncate3(alpha);
  alpha = in_between(1, alpha, x16);
  DrParams p;
  p.y = (int64_t) (iroot(x, 3) * alpha);
  p.z = (int64_t) (x / (u128) std::max<int64_t>(p.y, 1));
  p.c = get_c(p.y);
  return p;
}

// ---------------------------------------------------------------- contexts
Ctx::~Ctx()
{
  for (auto& e : ev) if (e) cudaEventDestroy(e);
  for (auto& e : kev) if (e) cudaEventDestroy(e);
  if (aux) cudaStreamDestroy(aux);
  if (own_stream && stream) cudaStreamDestroy(stream);
}

static void ctx_init(Ctx& c)
{
  int dev = 0;
  PCG_CUDA(cudaGetDevice(&dev));
  c.device = dev;
  PCG_CUDA(cudaDeviceGetAttribute(&c.num_sms, cudaDevAttrMultiProcessorCount, dev));
  int optin = 0;
  PCG_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  c.smem_optin = (size_t) optin;
  PCG_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
  c.own_stream = true;
  for (auto& e : c.ev) PCG_CUDA(cudaEventCreate(&e));
}

static std::mutex g_ctx_mu;
static Ctx* g_default[64] = {nullptr};

Ctx& default_ctx()
{
  int dev = 0;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    fail(PCG_ENODEV, "no CUDA device: libpcgpu computes on the GPU only");
  }
  PCG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> g(g_ctx_mu);
  if (!g_default[dev]) {
    Ctx* c = new Ctx();
    ctx_init(*c);
    g_default[dev] = c;
  }
  return *g_default[dev];
}

Ctx* ctx_from(const pcg_opts* o) { return (o && o->ctx) ? (Ctx*) o->ctx : &default_ctx(); }
cudaStream_t stream_from(Ctx& c, const pcg_opts* o) { return (o && o->stream) ? (cudaStream_t) o->stream : c.stream; }

}  // namespace pcg

using namespace pcg;

// The opaque handle is the Ctx itself.
struct pcg_ctx : public Ctx {};

template <class F>
static pcg_status guard(Ctx* c, F&& f)
{
  try {
    f();
    return PCG_OK;
  } catch (const Failure& e) {
    tl_error = e.msg;
    if (c) c->last_error = e.msg;
    return e.status;
  } catch (const std::bad_alloc&) {
    tl_error = "host allocation failed";
    if (c) c->last_error = tl_error;
    return PCG_ENOMEM;
  } catch (const std::exception& e) {
    tl_error = e.what();
    if (c) c->last_error = tl_error;
    return PCG_EINTERNAL;
  }
}

namespace pcg {
pcg_status guarded_call(const pcg_opts* opts, void (*fn)(Ctx&, cudaStream_t, void*), void* arg)
{
  Ctx* cp = nullptr;
  return guard(nullptr, [&] {
    cp = ctx_from(opts);
    std::lock_guard<std::recursive_mutex> lk(cp->call_mu);
    cp->last_error.clear();
    try {
      fn(*cp, stream_from(*cp, opts), arg);
    } catch (const Failure& e) {
      cp->last_error = e.msg;
      throw;
    }
  });
}
}  // namespace pcg

static Tuning tuning_from(const pcg_opts* o)
{
  Tuning t;
  if (o) {
    t.segment_words = o->segment_words;
    t.ctas_per_sm = o->ctas_per_sm;
    t.cta_threads = o->cta_threads;
    t.alpha_y = o->alpha_y;
    t.alpha_z = o->alpha_z;
    if (o->checkpoint) t.checkpoint = o->checkpoint;
    t.checkpoint_interval = o->checkpoint_interval;
    t.stop_after_waves = o->stop_after_waves;
  }
  return t;
}

static void print_result(const char* name, i128 v, double ms)
{
  std::printf("%s = %s\nSeconds: %.3f\n", name, to_string(v).c_str(), ms / 1000.0);
}

// checks of D.cpp:425-505 / FactorTableD.hpp:82-83 / main.cpp:224-229
static void check_hard_args(u128 x, int64_t y, int64_t z, int64_t k, bool gourdon)
{
  if (y < 1 || z < 1 || k < 0) fail(PCG_EINVAL, "y, z must be >= 1 and k >= 0");
  if (x > ((u128) y << 62)) fail(PCG_ERANGE, gourdon ? "D(x): x is too large" : "S2_hard(x): x is too large");
}

extern "C" {

pcg_status pcg_ctx_create(pcg_i128 max_x, uint64_t mem_budget, pcg_ctx** out)
{
  if (!out) return PCG_EINVAL;
  *out = nullptr;
  pcg_ctx* c = nullptr;
  pcg_status s = guard(nullptr, [&] {
    if (max_x.hi < 0) fail(PCG_EINVAL, "max_x must be >= 0");
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
      cudaGetLastError();
      fail(PCG_ENODEV, "no CUDA device: libpcgpu computes on the GPU only");
    }
    c = new pcg_ctx();
    ctx_init(*c);
    size_t free_b = 0, total_b = 0;
    PCG_CUDA(cudaMemGetInfo(&free_b, &total_b));
    c->mem_budget = mem_budget ? mem_budget : (uint64_t) (free_b * 0.9);
    u128 x = make_u128(max_x);
    if (x >= 10) {
      GourdonParams g = gourdon_params(x);
      ensure_prime_tables(*c, std::max<int64_t>(g.y, isqrt(x) / 1 > 0 ? g.y : g.y), c->stream);
      ensure_factor_d(*c, g.z, g.z, c->stream);
      if (pcg_ctx_device_bytes(c) > c->mem_budget)
        fail(PCG_ENOMEM, "resident tables exceed the memory budget");
    }
  });
  if (s != PCG_OK) {
    delete c;
    return s;
  }
  *out = c;
  return PCG_OK;
}

void pcg_ctx_destroy(pcg_ctx* c) { delete c; }

const char* pcg_last_error(const pcg_ctx* c)
{
  if (c) return c->last_error.c_str();
  return tl_error.c_str();
}

static uint64_t tmp_bytes(const Ctx& c)
{
  uint64_t t = 0;
  for (const DevBuf& b : c.tmp) t += b.bytes;
  return t;
}

uint64_t pcg_ctx_device_bytes(const pcg_ctx* c)
{
  if (!c) return 0;
  const Tables& t = c->tab;
  return t.primes.bytes + t.pitab.bytes + t.factor_d.bytes + t.factor_dr.bytes + t.coprime.bytes + t.cindex.bytes +
         t.pibig.bytes + t.pmagic.bytes + t.phi_bits.bytes + t.phi_pref.bytes + c->cnt.bytes + c->smu.bytes +
         c->segsum.bytes + c->run.bytes + c->acc.bytes + c->misc.bytes + c->msum.bytes + tmp_bytes(*c);
}

pcg_status pcg_last_stats(const pcg_ctx* c, pcg_stats* out)
{
  if (!out) return PCG_EINVAL;
  return guard(nullptr, [&] {
    const Ctx* cc = c ? (const Ctx*) c : &default_ctx();
    *out = cc->last;
  });
}

pcg_status pcg_gourdon_params(pcg_i128 xi, int64_t* y, int64_t* z, int64_t* k, int64_t* x_star)
{
  return guard(nullptr, [&] {
    if (xi.hi < 0) fail(PCG_EINVAL, "x must be >= 0");
    GourdonParams g = gourdon_params(make_u128(xi));
    if (y) *y = g.y;
    if (z) *z = g.z;
    if (k) *k = g.k;
    if (x_star) *x_star = g.x_star;
  });
}

pcg_status pcg_dr_params(pcg_i128 xi, int64_t* y, int64_t* z, int64_t* c)
{
  return guard(nullptr, [&] {
    if (xi.hi < 0) fail(PCG_EINVAL, "x must be >= 0");
    DrParams d = dr_params(make_u128(xi));
    if (y) *y = d.y;
    if (z) *z = d.z;
    if (c) *c = d.c;
  });
}

static pcg_status hard_leaves(bool gourdon, pcg_i128 xi, int64_t y, int64_t z, int64_t k,
                              const pcg_opts* opts, pcg_i128* out)
{
  if (!out) return PCG_EINVAL;
  Ctx* cp = nullptr;
  return guard(nullptr, [&] {
    cp = ctx_from(opts);
    std::lock_guard<std::recursive_mutex> lk(cp->call_mu);
    Ctx& c = *cp;
    c.last_error.clear();
    if (xi.hi < 0) fail(PCG_EINVAL, "x must be >= 0");
    u128 x = make_u128(xi);
    i128 result = 0;
    if (x >= 1) {
      check_hard_args(x, y, z, k, gourdon);
      SweepProblem p;
      p.gourdon = gourdon ? 1 : 0;
      p.x = x;
      p.y = y;
      p.z = z;
      p.k = k;
      SweepResult r = run_sweep(c, p, tuning_from(opts), stream_from(c, opts));
      result = r.sum;
      c.last = r.stats;
      if (opts && opts->print) print_result(gourdon ? "D" : "S2_hard", result, r.stats.total_ms);
    }
    *out = to_pcg(result);
  });
}

pcg_status pcg_D(pcg_i128 x, int64_t y, int64_t z, int64_t k, const pcg_opts* opts, pcg_i128* out)
{
  return hard_leaves(true, x, y, z, k, opts, out);
}

pcg_status pcg_S2_hard(pcg_i128 x, int64_t y, int64_t z, int64_t c, const pcg_opts* opts, pcg_i128* out)
{
  return hard_leaves(false, x, y, z, c, opts, out);
}

// One shard of D / S2_hard (several GPUs, one process each): the shard's
// per-level partials, combined in shard order by pcg_shard_combine.
static pcg_status hard_leaves_shard(bool gourdon, pcg_i128 xi, int64_t y, int64_t z, int64_t k, int shard,
                                    int nshards, const pcg_opts* opts, pcg_i128* acc, int64_t* msum,
                                    int64_t* csum, int64_t cap, int64_t* cols_out)
{
  if (!cols_out) return PCG_EINVAL;
  Ctx* cp = nullptr;
  return guard(nullptr, [&] {
    cp = ctx_from(opts);
    std::lock_guard<std::recursive_mutex> lk(cp->call_mu);
    Ctx& c = *cp;
    c.last_error.clear();
    if (xi.hi < 0) fail(PCG_EINVAL, "x must be >= 0");
    if (nshards < 1 || shard < 0 || shard >= nshards) fail(PCG_EINVAL, "shard must be in [0, nshards)");
    u128 x = make_u128(xi);
    *cols_out = 0;
    if (x < 1) return;
    check_hard_args(x, y, z, k, gourdon);
    SweepProblem p;
    p.gourdon = gourdon ? 1 : 0;
    p.x = x;
    p.y = y;
    p.z = z;
    p.k = k;
    p.shard = shard;
    p.nshards = nshards;
    p.parts = true;
    SweepResult r = run_sweep(c, p, tuning_from(opts), stream_from(c, opts));
    c.last = r.stats;
    const int64_t cols = (int64_t) r.acc.size();
    *cols_out = cols;
    if (cols > cap) fail(PCG_ERANGE, "partial arrays hold " + std::to_string(cap) + " levels, " +
                                         std::to_string(cols) + " needed");
    if (cols > 0 && (!acc || !msum || !csum)) fail(PCG_EINVAL, "null partial array");
    for (int64_t b = 0; b < cols; b++) {
      acc[b] = to_pcg(r.acc[(size_t) b]);
      msum[b] = r.msum[(size_t) b];
      csum[b] = r.csum[(size_t) b];
    }
  });
}

pcg_status pcg_D_shard(pcg_i128 x, int64_t y, int64_t z, int64_t k, int shard, int nshards, const pcg_opts* opts,
                       pcg_i128* acc, int64_t* msum, int64_t* csum, int64_t cap, int64_t* cols)
{
  return hard_leaves_shard(true, x, y, z, k, shard, nshards, opts, acc, msum, csum, cap, cols);
}

pcg_status pcg_S2_hard_shard(pcg_i128 x, int64_t y, int64_t z, int64_t c, int shard, int nshards,
                             const pcg_opts* opts, pcg_i128* acc, int64_t* msum, int64_t* csum, int64_t cap,
                             int64_t* cols)
{
  return hard_leaves_shard(false, x, y, z, c, shard, nshards, opts, acc, msum, csum, cap, cols);
}

pcg_status pcg_autotune(pcg_i128 xi, const pcg_opts* opts, pcg_tuning* best)
{
  if (!opts || !opts->ctx) return PCG_EINVAL;
  Ctx* cp = nullptr;
  return guard(nullptr, [&] {
    cp = ctx_from(opts);
    std::lock_guard<std::recursive_mutex> lk(cp->call_mu);
    Ctx& c = *cp;
    c.last_error.clear();
    if (xi.hi < 0) fail(PCG_EINVAL, "x must be >= 0");
    const u128 x = make_u128(xi);
    if (x < 1000) fail(PCG_EINVAL, "autotune needs x >= 1000");
    const GourdonParams g = gourdon_params(x);
    check_hard_args(x, g.y, g.z, g.k, true);
    const int e = (int) std::floor(std::log10((double) x));
    c.tuned[e] = false;
    cudaStream_t s = stream_from(c, opts);
    // candidates: the measured defaults first, then their neighbours
    static const int cand[][4] = {
        {8192, 0, 256, 32}, {8192, 0, 256, 16}, {8192, 0, 256, 64}, {8192, 0, 256, 0},
        {6144, 0, 256, 32}, {16384, 0, 512, 32}, {4096, 0, 128, 32}, {8192, 0, 128, 32}};
    SweepProblem p;
    p.gourdon = 1;
    p.x = x;
    p.y = g.y;
    p.z = g.z;
    p.k = g.k;
    Tuning t0;
    t0.group = 32;
    t0.segment_words = 8192;
    t0.cta_threads = 256;
    run_sweep(c, p, t0, s);   // tables and scratch built outside the timed runs
    Tuning bt;
    double bms = 1e300;
    i128 ref = 0;
    bool have = false;
    for (const auto& k : cand) {
      Tuning t;
      t.segment_words = k[0];
      t.ctas_per_sm = k[1];
      t.cta_threads = k[2];
      t.group = k[3];
      SweepResult r = run_sweep(c, p, t, s);
      if (!have) { ref = r.sum; have = true; }
      else if (r.sum != ref) fail(PCG_EINTERNAL, "autotune: configurations disagree");
      if (r.stats.sweep_ms < bms) { bms = r.stats.sweep_ms; bt = t; }
    }
    c.tuned_cfg[e] = bt;
    c.tuned[e] = true;
    if (best) {
      best->segment_words = bt.segment_words;
      best->ctas_per_sm = bt.ctas_per_sm;
      best->cta_threads = bt.cta_threads;
      best->group = bt.group;
      best->ms = bms;
    }
  });
}

pcg_status pcg_shard_combine(int nshards, int64_t cols, const pcg_i128* acc, const int64_t* msum,
                             const int64_t* csum, pcg_i128* out)
{
  if (!out || nshards < 1 || cols < 0) return PCG_EINVAL;
  return guard(nullptr, [&] {
    if (cols > 0 && (!acc || !msum || !csum)) fail(PCG_EINVAL, "null partial array");
    std::vector<i128> offset((size_t) cols, 0);   // survivors before the shard, per level
    i128 total = 0;
    for (int s = 0; s < nshards; s++) {
      const int64_t row = (int64_t) s * cols;
      for (int64_t b = 0; b < cols; b++) {
        total += make_i128(acc[row + b]) + (i128) msum[row + b] * offset[(size_t) b];
        offset[(size_t) b] += csum[row + b];
      }
    }
    *out = to_pcg(total);
  });
}

// Allocation-free D for callers that cannot allocate device memory at call
// time (see include/pcgpu.h): tables from the context, working memory from
// the library's static device scratch.
pcg_status pcg_D_noalloc(pcg_ctx* ctx, pcg_i128 xi, int64_t y, int64_t z, int64_t k, void* stream, pcg_i128* out)
{
  if (!out) return PCG_EINVAL;
  return guard(ctx, [&] {
    if (!ctx) fail(PCG_EINVAL, "pcg_D_noalloc needs a context created with pcg_ctx_create");
    std::lock_guard<std::recursive_mutex> lk(ctx->call_mu);
    Ctx& c = *ctx;
    c.last_error.clear();
    if (xi.hi < 0) fail(PCG_EINVAL, "x must be >= 0");
    u128 x = make_u128(xi);
    i128 result = 0;
    if (x >= 1) {
      check_hard_args(x, y, z, k, true);
      SweepProblem p;
      p.gourdon = 1;
      p.x = x;
      p.y = y;
      p.z = z;
      p.k = k;
      SweepResult r = run_sweep_noalloc(c, p, stream ? (cudaStream_t) stream : c.stream);
      result = r.sum;
      c.last = r.stats;
    }
    *out = to_pcg(result);
  });
}

pcg_status pcg_ctx_read_table(const pcg_ctx* ctx, int table, uint64_t first, uint64_t count, void* out,
                              uint64_t* entries, int* entry_bytes, int64_t* limit)
{
  if (!ctx) return PCG_EINVAL;
  Ctx* cp = (Ctx*) ctx;
  return guard(cp, [&] {
    std::lock_guard<std::recursive_mutex> lk(cp->call_mu);
    const Tables& t = cp->tab;
    const DevBuf* buf = nullptr;
    uint64_t n = 0;
    int eb = 0;
    int64_t lim = -1;
    switch (table) {
      case PCG_TABLE_PRIMES:
        if (t.prime_limit >= 0) { buf = &t.primes; n = (uint64_t) t.nprimes + 1; eb = 4; lim = t.prime_limit; }
        break;
      case PCG_TABLE_PI:
        if (t.prime_limit >= 0) { buf = &t.pitab; n = 2 * (uint64_t) (t.prime_limit / 240 + 1); eb = 8; lim = t.prime_limit; }
        break;
      case PCG_TABLE_FACTOR_D:
        if (t.fd_z >= 0) {
          buf = &t.factor_d;
          n = (uint64_t) wheel2310().to_index((uint64_t) std::max<int64_t>(t.fd_z, 1)) + 1;
          eb = t.fd_bytes;
          lim = t.fd_z;
        }
        break;
      case PCG_TABLE_FACTOR_DR:
        if (t.fr_y >= 0) {
          buf = &t.factor_dr;
          n = (uint64_t) wheel2310().to_index((uint64_t) std::max<int64_t>(t.fr_y, 1)) + 1;
          eb = t.fr_bytes;
          lim = t.fr_y;
        }
        break;
      default:
        fail(PCG_EINVAL, "unknown table " + std::to_string(table));
    }
    if (entries) *entries = n;
    if (entry_bytes) *entry_bytes = eb;
    if (limit) *limit = lim;
    if (count == 0) return;
    if (!buf || !out) fail(PCG_EINVAL, "the table is not resident or out is NULL");
    if (first > n || count > n - first) fail(PCG_ERANGE, "entries beyond the table");
    PCG_CUDA(cudaSetDevice(cp->device));
    PCG_CUDA(cudaStreamSynchronize(cp->stream));
    PCG_CUDA(cudaMemcpy(out, (const char*) buf->p + first * (uint64_t) eb, count * (uint64_t) eb,
                        cudaMemcpyDeviceToHost));
  });
}

// ---- serving support: device memory of a query, trimming, free memory
static int64_t pi_estimate(const Ctx& c, int64_t v)
{
  if (v < 2) return 0;
  if (v <= c.tab.prime_limit) return host_pi(c.tab, (uint64_t) v);
  const double d = (double) v;
  return (int64_t) (1.26 * d / std::log(d)) + 1;   // above pi(v) for v >= 17
}

static uint64_t table_bytes_beyond(const Ctx& c, int64_t y, int64_t z, int64_t sqrtx)
{
  uint64_t b = 0;
  if (y > c.tab.prime_limit) b += (uint64_t) (y / 240 + 1) * (16 + 20) + (uint64_t) pi_estimate(c, y) * 12;
  if (z > c.tab.fd_z) b += (uint64_t) (wheel2310().to_index((uint64_t) z) + 1) * (2 + 8);
  if (sqrtx + 240 > c.tab.pibig_limit) b += (uint64_t) (sqrtx / 240 + 2) * (16 + 20);
  return b;
}

// B's prime sieve over [lo, hi): per-segment sums and the sieving primes
static uint64_t psieve_bytes(int64_t lo, int64_t hi)
{
  if (hi <= lo) return 0;
  const int64_t seg = 12288ll * 240;
  return (uint64_t) ((hi - lo) / seg + 2) * 24 + (uint64_t) (isqrt((u128) hi) / 8 + 64) * 12;
}

static uint64_t pi_query_bytes(const Ctx& c, u128 x)
{
  if (x <= (u128) 10000000000ull) return psieve_bytes(0, (int64_t) x + 1) + 4096;
  const GourdonParams g = gourdon_params(x);
  const int64_t sqrtx = isqrt(x);
  const int64_t cols = pi_estimate(c, g.x_star) + 1;
  uint64_t b = sweep_device_bytes(c.num_sms, (int64_t) (x / (u128) g.z), cols, 8192);
  b += psieve_bytes(sqrtx, (int64_t) (x / (u128) g.y) + 1);
  b += (uint64_t) pi_estimate(c, iroot(x, 3)) * 4 * 64;      // A + C outer terms
  b += table_bytes_beyond(c, g.y, g.z, sqrtx);
  return b + 65536;
}

}  // extern "C"

namespace pcg {
// device bytes of one phi(x, a) query beyond the context's resident tables
static uint64_t phi_query_bytes(const Ctx& c, int64_t x, int64_t a)
{
  if (x < 1 || a <= 8 || a > x / 2) return 4096;
  const int64_t sq = isqrt((u128) x);
  const int64_t pis = pi_estimate(c, sq);
  if (a > pis) return pi_query_bytes(c, (u128) x);
  const double la = std::log((double) std::max<int64_t>(a, 3));
  const int64_t pa = (int64_t) ((double) a * (la + std::log(std::max(la, 1.0))));   // above p_a for a >= 6
  if ((u128) pa * pa * pa * pa > (u128) x)                    // P2 + P3
    return pi_query_bytes(c, (u128) x) + psieve_bytes(sq, x / std::max<int64_t>(pa / 2, 1) + 1) +
           (uint64_t) pi_estimate(c, iroot((u128) x, 3)) * 64;
  const int64_t y = std::max<int64_t>(pa, std::min<int64_t>(sq - 1, 8 * iroot((u128) x, 3)));
  uint64_t b = sweep_device_bytes(c.num_sms, x / y, a + 1, 8192);
  b += (uint64_t) (wheel2310().to_index((uint64_t) y) + 1) * (2 + 8) + (uint64_t) (y / 240 + 1) * 36;
  b += (uint64_t) c.num_sms * 8 * 16;                         // the ordinary leaves' partial sums
  return b + 65536;
}
}  // namespace pcg

extern "C" {

pcg_status pcg_query_device_bytes(const pcg_ctx* ctx, int kind, pcg_i128 x, int64_t a, uint64_t* bytes)
{
  if (!bytes) return PCG_EINVAL;
  return guard(nullptr, [&] {
    const Ctx& c = ctx ? *(const Ctx*) ctx : default_ctx();
    if (x.hi < 0) { *bytes = 0; return; }
    if (kind == PCG_QUERY_PI) *bytes = pi_query_bytes(c, make_u128(x));
    else if (kind == PCG_QUERY_PHI) {
      if (x.hi != 0 || x.lo > (uint64_t) INT64_MAX) fail(PCG_ERANGE, "phi(x, a): x must fit int64");
      *bytes = phi_query_bytes(c, (int64_t) x.lo, a);
    } else fail(PCG_EINVAL, "kind must be PCG_QUERY_PI or PCG_QUERY_PHI");
  });
}

pcg_status pcg_ctx_trim(pcg_ctx* ctx, uint64_t* freed)
{
  if (!ctx) return PCG_EINVAL;
  return guard(ctx, [&] {
    std::lock_guard<std::recursive_mutex> lk(ctx->call_mu);
    PCG_CUDA(cudaSetDevice(ctx->device));
    PCG_CUDA(cudaStreamSynchronize(ctx->stream));
    const uint64_t f = ctx_trim(*ctx);
    if (freed) *freed = f;
  });
}

pcg_status pcg_device_memory(uint64_t* free_bytes, uint64_t* total_bytes)
{
  return guard(nullptr, [&] {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
      cudaGetLastError();
      fail(PCG_ENODEV, "no CUDA device");
    }
    size_t f = 0, t = 0;
    PCG_CUDA(cudaMemGetInfo(&f, &t));
    if (free_bytes) *free_bytes = f;
    if (total_bytes) *total_bytes = t;
  });
}

pcg_status pcg_D_default(pcg_i128 xi, const pcg_opts* opts, pcg_i128* out, int64_t* y, int64_t* z, int64_t* k)
{
  int64_t yy = 1, zz = 1, kk = 0, xs = 0;
  if (xi.hi < 0 || (xi.hi == 0 && xi.lo < 1)) {
    if (out) *out = to_pcg(0);
    return xi.hi < 0 ? PCG_EINVAL : PCG_OK;
  }
  pcg_status s = pcg_gourdon_params(xi, &yy, &zz, &kk, &xs);
  if (s != PCG_OK) return s;
  if (y) *y = yy;
  if (z) *z = zz;
  if (k) *k = kk;
  return pcg_D(xi, yy, zz, kk, opts, out);
}

pcg_status pcg_S2_hard_default(pcg_i128 xi, const pcg_opts* opts, pcg_i128* out, int64_t* y, int64_t* z, int64_t* c)
{
  int64_t yy = 1, zz = 1, cc = 0;
  if (xi.hi < 0 || (xi.hi == 0 && xi.lo < 1)) {
    if (out) *out = to_pcg(0);
    return xi.hi < 0 ? PCG_EINVAL : PCG_OK;
  }
  pcg_status s = pcg_dr_params(xi, &yy, &zz, &cc);
  if (s != PCG_OK) return s;
  if (y) *y = yy;
  if (z) *z = zz;
  if (c) *c = cc;
  return pcg_S2_hard(xi, yy, zz, cc, opts, out);
}

}  // extern "C"
