// pi_api.cpp -- extern "C" entry points for pi(x), phi(x, a), the batch
// forms and the libprimecount C API names (include/pcgpu.h).
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <atomic>
#include <mutex>
#include <thread>
#include <vector>

#include "pcg_internal.hpp"

namespace pcg {
i128 pi_any(Ctx& c, u128 x, const Tuning& tune, cudaStream_t s, pcg_stats* st);
i128 pi_without_d(Ctx& c, u128 x, const Tuning& tune, cudaStream_t s, bool* needs_d);
void pi_gourdon_terms(Ctx& c, u128 x, const Tuning& tune, cudaStream_t s, i128 out[6]);
void pi_dr_terms(Ctx& c, u128 x, const Tuning& tune, cudaStream_t s, i128 out[7]);
int64_t phi_any(Ctx& c, int64_t x, int64_t a, const Tuning& tune, cudaStream_t s);
}  // namespace pcg

using namespace pcg;

namespace {

Tuning tune_of(const pcg_opts* o)
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

std::atomic<int> g_threads{0};

}  // namespace

extern "C" {

pcg_status pcg_pi(pcg_i128 xi, const pcg_opts* opts, pcg_i128* out)
{
  if (!out) return PCG_EINVAL;
  return pcg_guarded(opts, [&](Ctx& c, cudaStream_t s) {
    if (xi.hi < 0) { *out = to_pcg(0); return; }       // pi(x) = 0 for x < 2 (negative x included)
    pcg_stats st{};
    i128 r = pi_any(c, make_u128(xi), tune_of(opts), s, &st);
    c.last = st;
    if (opts && opts->print) std::printf("pi(x) = %s\nSeconds: %.3f\n", to_string(r).c_str(), st.total_ms / 1000);
    *out = to_pcg(r);
  });
}

pcg_status pcg_pi_deleglise_rivat(pcg_i128 xi, const pcg_opts* opts, pcg_i128* out)
{
  if (!out) return PCG_EINVAL;
  return pcg_guarded(opts, [&](Ctx& c, cudaStream_t s) {
    if (xi.hi < 0) { *out = to_pcg(0); return; }       // pi(x) = 0 for x < 2
    const u128 x = make_u128(xi);
    if (x <= (u128) 10000000000ull) {                  // small x: counted by the sieve, as pcg_pi does
      *out = to_pcg(pi_any(c, x, tune_of(opts), s, nullptr));
      return;
    }
    i128 t[7];
    pi_dr_terms(c, x, tune_of(opts), s, t);
    if (opts && opts->print) std::printf("pi(x) = %s\n", to_string(t[6]).c_str());
    *out = to_pcg(t[6]);
  });
}

pcg_status pcg_pi_dr_terms(pcg_i128 xi, const pcg_opts* opts, pcg_i128* out7)
{
  if (!out7) return PCG_EINVAL;
  return pcg_guarded(opts, [&](Ctx& c, cudaStream_t s) {
    if (xi.hi < 0) fail(PCG_EINVAL, "x must be >= 0");
    const u128 x = make_u128(xi);
    if (x <= (u128) 10000000000ull) fail(PCG_EINVAL, "pcg_pi_dr_terms needs x > 1e10 (smaller x is counted by a sieve)");
    i128 t[7];
    pi_dr_terms(c, x, tune_of(opts), s, t);
    for (int i = 0; i < 7; i++) out7[i] = to_pcg(t[i]);
  });
}

pcg_status pcg_pi_terms(pcg_i128 xi, const pcg_opts* opts, pcg_i128* out6)
{
  if (!out6) return PCG_EINVAL;
  return pcg_guarded(opts, [&](Ctx& c, cudaStream_t s) {
    if (xi.hi < 0) fail(PCG_EINVAL, "x must be >= 0");
    u128 x = make_u128(xi);
    if (x <= (u128) 10000000000ull) fail(PCG_EINVAL, "pcg_pi_terms needs x > 1e10 (smaller x is counted by a sieve)");
    i128 t[6];
    pi_gourdon_terms(c, x, tune_of(opts), s, t);
    for (int i = 0; i < 6; i++) out6[i] = to_pcg(t[i]);
  });
}

pcg_status pcg_phi(int64_t x, int64_t a, const pcg_opts* opts, int64_t* out)
{
  if (!out) return PCG_EINVAL;
  return pcg_guarded(opts, [&](Ctx& c, cudaStream_t s) { *out = phi_any(c, x, a, tune_of(opts), s); });
}

}  // extern "C"

// Batches: the queries run largest first on a pool of worker contexts, each
// with its own stream and its own device-resident tables sized for the
// largest x of the batch, so that the short launch sequences of small queries
// overlap on the GPU.  Results do not depend on the pool: each query is
// computed exactly as alone.
namespace {

struct WorkerPool {
  std::mutex mu;
  std::vector<pcg::Ctx*> ctx;
  int device = -1;
};
WorkerPool g_pool;

int pool_size(const pcg_opts* opts, size_t n)
{
  int w = (opts && opts->threads > 0) ? opts->threads : 8;
  w = std::max(1, std::min(w, 16));
  return (int) std::min<size_t>((size_t) w, std::max<size_t>(n, 1));
}

template <class F>
pcg_status run_pool(size_t n, const pcg_opts* opts, const std::vector<size_t>& order, F&& job)
{
  const int W = pool_size(opts, n);
  std::lock_guard<std::mutex> g(g_pool.mu);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return PCG_ENODEV; }
  if (g_pool.device != dev) {
    for (auto* c : g_pool.ctx) pcg_ctx_destroy((pcg_ctx*) c);
    g_pool.ctx.clear();
    g_pool.device = dev;
  }
  while ((int) g_pool.ctx.size() < W) {
    pcg_ctx* c = nullptr;
    pcg_i128 zero;
    zero.lo = 0;
    zero.hi = 0;
    pcg_status st = pcg_ctx_create(zero, 0, &c);
    if (st != PCG_OK) return st;
    g_pool.ctx.push_back((pcg::Ctx*) c);
  }
  std::atomic<size_t> next{0};
  std::atomic<int> err{PCG_OK};
  std::string msg;
  std::mutex msg_mu;
  std::vector<std::thread> th;
  for (int w = 0; w < W; w++) {
    th.emplace_back([&, w] {
      pcg_opts o{};
      if (opts) o = *opts;
      o.ctx = (pcg_ctx*) g_pool.ctx[(size_t) w];
      o.stream = nullptr;
      for (;;) {
        const size_t k = next.fetch_add(1);
        if (k >= n || err.load() != PCG_OK) break;
        pcg_status st = job(order[k], &o);
        if (st != PCG_OK) {
          int expected = PCG_OK;
          if (err.compare_exchange_strong(expected, (int) st)) {
            std::lock_guard<std::mutex> lk(msg_mu);
            msg = pcg_last_error(o.ctx);
          }
          break;
        }
      }
    });
  }
  for (auto& t : th) t.join();
  if (err.load() != PCG_OK) return (pcg_status) err.load();
  return PCG_OK;
}

}  // namespace

extern "C" {

// pi(x) of n queries.  The hard special leaves (Gourdon's D) of every query
// with x > 1e10 run as the work items of one batched sweep on the caller's
// context (one persistent kernel per wave over all queries' segments, the
// waves launched as one CUDA graph), while the worker pool computes the other
// terms of those queries and the small queries whole; each answer is then
// the pool's part plus its D.
pcg_status pcg_pi_batch(const pcg_i128* xs, size_t n, pcg_i128* out, const pcg_opts* opts)
{
  if ((!xs || !out) && n) return PCG_EINVAL;
  if (n == 0) return PCG_OK;
  std::vector<size_t> order(n);
  for (size_t i = 0; i < n; i++) order[i] = i;
  auto key = [&](size_t i) { return make_u128(xs[i]); };
  std::sort(order.begin(), order.end(), [&](size_t a, size_t b) {
    if (xs[a].hi < 0 || xs[b].hi < 0) return xs[a].hi > xs[b].hi;
    return key(a) > key(b);
  });
  const Tuning tune = tune_of(opts);
  // the queries whose D joins the batched sweep
  std::vector<int64_t> slot(n, -1);
  std::vector<SweepProblem> pbs;
  pcg_status st0 = pcg_guarded(opts, [&](Ctx&, cudaStream_t) {
    for (size_t i = 0; i < n; i++) {
      if (xs[i].hi < 0) continue;
      const u128 x = make_u128(xs[i]);
      if (x <= (u128) 10000000000ull) continue;
      const GourdonParams g = gourdon_params(x, tune.alpha_y, tune.alpha_z);
      if (g.y < g.z || x > ((u128) g.y << 62)) continue;
      SweepProblem p;
      p.gourdon = 1;
      p.x = x;
      p.y = g.y;
      p.z = g.z;
      p.k = g.k;
      slot[i] = (int64_t) pbs.size();
      pbs.push_back(p);
    }
  });
  if (st0 != PCG_OK) return st0;
  std::vector<i128> dsum;
  pcg_status sweep_st = PCG_OK;
  std::string sweep_msg;
  std::thread sweeper;
  if (!pbs.empty()) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return PCG_ENODEV; }
    sweeper = std::thread([&, dev] {
      cudaSetDevice(dev);
      sweep_st = pcg_guarded(opts, [&](Ctx& c, cudaStream_t s) {
        pcg_stats st{};
        run_sweep_batch(c, pbs, tune, s, dsum, &st);
        c.last = st;
      });
      if (sweep_st != PCG_OK) sweep_msg = pcg_last_error(opts ? opts->ctx : nullptr);
    });
  }
  pcg_status pst = run_pool(n, opts, order, [&](size_t i, const pcg_opts* o) {
    if (slot[i] < 0) return pcg_pi(xs[i], o, &out[i]);
    return pcg_guarded(o, [&](Ctx& c, cudaStream_t s) {
      bool needs_d = false;
      const i128 r = pi_without_d(c, make_u128(xs[i]), tune, s, &needs_d);
      if (!needs_d) fail(PCG_EINTERNAL, "batched pi: a query without D joined the sweep");
      out[i] = to_pcg(r);
    });
  });
  if (sweeper.joinable()) sweeper.join();
  if (pst != PCG_OK) return pst;
  if (sweep_st != PCG_OK) return sweep_st;
  for (size_t i = 0; i < n; i++)
    if (slot[i] >= 0) out[i] = to_pcg(make_i128(out[i]) + dsum[(size_t) slot[i]]);
  return PCG_OK;
}

pcg_status pcg_phi_batch(const int64_t* x, const int64_t* a, size_t n, int64_t* out, const pcg_opts* opts)
{
  if ((!x || !a || !out) && n) return PCG_EINVAL;
  if (n == 0) return PCG_OK;
  std::vector<size_t> order(n);
  for (size_t i = 0; i < n; i++) order[i] = i;
  std::sort(order.begin(), order.end(), [&](size_t p, size_t q) { return x[p] > x[q]; });
  return run_pool(n, opts, order, [&](size_t i, const pcg_opts* o) { return pcg_phi(x[i], a[i], o, &out[i]); });
}

}  // extern "C"

extern "C" {

// ---- libprimecount C API: same names; errors print to stderr and return -1
// (src/api_c.cpp:19-150)
int64_t primecount_pi(int64_t x)
{
  pcg_i128 r;
  pcg_i128 xi;
  xi.lo = (uint64_t) x;
  xi.hi = x < 0 ? -1 : 0;
  if (pcg_pi(xi, nullptr, &r) != PCG_OK) {
    std::fprintf(stderr, "primecount_pi: %s\n", pcg_last_error(nullptr));
    return -1;
  }
  return (int64_t) r.lo;
}

pcg_i128 primecount_pi_128(pcg_i128 x)
{
  pcg_i128 r;
  if (pcg_pi(x, nullptr, &r) != PCG_OK) {
    std::fprintf(stderr, "primecount_pi_128: %s\n", pcg_last_error(nullptr));
    r.lo = ~0ull;
    r.hi = -1;
  }
  return r;
}

int64_t primecount_phi(int64_t x, int64_t a)
{
  int64_t r = 0;
  if (pcg_phi(x, a, nullptr, &r) != PCG_OK) {
    std::fprintf(stderr, "primecount_phi: %s\n", pcg_last_error(nullptr));
    return -1;
  }
  return r;
}

int primecount_get_num_threads(void)
{
  int t = g_threads.load();
  if (t > 0) return t;
  unsigned h = std::thread::hardware_concurrency();
  return h ? (int) h : 1;
}

void primecount_set_num_threads(int num_threads) { g_threads.store(num_threads > 0 ? num_threads : 0); }

const char* primecount_version(void) { return "8.7"; }

}  // extern "C"
