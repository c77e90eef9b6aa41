// pcg_internal.hpp -- host-side declarations shared by the engine sources.
//
// The engine evaluates the hard special leaves of Gourdon's D(x, y, z, k)
// (reference: src/gourdon/D.cpp) and Deleglise-Rivat's S2_hard(x, y, z, c)
// (reference: src/deleglise-rivat/S2_hard.cpp) with one CUDA sweep over the
// sieve interval.  See sweep.cu for the device side.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <mutex>
#include <vector>

#include <cuda_runtime.h>

#include "pcgpu.h"

namespace pcg {

typedef unsigned __int128 u128;
typedef __int128 i128;

// ---------------------------------------------------------------- errors
struct Error {
  pcg_status status;
  std::string msg;
};

// Throwing helpers are internal only: every extern "C" entry point catches.
[[noreturn]] void fail(pcg_status s, const std::string& msg);
void cuda_check(cudaError_t e, const char* what);
#define PCG_CUDA(call) ::pcg::cuda_check((call), #call)

// ---------------------------------------------------------------- integer math
int64_t iroot(u128 x, int n);            // exact floor(x^(1/n)), n in {2,3,4,6}
inline int64_t isqrt(u128 x) { return iroot(x, 2); }
inline u128 make_u128(pcg_i128 v) { return ((u128) (uint64_t) v.hi << 64) | v.lo; }
inline pcg_i128 to_pcg(i128 v) { pcg_i128 r; r.lo = (uint64_t) v; r.hi = (int64_t) (v >> 64); return r; }
inline i128 make_i128(pcg_i128 v) { return (i128) make_u128(v); }
std::string to_string(i128 v);

// 2*3*5*7*11 wheel of the FactorTables (reference src/BaseFactorTable.hpp:36-47)
struct Wheel2310 {
  uint16_t coprime[480];     // numbers in [0, 2310) coprime to 2..11, ascending
  int16_t index[2310];       // index of the largest coprime <= r (-1 for r = 0)
  Wheel2310();
  int64_t to_index(uint64_t n) const { return 480 * (int64_t) (n / 2310) + index[n % 2310]; }
  int64_t to_number(uint64_t i) const { return 2310 * (int64_t) (i / 480) + coprime[i % 480]; }
};
const Wheel2310& wheel2310();

// ---------------------------------------------------------------- parameters
struct GourdonParams { int64_t y, z, k, x_star; };
struct DrParams { int64_t y, z, c; };
GourdonParams gourdon_params(u128 x);    // src/gourdon/pi_gourdon.cpp:44-62
// the same with alpha_y / alpha_z given (<= 0: default), clamped as the
// reference clamps --alpha-y / --alpha-z (src/gourdon/pi_gourdon.cpp:44-62)
GourdonParams gourdon_params(u128 x, double alpha_y, double alpha_z);
DrParams dr_params(u128 x);              // src/app/main.cpp:435-461
int64_t x_star_gourdon(u128 x, int64_t y);   // src/util.cpp:362-386
int64_t get_c(int64_t y);                // src/PhiTiny.hpp:47-50

// ---------------------------------------------------------------- device buffers
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  ~DevBuf();
  void alloc(size_t n);
  void free_();
  template <class T> T* as() const { return (T*) p; }
};

// Device-resident tables of one context.
struct Tables {
  // primes (uint32, 1-indexed, primes[0] = 0) and PiTable {count, bits} per 240
  int64_t prime_limit = -1;  // tables cover [0, prime_limit]
  int64_t nprimes = 0;
  DevBuf primes;             // uint32[nprimes + 2]
  DevBuf pmagic;             // uint64[nprimes + 2]: floor((2^64 - 1) / primes[i])
  DevBuf pitab;              // uint64[2 * (prime_limit / 240 + 1)]
  std::vector<uint32_t> h_primes;   // host copy of the primes (small part)
  std::vector<uint64_t> h_pitab;    // host copy of the PiTable
  // FactorTableD (Gourdon): entries for coprime-to-2310 n <= fd_z, mpf filter fd_y
  int64_t fd_y = -1, fd_z = -1;
  int fd_bytes = 2;          // 2 = uint16_t entries, 4 = uint32_t
  DevBuf factor_d;
  // FactorTable (Deleglise-Rivat): n <= fr_y
  int64_t fr_y = -1;
  int fr_bytes = 2;
  DevBuf factor_dr;
  // floor((2^64 - 1) / m) for the numbers m coprime to 2310, by factor-table
  // index, for the indices [0, finv_n)
  int64_t finv_n = 0;
  DevBuf finv;
  // PiTable up to sqrt(x) for the A, B, C formulas of pi(x) (no primes array)
  int64_t pibig_limit = -1;
  DevBuf pibig;
  // phi(r, k) for r < p_1 * ... * p_k: coprime bits and per-word prefix counts
  int phik = -1;
  uint64_t phi_P = 0, phi_tot = 0;
  DevBuf phi_bits, phi_pref;
  // wheel tables on device
  DevBuf coprime;            // uint16[480]
  DevBuf cindex;             // int16[2310]
  double build_ms = 0;
};

struct Ctx;

// Builds (or reuses) the prime tables up to `limit`.
void ensure_prime_tables(Ctx& c, int64_t limit, cudaStream_t s);
// FactorTableD for (y, z); FactorTable (DR) for y.
void ensure_factor_d(Ctx& c, int64_t y, int64_t z, cudaStream_t s);
void ensure_factor_dr(Ctx& c, int64_t y, cudaStream_t s);

// device exclusive scan (uint32 -> uint64), synchronous on s
void exclusive_scan_u32(const uint32_t* in, int64_t n, uint64_t* out, cudaStream_t s, DevBuf* sums = nullptr);

// slots of Ctx::tmp
enum TmpSlot {
  T_PS_BASE, T_PS_MAGIC, T_PS_C, T_PS_M, T_PS_L, T_PS_Q,      // prime sieve (B, small pi)
  T_LK_V, T_LK_R,                                             // PiTable lookups
  T_AC_QLO, T_AC_QCNT, T_AC_QOFF, T_AC_OUTS,                  // A + C outers
  T_PR_PIECES, T_PR_FIRST, T_PR_SPLIT, T_PR_PART, T_PR_SUMS,  // pair sums
  T_PHI0_PART, T_PHI_ONE, T_PHI_OUTS,                         // Phi0, phi(x, a)
  T_SW_SEG, T_SW_XP, T_SW_Q, T_SW_ROW, T_SW_JOB,              // sweep: segments, x/p, problems, rows, jobs
  T_COUNT
};
// PiTable {count, bits} over [0, limit] without the primes array
void build_pitab_only(DevBuf& out, int64_t limit, cudaStream_t s);

// host PiTable lookup on the host copy
int64_t host_pi(const Tables& t, uint64_t x);

// ---------------------------------------------------------------- sweep
struct SweepProblem {
  int gourdon;         // 1: D, 0: S2_hard
  u128 x;
  int64_t y, z, k;     // k = c for S2_hard
  // shard s of n: the contiguous segments [nseg s / n, nseg (s + 1) / n) of
  // the segment plan; n = 1 sweeps everything
  int shard = 0, nshards = 1;
  bool parts = false;  // return the per-level partials of the shard
};

struct Tuning {
  int segment_words = 0;
  int ctas_per_sm = 0;
  int cta_threads = 0;
  double alpha_y = 0, alpha_z = 0;   // pi(x) by Gourdon; <= 0: the reference's defaults
  std::string checkpoint;            // sweep checkpoint file ("" = none)
  double checkpoint_interval = 0;    // seconds between checkpoint writes
  int stop_after_waves = 0;          // > 0: stop (checkpointed) after this many waves
  int group = -1;                    // levels per group in the sweep (-1: default)
};

struct SweepResult {
  i128 sum = 0;
  pcg_stats stats{};
  // per level b (index 0 unused by levels): the shard's leaf sums with phi
  // offsets counted from the shard start (acc, the shard's local sums folded
  // into acc[0]), sum of the signed leaf counts M(s, b) and of the survivor
  // counts C(s, b) over the shard's segments; [lo, hi) = the shard's numbers
  std::vector<i128> acc;
  std::vector<int64_t> msum, csum;
  int64_t lo = 0, hi = 0;
};

SweepResult run_sweep(Ctx& c, const SweepProblem& p, const Tuning& t, cudaStream_t s);
// D of many problems (gourdon = 1, y >= z each) in one sweep whose waves run
// as one CUDA graph; sums[i] = D of pbs[i]
void run_sweep_batch(Ctx& c, const std::vector<SweepProblem>& pbs, const Tuning& t, cudaStream_t s,
                     std::vector<i128>& sums, pcg_stats* st);
// device working memory of one sweep over [0, L) with cols columns
uint64_t sweep_device_bytes(int num_sms, int64_t L, int64_t cols, int words);
// frees a context's per-call working memory (the tables stay); bytes freed
uint64_t ctx_trim(Ctx& c);
// D with working memory from a static device array; tables must be resident
SweepResult run_sweep_noalloc(Ctx& c, const SweepProblem& p, cudaStream_t s);

// ---------------------------------------------------------------- context
struct Ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int num_sms = 0;
  size_t smem_optin = 0;
  uint64_t mem_budget = 0;
  Tables tab;
  // scratch of the sweep (grown on demand)
  DevBuf cnt, smu, segsum, run, acc, misc, msum;
  // per-call temporaries, one slot per use site, kept and grown across calls
  // (no cudaMalloc / cudaFree per call: cudaFree synchronises the device and
  // would serialise the contexts of a worker pool)
  DevBuf tmp[32];
  // sweep configurations chosen by pcg_autotune, by decimal exponent of x
  bool tuned[64] = {};
  Tuning tuned_cfg[64];
  pcg_stats last{};
  std::string last_error;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  std::vector<cudaEvent_t> kev;   // per-launch timing events of the sweep
  // the last segment plan of the sweep and the problem and launch shape it was made for
  std::vector<int64_t> plan, plan_key;
  // second stream for work that runs beside the sweep (pi(x)'s other terms)
  cudaStream_t aux = nullptr;
  std::mutex aux_mu;
  // calls on one context run one at a time (threads wanting concurrency use
  // one context each, as the batch and serving forms do)
  std::recursive_mutex call_mu;
  ~Ctx();
};

Ctx& default_ctx();
Ctx* ctx_from(const pcg_opts* o);
cudaStream_t stream_from(Ctx& c, const pcg_opts* o);

// Runs f(ctx, stream) and turns internal failures into a pcg_status plus the
// message for pcg_last_error (defined in api.cpp).
pcg_status guarded_call(const pcg_opts* opts, void (*fn)(Ctx&, cudaStream_t, void*), void* arg);

}  // namespace pcg

template <class F>
inline pcg_status pcg_guarded(const pcg_opts* opts, F&& f)
{
  auto tramp = [](pcg::Ctx& c, cudaStream_t s, void* a) { (*(F*) a)(c, s); };
  return pcg::guarded_call(opts, tramp, (void*) &f);
}
