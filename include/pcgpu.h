/*
 * pcgpu.h -- C ABI of the GB300 hard-special-leaf engine (libpcgpu.so).
 *
 * The engine computes the hard special leaves of combinatorial prime
 * counting on one GPU: Gourdon's D(x, y, z, k) and Deleglise-Rivat's
 * S2_hard(x, y, z, c), and on top of them pi(x) and phi(x, a), single and
 * batched.  Every entry point is extern "C", takes plain integers and
 * pointers, never throws, and returns a pcg_status; the message of the last
 * failure is available from pcg_last_error().
 *
 * 128-bit integers use pcg_i128, the layout of the reference's
 * pc_int128_t (include/primecount.h:38-41): { uint64_t lo; int64_t hi; }.
 *
 * Reference interfaces replaced (kimwalisch/primecount 8.7):
 *   pcg_D          <- int64_t/int128_t D(x, y, z, k, threads, is_print)
 *                     include/gourdon.hpp:28,38; src/gourdon/D.cpp:425-505
 *   pcg_S2_hard    <- int64_t/int128_t S2_hard(x, y, z, c, threads, is_print)
 *                     include/S.hpp:25,32; src/deleglise-rivat/S2_hard.cpp:221-293
 *   pcg_pi         <- primecount::pi(int64_t / pc_int128_t)
 *                     include/primecount.hpp:57-66; src/api.cpp:44-91
 *   pcg_phi        <- primecount::phi(x, a)  include/primecount.hpp:99; src/api.cpp:246
 *   pcg_pi_batch, pcg_phi_batch: many queries per call (no counterpart: the
 *                     reference answers one query per call)
 *   pcg_ctx_*      : device-resident tables (no counterpart: the reference
 *                     builds its tables inside every call, D.cpp:443-446)
 *   primecount_pi / primecount_pi_128 / primecount_phi /
 *   primecount_get_num_threads / primecount_set_num_threads /
 *   primecount_version
 *                  <- the libprimecount C API, include/primecount.h:51-122,
 *                     src/api_c.cpp:19-150 (same names, same -1 error
 *                     convention, message printed to stderr)
 */
#ifndef PCGPU_H
#define PCGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  uint64_t lo;
  int64_t hi;
} pcg_i128;

typedef enum {
  PCG_OK = 0,
  PCG_EINVAL = 1,     /* invalid argument (negative x, y < 1, ...)          */
  PCG_ERANGE = 2,     /* input beyond the supported range (x > y * 2^62, ...)*/
  PCG_ENOMEM = 3,     /* device or host allocation failed / over budget     */
  PCG_ECUDA = 4,      /* a CUDA call failed                                 */
  PCG_ENODEV = 5,     /* no CUDA device                                     */
  PCG_ETIMEOUT = 6,   /* a bounded device wait gave up                      */
  PCG_ECANCELLED = 7, /* request cancelled (serving)                        */
  PCG_EINTERNAL = 8   /* internal consistency check failed                  */
} pcg_status;

typedef struct pcg_ctx pcg_ctx;

/* Options of one call.  A NULL pcg_opts* means all defaults. */
typedef struct {
  pcg_ctx* ctx;          /* NULL: the library's default context of the current device;
                            calls on one context run one at a time                    */
  void* stream;          /* cudaStream_t to launch on; NULL: the context's stream      */
  int threads;           /* batches: worker contexts on the GPU (0 = 8); else unused   */
  int print;             /* reference is_print: print variables and timings            */
  int segment_words;     /* sieve segment in 64-bit words (x240 numbers); 0 = autotune */
  int ctas_per_sm;       /* resident CTAs per SM for the sweep; 0 = autotune           */
  int cta_threads;       /* threads per sweep CTA: 128, 256 or 512; 0 = autotune       */
  double alpha_y;        /* pi(x) by Gourdon: y = alpha_y x^(1/3) (the reference's      */
  double alpha_z;        /* --alpha-y / --alpha-z, z = alpha_z y); <= 0 = default       */
  /* Checkpoint / resume of D and S2_hard (no counterpart in the reference).
   * With a file path, a sweep resumes from the file when it holds a
   * checkpoint of the same problem and segment plan, writes the file after a
   * wave once checkpoint_interval seconds have passed since the last write
   * (0: after every wave), and removes it when the result is complete.
   * stop_after_waves > 0 ends the call after that many waves of this call
   * with PCG_ECANCELLED and the checkpoint written (an orderly interruption). */
  const char* checkpoint;
  double checkpoint_interval;
  int stop_after_waves;
} pcg_opts;

/* Work and time of the last call on a context. */
typedef struct {
  uint64_t leaves;         /* hard special leaves evaluated                          */
  uint64_t two_prime_leaves;/* of which p_b * p_l leaves                              */
  uint64_t segments;       /* sieve segments                                          */
  uint64_t levels;         /* (segment, b) sieve steps                                */
  uint64_t factor_entries; /* FactorTable entries read by the leaf filter             */
  uint64_t kernel_launches;/* engine kernels launched by the call                     */
  double table_ms;         /* device table construction (0 when resident)            */
  double sweep_ms;         /* sieve + leaf kernels                                    */
  double combine_ms;       /* phi-offset scan and reduction                           */
  double total_ms;         /* whole call, host clock                                  */
  double sweep_kernel_ms;  /* sum of the sieve/leaf kernel launches (CUDA events)     */
  uint64_t sweep_launches; /* launches of the sieve/leaf kernel                       */
  uint64_t h2d_bytes;      /* host -> device bytes copied by the call                 */
  uint64_t d2h_bytes;      /* device -> host bytes copied by the call                 */
  int segment_words;       /* tuning actually used                                    */
  int ctas_per_sm;
  int threads_per_cta;
  double ac_ms, b_ms, phi0_ms, sigma_ms, d_ms; /* pi(x): time of each Gourdon term   */
  uint64_t crossoff_multiples; /* multiples of the sieving primes crossed off in the
                                  segments (the sieve's shared-memory updates)      */
} pcg_stats;

/* ---- contexts: device-resident prime / PiTable / FactorTable state ---- */

/* Create a context on the current CUDA device whose tables cover every
 * query with x <= max_x (Gourdon default parameters).  mem_budget bounds
 * the device memory the context may hold (0 = 90% of free memory). */
pcg_status pcg_ctx_create(pcg_i128 max_x, uint64_t mem_budget, pcg_ctx** out);
void pcg_ctx_destroy(pcg_ctx* ctx);
/* Message of the last failure on ctx (NULL: of the calling thread). */
const char* pcg_last_error(const pcg_ctx* ctx);
/* Statistics of the last D / S2_hard / pi call on ctx (NULL: default ctx). */
pcg_status pcg_last_stats(const pcg_ctx* ctx, pcg_stats* out);
/* Device bytes held by the context's resident tables. */
uint64_t pcg_ctx_device_bytes(const pcg_ctx* ctx);

/* Resident tables of a context, for inspection and table-level tests (no
 * counterpart in the reference, whose tables are local objects of each
 * call; its own tests check them entry by entry, test/gourdon/
 * FactorTableD.cpp, test/lmo/FactorTable.cpp, test/PiTable.cpp).  Entry
 * formats are the reference's:
 *   PCG_TABLE_PRIMES     uint32, primes[0] = 0, primes[1..] = 2, 3, 5, ...
 *                        (PiTable::get_primes, src/PiTable.hpp)
 *   PCG_TABLE_PI         uint64 pairs {count, bits} per 240 numbers (src/PiTable.cpp)
 *   PCG_TABLE_FACTOR_D   FactorTableD entries, 2 or 4 bytes (src/gourdon/FactorTableD.hpp)
 *   PCG_TABLE_FACTOR_DR  FactorTable entries, 2 or 4 bytes (src/FactorTable.hpp) */
enum {
  PCG_TABLE_PRIMES = 0,
  PCG_TABLE_PI = 1,
  PCG_TABLE_FACTOR_D = 2,
  PCG_TABLE_FACTOR_DR = 3
};
/* Copies entries [first, first + count) of a resident table to the host
 * buffer out (count * entry size bytes) and writes the table's number of
 * entries, entry size in bytes and the largest number it covers (0 / -1
 * when the table is not built yet).  count = 0 only reports the sizes. */
pcg_status pcg_ctx_read_table(const pcg_ctx* ctx, int table, uint64_t first, uint64_t count, void* out,
                              uint64_t* entries, int* entry_bytes, int64_t* limit);

/* ---- serving support (no counterpart in the reference) ---- */

enum { PCG_QUERY_PI = 0, PCG_QUERY_PHI = 1 };
/* Device working memory (bytes) that one pi(x) (kind PCG_QUERY_PI) or
 * phi(x, a) (PCG_QUERY_PHI) call on ctx needs beyond ctx's resident tables:
 * the sweep's count and sign rows and tables, the prime sieve's buffers, the
 * formulas' temporaries and any table the call would still have to build.
 * An estimate from the call's sizes, at or above what the call allocates;
 * for admission control by a serving loop.  ctx NULL: the default context. */
pcg_status pcg_query_device_bytes(const pcg_ctx* ctx, int kind, pcg_i128 x, int64_t a, uint64_t* bytes);
/* Frees the per-call working memory ctx keeps between calls (the resident
 * tables stay); *freed (may be NULL) receives the bytes released. */
pcg_status pcg_ctx_trim(pcg_ctx* ctx, uint64_t* freed);
/* Free and total memory of the current CUDA device. */
pcg_status pcg_device_memory(uint64_t* free_bytes, uint64_t* total_bytes);

/* ---- the hard-leaf formulas ---- */

/* D(x, y, z, k): Gourdon's hard special leaves. */
pcg_status pcg_D(pcg_i128 x, int64_t y, int64_t z, int64_t k,
                 const pcg_opts* opts, pcg_i128* out);

/* S2_hard(x, y, z, c): Deleglise-Rivat's hard special leaves. */
pcg_status pcg_S2_hard(pcg_i128 x, int64_t y, int64_t z, int64_t c,
                       const pcg_opts* opts, pcg_i128* out);

/* One shard of D / S2_hard, for one x swept by several GPUs (one process
 * per GPU, a contiguous range of the segment plan each).  No counterpart in
 * the reference, whose chunks of [0, x/z) play the same role inside one
 * process (src/gourdon/D.cpp:382-421, LoadBalancerS2.cpp).  Shard s of n
 * sweeps segments [nseg s / n, nseg (s + 1) / n) with the phi offsets counted
 * from the shard's first number and writes, per level b < cols:
 *   acc[b]  its leaf sums (the local leaf sums are folded into acc[0]),
 *   msum[b] the sum of the signed leaf counts -mu of level b,
 *   csum[b] the numbers of the shard that survive to level b.
 * *cols = cols (the same for every shard of x).  The arrays hold cap entries;
 * with cap < cols only *cols is written and PCG_ERANGE is returned.
 * pcg_shard_combine turns the partials of all shards into the result. */
pcg_status pcg_D_shard(pcg_i128 x, int64_t y, int64_t z, int64_t k, int shard, int nshards,
                       const pcg_opts* opts, pcg_i128* acc, int64_t* msum, int64_t* csum,
                       int64_t cap, int64_t* cols);
pcg_status pcg_S2_hard_shard(pcg_i128 x, int64_t y, int64_t z, int64_t c, int shard, int nshards,
                             const pcg_opts* opts, pcg_i128* acc, int64_t* msum, int64_t* csum,
                             int64_t cap, int64_t* cols);

/* Result of all shards ([nshards][cols] row-major, shards in order):
 *   sum_s ( sum_b acc_s[b] + msum_s[b] * sum_{s' < s} csum_s'[b] ).
 * Host arithmetic only (no device work). */
pcg_status pcg_shard_combine(int nshards, int64_t cols, const pcg_i128* acc, const int64_t* msum,
                             const int64_t* csum, pcg_i128* out);

/* D(x, y, z, k) without allocating device memory.  No counterpart in the
 * reference.  For callers that cannot call cudaMalloc when they need the
 * result: request paths of a serving loop that must not touch the
 * allocator, or processes whose device memory belongs to another
 * framework's pool (where a cudaMalloc fails or takes memory the pool
 * accounts for).  The tables are inputs: ctx must have been created
 * (pcg_ctx_create, which does allocate, at set-up time) with a max_x whose
 * tables cover y and z, else PCG_ERANGE.  All device working memory comes
 * from one 64 MiB static device array that every GPU loading the library
 * holds until exit; a call needing more (or more than 32768 levels) is
 * rejected with PCG_ERANGE.  The call runs on ctx's device.  The first call
 * on a device looks up the array's device address (cudaGetSymbolAddress),
 * so make that first call before any stream capture.  Calls share the array
 * and it keeps the last call's contents (what must start at zero is cleared
 * on the stream); calls run one at a time on the host and each waits for
 * its own work before returning, but calls whose work overlaps on the GPU
 * race on the array.  stream may be NULL (the context's stream); the result
 * is written to *out on return. */
pcg_status pcg_D_noalloc(pcg_ctx* ctx, pcg_i128 x, int64_t y, int64_t z, int64_t k,
                         void* stream, pcg_i128* out);

/* A sweep configuration: segment words, resident CTAs per SM, threads per
 * CTA, levels per group (the b-range answered in one pass), and its time. */
typedef struct {
  int segment_words;
  int ctas_per_sm;
  int cta_threads;
  int group;
  double ms;
} pcg_tuning;

/* Autotuner (no counterpart in the reference, whose LoadBalancerS2 adapts
 * chunk sizes at run time instead).  Times D(x) with the reference's default
 * parameters under each candidate configuration on the context's device and
 * keeps the fastest for x's decade in the context: later D / S2_hard / pi
 * calls on that context whose tuning fields are 0 use it.  *best (may be
 * NULL) receives the choice; the context must be opts->ctx (not NULL). */
pcg_status pcg_autotune(pcg_i128 x, const pcg_opts* opts, pcg_tuning* best);

/* D(x) / S2_hard(x) with the reference's default parameters
 * (the --D / --S2-hard command-line options, src/app/main.cpp:205-246,
 * 435-461).  y, z, k (c) are written when the pointers are non-NULL. */
pcg_status pcg_D_default(pcg_i128 x, const pcg_opts* opts, pcg_i128* out,
                         int64_t* y, int64_t* z, int64_t* k);
pcg_status pcg_S2_hard_default(pcg_i128 x, const pcg_opts* opts, pcg_i128* out,
                               int64_t* y, int64_t* z, int64_t* c);

/* Gourdon / Deleglise-Rivat parameters as the reference picks them
 * (src/gourdon/pi_gourdon.cpp:44-62, src/util.cpp:222-386). */
pcg_status pcg_gourdon_params(pcg_i128 x, int64_t* y, int64_t* z, int64_t* k,
                              int64_t* x_star);
pcg_status pcg_dr_params(pcg_i128 x, int64_t* y, int64_t* z, int64_t* c);

/* ---- prime counting on top of the engine ---- */

/* pi(x), x < 2^127; -1 semantics are left to the primecount_* wrappers. */
pcg_status pcg_pi(pcg_i128 x, const pcg_opts* opts, pcg_i128* out);
/* The terms of Gourdon's formula for x > 1e10: out6 = {A + C, B, D, Phi0,
 * Sigma, pi(x)} with pi = (A + C) - B + D + Phi0 + Sigma (the reference's
 * --AC, --B, --D, --Phi0, --Sigma options, src/app/main.cpp:465-579). */
pcg_status pcg_pi_terms(pcg_i128 x, const pcg_opts* opts, pcg_i128* out6);
/* pi(x) by the Deleglise-Rivat formula (pi_deleglise_rivat_64/128,
 * src/deleglise-rivat/pi_deleglise_rivat.cpp:61-136; the reference's -d
 * option): pi(y) + S1 + S2_trivial + S2_easy + S2_hard - 1 - P2, S2_hard by
 * the engine.  x <= 1e10 is counted by a sieve. */
pcg_status pcg_pi_deleglise_rivat(pcg_i128 x, const pcg_opts* opts, pcg_i128* out);
/* Its terms for x > 1e10: out7 = {S1, S2_trivial, S2_easy, S2_hard, P2,
 * pi(y), pi(x)} (the reference's --S1, --S2-trivial, --S2-easy, --S2-hard,
 * --P2 options, src/app/main.cpp:325-461), y, z, c as pcg_dr_params. */
pcg_status pcg_pi_dr_terms(pcg_i128 x, const pcg_opts* opts, pcg_i128* out7);
/* phi(x, a): numbers <= x not divisible by any of the first a primes. */
pcg_status pcg_phi(int64_t x, int64_t a, const pcg_opts* opts, int64_t* out);

/* n independent pi(x) queries (x may differ wildly in size). */
pcg_status pcg_pi_batch(const pcg_i128* xs, size_t n, pcg_i128* out,
                        const pcg_opts* opts);
/* n independent phi(x, a) queries. */
pcg_status pcg_phi_batch(const int64_t* x, const int64_t* a, size_t n,
                         int64_t* out, const pcg_opts* opts);

/* ---- libprimecount C API (same names and error convention) ---- */
int64_t primecount_pi(int64_t x);
pcg_i128 primecount_pi_128(pcg_i128 x);
int64_t primecount_phi(int64_t x, int64_t a);
int primecount_get_num_threads(void);
void primecount_set_num_threads(int num_threads);
const char* primecount_version(void);

#ifdef __cplusplus
}
#endif

#endif
