/*
 * pcg_oracle.h -- CPU oracle for the hard-special-leaf engine.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the
 * reference's algorithms for Gourdon's D(x, y, z, k) and Deleglise-Rivat's
 * S2_hard(x, y, z, c) (kimwalisch/primecount 8.7) and of the lookup tables
 * they read.  It is the checker for the CUDA engine: only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.  The
 * product library (libpcgpu) never links or calls it.
 *
 * Parity pin: the restatement is checked against the reference's own
 * golden vectors (test/gourdon/D.cpp:36-89, 51 tuples;
 * test/deleglise-rivat/S2_hard_alpha.cpp:36-73, 35 tuples) and against
 * fixtures produced by the reference binary compiled from its sources by
 * oracle/ref.mk (tests/golden/gen_golden.py).
 *
 * 128-bit integers cross this C ABI as two 64-bit halves (lo, hi), the
 * layout of the reference's pc_int128_t (include/primecount.h:38-41).
 */
#ifndef PCG_ORACLE_H
#define PCG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Work counters of one D / S2_hard evaluation (segmentation independent). */
typedef struct {
  int64_t leaves;          /* hard leaves = calls of the reference's sieve.count() */
  int64_t two_prime_leaves;/* leaves of the second family (p_b * p_l)             */
  int64_t indices_scanned; /* FactorTable entries read by the m filter             */
} ora_stats;

/* D(x, y, z, k), Gourdon.  Reference: src/gourdon/D.cpp:69-308, 382-505.
 * threads <= 1 runs the reference's loop over one chunk [0, x/z) exactly.
 * threads > 1 splits [0, x/z) into chunks; the phi offsets at each chunk
 * start come from a counting pass (the role of phi_vector, phi_vector.cpp).
 * Returns 0 on success, nonzero on invalid arguments. */
int ora_D(uint64_t x_lo, int64_t x_hi, int64_t y, int64_t z, int64_t k,
          int threads, uint64_t* out_lo, int64_t* out_hi, ora_stats* stats);

/* One shard [lo, hi) of D with the phi offsets counted from lo (lo a
 * multiple of 240): the shard's leaf sum, and per level b < ncols the sum of
 * -mu over its leaves (msum) and its survivors at level b (csum).  The
 * shards' results combine as sum_s (sum_s + sum_b msum_s[b] * sum_{s'<s}
 * csum_s'[b]).  Returns 3 when ncols < pi(x_star) + 1. */
int ora_D_partial(uint64_t x_lo, int64_t x_hi, int64_t y, int64_t z, int64_t k, int64_t lo, int64_t hi,
                  uint64_t* out_lo, int64_t* out_hi, int64_t* msum, int64_t* csum, int64_t ncols);

/* S2_hard(x, y, z, c), Deleglise-Rivat.
 * Reference: src/deleglise-rivat/S2_hard.cpp:51-161, 181-293. */
int ora_S2_hard(uint64_t x_lo, int64_t x_hi, int64_t y, int64_t z, int64_t c,
                int threads, uint64_t* out_lo, int64_t* out_hi, ora_stats* stats);

/* CPU baseline: leaves evaluated and wall seconds of the reference's chunk
 * loop over `nchunks` evenly spread sub-intervals (together `fraction` of
 * [0, x/z)), run on `threads` threads. */
int ora_D_sample(uint64_t x_lo, int64_t x_hi, int64_t y, int64_t z, int64_t k,
                 int nchunks, double fraction, int threads, int64_t* leaves, double* seconds);

/* Partial sieve function phi(x, a) by Legendre's recurrence with a small
 * cache (reference semantics: src/phi.cpp:410-430).  Small inputs only. */
int64_t ora_phi(int64_t x, int64_t a);

/* pi(x) by a plain sieve of Eratosthenes (x <= 2^32). */
int64_t ora_pi_sieve(int64_t x);

/* Table builders, for byte-for-byte parity with the device tables.
 * FactorTableD<uint16_t>: src/gourdon/FactorTableD.hpp:78-193.
 * FactorTable<uint16_t> : src/FactorTable.hpp:71-151.
 * PiTable {count, bits} per 240 numbers: src/PiTable.cpp:110-210.
 * out must hold ora_factor_size(limit) / (limit/240+1)*2 entries. */
int64_t ora_factor_size(int64_t limit);
int ora_factor_table_d16(int64_t y, int64_t z, uint16_t* out);
int ora_factor_table_dr16(int64_t y, uint16_t* out);
int ora_pi_table(int64_t max_x, uint64_t* out /* 2 * (max_x/240 + 1) */);

/* Gourdon parameters: y, z, k and x_star exactly as the reference picks them
 * (src/gourdon/pi_gourdon.cpp:44-62, src/util.cpp:276-386).  alpha_y and
 * alpha_z <= 0 select the defaults. */
void ora_gourdon_params(uint64_t x_lo, int64_t x_hi, double alpha_y, double alpha_z,
                        int64_t* y, int64_t* z, int64_t* k, int64_t* x_star);

/* Deleglise-Rivat parameters y, z = x / y, c (src/app/main.cpp:435-461,
 * src/util.cpp:222-263). */
void ora_dr_params(uint64_t x_lo, int64_t x_hi, double alpha,
                   int64_t* y, int64_t* z, int64_t* c);

#ifdef __cplusplus
}
#endif

#endif
