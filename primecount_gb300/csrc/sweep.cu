// sweep.cu -- sm_103a kernels of the hard-special-leaf engine.
//
// What is computed (reference semantics):
//   D(x, y, z, k)      src/gourdon/D.cpp:69-308 (D_thread_default)
//   S2_hard(x, y, z, c) src/deleglise-rivat/S2_hard.cpp:51-161
// Both are sums over "hard special leaves" n = x / (p_b * m) that fall in the
// sieve interval [0, L):  -mu(m) * phi(n, b-1)  (m square-free, lpf(m) > p_b)
// and  +phi(n, b-1) for n = x / (p_b * p_l).
//
// How (GB300 design, not the reference's):
//  * The interval is cut into segments of `words` 64-bit words; each word
//    holds the 64 numbers coprime to 30 of a block of 240 (the reference's
//    BitSieve240 layout, src/sieve/Sieve.hpp:8-12).  One CTA owns one
//    segment in shared memory and sieves it level by level, b = 1, 2, ...
//  * phi(n, b-1) = phi(low-1, b-1) + (# unsieved in [low, n]).  The first
//    term is the only thing that couples segments, and a leaf's contribution
//    is linear in it.  So each (segment, b) records
//        C(s, b)  = # numbers of the segment left after sieving p_1..p_{b-1}
//        M(s, b)  = sum over its leaves of the sign (-mu(m) or +1)
//    and the local counts are summed directly.  A scan over segments then
//    adds sum_b sum_s M(s, b) * sum_{s'<s} C(s', b).  This replaces the
//    reference's per-chunk phi_vector (src/phi_vector.cpp:302-336) and makes
//    every segment independent: no second sieve pass is needed.
//  * Leaf queries are random-order popcount prefix queries.  The counts of
//    the 8-word chunks are kept current by the cross-off; a level's queries
//    read their exclusive prefix, rebuilt by a block scan when the bitmap
//    changed since the last scan, or, for a level with few records, a warp
//    per record sums the chunk counts below it.
//  * Segments are handed out by an atomic counter (device work queue, the
//    role of LoadBalancerS2, src/LoadBalancerS2.cpp:139-193) in waves whose
//    C/M matrices fit a fixed HBM budget.
#include <cstdio>
#include <cstring>
#include <chrono>
#include <algorithm>
#include <atomic>
#include <exception>
#include <mutex>
#include <cmath>
#include <string>
#include <thread>

#include "pcg_internal.hpp"
#include "dev_common.cuh"

namespace pcg {

// ================================================================ prime tables
// PiTable bits: word w holds the primes >= 7 among 240w + {1,7,...}
__global__ void k_prime_bits(uint64_t* __restrict__ out_bits, uint32_t* __restrict__ out_pc,
                             int64_t nwords, int64_t limit,
                             const uint32_t* __restrict__ base, int nbase)
{
  extern __shared__ uint64_t sb[];
  const int WB = 2048;
  int64_t w0 = (int64_t) blockIdx.x * WB;
  int64_t wn = dmin(WB, nwords - w0);
  uint64_t lo = (uint64_t) w0 * 240;
  uint64_t hi = lo + (uint64_t) wn * 240;   // [lo, hi)
  for (int i = threadIdx.x; i < wn; i += blockDim.x) {
    uint64_t v = ~0ull;
    uint64_t wl = lo + (uint64_t) i * 240;
    if (wl + 239 > (uint64_t) limit) v = ((uint64_t) limit >= wl) ? mask_le((uint32_t) (limit - wl)) : 0;
    if (w0 + i == 0) v &= ~1ull;            // 1 is not prime
    sb[i] = v;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int k = warp; k < nbase; k += nw) {
    uint64_t p = base[k];
    if (p * p >= hi) break;
    uint64_t qlo = (lo + p - 1) / p;
    if (qlo < p) qlo = p;
    uint64_t qhi = (hi - 1) / p;
    if (qlo > qhi) continue;
    uint64_t jlo = cnt_le(qlo - 1), jhi = cnt_le(qhi);
    for (uint64_t j = jlo + lane; j < jhi; j += 32) {
      uint64_t q = 30 * (j >> 3) + woff((uint32_t) (j & 7));
      uint32_t off = (uint32_t) (p * q - lo);
      uint32_t w = off / 240, r = off - w * 240;
      atomicAnd((unsigned long long*) &sb[w], ~(1ull << bit_of(r)));
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < wn; i += blockDim.x) {
    out_bits[w0 + i] = sb[i];
    out_pc[w0 + i] = __popcll(sb[i]);
  }
}

// ---- exclusive scan uint32 -> uint64 (three phases)
#define SCAN_ITEMS 4096
__global__ void k_scan_sums(const uint32_t* __restrict__ in, int64_t n, uint64_t* __restrict__ sums)
{
  __shared__ uint64_t red[32];
  int64_t base = (int64_t) blockIdx.x * SCAN_ITEMS;
  uint64_t s = 0;
  for (int i = threadIdx.x; i < SCAN_ITEMS; i += blockDim.x)
    if (base + i < n) s += in[base + i];
  for (int d = 16; d > 0; d >>= 1) s += __shfl_down_sync(0xffffffffu, s, d);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint64_t t = 0;
    for (int i = 0; i < (int) (blockDim.x >> 5); i++) t += red[i];
    sums[blockIdx.x] = t;
  }
}

__global__ void k_scan_serial(uint64_t* sums, int64_t n)
{
  // one block: exclusive scan of n block sums (n is small)
  __shared__ uint64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t base = 0; base < n; base += blockDim.x) {
    int64_t i = base + threadIdx.x;
    uint64_t v = i < n ? sums[i] : 0;
    // inclusive warp scan then block scan
    __shared__ uint64_t wt[32];
    uint64_t incl = v;
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int d = 1; d < 32; d <<= 1) {
      uint64_t t = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += t;
    }
    if (lane == 31) wt[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      uint64_t a = lane < (int) (blockDim.x >> 5) ? wt[lane] : 0;
      uint64_t ai = a;
      for (int d = 1; d < 32; d <<= 1) {
        uint64_t t = __shfl_up_sync(0xffffffffu, ai, d);
        if (lane >= d) ai += t;
      }
      wt[lane] = ai - a;
    }
    __syncthreads();
    uint64_t excl = carry + wt[warp] + incl - v;
    if (i < n) sums[i] = excl;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = excl + v;
    __syncthreads();
  }
}

__global__ void k_scan_apply(const uint32_t* __restrict__ in, int64_t n, const uint64_t* __restrict__ sums,
                             uint64_t* __restrict__ out)
{
  // blockDim.x == 512, 8 items per thread, contiguous
  __shared__ uint64_t wt[16];
  int64_t base = (int64_t) blockIdx.x * SCAN_ITEMS + threadIdx.x * 8;
  uint32_t v[8];
  uint64_t s = 0;
  for (int i = 0; i < 8; i++) { v[i] = (base + i < n) ? in[base + i] : 0; s += v[i]; }
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint64_t incl = s;
  for (int d = 1; d < 32; d <<= 1) {
    uint64_t t = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += t;
  }
  if (lane == 31) wt[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint64_t a = lane < 16 ? wt[lane] : 0, ai = a;
    for (int d = 1; d < 32; d <<= 1) {
      uint64_t t = __shfl_up_sync(0xffffffffu, ai, d);
      if (lane >= d) ai += t;
    }
    if (lane < 16) wt[lane] = ai - a;
  }
  __syncthreads();
  uint64_t run = sums[blockIdx.x] + wt[warp] + incl - s;
  for (int i = 0; i < 8; i++) {
    if (base + i < n) out[base + i] = run;
    run += v[i];
  }
}

// pitab[2w] = 3 + #primes>=7 below 240w, pitab[2w+1] = bits; primes compaction
__global__ void k_pitab_primes(const uint64_t* __restrict__ bits, const uint64_t* __restrict__ excl,
                               int64_t nwords, uint64_t* __restrict__ pitab, uint32_t* __restrict__ primes)
{
  int64_t w = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nwords) return;
  uint64_t b = bits[w];
  uint64_t e = excl[w];
  pitab[2 * w] = 3 + e;
  pitab[2 * w + 1] = b;
  uint64_t idx = 4 + e;   // primes[1..3] = 2, 3, 5
  while (b) {
    int j = __ffsll((long long) b) - 1;
    b &= b - 1;
    primes[idx++] = (uint32_t) (240 * (uint64_t) w + 30 * (j >> 3) + woff(j & 7));
  }
}

// ================================================================ factor tables
// Entries for n = to_number(i) coprime to 2310 (reference layout,
// src/BaseFactorTable.hpp:36-47).  gourdon = 1 builds FactorTableD
// (src/gourdon/FactorTableD.hpp:20-39): 2*pi(lpf) + [mu = -1], T_MAX for a
// prime <= y, T_MAX - 1 for 1, 0 if mu = 0 or a prime factor > y.
// gourdon = 0 builds the Deleglise-Rivat FactorTable (src/FactorTable.hpp:
// 154-166): lpf if mu = -1, lpf - 1 if mu = 1, T_MAX for primes, 0 if mu = 0.
// Method: per block of E entries, every prime p <= sqrt(limit) marks its
// multiples p*q (q coprime to 2310) with shared-memory atomics: minimum
// prime index, product of distinct small primes, factor count and a square
// flag; the cofactor n / product is then the one prime factor > sqrt(limit).
#define FT_E 4096
template <typename T>
__global__ void k_factor(T* __restrict__ out, int64_t size, int64_t limit, int64_t y, int gourdon,
                         const uint32_t* __restrict__ primes, int64_t nsmall,
                         const uint16_t* __restrict__ g_coprime, const int16_t* __restrict__ g_cindex)
{
  extern __shared__ __align__(16) unsigned char fsm[];
  unsigned long long* prod = (unsigned long long*) fsm;
  uint32_t* lpfi = (uint32_t*) (prod + FT_E);
  uint32_t* nf = lpfi + FT_E;          // bits 0..7 count, bit 30 square, bits 8..29 max prime index
  uint16_t* cop = (uint16_t*) (nf + FT_E);
  int16_t* cid = (int16_t*) (cop + 480);
  for (int i = threadIdx.x; i < 480; i += blockDim.x) cop[i] = g_coprime[i];
  for (int i = threadIdx.x; i < 2310; i += blockDim.x) cid[i] = g_cindex[i];
  int64_t i0 = (int64_t) blockIdx.x * FT_E;
  int64_t en = dmin(FT_E, size - i0);
  for (int i = threadIdx.x; i < FT_E; i += blockDim.x) { prod[i] = 1; lpfi[i] = 0xFFFFFFFFu; nf[i] = 0; }
  __syncthreads();
  auto to_number = [&](uint64_t i) -> uint64_t { return 2310 * (i / 480) + cop[i % 480]; };
  auto to_index = [&](uint64_t n) -> int64_t { return 480 * (int64_t) (n / 2310) + cid[n % 2310]; };
  uint64_t nlo = to_number((uint64_t) i0), nhi = to_number((uint64_t) (i0 + en - 1));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  // small primes: index 6 (p = 13) .. nsmall
  for (int64_t k = 6 + warp; k <= nsmall; k += nw) {
    uint64_t p = primes[k];
    uint64_t qlo = (nlo + p - 1) / p;
    uint64_t qhi = nhi / p;
    if (qlo > qhi) continue;
    int64_t jlo = (qlo <= 1) ? 0 : to_index(qlo - 1) + 1;
    int64_t jhi = to_index(qhi);
    for (int64_t j = jlo + lane; j <= jhi; j += 32) {
      uint64_t q = to_number((uint64_t) j);
      uint64_t n = p * q;
      int64_t li = to_index(n) - i0;
      atomicMin(&lpfi[li], (uint32_t) k);
      atomicAdd(&nf[li], 1u);
      if (q % p == 0) atomicOr(&nf[li], 1u << 30);
      unsigned long long old = prod[li], assumed;
      do {
        assumed = old;
        old = atomicCAS(&prod[li], assumed, assumed * p);
      } while (old != assumed);
    }
  }
  __syncthreads();
  const uint64_t TMAX = sizeof(T) == 2 ? 0xFFFFull : 0xFFFFFFFFull;
  for (int i = threadIdx.x; i < en; i += blockDim.x) {
    uint64_t n = to_number((uint64_t) (i0 + i));
    uint64_t v;
    if (n == 1) v = TMAX ^ 1;
    else {
      uint64_t P = prod[i];
      uint64_t large = n / P;
      uint32_t cnt = (nf[i] & 0xFFu) + (large > 1 ? 1u : 0u);
      bool sq = (nf[i] >> 30) & 1u;
      if (sq) v = 0;
      else if (cnt == 1) v = (gourdon && (int64_t) n > y) ? 0 : TMAX;   // n is prime
      else if (gourdon && (int64_t) large > y) v = 0;
      else {
        uint32_t li = lpfi[i];
        if (gourdon) {
          v = 2 * (uint64_t) li + (cnt & 1);
        } else {
          uint64_t lpf = primes[li];
          v = (cnt & 1) ? lpf : lpf - 1;
        }
      }
    }
    out[i0 + i] = (T) v;
  }
}

// Small primes > y (possible only when sqrt(z) > y): zero their multiples.
template <typename T>
__global__ void k_factor_zero_small(T* __restrict__ out, int64_t size, int64_t limit,
                                    const uint32_t* __restrict__ primes, int64_t k_first, int64_t k_last,
                                    const uint16_t* __restrict__ g_coprime, const int16_t* __restrict__ g_cindex)
{
  int64_t k = k_first + blockIdx.x;
  if (k > k_last) return;
  uint64_t p = primes[k];
  for (int64_t j = threadIdx.x; ; j += blockDim.x) {
    uint64_t q = 2310 * (j / 480) + g_coprime[j % 480];
    uint64_t n = p * q;
    if ((int64_t) n > limit) break;
    int64_t li = 480 * (int64_t) (n / 2310) + g_cindex[n % 2310];
    if (li < size) out[li] = 0;
  }
}

// ================================================================ the sweep
struct LevelP {
  union {
    int64_t lo;       // leaf range (lo, hi] while the levels are set up ...
    uint64_t xlo;     // ... then the low word of x / p (flag 16: the high word is not 0)
  };
  int64_t hi;         // factor indices (family 1) or prime indices (family 2)
  uint64_t jlo;       // first 30-coprime rank of the cross-off co-factors
  uint32_t jn;        // number of cross-off co-factors
  uint32_t prime;
  uint32_t thr;       // factor-table threshold (family 1)
  uint32_t flags;     // 1: leaves, 2: family 2, 4: small prime (pattern cross-off), 8: formula count, 16: x / p >= 2^64
  int32_t level;      // b
  uint32_t fcount;    // flag 8: numbers of the segment removed at this level (PiTable formula)
};

// One problem of a sweep: D (gourdon = 1), S2_hard (0) or the special leaves
// of phi(x, a) (2).  A sweep runs the segments of one or of many problems
// (a batch): its work items are the problems' segments one after another,
// problem q owning the items [item0, item0 + nseg).
struct SweepQ {
  uint64_t x_lo, x_hi;
  int64_t y, z, k, L, x_star;
  int64_t item0;         // first work item of the problem
  const int64_t* seglo;  // its segment s = [seglo[s], seglo[s+1])
  const uint64_t* xp_tab;   // [bglob+1][3]: x/p lo, hi, min(x/p^3, 2^63-1)
  int32_t gourdon;
  int32_t pi_sqrt;       // last level of family 1
  int32_t bglob;         // columns = bglob + 1
  int32_t pad0;
};

struct SweepArgs {
  const SweepQ* qs;      // the problems, by item0 ascending
  int32_t nq;
  int32_t words;         // bitmap words per CTA (max segment = words * 240 numbers)
  int32_t rec_cap;       // leaf records per chunk
  int32_t wave_len;
  int64_t wave_first;    // first work item of the wave
  const int64_t* rowoff; // [wave_len]: first cell of the item's row in cnt / smu
  const uint32_t* primes;
  int64_t nprimes;
  const uint64_t* pitab;
  int64_t pi_max;
  const void* factor;
  const uint16_t* coprime;
  const int16_t* cindex;
  const uint64_t* finv;      // floor((2^64 - 1) / m) by factor-table index
  const uint64_t* pmagic;    // floor((2^64 - 1) / p) by prime index
  uint32_t* cnt;            // rows of the wave's items: [rowoff[i], rowoff[i] + bglob + 1)
  int32_t* smu;             // same cells
  int64_t* segsum;          // [wave_len]
  unsigned long long* counters;  // [0] leaves, [1] two-prime leaves, [2] levels, [3] factor entries,
                                 // [4] multiples crossed off
  int* queue;
  int group_max;            // levels answered together (<= GROUP_MAX; < 2: off)
};

// primes 7..61 sieved with wheel patterns (their multiples repeat every p words)
#define NSMALL 15
#define PAT_WORDS 491   // 7+11+13+17+19+23+29+31+37+41+43+47+53+59+61
__constant__ uint32_t c_small_p[NSMALL + 1] = {7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59, 61, 0};

// min(floor(a / d), cap) for d >= 1, cap >= 0, with md = floor((2^64 - 1) / d):
// one high product when a < 2^64
__device__ __forceinline__ int64_t divcap_m(u128 a, uint64_t d, uint64_t md, int64_t cap)
{
  if ((uint64_t) (a >> 64) == 0) {
    const uint64_t q = div_magic((uint64_t) a, d, md);
    return q < (uint64_t) cap ? (int64_t) q : cap;
  }
  return divcap(a, d, cap);
}

// x / m for m < 2^32 when the quotient is known to fit in 63 bits
__device__ __forceinline__ uint64_t div_xp32(uint64_t xlo, uint64_t xhi, uint32_t m)
{
  if (xhi == 0) return xlo / m;
  uint64_t t = (xhi << 32) | (xlo >> 32);
  uint64_t q1 = t / m;
  uint64_t r = t - q1 * m;
  uint64_t t2 = (r << 32) | (xlo & 0xFFFFFFFFull);
  return (q1 << 32) | (t2 / m);
}

__device__ __forceinline__ uint64_t div_xp(uint64_t xlo, uint64_t xhi, uint64_t m)
{
  if (m <= 0xFFFFFFFFull) return div_xp32(xlo, xhi, (uint32_t) m);
  u128 xp = ((u128) xhi << 64) | xlo;
  return (uint64_t) (xp / m);
}

// exclusive prefix of the chunk counts by the first SW warps (nch / SW chunks
// per warp, a multiple of 64; ccount and pref 16-byte aligned); the other
// warps only meet the two barriers
#define SCAN_WARPS 4
__device__ __forceinline__ void scan_chunks(const uint32_t* __restrict__ ccount, uint32_t* __restrict__ pref, int nch,
                                            uint32_t* wtmp)
{
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int cpl = nch / (32 * SCAN_WARPS);             // chunks per lane, a multiple of 2
  const int my = (warp * 32 + lane) * cpl;
  uint32_t sum = 0, incl = 0;
  if (warp < SCAN_WARPS) {
    for (int i = 0; i < cpl; i += 2) {
      const uint2 v = *(const uint2*) (ccount + my + i);
      sum += v.x + v.y;
    }
    incl = sum;
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += t;
    }
    if (lane == 31) wtmp[warp] = incl;
  }
  __syncthreads();
  if (warp < SCAN_WARPS) {
    uint32_t run = incl - sum;
    for (int w = 0; w < warp; w++) run += wtmp[w];
    for (int i = 0; i < cpl; i += 2) {
      const uint2 v = *(const uint2*) (ccount + my + i);
      uint2 o;
      o.x = run; run += v.x;
      o.y = run; run += v.y;
      *(uint2*) (pref + my + i) = o;
    }
  }
  __syncthreads();
}

// mask_le(r) from a shared table of the counts of wheel residues <= r
static __device__ __forceinline__ uint64_t mask_le_t(const uint8_t* nbt, uint32_t r) { return low_bits(nbt[r]); }

// dpi with the shared residue-count table
static __device__ __forceinline__ int64_t dpi_t(const uint64_t* __restrict__ pt, const uint8_t* nbt, uint64_t x)
{
  if (x < 6) return (0x322100u >> (4 * x)) & 15u;
  const uint64_t i = x / 240;
  return (int64_t) (pt[2 * i] + __popcll(pt[2 * i + 1] & mask_le_t(nbt, (uint32_t) (x - 240 * i))));
}

// # unsieved numbers in [low, low + off]: the chunk prefix plus the popcounts
// of the chunk's words up to the word of off, its 8 words read at once
__device__ __forceinline__ uint32_t query(const uint64_t* __restrict__ bits, const uint32_t* __restrict__ pref,
                                          const uint8_t* nbt, uint32_t off)
{
  const uint32_t w = off / 240;
  const uint32_t r = off - w * 240;
  const uint32_t c = w >> 3;
  const uint32_t k = w & 7;
  const ulonglong2* q = (const ulonglong2*) (bits + (c << 3));
  const ulonglong2 w01 = q[0], w23 = q[1], w45 = q[2], w67 = q[3];
  const uint64_t mk = mask_le_t(nbt, r);
  auto part = [&](uint32_t i, uint64_t v) -> uint32_t {
    return (uint32_t) __popcll(i < k ? v : (i == k ? (v & mk) : 0ull));
  };
  return pref[c] + part(0, w01.x) + part(1, w01.y) + part(2, w23.x) + part(3, w23.y) + part(4, w45.x) +
         part(5, w45.y) + part(6, w67.x) + part(7, w67.y);
}

// This lane's part of the sum of the chunk counts [0, ch): the lane takes the
// 4-chunk groups lane, lane + 32, ... (16-byte loads, ch <= the number of
// chunks, a multiple of 4), four groups' loads in flight together
__device__ __forceinline__ uint32_t chunk_sum_below(const uint32_t* __restrict__ ccount, uint32_t ch, int lane)
{
  uint32_t part = 0;
  for (uint32_t i0 = 0; i0 < ch; i0 += 512) {
    uint4 v[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const uint32_t i = i0 + 128 * u + 4 * lane;
      v[u] = i < ch ? *(const uint4*) (ccount + i) : make_uint4(0u, 0u, 0u, 0u);
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const uint32_t i = i0 + 128 * u + 4 * lane;
      part += v[u].x + (i + 1 < ch ? v[u].y : 0u) + (i + 2 < ch ? v[u].z : 0u) + (i + 3 < ch ? v[u].w : 0u);
    }
  }
  return part;
}

// Cross off the number at offset w * 240 + rr of the segment: a 32-bit atomic
// on the half of the 64-bit word that holds its bit (bits 0-31 of a word are
// the lower half), true when the number was still unsieved
__device__ __forceinline__ bool cross_off(uint64_t* bits, const uint8_t* bt, uint32_t w, uint32_t rr)
{
  const uint32_t bi = bt[rr];
  const uint32_t m = 1u << (bi & 31);
  return (atomicAnd((uint32_t*) bits + 2 * w + (bi >> 5), ~m) & m) != 0;
}

// Cross off the multiples of the levels [l0, l1) at once (their co-factor
// counts prefixed in hoff): with few multiples per level a warp takes each
// level and its lanes the level's multiples; otherwise the multiples are
// spread flat over the threads, each finding its level by a binary search.
// Different levels can share a half-word, so the clears are atomic.
template <int NT>
__device__ __forceinline__ void cross_off_levels(uint64_t* bits, uint32_t* ccount, const LevelP* lp,
                                                 const int64_t* hoff, int l0, int l1, uint64_t low,
                                                 const uint8_t* bt)
{
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t h0 = hoff[l0], h1 = hoff[l1];
  if (h1 - h0 <= 64 * (int64_t) (l1 - l0)) {
    for (int lv = l0 + warp; lv < l1; lv += NT / 32) {
      const uint64_t prime = lp[lv].prime, jlo = lp[lv].jlo;
      const uint32_t jn = (uint32_t) (hoff[lv + 1] - hoff[lv]);
      for (uint32_t j = lane; j < jn; j += 32) {
        const uint64_t jj = jlo + j;
        const uint64_t q = 30 * (jj >> 3) + woff((uint32_t) (jj & 7));
        const uint32_t off = (uint32_t) (prime * q - low);
        const uint32_t w = off / 240, rr = off - w * 240;
        if (cross_off(bits, bt, w, rr)) atomicSub(&ccount[w >> 3], 1u);
      }
    }
    return;
  }
  for (int64_t h = h0 + tid; h < h1; h += NT) {
    int lo = l0, hi = l1 - 1;       // last level with hoff <= h
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (hoff[mid] <= h) lo = mid; else hi = mid - 1;
    }
    const LevelP& Q = lp[lo];
    const uint64_t jj = Q.jlo + (uint64_t) (h - hoff[lo]);
    const uint64_t q = 30 * (jj >> 3) + woff((uint32_t) (jj & 7));
    const uint32_t off = (uint32_t) ((uint64_t) Q.prime * q - low);
    const uint32_t w = off / 240, rr = off - w * 240;
    if (cross_off(bits, bt, w, rr)) atomicSub(&ccount[w >> 3], 1u);
  }
}

// Record of one table entry: the offset of the leaf in the segment, bit 30 =
// negative sign, or REC_NONE when the factor-table filter rejects the entry.
#define REC_NONE 0xFFFFFFFFu
// table entries per thread and round of the record phase
#define PA_UNROLL 8
// levels (and groups of levels) with at most this many record slots in a
// window are answered without a chunk prefix scan
#ifndef SMALL_QUERIES
#define SMALL_QUERIES 32
#endif
// consecutive levels with p^3 >= high answered together (see k_sweep)
#define GROUP_MAX 64

// exclusive block scan of three int64 values per thread into out[NT + 1] arrays
template <int NT>
__device__ __forceinline__ void block_scan3(long long v0, long long v1, long long v2, int64_t* o0, int64_t* o1,
                                            int64_t* o2, long long (*wt)[3])
{
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  long long i0 = v0, i1 = v1, i2 = v2;
  for (int d = 1; d < 32; d <<= 1) {
    long long t0 = __shfl_up_sync(0xffffffffu, i0, d);
    long long t1 = __shfl_up_sync(0xffffffffu, i1, d);
    long long t2 = __shfl_up_sync(0xffffffffu, i2, d);
    if (lane >= d) { i0 += t0; i1 += t1; i2 += t2; }
  }
  if (lane == 31) { wt[warp][0] = i0; wt[warp][1] = i1; wt[warp][2] = i2; }
  __syncthreads();
  long long e0 = i0 - v0, e1 = i1 - v1, e2 = i2 - v2;
  for (int w = 0; w < warp; w++) { e0 += wt[w][0]; e1 += wt[w][1]; e2 += wt[w][2]; }
  o0[tid] = e0; o1[tid] = e1; o2[tid] = e2;
  if (tid == NT - 1) { o0[NT] = e0 + v0; o1[NT] = e1 + v1; o2[NT] = e2 + v2; }
}

// the level j in [l0, l1) of flat record pos: loff[j] <= pos < loff[j + 1]
// (loff[l0] <= pos < loff[l1]), by binary search
static __device__ __forceinline__ int level_of(const int64_t* loff, int l0, int l1, int64_t pos)
{
  int j = l0;
  for (int n = l1 - l0; n > 1;) {
    const int half = n >> 1;
    if (loff[j + half] <= pos) j += half;
    n -= half;
  }
  return j;
}

template <typename FT, int NT>
__global__ void __launch_bounds__(NT, (NT >= 512) ? 1 : ((NT >= 256) ? 2 : 4)) k_sweep(const SweepArgs A)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nch = A.words >> 3;
  uint64_t* bits = (uint64_t*) smem_raw;
  uint64_t* pat = bits + A.words;                      // wheel patterns of the primes 7..61
  int64_t* loff = (int64_t*) (pat + PAT_WORDS);        // record offsets of the batch levels
  int64_t* hoff = loff + (NT + 1);                     // cross-off co-factor offsets
  int64_t* rpre = hoff + (NT + 1);                     // prefix of the formula counts
  uint32_t* ccount = (uint32_t*) (((uintptr_t) (rpre + (NT + 1)) + 15) & ~(uintptr_t) 15);  // 16-byte aligned
  uint32_t* pref = ccount + nch;
  LevelP* lp = (LevelP*) (pref + nch);
  uint32_t* rec = (uint32_t*) (lp + NT);
  uint16_t* runend = (uint16_t*) (rec + A.rec_cap);    // end of the run of leafless levels from i
  uint16_t* cop = runend + NT;
  uint32_t* s_pc = (uint32_t*) (((uintptr_t) (cop + 480) + 3) & ~(uintptr_t) 3);   // pi(q_lo - 1) of flag-8 levels

  __shared__ int s_ws;
  __shared__ uint32_t wtmp[32];
  __shared__ int s_gsmu[GROUP_MAX];                    // signed leaf counts of a level group
  __shared__ uint64_t s_gmag[GROUP_MAX];               // reciprocals of the group's primes
  __shared__ int s_smu;
  __shared__ int s_ncomp[2];                           // accepted records of a compacted window, by window parity
  __shared__ int s_stop;
  __shared__ uint32_t s_rem[3];
  __shared__ uint32_t s_total;
  __shared__ uint64_t s_mlow, s_mhigh;                 // floor((2^64 - 1) / d) of low1 and high
  __shared__ long long wt3[32][3];
  __shared__ int s_brk[32];
  __shared__ long long s_red[NT / 32];
  __shared__ unsigned long long s_ctr[5];

  __shared__ SweepQ s_q;                               // the problem of the current segment
  __shared__ uint8_t s_nb[240];                        // # wheel residues <= r, r in [0, 240)
  __shared__ uint8_t s_bitt[240];                      // bit of residue r in its 64-bit word (r coprime to 30)
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int cap = A.rec_cap;
  const FT* __restrict__ factor = (const FT*) A.factor;
  for (int i = tid; i < 480; i += NT) cop[i] = A.coprime[i];
  for (int i = tid; i < 240; i += NT) {
    s_nb[i] = (uint8_t) ((i / 30) * 8 + cnt8((uint32_t) (i % 30)));
    s_bitt[i] = (uint8_t) bit_of((uint32_t) i);
  }
  // wheel patterns: word r of prime p keeps the numbers 240 r + {1,7,..,29}
  // (mod 240 p) that p does not divide
  for (int i = tid; i < PAT_WORDS; i += NT) {
    int k = 0, base = 0;
    while (k < NSMALL - 1 && i >= base + c_small_p[k]) { base += c_small_p[k]; k++; }
    const uint32_t p = c_small_p[k];
    const uint32_t r = (uint32_t) (i - base);
    uint64_t w = ~0ull;
    for (int j = 0; j < 64; j++) {
      const uint32_t v = 240 * r + 30 * (j >> 3) + woff(j & 7);
      if (v % p == 0) w &= ~(1ull << j);
    }
    pat[i] = w;
  }
  if (tid < 5) s_ctr[tid] = 0;

  for (;;) {
    __syncthreads();
    if (tid == 0) s_ws = atomicAdd(A.queue, 1);
    __syncthreads();
    const int ws = s_ws;
    if (ws >= A.wave_len) break;
    const int64_t item = A.wave_first + ws;
    if (tid == 0) {
      // the problem owning the item: the last with item0 <= item
      int lo = 0, hi = A.nq - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (A.qs[mid].item0 <= item) lo = mid; else hi = mid - 1;
      }
      s_q = A.qs[lo];
    }
    __syncthreads();
    const SweepQ& PQ = s_q;
    const u128 x = ((u128) PQ.x_hi << 64) | PQ.x_lo;
    const int64_t rowbase = A.rowoff[ws];
    const int64_t s = item - PQ.item0;
    const int64_t low = PQ.seglo[s];
    const int64_t high = PQ.seglo[s + 1];
    const int64_t low1 = dmax(low, 1);

    // level bounds of this segment (chunk bounds of D.cpp:83-94 / S2_hard.cpp:64-71)
    int64_t bmin_leaf, bmax_leaf, bcnt;
    if (PQ.gourdon == 2) {
      // phi(x, a) special leaves: p_b <= p_a (held in x_star), m <= y
      bmax_leaf = dpi(A.pitab, (uint64_t) dmin(disqrt(div128(x, (uint64_t) low1)), PQ.x_star));
      bmin_leaf = dpi(A.pitab, (uint64_t) dmin(PQ.L / high, PQ.x_star));
      bcnt = dpi(A.pitab, (uint64_t) dmin(disqrt(div128(x, (uint64_t) high)), PQ.x_star));
    } else if (PQ.gourdon) {
      bmax_leaf = dpi(A.pitab, (uint64_t) dmin(dmin(disqrt(div128(x, (uint64_t) low1)), disqrt((u128) high)), PQ.x_star));
      bmin_leaf = dpi(A.pitab, (uint64_t) dmin(PQ.L / high, PQ.x_star));
      bcnt = dpi(A.pitab, (uint64_t) dmin(disqrt(div128(x, (uint64_t) high)), PQ.x_star));
    } else {
      bmax_leaf = (high <= PQ.y) ? PQ.pi_sqrt
          : dpi(A.pitab, (uint64_t) dmin(dmin(disqrt(div128(x, (uint64_t) low1)), disqrt((u128) PQ.z)), PQ.y));
      uint64_t pmax = bmax_leaf > 0 ? A.primes[bmax_leaf] : 0;
      bmin_leaf = dpi(A.pitab, (uint64_t) dmin(PQ.z / high, (int64_t) pmax));
      bcnt = dmax(PQ.pi_sqrt, dpi(A.pitab, (uint64_t) dmin(dmin(disqrt(div128(x, (uint64_t) high)), disqrt((u128) PQ.z)), PQ.y)));
    }
    bmin_leaf = dmax(PQ.k, bmin_leaf) + 1;
    const int Bs = (int) dmin(dmax(bmax_leaf, bcnt), (int64_t) PQ.bglob);

    // fill the segment: every number coprime to 30 in [low, high)
    const uint32_t span = (uint32_t) (high - low);
    const int wused = (int) ((span + 239) / 240);
    for (int w = tid; w < A.words; w += NT) {
      uint64_t v = w < wused ? ~0ull : 0ull;
      if (w == wused - 1) v &= mask_le((span - 1) % 240);
      bits[w] = v;
    }
    if (tid == 0) {
      s_total = 0; s_rem[0] = s_rem[1] = s_rem[2] = 0; s_smu = 0; s_stop = 0x7FFFFFFF;
      s_mlow = UINT64_MAX / (uint64_t) low1;
      s_mhigh = UINT64_MAX / (uint64_t) high;
      s_ncomp[0] = s_ncomp[1] = 0;
    }
    __syncthreads();
    {
      uint32_t part = 0;
      for (int c = tid; c < nch; c += NT) {
        uint32_t t = 0;
        for (int i = 0; i < 8; i++) t += __popcll(bits[8 * c + i]);
        ccount[c] = t;
        part += t;
      }
      part = __reduce_add_sync(0xffffffffu, part);
      if (lane == 0) atomicAdd(&s_total, part);
    }
    __syncthreads();
    uint32_t total = s_total;
    bool dirty = true;
    long long lsum = 0;
    unsigned long long nleaves = 0, ntwo = 0, nentries = 0;
    unsigned win = 0;      // windows of the segment so far (parity selects the compaction counter)

    for (int b0 = 1; b0 <= Bs; b0 += NT) {
      // ---- per-level parameters of levels b0 .. b0+NT-1, one thread each
      int64_t E = 0;
      uint32_t fcnt = 0;
      {
        const int b = b0 + tid;
        LevelP P;
        P.lo = P.hi = 0; P.jlo = 0; P.jn = 0; P.prime = 0; P.thr = 0; P.flags = 0; P.level = b; P.fcount = 0;
        uint32_t pcv = 0;
        uint32_t ncross = 0;   // multiples of p_b in the segment (work counter)
        if (b <= Bs) {
          const uint64_t p = A.primes[b];
          const uint64_t pm = A.pmagic[b];     // floor((2^64 - 1) / p): the divisions by p below
          P.prime = (uint32_t) p;
          if (p >= 64) {
            uint64_t qlo = div_magic((uint64_t) low + p - 1, p, pm);
            if (qlo < 1) qlo = 1;
            uint64_t qhi = div_magic((uint64_t) high - 1, p, pm);
            if (qlo <= qhi) {
              P.jlo = cnt_le(qlo - 1);
              P.jn = (uint32_t) (cnt_le(qhi) - P.jlo);
            }
            // p^3 >= high: the numbers of the segment whose least prime factor
            // is p are p itself and p*q for primes q >= p, so the count of
            // level b follows from the PiTable
            if ((u128) p * p * p >= (u128) high && (int64_t) qhi <= A.pi_max) {
              uint32_t f = ((uint64_t) low <= p && p < (uint64_t) high) ? 1u : 0u;
              const uint64_t qa = qlo > p ? qlo : p;
              const int64_t pc = dpi(A.pitab, qa - 1);
              if (qhi >= qa) f += (uint32_t) (dpi(A.pitab, qhi) - pc);
              P.fcount = f;
              P.flags |= 8;
              pcv = (uint32_t) pc;
            }
          } else if (p >= 7) {
            P.jlo = (uint64_t) ((low / 240) % p);   // pattern phase of the first word
            P.flags |= 4;
            // its multiples in the segment, for the work counter only
            uint64_t qlo = ((uint64_t) low + p - 1) / p;
            if (qlo < 1) qlo = 1;
            const uint64_t qhi = ((uint64_t) high - 1) / p;
            if (qlo <= qhi) ncross = (uint32_t) (cnt_le(qhi) - cnt_le(qlo - 1));
          }
          if (p >= 64) ncross = P.jn;
          if (b >= bmin_leaf && b <= bmax_leaf) {
            const uint64_t* xt = PQ.xp_tab + 3 * b;
            const u128 xp = ((u128) xt[1] << 64) | xt[0];
            const int64_t xpp = (int64_t) xt[2];
            const int64_t prime = (int64_t) p;
            bool stop = false;
            if (b <= PQ.pi_sqrt) {
              int64_t min_m, max_m;
              if (PQ.gourdon == 2) {
                // phi(x, a): m in (max(y / p, x / (p high), p), min(y, x / (p low))]; the
                // bound m > p matters once p^2 > y, where the primes m in (y / p, p]
                // would pass the table's filter (a prime's entry is T_MAX)
                int64_t xp_high = divcap_m(xp, (uint64_t) high, s_mhigh, PQ.y);
                min_m = dmax(dmax(xp_high, (int64_t) div_magic((uint64_t) PQ.y, p, pm)), prime);
                max_m = divcap_m(xp, (uint64_t) low1, s_mlow, PQ.y);
                P.thr = (uint32_t) (2 * b + 1);
              } else if (PQ.gourdon) {
                int64_t xp_low = divcap_m(xp, (uint64_t) low1, s_mlow, PQ.z);
                int64_t xp_high = divcap_m(xp, (uint64_t) high, s_mhigh, PQ.z);
                min_m = dmax(xp_high, (int64_t) div_magic((uint64_t) PQ.z, p, pm));
                max_m = dmin(xpp, xp_low);
                P.thr = (uint32_t) (2 * b + 1);
              } else {
                int64_t xp_high = divcap_m(xp, (uint64_t) high, s_mhigh, PQ.y);
                min_m = dmax(xp_high, (int64_t) div_magic((uint64_t) PQ.y, p, pm));
                max_m = divcap_m(xp, (uint64_t) low1, s_mlow, PQ.y);
                P.thr = (uint32_t) prime;
              }
              if (prime >= max_m) stop = true;
              else {
                P.lo = 480 * (min_m / 2310) + A.cindex[min_m % 2310];
                P.hi = 480 * (max_m / 2310) + A.cindex[max_m % 2310];
                if (P.hi > P.lo) P.flags |= 1;
              }
            } else {
              int64_t xp_low = divcap_m(xp, (uint64_t) low1, s_mlow, PQ.y);
              int64_t xp_high = divcap_m(xp, (uint64_t) high, s_mhigh, PQ.y);
              int64_t l, min_hard;
              if (PQ.gourdon) {
                int64_t max_m = dmin(xpp, xp_low);
                l = dpi(A.pitab, (uint64_t) max_m);
                min_hard = dmax(xp_high, prime);
              } else {
                l = dpi(A.pitab, (uint64_t) dmin(xp_low, (int64_t) div_magic((uint64_t) PQ.z, p, pm)));
                min_hard = dmax(xp_high, prime);
              }
              if (prime >= (int64_t) A.primes[l]) stop = true;
              else {
                P.lo = dpi(A.pitab, (uint64_t) dmin(min_hard, A.pi_max));
                P.hi = l;
                if (P.hi > P.lo) P.flags |= 3;
              }
            }
            if (stop) atomicMin(&s_stop, b);
            if (P.flags & 1) {
              E = P.hi - P.lo;
              P.xlo = xt[0];
              if (xt[1]) P.flags |= 16;
            }
          }
        }
        fcnt = P.fcount;
        lp[tid] = P;
        s_pc[tid] = pcv;
        ncross = __reduce_add_sync(0xffffffffu, ncross);
        if (lane == 0 && ncross) atomicAdd(&s_ctr[4], (unsigned long long) ncross);
      }
      __syncthreads();
      const int nb = (int) dmin(NT, (int64_t) (Bs - b0 + 1));
      {
        // goto next_segment (D.cpp:131-132): no leaves from s_stop on
        const bool has_leaves = (b0 + tid < s_stop) && E > 0;
        if (!has_leaves) E = 0;
        const uint32_t jn = lp[tid].jn;
        // flat offsets of records, run cross-off co-factors and formula counts
        block_scan3<NT>(E, (lp[tid].flags & 8) ? (long long) jn : 0, (long long) fcnt, loff, hoff, rpre, wt3);
        // runs: levels without leaves whose count follows from the formula
        const bool breaker = (tid >= nb) || has_leaves || !(lp[tid].flags & 8);
        const unsigned bal = __ballot_sync(0xffffffffu, breaker);
        if (lane == 0) s_brk[warp] = bal ? warp * 32 + __ffs((int) bal) - 1 : NT;
        __syncthreads();
        const unsigned mine = bal & (0xffffffffu << lane);
        int re;
        if (mine) re = warp * 32 + __ffs((int) mine) - 1;
        else {
          re = NT;
          for (int w2 = warp + 1; w2 < NT / 32; w2++)
            if (s_brk[w2] < NT) { re = s_brk[w2]; break; }
        }
        runend[tid] = (uint16_t) dmin(re, nb);
        __syncthreads();
      }
      const int64_t total_e = loff[nb];
      // FactorTable entries read: every record of the batch's levels is
      // read once by the windows below (two-prime levels read primes instead)
      if (tid < nb && !(lp[tid].flags & 2)) nentries += (unsigned long long) (loff[tid + 1] - loff[tid]);

      int li = 0;          // next batch level to finish
      int64_t w0 = 0;      // first flat record of the window
      while (li < nb) {
        const int64_t wend = w0 + cap;
        win++;
        // ---- phase A: the window's leaf records, flat over levels, PA_UNROLL
        // entries per thread in three stages so that their table loads, then
        // their reciprocal loads, are in flight together
        const int nrec = (int) dmax(0, dmin(wend, total_e) - w0);
        // a window inside one level (the dense case): that level's constants
        // held in registers, no level lookup per entry
        const bool one_level = nrec > 0 && loff[li] <= w0 && loff[li + 1] >= w0 + nrec;
        // a window of one level of FactorTable entries whose records are all
        // answered by the per-level path: the accepted records are compacted
        // to the front (their order is free, all are answered against one
        // bitmap state), the rejected ones are dropped
        const bool compact = one_level && !(lp[li].flags & 2) && (loff[li] < w0 || !(lp[li].flags & 8));
        const int clev = compact ? li : -1;                // the level whose records are compacted
        if (tid == 0) s_ncomp[(win + 1) & 1] = 0;
        if (one_level) {
          const LevelP& Q = lp[li];
          const int64_t hi0 = Q.hi - (w0 - loff[li]);        // table index of entry f is hi0 - f
          const bool two = (Q.flags & 2) != 0;
          const uint32_t thr = Q.thr;
          const uint64_t* xt = PQ.xp_tab + 3 * (int64_t) Q.level;
          const uint64_t xlo = xt[0], xhi = xt[1];
          unsigned nl = 0;
          if (compact && hi0 < 0x7FFFFFFFll) {
            // filter first: the accepted entries' indices (bit 31: negative
            // sign) are compacted, then their reciprocals loaded and their
            // divisions done on full warps (about 1/3 of the entries pass)
            for (int f0 = tid; f0 - lane < nrec; f0 += PA_UNROLL * NT) {
              uint32_t fv[PA_UNROLL];
#pragma unroll
              for (int u = 0; u < PA_UNROLL; u++) {
                const int f = f0 + u * NT;
                fv[u] = f < nrec ? (uint32_t) __ldg(&factor[hi0 - f]) : 0u;
              }
              unsigned bal[PA_UNROLL];
              int tot = 0;
#pragma unroll
              for (int u = 0; u < PA_UNROLL; u++) {
                bal[u] = __ballot_sync(0xffffffffu, f0 + u * NT < nrec && fv[u] > thr);
                tot += __popc(bal[u]);
              }
              int base = 0;
              if (lane == 0 && tot) base = atomicAdd(&s_ncomp[win & 1], tot);
              base = __shfl_sync(0xffffffffu, base, 0);
              const unsigned lt = (1u << lane) - 1u;
              int pos = base;
#pragma unroll
              for (int u = 0; u < PA_UNROLL; u++) {
                if ((bal[u] >> lane) & 1u)
                  rec[pos + __popc(bal[u] & lt)] =
                      (uint32_t) (hi0 - (f0 + u * NT)) | ((fv[u] & 1u) ? 0u : 0x80000000u);
                pos += __popc(bal[u]);
              }
              __syncwarp();
              for (int j0 = 0; j0 < tot; j0 += 32 * 4) {
                uint32_t e[4];
                uint64_t mv[4];
#pragma unroll
                for (int d = 0; d < 4; d++) {
                  const int j = j0 + 32 * d + lane;
                  e[d] = j < tot ? rec[base + j] : 0u;
                  mv[d] = (j < tot && xhi == 0) ? __ldg(&A.finv[e[d] & 0x7FFFFFFFu]) : 0ull;
                }
#pragma unroll
                for (int d = 0; d < 4; d++) {
                  const int j = j0 + 32 * d + lane;
                  if (j < tot) {
                    const uint32_t mi = e[d] & 0x7FFFFFFFu;
                    const uint64_t m = 2310ull * (mi / 480u) + cop[mi % 480u];
                    const uint64_t nn = xhi == 0 ? div_magic(xlo, m, mv[d]) : div_xp(xlo, xhi, m);
                    uint32_t r = (uint32_t) (nn - (uint64_t) low);
                    if (e[d] & 0x80000000u) r |= 1u << 30;
                    rec[base + j] = r;
                  }
                }
              }
              if (lane == 0) nl += (unsigned) tot;
            }
          } else
          // f0 - lane is the same for the lanes of a warp: the loop is warp-uniform
          for (int f0 = tid; f0 - lane < nrec; f0 += PA_UNROLL * NT) {
            uint32_t fv[PA_UNROLL];
            uint64_t minv[PA_UNROLL];
#pragma unroll
            for (int u = 0; u < PA_UNROLL; u++) {
              const int f = f0 + u * NT;
              fv[u] = 0;
              minv[u] = 0;
              if (f < nrec) {
                const int64_t idx = hi0 - f;
                if (two) {
                  fv[u] = __ldg(&A.primes[idx]);
                  minv[u] = __ldg(&A.pmagic[idx]);
                } else {
                  fv[u] = (uint32_t) __ldg(&factor[idx]);
                  minv[u] = __ldg(&A.finv[idx]);
                }
              }
            }
            uint32_t rv[PA_UNROLL];
#pragma unroll
            for (int u = 0; u < PA_UNROLL; u++) {
              const int f = f0 + u * NT;
              rv[u] = REC_NONE;
              if (f < nrec) {
                const int64_t idx = hi0 - f;
                uint64_t m = 0;
                if (two) m = fv[u];
                else if (fv[u] > thr) {
                  if ((uint64_t) idx <= 0xFFFFFFFFull) {
                    const uint32_t mi = (uint32_t) idx;
                    m = 2310ull * (mi / 480u) + cop[mi % 480u];
                  } else {
                    m = 2310ull * ((uint64_t) idx / 480) + cop[(uint64_t) idx % 480];
                  }
                }
                if (m) {
                  const uint64_t nn = xhi == 0 ? div_magic(xlo, m, minv[u]) : div_xp(xlo, xhi, m);
                  uint32_t r = (uint32_t) (nn - (uint64_t) low);
                  if (!two && !(fv[u] & 1)) r |= 1u << 30;
                  rv[u] = r;
                  nl++;
                }
                if (!compact) rec[f] = rv[u];
              }
            }
            if (compact) {
              // one shared counter update per warp for its PA_UNROLL x 32 entries
              unsigned bal[PA_UNROLL];
              int tot = 0;
#pragma unroll
              for (int u = 0; u < PA_UNROLL; u++) {
                bal[u] = __ballot_sync(0xffffffffu, rv[u] != REC_NONE);
                tot += __popc(bal[u]);
              }
              int base = 0;
              if (lane == 0 && tot) base = atomicAdd(&s_ncomp[win & 1], tot);
              base = __shfl_sync(0xffffffffu, base, 0);
              const unsigned lt = (1u << lane) - 1u;
#pragma unroll
              for (int u = 0; u < PA_UNROLL; u++) {
                if (rv[u] != REC_NONE) rec[base + __popc(bal[u] & lt)] = rv[u];
                base += __popc(bal[u]);
              }
            }
          }
          nleaves += nl;
          if (two) ntwo += nl;
        }
        if (nrec > 0 && !one_level) {
          // the window's records belong to levels li .. lw
          int lw = li;
          {
            const int64_t last = w0 + nrec - 1;
            int hi = nb - 1;
            while (lw < hi) {
              const int mid = (lw + hi + 1) >> 1;
              if (loff[mid] <= last) lw = mid; else hi = mid - 1;
            }
          }
          for (int f0 = tid; f0 < nrec; f0 += PA_UNROLL * NT) {
            int jl[PA_UNROLL];
            int el[PA_UNROLL];
            uint32_t fv[PA_UNROLL];
            // the level of each entry, the last with loff <= its position: a
            // branch-free binary search over li .. lw, the entries' searches
            // interleaved so that their shared-memory loads overlap
#pragma unroll
            for (int u = 0; u < PA_UNROLL; u++) jl[u] = li;
            for (int n = lw - li + 1; n > 1;) {
              const int half = n >> 1;
#pragma unroll
              for (int u = 0; u < PA_UNROLL; u++) {
                const int64_t pos = w0 + min(f0 + u * NT, nrec - 1);
                const int c = jl[u] + half;
                jl[u] = loff[c] <= pos ? c : jl[u];
              }
              n -= half;
            }
#pragma unroll
            for (int u = 0; u < PA_UNROLL; u++) {
              const int f = f0 + u * NT;
              el[u] = (int) (w0 + f - loff[jl[u]]);
              fv[u] = 0;
              if (f >= nrec) jl[u] = -1;
            }
            // table entries and the reciprocals of their divisors, loaded
            // together (the reciprocal of a rejected entry goes unused)
            uint64_t mdiv[PA_UNROLL], minv[PA_UNROLL];
#pragma unroll
            for (int u = 0; u < PA_UNROLL; u++) {
              minv[u] = 0;
              if (jl[u] >= 0) {
                const LevelP& Q = lp[jl[u]];
                const int64_t idx = Q.hi - el[u];
                if (Q.flags & 2) {
                  fv[u] = __ldg(&A.primes[idx]);
                  minv[u] = __ldg(&A.pmagic[idx]);
                } else {
                  fv[u] = (uint32_t) __ldg(&factor[idx]);
                  minv[u] = __ldg(&A.finv[idx]);
                }
              }
            }
            // the divisor m of each accepted entry (0: rejected by the
            // factor-table filter)
#pragma unroll
            for (int u = 0; u < PA_UNROLL; u++) {
              mdiv[u] = 0;
              if (jl[u] >= 0) {
                const LevelP& Q = lp[jl[u]];
                const int64_t idx = Q.hi - el[u];
                if (Q.flags & 2) {
                  mdiv[u] = fv[u];
                } else if (fv[u] > Q.thr) {
                  if ((uint64_t) idx <= 0xFFFFFFFFull) {
                    const uint32_t mi = (uint32_t) idx;
                    mdiv[u] = 2310ull * (mi / 480u) + cop[mi % 480u];
                  } else {
                    mdiv[u] = 2310ull * ((uint64_t) idx / 480) + cop[(uint64_t) idx % 480];
                  }
                }
              }
            }
            // n = (x / p) / m, the record: offset in the segment, bit 30 for
            // the negative sign of -mu(m) (an even factor-table entry)
#pragma unroll
            for (int u = 0; u < PA_UNROLL; u++) {
              const int f = f0 + u * NT;
              if (jl[u] >= 0) {
                const LevelP& Q = lp[jl[u]];
                uint32_t r = REC_NONE;
                if (mdiv[u]) {
                  const uint64_t nn = (Q.flags & 16) ? div_xp(Q.xlo, PQ.xp_tab[3 * (int64_t) Q.level + 1], mdiv[u])
                                                     : div_magic(Q.xlo, mdiv[u], minv[u]);
                  r = (uint32_t) (nn - (uint64_t) low);
                  if (!(Q.flags & 2) && !(fv[u] & 1)) r |= 1u << 30;
                  nleaves++;
                  if (Q.flags & 2) ntwo++;
                }
                rec[f] = r;
              }
            }
          }
        }
        if (nrec > 0) __syncthreads();
        // ---- phase B: levels in order
        while (li < nb) {
          // the level's shared-memory fields, loaded together
          const int re = runend[li];
          const uint32_t lflags = lp[li].flags;
          const int64_t la = loff[li], lz = loff[li + 1];
          if (re > li) {
            // a run of leafless levels li .. re-1 with formula counts: their
            // counts from the prefix, all their multiples crossed off at once
            const int64_t r0 = rpre[li];
            for (int t = tid; t < re - li; t += NT)
              A.cnt[rowbase + b0 + li + t] = total - (uint32_t) (rpre[li + t] - r0);
            const int64_t h0 = hoff[li], h1 = hoff[re];
            cross_off_levels<NT>(bits, ccount, lp, hoff, li, re, (uint64_t) low, s_bitt);
            const uint32_t removed = (uint32_t) (rpre[re] - r0);
            total -= removed;
            if (h1 > h0) dirty = true;
            li = re;
            __syncthreads();
            continue;
          }
          // ---- levels li .. lj-1 with p^3 >= high whose records all lie in this
          // window: the numbers such a level removes are p and the p q with
          // prime q >= p, so the count at level l of a record's n is the count
          // at level li minus sum_{li <= b < l} ([low <= p_b <= n] +
          // pi(n / p_b) - pi(q_lo_b - 1)).  All their records are answered
          // against one bitmap state, then all their multiples crossed off at
          // once: one barrier pass instead of one per level.
          if ((lflags & 8) && la >= w0) {
            // lj: the first level from li on that cannot join the group, found
            // by each warp's lanes checking 32 levels at once
            int lj;
            {
              const int gm = A.group_max;
              int j = li + lane;
              bool no = !(j < nb && j - li < gm && (lp[j].flags & 8) && loff[j + 1] <= wend);
              unsigned bal = __ballot_sync(0xffffffffu, no);
              if (bal) lj = li + __ffs((int) bal) - 1;
              else {
                j += 32;
                no = !(j < nb && j - li < gm && (lp[j].flags & 8) && loff[j + 1] <= wend);
                bal = __ballot_sync(0xffffffffu, no);
                lj = bal ? li + 32 + __ffs((int) bal) - 1 : li + 64;
              }
            }
            if (lj - li >= 2) {
              const int ra = (int) (loff[li] - w0), rb = (int) (loff[lj] - w0);
              if (tid < lj - li) {
                s_gsmu[tid] = 0;
                s_gmag[tid] = A.pmagic[b0 + li + tid];
              }
              // a few records: a warp per record, its lanes summing the chunk
              // counts below the record's chunk and the removals of one group
              // level each (no prefix scan)
              const bool few = dirty && rb > ra && rb - ra <= SMALL_QUERIES;
              if (rb > ra && dirty && !few) { scan_chunks(ccount, pref, nch, wtmp); dirty = false; }
              else __syncthreads();
              if (few) {
                for (int k2 = ra + warp; k2 < rb; k2 += NT / 32) {
                  const uint32_t r = rec[k2];
                  if (r == REC_NONE) continue;
                  // the record's level: the levels li + t whose records end at or
                  // before it, counted by the lanes (a group has at most 64 levels)
                  const int64_t pos = w0 + k2;
                  int lv = li + __popc(__ballot_sync(0xffffffffu, li + lane < lj && loff[li + lane + 1] <= pos));
                  if (lj - li > 32)
                    lv += __popc(__ballot_sync(0xffffffffu, li + 32 + lane < lj && loff[li + 33 + lane] <= pos));
                  const uint32_t off = r & 0x3FFFFFFFu;
                  const uint64_t n = (uint64_t) low + off;
                  const uint32_t wd = off / 240, ch = wd >> 3, kw = wd & 7;
                  uint32_t part = chunk_sum_below(ccount, ch, lane);
                  if (lane < 8) {
                    const uint64_t v = bits[8 * ch + lane];
                    const uint32_t j = (uint32_t) lane;
                    part += (uint32_t) __popcll(j < kw ? v : (j == kw ? (v & mask_le_t(s_nb, off - wd * 240)) : 0ull));
                  }
                  // the numbers <= n removed by the levels li .. lv-1, one per lane
                  for (int b = li + lane; b < lv; b += 32) {
                    const uint64_t pb = lp[b].prime;
                    if (pb <= n && pb >= (uint64_t) low) part--;
                    const int64_t d = dpi_t(A.pitab, s_nb, div_magic(n, pb, s_gmag[b - li])) - (int64_t) s_pc[b];
                    if (d > 0) part -= (uint32_t) d;
                  }
                  // the count is below 2^32: the sum modulo 2^32 is exact
                  const uint32_t c = __reduce_add_sync(0xffffffffu, part);
                  if (lane == 0) {
                    if (r & (1u << 30)) { lsum -= c; atomicAdd(&s_gsmu[lv - li], -1); }
                    else { lsum += c; atomicAdd(&s_gsmu[lv - li], 1); }
                  }
                }
              } else if (rb > ra) {
                for (int k2 = ra + tid; k2 < rb; k2 += NT) {
                  const int lv = level_of(loff, li, lj, w0 + k2);
                  const uint32_t r = rec[k2];
                  int sg = 0;
                  if (r != REC_NONE) {
                    const uint32_t off = r & 0x3FFFFFFFu;
                    uint32_t c = query(bits, pref, s_nb, off);
                    const uint64_t n = (uint64_t) low + off;
                    // four levels at a time: their PiTable words are loaded together
                    int b = li;
                    for (; b + 4 <= lv; b += 4) {
                      uint64_t t[4];
#pragma unroll
                      for (int u = 0; u < 4; u++) {
                        const uint64_t pb = lp[b + u].prime;
                        if (pb <= n && pb >= (uint64_t) low) c--;
                        t[u] = div_magic(n, pb, s_gmag[b + u - li]);
                      }
                      ulonglong2 e[4];
#pragma unroll
                      for (int u = 0; u < 4; u++) e[u] = ((const ulonglong2*) A.pitab)[t[u] / 240];
#pragma unroll
                      for (int u = 0; u < 4; u++) {
                        // for t < 6 this reads 3 + a few bits, still below s_pc[b] >= pi(63): dropped by d > 0
                        const int64_t pt = (int64_t) (e[u].x + __popcll(e[u].y & mask_le_t(s_nb, (uint32_t) (t[u] % 240))));
                        const int64_t d = pt - (int64_t) s_pc[b + u];
                        if (d > 0) c -= (uint32_t) d;
                      }
                    }
                    for (; b < lv; b++) {
                      const uint64_t pb = lp[b].prime;
                      if (pb <= n && pb >= (uint64_t) low) c--;
                      const int64_t d = dpi_t(A.pitab, s_nb, div_magic(n, pb, s_gmag[b - li])) - (int64_t) s_pc[b];
                      if (d > 0) c -= (uint32_t) d;
                    }
                    if (r & (1u << 30)) { lsum -= c; sg = -1; }
                    else { lsum += c; sg = 1; }
                  }
                  // signed counts per level, aggregated over the lanes of one level
                  const unsigned act = __activemask();
                  const unsigned same = __match_any_sync(act, lv);
                  const int tot = __reduce_add_sync(same, sg);
                  if (tot && lane == __ffs((int) same) - 1) atomicAdd(&s_gsmu[lv - li], tot);
                }
              }
              __syncthreads();
              // the levels' counts C(s, b) and signed leaf counts M(s, b)
              const int64_t r0 = rpre[li];
              for (int t = tid; t < lj - li; t += NT) {
                const int64_t cell = rowbase + b0 + li + t;
                A.cnt[cell] = total - (uint32_t) (rpre[li + t] - r0);
                if (s_gsmu[t]) A.smu[cell] = s_gsmu[t];
              }
              // all their multiples crossed off at once
              const int64_t h0 = hoff[li], h1 = hoff[lj];
              cross_off_levels<NT>(bits, ccount, lp, hoff, li, lj, (uint64_t) low, s_bitt);
              total -= (uint32_t) (rpre[lj] - r0);
              if (h1 > h0) dirty = true;
              li = lj;
              __syncthreads();
              continue;
            }
          }
          if (lz > la && la >= wend) break;               // records start in a later window
          const int l = b0 + li;
          if (la >= w0 && tid == NT - 1) A.cnt[rowbase + l] = total;   // the last thread: rarely a multiple to cross off
          const int ra = (int) (dmax(la, w0) - w0);
          const int rz = (int) (dmin(lz, wend) - w0);           // end of the level's window records
          const int rb = li == clev ? s_ncomp[win & 1] : rz;   // end of those still to answer
          if (rb > ra) {
            if (dirty && rb - ra <= SMALL_QUERIES) {
              // a few records: a warp per record sums the chunk counts below
              // the record's chunk itself, instead of a block-wide prefix
              // scan (the prefix array stays out of date)
              int smu_w = 0;
              for (int k2 = ra + warp; k2 < rb; k2 += NT / 32) {
                const uint32_t r = rec[k2];
                if (r == REC_NONE) continue;
                const uint32_t off = r & 0x3FFFFFFFu;
                const uint32_t wd = off / 240, ch = wd >> 3, kw = wd & 7;
                uint32_t part = chunk_sum_below(ccount, ch, lane);
                if (lane < 8) {
                  const uint64_t v = bits[8 * ch + lane];
                  const uint32_t j = (uint32_t) lane;
                  part += (uint32_t) __popcll(j < kw ? v : (j == kw ? (v & mask_le_t(s_nb, off - wd * 240)) : 0ull));
                }
                const uint32_t c = __reduce_add_sync(0xffffffffu, part);
                if (r & (1u << 30)) { if (lane == 0) lsum -= c; smu_w--; }
                else { if (lane == 0) lsum += c; smu_w++; }
              }
              if (lane == 0 && smu_w) atomicAdd(&s_smu, smu_w);
            } else {
              if (dirty) { scan_chunks(ccount, pref, nch, wtmp); dirty = false; }
              if (ra + 32 * warp < rb) {
                int smu_t = 0;
                for (int k2 = ra + tid; k2 < rb; k2 += NT) {
                  const uint32_t r = rec[k2];
                  if (r != REC_NONE) {
                    const uint32_t c = query(bits, pref, s_nb, r & 0x3FFFFFFFu);
                    if (r & (1u << 30)) { lsum -= c; smu_t--; }
                    else { lsum += c; smu_t++; }
                  }
                }
                smu_t = __reduce_add_sync(0xffffffffu, smu_t);
                if (lane == 0 && smu_t) atomicAdd(&s_smu, smu_t);
              }
            }
            __syncthreads();
          }
          if (rz > ra && lz <= wend && tid == NT - 1) { A.smu[rowbase + l] = s_smu; s_smu = 0; }
          if (lz > wend) break;                            // the level continues in the next window
          // ---- cross off p_l and its multiples, count the numbers removed first
          const LevelP& P = lp[li];
          const uint32_t pjn = P.jn, pprime = P.prime;
          const uint64_t pjlo = P.jlo;
          uint32_t rem = 0;
          if (lflags & 4) {
            // small prime: AND with its wheel pattern, one owner thread per word
            const uint32_t p = P.prime;
            int po = 0;
            for (int k = 0; c_small_p[k] != p; k++) po += c_small_p[k];
            // four consecutive words per thread and round (two 16-byte accesses)
            uint32_t r = (uint32_t) ((P.jlo + 4 * tid) % p);
            const uint32_t step = (4 * NT) % p;
            for (int w = 4 * tid; w < A.words; w += 4 * NT) {
              uint32_t d = 0;
              if (w < wused) {
                const ulonglong2 o0 = *(const ulonglong2*) (bits + w);
                const ulonglong2 o1 = *(const ulonglong2*) (bits + w + 2);
                const uint32_t r1 = r + 1 == p ? 0u : r + 1;
                const uint32_t r2 = r1 + 1 == p ? 0u : r1 + 1;
                const uint32_t r3 = r2 + 1 == p ? 0u : r2 + 1;
                ulonglong2 n0, n1;
                n0.x = o0.x & pat[po + r];
                n0.y = (w + 1 < wused) ? (o0.y & pat[po + r1]) : o0.y;
                n1.x = (w + 2 < wused) ? (o1.x & pat[po + r2]) : o1.x;
                n1.y = (w + 3 < wused) ? (o1.y & pat[po + r3]) : o1.y;
                if (n0.x != o0.x || n0.y != o0.y) {
                  *(ulonglong2*) (bits + w) = n0;
                  d = __popcll(o0.x ^ n0.x) + __popcll(o0.y ^ n0.y);
                }
                if (n1.x != o1.x || n1.y != o1.y) {
                  *(ulonglong2*) (bits + w + 2) = n1;
                  d += __popcll(o1.x ^ n1.x) + __popcll(o1.y ^ n1.y);
                }
              }
              rem += d;
              // 2 consecutive lanes own the 8 words of one chunk
              d += __shfl_down_sync(0xffffffffu, d, 1, 2);
              if ((lane & 1) == 0 && d) ccount[w >> 3] -= d;
              r += step;
              if (r >= p) r -= p;
            }
          } else if (pjn) {
            if ((uint32_t) tid < pjn) {
              // co-factors tid, tid + NT, ...: NT / 8 wheel turns apart, so
              // the multiples are NT p / 64 words apart with the same bit
              const uint64_t p = pprime;
              const uint64_t jj = pjlo + (uint64_t) tid;
              const uint64_t q = 30 * (jj >> 3) + woff((uint32_t) (jj & 7));
              const uint32_t off = (uint32_t) (p * q - (uint64_t) low);
              const uint32_t w = off / 240;
              const uint32_t bi = s_bitt[off - w * 240];
              const uint32_t m = 1u << (bi & 31);
              // the number's 32-bit half-word, and the half-word stride
              uint32_t h = 2 * w + (bi >> 5);
              const uint32_t hstep = (uint32_t) p * (NT / 32);
              uint32_t* const hw = (uint32_t*) bits;
              for (uint32_t j = tid; j < pjn; j += NT, h += hstep) {
                const uint32_t old = hw[h];
                if (old & m) { hw[h] = old & ~m; rem++; atomicSub(&ccount[h >> 4], 1u); }
              }
            }
          }
          if (lflags & 8) {
            __syncthreads();
            total -= P.fcount;
            if (pjn) dirty = true;
          } else if (!(lflags & 4) && pjn <= (uint32_t) NT) {
            // at most one multiple per thread: the barrier counts the removals
            const uint32_t rr = (uint32_t) __syncthreads_count(rem != 0);
            total -= rr;
            if (rr) dirty = true;
            if (tid == NT - 1) s_rem[(l + 2) % 3] = 0;
          } else {
            rem = __reduce_add_sync(0xffffffffu, rem);
            if (lane == 0 && rem) atomicAdd(&s_rem[l % 3], rem);
            __syncthreads();
            const uint32_t rr = s_rem[l % 3];
            total -= rr;
            if (rr) dirty = true;
            if (tid == NT - 1) s_rem[(l + 2) % 3] = 0;
          }
          li++;
        }
        w0 = wend;
      }
    }
    // segment result
    for (int d = 16; d > 0; d >>= 1) lsum += __shfl_down_sync(0xffffffffu, lsum, d);
    if (lane == 0) s_red[warp] = lsum;
    for (int d = 16; d > 0; d >>= 1) {
      nleaves += __shfl_down_sync(0xffffffffu, nleaves, d);
      ntwo += __shfl_down_sync(0xffffffffu, ntwo, d);
      nentries += __shfl_down_sync(0xffffffffu, nentries, d);
    }
    if (lane == 0) {
      if (nleaves) atomicAdd(&s_ctr[0], nleaves);
      if (ntwo) atomicAdd(&s_ctr[1], ntwo);
      if (nentries) atomicAdd(&s_ctr[3], nentries);
    }
    if (tid == 0) atomicAdd(&s_ctr[2], (unsigned long long) Bs);
    __syncthreads();
    if (tid == 0) {
      long long t = 0;
      for (int i = 0; i < NT / 32; i++) t += s_red[i];
      A.segsum[ws] = t;
    }
  }
  __syncthreads();
  if (tid < 5 && s_ctr[tid]) atomicAdd(&A.counters[tid], s_ctr[tid]);
}

// ---- phi offsets: acc[b] += sum_s M(s, b) * sum_{s'<s} C(s', b), in segment order.
// One block per job.  A level job takes 32 levels of one problem; its
// COMBINE_WARPS warps take consecutive runs of the problem's items in the
// wave and sum them from a local count of 0, then the runs are chained: a
// run k whose segments see the count R_k + r (r its local prefix) adds
// a_k + ms_k R_k, with a_k = sum M r and ms_k = sum M over the run.  A sum
// job (slab < 0) adds the items' local leaf sums into the problem's column 0
// (never a level: level jobs leave it alone).
#define COMBINE_WARPS 16
struct CombineJob {
  int64_t colbase;   // the problem's first cell in run / acc / msum
  int32_t item0;     // its first item in the wave (wave-local)
  int32_t n;         // its items in the wave
  int32_t cols;      // its columns (levels 0 .. cols - 1)
  int32_t slab;      // levels [32 slab, 32 slab + 32); < 0: the local sums
};

__global__ void __launch_bounds__(32 * COMBINE_WARPS)
k_combine(const uint32_t* __restrict__ cnt, const int32_t* __restrict__ smu, const int64_t* __restrict__ rowoff,
          const int64_t* __restrict__ segsum, const CombineJob* __restrict__ jobs, int64_t* __restrict__ run,
          i128* __restrict__ acc, int64_t* __restrict__ msum)
{
  __shared__ i128 s_a[COMBINE_WARPS][32];
  __shared__ long long s_m[COMBINE_WARPS][32], s_c[COMBINE_WARPS][32];
  const CombineJob J = jobs[blockIdx.x];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (J.slab < 0) {
    // per-thread partial sums fit int64 (each segment's sum does, n is small)
    long long v = 0;
    for (int i = threadIdx.x; i < J.n; i += blockDim.x) v += segsum[J.item0 + i];
    for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
    if (lane == 0) s_m[w][0] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      i128 t = 0;
      for (int i = 0; i < COMBINE_WARPS; i++) t += s_m[i][0];
      acc[J.colbase] += t;
    }
    return;
  }
  const int b = J.slab * 32 + lane;
  const int per = (J.n + COMBINE_WARPS - 1) / COMBINE_WARPS;
  const int s0 = J.item0 + min(J.n, w * per), s1 = J.item0 + min(J.n, w * per + per);
  i128 a = 0;
  long long ms = 0, r = 0;
  if (b < J.cols) {
    int s = s0;
    for (; s + 4 <= s1; s += 4) {
      const int64_t o0 = rowoff[s] + b, o1 = rowoff[s + 1] + b, o2 = rowoff[s + 2] + b, o3 = rowoff[s + 3] + b;
      const int32_t m0 = smu[o0], m1 = smu[o1], m2 = smu[o2], m3 = smu[o3];
      const uint32_t c0 = cnt[o0], c1 = cnt[o1], c2 = cnt[o2], c3 = cnt[o3];
      a += (i128) m0 * r; r += c0;
      a += (i128) m1 * r; r += c1;
      a += (i128) m2 * r; r += c2;
      a += (i128) m3 * r; r += c3;
      ms += (long long) m0 + m1 + m2 + m3;
    }
    for (; s < s1; s++) {
      const int64_t o = rowoff[s] + b;
      const int32_t m = smu[o];
      a += (i128) m * r;
      ms += m;
      r += cnt[o];
    }
  }
  s_a[w][lane] = a;
  s_m[w][lane] = ms;
  s_c[w][lane] = r;
  __syncthreads();
  if (w == 0 && b < J.cols && b > 0) {
    const int64_t cb = J.colbase + b;
    long long R = run[cb], M = 0;
    i128 A = 0;
    for (int k = 0; k < COMBINE_WARPS; k++) {
      A += s_a[k][lane] + (i128) s_m[k][lane] * R;
      R += s_c[k][lane];
      M += s_m[k][lane];
    }
    run[cb] = R;
    acc[cb] += A;
    if (msum) msum[cb] += M;
  }
}

// ================================================================ host side
static double now_ms()
{
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

void DevBuf::alloc(size_t n)
{
  if (n <= bytes && p) return;
  free_();
  if (n == 0) n = 16;
  cudaError_t e = cudaMalloc(&p, n);
  if (e != cudaSuccess) {
    p = nullptr;
    bytes = 0;
    cudaGetLastError();
    fail(PCG_ENOMEM, std::string("cudaMalloc of ") + std::to_string(n) + " bytes failed: " + cudaGetErrorString(e));
  }
  bytes = n;
}

void DevBuf::free_()
{
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
}

DevBuf::~DevBuf() { free_(); }

static std::vector<uint32_t> small_primes(int64_t limit)
{
  std::vector<uint8_t> c((size_t) limit + 1, 0);
  std::vector<uint32_t> p;
  for (int64_t i = 2; i <= limit; i++) {
    if (c[i]) continue;
    p.push_back((uint32_t) i);
    for (int64_t m = i * i; m <= limit; m += i) c[m] = 1;
  }
  return p;
}

static void ensure_wheel(Ctx& c, cudaStream_t s)
{
  Tables& t = c.tab;
  if (t.coprime.p) return;
  const Wheel2310& w = wheel2310();
  t.coprime.alloc(sizeof(w.coprime));
  t.cindex.alloc(sizeof(w.index));
  PCG_CUDA(cudaMemcpyAsync(t.coprime.p, w.coprime, sizeof(w.coprime), cudaMemcpyHostToDevice, s));
  PCG_CUDA(cudaMemcpyAsync(t.cindex.p, w.index, sizeof(w.index), cudaMemcpyHostToDevice, s));
}

int64_t host_pi(const Tables& t, uint64_t x)
{
  static const int64_t tiny[6] = {0, 0, 1, 2, 2, 3};
  if (x < 6) return tiny[x];
  if ((int64_t) x > t.prime_limit) fail(PCG_EINTERNAL, "host_pi beyond the prime tables");
  uint64_t i = x / 240;
  uint64_t r = x % 240;
  uint64_t m = 0;
  for (int j = 0; j < 64; j++) {
    static const int W[8] = {1, 7, 11, 13, 17, 19, 23, 29};
    if ((uint64_t) (30 * (j / 8) + W[j % 8]) <= r) m |= 1ull << j;
  }
  return (int64_t) (t.h_pitab[2 * i] + (uint64_t) __builtin_popcountll(t.h_pitab[2 * i + 1] & m));
}

// floor((2^64 - 1) / p) for the primes p = primes[1 .. n]: x / p then costs a
// 64x64 high multiply and one correction step (the reference divides by
// libdivide's precomputed reciprocals for the same reason)
__global__ void k_prime_magic(const uint32_t* __restrict__ primes, int64_t n, uint64_t* __restrict__ magic)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < 1 || i > n) return;
  magic[i] = UINT64_MAX / primes[i];
}

// floor((2^64 - 1) / m) for the numbers m coprime to 2310 with factor-table
// index in [0, n)
__global__ void k_factor_inv(const uint16_t* __restrict__ cop, int64_t n, uint64_t* __restrict__ inv)
{
  const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t m = 2310 * (uint64_t) (i / 480) + cop[i % 480];
  inv[i] = UINT64_MAX / m;
}

void ensure_prime_tables(Ctx& c, int64_t limit, cudaStream_t s)
{
  Tables& t = c.tab;
  limit = std::max<int64_t>(limit, 240 * 4);
  if (t.prime_limit >= limit) return;
  ensure_wheel(c, s);
  double t0 = now_ms();
  int64_t nwords = limit / 240 + 1;
  std::vector<uint32_t> base = small_primes(isqrt((u128) limit) + 1);
  // base primes >= 7
  std::vector<uint32_t> b7;
  for (uint32_t p : base) if (p >= 7) b7.push_back(p);
  DevBuf d_base, d_bits, d_pc, d_excl, d_sums;
  d_base.alloc(std::max<size_t>(b7.size(), 1) * 4);
  d_bits.alloc((size_t) nwords * 8);
  d_pc.alloc((size_t) nwords * 4);
  d_excl.alloc((size_t) nwords * 8);
  int64_t nblk = (nwords + SCAN_ITEMS - 1) / SCAN_ITEMS;
  d_sums.alloc((size_t) nblk * 8);
  if (!b7.empty())
    PCG_CUDA(cudaMemcpyAsync(d_base.p, b7.data(), b7.size() * 4, cudaMemcpyHostToDevice, s));
  int64_t pblocks = (nwords + 2047) / 2048;
  k_prime_bits<<<(unsigned) pblocks, 512, 2048 * 8, s>>>(d_bits.as<uint64_t>(), d_pc.as<uint32_t>(), nwords, limit,
                                                         d_base.as<uint32_t>(), (int) b7.size());
  PCG_CUDA(cudaGetLastError());
  k_scan_sums<<<(unsigned) nblk, 512, 0, s>>>(d_pc.as<uint32_t>(), nwords, d_sums.as<uint64_t>());
  k_scan_serial<<<1, 1024, 0, s>>>(d_sums.as<uint64_t>(), nblk);
  k_scan_apply<<<(unsigned) nblk, 512, 0, s>>>(d_pc.as<uint32_t>(), nwords, d_sums.as<uint64_t>(), d_excl.as<uint64_t>());
  PCG_CUDA(cudaGetLastError());
  // total count -> nprimes
  uint64_t last_excl = 0;
  uint32_t last_pc = 0;
  PCG_CUDA(cudaMemcpyAsync(&last_excl, d_excl.as<uint64_t>() + nwords - 1, 8, cudaMemcpyDeviceToHost, s));
  PCG_CUDA(cudaMemcpyAsync(&last_pc, d_pc.as<uint32_t>() + nwords - 1, 4, cudaMemcpyDeviceToHost, s));
  PCG_CUDA(cudaStreamSynchronize(s));
  int64_t np = 3 + (int64_t) last_excl + last_pc;
  t.primes.alloc((size_t) (np + 2) * 4);
  t.pitab.alloc((size_t) nwords * 16);
  uint32_t head[4] = {0, 2, 3, 5};
  PCG_CUDA(cudaMemcpyAsync(t.primes.p, head, sizeof(head), cudaMemcpyHostToDevice, s));
  k_pitab_primes<<<(unsigned) ((nwords + 255) / 256), 256, 0, s>>>(d_bits.as<uint64_t>(), d_excl.as<uint64_t>(), nwords,
                                                                   t.pitab.as<uint64_t>(), t.primes.as<uint32_t>());
  t.pmagic.alloc((size_t) (np + 2) * 8);
  PCG_CUDA(cudaMemsetAsync(t.pmagic.p, 0, (size_t) (np + 2) * 8, s));
  k_prime_magic<<<(unsigned) ((np + 256) / 256), 256, 0, s>>>(t.primes.as<uint32_t>(), np, t.pmagic.as<uint64_t>());
  PCG_CUDA(cudaGetLastError());
  t.h_pitab.resize((size_t) nwords * 2);
  PCG_CUDA(cudaMemcpyAsync(t.h_pitab.data(), t.pitab.p, (size_t) nwords * 16, cudaMemcpyDeviceToHost, s));
  t.h_primes.resize((size_t) np + 1);
  PCG_CUDA(cudaMemcpyAsync(t.h_primes.data(), t.primes.p, ((size_t) np + 1) * 4, cudaMemcpyDeviceToHost, s));
  PCG_CUDA(cudaStreamSynchronize(s));
  t.prime_limit = limit;
  t.nprimes = np;
  t.build_ms += now_ms() - t0;
}

void exclusive_scan_u32(const uint32_t* in, int64_t n, uint64_t* out, cudaStream_t s, DevBuf* sums_buf)
{
  int64_t nblk = (n + SCAN_ITEMS - 1) / SCAN_ITEMS;
  DevBuf local;
  DevBuf& sums = sums_buf ? *sums_buf : local;
  sums.alloc((size_t) std::max<int64_t>(nblk, 1) * 8);
  k_scan_sums<<<(unsigned) nblk, 512, 0, s>>>(in, n, sums.as<uint64_t>());
  k_scan_serial<<<1, 1024, 0, s>>>(sums.as<uint64_t>(), nblk);
  k_scan_apply<<<(unsigned) nblk, 512, 0, s>>>(in, n, sums.as<uint64_t>(), out);
  PCG_CUDA(cudaGetLastError());
  PCG_CUDA(cudaStreamSynchronize(s));
}

__global__ void k_pitab_pack(const uint64_t* __restrict__ bits, const uint64_t* __restrict__ excl, int64_t nwords,
                             uint64_t* __restrict__ pitab)
{
  int64_t w = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nwords) return;
  pitab[2 * w] = 3 + excl[w];
  pitab[2 * w + 1] = bits[w];
}

// PiTable {count, bits} per 240 numbers over [0, limit] without the primes
// array (for the lookups of pi(n), n <= sqrt(x), of the A, B, C formulas).
void build_pitab_only(DevBuf& out, int64_t limit, cudaStream_t s)
{
  limit = std::max<int64_t>(limit, 240 * 4);
  int64_t nwords = limit / 240 + 1;
  std::vector<uint32_t> base = small_primes(isqrt((u128) limit) + 1);
  std::vector<uint32_t> b7;
  for (uint32_t p : base) if (p >= 7) b7.push_back(p);
  DevBuf d_base, d_bits, d_pc, d_excl;
  d_base.alloc(std::max<size_t>(b7.size(), 1) * 4);
  d_bits.alloc((size_t) nwords * 8);
  d_pc.alloc((size_t) nwords * 4);
  d_excl.alloc((size_t) nwords * 8);
  if (!b7.empty())
    PCG_CUDA(cudaMemcpyAsync(d_base.p, b7.data(), b7.size() * 4, cudaMemcpyHostToDevice, s));
  int64_t pblocks = (nwords + 2047) / 2048;
  k_prime_bits<<<(unsigned) pblocks, 512, 2048 * 8, s>>>(d_bits.as<uint64_t>(), d_pc.as<uint32_t>(), nwords, limit,
                                                         d_base.as<uint32_t>(), (int) b7.size());
  PCG_CUDA(cudaGetLastError());
  exclusive_scan_u32(d_pc.as<uint32_t>(), nwords, d_excl.as<uint64_t>(), s);
  out.alloc((size_t) nwords * 16);
  k_pitab_pack<<<(unsigned) ((nwords + 255) / 256), 256, 0, s>>>(d_bits.as<uint64_t>(), d_excl.as<uint64_t>(), nwords,
                                                                 out.as<uint64_t>());
  PCG_CUDA(cudaGetLastError());
  PCG_CUDA(cudaStreamSynchronize(s));
}

template <typename T>
static void build_factor(Ctx& c, DevBuf& out, int64_t limit, int64_t y, int gourdon, cudaStream_t s)
{
  Tables& t = c.tab;
  const Wheel2310& w = wheel2310();
  int64_t size = w.to_index((uint64_t) std::max<int64_t>(limit, 1)) + 1;
  out.alloc((size_t) size * sizeof(T));
  int64_t sq = isqrt((u128) limit);
  int64_t nsmall = host_pi(t, (uint64_t) sq);
  int64_t blocks = (size + FT_E - 1) / FT_E;
  size_t smem = FT_E * (8 + 4 + 4) + 480 * 2 + 2310 * 2;
  PCG_CUDA(cudaFuncSetAttribute(k_factor<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem));
  k_factor<T><<<(unsigned) blocks, 512, smem, s>>>(out.as<T>(), size, limit, y, gourdon, t.primes.as<uint32_t>(),
                                                   nsmall, t.coprime.as<uint16_t>(), t.cindex.as<int16_t>());
  PCG_CUDA(cudaGetLastError());
  if (gourdon && sq > y) {
    // small primes in (y, sqrt(limit)]: their multiples have a prime factor > y
    int64_t kf = host_pi(t, (uint64_t) y) + 1;
    kf = std::max<int64_t>(kf, 6);
    if (kf <= nsmall)
      k_factor_zero_small<T><<<(unsigned) (nsmall - kf + 1), 256, 0, s>>>(out.as<T>(), size, limit, t.primes.as<uint32_t>(),
                                                                           kf, nsmall, t.coprime.as<uint16_t>(),
                                                                           t.cindex.as<int16_t>());
    PCG_CUDA(cudaGetLastError());
  }
}

// reciprocals of the factor-table numbers for the indices [0, n)
static void ensure_finv(Ctx& c, int64_t n, cudaStream_t s)
{
  Tables& t = c.tab;
  if (t.finv_n >= n) return;
  t.finv.alloc((size_t) n * 8);
  k_factor_inv<<<(unsigned) ((n + 255) / 256), 256, 0, s>>>(t.coprime.as<uint16_t>(), n, t.finv.as<uint64_t>());
  PCG_CUDA(cudaGetLastError());
  t.finv_n = n;
}

void ensure_factor_d(Ctx& c, int64_t y, int64_t z, cudaStream_t s)
{
  Tables& t = c.tab;
  bool ok = t.fd_z >= z && (t.fd_y == y || (y >= z && t.fd_y >= z));
  if (ok) return;
  double t0 = now_ms();
  ensure_prime_tables(c, std::max<int64_t>(y, isqrt((u128) z) + 1), s);
  // 16-bit entries whenever possible, as the reference's D() chooses
  // (src/gourdon/D.cpp:477-499); PCG_FACTOR_D_U32=1 forces the 32-bit table,
  // whose size limit no practical z reaches, so that it can be tested
  const char* f32 = getenv("PCG_FACTOR_D_U32");
  const bool force32 = f32 && atoi(f32) == 1;
  t.fd_bytes = (z <= 386083ll * 386083 - 1 && !force32) ? 2 : 4;
  if (t.fd_bytes == 2) build_factor<uint16_t>(c, t.factor_d, z, y, 1, s);
  else build_factor<uint32_t>(c, t.factor_d, z, y, 1, s);
  ensure_finv(c, wheel2310().to_index((uint64_t) std::max<int64_t>(z, 1)) + 1, s);
  PCG_CUDA(cudaStreamSynchronize(s));
  t.fd_y = y;
  t.fd_z = z;
  t.build_ms += now_ms() - t0;
}

void ensure_factor_dr(Ctx& c, int64_t y, cudaStream_t s)
{
  Tables& t = c.tab;
  if (t.fr_y >= y) return;
  double t0 = now_ms();
  ensure_prime_tables(c, std::max<int64_t>(y, isqrt((u128) y) + 1), s);
  t.fr_bytes = (y <= 65534ll * 65534 - 1) ? 2 : 4;
  if (t.fr_bytes == 2) build_factor<uint16_t>(c, t.factor_dr, y, y, 0, s);
  else build_factor<uint32_t>(c, t.factor_dr, y, y, 0, s);
  ensure_finv(c, wheel2310().to_index((uint64_t) std::max<int64_t>(y, 1)) + 1, s);
  PCG_CUDA(cudaStreamSynchronize(s));
  t.fr_y = y;
  t.build_ms += now_ms() - t0;
}

// Combine jobs of n consecutive items (wave-local item0) of one problem with
// cols columns whose cells start at colbase: one job per 32 levels and one
// for the local sums.
static void add_combine_jobs(std::vector<CombineJob>& jobs, int64_t colbase, int item0, int n, int cols)
{
  for (int sl = 0; sl * 32 < cols; sl++) jobs.push_back(CombineJob{colbase, item0, n, cols, sl});
  jobs.push_back(CombineJob{colbase, item0, n, cols, -1});
}

template <typename FT, int NT>
static void set_sweep_attr(size_t smem)
{
  // per device and cheap: set on every call (worker threads and several
  // devices share the function)
  PCG_CUDA(cudaFuncSetAttribute(k_sweep<FT, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem));
}

template <typename FT, int NT>
static void occupancy_sweep(int* occ, size_t smem)
{
  set_sweep_attr<FT, NT>(smem);
  PCG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, k_sweep<FT, NT>, NT, smem));
}

template <typename FT, int NT>
static void launch_sweep(const SweepArgs& a, int grid, size_t smem, cudaStream_t s)
{
  set_sweep_attr<FT, NT>(smem);
  k_sweep<FT, NT><<<grid, NT, smem, s>>>(a);
}

// Segment planner (the role of LoadBalancerS2's growing segment sizes,
// src/LoadBalancerS2.cpp:195-264, decided up front): an analytic estimate of
// the leaves of every family per interval (m-range length times the density
// of square-free numbers without prime factors <= p_b, or the prime density
// for the p_b * p_l leaves) plus a per-level cost, integrated on a geometric
// grid; segments are cut at equal estimated cost, never longer than smax.
// dens[b] = 0.56 / log(p_b) for b in [1, bglob].  The grid cells are costed
// on nth host threads (1: the calling thread only, no thread is created).
// Each segment end is passed to push(end) in order, starting with 0; a push
// returning false stops the plan (the return value is then false).  G grid
// cells (at most PLAN_GRID).
#define PLAN_GRID 1200
template <class Push>
static bool plan_segments_core(const SweepProblem& pb, const Tables& t, int64_t L, int64_t x_star,
                               int64_t pi_sqrt, int64_t bglob, int64_t smax, int grid, const double* dens,
                               unsigned nth, Push push, int G = PLAN_GRID)
{
  const double x = (double) pb.x;
  const double y = (double) pb.y, z = (double) pb.z;
  G = std::max(2, std::min(G, PLAN_GRID));
  double g[PLAN_GRID + 1], cost[PLAN_GRID], cum[PLAN_GRID + 1];
  g[0] = 0;
  const double a0 = 240;
  const double ratio = std::pow((double) L / a0, 1.0 / (G - 1));
  for (int i = 0; i < G; i++) g[i + 1] = std::min((double) L, a0 * std::pow(ratio, i));
  g[G] = (double) L;
  auto leaves = [&](double lo, double hi) {
    double sum = 0;
    double l1 = std::max(lo, 1.0);
    for (int64_t b = pb.k + 1; b <= bglob; b++) {
      const double p = (double) t.h_primes[(size_t) b], xp = x / p;
      double mlo, mhi;
      if (pb.gourdon == 2) { mlo = std::max({y / p, xp / hi, p}); mhi = std::min(xp / l1, y); }
      else if (pb.gourdon) {
        if (b <= pi_sqrt) { mlo = std::max(z / p, xp / hi); mhi = std::min({xp / (p * p), z, xp / l1}); }
        else { mlo = std::max(p, xp / hi); mhi = std::min({xp / (p * p), y, xp / l1}); }
      } else {
        if (b <= pi_sqrt) { mlo = std::max(y / p, xp / hi); mhi = std::min(xp / l1, y); }
        else { mlo = std::max(p, xp / hi); mhi = std::min({xp / l1, y, z / p}); }
      }
      if (mhi <= mlo) continue;
      sum += (b <= pi_sqrt) ? (mhi - mlo) * dens[b] : (mhi - mlo) / std::log(std::max(mhi, 3.0));
    }
    return sum;
  };
  auto levels = [&](double a) {
    double lim = pb.gourdon ? std::min((double) x_star, std::sqrt(x / std::max(a, 1.0)))
                            : std::min(std::sqrt(z), std::sqrt(x / std::max(a, 1.0)));
    return (double) host_pi(t, (uint64_t) std::min(lim, (double) t.prime_limit));
  };
  const double c_level = 30.0;
  auto cell = [&](unsigned k, unsigned step) {
    for (int i = (int) k; i < G; i += (int) step) {
      const double len = g[i + 1] - g[i];
      cost[i] = len > 0 ? leaves(g[i], g[i + 1]) + c_level * levels(g[i]) * len / (double) smax : 0;
    }
  };
  if (nth <= 1) cell(0, 1);
  else {
    std::vector<std::thread> th;
    for (unsigned k = 0; k < nth; k++) th.emplace_back(cell, k, nth);
    for (auto& h : th) h.join();
  }
  cum[0] = 0;
  for (int i = 0; i < G; i++) cum[i + 1] = cum[i] + cost[i];
  const double total = cum[G];
  const double target = std::max(total / (grid * 6.0), 1.0);
  // cumulative cost at n (linear inside a grid cell)
  auto C = [&](double n) {
    const int i = (int) (std::upper_bound(g, g + G + 1, n) - g);
    if (i == 0) return 0.0;
    if (i > G) return total;
    const double f = (g[i] > g[i - 1]) ? (n - g[i - 1]) / (g[i] - g[i - 1]) : 0;
    return cum[i - 1] + f * (cum[i] - cum[i - 1]);
  };
  // largest n with C(n) <= v (C is piecewise linear and non-decreasing)
  auto Cinv = [&](double v) {
    if (v >= total) return (double) L;
    const int i = (int) (std::upper_bound(cum, cum + G + 1, v) - cum);   // cum[i - 1] <= v < cum[i]
    const double d = cum[i] - cum[i - 1];
    const double f = d > 0 ? (v - cum[i - 1]) / d : 0;
    return g[i - 1] + f * (g[i] - g[i - 1]);
  };
  int64_t a = 0;
  if (!push(a)) return false;
  while (a < L) {
    const int64_t lo = a + 240, hi = std::min(a + smax, L);
    if (hi <= lo) {
      a = std::min(a + smax, L);
      if (!push(a)) return false;
      continue;
    }
    // the largest end (a multiple of 240, or hi) with cost <= target
    const double n = Cinv(C((double) a) + target);
    int64_t best = n >= (double) hi ? hi : (int64_t) (n / 240) * 240;
    best = std::max(lo, std::min(best, hi));
    a = std::min(best, L);
    if (!push(a)) return false;
  }
  return true;
}

static std::vector<int64_t> plan_segments(const SweepProblem& pb, const Tables& t, int64_t L, int64_t x_star,
                                          int64_t pi_sqrt, int64_t bglob, int64_t smax, int grid)
{
  std::vector<double> dens((size_t) bglob + 1, 0.0);
  for (int64_t b = 1; b <= bglob; b++) dens[b] = 0.56 / std::log(std::max((double) t.h_primes[(size_t) b], 3.0));
  std::vector<int64_t> seg;
  const unsigned nth = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  plan_segments_core(pb, t, L, x_star, pi_sqrt, bglob, smax, grid, dens.data(), nth,
                     [&](int64_t v) { seg.push_back(v); return true; });
  return seg;
}

// levels with p^3 >= high answered in one pass (PCG_SWEEP_GROUP overrides)
static int sweep_group_max()
{
  static const int g = [] {
    const char* e = getenv("PCG_SWEEP_GROUP");
    const int v = e ? atoi(e) : 32;
    return v < 0 ? 0 : (v > GROUP_MAX ? GROUP_MAX : v);
  }();
  return g;
}

// ---- checkpoint / resume of a sweep: the phi-offset totals run[b], the leaf
// sums acc[b] and msum[b] after the last finished wave, with the problem and
// a hash of the segment plan they belong to
struct CkptHeader {
  char magic[8];
  uint32_t version;
  int32_t gourdon;
  uint64_t x_lo, x_hi;
  int64_t y, z, k;
  int32_t shard, nshards;
  int32_t words, nt;
  int64_t nseg, cols;
  uint64_t plan_hash;
  int64_t next_first;      // first segment not swept yet
  int64_t waves;
  uint64_t counters[5];
};

static uint64_t plan_hash(const std::vector<int64_t>& seglo)
{
  uint64_t h = 1469598103934665603ull;   // FNV-1a over the segment bounds
  for (int64_t v : seglo)
    for (int i = 0; i < 8; i++) { h ^= (uint64_t) (v >> (8 * i)) & 0xFF; h *= 1099511628211ull; }
  return h;
}

static bool same_problem(const CkptHeader& a, const CkptHeader& b)
{
  return memcmp(a.magic, b.magic, 8) == 0 && a.version == b.version && a.gourdon == b.gourdon &&
         a.x_lo == b.x_lo && a.x_hi == b.x_hi && a.y == b.y && a.z == b.z && a.k == b.k && a.shard == b.shard &&
         a.nshards == b.nshards && a.words == b.words && a.nt == b.nt && a.nseg == b.nseg && a.cols == b.cols &&
         a.plan_hash == b.plan_hash;
}

static bool read_checkpoint(const std::string& path, const CkptHeader& want, CkptHeader& got,
                            std::vector<int64_t>& run, std::vector<i128>& acc, std::vector<int64_t>& msum)
{
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) return false;
  bool ok = fread(&got, sizeof(got), 1, f) == 1 && same_problem(got, want) && got.next_first >= 0 &&
            got.next_first <= got.nseg;
  const size_t n = (size_t) want.cols;
  if (ok) {
    run.resize(n);
    acc.resize(n);
    msum.resize(n);
    ok = fread(run.data(), 8, n, f) == n && fread(acc.data(), 16, n, f) == n && fread(msum.data(), 8, n, f) == n;
  }
  fclose(f);
  return ok;
}

static void write_checkpoint(const std::string& path, const CkptHeader& h, const std::vector<int64_t>& run,
                             const std::vector<i128>& acc, const std::vector<int64_t>& msum)
{
  const std::string tmp = path + ".tmp";
  FILE* f = fopen(tmp.c_str(), "wb");
  if (!f) fail(PCG_EINVAL, "cannot write the checkpoint " + tmp);
  const size_t n = run.size();
  bool ok = fwrite(&h, sizeof(h), 1, f) == 1 && fwrite(run.data(), 8, n, f) == n &&
            fwrite(acc.data(), 16, n, f) == n && fwrite(msum.data(), 8, n, f) == n;
  ok = (fclose(f) == 0) && ok;
  if (!ok || rename(tmp.c_str(), path.c_str()) != 0) fail(PCG_EINVAL, "cannot write the checkpoint " + path);
}

SweepResult run_sweep(Ctx& c, const SweepProblem& pb, const Tuning& tune_in, cudaStream_t s)
{
  SweepResult res;
  pcg_stats& st = res.stats;
  double t_start = now_ms();
  c.tab.build_ms = 0;
  const u128 x = pb.x;
  int64_t L, x_star = 0, pi_sqrt, bglob;
  int64_t pi_limit;
  if (pb.gourdon == 2) {
    // phi(x, a) special leaves: y = pb.y (m <= y), a = pb.z, c = pb.k;
    // FactorTableD built with the prime-factor limit p_a over n <= y
    L = (int64_t) (x / (u128) pb.y);
    pi_limit = pb.y;
    ensure_prime_tables(c, pi_limit, s);
    x_star = c.tab.h_primes[(size_t) pb.z];   // p_a
    ensure_factor_d(c, x_star, pb.y, s);
    pi_sqrt = pb.z;
    bglob = pb.z;
  } else if (pb.gourdon) {
    L = (int64_t) (x / (u128) pb.z);
    x_star = x_star_gourdon(x, pb.y);
    pi_limit = pb.y;
    ensure_prime_tables(c, pi_limit, s);
    ensure_factor_d(c, pb.y, pb.z, s);
    pi_sqrt = host_pi(c.tab, (uint64_t) isqrt((u128) pb.z));
    bglob = host_pi(c.tab, (uint64_t) x_star);
  } else {
    L = pb.z;
    int64_t max_prime = std::min<int64_t>(pb.y, pb.z / std::max<int64_t>(isqrt((u128) pb.y), 1));
    pi_limit = std::max<int64_t>(pb.y, max_prime);
    ensure_prime_tables(c, pi_limit, s);
    ensure_factor_dr(c, pb.y, s);
    pi_sqrt = host_pi(c.tab, (uint64_t) isqrt((u128) pb.y));
    bglob = std::max<int64_t>(pi_sqrt, host_pi(c.tab, (uint64_t) std::min<int64_t>(isqrt((u128) pb.z), pb.y)));
    bglob = std::min<int64_t>(bglob, host_pi(c.tab, (uint64_t) max_prime));
  }
  st.table_ms = c.tab.build_ms;
  if (L <= 0 || bglob < 1) {
    st.total_ms = now_ms() - t_start;
    return res;
  }
  const int cols = (int) bglob + 1;

  // x / p_b and x / p_b^3 per level
  std::vector<uint64_t> xp((size_t) cols * 3, 0);
  for (int64_t b = 1; b <= bglob; b++) {
    u128 p = c.tab.h_primes[(size_t) b];
    u128 q = x / p;
    u128 q3 = q / (p * p);
    xp[3 * b] = (uint64_t) q;
    xp[3 * b + 1] = (uint64_t) (q >> 64);
    xp[3 * b + 2] = q3 > (u128) INT64_MAX ? (uint64_t) INT64_MAX : (uint64_t) q3;
  }

  // tuning: threads per CTA, bitmap words per CTA, leaf-record capacity,
  // resident CTAs per SM; a configuration chosen by pcg_autotune for this
  // decade of x replaces the defaults the caller left at 0
  Tuning tune = tune_in;
  {
    const int e = (int) std::floor(std::log10((double) x));
    if (e >= 0 && e < 64 && c.tuned[e] && !tune.segment_words && !tune.cta_threads && !tune.ctas_per_sm &&
        tune.group < 0) {
      tune.segment_words = c.tuned_cfg[e].segment_words;
      tune.cta_threads = c.tuned_cfg[e].cta_threads;
      tune.ctas_per_sm = c.tuned_cfg[e].ctas_per_sm;
      tune.group = c.tuned_cfg[e].group;
    }
  }
  const int NT = (tune.cta_threads == 512 || tune.cta_threads == 128) ? tune.cta_threads : 256;
  int words = tune.segment_words > 0 ? tune.segment_words : 8192;
  const int wq = std::max(8 * NT, 2048);   // whole chunks per thread and per scan lane pair
  words = std::max(words, wq);
  words = (words + wq - 1) / wq * wq;
  const int cap = 3584;
  size_t smem = (size_t) words * 8 + PAT_WORDS * 8 + (size_t) (NT + 1) * 8 * 3 + (size_t) (words / 8) * 8 +
                sizeof(LevelP) * NT + (size_t) cap * 4 + (size_t) NT * 2 + 480 * 2 + (size_t) NT * 4 + 32;
  if (smem > c.smem_optin) fail(PCG_EINVAL, "segment too large for shared memory");
  int fbytes = pb.gourdon ? c.tab.fd_bytes : c.tab.fr_bytes;
  auto occupancy = [&](int* occ) {
    if (NT == 512) { if (fbytes == 2) occupancy_sweep<uint16_t, 512>(occ, smem); else occupancy_sweep<uint32_t, 512>(occ, smem); }
    else if (NT == 256) { if (fbytes == 2) occupancy_sweep<uint16_t, 256>(occ, smem); else occupancy_sweep<uint32_t, 256>(occ, smem); }
    else { if (fbytes == 2) occupancy_sweep<uint16_t, 128>(occ, smem); else occupancy_sweep<uint32_t, 128>(occ, smem); }
  };
  int occ = 0;
  occupancy(&occ);
  int ctas = tune.ctas_per_sm > 0 ? std::min(tune.ctas_per_sm, std::max(occ, 1)) : std::max(occ, 1);
  int grid = c.num_sms * ctas;

  // segment table: small segments where leaves are dense, full ones elsewhere
  // the plan depends on the problem and the launch shape only: reused while they repeat
  const std::vector<int64_t> key = {(int64_t) (uint64_t) x, (int64_t) (uint64_t) (x >> 64), pb.y, pb.z, pb.k,
                                    (int64_t) pb.gourdon, (int64_t) words, (int64_t) grid};
  if (c.plan_key != key) {
    c.plan = plan_segments(pb, c.tab, L, x_star, pi_sqrt, bglob, (int64_t) words * 240, grid);
    c.plan_key = key;
  }
  const std::vector<int64_t>& seglo = c.plan;
  int64_t nseg = (int64_t) seglo.size() - 1;
  DevBuf& segbuf = c.tmp[T_SW_SEG];
  segbuf.alloc(seglo.size() * 8);
  PCG_CUDA(cudaMemcpyAsync(segbuf.p, seglo.data(), seglo.size() * 8, cudaMemcpyHostToDevice, s));

  // this call's segments: shard pb.shard of pb.nshards (all of them by default)
  if (pb.nshards < 1 || pb.shard < 0 || pb.shard >= pb.nshards) fail(PCG_EINVAL, "invalid shard");
  const int64_t seg_begin = nseg * pb.shard / pb.nshards;
  const int64_t seg_end = nseg * (pb.shard + 1) / pb.nshards;
  const int64_t nmine = seg_end - seg_begin;
  res.lo = seglo[(size_t) seg_begin];
  res.hi = seglo[(size_t) seg_end];

  int64_t wave_cap = (int64_t) grid * 8;
  // budget of the C/M matrices: 1 GiB
  int64_t max_rows = std::max<int64_t>(1, (int64_t) (1ull << 30) / ((int64_t) cols * 8));
  int64_t wave_len = std::max<int64_t>(1, std::min<int64_t>({nmine, wave_cap, max_rows}));

  c.cnt.alloc((size_t) wave_len * cols * 4);
  c.smu.alloc((size_t) wave_len * cols * 4);
  c.segsum.alloc((size_t) wave_len * 8);
  c.run.alloc((size_t) cols * 8);
  c.acc.alloc((size_t) cols * 16);
  c.msum.alloc((size_t) cols * 8);
  c.misc.alloc(4096);
  uint64_t* d_xp = nullptr;
  DevBuf& xpbuf = c.tmp[T_SW_XP];
  xpbuf.alloc(xp.size() * 8);
  d_xp = xpbuf.as<uint64_t>();
  PCG_CUDA(cudaMemcpyAsync(d_xp, xp.data(), xp.size() * 8, cudaMemcpyHostToDevice, s));
  PCG_CUDA(cudaMemsetAsync(c.run.p, 0, (size_t) cols * 8, s));
  PCG_CUDA(cudaMemsetAsync(c.acc.p, 0, (size_t) cols * 16, s));
  PCG_CUDA(cudaMemsetAsync(c.msum.p, 0, (size_t) cols * 8, s));
  PCG_CUDA(cudaMemsetAsync(c.misc.p, 0, 4096, s));
  unsigned long long* d_counters = (unsigned long long*) c.misc.p;
  int* d_queue = (int*) ((char*) c.misc.p + 256);   // after the 32 counters

  // the problem, the row offsets of a wave's items and the combine jobs of a
  // full wave and of the last (shorter) one
  SweepQ q0;
  memset(&q0, 0, sizeof(q0));
  q0.x_lo = (uint64_t) x;
  q0.x_hi = (uint64_t) (x >> 64);
  q0.y = pb.y;
  q0.z = pb.z;
  q0.k = pb.k;
  q0.L = L;
  q0.x_star = x_star;
  q0.item0 = 0;
  q0.seglo = segbuf.as<int64_t>();
  q0.xp_tab = d_xp;
  q0.gourdon = pb.gourdon;
  q0.pi_sqrt = (int) pi_sqrt;
  q0.bglob = (int) bglob;
  std::vector<int64_t> rowoff((size_t) wave_len);
  for (int64_t i = 0; i < wave_len; i++) rowoff[(size_t) i] = i * cols;
  DevBuf& qbuf = c.tmp[T_SW_Q];
  DevBuf& rowbuf = c.tmp[T_SW_ROW];
  DevBuf& jobbuf = c.tmp[T_SW_JOB];
  qbuf.alloc(sizeof(SweepQ));
  rowbuf.alloc(rowoff.size() * 8);
  PCG_CUDA(cudaMemcpyAsync(qbuf.p, &q0, sizeof(SweepQ), cudaMemcpyHostToDevice, s));
  PCG_CUDA(cudaMemcpyAsync(rowbuf.p, rowoff.data(), rowoff.size() * 8, cudaMemcpyHostToDevice, s));

  SweepArgs a;
  memset(&a, 0, sizeof(a));
  a.qs = qbuf.as<SweepQ>();
  a.nq = 1;
  a.rowoff = rowbuf.as<int64_t>();
  a.words = words;
  a.rec_cap = cap;
  a.primes = c.tab.primes.as<uint32_t>();
  a.nprimes = c.tab.nprimes;
  a.pitab = c.tab.pitab.as<uint64_t>();
  a.pi_max = c.tab.prime_limit;
  a.factor = pb.gourdon ? c.tab.factor_d.p : c.tab.factor_dr.p;
  a.coprime = c.tab.coprime.as<uint16_t>();
  a.group_max = tune.group >= 0 ? std::min(tune.group, GROUP_MAX) : sweep_group_max();
  a.cindex = c.tab.cindex.as<int16_t>();
  a.finv = c.tab.finv.as<uint64_t>();
  a.pmagic = c.tab.pmagic.as<uint64_t>();
  a.cnt = c.cnt.as<uint32_t>();
  a.smu = c.smu.as<int32_t>();
  a.segsum = c.segsum.as<int64_t>();
  a.counters = d_counters;

  // resume from a checkpoint of the same problem and plan
  CkptHeader ck;
  memset(&ck, 0, sizeof(ck));
  memcpy(ck.magic, "PCGSWEEP", 8);
  ck.version = 2;
  ck.gourdon = pb.gourdon;
  ck.x_lo = (uint64_t) x;
  ck.x_hi = (uint64_t) (x >> 64);
  ck.y = pb.y;
  ck.z = pb.z;
  ck.k = pb.k;
  ck.shard = pb.shard;
  ck.nshards = pb.nshards;
  ck.words = words;
  ck.nt = NT;
  ck.nseg = nseg;
  ck.cols = cols;
  ck.plan_hash = plan_hash(seglo);
  const bool use_ckpt = !tune.checkpoint.empty();
  int64_t start_first = seg_begin;
  if (use_ckpt) {
    CkptHeader got;
    std::vector<int64_t> r0, m0;
    std::vector<i128> a0;
    if (read_checkpoint(tune.checkpoint, ck, got, r0, a0, m0) && got.next_first >= seg_begin &&
        got.next_first <= seg_end) {
      PCG_CUDA(cudaMemcpyAsync(c.run.p, r0.data(), (size_t) cols * 8, cudaMemcpyHostToDevice, s));
      PCG_CUDA(cudaMemcpyAsync(c.acc.p, a0.data(), (size_t) cols * 16, cudaMemcpyHostToDevice, s));
      PCG_CUDA(cudaMemcpyAsync(c.msum.p, m0.data(), (size_t) cols * 8, cudaMemcpyHostToDevice, s));
      PCG_CUDA(cudaMemcpyAsync(d_counters, got.counters, sizeof(got.counters), cudaMemcpyHostToDevice, s));
      PCG_CUDA(cudaStreamSynchronize(s));
      start_first = got.next_first;
      ck.waves = got.waves;
    }
  }
  double last_write = now_ms();
  auto save = [&](int64_t next_first) {
    std::vector<int64_t> r0((size_t) cols), m0((size_t) cols);
    std::vector<i128> a0((size_t) cols);
    PCG_CUDA(cudaMemcpyAsync(r0.data(), c.run.p, (size_t) cols * 8, cudaMemcpyDeviceToHost, s));
    PCG_CUDA(cudaMemcpyAsync(a0.data(), c.acc.p, (size_t) cols * 16, cudaMemcpyDeviceToHost, s));
    PCG_CUDA(cudaMemcpyAsync(m0.data(), c.msum.p, (size_t) cols * 8, cudaMemcpyDeviceToHost, s));
    PCG_CUDA(cudaMemcpyAsync(ck.counters, d_counters, sizeof(ck.counters), cudaMemcpyDeviceToHost, s));
    PCG_CUDA(cudaStreamSynchronize(s));
    ck.next_first = next_first;
    write_checkpoint(tune.checkpoint, ck, r0, a0, m0);
    last_write = now_ms();
  };

  // combine jobs of a full wave and of the last one (from start_first on)
  const int64_t last_len = seg_end > start_first ? (seg_end - start_first - 1) % wave_len + 1 : wave_len;
  std::vector<CombineJob> jobs;
  add_combine_jobs(jobs, 0, 0, (int) wave_len, cols);
  const int njobs = (int) jobs.size();
  add_combine_jobs(jobs, 0, 0, (int) last_len, cols);
  jobbuf.alloc(jobs.size() * sizeof(CombineJob));
  PCG_CUDA(cudaMemcpyAsync(jobbuf.p, jobs.data(), jobs.size() * sizeof(CombineJob), cudaMemcpyHostToDevice, s));

  PCG_CUDA(cudaEventRecord(c.ev[0], s));
  uint64_t launches = 0;
  float ms_sweep = 0;
  int waves = 0;
  for (int64_t first = start_first; first < seg_end; first += wave_len) {
    int wl = (int) std::min<int64_t>(wave_len, seg_end - first);
    a.wave_first = first;
    a.wave_len = wl;
    a.queue = d_queue + (waves % 16);
    PCG_CUDA(cudaMemsetAsync(c.cnt.p, 0, (size_t) wl * cols * 4, s));
    PCG_CUDA(cudaMemsetAsync(c.smu.p, 0, (size_t) wl * cols * 4, s));
    if (waves % 16 == 0 && waves > 0) PCG_CUDA(cudaMemsetAsync(d_queue, 0, 64, s));
    int g = (int) std::min<int64_t>(grid, wl);
    if ((size_t) (2 * waves + 2) > c.kev.size()) {
      size_t n0 = c.kev.size();
      c.kev.resize((size_t) (2 * waves + 2) * 2);
      for (size_t i = n0; i < c.kev.size(); i++) PCG_CUDA(cudaEventCreate(&c.kev[i]));
    }
    PCG_CUDA(cudaEventRecord(c.kev[2 * waves], s));
    if (NT == 512) { if (fbytes == 2) launch_sweep<uint16_t, 512>(a, g, smem, s); else launch_sweep<uint32_t, 512>(a, g, smem, s); }
    else if (NT == 256) { if (fbytes == 2) launch_sweep<uint16_t, 256>(a, g, smem, s); else launch_sweep<uint32_t, 256>(a, g, smem, s); }
    else { if (fbytes == 2) launch_sweep<uint16_t, 128>(a, g, smem, s); else launch_sweep<uint32_t, 128>(a, g, smem, s); }
    PCG_CUDA(cudaGetLastError());
    PCG_CUDA(cudaEventRecord(c.kev[2 * waves + 1], s));
    const CombineJob* wj = jobbuf.as<CombineJob>() + (wl == wave_len ? 0 : njobs);
    k_combine<<<njobs, 32 * COMBINE_WARPS, 0, s>>>(a.cnt, a.smu, a.rowoff, a.segsum, wj, c.run.as<int64_t>(),
                                                  c.acc.as<i128>(), c.msum.as<int64_t>());
    PCG_CUDA(cudaGetLastError());
    launches += 2;
    waves++;
    ck.waves++;
    const int64_t next = std::min<int64_t>(first + wave_len, seg_end);
    if (use_ckpt && next < seg_end) {
      const bool stop = tune.stop_after_waves > 0 && waves >= tune.stop_after_waves;
      if (stop || now_ms() - last_write >= 1000.0 * tune.checkpoint_interval) save(next);
      if (stop)
        fail(PCG_ECANCELLED, "sweep stopped after " + std::to_string(waves) + " waves; checkpoint written to " +
                                 tune.checkpoint);
    }
  }
  PCG_CUDA(cudaEventRecord(c.ev[1], s));
  std::vector<i128> acc((size_t) cols);
  unsigned long long ctr[5];
  PCG_CUDA(cudaMemcpyAsync(acc.data(), c.acc.p, (size_t) cols * 16, cudaMemcpyDeviceToHost, s));
  PCG_CUDA(cudaMemcpyAsync(ctr, d_counters, sizeof(ctr), cudaMemcpyDeviceToHost, s));
  if (pb.parts) {
    res.msum.resize((size_t) cols);
    res.csum.resize((size_t) cols);
    PCG_CUDA(cudaMemcpyAsync(res.msum.data(), c.msum.p, (size_t) cols * 8, cudaMemcpyDeviceToHost, s));
    PCG_CUDA(cudaMemcpyAsync(res.csum.data(), c.run.p, (size_t) cols * 8, cudaMemcpyDeviceToHost, s));
  }
  PCG_CUDA(cudaStreamSynchronize(s));
  if (pb.parts) res.acc = acc;
  PCG_CUDA(cudaEventElapsedTime(&ms_sweep, c.ev[0], c.ev[1]));
  double kms = 0;
  for (int w = 0; w < waves; w++) {
    float m = 0;
    PCG_CUDA(cudaEventElapsedTime(&m, c.kev[2 * w], c.kev[2 * w + 1]));
    kms += m;
  }
  st.sweep_kernel_ms = kms;
  st.sweep_launches = (uint64_t) waves;
  st.h2d_bytes = xp.size() * 8 + seglo.size() * 8 + sizeof(SweepQ) + rowoff.size() * 8 +
                 jobs.size() * sizeof(CombineJob);
  st.d2h_bytes = (uint64_t) cols * 16 + sizeof(ctr);
  i128 sum = 0;
  for (int b = 0; b < cols; b++) sum += acc[(size_t) b];
  res.sum = sum;
  st.leaves = ctr[0];
  st.two_prime_leaves = ctr[1];
  st.levels = ctr[2];
  st.factor_entries = ctr[3];
  st.crossoff_multiples = ctr[4];
  st.segments = (uint64_t) nmine;
  st.kernel_launches = launches;
  if (use_ckpt) remove(tune.checkpoint.c_str());
  st.sweep_ms = ms_sweep;
  st.combine_ms = ms_sweep - kms;
  st.segment_words = words;
  st.ctas_per_sm = ctas;
  st.threads_per_cta = NT;
  st.total_ms = now_ms() - t_start;
  return res;
}


// Device working memory of one sweep over [0, L) with cols columns, at the
// default launch shape (words per segment, 2 CTAs per SM): the count and sign
// rows of a wave, the segment, x / p, row and job tables and the sums.  The
// segment planner cuts at most about L / (words * 240) + 6 grid segments.
uint64_t sweep_device_bytes(int num_sms, int64_t L, int64_t cols, int words)
{
  if (L <= 0 || cols <= 1) return 0;
  const int64_t grid = (int64_t) num_sms * 2;
  const int64_t nseg = L / ((int64_t) words * 240) + 6 * grid + 2;
  const int64_t max_rows = std::max<int64_t>(1, (int64_t) (1ull << 30) / (cols * 8));
  const int64_t wave = std::max<int64_t>(1, std::min<int64_t>({nseg, grid * 8, max_rows}));
  return (uint64_t) (wave * cols * 8 + wave * 16 + (nseg + 1) * 8 + cols * 56 +
                     ((cols + 31) / 32 + 1) * 2 * (int64_t) sizeof(CombineJob) + 4096 + sizeof(SweepQ));
}

// The per-call working memory a context keeps between calls (count and sign
// rows, per-call temporaries), freed; the resident tables stay.
uint64_t ctx_trim(Ctx& c)
{
  uint64_t freed = c.cnt.bytes + c.smu.bytes + c.segsum.bytes + c.run.bytes + c.acc.bytes + c.msum.bytes;
  c.cnt.free_();
  c.smu.free_();
  c.segsum.free_();
  c.run.free_();
  c.acc.free_();
  c.msum.free_();
  for (DevBuf& b : c.tmp) {
    freed += b.bytes;
    b.free_();
  }
  return freed;
}

// ================================================================ batched sweep
// D(x, y, z, k) of many problems in one sweep.  Every problem's segments are
// the work items of one persistent kernel launch per wave (CTAs pull items
// of all problems from one atomic counter); a wave is a run of consecutive
// items whose count and sign rows fit the budget, and its combine jobs scan
// each problem's items in order.  The whole launch sequence is captured in a
// CUDA graph and launched once.  The tables are shared: primes and PiTable up
// to the largest y, one FactorTableD for the largest z built without the
// mpf <= y filter -- exact for problems with y >= z, whose filter passes
// every n <= z (the reference's default parameters have y = z).
void run_sweep_batch(Ctx& c, const std::vector<SweepProblem>& pbs, const Tuning& tune_in, cudaStream_t s,
                     std::vector<i128>& sums, pcg_stats* stp)
{
  pcg_stats st{};
  const double t_start = now_ms();
  c.tab.build_ms = 0;
  const size_t nq = pbs.size();
  sums.assign(nq, 0);
  if (nq == 0) { if (stp) *stp = st; return; }
  int64_t ymax = 1, zmax = 1;
  u128 xmax = 0;
  for (const SweepProblem& p : pbs) {
    if (p.gourdon != 1 || p.y < p.z || p.y < 1 || p.z < 1) fail(PCG_EINVAL, "batched sweep: D problems with y >= z only");
    ymax = std::max(ymax, p.y);
    zmax = std::max(zmax, p.z);
    xmax = std::max(xmax, p.x);
  }
  ensure_prime_tables(c, ymax, s);
  ensure_factor_d(c, zmax, zmax, s);
  const Tables& T = c.tab;
  st.table_ms = T.build_ms;

  // tuning: the context's autotuned choice for the largest x's decade, else the defaults
  Tuning tune = tune_in;
  {
    const int e = (int) std::floor(std::log10((double) xmax));
    if (e >= 0 && e < 64 && c.tuned[e] && !tune.segment_words && !tune.cta_threads && !tune.ctas_per_sm &&
        tune.group < 0) {
      tune.segment_words = c.tuned_cfg[e].segment_words;
      tune.cta_threads = c.tuned_cfg[e].cta_threads;
      tune.ctas_per_sm = c.tuned_cfg[e].ctas_per_sm;
      tune.group = c.tuned_cfg[e].group;
    }
  }
  const int NT = (tune.cta_threads == 512 || tune.cta_threads == 128) ? tune.cta_threads : 256;
  int words = tune.segment_words > 0 ? tune.segment_words : 8192;
  const int wq = std::max(8 * NT, 2048);
  words = std::max(words, wq);
  words = (words + wq - 1) / wq * wq;
  const int cap = 3584;
  const size_t smem = (size_t) words * 8 + PAT_WORDS * 8 + (size_t) (NT + 1) * 8 * 3 + (size_t) (words / 8) * 8 +
                      sizeof(LevelP) * NT + (size_t) cap * 4 + (size_t) NT * 2 + 480 * 2 + (size_t) NT * 4 + 32;
  if (smem > c.smem_optin) fail(PCG_EINVAL, "segment too large for shared memory");
  const int fbytes = T.fd_bytes;
  int occ = 0;
  if (NT == 512) { if (fbytes == 2) occupancy_sweep<uint16_t, 512>(&occ, smem); else occupancy_sweep<uint32_t, 512>(&occ, smem); }
  else if (NT == 256) { if (fbytes == 2) occupancy_sweep<uint16_t, 256>(&occ, smem); else occupancy_sweep<uint32_t, 256>(&occ, smem); }
  else { if (fbytes == 2) occupancy_sweep<uint16_t, 128>(&occ, smem); else occupancy_sweep<uint32_t, 128>(&occ, smem); }
  const int ctas = tune.ctas_per_sm > 0 ? std::min(tune.ctas_per_sm, std::max(occ, 1)) : std::max(occ, 1);
  const int grid = c.num_sms * ctas;
  const int64_t smax = (int64_t) words * 240;

  // per problem: parameters, x / p table and segment plan (host threads)
  struct Plan {
    SweepQ q;
    std::vector<uint64_t> xp;
    std::vector<int64_t> seg;
    int64_t cols = 0;
  };
  std::vector<Plan> plans(nq);
  {
    std::vector<double> dens((size_t) host_pi(T, (uint64_t) std::min<int64_t>(ymax, T.prime_limit)) + 2, 0.0);
    for (size_t b = 1; b < dens.size() && (int64_t) b <= T.nprimes; b++)
      dens[b] = 0.56 / std::log(std::max((double) T.h_primes[b], 3.0));
    std::atomic<size_t> next{0};
    std::exception_ptr err;
    std::mutex err_mu;
    auto work = [&] {
      for (;;) {
        const size_t i = next.fetch_add(1);
        if (i >= nq) return;
        try {
          const SweepProblem& pb = pbs[i];
          Plan& P = plans[i];
          memset(&P.q, 0, sizeof(P.q));
          const u128 x = pb.x;
          const int64_t L = (int64_t) (x / (u128) pb.z);
          const int64_t x_star = x_star_gourdon(x, pb.y);
          const int64_t pi_sqrt = host_pi(T, (uint64_t) isqrt((u128) pb.z));
          const int64_t bglob = host_pi(T, (uint64_t) x_star);
          if (L <= 0 || bglob < 1) continue;
          P.cols = bglob + 1;
          P.xp.assign((size_t) P.cols * 3, 0);
          for (int64_t b = 1; b <= bglob; b++) {
            const u128 p = T.h_primes[(size_t) b];
            const u128 q = x / p, q3 = q / (p * p);
            P.xp[3 * b] = (uint64_t) q;
            P.xp[3 * b + 1] = (uint64_t) (q >> 64);
            P.xp[3 * b + 2] = q3 > (u128) INT64_MAX ? (uint64_t) INT64_MAX : (uint64_t) q3;
          }
          // small problems: one cost cell per segment is plenty
          const int G = (int) std::min<int64_t>(PLAN_GRID, std::max<int64_t>(16, 4 * (L / smax + 1)));
          plan_segments_core(pb, T, L, x_star, pi_sqrt, bglob, smax, grid, dens.data(), 1,
                             [&](int64_t v) { P.seg.push_back(v); return true; }, G);
          P.q.x_lo = (uint64_t) x;
          P.q.x_hi = (uint64_t) (x >> 64);
          P.q.y = pb.y;
          P.q.z = pb.z;
          P.q.k = pb.k;
          P.q.L = L;
          P.q.x_star = x_star;
          P.q.gourdon = 1;
          P.q.pi_sqrt = (int) pi_sqrt;
          P.q.bglob = (int) bglob;
        } catch (...) {
          std::lock_guard<std::mutex> g(err_mu);
          if (!err) err = std::current_exception();
          return;
        }
      }
    };
    const unsigned nth = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (unsigned k = 0; k < nth; k++) th.emplace_back(work);
    for (auto& h : th) h.join();
    if (err) std::rethrow_exception(err);
  }

  // concatenated problem tables; items numbered problem by problem
  std::vector<size_t> live;
  int64_t nitems = 0, ncells = 0, nseg_all = 0, nxp = 0;
  for (size_t i = 0; i < nq; i++) {
    if (plans[i].cols == 0) continue;
    live.push_back(i);
    nseg_all += (int64_t) plans[i].seg.size();
    nxp += (int64_t) plans[i].xp.size();
    ncells += plans[i].cols;
    nitems += (int64_t) plans[i].seg.size() - 1;
  }
  if (live.empty()) { st.total_ms = now_ms() - t_start; if (stp) *stp = st; return; }
  std::vector<int64_t> seg_all;
  std::vector<uint64_t> xp_all;
  seg_all.reserve((size_t) nseg_all);
  xp_all.reserve((size_t) nxp);
  DevBuf& segbuf = c.tmp[T_SW_SEG];
  DevBuf& xpbuf = c.tmp[T_SW_XP];
  segbuf.alloc((size_t) nseg_all * 8);
  xpbuf.alloc((size_t) nxp * 8);
  std::vector<SweepQ> qs;
  std::vector<int64_t> colbase;   // by live index
  std::vector<int64_t> first_item;
  {
    int64_t item = 0, cb = 0;
    for (size_t li = 0; li < live.size(); li++) {
      Plan& P = plans[live[li]];
      P.q.item0 = item;
      P.q.seglo = segbuf.as<int64_t>() + seg_all.size();
      P.q.xp_tab = xpbuf.as<uint64_t>() + xp_all.size();
      seg_all.insert(seg_all.end(), P.seg.begin(), P.seg.end());
      xp_all.insert(xp_all.end(), P.xp.begin(), P.xp.end());
      qs.push_back(P.q);
      colbase.push_back(cb);
      first_item.push_back(item);
      item += (int64_t) P.seg.size() - 1;
      cb += P.cols;
    }
  }
  // waves: consecutive items whose rows fit the budget; per wave the items'
  // row offsets and the combine jobs of each problem run in it
  const int64_t cell_budget = (int64_t) (1ull << 30) / 8;
  const int64_t item_cap = (int64_t) grid * 16;
  struct Wave { int64_t first, len, row_at, job_at, njobs, cells; };
  std::vector<Wave> waves;
  std::vector<int64_t> rows;
  std::vector<CombineJob> jobs;
  {
    size_t li = 0;
    int64_t item = 0;
    while (item < nitems) {
      Wave w{item, 0, (int64_t) rows.size(), (int64_t) jobs.size(), 0, 0};
      while (item < nitems) {
        while (li + 1 < live.size() && first_item[li + 1] <= item) li++;
        const int64_t cols = plans[live[li]].cols;
        if (w.len > 0 && (w.len >= item_cap || w.cells + cols > cell_budget)) break;
        rows.push_back(w.cells);
        w.cells += cols;
        w.len++;
        item++;
      }
      // jobs: the runs of each problem's items inside the wave
      int64_t i = w.first;
      size_t lj = 0;
      while (lj + 1 < live.size() && first_item[lj + 1] <= i) lj++;
      while (i < w.first + w.len) {
        const int64_t pend = (lj + 1 < live.size()) ? first_item[lj + 1] : nitems;
        const int64_t e = std::min(pend, w.first + w.len);
        add_combine_jobs(jobs, colbase[lj], (int) (i - w.first), (int) (e - i), (int) plans[live[lj]].cols);
        i = e;
        lj++;
      }
      w.njobs = (int64_t) jobs.size() - w.job_at;
      waves.push_back(w);
    }
  }
  int64_t max_cells = 0, max_len = 0;
  for (const Wave& w : waves) { max_cells = std::max(max_cells, w.cells); max_len = std::max(max_len, w.len); }

  DevBuf& qbuf = c.tmp[T_SW_Q];
  DevBuf& rowbuf = c.tmp[T_SW_ROW];
  DevBuf& jobbuf = c.tmp[T_SW_JOB];
  qbuf.alloc(qs.size() * sizeof(SweepQ));
  rowbuf.alloc(rows.size() * 8);
  jobbuf.alloc(jobs.size() * sizeof(CombineJob));
  c.cnt.alloc((size_t) max_cells * 4);
  c.smu.alloc((size_t) max_cells * 4);
  c.segsum.alloc((size_t) max_len * 8);
  c.run.alloc((size_t) ncells * 8);
  c.acc.alloc((size_t) ncells * 16);
  c.misc.alloc(4096);
  PCG_CUDA(cudaMemcpyAsync(segbuf.p, seg_all.data(), seg_all.size() * 8, cudaMemcpyHostToDevice, s));
  PCG_CUDA(cudaMemcpyAsync(xpbuf.p, xp_all.data(), xp_all.size() * 8, cudaMemcpyHostToDevice, s));
  PCG_CUDA(cudaMemcpyAsync(qbuf.p, qs.data(), qs.size() * sizeof(SweepQ), cudaMemcpyHostToDevice, s));
  PCG_CUDA(cudaMemcpyAsync(rowbuf.p, rows.data(), rows.size() * 8, cudaMemcpyHostToDevice, s));
  PCG_CUDA(cudaMemcpyAsync(jobbuf.p, jobs.data(), jobs.size() * sizeof(CombineJob), cudaMemcpyHostToDevice, s));
  PCG_CUDA(cudaMemsetAsync(c.run.p, 0, (size_t) ncells * 8, s));
  PCG_CUDA(cudaMemsetAsync(c.acc.p, 0, (size_t) ncells * 16, s));
  PCG_CUDA(cudaMemsetAsync(c.misc.p, 0, 4096, s));
  unsigned long long* d_counters = (unsigned long long*) c.misc.p;
  int* d_queue = (int*) ((char*) c.misc.p + 256);
  // the launch attributes are set before the capture
  if (NT == 512) { if (fbytes == 2) set_sweep_attr<uint16_t, 512>(smem); else set_sweep_attr<uint32_t, 512>(smem); }
  else if (NT == 256) { if (fbytes == 2) set_sweep_attr<uint16_t, 256>(smem); else set_sweep_attr<uint32_t, 256>(smem); }
  else { if (fbytes == 2) set_sweep_attr<uint16_t, 128>(smem); else set_sweep_attr<uint32_t, 128>(smem); }
  PCG_CUDA(cudaStreamSynchronize(s));

  SweepArgs a;
  memset(&a, 0, sizeof(a));
  a.qs = qbuf.as<SweepQ>();
  a.nq = (int) qs.size();
  a.words = words;
  a.rec_cap = cap;
  a.primes = T.primes.as<uint32_t>();
  a.nprimes = T.nprimes;
  a.pitab = T.pitab.as<uint64_t>();
  a.pi_max = T.prime_limit;
  a.factor = T.factor_d.p;
  a.coprime = T.coprime.as<uint16_t>();
  a.group_max = tune.group >= 0 ? std::min(tune.group, GROUP_MAX) : sweep_group_max();
  a.cindex = T.cindex.as<int16_t>();
  a.finv = T.finv.as<uint64_t>();
  a.pmagic = T.pmagic.as<uint64_t>();
  a.cnt = c.cnt.as<uint32_t>();
  a.smu = c.smu.as<int32_t>();
  a.segsum = c.segsum.as<int64_t>();
  a.counters = d_counters;

  // the wave sequence, captured into one graph
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  PCG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  try {
    for (size_t wi = 0; wi < waves.size(); wi++) {
      const Wave& w = waves[wi];
      a.wave_first = w.first;
      a.wave_len = (int32_t) w.len;
      a.rowoff = rowbuf.as<int64_t>() + w.row_at;
      a.queue = d_queue + (wi % 16);
      PCG_CUDA(cudaMemsetAsync(c.cnt.p, 0, (size_t) w.cells * 4, s));
      PCG_CUDA(cudaMemsetAsync(c.smu.p, 0, (size_t) w.cells * 4, s));
      if (wi % 16 == 0 && wi > 0) PCG_CUDA(cudaMemsetAsync(d_queue, 0, 64, s));
      const int g = (int) std::min<int64_t>(grid, w.len);
      if (NT == 512) { if (fbytes == 2) k_sweep<uint16_t, 512><<<g, 512, smem, s>>>(a); else k_sweep<uint32_t, 512><<<g, 512, smem, s>>>(a); }
      else if (NT == 256) { if (fbytes == 2) k_sweep<uint16_t, 256><<<g, 256, smem, s>>>(a); else k_sweep<uint32_t, 256><<<g, 256, smem, s>>>(a); }
      else { if (fbytes == 2) k_sweep<uint16_t, 128><<<g, 128, smem, s>>>(a); else k_sweep<uint32_t, 128><<<g, 128, smem, s>>>(a); }
      PCG_CUDA(cudaGetLastError());
      k_combine<<<(unsigned) w.njobs, 32 * COMBINE_WARPS, 0, s>>>(a.cnt, a.smu, a.rowoff, a.segsum,
                                                                  jobbuf.as<CombineJob>() + w.job_at, c.run.as<int64_t>(),
                                                                  c.acc.as<i128>(), nullptr);
      PCG_CUDA(cudaGetLastError());
    }
    PCG_CUDA(cudaStreamEndCapture(s, &graph));
  } catch (...) {
    cudaGraph_t g2 = nullptr;
    cudaStreamEndCapture(s, &g2);
    if (g2) cudaGraphDestroy(g2);
    cudaGetLastError();
    throw;
  }
  try {
    PCG_CUDA(cudaGraphInstantiate(&exec, graph, 0));
    PCG_CUDA(cudaEventRecord(c.ev[0], s));
    PCG_CUDA(cudaGraphLaunch(exec, s));
    PCG_CUDA(cudaEventRecord(c.ev[1], s));
    std::vector<i128> acc((size_t) ncells);
    unsigned long long ctr[5];
    PCG_CUDA(cudaMemcpyAsync(acc.data(), c.acc.p, (size_t) ncells * 16, cudaMemcpyDeviceToHost, s));
    PCG_CUDA(cudaMemcpyAsync(ctr, d_counters, sizeof(ctr), cudaMemcpyDeviceToHost, s));
    PCG_CUDA(cudaStreamSynchronize(s));
    for (size_t li = 0; li < live.size(); li++) {
      i128 t = 0;
      for (int64_t b = 0; b < plans[live[li]].cols; b++) t += acc[(size_t) (colbase[li] + b)];
      sums[live[li]] = t;
    }
    float ms = 0;
    PCG_CUDA(cudaEventElapsedTime(&ms, c.ev[0], c.ev[1]));
    st.leaves = ctr[0];
    st.two_prime_leaves = ctr[1];
    st.levels = ctr[2];
    st.factor_entries = ctr[3];
    st.crossoff_multiples = ctr[4];
    st.sweep_ms = ms;
    st.sweep_kernel_ms = ms;
    st.sweep_launches = waves.size();
    st.kernel_launches = 2 * waves.size();
    st.segments = (uint64_t) nitems;
    st.h2d_bytes = seg_all.size() * 8 + xp_all.size() * 8 + qs.size() * sizeof(SweepQ) + rows.size() * 8 +
                   jobs.size() * sizeof(CombineJob);
    st.d2h_bytes = (uint64_t) ncells * 16 + sizeof(ctr);
    st.segment_words = words;
    st.ctas_per_sm = ctas;
    st.threads_per_cta = NT;
  } catch (...) {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    throw;
  }
  cudaGraphExecDestroy(exec);
  cudaGraphDestroy(graph);
  st.total_ms = now_ms() - t_start;
  if (stp) *stp = st;
}

// ================================================================ allocation-free D
// Some callers cannot allocate device memory at the time they need D(x): a
// serving loop that must not touch the allocator on its request path, or a
// host whose device memory is owned by another framework's pool, where a
// cudaMalloc would fail or would take memory the pool accounts for.
// pcg_D_noalloc serves them: it reads the tables a context built earlier (at
// set-up, when allocating was allowed) and takes all of its device working
// memory -- the per-(segment, level) count and sign matrices, the segment
// and x/p tables, the counters and the work queue -- from the file-scope
// array below, and its host working memory from static arrays.  Every GPU
// that loads this library holds the device array until the process exits.
// All calls share it and it keeps the previous call's contents, so
// everything that must start at zero is cleared on the stream at the start
// of a call.  Calls are serialised on the host by a mutex and each call
// waits for its own work before it returns (also when it fails), but two
// calls whose work overlaps on the GPU race on the array.
#define PCG_NOALLOC_SCRATCH_BYTES (64ull << 20)
#define PCG_NOALLOC_MAX_COLS 32768
#define PCG_NOALLOC_MAX_SEGS (1 << 20)
#define PCG_NOALLOC_MAX_ROWS (1 << 16)
static __device__ __align__(256) unsigned char g_noalloc_scratch[PCG_NOALLOC_SCRATCH_BYTES];

// Device address of the scratch array for device dev.  Host code only holds
// a host-side stand-in for the symbol, so the address comes from
// cudaGetSymbolAddress, once per device with that device current (the
// caller makes dev current).  The first call on a device does this set-up,
// so it should come before any stream capture.
static unsigned char* noalloc_scratch(int dev)
{
  static std::mutex mu;
  static unsigned char* addr[64] = {nullptr};
  if (dev < 0 || dev >= 64) fail(PCG_EINVAL, "device index out of range");
  std::lock_guard<std::mutex> g(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      cudaGetLastError();
      fail(PCG_ECUDA, std::string("cudaGetSymbolAddress of the no-alloc scratch failed: ") + cudaGetErrorString(e));
    }
    addr[dev] = (unsigned char*) p;
  }
  return addr[dev];
}

SweepResult run_sweep_noalloc(Ctx& c, const SweepProblem& pb, cudaStream_t s)
{
  static std::mutex call_mu;
  static uint64_t h_xp[3 * PCG_NOALLOC_MAX_COLS];
  static double h_dens[PCG_NOALLOC_MAX_COLS];
  static int64_t h_seg[PCG_NOALLOC_MAX_SEGS + 1];
  static int64_t h_nseg = -1;
  static int64_t h_plan_key[8];
  static i128 h_acc[PCG_NOALLOC_MAX_COLS];
  static SweepQ h_q;
  static int64_t h_row[PCG_NOALLOC_MAX_ROWS];
  static CombineJob h_jobs[2 * (PCG_NOALLOC_MAX_COLS / 32 + 2)];
  std::lock_guard<std::mutex> guard(call_mu);
  SweepResult res;
  pcg_stats& st = res.stats;
  double t_start = now_ms();
  // the context's device, whichever device the calling thread has current
  PCG_CUDA(cudaSetDevice(c.device));
  unsigned char* scratch = noalloc_scratch(c.device);
  const u128 x = pb.x;
  const Tables& T = c.tab;
  // the tables are inputs: they must already be resident (no building here)
  if (!pb.gourdon) fail(PCG_EINVAL, "pcg_D_noalloc computes D only");
  if (T.prime_limit < pb.y || !(T.fd_z >= pb.z && (T.fd_y == pb.y || (pb.y >= pb.z && T.fd_y >= pb.z))))
    fail(PCG_ERANGE, "pcg_D_noalloc: the context's resident tables do not cover y = " + std::to_string(pb.y) +
                         ", z = " + std::to_string(pb.z) + " (create the context with a larger max_x)");
  const int64_t L = (int64_t) (x / (u128) pb.z);
  const int64_t x_star = x_star_gourdon(x, pb.y);
  const int64_t pi_sqrt = host_pi(T, (uint64_t) isqrt((u128) pb.z));
  const int64_t bglob = host_pi(T, (uint64_t) x_star);
  if (L <= 0 || bglob < 1) {
    st.total_ms = now_ms() - t_start;
    return res;
  }
  const int cols = (int) bglob + 1;
  if (cols > PCG_NOALLOC_MAX_COLS)
    fail(PCG_ERANGE, "pcg_D_noalloc: " + std::to_string(cols) + " levels exceed the maximum of " +
                         std::to_string(PCG_NOALLOC_MAX_COLS));
  for (int64_t b = 1; b <= bglob; b++) {
    u128 p = T.h_primes[(size_t) b];
    u128 q = x / p;
    u128 q3 = q / (p * p);
    h_xp[3 * b] = (uint64_t) q;
    h_xp[3 * b + 1] = (uint64_t) (q >> 64);
    h_xp[3 * b + 2] = q3 > (u128) INT64_MAX ? (uint64_t) INT64_MAX : (uint64_t) q3;
  }
  h_xp[0] = h_xp[1] = h_xp[2] = 0;

  const int NT = 256;
  const int words = 8192;
  const int cap = 3584;
  size_t smem = (size_t) words * 8 + PAT_WORDS * 8 + (size_t) (NT + 1) * 8 * 3 + (size_t) (words / 8) * 8 +
                sizeof(LevelP) * NT + (size_t) cap * 4 + (size_t) NT * 2 + 480 * 2 + (size_t) NT * 4 + 32;
  const int fbytes = T.fd_bytes;
  int occ = 0;
  if (fbytes == 2) occupancy_sweep<uint16_t, 256>(&occ, smem);
  else occupancy_sweep<uint32_t, 256>(&occ, smem);
  const int ctas = std::max(occ, 1);
  const int grid = c.num_sms * ctas;
  // the segment plan of run_sweep's planner, costed on this thread and kept
  // for the next call with the same problem and launch shape
  const int64_t key[8] = {(int64_t) (uint64_t) x, (int64_t) (uint64_t) (x >> 64), pb.y, pb.z, pb.k, words, grid,
                          (int64_t) T.prime_limit};
  if (h_nseg < 0 || memcmp(key, h_plan_key, sizeof(key)) != 0) {
    for (int64_t b = 1; b <= bglob; b++) h_dens[b] = 0.56 / std::log(std::max((double) T.h_primes[(size_t) b], 3.0));
    int64_t n = 0;
    h_nseg = -1;
    const bool ok = plan_segments_core(pb, T, L, x_star, pi_sqrt, bglob, (int64_t) words * 240, grid, h_dens, 1,
                                       [&](int64_t v) {
                                         if (n > PCG_NOALLOC_MAX_SEGS) return false;
                                         h_seg[n++] = v;
                                         return true;
                                       });
    if (!ok) fail(PCG_ERANGE, "pcg_D_noalloc: too many segments for the fixed segment table");
    h_nseg = n - 1;
    memcpy(h_plan_key, key, sizeof(key));
  }
  const int64_t nseg = h_nseg;

  // carve the scratch: counters and queue, x/p table, segment table, run,
  // acc, segsum, then the count and sign matrices with as many rows as fit
  auto align = [](size_t v) { return (v + 255) & ~(size_t) 255; };
  size_t off = 0;
  unsigned long long* d_counters = (unsigned long long*) (scratch + off);
  int* d_queue = (int*) (scratch + off + 256);
  off = align(off + 4096);
  uint64_t* d_xp = (uint64_t*) (scratch + off);
  off = align(off + (size_t) cols * 24);
  int64_t* d_seg = (int64_t*) (scratch + off);
  off = align(off + (size_t) (nseg + 1) * 8);
  int64_t* d_run = (int64_t*) (scratch + off);
  off = align(off + (size_t) cols * 8);
  i128* d_acc = (i128*) (scratch + off);
  off = align(off + (size_t) cols * 16);
  const size_t fixed = off;
  const size_t per_row = (size_t) cols * 8 + 8 + 512;
  if (fixed + per_row > PCG_NOALLOC_SCRATCH_BYTES)
    fail(PCG_ERANGE, "pcg_D_noalloc: needs more than the " + std::to_string(PCG_NOALLOC_SCRATCH_BYTES) +
                         "-byte static scratch (x too large for the allocation-free path)");
  const int njobs = (cols + 31) / 32 + 1;
  const size_t jobs_bytes = (size_t) 2 * njobs * sizeof(CombineJob);
  int64_t wave_len = std::min<int64_t>({nseg, (int64_t) grid * 8, (int64_t) PCG_NOALLOC_MAX_ROWS,
                                        (int64_t) ((PCG_NOALLOC_SCRATCH_BYTES - fixed - align(jobs_bytes) - 512) /
                                                   (per_row + 8))});
  if (wave_len < 1) fail(PCG_ERANGE, "pcg_D_noalloc: x too large for the allocation-free path");
  SweepQ* d_q = (SweepQ*) (scratch + off);
  off = align(off + sizeof(SweepQ));
  CombineJob* d_jobs = (CombineJob*) (scratch + off);
  off = align(off + jobs_bytes);
  int64_t* d_row = (int64_t*) (scratch + off);
  off = align(off + (size_t) wave_len * 8);
  int64_t* d_segsum = (int64_t*) (scratch + off);
  off = align(off + (size_t) wave_len * 8);
  uint32_t* d_cnt = (uint32_t*) (scratch + off);
  off = align(off + (size_t) wave_len * cols * 4);
  int32_t* d_smu = (int32_t*) (scratch + off);
  off = align(off + (size_t) wave_len * cols * 4);
  if (off > PCG_NOALLOC_SCRATCH_BYTES) fail(PCG_EINTERNAL, "no-alloc scratch carve overflow");

  memset(&h_q, 0, sizeof(h_q));
  h_q.x_lo = (uint64_t) x;
  h_q.x_hi = (uint64_t) (x >> 64);
  h_q.y = pb.y;
  h_q.z = pb.z;
  h_q.k = pb.k;
  h_q.L = L;
  h_q.x_star = x_star;
  h_q.item0 = 0;
  h_q.seglo = d_seg;
  h_q.xp_tab = d_xp;
  h_q.gourdon = 1;
  h_q.pi_sqrt = (int) pi_sqrt;
  h_q.bglob = (int) bglob;
  for (int64_t i = 0; i < wave_len; i++) h_row[i] = i * cols;
  const int64_t last_len = (nseg - 1) % wave_len + 1;
  for (int pass = 0; pass < 2; pass++) {
    const int n = (int) (pass == 0 ? wave_len : last_len);
    CombineJob* J = h_jobs + pass * njobs;
    for (int sl = 0; sl * 32 < cols; sl++) J[sl] = CombineJob{0, 0, n, cols, sl};
    J[njobs - 1] = CombineJob{0, 0, n, cols, -1};
  }

  SweepArgs a;
  memset(&a, 0, sizeof(a));
  a.qs = d_q;
  a.nq = 1;
  a.rowoff = d_row;
  a.words = words;
  a.rec_cap = cap;
  a.primes = T.primes.as<uint32_t>();
  a.nprimes = T.nprimes;
  a.pitab = T.pitab.as<uint64_t>();
  a.pi_max = T.prime_limit;
  a.factor = T.factor_d.p;
  a.coprime = T.coprime.as<uint16_t>();
  a.group_max = sweep_group_max();
  a.cindex = T.cindex.as<int16_t>();
  a.finv = T.finv.as<uint64_t>();
  a.pmagic = T.pmagic.as<uint64_t>();
  a.cnt = d_cnt;
  a.smu = d_smu;
  a.segsum = d_segsum;
  a.counters = d_counters;
  uint64_t launches = 0;
  int waves = 0;
  unsigned long long ctr[5];
  try {
    // everything that must start at zero, then the call's inputs
    PCG_CUDA(cudaMemsetAsync(d_counters, 0, 4096, s));
    PCG_CUDA(cudaMemsetAsync(d_run, 0, (size_t) cols * 8, s));
    PCG_CUDA(cudaMemsetAsync(d_acc, 0, (size_t) cols * 16, s));
    PCG_CUDA(cudaMemcpyAsync(d_xp, h_xp, (size_t) cols * 24, cudaMemcpyHostToDevice, s));
    PCG_CUDA(cudaMemcpyAsync(d_seg, h_seg, (size_t) (nseg + 1) * 8, cudaMemcpyHostToDevice, s));
    PCG_CUDA(cudaMemcpyAsync(d_q, &h_q, sizeof(SweepQ), cudaMemcpyHostToDevice, s));
    PCG_CUDA(cudaMemcpyAsync(d_row, h_row, (size_t) wave_len * 8, cudaMemcpyHostToDevice, s));
    PCG_CUDA(cudaMemcpyAsync(d_jobs, h_jobs, jobs_bytes, cudaMemcpyHostToDevice, s));
    for (int64_t first = 0; first < nseg; first += wave_len) {
      int wl = (int) std::min<int64_t>(wave_len, nseg - first);
      a.wave_first = first;
      a.wave_len = wl;
      a.queue = d_queue + (waves % 16);
      PCG_CUDA(cudaMemsetAsync(d_cnt, 0, (size_t) wl * cols * 4, s));
      PCG_CUDA(cudaMemsetAsync(d_smu, 0, (size_t) wl * cols * 4, s));
      if (waves % 16 == 0 && waves > 0) PCG_CUDA(cudaMemsetAsync(d_queue, 0, 64, s));
      int g = (int) std::min<int64_t>(grid, wl);
      if (fbytes == 2) launch_sweep<uint16_t, 256>(a, g, smem, s);
      else launch_sweep<uint32_t, 256>(a, g, smem, s);
      PCG_CUDA(cudaGetLastError());
      k_combine<<<njobs, 32 * COMBINE_WARPS, 0, s>>>(d_cnt, d_smu, d_row, d_segsum,
                                                    d_jobs + (wl == wave_len ? 0 : njobs), d_run, d_acc, nullptr);
      PCG_CUDA(cudaGetLastError());
      launches += 2;
      waves++;
    }
    PCG_CUDA(cudaMemcpyAsync(h_acc, d_acc, (size_t) cols * 16, cudaMemcpyDeviceToHost, s));
    PCG_CUDA(cudaMemcpyAsync(ctr, d_counters, sizeof(ctr), cudaMemcpyDeviceToHost, s));
    PCG_CUDA(cudaStreamSynchronize(s));
  } catch (...) {
    // work already queued may still use the scratch: wait for it before the
    // mutex lets the next call clear and refill the array
    cudaStreamSynchronize(s);
    cudaGetLastError();
    throw;
  }
  i128 sum = 0;
  for (int b = 0; b < cols; b++) sum += h_acc[b];
  res.sum = sum;
  st.leaves = ctr[0];
  st.two_prime_leaves = ctr[1];
  st.levels = ctr[2];
  st.factor_entries = ctr[3];
  st.crossoff_multiples = ctr[4];
  st.segments = (uint64_t) nseg;
  st.kernel_launches = launches;
  st.sweep_launches = (uint64_t) waves;
  st.h2d_bytes = (uint64_t) cols * 24 + (uint64_t) (nseg + 1) * 8 + sizeof(SweepQ) + (uint64_t) wave_len * 8 +
                 jobs_bytes;
  st.d2h_bytes = (uint64_t) cols * 16 + sizeof(ctr);
  st.segment_words = words;
  st.ctas_per_sm = ctas;
  st.threads_per_cta = NT;
  st.total_ms = now_ms() - t_start;
  return res;
}

}  // namespace pcg
