// dev_common.cuh -- device helpers shared by the engine's CUDA sources:
// the 240-wheel bit layout (the reference's BitSieve240 layout,
// src/sieve/Sieve.hpp:8-12), PiTable lookups and exact integer helpers.
#pragma once

#include "pcg_internal.hpp"

namespace pcg {

// ---------------------------------------------------------------- constants
// # of wheel offsets {1,7,11,13,17,19,23,29} that are <= t, for t in [0, 30):
// nibble t of these two words.
#define PCG_CNT8_LO 0x4443322221111110ull
#define PCG_CNT8_HI 0x0087777776666554ull
// wheel offsets packed as bytes
#define PCG_WOFF 0x1D1713110D0B0701ull

static __device__ __forceinline__ uint32_t cnt8(uint32_t t)
{
  uint64_t v = t < 16 ? PCG_CNT8_LO : PCG_CNT8_HI;
  uint32_t sh = (t < 16 ? t : t - 16) * 4;
  return (uint32_t) (v >> sh) & 15u;
}

// the low nb bits set (nb in [0, 64]; the PTX shift clamps 64 to an empty result)
static __device__ __forceinline__ uint64_t low_bits(uint32_t nb)
{
  uint64_t m;
  asm("shr.b64 %0, %1, %2;" : "=l"(m) : "l"(~0ull), "r"(64u - nb));
  return m;
}

// bits of a 240-block for the numbers <= r (r in [0, 240))
static __device__ __forceinline__ uint64_t mask_le(uint32_t r)
{
  uint32_t byte = r / 30;
  uint32_t nb = byte * 8 + cnt8(r - byte * 30);
  return nb >= 64 ? ~0ull : ((1ull << nb) - 1);
}

static __device__ __forceinline__ uint32_t woff(uint32_t j) { return (uint32_t) (PCG_WOFF >> (8 * j)) & 0xFFu; }

// # numbers in [1, q] coprime to 30
static __device__ __forceinline__ uint64_t cnt_le(uint64_t q) { return 8 * (q / 30) + cnt8((uint32_t) (q % 30)); }

// bit of number offset `off` (coprime to 30) inside its word
static __device__ __forceinline__ uint32_t bit_of(uint32_t r) { return (r / 30) * 8 + cnt8(r % 30) - 1; }

// PiTable lookup: {count, bits} per 240 numbers (count includes 2, 3, 5)
static __device__ __forceinline__ int64_t dpi(const uint64_t* __restrict__ pt, uint64_t x)
{
  if (x < 6) return (0x322100u >> (4 * x)) & 15u;
  uint64_t i = x / 240;
  return (int64_t) (pt[2 * i] + __popcll(pt[2 * i + 1] & mask_le((uint32_t) (x - 240 * i))));
}

static __device__ __forceinline__ int64_t dmin(int64_t a, int64_t b) { return a < b ? a : b; }
static __device__ __forceinline__ int64_t dmax(int64_t a, int64_t b) { return a > b ? a : b; }

// exact floor(sqrt(x)) for x < 2^126
static __device__ int64_t disqrt(u128 x)
{
  if (x == 0) return 0;
  int64_t r = (int64_t) sqrt((double) x);
  while (r > 0 && (u128) r * (u128) r > x) r--;
  while ((u128) (r + 1) * (u128) (r + 1) <= x) r++;
  return r;
}

// min(floor(a / d), cap) for d >= 1, cap >= 0
static __device__ __forceinline__ int64_t divcap(u128 a, uint64_t d, int64_t cap)
{
  if ((u128) d * (u128) cap <= a) return cap;
  if ((uint64_t) (a >> 64) == 0) return (int64_t) ((uint64_t) a / d);
  return (int64_t) (a / d);
}

// a / d for a 128-bit a, 64-bit division when the high word is zero
static __device__ __forceinline__ u128 div128(u128 a, uint64_t d)
{
  if ((uint64_t) (a >> 64) == 0) return (u128) ((uint64_t) a / d);
  return a / d;
}


// floor(n / q) from m = floor((2^64 - 1) / q), q >= 1: the high product is
// floor(n / q) or one less
static __device__ __forceinline__ uint64_t div_magic(uint64_t n, uint64_t q, uint64_t m)
{
  uint64_t t = __umul64hi(n, m);
  if (n - t * q >= q) t++;
  return t;
}

}  // namespace pcg
