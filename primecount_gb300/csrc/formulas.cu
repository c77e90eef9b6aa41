// formulas.cu -- pi(x) by Gourdon's formula on the GPU, and phi(x, a).
//
// pi(x) = A - B + C + D + Phi0 + Sigma (reference: src/gourdon/pi_gourdon.cpp:
// 37-163).  D comes from the hard-leaf sweep (sweep.cu); the easy terms are
// evaluated here, each as the sum the reference's code computes, restated
// over the whole interval instead of the reference's segments:
//   A, C1, C2   src/gourdon/AC.cpp:40-300 (sums of pi(x / (p q)) and
//               pi(x / (p q r)) over primes; the PiTable up to sqrt(x) lives
//               in HBM and every (p, q) pair is one thread)
//   B           src/gourdon/B.cpp:38-131 (sum of pi(x / p), y < p <= sqrt(x):
//               a segmented prime sieve of [sqrt(x), x / y) whose segments
//               are joined by the same offset scan as the hard leaves)
//   Phi0        src/gourdon/Phi0.cpp:38-96 (mu(n) phi(x / n, k) over the
//               FactorTableD entries)
//   Sigma       src/gourdon/Sigma.cpp:25-140 (closed forms, on the host)
// pi(x) for x <= 1e10 is a direct sieve count (the reference routes small x
// to other algorithms, src/api.cpp:75-91).
#include <cstdio>
#include <cstring>
#include <chrono>
#include <algorithm>
#include <vector>

#include <thread>
#include <exception>
#include <mutex>
#include <cstdlib>
#include "pcg_internal.hpp"
#include "dev_common.cuh"

namespace pcg {

static double fnow_ms()
{
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

// ---------------------------------------------------------------- i128 block sums
template <int NT>
__device__ __forceinline__ void block_sum_i128(i128 v, i128* out)
{
  __shared__ long long lo_s[NT], hi_s[NT];
  // split into 2^62-bounded halves so that a block of partial sums cannot overflow
  lo_s[threadIdx.x] = (long long) (v & (i128) 0x3FFFFFFFFFFFFFFFll);
  hi_s[threadIdx.x] = (long long) (v >> 62);
  __syncthreads();
  if (threadIdx.x == 0) {
    i128 lo = 0, hi = 0;
    for (int i = 0; i < NT; i++) { lo += lo_s[i]; hi += hi_s[i]; }
    *out += lo + hi * ((i128) 1 << 62);
  }
  __syncthreads();
}

static i128 sum_partials(const DevBuf& buf, int n, cudaStream_t s)
{
  std::vector<i128> h((size_t) n);
  PCG_CUDA(cudaMemcpyAsync(h.data(), buf.p, (size_t) n * 16, cudaMemcpyDeviceToHost, s));
  PCG_CUDA(cudaStreamSynchronize(s));
  i128 t = 0;
  for (int i = 0; i < n; i++) t += h[(size_t) i];
  return t;
}

// ---------------------------------------------------------------- phi(v, k), k <= 8
// phi(v, k) = (v / P) * phi(P) + phi(v mod P, k), P = p_1 ... p_k
// (the identity of the reference's PhiTiny, src/PhiTiny.hpp:2-12); phi(r, k)
// for r < P from a bitmap of the numbers coprime to p_1..p_k.
__global__ void k_phi_bits(uint64_t* __restrict__ bits, uint32_t* __restrict__ pc, int64_t nwords, uint64_t P, int k)
{
  int64_t w = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nwords) return;
  const uint32_t pr[8] = {2, 3, 5, 7, 11, 13, 17, 19};
  uint64_t v = 0;
  for (int j = 0; j < 64; j++) {
    uint64_t t = 64 * (uint64_t) w + j;
    if (t >= P) break;
    bool ok = true;
    for (int i = 0; i < k; i++) ok = ok && (t % pr[i] != 0);
    if (ok) v |= 1ull << j;
  }
  bits[w] = v;
  pc[w] = __popcll(v);
}

struct PhiTab {
  const uint64_t* bits;
  const uint64_t* pref;
  uint64_t P, tot;
  int k;
};

__device__ __forceinline__ i128 dphi_tiny(u128 v, const PhiTab& T)
{
  if (T.k == 0) return (i128) v;
  const u128 q = div128(v, T.P);
  const uint64_t r = (uint64_t) (v - q * T.P);
  const uint64_t w = r >> 6;
  const uint64_t c = T.pref[w] + __popcll(T.bits[w] & ((2ull << (r & 63)) - 1));
  return (i128) q * (i128) T.tot + (i128) c;
}

static void ensure_phi_tiny(Ctx& c, int k, cudaStream_t s)
{
  Tables& t = c.tab;
  if (t.phik == k) return;
  static const uint64_t pr[8] = {2, 3, 5, 7, 11, 13, 17, 19};
  uint64_t P = 1, tot = 1;
  for (int i = 0; i < k; i++) { P *= pr[i]; tot *= pr[i] - 1; }
  int64_t nwords = (int64_t) ((P + 63) / 64);
  t.phi_bits.alloc((size_t) nwords * 8);
  t.phi_pref.alloc((size_t) nwords * 8);
  DevBuf pc;
  pc.alloc((size_t) nwords * 4);
  k_phi_bits<<<(unsigned) ((nwords + 255) / 256), 256, 0, s>>>(t.phi_bits.as<uint64_t>(), pc.as<uint32_t>(), nwords, P, k);
  PCG_CUDA(cudaGetLastError());
  exclusive_scan_u32(pc.as<uint32_t>(), nwords, t.phi_pref.as<uint64_t>(), s);
  t.phik = k;
  t.phi_P = P;
  t.phi_tot = tot;
}

static PhiTab phi_tab(const Ctx& c)
{
  PhiTab T;
  T.bits = c.tab.phi_bits.as<uint64_t>();
  T.pref = c.tab.phi_pref.as<uint64_t>();
  T.P = c.tab.phi_P;
  T.tot = c.tab.phi_tot;
  T.k = c.tab.phik;
  return T;
}

// ---------------------------------------------------------------- Phi0
// Phi0 = sum over n = 1 and the square-free n <= z whose prime factors lie
// in (p_k, y] of mu(n) phi(x / n, k) (Phi0.cpp:38-96).  Those n are the
// FactorTableD entries above 2k + 1 (1 -> T_MAX - 1, composites 2 pi(lpf) +
// [mu = -1]) except the primes <= p_k, which the table marks T_MAX like every
// prime <= y.
template <typename FT>
__global__ void __launch_bounds__(256) k_phi0(uint64_t x_lo, uint64_t x_hi, const FT* __restrict__ factor,
                                              int64_t size, uint32_t thr, uint64_t pk, PhiTab T,
                                              const uint16_t* __restrict__ coprime, i128* __restrict__ partial)
{
  const u128 x = ((u128) x_hi << 64) | x_lo;
  i128 acc = 0;
  for (int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x; i < size; i += (int64_t) gridDim.x * blockDim.x) {
    const uint32_t f = (uint32_t) factor[i];
    if (f > thr) {
      const uint64_t n = 2310 * (uint64_t) (i / 480) + coprime[i % 480];
      if (n > 1 && n <= pk) continue;
      const i128 t = dphi_tiny(div128(x, n), T);
      acc += (f & 1) ? -t : t;
    }
  }
  block_sum_i128<256>(acc, &partial[blockIdx.x]);
}

// ---------------------------------------------------------------- A and C
// One outer item: a prime p_b (or p_b q for the C1 products) and a range
// (i_lo, i_hi] of prime indices q = primes[i]; the term of q is
//   mode 0 (A):  w * pi(xp / q), w = 1 if q <= xp / y else 2 (AC.cpp:40-83);
//                cap holds the index pi(xp / y)
//   mode 1 (C):  pi(xp / q) - b + 2                         (AC.cpp:112-129, 186-300)
//   mode 2 (C1 products): -(pi(xp / q) - b + 2)              (AC.cpp:131-177)
//   mode 3 (P3 of phi):   pi(xp / q) - i + 1, i = index of q
//   modes 5, 6: modes 1, 2 of an outer whose xp / q can fall below 6
struct PairOuter {
  uint64_t xp_lo, xp_hi;
  uint64_t cap;
  int64_t i_lo, i_hi;
  int32_t b;
  int32_t mode;
};

// pi(n) for n >= 6 from the PiTable {count, bits} per 240 numbers (the
// count of a word includes 2, 3 and 5); s_mask[r] = # wheel residues <= r.
// Below 2^36 the word index is a 32-bit division: n / 240 = (n / 16) / 15.
static __device__ __forceinline__ long long pi_pt(const ulonglong2* __restrict__ pt, const uint8_t* s_mask,
                                                  uint64_t n)
{
  uint64_t w;
  uint32_t r;
  if ((n >> 36) == 0) {
    const uint32_t w32 = (uint32_t) (n >> 4) / 15u;
    w = w32;
    r = (uint32_t) n - 240u * w32;                   // exact modulo 2^32
  } else {
    w = n / 240;
    r = (uint32_t) (n - 240 * w);
  }
  const ulonglong2 e = pt[w];
  return (long long) e.x + __popcll(e.y & low_bits(s_mask[r]));
}

// pi(n) for n < 2^36: the word index by a 32-bit division
static __device__ __forceinline__ long long pi_pt36(const ulonglong2* __restrict__ pt, const uint8_t* s_mask,
                                                    uint64_t n)
{
  const uint32_t w32 = (uint32_t) (n >> 4) / 15u;
  const uint32_t r = (uint32_t) n - 240u * w32;
  const ulonglong2 e = pt[w32];
  return (long long) e.x + __popcll(e.y & low_bits(s_mask[r]));
}

// pi(xp / q) for the prime q = primes[i] with m = floor((2^64 - 1) / q), by
// shape of the outer:
//   SHAPE 0: xp < 2^64, q < 2^31 and n < 2^36 (tables below those bounds):
//            t = floor(xp * m / 2^64) is n or n - 1, and xp - t q < 2 q < 2^32,
//            so its low 32 bits decide the correction;
//   SHAPE 1: xp < 2^64 (64-bit remainder);  SHAPE 2: xp >= 2^64.
// LOWN: the outer can reach n < 6, where the PiTable's first word (which
// counts 2, 3 and 5 in every n) does not hold
template <int SHAPE, bool LOWN>
__device__ __forceinline__ long long pair_pi(const PairOuter& O, uint32_t q, uint64_t m,
                                            const ulonglong2* __restrict__ pt, const uint8_t* s_mask)
{
  uint64_t n;
  if (SHAPE == 0) {
    n = __umul64hi(O.xp_lo, m);
    n += ((uint32_t) O.xp_lo - (uint32_t) n * q) >= q;
  } else if (SHAPE == 1) {
    n = div_magic(O.xp_lo, q, m);
  } else {
    n = (uint64_t) ((((u128) O.xp_hi << 64) | O.xp_lo) / q);
  }
  if (LOWN && n < 6) return (long long) ((0x322100u >> (4 * n)) & 15u);
  return SHAPE == 0 ? pi_pt36(pt, s_mask, n) : pi_pt(pt, s_mask, n);
}

// sum of pi(xp / q) over this thread's prime indices i in (lo, hi], i = lo +
// 1 + threadIdx.x + 256 t (indices < 2^32), four terms in flight
template <int SHAPE, bool LOWN>
__device__ __forceinline__ long long pi_sum(const PairOuter& O, uint32_t lo, uint32_t hi,
                                            const uint32_t* __restrict__ primes, const uint64_t* __restrict__ magic,
                                            const ulonglong2* __restrict__ pt, const uint8_t* s_mask)
{
  long long s = 0;
  uint32_t i = lo + 1 + threadIdx.x;
  for (; i + 3 * 256 <= hi; i += 4 * 256) {
    uint32_t q[4];
    uint64_t m[4];
#pragma unroll
    for (int u = 0; u < 4; u++) { q[u] = primes[i + 256 * u]; m[u] = magic[i + 256 * u]; }
#pragma unroll
    for (int u = 0; u < 4; u++) s += pair_pi<SHAPE, LOWN>(O, q[u], m[u], pt, s_mask);
  }
  for (; i <= hi; i += 256) s += pair_pi<SHAPE, LOWN>(O, primes[i], magic[i], pt, s_mask);
  return s;
}

// the terms of one outer for this thread; the per-term constants come out of
// the sums: with c terms of indices i_1..i_c,
//   mode 0: sum over i <= icap of pi + 2 * sum over i > icap  (icap = pi(cap))
//   mode 1: sum pi - c (b - 2);   mode 2: -(sum pi - c (b - 2));
//   mode 3: sum pi - sum (i - 1)
template <int MODE, int SHAPE, bool LOWN>
__device__ __forceinline__ long long pair_terms(const PairOuter& O, const uint32_t* __restrict__ primes,
                                                const uint64_t* __restrict__ magic,
                                                const ulonglong2* __restrict__ pt, const uint8_t* s_mask)
{
  const uint32_t lo = (uint32_t) O.i_lo, hi = (uint32_t) O.i_hi;
  if (MODE == 0) {
    const uint32_t ic = (uint32_t) min((uint64_t) hi, max((uint64_t) lo, O.cap));
    return pi_sum<SHAPE, false>(O, lo, ic, primes, magic, pt, s_mask) +
           2 * pi_sum<SHAPE, false>(O, ic, hi, primes, magic, pt, s_mask);
  }
  const long long s = pi_sum<SHAPE, LOWN>(O, lo, hi, primes, magic, pt, s_mask);
  const uint32_t first = lo + 1 + threadIdx.x;
  const long long c = first <= hi ? (long long) ((hi - first) / 256 + 1) : 0;
  if (MODE == 1) return s - c * ((long long) O.b - 2);
  if (MODE == 2) return -(s - c * ((long long) O.b - 2));
  return s - c * ((long long) first - 1) - 256ll * (c * (c - 1) / 2);
}

template <int MODE, bool SMALL, bool LOWN>
__device__ __forceinline__ long long outer_terms(const PairOuter& O, const uint32_t* __restrict__ primes,
                                                 const uint64_t* __restrict__ magic,
                                                 const ulonglong2* __restrict__ pt, const uint8_t* s_mask)
{
  if (O.xp_hi != 0) return pair_terms<MODE, 2, LOWN>(O, primes, magic, pt, s_mask);
  if (SMALL) return pair_terms<MODE, 0, LOWN>(O, primes, magic, pt, s_mask);
  return pair_terms<MODE, 1, LOWN>(O, primes, magic, pt, s_mask);
}

// outers of more than PAIR_SPLIT terms are cut into pieces of PAIR_SPLIT so
// that the pieces spread evenly over the blocks
#define PAIR_SPLIT 16384
__global__ void k_pair_pieces(const PairOuter* __restrict__ outs, int64_t n, uint32_t* __restrict__ pieces)
{
  const int64_t j = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (j > n) return;
  const int64_t c = j < n ? dmax(0, outs[j].i_hi - outs[j].i_lo) : 0;
  pieces[j] = (uint32_t) ((c + PAIR_SPLIT - 1) / PAIR_SPLIT);
}

__global__ void k_pair_split(const PairOuter* __restrict__ outs, int64_t n, const uint64_t* __restrict__ first,
                             PairOuter* __restrict__ split)
{
  const int64_t j = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const PairOuter O = outs[j];
  const int64_t np = (int64_t) (first[j + 1] - first[j]);
  for (int64_t t = 0; t < np; t++) {
    PairOuter P = O;
    P.i_lo = O.i_lo + t * PAIR_SPLIT;
    P.i_hi = dmin(O.i_hi, P.i_lo + PAIR_SPLIT);
    split[first[j] + t] = P;
  }
}

// SMALL: every prime of the table is below 2^31 and the PiTable ends below 2^36
template <bool SMALL>
__global__ void __launch_bounds__(256) k_pairs(const PairOuter* __restrict__ outs, int64_t n_outer,
                                               const uint32_t* __restrict__ primes,
                                               const uint64_t* __restrict__ magic,
                                               const uint64_t* __restrict__ pibig, i128* __restrict__ partial)
{
  __shared__ uint8_t s_mask[240];       // # wheel residues <= r
  for (int r = threadIdx.x; r < 240; r += blockDim.x) s_mask[r] = (uint8_t) ((r / 30) * 8 + cnt8((uint32_t) (r % 30)));
  __syncthreads();
  const ulonglong2* __restrict__ pt = (const ulonglong2*) pibig;
  i128 acc = 0;
  for (int64_t o = blockIdx.x; o < n_outer; o += gridDim.x) {
    const PairOuter O = outs[o];
    long long s;
    if (O.mode == 0) s = outer_terms<0, SMALL, false>(O, primes, magic, pt, s_mask);
    else if (O.mode == 1) s = outer_terms<1, SMALL, false>(O, primes, magic, pt, s_mask);
    else if (O.mode == 2) s = outer_terms<2, SMALL, false>(O, primes, magic, pt, s_mask);
    else if (O.mode == 3) s = outer_terms<3, SMALL, false>(O, primes, magic, pt, s_mask);
    else if (O.mode == 5) s = outer_terms<1, SMALL, true>(O, primes, magic, pt, s_mask);
    else s = outer_terms<2, SMALL, true>(O, primes, magic, pt, s_mask);
    acc += s;
  }
  block_sum_i128<256>(acc, &partial[blockIdx.x]);
}

// sum of the terms of nout outers: big outers cut into pieces, then one
// block per piece
static i128 run_pairs(Ctx& c, const PairOuter* outs, int64_t nout, cudaStream_t s, uint64_t* launches)
{
  if (nout <= 0) return 0;
  DevBuf& pieces = c.tmp[T_PR_PIECES];
  DevBuf& first = c.tmp[T_PR_FIRST];
  pieces.alloc((size_t) (nout + 1) * 4);
  first.alloc((size_t) (nout + 1) * 8);
  k_pair_pieces<<<(unsigned) ((nout + 256) / 256), 256, 0, s>>>(outs, nout, pieces.as<uint32_t>());
  PCG_CUDA(cudaGetLastError());
  exclusive_scan_u32(pieces.as<uint32_t>(), nout + 1, first.as<uint64_t>(), s, &c.tmp[T_PR_SUMS]);
  uint64_t np = 0;
  PCG_CUDA(cudaMemcpyAsync(&np, first.as<uint64_t>() + nout, 8, cudaMemcpyDeviceToHost, s));
  PCG_CUDA(cudaStreamSynchronize(s));
  if (np == 0) return 0;
  DevBuf& split = c.tmp[T_PR_SPLIT];
  split.alloc((size_t) np * sizeof(PairOuter));
  k_pair_split<<<(unsigned) ((nout + 127) / 128), 128, 0, s>>>(outs, nout, first.as<uint64_t>(),
                                                               split.as<PairOuter>());
  PCG_CUDA(cudaGetLastError());
  const int grid = (int) std::min<uint64_t>(np, (uint64_t) c.num_sms * 8);
  DevBuf& part = c.tmp[T_PR_PART];
  part.alloc((size_t) grid * 16);
  PCG_CUDA(cudaMemsetAsync(part.p, 0, (size_t) grid * 16, s));
  const bool small = c.tab.prime_limit < (1ll << 31) && c.tab.pibig_limit + 240 < (1ll << 36);
  if (small)
    k_pairs<true><<<grid, 256, 0, s>>>(split.as<PairOuter>(), (int64_t) np, c.tab.primes.as<uint32_t>(),
                                       c.tab.pmagic.as<uint64_t>(), c.tab.pibig.as<uint64_t>(), part.as<i128>());
  else
    k_pairs<false><<<grid, 256, 0, s>>>(split.as<PairOuter>(), (int64_t) np, c.tab.primes.as<uint32_t>(),
                                        c.tab.pmagic.as<uint64_t>(), c.tab.pibig.as<uint64_t>(), part.as<i128>());
  PCG_CUDA(cudaGetLastError());
  if (launches) *launches += 6;
  return sum_partials(part, grid, s);
}

struct AcParams {
  uint64_t x_lo, x_hi;
  int64_t y, z, k, x_star, x13, sqrtx;
  int64_t bA0, bA1;      // A:  b in (bA0, bA1]
  int64_t bC10, bC11;    // C1: b in (bC10, bC11]
  int64_t bC20, bC21;    // C2: b in (bC20, bC21]
  const uint32_t* primes;
  const uint64_t* pismall;  // PiTable up to y
  const uint64_t* pibig;    // PiTable up to sqrt(x)
};

// A outers: b in (pi(x*), pi(x^(1/3))], q in (max(p, xp / sqrt(x)), sqrt(xp)]
__global__ void k_outer_A(AcParams P, PairOuter* __restrict__ outs)
{
  const int64_t j = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t b = P.bA0 + 1 + j;
  if (b > P.bA1) return;
  const u128 x = ((u128) P.x_hi << 64) | P.x_lo;
  const uint64_t p = P.primes[b];
  const u128 xp = div128(x, p);
  PairOuter O;
  O.xp_lo = (uint64_t) xp;
  O.xp_hi = (uint64_t) (xp >> 64);
  O.b = (int32_t) b;
  O.mode = 0;
  const int64_t sq = disqrt(xp);
  // xp / y <= sqrt(xp) since xp <= x / x* <= y^2
  O.cap = (uint64_t) dpi(P.pibig, (uint64_t) dmin(sq, (int64_t) (xp / (u128) P.y)));
  const int64_t lowq = (int64_t) (xp / (u128) P.sqrtx);
  O.i_hi = dpi(P.pibig, (uint64_t) sq);
  O.i_lo = dmax(b, dpi(P.pibig, (uint64_t) lowq));
  if (O.i_hi < O.i_lo) O.i_hi = O.i_lo;
  outs[j] = O;
}

// the m-range of C1 for p_b: (max(x / p^3, z / p), min(x / p, z)]
__device__ __forceinline__ void c1_range(const AcParams& P, int64_t b, u128& xp, int64_t& min_m, int64_t& max_m)
{
  const u128 x = ((u128) P.x_hi << 64) | P.x_lo;
  const uint64_t p = P.primes[b];
  xp = div128(x, p);
  max_m = (xp < (u128) P.z) ? (int64_t) xp : P.z;
  const u128 xpp = xp / ((u128) p * p);
  min_m = dmax(xpp > (u128) INT64_MAX ? INT64_MAX : (int64_t) xpp, P.z / (int64_t) p);
}

// C1 outers with m prime: primes m in (min_m, min(y, max_m)]
__global__ void k_outer_C1(AcParams P, PairOuter* __restrict__ outs)
{
  const int64_t j = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t b = P.bC10 + 1 + j;
  if (b > P.bC11) return;
  u128 xp;
  int64_t min_m, max_m;
  c1_range(P, b, xp, min_m, max_m);
  PairOuter O;
  O.xp_lo = (uint64_t) xp;
  O.xp_hi = (uint64_t) (xp >> 64);
  O.cap = 0;
  O.b = (int32_t) b;
  O.mode = 1;
  O.i_lo = O.i_hi = 0;
  const int64_t top = dmin(P.y, max_m);
  if (min_m < max_m && min_m < top) {
    O.i_lo = dpi(P.pismall, (uint64_t) min_m);
    O.i_hi = dpi(P.pismall, (uint64_t) top);
    if (O.i_hi > O.i_lo && xp / P.primes[O.i_hi] < 6) O.mode = 5;
  }
  outs[j] = O;
}

// C1 products m = q r: number of q per b, then one outer per (b, q)
__global__ void k_c1_qcount(AcParams P, int64_t* __restrict__ qlo, int64_t* __restrict__ qcnt)
{
  const int64_t j = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t b = P.bC10 + 1 + j;
  if (b > P.bC11) return;
  u128 xp;
  int64_t min_m, max_m;
  c1_range(P, b, xp, min_m, max_m);
  const int64_t p = P.primes[b];
  int64_t lo = 0, cnt = 0;
  if (min_m < max_m) {
    const int64_t max_q = dmin(P.y, disqrt((u128) max_m));
    const int64_t min_q = dmax(p, min_m / P.y);
    if (min_q < max_q) {
      lo = dpi(P.pismall, (uint64_t) min_q);
      cnt = dpi(P.pismall, (uint64_t) max_q) - lo;
    }
  }
  qlo[j] = lo;
  qcnt[j] = cnt;
}

__global__ void k_c1_expand(AcParams P, const int64_t* __restrict__ qlo, const int64_t* __restrict__ qcnt,
                            const int64_t* __restrict__ qoff, PairOuter* __restrict__ outs)
{
  const int64_t j = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t b = P.bC10 + 1 + j;
  if (b > P.bC11) return;
  u128 xp;
  int64_t min_m, max_m;
  c1_range(P, b, xp, min_m, max_m);
  for (int64_t t = 0; t < qcnt[j]; t++) {
    const int64_t qi = qlo[j] + 1 + t;
    const uint64_t q = P.primes[qi];
    const int64_t min_r = dmax((int64_t) q, min_m / (int64_t) q);
    const int64_t max_r = dmin(P.y, max_m / (int64_t) q);
    PairOuter O;
    const u128 xpq = div128(xp, q);
    O.xp_lo = (uint64_t) xpq;
    O.xp_hi = (uint64_t) (xpq >> 64);
    O.cap = 0;
    O.b = (int32_t) b;
    O.mode = 2;
    O.i_lo = O.i_hi = 0;
    if (min_r < max_r) {
      O.i_lo = dpi(P.pismall, (uint64_t) min_r);
      O.i_hi = dpi(P.pismall, (uint64_t) max_r);
      if (O.i_hi > O.i_lo && xpq / P.primes[O.i_hi] < 6) O.mode = 6;
    }
    outs[qoff[j] + t] = O;
  }
}

// C2 outers: primes q in (max(x / p^3, p, xp / sqrt(x)), min(x / p^2, y)]
__global__ void k_outer_C2(AcParams P, PairOuter* __restrict__ outs)
{
  const int64_t j = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t b = P.bC20 + 1 + j;
  if (b > P.bC21) return;
  const u128 x = ((u128) P.x_hi << 64) | P.x_lo;
  const uint64_t p = P.primes[b];
  const u128 xp = div128(x, p);
  const u128 xpp = xp / (u128) p;
  const int64_t max_m = (xpp < (u128) P.y) ? (int64_t) xpp : P.y;
  const u128 x3 = xp / ((u128) p * p);
  int64_t min_m = x3 > (u128) INT64_MAX ? INT64_MAX : (int64_t) x3;
  min_m = dmax(min_m, (int64_t) p);
  min_m = dmax(min_m, (int64_t) (xp / (u128) P.sqrtx));
  PairOuter O;
  O.xp_lo = (uint64_t) xp;
  O.xp_hi = (uint64_t) (xp >> 64);
  O.cap = 0;
  O.b = (int32_t) b;
  O.mode = 1;
  O.i_lo = O.i_hi = 0;
  if (min_m < max_m) {
    O.i_lo = dpi(P.pismall, (uint64_t) min_m);
    O.i_hi = dpi(P.pismall, (uint64_t) max_m);
    if (O.i_hi > O.i_lo && xp / P.primes[O.i_hi] < 6) O.mode = 5;
  }
  outs[j] = O;
}

// S2_easy outers (Deleglise-Rivat, S2_easy.cpp:60-140): b in (b0, b1] =
// (max(c, pi(sqrt y)), pi(x^(1/3))], the primes q = primes[i] with i in
// (pi(in_between(p, z / p, y)), pi(min(x / p^2, y))]; term pi(x / (p q)) - b + 2.
// The reference's clustered leaves (equal successive terms) are the same terms.
__global__ void k_outer_S2e(uint64_t x_lo, uint64_t x_hi, int64_t y, int64_t z, int64_t b0, int64_t b1,
                            const uint32_t* __restrict__ primes, const uint64_t* __restrict__ pismall,
                            PairOuter* __restrict__ outs)
{
  const int64_t j = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t b = b0 + 1 + j;
  if (b > b1) return;
  const u128 x = ((u128) x_hi << 64) | x_lo;
  const uint64_t p = primes[b];
  const u128 xp = div128(x, p);
  const u128 xpp = xp / p;
  const int64_t min_trivial = xpp < (u128) y ? (int64_t) xpp : y;
  int64_t min_sparse = z / (int64_t) p;
  if (min_sparse < (int64_t) p || y < (int64_t) p) min_sparse = (int64_t) p;
  else if (min_sparse > y) min_sparse = y;
  PairOuter O;
  O.xp_lo = (uint64_t) xp;
  O.xp_hi = (uint64_t) (xp >> 64);
  O.cap = 0;
  O.b = (int32_t) b;
  O.mode = 1;
  O.i_hi = dpi(pismall, (uint64_t) min_trivial);
  O.i_lo = dpi(pismall, (uint64_t) min_sparse);
  if (O.i_hi < O.i_lo) O.i_hi = O.i_lo;
  outs[j] = O;
}

// ---------------------------------------------------------------- prime sieve segments (B, small pi)
// Each CTA sieves a segment [lo, hi) (lo a multiple of 240) of the numbers
// coprime to 30, leaving the primes.  Mode count: seg_c[s] = # primes >= 7 in
// the segment.  Mode B additionally answers the queries x / p for the primes p
// in (max(qlo, x / hi), min(qhi, x / lo)] (enumerated from the PiTable bits up
// to sqrt(x)): seg_m[s] = # of them, seg_l[s] = sum of # primes in [lo, x / p].
//
// Cross-off in three tiers:
//  * 7..61: each word starts as the AND of the primes' wheel patterns (the
//    multiples of p repeat every p words of 240 numbers);
//  * 67 <= p < mid_limit: a warp per prime, lane l owning the multiples p q
//    with q = c_l (mod 120), c_l the l-th residue coprime to 30.  Those
//    multiples are 120 p apart, i.e. exactly p 32-bit words (120 numbers) with
//    the same bit, so the inner loop is one shared atomicAnd and one add;
//  * larger p: a lane per prime stepping q along the 30-wheel.
// ceil(lo / p) comes from a precomputed reciprocal floor((2^64 - 1) / p) and
// one correction step.
#define PS_NT 512
#define PS_SMALL 15
#define PS_PAT 491                // 7 + 11 + ... + 61 pattern words
#define PS_GAPS 0x26424246u       // gaps between consecutive wheel offsets, a nibble each
struct PsArgs {
  uint64_t x_lo, x_hi;
  int64_t lo0;           // first segment start (multiple of 240)
  int64_t end;           // sieve [lo0, end)
  int64_t seg;           // numbers per segment = words * 240
  int64_t nseg;
  int64_t qlo, qhi;      // B queries: primes p in (qlo, qhi]
  int32_t mode;          // 0 count, 1 B
  int32_t words;         // 64-bit words per segment (a multiple of 4096, at most 16384)
  int32_t nbase;         // primes >= 67 up to sqrt(end)
  int32_t nmid;          // base[0, nmid) crossed off a warp per prime
  const uint32_t* base;
  const uint64_t* magic; // floor((2^64 - 1) / base[k])
  const uint64_t* pibig; // PiTable bits for the B queries
  int64_t* seg_c;
  int64_t* seg_m;
  int64_t* seg_l;
  int* queue;
};

static __device__ __forceinline__ uint64_t ceil_div_magic(uint64_t n, uint32_t p, uint64_t m)
{
  uint64_t q = __umul64hi(n, m);     // floor(n / p) or one less
  if (n - q * p >= p) q++;
  return q + (q * p != n);
}

__constant__ uint32_t c_ps_small[PS_SMALL] = {7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59, 61};

__global__ void __launch_bounds__(PS_NT, 2) k_psieve(const PsArgs A)
{
  constexpr uint32_t SP[PS_SMALL] = {7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59, 61};
  extern __shared__ __align__(16) unsigned char psm[];
  const int words = A.words;
  uint64_t* bits = (uint64_t*) psm;
  uint32_t* bits32 = (uint32_t*) psm;
  uint32_t* pref = (uint32_t*) (bits + words);           // words / 8 chunk prefixes
  uint64_t* pat = (uint64_t*) (pref + words / 8);        // wheel patterns of 7..61
  __shared__ uint8_t s_bit[120];                         // bit of residue r in a 32-bit word
  __shared__ int s_s;
  __shared__ uint32_t wt[32];
  __shared__ long long red[3][32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nch = words / 8;
  const u128 x = ((u128) A.x_hi << 64) | A.x_lo;
  for (int i = tid; i < 120; i += PS_NT) s_bit[i] = (uint8_t) bit_of((uint32_t) i);
  for (int i = tid; i < PS_PAT; i += PS_NT) {
    int k = 0, b0 = 0;
    while (i >= b0 + (int) c_ps_small[k]) { b0 += c_ps_small[k]; k++; }
    const uint32_t p = c_ps_small[k], r = (uint32_t) (i - b0);
    uint64_t v = 0;
    for (int b = 0; b < 64; b++) {
      const uint32_t n = 240u * r + 30u * (b >> 3) + woff(b & 7);
      if (n % p) v |= 1ull << b;
    }
    pat[i] = v;
  }
  uint64_t small_mask = 0;                               // 7..61 in word 0
#pragma unroll
  for (int i = 0; i < PS_SMALL; i++) small_mask |= 1ull << bit_of(SP[i]);
  const uint32_t lane_res = 30u * (uint32_t) (lane >> 3) + woff((uint32_t) lane & 7);
  for (;;) {
    __syncthreads();
    if (tid == 0) s_s = atomicAdd(A.queue, 1);
    __syncthreads();
    const int64_t s = s_s;
    if (s >= A.nseg) break;
    const uint64_t lo = (uint64_t) (A.lo0 + s * A.seg);
    const uint64_t hi = (uint64_t) dmin((int64_t) lo + A.seg, A.end);
    const uint32_t span = (uint32_t) (hi - lo);
    const int wused = (int) ((span + 239) / 240);
    const uint32_t nw32 = (span + 119) / 120;
    {
      // pattern phases of this thread's first word, advanced by PS_NT words per step
      const uint64_t g0 = lo / 240 + (uint64_t) tid;
      uint32_t ph[PS_SMALL];
#pragma unroll
      for (int i = 0; i < PS_SMALL; i++) ph[i] = (uint32_t) (g0 % SP[i]);
      for (int w = tid; w < words; w += PS_NT) {
        uint64_t v = 0;
        if (w < wused) {
          v = ~0ull;
          uint32_t po = 0;
#pragma unroll
          for (int i = 0; i < PS_SMALL; i++) {
            v &= pat[po + ph[i]];
            po += SP[i];
          }
          if (lo == 0 && w == 0) v = (v | small_mask) & ~1ull;   // 7..61 are prime, 1 is not
          if (w == wused - 1) v &= mask_le((span - 1) % 240);
        }
        bits[w] = v;
#pragma unroll
        for (int i = 0; i < PS_SMALL; i++) {
          ph[i] += PS_NT % SP[i];
          if (ph[i] >= SP[i]) ph[i] -= SP[i];
        }
      }
    }
    __syncthreads();
    // medium primes: a warp per prime, a residue class of q mod 120 per lane
    for (int k = warp; k < A.nmid; k += PS_NT / 32) {
      const uint32_t p = A.base[k];
      if ((uint64_t) p * p >= hi) break;
      uint64_t qmin = ceil_div_magic(lo, p, A.magic[k]);
      if (qmin < p) qmin = p;
      const uint32_t qm = (uint32_t) (qmin % 120);
      const uint64_t q = qmin + (lane_res >= qm ? lane_res - qm : lane_res + 120 - qm);
      const uint64_t pq = (uint64_t) p * q;
      if (pq < hi) {
        const uint32_t off = (uint32_t) (pq - lo);
        uint32_t w = off / 120;
        const uint32_t msk = ~(1u << s_bit[off - 120 * w]);
        for (; w < nw32; w += p) atomicAnd(&bits32[w], msk);
      }
    }
    // large primes: a lane per prime along the 30-wheel
    for (int k = A.nmid + tid; k < A.nbase; k += PS_NT) {
      const uint32_t p = A.base[k];
      if ((uint64_t) p * p >= hi) break;
      uint64_t qmin = ceil_div_magic(lo, p, A.magic[k]);
      if (qmin < p) qmin = p;
      const uint64_t j = cnt_le(qmin - 1);              // wheel index of the first q >= qmin
      const uint64_t q = 30 * (j >> 3) + woff((uint32_t) (j & 7));
      const uint64_t pq = (uint64_t) p * q;
      if (pq >= hi) continue;
      uint32_t off = (uint32_t) (pq - lo);
      uint32_t jj = (uint32_t) (j & 7);
      while (off < span) {
        const uint32_t w = off / 120;
        atomicAnd(&bits32[w], ~(1u << s_bit[off - 120 * w]));
        off += p * ((PS_GAPS >> (4 * jj)) & 15u);
        jj = (jj + 1) & 7;
      }
    }
    __syncthreads();
    // chunk prefix (8 words per chunk; nch / PS_NT chunks per thread)
    {
      const int cpt = nch / PS_NT;
      const int base = tid * cpt;
      uint32_t loc[4];
      uint32_t sum = 0;
#pragma unroll
      for (int c = 0; c < 4; c++) {
        uint32_t t = 0;
        if (c < cpt)
          for (int i = 0; i < 8; i++) t += __popcll(bits[8 * (base + c) + i]);
        loc[c] = t;
        sum += t;
      }
      uint32_t incl = sum;
      for (int d = 1; d < 32; d <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += t;
      }
      if (lane == 31) wt[warp] = incl;
      __syncthreads();
      uint32_t run = incl - sum;
      for (int w = 0; w < warp; w++) run += wt[w];
#pragma unroll
      for (int c = 0; c < 4; c++)
        if (c < cpt) { pref[base + c] = run; run += loc[c]; }
      if (tid == PS_NT - 1 && A.seg_c) A.seg_c[s] = run;
      __syncthreads();
    }
    if (A.mode == 1) {
      // primes p with x / p in [lo, hi): p in (x / hi, x / lo], inside (qlo, qhi]
      const int64_t pa = dmax(A.qlo, (int64_t) div128(x, hi));
      const int64_t pb = (lo == 0) ? A.qhi : dmin(A.qhi, (int64_t) div128(x, lo));
      long long lsum = 0, cnt = 0;
      if (pb > pa) {
        const int64_t w0 = (pa + 1) / 240, w1 = pb / 240;
        for (int64_t w = w0 + tid; w <= w1; w += PS_NT) {
          uint64_t bw = A.pibig[2 * w + 1];
          while (bw) {
            const int j = __ffsll((long long) bw) - 1;
            bw &= bw - 1;
            const int64_t p = 240 * w + 30 * (j >> 3) + woff(j & 7);
            if (p <= pa || p > pb) continue;
            const uint64_t n = (uint64_t) div128(x, (uint64_t) p);
            const uint32_t off = (uint32_t) (n - lo);
            const uint32_t ww = off / 240, r = off - ww * 240;
            uint32_t v = pref[ww >> 3];
            for (uint32_t i = ww & ~7u; i < ww; i++) v += __popcll(bits[i]);
            v += __popcll(bits[ww] & mask_le(r));
            lsum += v;
            cnt++;
          }
        }
      }
      for (int d = 16; d > 0; d >>= 1) {
        lsum += __shfl_down_sync(0xffffffffu, lsum, d);
        cnt += __shfl_down_sync(0xffffffffu, cnt, d);
      }
      if (lane == 0) { red[0][warp] = lsum; red[1][warp] = cnt; }
      __syncthreads();
      if (tid == 0) {
        long long a = 0, b = 0;
        for (int i = 0; i < PS_NT / 32; i++) { a += red[0][i]; b += red[1][i]; }
        A.seg_l[s] = a;
        A.seg_m[s] = b;
      }
    }
  }
}

// primes 67 <= p <= limit (the sieve's cross-off primes above the patterns)
static std::vector<uint32_t> base_primes67(int64_t limit)
{
  std::vector<uint8_t> c((size_t) std::max<int64_t>(limit, 1) + 1, 0);
  std::vector<uint32_t> p;
  for (int64_t i = 2; i <= limit; i++) {
    if (c[(size_t) i]) continue;
    if (i >= 67) p.push_back((uint32_t) i);
    for (int64_t m = i * i; m <= limit; m += i) c[(size_t) m] = 1;
  }
  return p;
}

struct PsOut {
  std::vector<int64_t> c, m, l;
  int64_t lo0 = 0, nseg = 0;
};

// segment words and the warp/lane split of the prime sieve (PCG_PS_WORDS,
// PCG_PS_MID override them; words must be 4096, 8192, 12288 or 16384)
static int ps_words()
{
  static const int w = [] {
    const char* e = getenv("PCG_PS_WORDS");
    const int v = e ? atoi(e) : 12288;
    return (v >= 4096 && v <= 16384 && v % 4096 == 0) ? v : 12288;
  }();
  return w;
}

static int64_t ps_mid_div()
{
  static const int64_t d = [] {
    const char* e = getenv("PCG_PS_MID");
    const int64_t v = e ? atoll(e) : 256;
    return v > 0 ? v : 256;
  }();
  return d;
}

// sieve [lo0, end) in segments; B queries for primes in (qlo, qhi] when b_mode
static PsOut run_psieve(Ctx& c, u128 x, int64_t lo0, int64_t end, bool b_mode, int64_t qlo, int64_t qhi,
                        cudaStream_t s, uint64_t* launches)
{
  PsOut o;
  lo0 -= lo0 % 240;
  o.lo0 = lo0;
  const int words = ps_words();
  const int64_t seg = (int64_t) words * 240;
  o.nseg = (end - lo0 + seg - 1) / seg;
  if (o.nseg <= 0) return o;
  std::vector<uint32_t> base = base_primes67(isqrt((u128) end) + 1);
  std::vector<uint64_t> magic(base.size());
  int nmid = 0;
  const int64_t mid_limit = seg / ps_mid_div();
  for (size_t i = 0; i < base.size(); i++) {
    magic[i] = UINT64_MAX / base[i];
    if ((int64_t) base[i] < mid_limit) nmid = (int) i + 1;
  }
  DevBuf& d_base = c.tmp[T_PS_BASE];
  DevBuf& d_magic = c.tmp[T_PS_MAGIC];
  DevBuf& d_c = c.tmp[T_PS_C];
  DevBuf& d_m = c.tmp[T_PS_M];
  DevBuf& d_l = c.tmp[T_PS_L];
  DevBuf& d_q = c.tmp[T_PS_Q];
  d_base.alloc(std::max<size_t>(base.size(), 1) * 4);
  d_magic.alloc(std::max<size_t>(base.size(), 1) * 8);
  d_c.alloc((size_t) o.nseg * 8);
  d_m.alloc((size_t) o.nseg * 8);
  d_l.alloc((size_t) o.nseg * 8);
  d_q.alloc(64);
  if (!base.empty()) {
    PCG_CUDA(cudaMemcpyAsync(d_base.p, base.data(), base.size() * 4, cudaMemcpyHostToDevice, s));
    PCG_CUDA(cudaMemcpyAsync(d_magic.p, magic.data(), magic.size() * 8, cudaMemcpyHostToDevice, s));
  }
  PCG_CUDA(cudaMemsetAsync(d_q.p, 0, 64, s));
  PCG_CUDA(cudaMemsetAsync(d_m.p, 0, (size_t) o.nseg * 8, s));
  PCG_CUDA(cudaMemsetAsync(d_l.p, 0, (size_t) o.nseg * 8, s));
  PsArgs a;
  memset(&a, 0, sizeof(a));
  a.x_lo = (uint64_t) x;
  a.x_hi = (uint64_t) (x >> 64);
  a.lo0 = lo0;
  a.end = end;
  a.seg = seg;
  a.nseg = o.nseg;
  a.qlo = qlo;
  a.qhi = qhi;
  a.mode = b_mode ? 1 : 0;
  a.words = words;
  a.nbase = (int) base.size();
  a.nmid = nmid;
  a.base = d_base.as<uint32_t>();
  a.magic = d_magic.as<uint64_t>();
  a.pibig = c.tab.pibig.as<uint64_t>();
  a.seg_c = d_c.as<int64_t>();
  a.seg_m = d_m.as<int64_t>();
  a.seg_l = d_l.as<int64_t>();
  a.queue = d_q.as<int>();
  const size_t smem = (size_t) words * 8 + (size_t) (words / 8) * 4 + PS_PAT * 8;
  PCG_CUDA(cudaFuncSetAttribute(k_psieve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem));
  int occ = 0;
  PCG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_psieve, PS_NT, smem));
  const int grid = (int) std::min<int64_t>((int64_t) c.num_sms * std::max(occ, 1), o.nseg);
  k_psieve<<<grid, PS_NT, smem, s>>>(a);
  PCG_CUDA(cudaGetLastError());
  if (launches) *launches += 1;
  o.c.resize((size_t) o.nseg);
  o.m.resize((size_t) o.nseg);
  o.l.resize((size_t) o.nseg);
  PCG_CUDA(cudaMemcpyAsync(o.c.data(), d_c.p, (size_t) o.nseg * 8, cudaMemcpyDeviceToHost, s));
  PCG_CUDA(cudaMemcpyAsync(o.m.data(), d_m.p, (size_t) o.nseg * 8, cudaMemcpyDeviceToHost, s));
  PCG_CUDA(cudaMemcpyAsync(o.l.data(), d_l.p, (size_t) o.nseg * 8, cudaMemcpyDeviceToHost, s));
  PCG_CUDA(cudaStreamSynchronize(s));
  return o;
}

// pi(x) for small x: a direct sieve count (2, 3, 5 are not in the bitmap)
static i128 pi_sieve_count(Ctx& c, int64_t x, cudaStream_t s, uint64_t* launches)
{
  if (x < 2) return 0;
  if (x < 7) return x >= 5 ? 3 : (x >= 3 ? 2 : 1);
  PsOut o = run_psieve(c, (u128) x, 0, x + 1, false, 0, 0, s, launches);
  i128 t = 3;
  for (int64_t i = 0; i < o.nseg; i++) t += o.c[(size_t) i];
  return t;
}

// device pi lookups of a batch of values in the PiTable up to sqrt(x)
__global__ void k_pi_lookup(const uint64_t* __restrict__ pt, const uint64_t* __restrict__ v, int64_t n,
                            int64_t* __restrict__ out)
{
  int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = dpi(pt, v[i]);
}

static std::vector<int64_t> pi_lookup(Ctx& c, const std::vector<uint64_t>& v, cudaStream_t s)
{
  std::vector<int64_t> r(v.size());
  if (v.empty()) return r;
  for (uint64_t t : v)
    if ((int64_t) t < 0 || (int64_t) t > c.tab.pibig_limit) fail(PCG_EINTERNAL, "pi lookup beyond the PiTable");
  DevBuf& dv = c.tmp[T_LK_V];
  DevBuf& dr = c.tmp[T_LK_R];
  dv.alloc(v.size() * 8);
  dr.alloc(v.size() * 8);
  PCG_CUDA(cudaMemcpyAsync(dv.p, v.data(), v.size() * 8, cudaMemcpyHostToDevice, s));
  k_pi_lookup<<<(unsigned) ((v.size() + 255) / 256), 256, 0, s>>>(c.tab.pibig.as<uint64_t>(), dv.as<uint64_t>(),
                                                                   (int64_t) v.size(), dr.as<int64_t>());
  PCG_CUDA(cudaGetLastError());
  PCG_CUDA(cudaMemcpyAsync(r.data(), dr.p, v.size() * 8, cudaMemcpyDeviceToHost, s));
  PCG_CUDA(cudaStreamSynchronize(s));
  return r;
}

// ---------------------------------------------------------------- pi(x), Gourdon
struct PiParts {
  i128 ac = 0, b = 0, d = 0, phi0 = 0, sigma = 0, pi = 0;
  double ms_d = 0, ms_ac = 0, ms_b = 0, ms_phi0 = 0, ms_sigma = 0, ms_tables = 0;
  uint64_t launches = 0;
  pcg_stats dstats{};
};

static void ensure_pibig(Ctx& c, int64_t limit, cudaStream_t s)
{
  if (c.tab.pibig_limit >= limit) return;
  build_pitab_only(c.tab.pibig, limit, s);
  c.tab.pibig_limit = limit;
}

// D runs beside the other terms of pi(x) unless PCG_PI_OVERLAP=0
static bool pi_overlap()
{
  static const bool on = [] {
    const char* e = getenv("PCG_PI_OVERLAP");
    return !(e && atoi(e) == 0);
  }();
  return on;
}

// the context's second stream (created on first use)
static cudaStream_t aux_stream(Ctx& c)
{
  std::lock_guard<std::mutex> g(c.aux_mu);
  if (!c.aux) PCG_CUDA(cudaStreamCreateWithFlags(&c.aux, cudaStreamNonBlocking));
  return c.aux;
}

// sum over the primes y < p <= sqrt(x) of pi(x / p): Gourdon's B (B.cpp:38-131)
// and, less the arithmetic series of the prime indices, Deleglise-Rivat's P2
// (P2.cpp).  A prime sieve of [x / sqrt(x), x / y] answers the queries x / p
// in each segment; the segments are joined by the running count pi(lo - 1).
static i128 sum_pi_x_over_p(Ctx& c, u128 x, int64_t y, int64_t sqrtx, cudaStream_t s, uint64_t* nl)
{
  const int64_t n0 = (int64_t) (x / (u128) sqrtx);        // smallest x / p
  const int64_t n1 = (int64_t) (x / (u128) (y + 1)) + 1;  // x / p < n1 for p > y
  i128 B = 0;
  if (sqrtx > y && n1 > n0) {
    PsOut o = run_psieve(c, x, n0, n1, true, y, sqrtx, s, nl);
    // pi(lo0 - 1) from the PiTable up to sqrt(x) (lo0 >= sqrt(x) > 1e5 here)
    i128 run = 0;
    if (o.lo0 >= 7) run = pi_lookup(c, std::vector<uint64_t>{(uint64_t) (o.lo0 - 1)}, s)[0];
    for (int64_t i = 0; i < o.nseg; i++) {
      B += (i128) o.l[(size_t) i] + (i128) o.m[(size_t) i] * run;
      run += o.c[(size_t) i];
    }
  }
  return B;
}

// with_d = false leaves D out (R.d = 0, R.pi without it): the batch form
// computes the D of all its queries in one batched sweep
static PiParts pi_gourdon(Ctx& c, u128 x, const Tuning& tune, cudaStream_t s, bool with_d = true)
{
  PiParts R;
  GourdonParams g = gourdon_params(x, tune.alpha_y, tune.alpha_z);
  const int64_t y = g.y, z = g.z, k = g.k, x_star = g.x_star;
  if (x > ((u128) y << 62)) fail(PCG_ERANGE, "pi_gourdon(x): x is too large");
  const int64_t sqrtx = isqrt(x);
  const int64_t x13 = iroot(x, 3);
  double t0 = fnow_ms();
  ensure_prime_tables(c, std::max<int64_t>(y, sqrtx > 0 ? std::min<int64_t>(y, sqrtx) : y), s);
  ensure_factor_d(c, y, z, s);
  ensure_pibig(c, sqrtx + 240, s);
  ensure_phi_tiny(c, (int) k, s);
  R.ms_tables = fnow_ms() - t0;
  const Tables& T = c.tab;

  // ---- D (hard special leaves) on s and, from a second host thread on the
  // context's second stream, A + C, B, Phi0 and Sigma: their launches fill
  // the SMs that the sweep's waves leave idle at their ends
  auto d_term = [&]() {
    double t1 = fnow_ms();
    SweepProblem p;
    p.gourdon = 1;
    p.x = x;
    p.y = y;
    p.z = z;
    p.k = k;
    SweepResult r = run_sweep(c, p, tune, s);
    R.d = r.sum;
    R.dstats = r.stats;
    R.launches += r.stats.kernel_launches;
    R.ms_d = fnow_ms() - t1;
  };
  auto other_terms = [&](cudaStream_t s, uint64_t* nl) {
    // ---- A + C
    {
      double t1 = fnow_ms();
      const u128 xy = x / (u128) y, xz = x / (u128) z;
      AcParams P;
      memset(&P, 0, sizeof(P));
      P.x_lo = (uint64_t) x;
      P.x_hi = (uint64_t) (x >> 64);
      P.y = y;
      P.z = z;
      P.k = k;
      P.x_star = x_star;
      P.x13 = x13;
      P.sqrtx = sqrtx;
      P.primes = T.primes.as<uint32_t>();
      P.pismall = T.pitab.as<uint64_t>();
      P.pibig = T.pibig.as<uint64_t>();
      const int64_t pi_sqrtz = host_pi(T, (uint64_t) isqrt((u128) z));
      P.bA0 = host_pi(T, (uint64_t) x_star);
      P.bA1 = host_pi(T, (uint64_t) x13);
      P.bC10 = std::max<int64_t>(k, host_pi(T, (uint64_t) iroot(xz, 3)));
      P.bC11 = pi_sqrtz;
      P.bC20 = std::max<int64_t>({k, host_pi(T, (uint64_t) iroot(xy, 3)), pi_sqrtz});
      P.bC21 = host_pi(T, (uint64_t) x_star);
      const int64_t nA = std::max<int64_t>(0, P.bA1 - P.bA0);
      const int64_t nC1 = std::max<int64_t>(0, P.bC11 - P.bC10);
      const int64_t nC2 = std::max<int64_t>(0, P.bC21 - P.bC20);
      // C1 products: count q per b, then expand
      int64_t nQ = 0;
      DevBuf& qlo = c.tmp[T_AC_QLO];
      DevBuf& qcnt = c.tmp[T_AC_QCNT];
      DevBuf& qoff = c.tmp[T_AC_QOFF];
      std::vector<int64_t> hq;
      if (nC1 > 0) {
        qlo.alloc((size_t) nC1 * 8);
        qcnt.alloc((size_t) nC1 * 8);
        qoff.alloc((size_t) nC1 * 8);
        k_c1_qcount<<<(unsigned) ((nC1 + 127) / 128), 128, 0, s>>>(P, qlo.as<int64_t>(), qcnt.as<int64_t>());
        PCG_CUDA(cudaGetLastError());
        (*nl)++;
        hq.resize((size_t) nC1);
        PCG_CUDA(cudaMemcpyAsync(hq.data(), qcnt.p, (size_t) nC1 * 8, cudaMemcpyDeviceToHost, s));
        PCG_CUDA(cudaStreamSynchronize(s));
        std::vector<int64_t> off((size_t) nC1);
        for (int64_t j = 0; j < nC1; j++) { off[(size_t) j] = nQ; nQ += hq[(size_t) j]; }
        PCG_CUDA(cudaMemcpyAsync(qoff.p, off.data(), (size_t) nC1 * 8, cudaMemcpyHostToDevice, s));
      }
      const int64_t nout = nA + nC1 + nQ + nC2;
      i128 sum = 0;
      if (nout > 0) {
        DevBuf& outs = c.tmp[T_AC_OUTS];
        outs.alloc((size_t) nout * sizeof(PairOuter));
        PairOuter* o = outs.as<PairOuter>();
        if (nA) k_outer_A<<<(unsigned) ((nA + 127) / 128), 128, 0, s>>>(P, o);
        if (nC1) k_outer_C1<<<(unsigned) ((nC1 + 127) / 128), 128, 0, s>>>(P, o + nA);
        if (nQ) k_c1_expand<<<(unsigned) ((nC1 + 127) / 128), 128, 0, s>>>(P, qlo.as<int64_t>(), qcnt.as<int64_t>(),
                                                                            qoff.as<int64_t>(), o + nA + nC1);
        if (nC2) k_outer_C2<<<(unsigned) ((nC2 + 127) / 128), 128, 0, s>>>(P, o + nA + nC1 + nQ);
        PCG_CUDA(cudaGetLastError());
        *nl += 4;
        sum = run_pairs(c, o, nout, s, nl);
      }
      R.ac = sum;
      R.ms_ac = fnow_ms() - t1;
    }

    // ---- B = sum over primes y < p <= sqrt(x) of pi(x / p)
    {
      double t1 = fnow_ms();
      R.b = sum_pi_x_over_p(c, x, y, sqrtx, s, nl);
      R.ms_b = fnow_ms() - t1;
    }

    // ---- Phi0
    {
      double t1 = fnow_ms();
      const int64_t size = wheel2310().to_index((uint64_t) z) + 1;
      const int grid = c.num_sms * 8;
      DevBuf& part = c.tmp[T_PHI0_PART];
      part.alloc((size_t) grid * 16);
      PCG_CUDA(cudaMemsetAsync(part.p, 0, (size_t) grid * 16, s));
      PhiTab PT = phi_tab(c);
      if (T.fd_bytes == 2)
        k_phi0<uint16_t><<<grid, 256, 0, s>>>((uint64_t) x, (uint64_t) (x >> 64), T.factor_d.as<uint16_t>(), size,
                                              (uint32_t) (2 * k + 1), (uint64_t) T.h_primes[(size_t) k], PT, T.coprime.as<uint16_t>(), part.as<i128>());
      else
        k_phi0<uint32_t><<<grid, 256, 0, s>>>((uint64_t) x, (uint64_t) (x >> 64), T.factor_d.as<uint32_t>(), size,
                                              (uint32_t) (2 * k + 1), (uint64_t) T.h_primes[(size_t) k], PT, T.coprime.as<uint16_t>(), part.as<i128>());
      PCG_CUDA(cudaGetLastError());
      (*nl)++;
      R.phi0 = sum_partials(part, grid, s);
      R.ms_phi0 = fnow_ms() - t1;
    }

    // ---- Sigma (Sigma.cpp:25-140)
    {
      double t1 = fnow_ms();
      const i128 a = host_pi(T, (uint64_t) y);
      const i128 b = host_pi(T, (uint64_t) x13);
      const int64_t sqrt_xy = isqrt(x / (u128) y);
      std::vector<uint64_t> q;
      q.push_back((uint64_t) sqrtx);
      q.push_back((uint64_t) sqrt_xy);
      // primes in (x_star, x^(1/3)]: arguments of Sigma4..6
      const int64_t i0 = host_pi(T, (uint64_t) x_star) + 1, i1 = host_pi(T, (uint64_t) x13);
      for (int64_t i = i0; i <= i1; i++) {
        const u128 p = T.h_primes[(size_t) i];
        if ((int64_t) p <= sqrt_xy) q.push_back((uint64_t) (x / (p * (u128) y)));
        else q.push_back((uint64_t) (x / (p * p)));
        q.push_back((uint64_t) isqrt(x / p));
      }
      std::vector<int64_t> r = pi_lookup(c, q, s);
      const i128 pi_sqrtx = r[0];
      const i128 cc = r[1];
      const i128 d = host_pi(T, (uint64_t) x_star);
      i128 s0 = a - 1 + (pi_sqrtx * (pi_sqrtx - 1)) / 2 - (a * (a - 1)) / 2;
      i128 s1 = (a - b) * (a - b - 1) / 2;
      i128 s2 = a * (b - cc - (cc * (cc - 3)) / 2 + (d * (d - 3)) / 2);
      i128 s3 = (b * (b - 1) * (2 * b - 1)) / 6 - b - (d * (d - 1) * (2 * d - 1)) / 6 + d;
      i128 s4 = 0, s5 = 0, s6 = 0;
      size_t j = 2;
      for (int64_t i = i0; i <= i1; i++) {
        const int64_t p = T.h_primes[(size_t) i];
        if (p <= sqrt_xy) s4 += r[j]; else s5 += r[j];
        j++;
        s6 += (i128) r[j] * r[j];
        j++;
      }
      R.sigma = s0 + s1 + s2 + s3 + s4 * a + s5 - s6;
      R.ms_sigma = fnow_ms() - t1;
    }
  };
  uint64_t launches2 = 0;
  if (!with_d) {
    other_terms(s, &launches2);
  } else if (pi_overlap()) {
    cudaStream_t s2 = aux_stream(c);
    PCG_CUDA(cudaEventRecord(c.ev[2], s));          // the tables are built on s
    PCG_CUDA(cudaStreamWaitEvent(s2, c.ev[2], 0));
    std::exception_ptr err;
    std::thread th([&] {
      try {
        PCG_CUDA(cudaSetDevice(c.device));
        other_terms(s2, &launches2);
      } catch (...) {
        err = std::current_exception();
      }
    });
    try {
      d_term();
    } catch (...) {
      th.join();
      throw;
    }
    th.join();
    if (err) std::rethrow_exception(err);
  } else {
    d_term();
    other_terms(s, &launches2);
  }
  R.launches += launches2;
  R.pi = R.ac - R.b + R.d + R.phi0 + R.sigma;
  return R;
}

// ---- pi(x) by the Deleglise-Rivat formula (pi_deleglise_rivat.cpp:61-136):
// pi(x) = pi(y) + S1 + S2_trivial + S2_easy + S2_hard - 1 - P2 with y =
// alpha x^(1/3), z = x / y, c = PhiTiny::get_c(y).  out7 = {S1, S2_trivial,
// S2_easy, S2_hard, P2, pi(y), pi(x)}.  S2_hard is the engine's sweep; S1 the
// ordinary leaves over the FactorTable; S2_easy the pair-sum kernel;
// S2_trivial closed forms on the host; P2 the prime sieve of B.
void pi_dr_terms(Ctx& c, u128 x, const Tuning& tune, cudaStream_t s, i128 out[7])
{
  const DrParams g = dr_params(x);
  const int64_t y = g.y, z = g.z, cc = g.c;
  if (x > ((u128) y << 62)) fail(PCG_ERANGE, "pi_deleglise_rivat(x): x is too large");
  const int64_t sqrtx = isqrt(x);
  const int64_t x13 = iroot(x, 3);
  ensure_prime_tables(c, std::max<int64_t>(y, 1000), s);
  ensure_factor_dr(c, y, s);
  ensure_pibig(c, sqrtx + 240, s);
  ensure_phi_tiny(c, (int) cc, s);
  const Tables& T = c.tab;
  const int64_t pi_y = host_pi(T, (uint64_t) y);
  const int64_t prime_c = T.h_primes[(size_t) cc];

  // S2_hard (S2_hard.cpp:221-293): the sweep
  i128 s2_hard;
  {
    SweepProblem p;
    p.gourdon = 0;
    p.x = x;
    p.y = y;
    p.z = z;
    p.k = cc;
    s2_hard = run_sweep(c, p, tune, s).sum;
  }

  // S1 (S1.cpp): sum over the square-free n <= y with lpf(n) > p_c of
  // mu(n) phi(x / n, c): the FactorTable entries above p_c (1 -> T_MAX - 1,
  // composites lpf or lpf - 1 by mu, primes T_MAX) except the primes <= p_c
  i128 s1;
  {
    const int64_t size = wheel2310().to_index((uint64_t) y) + 1;
    const int grid = c.num_sms * 8;
    DevBuf& part = c.tmp[T_PHI0_PART];
    part.alloc((size_t) grid * 16);
    PCG_CUDA(cudaMemsetAsync(part.p, 0, (size_t) grid * 16, s));
    PhiTab PT = phi_tab(c);
    if (T.fr_bytes == 2)
      k_phi0<uint16_t><<<grid, 256, 0, s>>>((uint64_t) x, (uint64_t) (x >> 64), T.factor_dr.as<uint16_t>(), size,
                                            (uint32_t) prime_c, (uint64_t) prime_c, PT, T.coprime.as<uint16_t>(),
                                            part.as<i128>());
    else
      k_phi0<uint32_t><<<grid, 256, 0, s>>>((uint64_t) x, (uint64_t) (x >> 64), T.factor_dr.as<uint32_t>(), size,
                                            (uint32_t) prime_c, (uint64_t) prime_c, PT, T.coprime.as<uint16_t>(),
                                            part.as<i128>());
    PCG_CUDA(cudaGetLastError());
    s1 = sum_partials(part, grid, s);
  }

  // S2_trivial (S2_trivial.cpp:34-88): the leaves p_b p_l with phi(x / n, b - 1) = 1
  i128 s2_trivial = 0;
  if (y >= 2) {
    const int64_t start = std::max<int64_t>(prime_c, isqrt((u128) z)) + 1;
    if (start < y) {
      int64_t j = host_pi(T, (uint64_t) (start - 1)) + 1;
      int64_t prime = INT64_MAX;
      for (; j <= T.nprimes; j++) {
        prime = T.h_primes[(size_t) j];
        if (prime >= y) break;
        const int64_t xpp = (int64_t) (x / ((u128) prime * (u128) prime));
        if (xpp <= prime) break;
        s2_trivial += (i128) (pi_y - host_pi(T, (uint64_t) xpp));
      }
      if (j > T.nprimes) prime = INT64_MAX;
      if (prime < y) {
        const i128 n = (i128) (host_pi(T, (uint64_t) (y - 1)) - host_pi(T, (uint64_t) prime)) + 1;
        const i128 a1 = (i128) (pi_y - host_pi(T, (uint64_t) (y - 1)));
        const i128 a2 = (i128) (pi_y - host_pi(T, (uint64_t) prime));
        s2_trivial += n * (a1 + a2) / 2;
      }
    }
  }

  // S2_easy (S2_easy.cpp): pair sums pi(x / (p_b q)) - b + 2
  i128 s2_easy = 0;
  {
    const int64_t b0 = std::max<int64_t>(cc, host_pi(T, (uint64_t) isqrt((u128) y)));
    const int64_t b1 = host_pi(T, (uint64_t) x13);
    const int64_t n = std::max<int64_t>(0, b1 - b0);
    if (n > 0) {
      DevBuf& outs = c.tmp[T_AC_OUTS];
      outs.alloc((size_t) n * sizeof(PairOuter));
      k_outer_S2e<<<(unsigned) ((n + 127) / 128), 128, 0, s>>>((uint64_t) x, (uint64_t) (x >> 64), y, z, b0, b1,
                                                              T.primes.as<uint32_t>(), T.pitab.as<uint64_t>(),
                                                              outs.as<PairOuter>());
      PCG_CUDA(cudaGetLastError());
      s2_easy = run_pairs(c, outs.as<PairOuter>(), n, s, nullptr);
    }
  }

  // P2 (P2.cpp): sum over y < p <= sqrt(x) of pi(x / p) - pi(p) + 1
  i128 p2;
  {
    const i128 B = sum_pi_x_over_p(c, x, y, sqrtx, s, nullptr);
    const i128 n2 = pi_lookup(c, std::vector<uint64_t>{(uint64_t) sqrtx}, s)[0];   // PiTable up to sqrt(x)
    const i128 a = pi_y;
    p2 = sqrtx > y ? B - (n2 * (n2 - 1) - a * (a - 1)) / 2 : 0;
  }
  out[0] = s1;
  out[1] = s2_trivial;
  out[2] = s2_easy;
  out[3] = s2_hard;
  out[4] = p2;
  out[5] = pi_y;
  out[6] = (i128) pi_y + s1 + s2_trivial + s2_easy + s2_hard - 1 - p2;
}

// x <= 1e10 is counted by the sieve directly
static const int64_t PI_SIEVE_LIMIT = 10000000000ll;

i128 pi_any(Ctx& c, u128 x, const Tuning& tune, cudaStream_t s, pcg_stats* st)
{
  double t0 = fnow_ms();
  i128 r;
  pcg_stats z{};
  if (x < 2) r = 0;
  else if (x <= (u128) PI_SIEVE_LIMIT) {
    uint64_t l = 0;
    r = pi_sieve_count(c, (int64_t) x, s, &l);
    z.kernel_launches = l;
  } else {
    PiParts P = pi_gourdon(c, x, tune, s);
    r = P.pi;
    z = P.dstats;
    z.kernel_launches = P.launches;
    z.table_ms = P.ms_tables;
    z.ac_ms = P.ms_ac;
    z.b_ms = P.ms_b;
    z.phi0_ms = P.ms_phi0;
    z.sigma_ms = P.ms_sigma;
    z.d_ms = P.ms_d;
  }
  z.total_ms = fnow_ms() - t0;
  if (st) *st = z;
  return r;
}

// pi(x) without Gourdon's D term (x > 1e10), or pi(x) itself (x <= 1e10,
// counted by the sieve): *needs_d tells whether D must still be added
i128 pi_without_d(Ctx& c, u128 x, const Tuning& tune, cudaStream_t s, bool* needs_d)
{
  if (x <= (u128) PI_SIEVE_LIMIT) {
    *needs_d = false;
    return pi_any(c, x, tune, s, nullptr);
  }
  *needs_d = true;
  return pi_gourdon(c, x, tune, s, false).pi;
}

// per-term values of Gourdon's formula (for parity tests against the
// reference's --AC, --B, --Phi0, --Sigma, --D outputs)
void pi_gourdon_terms(Ctx& c, u128 x, const Tuning& tune, cudaStream_t s, i128 out[6])
{
  PiParts P = pi_gourdon(c, x, tune, s);
  out[0] = P.ac;
  out[1] = P.b;
  out[2] = P.d;
  out[3] = P.phi0;
  out[4] = P.sigma;
  out[5] = P.pi;
}


// ================================================================ phi(x, a)
// phi(x, a) = # of n <= x not divisible by any of the first a primes
// (reference semantics and shortcuts: src/phi.cpp:341-430).
//   a <= 8:               the primorial identity (phi_tiny)
//   a > pi(sqrt(x)):      pi(x) - a + 1 (1 once a >= pi(x))       (phi_pix)
//   p_{a+1}^4 > x:        1 + (pi(x) - a) + P2(x, a) + P3(x, a), the
//                         counts of n <= x with 2 and 3 prime factors > p_a
//   otherwise:            ordinary leaves n <= y plus the special leaves
//                         x / (p_b m), m <= y < p_b m, of the Legendre
//                         recursion, the latter by the sweep (mode phi)
__global__ void k_phi_one(uint64_t x, PhiTab T, i128* out) { *out = dphi_tiny((u128) x, T); }

// P3 outers: i in (a, pi(x^(1/3))], j in [i, pi(sqrt(x / p_i))]
__global__ void k_outer_P3(uint64_t x, int64_t a, int64_t i1, const uint32_t* __restrict__ primes,
                           const uint64_t* __restrict__ pibig, PairOuter* __restrict__ outs)
{
  const int64_t t = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t i = a + 1 + t;
  if (i > i1) return;
  const uint64_t p = primes[i];
  const uint64_t xp = x / p;
  PairOuter O;
  O.xp_lo = xp;
  O.xp_hi = 0;
  O.cap = 0;
  O.b = (int32_t) i;
  O.mode = 3;
  O.i_lo = i - 1;
  O.i_hi = dpi(pibig, (uint64_t) disqrt((u128) xp));
  if (O.i_hi < O.i_lo) O.i_hi = O.i_lo;
  outs[t] = O;
}

int64_t phi_any(Ctx& c, int64_t x, int64_t a, const Tuning& tune, cudaStream_t s)
{
  if (x < 1) return 0;
  if (a < 1) return x;
  if (a > x / 2) return 1;
  if (a <= 8) {
    ensure_phi_tiny(c, (int) a, s);
    DevBuf& o = c.tmp[T_PHI_ONE];
    o.alloc(16);
    k_phi_one<<<1, 1, 0, s>>>((uint64_t) x, phi_tab(c), o.as<i128>());
    PCG_CUDA(cudaGetLastError());
    i128 r = 0;
    PCG_CUDA(cudaMemcpyAsync(&r, o.p, 16, cudaMemcpyDeviceToHost, s));
    PCG_CUDA(cudaStreamSynchronize(s));
    return (int64_t) r;
  }
  const int64_t sq = isqrt((u128) x);
  const int64_t pi_sq = (int64_t) pi_any(c, (u128) sq, tune, s, nullptr);
  if (a > pi_sq) {
    const int64_t pix = (int64_t) pi_any(c, (u128) x, tune, s, nullptr);
    return a >= pix ? 1 : pix - a + 1;
  }
  // a <= pi(sqrt x): p_a and p_{a+1} < 2 sqrt(x) + 2 are in the table
  ensure_prime_tables(c, std::max<int64_t>(2 * sq + 10, 1000), s);
  if (a + 1 > c.tab.nprimes) fail(PCG_EINTERNAL, "phi: prime table too small");
  const int64_t pa = c.tab.h_primes[(size_t) a];
  const int64_t pa1 = c.tab.h_primes[(size_t) a + 1];
  if ((u128) pa1 * pa1 * pa1 * pa1 > (u128) x) {
    // 1 + (pi(x) - a) + P2 + P3
    const int64_t pix = (int64_t) pi_any(c, (u128) x, tune, s, nullptr);
    ensure_pibig(c, sq + 240, s);
    // P2 = sum_{a < i <= pi(sqrt x)} (pi(x / p_i) - i + 1)
    i128 B = 0;
    {
      const int64_t n0 = x / sq, n1 = x / (pa + 1) + 1;
      PsOut o = run_psieve(c, (u128) x, n0, n1, true, pa, sq, s, nullptr);
      // pi(n) = pi(lo0 - 1) + (primes >= 7 counted by the segments up to n),
      // plus 2, 3, 5 when the sieve starts at 0 (lo0 is a multiple of 240)
      i128 run = 3;
      if (o.lo0 > 0) run = pi_lookup(c, std::vector<uint64_t>{(uint64_t) (o.lo0 - 1)}, s)[0];
      for (int64_t i = 0; i < o.nseg; i++) {
        B += (i128) o.l[(size_t) i] + (i128) o.m[(size_t) i] * run;
        run += o.c[(size_t) i];
      }
    }
    const i128 n2 = pi_sq;
    const i128 P2 = B - (n2 * (n2 - 1) - (i128) a * (a - 1)) / 2;
    // P3 = sum_{a < i <= pi(x^(1/3))} sum_{i <= j <= pi(sqrt(x / p_i))} (pi(x / (p_i p_j)) - j + 1)
    i128 P3 = 0;
    const int64_t i1 = host_pi(c.tab, (uint64_t) iroot((u128) x, 3));
    if (i1 > a) {
      const int64_t n = i1 - a;
      DevBuf& outs = c.tmp[T_PHI_OUTS];
      outs.alloc((size_t) n * sizeof(PairOuter));
      k_outer_P3<<<(unsigned) ((n + 127) / 128), 128, 0, s>>>((uint64_t) x, a, i1, c.tab.primes.as<uint32_t>(),
                                                              c.tab.pibig.as<uint64_t>(), outs.as<PairOuter>());
      PCG_CUDA(cudaGetLastError());
      P3 = run_pairs(c, outs.as<PairOuter>(), n, s, nullptr);
    }
    return (int64_t) (1 + (i128) (pix - a) + P2 + P3);
  }
  // ordinary + special leaves with m <= y
  const int64_t cc = 8;
  int64_t y = std::max<int64_t>(pa, std::min<int64_t>(sq - 1, 8 * iroot((u128) x, 3)));
  y = std::max<int64_t>(y, pa);
  ensure_prime_tables(c, y, s);
  ensure_factor_d(c, pa, y, s);
  ensure_phi_tiny(c, (int) cc, s);
  i128 s1 = 0;
  {
    const Tables& T = c.tab;
    const int64_t size = wheel2310().to_index((uint64_t) y) + 1;
    const int grid = c.num_sms * 8;
    DevBuf& part = c.tmp[T_PHI0_PART];
    part.alloc((size_t) grid * 16);
    PCG_CUDA(cudaMemsetAsync(part.p, 0, (size_t) grid * 16, s));
    PhiTab PT = phi_tab(c);
    if (T.fd_bytes == 2)
      k_phi0<uint16_t><<<grid, 256, 0, s>>>((uint64_t) x, 0, T.factor_d.as<uint16_t>(), size, (uint32_t) (2 * cc + 1),
                                            (uint64_t) T.h_primes[(size_t) cc], PT, T.coprime.as<uint16_t>(), part.as<i128>());
    else
      k_phi0<uint32_t><<<grid, 256, 0, s>>>((uint64_t) x, 0, T.factor_d.as<uint32_t>(), size, (uint32_t) (2 * cc + 1),
                                            (uint64_t) T.h_primes[(size_t) cc], PT, T.coprime.as<uint16_t>(), part.as<i128>());
    PCG_CUDA(cudaGetLastError());
    s1 = sum_partials(part, grid, s);
  }
  SweepProblem p;
  p.gourdon = 2;
  p.x = (u128) x;
  p.y = y;
  p.z = a;
  p.k = cc;
  SweepResult r = run_sweep(c, p, tune, s);
  return (int64_t) (s1 + r.sum);
}

}  // namespace pcg
