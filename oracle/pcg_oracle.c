/*
 * pcg_oracle.c -- CPU oracle (test infrastructure, never shipped).
 *
 * Plain-C restatement of the reference's hard-special-leaf algorithms
 * (kimwalisch/primecount 8.7).  Every function cites the reference file and
 * lines it follows.  It exists to check the CUDA engine; see pcg_oracle.h.
 *
 * Build: cc -O2 -fopenmp -shared -fPIC pcg_oracle.c -o liboracle.so
 */
#include "pcg_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef __int128 i128;
typedef unsigned __int128 u128;

/* ------------------------------------------------------------------ */
/* integer helpers (include/imath.hpp, include/isqrt.hpp semantics)    */
/* ------------------------------------------------------------------ */

static u128 ipow_u128(u128 r, int n)
{
  u128 p = 1;
  for (int i = 0; i < n; i++) p *= r;
  return p;
}

/* exact floor(x^(1/n)) for n = 2, 3, 4, 6 (imath.hpp:153-174) */
static int64_t iroot_u128(u128 x, int n)
{
  if (x == 0) return 0;
  int64_t r = (int64_t) pow((double) x, 1.0 / n);
  if (r < 0) r = 0;
  for (; r > 0; r--)
    if (ipow_u128((u128) r, n - 1) <= x / (u128) r) break;
  while (ipow_u128((u128) (r + 1), n - 1) <= x / (u128) (r + 1)) r++;
  return r;
}

static int64_t isqrt_u128(u128 x) { return iroot_u128(x, 2); }
static int64_t isqrt64(int64_t x) { return x <= 0 ? 0 : iroot_u128((u128) x, 2); }
static int64_t min64(int64_t a, int64_t b) { return a < b ? a : b; }
static int64_t max64(int64_t a, int64_t b) { return a > b ? a : b; }
static int64_t min3_64(int64_t a, int64_t b, int64_t c) { return min64(min64(a, b), c); }

/* min(a, b) for a 128-bit a and a non-negative 64-bit b */
static int64_t min_u128_64(u128 a, int64_t b) { return a < (u128) b ? (int64_t) a : b; }

static u128 make_u128(uint64_t lo, int64_t hi) { return ((u128) (uint64_t) hi << 64) | lo; }

/* ------------------------------------------------------------------ */
/* 240-wheel bit layout (src/BitSieve240.cpp, src/sieve/Sieve.hpp:8-12) */
/* bit j of byte i <-> low + 30 i + {1,7,11,13,17,19,23,29}[j]          */
/* ------------------------------------------------------------------ */

static const int WOFF[8] = {1, 7, 11, 13, 17, 19, 23, 29};
static int bitpos30[30];          /* index in WOFF or -1 */
static uint64_t unset_larger[240];/* bits of values <= r within a 240 block */
static uint16_t coprime2310[480]; /* numbers in [0, 2310) coprime to 2..11 (FactorTable.cpp:27) */
static int16_t coprime_idx[2310]; /* index of the largest coprime <= r, -1 for 0 (FactorTable.cpp:84) */
static int tables_ready = 0;

static void init_tables(void)
{
  if (tables_ready) return;
  for (int r = 0; r < 30; r++) bitpos30[r] = -1;
  for (int j = 0; j < 8; j++) bitpos30[WOFF[j]] = j;
  for (int r = 0; r < 240; r++) {
    uint64_t m = 0;
    for (int j = 0; j < 64; j++) {
      int v = 30 * (j / 8) + WOFF[j % 8];
      if (v <= r) m |= 1ull << j;
    }
    unset_larger[r] = m;
  }
  int n = 0, last = -1;
  for (int r = 0; r < 2310; r++) {
    if (r % 2 && r % 3 && r % 5 && r % 7 && r % 11) { coprime2310[n] = (uint16_t) r; last = n; n++; }
    coprime_idx[r] = (int16_t) last;
  }
  /* r = 1 is coprime: coprime_idx[1] = 0 and coprime_idx[0] = -1 */
  __atomic_store_n(&tables_ready, 1, __ATOMIC_RELEASE);
}

/* BaseFactorTable::to_index / to_number (BaseFactorTable.hpp:36-47) */
static int64_t to_index(uint64_t n) { return 480 * (int64_t) (n / 2310) + coprime_idx[n % 2310]; }
static int64_t to_number(uint64_t i) { return 2310 * (int64_t) (i / 480) + coprime2310[i % 480]; }

/* ------------------------------------------------------------------ */
/* primes and PiTable (src/PiTable.cpp:110-262)                        */
/* ------------------------------------------------------------------ */

typedef struct { uint64_t count, bits; } pi_t;
typedef struct { pi_t* t; int64_t max_x; } pitable;

/* odd-only sieve of Eratosthenes: is_composite bytes for odd n <= limit */
static uint8_t* odd_sieve(int64_t limit)
{
  int64_t n = limit / 2 + 1;
  uint8_t* c = (uint8_t*) calloc((size_t) n, 1);
  for (int64_t p = 3; p * p <= limit; p += 2)
    if (!c[p / 2])
      for (int64_t m = p * p; m <= limit; m += 2 * p) c[m / 2] = 1;
  return c;
}

static int is_prime_in(const uint8_t* c, int64_t n)
{
  if (n < 2) return 0;
  if (n == 2) return 1;
  if (n % 2 == 0) return 0;
  return !c[n / 2];
}

/* PiTable {count, bits} per 240 numbers; count includes 2, 3, 5 (pi_cache_[0].count = 3) */
static void pitable_build(pitable* pt, int64_t max_x)
{
  init_tables();
  int64_t limit = max64(max_x, 7);
  uint8_t* c = odd_sieve(limit);
  int64_t blocks = limit / 240 + 1;
  pt->t = (pi_t*) calloc((size_t) blocks, sizeof(pi_t));
  pt->max_x = max_x;
  uint64_t count = 3;
  for (int64_t b = 0; b < blocks; b++) {
    uint64_t bits = 0;
    for (int j = 0; j < 64; j++) {
      int64_t v = 240 * b + 30 * (j / 8) + WOFF[j % 8];
      if (v >= 7 && v <= limit && is_prime_in(c, v)) bits |= 1ull << j;
    }
    pt->t[b].count = count;
    pt->t[b].bits = bits;
    count += (uint64_t) __builtin_popcountll(bits);
  }
  free(c);
}

/* PiTable::operator[] (PiTable.hpp:46-57) */
static int64_t pit(const pitable* pt, uint64_t x)
{
  static const int64_t tiny[6] = {0, 0, 1, 2, 2, 3};
  if (x < 6) return tiny[x];
  const pi_t* e = &pt->t[x / 240];
  return (int64_t) (e->count + (uint64_t) __builtin_popcountll(e->bits & unset_larger[x % 240]));
}

/* 1-indexed primes <= limit (PiTable::get_primes_u32, primes[0] = 0) */
static int64_t* primes_upto(int64_t limit, int64_t* count)
{
  int64_t lim = max64(limit, 2);
  uint8_t* c = odd_sieve(lim);
  int64_t n = 0;
  for (int64_t v = 2; v <= limit; v++) n += is_prime_in(c, v);
  int64_t* p = (int64_t*) malloc(sizeof(int64_t) * (size_t) (n + 2));
  p[0] = 0;
  int64_t i = 1;
  for (int64_t v = 2; v <= limit; v++)
    if (is_prime_in(c, v)) p[i++] = v;
  free(c);
  *count = n;
  return p;
}

/* ------------------------------------------------------------------ */
/* FactorTableD<uint16_t> (src/gourdon/FactorTableD.hpp:78-193)        */
/* FactorTable<uint16_t>  (src/FactorTable.hpp:71-151)                 */
/* ------------------------------------------------------------------ */

int64_t ora_factor_size(int64_t limit)
{
  init_tables();
  return to_index((uint64_t) max64(limit, 1)) + 1;
}

/* next multiple of prime >= low with a cofactor coprime to 2310
 * (BaseFactorTable::next_multiple, BaseFactorTable.hpp:56-70) */
static int64_t next_multiple(int64_t prime, int64_t low, int64_t* index)
{
  int64_t quotient = (low + prime - 1) / prime;
  int64_t i = max64(*index, to_index((uint64_t) max64(quotient, 1)));
  if (quotient == 0) i = max64(*index, 0);
  int64_t multiple = 0;
  for (; multiple < low; i++) multiple = prime * to_number((uint64_t) i);
  *index = i;
  return multiple;
}

/* gourdon = 1: FactorTableD (entries 2*pi(lpf)+[mu=-1], mpf <= y)
 * gourdon = 0: FactorTable  (entries lpf / lpf-1), limit = y */
static int factor_build(int gourdon, int64_t y, int64_t limit, uint32_t tmax, uint32_t* out)
{
  init_tables();
  limit = max64(limit, 1);
  int64_t size = to_index((uint64_t) limit) + 1;
  for (int64_t i = 0; i < size; i++) out[i] = tmax;
  out[0] = tmax ^ 1;
  int64_t low = 13, high = limit;
  if (low > high) return 0;
  int64_t sqrtz = isqrt64(limit);
  int64_t cnt;
  int64_t* primes = primes_upto(max64(limit / 13, 13), &cnt);
  /* primes >= 13 whose smallest co-factor 13 keeps the multiple <= high */
  for (int64_t pi_idx = 6; pi_idx <= cnt; pi_idx++) {
    int64_t prime = primes[pi_idx];
    if (prime * 13 > high) break;
    int64_t i = 1;
    int64_t multiple = next_multiple(prime, low, &i);
    for (; multiple <= high; multiple = prime * to_number((uint64_t) i++)) {
      int64_t mi = to_index((uint64_t) multiple);
      if (out[mi] == tmax)
        out[mi] = gourdon ? (uint32_t) (2 * pi_idx + 1) : (uint32_t) prime;
      else if (out[mi] != 0)
        out[mi] ^= 1;
    }
    if (prime <= sqrtz) {
      int64_t j = 0;
      int64_t square = prime * prime;
      multiple = next_multiple(square, low, &j);
      for (; multiple <= high; multiple = square * to_number((uint64_t) j++))
        out[to_index((uint64_t) multiple)] = 0;
    }
  }
  free(primes);
  if (gourdon) {
    /* primes in (y, z] and their multiples: mpf > y -> 0 */
    int64_t start = max64(13, y + 1);
    if (start <= high) {
      uint8_t* c = odd_sieve(high);
      for (int64_t p = start; p <= high; p++) {
        if (!is_prime_in(c, p)) continue;
        int64_t i = 0;
        int64_t next = next_multiple(p, low, &i);
        for (; next <= high; next = p * to_number((uint64_t) i++))
          out[to_index((uint64_t) next)] = 0;
      }
      free(c);
    }
  }
  return 0;
}

int ora_factor_table_d16(int64_t y, int64_t z, uint16_t* out)
{
  if (z > 386083ll * 386083 - 1) return 1;
  int64_t n = ora_factor_size(z);
  uint32_t* tmp = (uint32_t*) malloc(sizeof(uint32_t) * (size_t) n);
  factor_build(1, y, z, 0xFFFF, tmp);
  for (int64_t i = 0; i < n; i++) out[i] = (uint16_t) tmp[i];
  free(tmp);
  return 0;
}

int ora_factor_table_dr16(int64_t y, uint16_t* out)
{
  if (y > 65534ll * 65534 - 1) return 1;
  int64_t n = ora_factor_size(y);
  uint32_t* tmp = (uint32_t*) malloc(sizeof(uint32_t) * (size_t) n);
  factor_build(0, y, y, 0xFFFF, tmp);
  for (int64_t i = 0; i < n; i++) out[i] = (uint16_t) tmp[i];
  free(tmp);
  return 0;
}

int ora_pi_table(int64_t max_x, uint64_t* out)
{
  pitable pt;
  pitable_build(&pt, max_x);
  int64_t blocks = max64(max_x, 7) / 240 + 1;
  int64_t want = max_x / 240 + 1;
  for (int64_t b = 0; b < want && b < blocks; b++) {
    out[2 * b] = pt.t[b].count;
    out[2 * b + 1] = pt.t[b].bits;
  }
  free(pt.t);
  return 0;
}

/* ------------------------------------------------------------------ */
/* Sieve (src/sieve/Sieve.cpp, count_stop.hpp): bitmap of numbers      */
/* coprime to 30 in [low, high); crossing off a prime also removes the */
/* prime itself; count(stop) is monotone between cross-offs.           */
/* ------------------------------------------------------------------ */

#define CTR_WORDS 8

typedef struct {
  uint64_t* w;
  int64_t nwords;
  uint32_t* ctr;
  int64_t nctr;
  int64_t low, high;
  uint64_t total;
  /* monotone cursor of count(stop) */
  int64_t cur_ctr;
  uint64_t cur_sum;
} osieve;

static void sieve_alloc(osieve* s, int64_t segment_size)
{
  s->nwords = segment_size / 240;
  s->w = (uint64_t*) malloc(sizeof(uint64_t) * (size_t) s->nwords);
  s->nctr = (s->nwords + CTR_WORDS - 1) / CTR_WORDS;
  s->ctr = (uint32_t*) malloc(sizeof(uint32_t) * (size_t) s->nctr);
}

static void sieve_free(osieve* s) { free(s->w); free(s->ctr); }

/* Multiples p q (q coprime to 30) of one prime inside a segment, stepped
 * along the 30-wheel the way the reference's wheel does (Sieve.cpp:192-216,
 * lookup_tables.hpp:31-65): the gap to the next co-factor is one of
 * {6,4,2,4,2,4,6,2}, so the byte (30 numbers) advances by p gap / 30 and the
 * residue by p gap mod 30, precomputed per prime. */
static const int WGAP[8] = {6, 4, 2, 4, 2, 4, 6, 2};
typedef struct {
  int64_t byte;      /* (p q - low) / 30 */
  int r;             /* (p q - low) mod 30, coprime to 30 */
  int j;             /* index of q mod 30 in WOFF */
  int64_t n;         /* co-factors left */
  int64_t dbyte[8];
  int dr[8];
} wstep;

static int wheel_rank(int64_t q) { return bitpos30[q % 30]; }

/* first co-factor q >= qlo coprime to 30 and the count up to qhi */
static void wstep_init(wstep* w, int64_t p, int64_t low, int64_t qlo, int64_t qhi)
{
  while (qlo <= qhi && wheel_rank(qlo) < 0) qlo++;
  w->n = 0;
  if (qlo > qhi) return;
  /* co-factors coprime to 30 in [qlo, qhi] */
  int64_t below_hi = 8 * (qhi / 30), below_lo = 8 * ((qlo - 1) / 30);
  for (int k = 0; k < 8; k++) {
    if (WOFF[k] <= qhi % 30) below_hi++;
    if (WOFF[k] <= (qlo - 1) % 30) below_lo++;
  }
  w->n = below_hi - below_lo;
  int64_t off = p * qlo - low;
  w->byte = off / 30;
  w->r = (int) (off % 30);
  w->j = wheel_rank(qlo);
  for (int k = 0; k < 8; k++) {
    w->dbyte[k] = p * WGAP[k] / 30;
    w->dr[k] = (int) (p * WGAP[k] % 30);
  }
}

/* the current multiple as (word, bit), then advance */
static inline void wstep_next(wstep* w, int64_t* wi, uint64_t* bit)
{
  *wi = w->byte >> 3;
  *bit = 1ull << ((w->byte & 7) * 8 + bitpos30[w->r]);
  int k = w->j;
  w->r += w->dr[k];
  w->byte += w->dbyte[k];
  if (w->r >= 30) { w->r -= 30; w->byte++; }
  w->j = (k + 1) & 7;
  w->n--;
}

static void cross_off_plain(osieve* s, int64_t p)
{
  /* n = p * q, q coprime to 30, low <= n < high */
  wstep w;
  wstep_init(&w, p, s->low, max64((s->low + p - 1) / p, 1), (s->high - 1) / p);
  while (w.n > 0) {
    int64_t wi;
    uint64_t bit;
    wstep_next(&w, &wi, &bit);
    s->w[wi] &= ~bit;
  }
}

/* Sieve::pre_sieve + resize_sieve + init_counter: fill the segment and
 * remove primes[4..c] (Sieve.hpp:63-71, pre_sieve.cpp:102-147) */
static void sieve_segment_init(osieve* s, int64_t low, int64_t high,
                               const int64_t* primes, int64_t c)
{
  s->low = low;
  s->high = high;
  int64_t size = high - low;
  int64_t words = (size + 239) / 240;
  for (int64_t i = 0; i < s->nwords; i++) s->w[i] = (i < words) ? ~0ull : 0;
  if (words > 0) s->w[words - 1] &= unset_larger[(size - 1) % 240];
  for (int64_t i = 4; i <= c; i++) cross_off_plain(s, primes[i]);
  s->total = 0;
  for (int64_t ci = 0; ci < s->nctr; ci++) {
    uint32_t t = 0;
    for (int64_t i = ci * CTR_WORDS; i < min64((ci + 1) * CTR_WORDS, s->nwords); i++)
      t += (uint32_t) __builtin_popcountll(s->w[i]);
    s->ctr[ci] = t;
    s->total += t;
  }
  s->cur_ctr = 0;
  s->cur_sum = 0;
}

static void reset_cursor(osieve* s) { s->cur_ctr = 0; s->cur_sum = 0; }

/* number of unsieved numbers in [low, low + stop] (count_stop.hpp:41-89) */
static inline uint64_t sieve_count(osieve* s, int64_t stop)
{
  int64_t wi = stop / 240;
  int64_t ci = wi / CTR_WORDS;
  while (s->cur_ctr < ci) s->cur_sum += s->ctr[s->cur_ctr++];
  uint64_t c = s->cur_sum;
  for (int64_t i = ci * CTR_WORDS; i < wi; i++) c += (uint64_t) __builtin_popcountll(s->w[i]);
  c += (uint64_t) __builtin_popcountll(s->w[wi] & unset_larger[stop % 240]);
  return c;
}

/* Sieve::cross_off_count (Sieve.cpp:497-845): remove p and its multiples,
 * count the elements removed for the first time */
static void sieve_cross_off_count(osieve* s, int64_t p)
{
  reset_cursor(s);
  if (p < 7) return; /* 2, 3, 5 are not represented in the bitmap */
  uint64_t removed = 0;
  wstep w;
  wstep_init(&w, p, s->low, max64((s->low + p - 1) / p, 1), (s->high - 1) / p);
  while (w.n > 0) {
    int64_t wi;
    uint64_t bit;
    wstep_next(&w, &wi, &bit);
    if (s->w[wi] & bit) {
      s->w[wi] &= ~bit;
      s->ctr[wi / CTR_WORDS]--;
      removed++;
    }
  }
  s->total -= removed;
}

/* ------------------------------------------------------------------ */
/* parameters (src/util.cpp:276-386, src/gourdon/pi_gourdon.cpp:44-62) */
/* ------------------------------------------------------------------ */

static double in_between(double lo, double x, double hi) { return x < lo ? lo : (x > hi ? hi : x); }
static double truncate3(double n) { return (double) ((int64_t) (n * 1000)) / 1000.0; }

/* get_x_star_gourdon (util.cpp:362-386) */
static int64_t x_star_gourdon(u128 x, int64_t y)
{
  y = max64(y, 1);
  u128 yy = (u128) y * (u128) y;
  u128 x_div_yy = (x + yy - 1) / yy;
  int64_t r4 = iroot_u128(x, 4);
  int64_t x_star = (u128) r4 > x_div_yy ? r4 : (int64_t) x_div_yy;
  int64_t sqrt_xy = isqrt_u128(x / (u128) y);
  x_star = min64(x_star, y);
  x_star = min64(x_star, sqrt_xy);
  x_star = max64(x_star, 1);
  return x_star;
}

/* PhiTiny::get_c / get_k (PhiTiny.hpp:47-63) */
static int64_t get_c(int64_t y)
{
  static const int64_t pi20[20] = {0, 0, 1, 2, 2, 3, 3, 4, 4, 4, 4, 5, 5, 6, 6, 6, 6, 7, 7, 8};
  return (y >= 0 && y < 20) ? pi20[y] : 8;
}

void ora_gourdon_params(uint64_t x_lo, int64_t x_hi, double alpha_y, double alpha_z,
                        int64_t* y_out, int64_t* z_out, int64_t* k_out, int64_t* x_star_out)
{
  u128 x = make_u128(x_lo, x_hi);
  double x16 = (double) iroot_u128(x, 6);
  double logx = log((double) x);
  double alpha_yz;
  if ((double) x <= 1e11 && x <= (u128) 100000000000ull)
    alpha_yz = 0.078173 * logx + 1;
  else {
    double a = 0.007888745747017503, b = -0.7610431057184933;
    double c = 25.74106177417062, d = -288.9823576050215;
    alpha_yz = a * logx * logx * logx + b * logx * logx + c * logx + d;
  }
  if (alpha_z < 1) {
    alpha_z = 1.0;
    alpha_z = in_between(1, alpha_yz / 5, alpha_z);
  }
  if (alpha_y < 1) alpha_y = alpha_yz / alpha_z;
  alpha_y = in_between(1, alpha_y, x16);
  alpha_y = truncate3(alpha_y);
  alpha_z = truncate3(alpha_z);
  alpha_y = in_between(1, alpha_y, x16);
  double max_alpha_z = x16 / alpha_y > 1.0 ? x16 / alpha_y : 1.0;
  alpha_z = in_between(1, alpha_z, max_alpha_z);

  int64_t x13 = iroot_u128(x, 3);
  int64_t sqrtx = isqrt_u128(x);
  int64_t y = (int64_t) (x13 * alpha_y);
  y = max64(y, x13 + 1);
  y = min64(y, sqrtx - 1);
  y = max64(y, 1);
  int64_t k = get_c(iroot_u128(x, 4));
  int64_t z = (int64_t) (y * alpha_z);
  z = max64(z, y);
  z = min64(z, sqrtx - 1);
  z = max64(z, 1);
  *y_out = y;
  *z_out = z;
  *k_out = k;
  *x_star_out = x_star_gourdon(x, y);
}

void ora_dr_params(uint64_t x_lo, int64_t x_hi, double alpha,
                   int64_t* y_out, int64_t* z_out, int64_t* c_out)
{
  u128 x = make_u128(x_lo, x_hi);
  double x16 = (double) iroot_u128(x, 6);
  if (alpha < 1) {
    double logx = log((double) x);
    if ((double) x <= 1e9)
      alpha = 0.078173 * logx + 1;
    else
      alpha = 0.00148918 * logx * logx * logx - 0.0691909 * logx * logx + 1.00165 * logx + 0.372253;
  }
  alpha = in_between(1, alpha, x16);
  alpha = truncate3(alpha);
  alpha = in_between(1, alpha, x16);
  int64_t y = (int64_t) (iroot_u128(x, 3) * alpha);
  int64_t z = (int64_t) (x / (u128) max64(y, 1));
  *y_out = y;
  *z_out = z;
  *c_out = get_c(y);
}

/* ------------------------------------------------------------------ */
/* the hard-leaf sweep shared by D and S2_hard                         */
/* ------------------------------------------------------------------ */

typedef struct {
  int gourdon;          /* 1: D (Gourdon), 0: S2_hard (Deleglise-Rivat) */
  u128 x;
  int64_t y, z, k;      /* k = c for S2_hard */
  int64_t limit;        /* sieve limit: x/z (D) or z (S2_hard) */
  int64_t x_star;       /* D only */
  int64_t pi_sqrt;      /* pi(sqrt z) for D, pi(sqrt y) for S2 */
  const int64_t* primes;
  int64_t nprimes;
  const pitable* pi;
  const uint32_t* factor;
} sweep;

/* b bounds of a chunk [low, limit) (D.cpp:83-94, S2_hard.cpp:64-71) */
static void chunk_b_bounds(const sweep* w, int64_t low, int64_t limit,
                           int64_t* min_b, int64_t* max_b)
{
  int64_t low1 = max64(low, 1);
  if (w->gourdon) {
    *max_b = pit(w->pi, (uint64_t) min3_64(isqrt_u128(w->x / (u128) low1), isqrt64(limit), w->x_star));
    *min_b = pit(w->pi, (uint64_t) min64(w->limit / limit, w->x_star));
  } else {
    *max_b = (limit <= w->y) ? w->pi_sqrt
        : pit(w->pi, (uint64_t) min3_64(isqrt_u128(w->x / (u128) low1), isqrt64(w->z), w->y));
    *min_b = pit(w->pi, (uint64_t) min64(w->z / limit, w->primes[*max_b]));
  }
  *min_b = max64(w->k, *min_b) + 1;
}

/* Reference leaf loop over one chunk [low, limit) with phi[b] = phi(low-1, b-1)
 * (D.cpp:106-305; S2_hard.cpp:77-158).  Scalar restatement: the SIMD filter
 * and batching of the reference do not change the set of leaves. */
static i128 sweep_chunk_m(const sweep* w, int64_t low, int64_t limit, int64_t segment_size,
                          int64_t* phi, ora_stats* st, int64_t* msum);

static i128 sweep_chunk(const sweep* w, int64_t low, int64_t limit, int64_t segment_size,
                        int64_t* phi, ora_stats* st)
{
  return sweep_chunk_m(w, low, limit, segment_size, phi, st, NULL);
}

/* msum (optional): per level b, the sum of -mu over the chunk's leaves */
static i128 sweep_chunk_m(const sweep* w, int64_t low, int64_t limit, int64_t segment_size,
                          int64_t* phi, ora_stats* st, int64_t* msum)
{
  i128 sum = 0;
  int64_t min_b, max_b;
  chunk_b_bounds(w, low, limit, &min_b, &max_b);
  if (min_b > max_b) return 0;

  osieve s;
  sieve_alloc(&s, segment_size);
  u128 x = w->x;

  for (; low < limit; low += segment_size) {
    int64_t high = min64(low + segment_size, limit);
    int64_t low1 = max64(low, 1);
    sieve_segment_init(&s, low, high, w->primes, min_b - 1);
    int64_t b = min_b;

    int64_t last = min64(w->pi_sqrt, max_b);
    for (; b <= last; b++) {
      int64_t prime = w->primes[b];
      u128 xp = x / (u128) prime;
      int64_t min_m, max_m;
      if (w->gourdon) {
        int64_t xp_low = min_u128_64(xp / (u128) low1, w->z);
        int64_t xp_high = min_u128_64(xp / (u128) high, w->z);
        min_m = max64(xp_high, w->z / prime);
        u128 xpp = xp / ((u128) prime * (u128) prime);
        max_m = min_u128_64(xpp, xp_low);
      } else {
        int64_t xp_high = min_u128_64(xp / (u128) high, w->y);
        min_m = max64(xp_high, w->y / prime);
        max_m = min_u128_64(xp / (u128) low1, w->y);
      }
      if (prime >= max_m) goto next_segment;

      int64_t mi_lo = to_index((uint64_t) min_m);
      int64_t mi_hi = to_index((uint64_t) max_m);
      int64_t threshold = w->gourdon ? 2 * b + 1 : prime;
      if (st && mi_hi > mi_lo) st->indices_scanned += mi_hi - mi_lo;
      for (int64_t m = mi_hi; m > mi_lo; m--) {
        uint32_t f = w->factor[m];
        if ((int64_t) f > threshold) {
          int64_t mnum = to_number((uint64_t) m);
          int64_t xpm = (xp >> 64) == 0 ? (int64_t) ((uint64_t) xp / (uint64_t) mnum)
                                         : (int64_t) (xp / (u128) mnum);
          int64_t count = (int64_t) sieve_count(&s, xpm - low);
          int64_t phi_xpm = phi[b] + count;
          int64_t mu = (f & 1) ? -1 : 1;
          sum -= (i128) mu * phi_xpm;
          if (msum) msum[b] -= mu;
          if (st) st->leaves++;
        }
      }
      phi[b] += (int64_t) s.total;
      sieve_cross_off_count(&s, prime);
    }

    for (; b <= max_b; b++) {
      int64_t prime = w->primes[b];
      u128 xp = x / (u128) prime;
      int64_t xp_low = min_u128_64(xp / (u128) low1, w->y);
      int64_t xp_high = min_u128_64(xp / (u128) high, w->y);
      int64_t l, min_hard;
      if (w->gourdon) {
        int64_t min_m = max64(xp_high, prime);
        u128 xpp = xp / ((u128) prime * (u128) prime);
        int64_t max_m = min_u128_64(xpp, xp_low);
        l = pit(w->pi, (uint64_t) max_m);
        min_hard = min_m;
      } else {
        l = pit(w->pi, (uint64_t) min64(xp_low, w->z / prime));
        min_hard = max64(xp_high, prime);
      }
      if (prime >= w->primes[l]) goto next_segment;
      for (; w->primes[l] > min_hard; l--) {
        int64_t xpq = (xp >> 64) == 0 ? (int64_t) ((uint64_t) xp / (uint64_t) w->primes[l])
                                       : (int64_t) (xp / (u128) w->primes[l]);
        int64_t count = (int64_t) sieve_count(&s, xpq - low);
        sum += phi[b] + count;
        if (msum) msum[b] += 1;
        if (st) { st->leaves++; st->two_prime_leaves++; }
      }
      phi[b] += (int64_t) s.total;
      sieve_cross_off_count(&s, prime);
    }
  next_segment:;
  }
  sieve_free(&s);
  return sum;
}

/* Counting pass of one chunk: survivors per level b for b <= bmax, i.e. the
 * total_count the reference adds to phi[b] before crossing off primes[b]
 * (D.cpp:271) accumulated over all segments of the chunk. */
static void count_chunk(const sweep* w, int64_t low, int64_t limit, int64_t segment_size,
                        int64_t bmax, int64_t* cnt)
{
  osieve s;
  sieve_alloc(&s, segment_size);
  for (; low < limit; low += segment_size) {
    int64_t high = min64(low + segment_size, limit);
    sieve_segment_init(&s, low, high, w->primes, 0);
    for (int64_t b = 1; b <= bmax; b++) {
      cnt[b] += (int64_t) s.total;
      sieve_cross_off_count(&s, w->primes[b]);
    }
  }
  sieve_free(&s);
}

static int64_t pick_segment_size(int64_t limit)
{
  int64_t s = 240;
  int64_t target = isqrt64(limit);
  while (s < target && s < (1ll << 22)) s *= 2;
  s = (s / 240 + 1) * 240;
  return s;
}

static i128 sweep_run(sweep* w, int threads, ora_stats* st)
{
  int64_t limit = w->limit;
  if (limit <= 0) return 0;
  int64_t seg = pick_segment_size(limit);
  int64_t nseg = (limit + seg - 1) / seg;
  int64_t bglob = w->gourdon ? pit(w->pi, (uint64_t) w->x_star)
                             : pit(w->pi, (uint64_t) min64(isqrt64(w->z), w->y));
  bglob = min64(bglob, w->nprimes);

  if (threads <= 1 || nseg < 2) {
    int64_t* phi = (int64_t*) calloc((size_t) (w->nprimes + 2), sizeof(int64_t));
    i128 r = sweep_chunk(w, 0, limit, seg, phi, st);
    free(phi);
    return r;
  }

  int64_t nchunks = min64(nseg, (int64_t) threads * 8);
  int64_t segs_per = (nseg + nchunks - 1) / nchunks;
  nchunks = (nseg + segs_per - 1) / segs_per;
  int64_t stride = bglob + 2;
  int64_t* cnt = (int64_t*) calloc((size_t) (nchunks * stride), sizeof(int64_t));
  i128* sums = (i128*) calloc((size_t) nchunks, sizeof(i128));
  ora_stats* cst = (ora_stats*) calloc((size_t) nchunks, sizeof(ora_stats));

  /* pass 1: per-chunk survivor counts per level */
  #pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
  for (int64_t c = 0; c < nchunks; c++) {
    int64_t lo = c * segs_per * seg;
    int64_t hi = min64(lo + segs_per * seg, limit);
    if (c + 1 < nchunks) count_chunk(w, lo, hi, seg, bglob, &cnt[c * stride]);
  }
  /* exclusive scan over chunks: phi(low_c - 1, b - 1) */
  int64_t* run = (int64_t*) calloc((size_t) stride, sizeof(int64_t));
  for (int64_t c = 0; c < nchunks; c++)
    for (int64_t b = 0; b < stride; b++) {
      int64_t v = cnt[c * stride + b];
      cnt[c * stride + b] = run[b];
      run[b] += v;
    }
  free(run);

  /* pass 2: leaves */
  #pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
  for (int64_t c = 0; c < nchunks; c++) {
    int64_t lo = c * segs_per * seg;
    int64_t hi = min64(lo + segs_per * seg, limit);
    int64_t* phi = (int64_t*) calloc((size_t) (w->nprimes + 2), sizeof(int64_t));
    for (int64_t b = 0; b < stride && b <= w->nprimes + 1; b++) phi[b] = cnt[c * stride + b];
    sums[c] = sweep_chunk(w, lo, hi, seg, phi, &cst[c]);
    free(phi);
  }
  i128 total = 0;
  for (int64_t c = 0; c < nchunks; c++) {
    total += sums[c];
    if (st) {
      st->leaves += cst[c].leaves;
      st->two_prime_leaves += cst[c].two_prime_leaves;
      st->indices_scanned += cst[c].indices_scanned;
    }
  }
  free(cnt);
  free(sums);
  free(cst);
  return total;
}

/* CPU-baseline sample: run the reference's chunk loop (sweep_chunk) over
 * `nchunks` sub-intervals spread evenly over [0, x/z), together `fraction`
 * of the interval, in parallel.  phi offsets are zero (they do not change the
 * work); the leaves evaluated and the wall time are returned. */
int ora_D_sample(uint64_t x_lo, int64_t x_hi, int64_t y, int64_t z, int64_t k,
                 int nchunks, double fraction, int threads, int64_t* leaves, double* seconds)
{
  init_tables();
  u128 x = make_u128(x_lo, x_hi);
  sweep w;
  memset(&w, 0, sizeof(w));
  w.gourdon = 1;
  w.x = x;
  w.y = y;
  w.z = z;
  w.k = k;
  w.limit = (int64_t) (x / (u128) z);
  w.x_star = x_star_gourdon(x, y);
  pitable pt;
  pitable_build(&pt, y);
  w.pi = &pt;
  w.pi_sqrt = pit(&pt, (uint64_t) isqrt64(z));
  int64_t np;
  int64_t* primes = primes_upto(y, &np);
  w.primes = primes;
  w.nprimes = np;
  int64_t fsz = ora_factor_size(z);
  uint32_t* factor = (uint32_t*) malloc(sizeof(uint32_t) * (size_t) fsz);
  factor_build(1, y, z, 0xFFFF, factor);
  w.factor = factor;
  int64_t seg = 1 << 20;
  seg = (seg / 240 + 1) * 240;
  int64_t span = (int64_t) ((double) w.limit * fraction / nchunks);
  span = (span / seg + 1) * seg;
  int64_t total = 0;
  double t0 = 0;
#ifdef _OPENMP
  t0 = omp_get_wtime();
#endif
  #pragma omp parallel for schedule(dynamic, 1) num_threads(threads) reduction(+:total)
  for (int c = 0; c < nchunks; c++) {
    int64_t lo = (int64_t) ((double) w.limit * c / nchunks);
    lo -= lo % seg;
    int64_t hi = lo + span < w.limit ? lo + span : w.limit;
    int64_t* phi = (int64_t*) calloc((size_t) (np + 2), sizeof(int64_t));
    ora_stats st;
    memset(&st, 0, sizeof(st));
    for (int64_t a = lo; a < hi; a += seg) sweep_chunk(&w, a, a + seg < hi ? a + seg : hi, seg, phi, &st);
    total += st.leaves;
    free(phi);
  }
#ifdef _OPENMP
  *seconds = omp_get_wtime() - t0;
#else
  *seconds = 0;
#endif
  *leaves = total;
  free(factor);
  free(primes);
  free(pt.t);
  return 0;
}

static void split128(i128 v, uint64_t* lo, int64_t* hi)
{
  *lo = (uint64_t) v;
  *hi = (int64_t) (v >> 64);
}

int ora_D(uint64_t x_lo, int64_t x_hi, int64_t y, int64_t z, int64_t k,
          int threads, uint64_t* out_lo, int64_t* out_hi, ora_stats* stats)
{
  init_tables();
  if (stats) memset(stats, 0, sizeof(*stats));
  u128 x = make_u128(x_lo, x_hi);
  if (x_hi < 0 || y < 1 || z < 1 || k < 0) return 1;
  if (z > 386083ll * 386083 - 1) return 2; /* FactorTableD<uint16_t>::max() */
  sweep w;
  memset(&w, 0, sizeof(w));
  w.gourdon = 1;
  w.x = x;
  w.y = y;
  w.z = z;
  w.k = k;
  w.limit = (int64_t) (x / (u128) z);
  w.x_star = x_star_gourdon(x, y);
  pitable pt;
  pitable_build(&pt, y);
  w.pi = &pt;
  w.pi_sqrt = pit(&pt, (uint64_t) isqrt64(z));
  int64_t np;
  int64_t* primes = primes_upto(y, &np);
  w.primes = primes;
  w.nprimes = np;
  int64_t fsz = ora_factor_size(z);
  uint32_t* factor = (uint32_t*) malloc(sizeof(uint32_t) * (size_t) fsz);
  factor_build(1, y, z, 0xFFFF, factor);
  w.factor = factor;
  i128 r = sweep_run(&w, threads, stats);
  free(factor);
  free(primes);
  free(pt.t);
  split128(r, out_lo, out_hi);
  return 0;
}

/* One shard [lo, hi) of D with phi offsets counted from lo (the
 * decomposition of pcg_D_shard): the shard's leaf sum *out, per level b the
 * sum of -mu over its leaves (msum[b]) and the numbers of [lo, hi) that
 * survive to level b (csum[b], the total_count of D.cpp:271 summed over the
 * shard's segments).  lo is a multiple of 240.  Single-threaded. */
int ora_D_partial(uint64_t x_lo, int64_t x_hi, int64_t y, int64_t z, int64_t k, int64_t lo, int64_t hi,
                  uint64_t* out_lo, int64_t* out_hi, int64_t* msum, int64_t* csum, int64_t ncols)
{
  init_tables();
  u128 x = make_u128(x_lo, x_hi);
  if (x_hi < 0 || y < 1 || z < 1 || k < 0 || lo < 0 || lo % 240 != 0 || hi < lo) return 1;
  if (z > 386083ll * 386083 - 1) return 2;
  sweep w;
  memset(&w, 0, sizeof(w));
  w.gourdon = 1;
  w.x = x;
  w.y = y;
  w.z = z;
  w.k = k;
  w.limit = (int64_t) (x / (u128) z);
  w.x_star = x_star_gourdon(x, y);
  pitable pt;
  pitable_build(&pt, y);
  w.pi = &pt;
  w.pi_sqrt = pit(&pt, (uint64_t) isqrt64(z));
  int64_t np;
  int64_t* primes = primes_upto(y, &np);
  w.primes = primes;
  w.nprimes = np;
  int64_t bglob = min64(pit(&pt, (uint64_t) w.x_star), np);
  int rc = 0;
  if (ncols < bglob + 1) { rc = 3; goto done; }
  {
    int64_t fsz = ora_factor_size(z);
    uint32_t* factor = (uint32_t*) malloc(sizeof(uint32_t) * (size_t) fsz);
    factor_build(1, y, z, 0xFFFF, factor);
    w.factor = factor;
    for (int64_t b = 0; b < ncols; b++) { msum[b] = 0; csum[b] = 0; }
    hi = min64(hi, w.limit);
    i128 r = 0;
    if (hi > lo) {
      int64_t seg = pick_segment_size(w.limit);
      count_chunk(&w, lo, hi, seg, bglob, csum);
      int64_t* phi = (int64_t*) calloc((size_t) (np + 2), sizeof(int64_t));
      r = sweep_chunk_m(&w, lo, hi, seg, phi, NULL, msum);
      free(phi);
    }
    free(factor);
    split128(r, out_lo, out_hi);
  }
done:
  free(primes);
  free(pt.t);
  return rc;
}

int ora_S2_hard(uint64_t x_lo, int64_t x_hi, int64_t y, int64_t z, int64_t c,
                int threads, uint64_t* out_lo, int64_t* out_hi, ora_stats* stats)
{
  init_tables();
  if (stats) memset(stats, 0, sizeof(*stats));
  u128 x = make_u128(x_lo, x_hi);
  if (x_hi < 0 || y < 1 || z < 1 || c < 0) return 1;
  if (y > 65534ll * 65534 - 1) return 2; /* FactorTable<uint16_t>::max() */
  sweep w;
  memset(&w, 0, sizeof(w));
  w.gourdon = 0;
  w.x = x;
  w.y = y;
  w.z = z;
  w.k = c;
  w.limit = z;
  int64_t max_prime = min64(y, z / max64(isqrt64(y), 1));
  pitable pt;
  pitable_build(&pt, max_prime);
  w.pi = &pt;
  w.pi_sqrt = pit(&pt, (uint64_t) isqrt64(y));
  int64_t np;
  int64_t* primes = primes_upto(max_prime, &np);
  w.primes = primes;
  w.nprimes = np;
  int64_t fsz = ora_factor_size(y);
  uint32_t* factor = (uint32_t*) malloc(sizeof(uint32_t) * (size_t) fsz);
  factor_build(0, y, y, 0xFFFF, factor);
  w.factor = factor;
  i128 r = sweep_run(&w, threads, stats);
  free(factor);
  free(primes);
  free(pt.t);
  split128(r, out_lo, out_hi);
  return 0;
}

/* ------------------------------------------------------------------ */
/* phi(x, a) and pi(x), small inputs                                   */
/* ------------------------------------------------------------------ */

static int64_t phi_rec(int64_t x, int64_t a, const int64_t* primes)
{
  if (a == 0 || x == 0) return x;
  if (a == 1) return x - x / 2;
  if (x < primes[a]) return 1; /* only 1 survives */
  return phi_rec(x, a - 1, primes) - phi_rec(x / primes[a], a - 1, primes);
}

/* phi(x, a): numbers in [1, x] not divisible by any of the first a primes */
int64_t ora_phi(int64_t x, int64_t a)
{
  if (x < 1) return 0;
  if (a < 1) return x;
  int64_t n;
  int64_t lim = 100;
  int64_t* primes = primes_upto(lim, &n);
  while (n < a && lim < x) {
    free(primes);
    lim *= 4;
    primes = primes_upto(lim, &n);
  }
  if (n < a) {
    /* more primes requested than exist <= x: phi = 1 */
    free(primes);
    return 1;
  }
  int64_t r = phi_rec(x, a, primes);
  free(primes);
  return r;
}

int64_t ora_pi_sieve(int64_t x)
{
  if (x < 2) return 0;
  uint8_t* c = odd_sieve(x);
  int64_t n = 1;
  for (int64_t v = 3; v <= x; v += 2) n += !c[v / 2];
  free(c);
  return n;
}
