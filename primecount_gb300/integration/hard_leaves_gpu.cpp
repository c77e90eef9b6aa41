// hard_leaves_gpu.cpp -- primecount's D() and S2_hard() computed by libpcgpu.
//
// A source file for the primecount tree (beside src/gourdon/D.cpp), the
// reference-side half of the drop-in: it defines the reference's own entry
// points for the hard special leaves with their signatures unchanged
//   D(x, y, z, k, threads, is_print)        include/gourdon.hpp:28,38
//   S2_hard(x, y, z, c, threads, is_print)  include/S.hpp:25,32
// and computes them on the GPU through the C ABI of include/pcgpu.h, so that
// pi_gourdon_64/128, S2(), the --D / --S2-hard options and the test programs
// run unchanged.  The reference's own bodies, compiled under the names
// D_cpu / S2_hard_cpu (e.g. -DD=D_cpu on src/gourdon/D.cpp), stay the
// fallback when the machine has no CUDA device or PCG_DISABLE=1 is set
// (PCG_REQUIRE=1 makes a missing device an error instead); any other failure
// becomes the reference's primecount_error, as its own failures do.  pcg_i128 has the layout of pc_int128_t
// (include/primecount.h:38-41).
#include <gourdon.hpp>
#include <S.hpp>
#include <int128_t.hpp>
#include <primecount.hpp>

#include <pcgpu.h>

#include <cstdlib>
#include <stdint.h>

namespace primecount {

// the reference's own implementations, renamed
int64_t D_cpu(int64_t x, int64_t y, int64_t z, int64_t k, int threads, bool is_print);
int64_t S2_hard_cpu(int64_t x, int64_t y, int64_t z, int64_t c, int threads, bool is_print);
#ifdef HAVE_INT128_T
int128_t D_cpu(int128_t x, int64_t y, int64_t z, int64_t k, int threads, bool is_print);
int128_t S2_hard_cpu(int128_t x, int64_t y, int64_t z, int64_t c, int threads, bool is_print);
#endif

namespace {

typedef pcg_status (*hard_fn)(pcg_i128, int64_t, int64_t, int64_t, const pcg_opts*, pcg_i128*);

pcg_i128 to_pcg(int64_t v)
{
  pcg_i128 r;
  r.lo = (uint64_t) v;
  r.hi = v < 0 ? -1 : 0;
  return r;
}

#ifdef HAVE_INT128_T
pcg_i128 to_pcg(int128_t v)
{
  pcg_i128 r;
  r.lo = (uint64_t) v;
  r.hi = (int64_t) (v >> 64);
  return r;
}

int128_t from_pcg(pcg_i128 v) { return (int128_t) (((uint128_t) (uint64_t) v.hi << 64) | v.lo); }
#endif

bool gpu_disabled()
{
  const char* e = std::getenv("PCG_DISABLE");
  return e && *e == '1';
}

// false: no CUDA device (the caller runs the CPU body); throws on any other failure
bool gpu_call(hard_fn fn, pcg_i128 x, int64_t y, int64_t z, int64_t k, bool is_print, pcg_i128* out)
{
  if (gpu_disabled())
    return false;
  pcg_opts o = {};
  o.print = is_print ? 1 : 0;    // the threads argument sizes host threads only: the sweep has none
  pcg_status st = fn(x, y, z, k, &o, out);
  const char* req = std::getenv("PCG_REQUIRE");
  if (st == PCG_ENODEV && !(req && *req == '1'))
    return false;
  if (st != PCG_OK)
    throw primecount_error(pcg_last_error(nullptr));
  return true;
}

} // namespace

int64_t D(int64_t x, int64_t y, int64_t z, int64_t k, int threads, bool is_print)
{
  pcg_i128 r;
  if (gpu_call(pcg_D, to_pcg(x), y, z, k, is_print, &r))
    return (int64_t) r.lo;
  return D_cpu(x, y, z, k, threads, is_print);
}

int64_t S2_hard(int64_t x, int64_t y, int64_t z, int64_t c, int threads, bool is_print)
{
  pcg_i128 r;
  if (gpu_call(pcg_S2_hard, to_pcg(x), y, z, c, is_print, &r))
    return (int64_t) r.lo;
  return S2_hard_cpu(x, y, z, c, threads, is_print);
}

#ifdef HAVE_INT128_T

int128_t D(int128_t x, int64_t y, int64_t z, int64_t k, int threads, bool is_print)
{
  pcg_i128 r;
  if (gpu_call(pcg_D, to_pcg(x), y, z, k, is_print, &r))
    return from_pcg(r);
  return D_cpu(x, y, z, k, threads, is_print);
}

int128_t S2_hard(int128_t x, int64_t y, int64_t z, int64_t c, int threads, bool is_print)
{
  pcg_i128 r;
  if (gpu_call(pcg_S2_hard, to_pcg(x), y, z, c, is_print, &r))
    return from_pcg(r);
  return S2_hard_cpu(x, y, z, c, threads, is_print);
}

#endif

} // namespace primecount
