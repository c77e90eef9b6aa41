// Compiler probe of oracle/ref.mk: does the compiler accept an AVX512
// VPOPCNTDQ function under a target attribute (run-time dispatch)?
#include <immintrin.h>
#include <stdint.h>

__attribute__((target("avx512f,avx512bw,avx512vl,avx512vpopcntdq")))
uint64_t probe_popcount8(const uint64_t* a)
{
  __m512i v = _mm512_loadu_si512((const void*) a);
  return (uint64_t) _mm512_reduce_add_epi64(_mm512_popcnt_epi64(v));
}
