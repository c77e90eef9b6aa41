// Compiler probe of oracle/ref.mk: does the compiler accept SVE intrinsics
// under a target attribute (run-time dispatch)?
#include <arm_sve.h>
#include <stdint.h>

__attribute__((target("+sve")))
uint64_t probe_popcount(const uint64_t* a, uint64_t n)
{
  svbool_t pg = svwhilelt_b64((uint64_t) 0, n);
  svuint64_t v = svcnt_u64_z(pg, svld1_u64(pg, a));
  return svaddv_u64(svptrue_b64(), v);
}
