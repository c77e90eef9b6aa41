// formulas.cpp -- pi(x) and phi(x, a) on top of the hard-leaf engine.
// (work in progress: entry points return PCG_EINTERNAL until implemented)
#include "pcg_internal.hpp"

extern "C" {

pcg_status pcg_pi(pcg_i128, const pcg_opts*, pcg_i128*) { return PCG_EINTERNAL; }
pcg_status pcg_phi(int64_t, int64_t, const pcg_opts*, int64_t*) { return PCG_EINTERNAL; }
pcg_status pcg_pi_batch(const pcg_i128*, size_t, pcg_i128*, const pcg_opts*) { return PCG_EINTERNAL; }
pcg_status pcg_phi_batch(const int64_t*, const int64_t*, size_t, int64_t*, const pcg_opts*) { return PCG_EINTERNAL; }
int64_t primecount_pi(int64_t) { return -1; }
pcg_i128 primecount_pi_128(pcg_i128) { pcg_i128 r; r.lo = ~0ull; r.hi = -1; return r; }
int64_t primecount_phi(int64_t, int64_t) { return -1; }
static int g_threads = 0;
int primecount_get_num_threads(void) { return g_threads; }
void primecount_set_num_threads(int n) { g_threads = n; }
const char* primecount_version(void) { return "8.7"; }

}
