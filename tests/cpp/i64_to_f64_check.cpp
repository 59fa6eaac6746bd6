// sgx::i64_to_f64_rn (the integer int64-to-double conversion of the
// float-float lookup) against the compiler's static_cast<double>: 20 million
// seeded values of every magnitude and every exact tie from 2^54 to 2^62.
// Built and run by tests/test_cpu_library.py with the host compiler.
#include <cstdio>
#include <random>
#include "sgx_math.cuh"
int main() {
  std::mt19937_64 g(1);
  long bad = 0;
  for (long i = 0; i < 20000000; ++i) {
    int64_t v = (int64_t)g();
    const int sh = (int)(g() % 64);
    v >>= sh;  // all magnitudes
    if (i % 7 == 0) v = (v | 0x3FF) ;  // ties/odd patterns
    if (v == INT64_MIN) continue;
    const double a = sgx::i64_to_f64_rn(v), b = (double)v;
    if (a != b) { if (bad < 5) printf("%lld %.17g %.17g\n", (long long)v, a, b); ++bad; }
  }
  // exact ties around 2^53.. 2^62
  for (int e = 53; e < 63; ++e) for (int k = 0; k < 4096; ++k) {
    int64_t v = ((int64_t)1 << e) + ((int64_t)k << (e - 53)) + (((int64_t)1 << (e-53)) >> 1);
    for (int s = -1; s <= 1; s += 2) { const int64_t w = s * v; if (sgx::i64_to_f64_rn(w) != (double)w) ++bad; }
  }
  printf("bad=%ld\n", bad);
  return bad != 0;
}
