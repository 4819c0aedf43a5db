// Checks strm::xdiv (correctly rounded division from a precomputed
// reciprocal) against IEEE division on the host: random numerators over a
// wide exponent range and the divisors the solver uses plus adversarial ones.
// Built and run by tests/test_exact_division.py.
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "strm_internal.cuh"

static uint64_t s = 88172645463325252ULL;
static uint64_t next() {
  s ^= s << 13;
  s ^= s >> 7;
  s ^= s << 17;
  return s;
}
static double rnd_double(int emin, int emax) {
  uint64_t m = next() & ((1ULL << 52) - 1);
  int e = emin + (int)(next() % (uint64_t)(emax - emin + 1));
  uint64_t bits = ((uint64_t)(e + 1023) << 52) | m;
  if (next() & 1) bits |= 1ULL << 63;
  double d;
  memcpy(&d, &bits, 8);
  return d;
}

int main(int argc, char **argv) {
  long n = argc > 1 ? atol(argv[1]) : 2000000;
  double divisors[64];
  int nd = 0;
  const double base[] = {0.1, 0.2, 0.01, 1.0 / 2048.0, 40.96 / 4096.0, 400.0, 1000.0, 100.0,
                         3.0, 7.0, 0.005, 0.0001234, 1.9999999999999998, 1.0000000000000002,
                         0.30000000000000004, 1.5, 49.0, 1e-3};
  for (double b : base) {
    divisors[nd++] = b;
    divisors[nd++] = b * b;
    divisors[nd++] = 4.0 * b;
  }
  for (int i = 0; i < 8; ++i) divisors[nd++] = fabs(rnd_double(-20, 20));
  long bad = 0;
  for (int k = 0; k < nd; ++k) {
    const double b = divisors[k], rb = 1.0 / b;
    for (long i = 0; i < n; ++i) {
      const double a = (i % 7 == 0) ? (double)(int64_t)(next() % 2001) - 1000.0
                                    : rnd_double(-200, 200);
      const double q = strm::xdiv(a, b, rb), ref = a / b;
      if (memcmp(&q, &ref, 8) != 0) {
        if (bad < 10) printf("mismatch a=%a b=%a got %a want %a\n", a, b, q, ref);
        ++bad;
      }
    }
    // signed zeros
    const double z = strm::xdiv(-0.0, b, rb);
    if (!signbit(z)) { printf("-0/b lost its sign for b=%a\n", b); ++bad; }
  }
  printf("divisors=%d samples=%ld mismatches=%ld\n", nd, n * nd, bad);
  return bad ? 1 : 0;
}
