// Checks strm::widen / strm::narrow (FP32 <-> FP64 conversions in integer
// arithmetic) against the host's IEEE conversions: random values over the
// whole exponent range, rounding ties, the edges of the FP32 range,
// infinities, NaNs and zeros.  Values the conversions flush (magnitudes
// below 2^-126) must come back as zero of the same sign.  Built and run by
// tests/test_conversions.py.
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "strm_internal.cuh"

static uint64_t s = 0x9E3779B97F4A7C15ULL;
static uint64_t next() {
  s ^= s << 13;
  s ^= s >> 7;
  s ^= s << 17;
  return s;
}

static long bad = 0;

static void check_narrow(double x) {
  const float got = strm::narrow(x);
  float want = (float)x;
  if (fabs(x) < 1.1754943508222875e-38 && !isnan(x)) want = signbit(x) ? -0.0f : 0.0f;
  uint32_t g, w;
  memcpy(&g, &got, 4);
  memcpy(&w, &want, 4);
  if (isnan(want) ? !isnan(got) : g != w) {
    if (bad < 5) printf("narrow(%.17g) = %08x, want %08x\n", x, g, w);
    ++bad;
  }
}

static void check_widen(float f) {
  const double got = strm::widen(f);
  double want = (double)f;
  if (fabsf(f) < 1.17549435e-38f && !isnan(f)) want = signbit(f) ? -0.0 : 0.0;
  uint64_t g, w;
  memcpy(&g, &got, 8);
  memcpy(&w, &want, 8);
  if (isnan(want) ? !isnan(got) : g != w) {
    if (bad < 5) printf("widen(%.9g) = %016llx, want %016llx\n", f, (unsigned long long)g,
                        (unsigned long long)w);
    ++bad;
  }
}

int main(int argc, char **argv) {
  const long n = argc > 1 ? atol(argv[1]) : 1000000;
  for (long i = 0; i < n; ++i) {
    // random doubles across every exponent (NaN and Inf included)
    uint64_t b = next();
    double x;
    memcpy(&x, &b, 8);
    check_narrow(x);
    // doubles near the FP32 range, and exact ties between two floats
    const int e = -130 + (int)(next() % 262);
    const uint64_t m = next() & ((1ULL << 52) - 1);
    uint64_t bb = ((uint64_t)(e + 1023) << 52) | m | (next() & (1ULL << 63));
    memcpy(&x, &bb, 8);
    check_narrow(x);
    bb = (bb & ~((1ULL << 29) - 1)) | (1ULL << 28);  // halfway between two floats
    memcpy(&x, &bb, 8);
    check_narrow(x);
    // random floats (every bit pattern)
    const uint32_t u = (uint32_t)next();
    float f;
    memcpy(&f, &u, 4);
    check_widen(f);
  }
  const double edges[] = {0.0, -0.0, INFINITY, -INFINITY, NAN, 3.4028234663852886e38,
                          3.4028235677973366e38, 1.1754943508222875e-38, 1e-40, -1e-45, 1.0,
                          -1.0, 0.1, 16777217.0};
  for (double x : edges) {
    check_narrow(x);
    check_widen((float)x);
  }
  printf("checked=%ld mismatches=%ld\n", 4 * n, bad);
  return bad ? 1 : 0;
}
