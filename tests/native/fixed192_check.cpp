// Host check of gravhopper_gb300/csrc/fixed192.cuh: exact fixed-point prefix sums of
// FP64 values and their correctly rounded differences.
//
//   fixed192_check <n values> <ranges> <rng seed> <min exponent> <max exponent> [mantissa bits]
//
// Draws n doubles with random signs and exponents in [min, max] (with only the top
// `mantissa bits` of the significand random, default 52, so that short values make
// rounding ties common), sums prefixes in 192-bit fixed point with lsb = B - 167 (B
// the bound exponent of the largest |v|), and prints: "lsb L", then one line per value
// "v <bits hex>", then per random range [s, e) "r s e <bits of the rounded difference
// P(e) - P(s) hex>".  The test compares these with exact rational arithmetic.
#include <stdio.h>
#include <stdlib.h>

#include <vector>

#include "../../gravhopper_gb300/csrc/fixed192.cuh"

static uint64_t g_rng = 88172645463325252ull;
static uint64_t next_u64() {
  g_rng ^= g_rng << 13;
  g_rng ^= g_rng >> 7;
  g_rng ^= g_rng << 17;
  return g_rng;
}

int main(int argc, char** argv) {
  if (argc < 6) return 2;
  const long n = atol(argv[1]), ranges = atol(argv[2]);
  g_rng ^= (uint64_t)atoll(argv[3]) * 0x9E3779B97F4A7C15ull;
  const int emin = atoi(argv[4]), emax = atoi(argv[5]);
  const int mbits = argc > 6 ? atoi(argv[6]) : 52;
  const uint64_t mmask =
      mbits >= 52 ? 0x000fffffffffffffull : (0x000fffffffffffffull & ~((1ull << (52 - mbits)) - 1ull));
  using namespace gh::fx;
  std::vector<double> v(n);
  double amax = 0.0;
  for (long i = 0; i < n; i++) {
    const uint64_t r = next_u64();
    const int e = emin + (int)(next_u64() % (uint64_t)(emax - emin + 1));
    const uint64_t bits = ((uint64_t)(e + 1023) << 52) | (r & mmask) | ((r >> 63) << 63);
    v[i] = double_of(bits);
    if ((next_u64() & 15) == 0) v[i] = 0.0;
    const double a = v[i] < 0 ? -v[i] : v[i];
    if (a > amax) amax = a;
  }
  const int lsb = bound_exponent(amax) - FX_HEADROOM;
  printf("lsb %d\n", lsb);
  std::vector<I192> P(n + 1);
  P[0] = zero();
  for (long i = 0; i < n; i++) {
    P[i + 1] = add(P[i], from_double(v[i], lsb));
    printf("v %016llx\n", (unsigned long long)bits_of(v[i]));
  }
  for (long k = 0; k < ranges; k++) {
    long s = (long)(next_u64() % (uint64_t)(n + 1)), e = (long)(next_u64() % (uint64_t)(n + 1));
    if (s > e) {
      const long t = s;
      s = e;
      e = t;
    }
    const double d = to_double(sub(P[e], P[s]), lsb);
    printf("r %ld %ld %016llx\n", s, e, (unsigned long long)bits_of(d));
  }
  return 0;
}
