// Host check of gravhopper_gb300/csrc/f64emu.cuh: inv_cube_rn(s) against the IEEE
// double expression 1.0 / s / sqrt(s) on random, boundary and near-midpoint inputs.
//
//   f64emu_check <cases> <rng seed> <seed perturbation exponent, 0 = none>
//
// With a perturbation exponent k > 0 every FP32 rsqrt seed is scaled by a random
// factor in [1 - 2^-k, 1 + 2^-k].  Prints "cases wrong fallback"; a wrong result is
// a fast-path result that differs from the IEEE one (must be 0 for any seed).
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static uint64_t g_rng = 88172645463325252ull;
static uint64_t next_u64() {
  g_rng ^= g_rng << 13;
  g_rng ^= g_rng >> 7;
  g_rng ^= g_rng << 17;
  return g_rng;
}
static int g_perturb = 0;
static float perturbed_rsqrt(float x) {
  float r = 1.0f / sqrtf(x);
  if (g_perturb > 0) {
    const double u = (double)(next_u64() >> 11) * 0x1p-53 * 2.0 - 1.0;  // [-1, 1)
    r = (float)((double)r * (1.0 + u * ldexp(1.0, -g_perturb)));
  }
  return r;
}
#define GH_EMU_HOST_RSQRT(x) perturbed_rsqrt(x)
#include "../../gravhopper_gb300/csrc/f64emu.cuh"

static uint64_t bits_of(double x) {
  uint64_t u;
  memcpy(&u, &x, 8);
  return u;
}

static long long n_cases = 0, n_wrong = 0, n_fallback = 0, n_out = 0;

static void check(double s) {
  const double want = 1.0 / s / sqrt(s);
  double got = 0.0;
  const int E = (int)(bits_of(s) >> 52);
  const bool in_range = E >= 446 && E <= 1624;
  n_cases++;
  if (gh::emu::inv_cube_rn(s, got)) {
    if (bits_of(got) != bits_of(want)) {
      if (n_wrong < 10) printf("WRONG s=%.17g got=%.17g want=%.17g\n", s, got, want);
      n_wrong++;
    }
    if (!in_range) n_out++;
  } else if (in_range) {
    n_fallback++;
  }
}

int main(int argc, char** argv) {
  const long long cases = argc > 1 ? atoll(argv[1]) : 1000000;
  g_rng ^= argc > 2 ? strtoull(argv[2], nullptr, 10) * 0x9E3779B97F4A7C15ull : 0;
  g_perturb = argc > 3 ? atoi(argv[3]) : 0;
  // exact powers, significand extremes
  for (int e = -700; e <= 700; e++) {
    check(ldexp(1.0, e));
    check(ldexp(1.0 + 0x1p-52, e));
    check(ldexp(2.0 - 0x1p-52, e));
    check(ldexp(1.5, e));
  }
  const double special[] = {0.0, -0.0, -1.0, INFINITY, NAN, 4.9406564584124654e-324, 2.2250738585072014e-308,
                            1.7976931348623157e308};
  for (double s : special) check(s);
  const long long per = cases / 6;
  // uniform significand and exponent over the fast range and beyond
  for (long long i = 0; i < per; i++) {
    const uint64_t b = (next_u64() & 0x000FFFFFFFFFFFFFull) | ((uint64_t)(300 + next_u64() % 1450) << 52);
    double s;
    memcpy(&s, &b, 8);
    check(s);
  }
  // square roots near a rounding boundary: X = N 2^54 close to c^2, c odd
  for (long long i = 0; i < per; i++) {
    const uint64_t c = ((next_u64() >> 10) | (1ull << 53) | 1ull) & ((1ull << 54) - 1);
    const unsigned __int128 c2 = (unsigned __int128)c * c;
    uint64_t N = (uint64_t)(c2 >> 54) + (uint64_t)((c2 >> 53) & 1);
    const int d = (int)(next_u64() % 5) - 2;
    N += d;
    if (N >= (1ull << 53)) N &= ~1ull;  // representable
    if (N < (1ull << 52) || N >= (1ull << 54)) continue;
    const int p = 2 * ((int)(next_u64() % 600) - 300);
    check(ldexp((double)N, p - 52));
  }
  // reciprocals near a rounding boundary: M close to 2^106 / c, c odd
  for (long long i = 0; i < per; i++) {
    const uint64_t c = ((next_u64() >> 10) | (1ull << 53) | 1ull) & ((1ull << 54) - 1);
    const unsigned __int128 t = ((unsigned __int128)1 << 106) / c;
    uint64_t M = (uint64_t)t + (uint64_t)((int)(next_u64() % 5) - 2);
    if (M < (1ull << 52) || M >= (1ull << 53)) continue;
    const int e = (int)(next_u64() % 1100) - 550;
    check(ldexp((double)M, e - 52));
  }
  // values of the shape r^2 + eps^2 met by the direct sum
  for (long long i = 0; i < per; i++) {
    const double u = (double)(next_u64() >> 11) * 0x1p-53;
    const double dx = ldexp(u - 0.5, -(int)(next_u64() % 40));
    const double dy = ldexp((double)(next_u64() >> 11) * 0x1p-53 - 0.5, -(int)(next_u64() % 40));
    const double dz = (double)(next_u64() >> 11) * 0x1p-60;
    const double eps = 5e-5 * (double)(next_u64() % 3);
    check(dx * dx + dy * dy + dz * dz + eps * eps);
  }
  // pair factors: s = ((dx^2 + dy^2) + dz^2) + eps2 and 1/s/sqrt(s), signed components
  // often in one binade (ties in the sums), short significands (ties in the squares)
  const double eps_list[] = {0.0, 5e-5, 1e-3, 0.1, 3.0};
  for (long long i = 0; i < per; i++) {
    double d[3];
    const int e0 = (int)(next_u64() % 60) - 40;
    for (int k = 0; k < 3; k++) {
      const uint64_t r = next_u64();
      int e = (r & 3) ? e0 : e0 - (int)(next_u64() % 60);
      double sig;
      if ((r >> 2) % 7 == 0)
        sig = (double)((next_u64() >> 37) | 1) * 0x1p-27;  // short significand
      else
        sig = 1.0 + (double)(next_u64() >> 12) * 0x1p-52;
      d[k] = ldexp((r >> 8) & 1 ? -sig : sig, e);
    }
    const double eps = eps_list[next_u64() % 5] * ((next_u64() & 1) ? 1.0 : 1.0 + (double)(next_u64() >> 40) * 0x1p-24);
    const double eps2 = eps * eps;
    const double ss = d[0] * d[0] + d[1] * d[1] + d[2] * d[2] + eps2;
    const double want = 1.0 / ss / sqrt(ss);
    int eE = 0;
    uint64_t eM = 0;
    if (eps2 != 0.0) gh::emu::unpack_mid(eps2, eE, eM);
    double got = 0.0;
    n_cases++;
    if (gh::emu::pair_inv_cube_rn(d[0], d[1], d[2], eE, eM, got)) {
      if (bits_of(got) != bits_of(want)) {
        if (n_wrong < 10) printf("WRONG pair d=%.17g %.17g %.17g eps2=%.17g\n", d[0], d[1], d[2], eps2);
        n_wrong++;
      }
    } else {
      n_fallback++;
    }
    // the squared distance itself
    int E1, E2, E;
    uint64_t M1, M2, M;
    int ex, ey, ez;
    uint64_t mx, my, mz;
    gh::emu::unpack_mid(d[0], ex, mx);
    gh::emu::unpack_mid(d[1], ey, my);
    gh::emu::unpack_mid(d[2], ez, mz);
    gh::emu::square_rn(ex, mx, E1, M1);
    gh::emu::square_rn(ey, my, E2, M2);
    gh::emu::add_pos_rn(E1, M1, E2, M2, E, M);
    const double s2 = d[0] * d[0] + d[1] * d[1];
    const double s3 = s2 + d[2] * d[2];
    if ((((uint64_t)(E - 1) << 52) + M) != bits_of(s2)) {
      if (n_wrong < 10) printf("WRONG sum2 %.17g %.17g\n", d[0], d[1]);
      n_wrong++;
    }
    gh::emu::square_rn(ez, mz, E1, M1);
    gh::emu::add_pos_rn(E, M, E1, M1, E2, M2);
    if ((((uint64_t)(E2 - 1) << 52) + M2) != bits_of(s3)) {
      if (n_wrong < 10) printf("WRONG sum3 %.17g %.17g %.17g\n", d[0], d[1], d[2]);
      n_wrong++;
    }
  }
  // s^(-3/2) for the tree walk: within 1 ulp of the correctly rounded value (long double)
  for (long long i = 0; i < per; i++) {
    const uint64_t b = (next_u64() & 0x000FFFFFFFFFFFFFull) | ((uint64_t)(446 + next_u64() % 1179) << 52);
    double s;
    memcpy(&s, &b, 8);
    double got;
    n_cases++;
    if (!gh::emu::rsqrt_cube(s, got)) {
      n_fallback++;
      continue;
    }
    const long double ref = 1.0L / ((long double)s * sqrtl((long double)s));
    const double want = (double)ref;
    const long long ulps = (long long)bits_of(got) - (long long)bits_of(want);
    if (ulps > 1 || ulps < -1) {
      if (n_wrong < 10) printf("WRONG rsqrt_cube s=%.17g got=%.17g want=%.17g\n", s, got, want);
      n_wrong++;
    }
    double r1;  // s^(-1/2)
    if (!gh::emu::rsqrt1(s, r1)) {
      n_fallback++;
      continue;
    }
    const long long u0 = (long long)bits_of(r1) - (long long)bits_of((double)(1.0L / sqrtl((long double)s)));
    if (u0 > 1 || u0 < -1) {
      if (n_wrong < 10) printf("WRONG rsqrt1 s=%.17g\n", s);
      n_wrong++;
    }
    double p1, p3;  // s^-1 and s^(-3/2) together
    if (!gh::emu::rsqrt_powers(s, p1, p3)) {
      n_fallback++;
      continue;
    }
    const long long u1 = (long long)bits_of(p1) - (long long)bits_of((double)(1.0L / (long double)s));
    const long long u3 = (long long)bits_of(p3) - (long long)bits_of(want);
    if (u1 > 1 || u1 < -1 || u3 > 1 || u3 < -1) {
      if (n_wrong < 10) printf("WRONG rsqrt_powers s=%.17g\n", s);
      n_wrong++;
    }
  }
  printf("%lld %lld %lld %lld\n", n_cases, n_wrong, n_fallback, n_out);
  return n_wrong || n_out ? 1 : 0;
}
