// Correctly rounded FP64 reciprocal, square root and quotient on the integer
// pipes, for the softened inverse cube of the FP64 direct sum:
//
//     inv = RN( RN(1/s) / RN(sqrt(s)) )      (gravhopper/_jbgrav.c:166, :330)
//
// GB300 issues FP64 at 1/74 of the FP32 rate, and the two IEEE divisions and the
// square root take more than half of the FP64 instructions of a pair.  Here the
// three results are computed from the double's integer significand instead:
//
//   1. seed y0 ~ 1/sqrt(n) from the FP32 rsqrt approximation, n = N 2^-52 in [1, 4);
//   2. two Newton-Raphson steps for the reciprocal square root in 64-bit fixed
//      point, y' = y + y (1 - n y^2) / 2 (relative error below 2^-59);
//   3. each result from y: sqrt(n) = n y, 1/n = y^2, A/B = A y 2^-52 (one extra
//      residual correction for the quotient, whose divisor is the rounded root);
//   4. the round-to-nearest significand m of each result is confirmed by the sign of
//      exact integer remainders at the rounding boundaries 2m -+ 1 (scaled), the
//      textbook exact-rounding test for division and square root (J.-M. Muller et
//      al., Handbook of Floating-Point Arithmetic, 2nd ed., sections 4.7 and 5.4;
//      P. Markstein, IBM J. Res. Dev. 34 (1990) 111).  Quotients and square roots of
//      53-bit significands never fall on a midpoint, so no tie rule is needed.
//
// The remainders are exact modulo 2^64 and every one is proven smaller than 2^57 in
// magnitude once the first Newton residual passes its range check, so a confirmed
// result is the IEEE result.  When a check fails, or s lies outside [2^-577, 2^602)
// (zero, subnormal, negative, infinite, NaN and the far ranges included), the
// function returns false and the caller takes the native IEEE operations.
#pragma once

#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define GH_EMU_HD __host__ __device__ __forceinline__
#else
#define GH_EMU_HD inline
#endif

#ifndef __CUDA_ARCH__
#include <math.h>
// FP32 reciprocal square root used as the seed by host builds (unit tests); a test
// may define this to perturb the seed and exercise the range checks.
#ifndef GH_EMU_HOST_RSQRT
#define GH_EMU_HOST_RSQRT(x) (1.0f / sqrtf(x))
#endif
#endif

namespace gh {
namespace emu {

GH_EMU_HD uint64_t umulhi(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

GH_EMU_HD uint64_t dbits(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  memcpy(&u, &x, 8);
  return u;
#endif
}

GH_EMU_HD double bitsd(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, 8);
  return x;
#endif
}

GH_EMU_HD float bitsf(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float x;
  memcpy(&x, &u, 4);
  return x;
#endif
}

GH_EMU_HD uint32_t fbits(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  uint32_t u;
  memcpy(&u, &x, 4);
  return u;
#endif
}

GH_EMU_HD float rsqrt_seed(float x) {
#ifdef __CUDA_ARCH__
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  return GH_EMU_HOST_RSQRT(x);
#endif
}

// Reciprocal square root in fixed point: for s = M 2^(E - 1075) (M in [2^52, 2^53))
// writes s = N 2^p with p even and N in [2^52, 2^54), and Y2 = 2^63 / sqrt(n),
// n = N 2^-52, to a relative error below 2^-59; false when the seed check fails.
GH_EMU_HD bool rsqrt_fixed(int E, uint64_t M, int& odd, uint64_t& N, int& p, uint64_t& Y2) {
  odd = ~E & 1;  // s = M 2^(E - 1075); E - 1075 is odd when E is even
  N = M << odd;
  p = E - 1075 - odd;

  // seed: y0 ~ 1/sqrt(n), n = N 2^-52, as Y0 = y0 2^30
  const float nf = bitsf(0x3F800000u + ((uint32_t)odd << 23) + ((uint32_t)(M >> 29) & 0x7FFFFFu));
  const uint32_t rb = fbits(rsqrt_seed(nf));
  const uint32_t ex = (rb >> 23) & 0xFFu;
  if (ex - 121u > 6u) return false;  // y0 in [2^-6, 2)
  const int32_t Y0 = (int32_t)(((rb & 0x7FFFFFu) | 0x800000u) << (ex - 120u));

  // Newton step 1: h = 1 - n y0^2 as H = h 2^60; Y1 = y1 2^63
  const uint64_t Y0sq = (uint64_t)((int64_t)Y0 * Y0);  // y0^2 2^60 <= 2^60
  const int64_t H = (int64_t)((1ull << 60) - umulhi(N << 10, Y0sq << 2));
  if ((uint64_t)(H + (1ll << 41)) >= (1ull << 42)) return false;  // |h| < 2^-19
  uint64_t Y1 = ((uint64_t)Y0 << 33) + (uint64_t)(((int64_t)Y0 * (int32_t)(H >> 10)) >> 18);
  if (Y1 >= (1ull << 63)) Y1 = (1ull << 63) - 1;

  // Newton step 2: h2 = 1 - n y1^2 as H2 = h2 2^62 (|h2| < 2^-37, fits 32 bits)
  const uint64_t Y1sq = umulhi(Y1, Y1);  // y1^2 2^62 < 2^62
  const int32_t H2 = (int32_t)(uint32_t)((1ull << 62) - umulhi(N << 10, Y1sq << 2));
  Y2 = Y1 + (uint64_t)(((int64_t)(int32_t)(Y1 >> 32) * H2) >> 31);
  if (Y2 >= (1ull << 63)) Y2 = (1ull << 63) - 1;
  return true;
}

// RN(RN(1/s) / RN(sqrt(s))) into `out` for s = M 2^(E - 1075) with M in
// [2^52, 2^53) and 446 <= E <= 1624 (the caller checks the range); false when a
// check fails (then `out` is untouched).
GH_EMU_HD bool inv_cube_core(int E, uint64_t M, double& out) {
  int odd, p;
  uint64_t N, Y2;
  if (!rsqrt_fixed(E, M, odd, N, p, Y2)) return false;

  // square root: sqrt(s) = B 2^(p/2 - 26), B = RN(sqrt(X) / 2), X = N 2^54, i.e.
  // c = 2B - 1 <= sqrt(X) < c + 2
  uint64_t B = (umulhi(N << 2, Y2) + 1) >> 1;
  {
    const uint64_t c = 2 * B - 1;
    const int64_t R = (int64_t)((N << 54) - c * c);  // X - c^2
    if (R < 0) {
      if (R + (int64_t)(4 * c) - 4 < 0) return false;
      B--;
    } else if (R >= (int64_t)(4 * c + 4)) {
      if (R >= (int64_t)(8 * c + 16)) return false;
      B++;
    }
  }

  // reciprocal: 1/s = A 2^(970 - E), A = RN(2^105 / M) in [2^52, 2^53], i.e.
  // c = 2A - 1 <= 2^106 / M < c + 2
  uint64_t A = ((umulhi(Y2, Y2) >> (8 - odd)) + 1) >> 1;
  {
    const uint64_t c = 2 * A - 1;
    const int64_t R = (int64_t)(0 - c * M);  // 2^106 - c M
    if (R < 0) {
      if (R + (int64_t)(2 * M) < 0) return false;
      A--;
    } else if (R >= (int64_t)(2 * M)) {
      if (R >= (int64_t)(4 * M)) return false;
      A++;
    }
  }

  // quotient: Qx = A 2^54 / B in (2^53, 2^55]; inv = RN(Qx 2^-sh) 2^(sh - 54 + a - b)
  const uint64_t A54 = A << 54;  // A 2^54 mod 2^64
  uint64_t Q = umulhi(A << 3, Y2);  // A 2^54 / (sqrt(n) 2^52): within 6 of Qx
  {
    const int64_t R0 = (int64_t)(A54 - Q * B);  // A 2^54 - Q B, |.| < 2^56
    Q += (uint64_t)(((int64_t)(int32_t)(R0 >> 26) * (int64_t)(int32_t)(Y2 >> 32)) >> 57);  // + R0 / B
  }
  const int sh = A >= B ? 2 : 1;
  uint64_t m = (Q + (1ull << (sh - 1))) >> sh;
  {
    const uint64_t c = (m << sh) - (1ull << (sh - 1));  // c <= Qx < c + 2^sh
    const int64_t R = (int64_t)(A54 - c * B);
    const int64_t W = (int64_t)(B << sh);
    if (R < 0) {
      if (R + W < 0) return false;
      m--;
    } else if (R >= W) {
      if (R >= 2 * W) return false;
      m++;
    }
  }
  const int k = sh - 54 + (970 - E) - (p / 2 - 26);
  out = bitsd(((uint64_t)(k + 1074) << 52) + m);  // m = 2^53 carries into the exponent
  return true;
}

// RN(RN(1/s) / RN(sqrt(s))) into `out`; false when s is out of range or a check
// fails (then `out` is untouched).
GH_EMU_HD bool inv_cube_rn(double s, double& out) {
  const uint64_t bits = dbits(s);
  const int E = (int)(bits >> 52);  // biased exponent; the sign bit makes it >= 2048
  if ((unsigned)(E - 446) > 1178u) return false;  // 2^-577 <= s < 2^602
  return inv_cube_core(E, (bits & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull, out);
}

// s^(-3/2) within about half an ulp (not correctly rounded: the tree walk's FP64
// interactions, which sum in their own order anyway); false outside [2^-577, 2^602).
GH_EMU_HD bool rsqrt_cube(double s, double& out) {
  const uint64_t bits = dbits(s);
  const int E = (int)(bits >> 52);
  if ((unsigned)(E - 446) > 1178u) return false;
  int odd, p;
  uint64_t N, Y2;
  if (!rsqrt_fixed(E, (bits & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull, odd, N, p, Y2)) return false;
  // y^3 = Y3 2^-62, y = 1/sqrt(n) in (1/2, 1]
  const uint64_t Y3 = umulhi(umulhi(Y2, Y2) << 1, Y2);
#ifdef __CUDA_ARCH__
  const int lz = __clzll((long long)Y3);
#else
  const int lz = __builtin_clzll(Y3);
#endif
  const uint64_t T = Y3 << lz;  // in [2^63, 2^64)
  const uint64_t m = (T >> 11) + ((T >> 10) & 1);  // in [2^52, 2^53]
  // s^(-3/2) = y^3 2^(-3 (26 + p/2)) = m 2^(11 - 62 - lz - 78 - 3p/2)
  const int k = -129 - lz - 3 * (p / 2);
  out = bitsd(((uint64_t)(k + 1074) << 52) + m);
  return true;
}

// s^(-1/2) within about half an ulp (the FP64 potential); false outside
// [2^-577, 2^602).
GH_EMU_HD bool rsqrt1(double s, double& out) {
  const uint64_t bits = dbits(s);
  const int E = (int)(bits >> 52);
  if ((unsigned)(E - 446) > 1178u) return false;
  int odd, p;
  uint64_t N, Y2;
  if (!rsqrt_fixed(E, (bits & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull, odd, N, p, Y2)) return false;
#ifdef __CUDA_ARCH__
  const int lz = __clzll((long long)Y2);
#else
  const int lz = __builtin_clzll(Y2);
#endif
  const uint64_t T = Y2 << lz;  // y 2^63 << lz, in [2^63, 2^64)
  const uint64_t m = (T >> 11) + ((T >> 10) & 1);
  // s^(-1/2) = y 2^(-26 - p/2) = m 2^(11 - 63 - lz - 26 - p/2)
  out = bitsd(((uint64_t)(-78 - lz - p / 2 + 1074) << 52) + m);
  return true;
}

// s^(-1) and s^(-3/2), each within about half an ulp (the FP64 adjoint's pair factors);
// false outside [2^-577, 2^602).
GH_EMU_HD bool rsqrt_powers(double s, double& inv1, double& inv3) {
  const uint64_t bits = dbits(s);
  const int E = (int)(bits >> 52);
  if ((unsigned)(E - 446) > 1178u) return false;
  int odd, p;
  uint64_t N, Y2;
  if (!rsqrt_fixed(E, (bits & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull, odd, N, p, Y2)) return false;
  const uint64_t Y2sq = umulhi(Y2, Y2);         // y^2 2^62, y = 1/sqrt(n) in (1/2, 1]
  const uint64_t Y3 = umulhi(Y2sq << 1, Y2);    // y^3 2^62
#ifdef __CUDA_ARCH__
  const int l2 = __clzll((long long)Y2sq), l3 = __clzll((long long)Y3);
#else
  const int l2 = __builtin_clzll(Y2sq), l3 = __builtin_clzll(Y3);
#endif
  const uint64_t T2 = Y2sq << l2, T3 = Y3 << l3;  // in [2^63, 2^64)
  const uint64_t m2 = (T2 >> 11) + ((T2 >> 10) & 1), m3 = (T3 >> 11) + ((T3 >> 10) & 1);
  // s^-1 = y^2 2^(-52 - p) = m2 2^(11 - 62 - l2 - 52 - p); s^(-3/2) as in rsqrt_cube
  inv1 = bitsd(((uint64_t)(-103 - l2 - p + 1074) << 52) + m2);
  inv3 = bitsd(((uint64_t)(-129 - l3 - 3 * (p / 2) + 1074) << 52) + m3);
  return true;
}

// ---------------------------------------------------------------------------
// The softened squared distance s = RN(RN(RN(dx^2 + dy^2) + dz^2) + eps^2) with
// every product and sum rounded as the FPU does (round to nearest even).  All terms
// are positive, so a sum needs at most a one-bit renormalisation.  Values are
// (E, M): M in [2^52, 2^53), value M 2^(E - 1075), E the biased exponent.

// RN(d^2) of a normal d = D 2^(Ed - 1075); D^2 is formed exactly from 32-bit halves.
GH_EMU_HD void square_rn(int Ed, uint64_t D, int& E, uint64_t& M) {
  const uint32_t h = (uint32_t)(D >> 32), l = (uint32_t)D;  // h < 2^21
  const uint64_t ll = (uint64_t)l * l;
  const uint64_t x = (uint64_t)(2 * h) * l;  // < 2^54
  const uint64_t lo = ll + (x << 32);
  const uint64_t hi = (uint64_t)h * h + (x >> 32) + (lo < ll);  // D^2 = hi 2^64 + lo, hi in [2^40, 2^42)
  const int big = (int)(hi >> 41);  // D^2 >= 2^105
  uint64_t m;
  uint64_t rest;  // the bits below m, left-aligned
  if (big) {
    m = (hi << 11) | (lo >> 53);
    rest = lo << 11;
  } else {
    m = (hi << 12) | (lo >> 52);
    rest = lo << 12;
  }
  m += (rest >> 63) & (uint64_t)(((rest << 1) != 0) | (m & 1));
  E = 2 * Ed - 1023 + big;  // D^2 2^(2 Ed - 2150) = m 2^(52 + big + 2 Ed - 2150)
  const int carry = (int)(m >> 53);
  M = m >> carry;
  E += carry;
}

// RN(a + b) of two positive normals.
GH_EMU_HD void add_pos_rn(int Ea, uint64_t Ma, int Eb, uint64_t Mb, int& E, uint64_t& M) {
  if (Ea < Eb) {
    const int te = Ea;
    Ea = Eb;
    Eb = te;
    const uint64_t tm = Ma;
    Ma = Mb;
    Mb = tm;
  }
  const int d = Ea - Eb;
  if (d >= 54) {  // b < ulp(a) / 2
    E = Ea;
    M = Ma;
    return;
  }
  const uint64_t bs = Mb << 10;
  const uint64_t S = (Ma << 10) + (bs >> d);  // < 2^64
  const bool lost = (bs & ((1ull << d) - 1)) != 0;
  const int big = (int)(S >> 63);
  uint64_t m, rest;
  if (big) {
    m = S >> 11;
    rest = S << 53;
  } else {
    m = S >> 10;
    rest = S << 54;
  }
  m += (rest >> 63) & (uint64_t)(((rest << 1) != 0) | lost | (m & 1));
  const int carry = (int)(m >> 53);
  M = m >> carry;
  E = Ea + big + carry;
}

// Unpacks a double whose magnitude lies in [2^-250, 2^251) (zero excluded) into
// (E, |significand|); false otherwise.
GH_EMU_HD bool unpack_mid(double d, int& E, uint64_t& M) {
  const uint64_t b = dbits(d);
  E = (int)((b >> 52) & 0x7FF);
  M = (b & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull;
  return (unsigned)(E - 773) <= 500u;
}

// Unpacks the squared softening for pair_inv_cube_rn: E = 0 for eps2 = 0; false
// when eps2 lies outside [2^-500, 2^502) (then the caller uses the native path).
GH_EMU_HD bool unpack_eps2(double eps2, int& E, uint64_t& M) {
  const uint64_t b = dbits(eps2);
  E = (int)(b >> 52);
  M = (b & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull;
  if (b == 0) {
    E = 0;
    return true;
  }
  return (unsigned)(E - 523) <= 1001u;
}

// inv = RN(RN(1/s) / RN(sqrt(s))) with s = RN(RN(RN(dx^2 + dy^2) + dz^2) + eps2),
// the pair factor of gravhopper/_jbgrav.c:159-166.  eps2 is given unpacked
// (eps2_E = 0 for eps2 = 0; otherwise 2^-500 <= eps2 < 2^502).  False when a
// component is zero or outside [2^-250, 2^251), or a check fails.
GH_EMU_HD bool pair_inv_cube_rn(double dx, double dy, double dz, int eps2_E, uint64_t eps2_M, double& out) {
  int ex, ey, ez;
  uint64_t mx, my, mz;
  const bool ok = unpack_mid(dx, ex, mx) & unpack_mid(dy, ey, my) & unpack_mid(dz, ez, mz);
  if (!ok) return false;
  int E1, E2, E;
  uint64_t M1, M2, M;
  square_rn(ex, mx, E1, M1);
  square_rn(ey, my, E2, M2);
  add_pos_rn(E1, M1, E2, M2, E, M);
  square_rn(ez, mz, E1, M1);
  add_pos_rn(E, M, E1, M1, E2, M2);
  if (eps2_E) {
    add_pos_rn(E2, M2, eps2_E, eps2_M, E, M);
  } else {
    E = E2;
    M = M2;
  }
  return inv_cube_core(E, M, out);
}

}  // namespace emu
}  // namespace gh
