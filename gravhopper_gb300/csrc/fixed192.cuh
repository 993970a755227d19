// Exact sums of FP64 values in 192-bit two's-complement fixed point, for the
// tree's monopoles: a cell's mass and first moment are differences of prefix sums
// over the key-ordered particles, so every cell is summed exactly (in any order, with
// the same result) and rounded to FP64 once.  The reference sums each cell's
// particles one at a time in insertion order (gravoct_add_particle,
// gravhopper/_jbgrav.c:396-398, 431-434), rounding after every addition.
//
// A value v = M 2^e (M the 53-bit significand) is held as the integer
// trunc(v / 2^lsb) in three 64-bit words (w[0] least significant).  With every
// |v| < 2^B and at most 2^24 summands, lsb = B - 167 keeps each value below 2^167
// units and every sum below 2^191: nothing overflows, and only the parts of values
// below 2^lsb (2^-167 of the largest) are dropped.
//
// Plain C++ apart from the CUDA qualifiers, so a host build can check it.
#pragma once

#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define FX_HD __host__ __device__ __forceinline__
#else
#define FX_HD inline
#endif

namespace gh {
namespace fx {

constexpr int FX_HEADROOM = 167;  // lsb = B - 167 for |v| < 2^B, up to 2^24 summands

struct I192 {
  uint64_t w[3];
};

FX_HD I192 zero() {
  I192 r;
  r.w[0] = r.w[1] = r.w[2] = 0;
  return r;
}

FX_HD I192 add(const I192& a, const I192& b) {
  I192 r;
#ifdef __CUDA_ARCH__
  asm("add.cc.u64 %0, %3, %6;\n\taddc.cc.u64 %1, %4, %7;\n\taddc.u64 %2, %5, %8;"
      : "=l"(r.w[0]), "=l"(r.w[1]), "=l"(r.w[2])
      : "l"(a.w[0]), "l"(a.w[1]), "l"(a.w[2]), "l"(b.w[0]), "l"(b.w[1]), "l"(b.w[2]));
#else
  r.w[0] = a.w[0] + b.w[0];
  const uint64_t c0 = r.w[0] < a.w[0];
  const uint64_t t1 = a.w[1] + b.w[1];
  const uint64_t c1a = t1 < a.w[1];
  r.w[1] = t1 + c0;
  const uint64_t c1 = c1a | (r.w[1] < t1);
  r.w[2] = a.w[2] + b.w[2] + c1;
#endif
  return r;
}

FX_HD I192 sub(const I192& a, const I192& b) {
  I192 r;
#ifdef __CUDA_ARCH__
  asm("sub.cc.u64 %0, %3, %6;\n\tsubc.cc.u64 %1, %4, %7;\n\tsubc.u64 %2, %5, %8;"
      : "=l"(r.w[0]), "=l"(r.w[1]), "=l"(r.w[2])
      : "l"(a.w[0]), "l"(a.w[1]), "l"(a.w[2]), "l"(b.w[0]), "l"(b.w[1]), "l"(b.w[2]));
#else
  r.w[0] = a.w[0] - b.w[0];
  const uint64_t b0 = a.w[0] < b.w[0];
  const uint64_t t1 = a.w[1] - b.w[1];
  const uint64_t b1a = a.w[1] < b.w[1];
  r.w[1] = t1 - b0;
  const uint64_t b1 = b1a | (t1 < b0);
  r.w[2] = a.w[2] - b.w[2] - b1;
#endif
  return r;
}

FX_HD I192 neg(const I192& a) { return sub(zero(), a); }

FX_HD int clz64(uint64_t x) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}

FX_HD uint64_t bits_of(double v) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(v);
#else
  uint64_t u;
  memcpy(&u, &v, 8);
  return u;
#endif
}

FX_HD double double_of(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double v;
  memcpy(&v, &u, 8);
  return v;
#endif
}

// Smallest B with |v| < 2^B for every finite v of magnitude <= a (a >= 0, finite);
// -1074 for a == 0.
FX_HD int bound_exponent(double a) {
  const uint64_t u = bits_of(a) & 0x7fffffffffffffffull;
  const int E = (int)(u >> 52);
  if (E == 0) return -1074 + 64 - clz64(u);  // subnormal or zero: below 2^-1022
  return E - 1022;                           // a < 2^(E - 1023 + 1)
}

// trunc(v / 2^lsb) as I192 (v finite, |v| < 2^(lsb + 167)).
FX_HD I192 from_double(double v, int lsb) {
  const uint64_t u = bits_of(v);
  const int E = (int)((u >> 52) & 0x7ff);
  I192 r = zero();
  if (E == 0) return r;  // zero or subnormal: below 2^-1022, taken as below 2^lsb
  const uint64_t M = (u & 0x000fffffffffffffull) | 0x0010000000000000ull;
  const int t = (E - 1075) - lsb;  // |v| = M 2^t units
  if (t >= 0) {
    const int q = t >> 6, s = t & 63;  // word offset and bit shift (t <= 114)
    const uint64_t lo = M << s, hi = s ? (M >> (64 - s)) : 0ull;
    if (q == 0) {
      r.w[0] = lo;
      r.w[1] = hi;
    } else if (q == 1) {
      r.w[1] = lo;
      r.w[2] = hi;
    } else {
      r.w[2] = lo;
    }
  } else if (t > -53) {
    r.w[0] = M >> (-t);
  }
  return (u >> 63) ? neg(r) : r;
}

// x 2^k for a significand x < 2^53 and an exponent that keeps the result normal.
FX_HD double scale_pow2(uint64_t x, int k) {
  if (x == 0) return 0.0;
  const int top = 63 - clz64(x);  // x in [2^top, 2^(top+1))
  const uint64_t mant = x << (52 - top);
  const int E = top + k + 1023;
  return double_of(((uint64_t)E << 52) | (mant & 0x000fffffffffffffull));
}

// The I192 value times 2^lsb, rounded to the nearest double (ties to even).  The
// result must be a normal double (it is for cell sums of finite inputs).
FX_HD double to_double(I192 a, int lsb) {
  const bool negative = (a.w[2] >> 63) != 0;
  if (negative) a = neg(a);
  int top;
  if (a.w[2])
    top = 128 + 63 - clz64(a.w[2]);
  else if (a.w[1])
    top = 64 + 63 - clz64(a.w[1]);
  else if (a.w[0])
    top = 63 - clz64(a.w[0]);
  else
    return 0.0;
  double r;
  if (top <= 52) {
    r = scale_pow2(a.w[0], lsb);  // exact
  } else {
    const int sh = top - 52;  // keep bits [sh, top]
    // mant = (a >> sh) truncated to 53 bits; round bit sh-1; sticky bits below
    const int q = sh >> 6, s = sh & 63;
    uint64_t mant;
    if (s == 0)
      mant = a.w[q];
    else
      mant = (a.w[q] >> s) | (q + 1 < 3 ? (a.w[q + 1] << (64 - s)) : 0ull);
    mant &= 0x001fffffffffffffull;
    const int rb = sh - 1;
    const bool round = (a.w[rb >> 6] >> (rb & 63)) & 1ull;
    bool sticky = false;
    for (int w = 0; w < (rb >> 6); w++) sticky = sticky || a.w[w] != 0;
    if ((rb & 63) != 0) sticky = sticky || (a.w[rb >> 6] & ((1ull << (rb & 63)) - 1ull)) != 0;
    int k = sh;
    if (round && (sticky || (mant & 1ull))) {
      mant++;
      if (mant == (1ull << 53)) {
        mant >>= 1;
        k++;
      }
    }
    r = scale_pow2(mant, k + lsb);
  }
  return negative ? -r : r;
}

}  // namespace fx
}  // namespace gh
