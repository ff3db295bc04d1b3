// Correctly rounded FP64 division with few FP64 instructions, and the exact
// shortcut of the limiters' 1e-30 + x.  GB300 issues FP64 at 1/64 of the FP32
// rate, so the exact schemes are bound by their FP64 instruction count; a
// quotient here costs six FP64 instructions (a seeded reciprocal refined once,
// the Markstein-corrected quotient and one residual for its proof), and a lane
// whose result cannot be proven correctly rounded takes the division
// instruction, so every function returns exactly the IEEE result.
#pragma once
#include <math.h>

namespace mom5 {
namespace fp64 {

#define DEVI __device__ __forceinline__

// Bit pattern of a double and back through an opaque move.  With a plain bit
// cast the compiler rewrites some integer tests as FP64 instructions (a masked
// sign bit becomes an FP64 absolute value); through the move they stay on the
// integer pipe.
DEVI long long bits_of(double x) {
  long long b;
  asm("mov.b64 %0, %1;" : "=l"(b) : "d"(x));
  return b;
}
DEVI double double_of(long long b) {
  double x;
  asm("mov.b64 %0, %1;" : "=d"(x) : "l"(b));
  return x;
}

// FP64 -> FP32 by truncation of the significand, on the integer pipe.  Below
// the FP32 normal range the result is +-0, above it +-Inf (NaN too); only the
// reciprocal seed uses it, and a seed from either is rejected downstream.
DEVI float f32_trunc(double x) {
  unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  unsigned sign = hi & 0x80000000u, mag = hi & 0x7fffffffu;
  if (mag < (897u << 20)) return __uint_as_float(sign);
  if (mag >= (1151u << 20)) return __uint_as_float(sign | 0x7f800000u);
  return __uint_as_float(sign | ((mag - (896u << 20)) << 3) | (lo >> 29));
}
// FP32 -> FP64, exact for normal and infinite values (FP32 subnormals read as
// +-0), on the integer pipe.
DEVI double f64_widen(float f) {
  unsigned b = __float_as_uint(f);
  unsigned sign = b & 0x80000000u, mag = b & 0x7fffffffu;
  if (mag < 0x00800000u) return __hiloint2double((int)sign, 0);
  if (mag >= 0x7f800000u) return __hiloint2double((int)(sign | 0x7ff00000u), 0);
  return __hiloint2double((int)(sign | ((mag >> 3) + (896u << 20))), (int)(mag << 29));
}

// Approximate reciprocal of b: the FP32 hardware reciprocal (rcp.approx, at most
// one FP32 ulp of error) of b truncated to FP32, widened and refined by one
// Newton-Raphson step in FP64, y1 = y0 + y0*(1 - b*y0).  The seed's relative
// error is below 2^-22, so y1's is below about 2^-43 for b in the FP32 normal
// range; outside it the seed is 0 or Inf and y1 is NaN.
DEVI double recip_seed(double b) {
  float yf;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(yf) : "f"(f32_trunc(b)));
  double y0 = f64_widen(yf);
  return fma(y0, fma(-b, y0, 1.0), y0);
}

// a / b from an approximate reciprocal y of b (Markstein's correction:
// P. Markstein, IBM J. Res. Dev. 34(1), 1990; J.-M. Muller et al., Handbook of
// Floating-Point Arithmetic, ch. 5): q = RN(a*y), r = RN(a - b*q) (one FMA),
// q1 = RN(q + r*y).  For y within 2^-40 of 1/b, q1 is within 2^-80 of a/b
// before its rounding.  It is then proven correctly rounded at run time: with
// r1 = a - b*q1 from one more FMA (exact when q1 is within an ulp of a/b),
// q1 = RN(a/b) when |r1| < |b|*ulp(q1)/2 and q1 is normal and not a power of
// two, or when r1 is zero (q1 is the exact quotient).  A lane that cannot prove
// it (a tie, a binade edge, extreme exponents, an unusable y) takes the
// division instruction, so the result always equals a / b.
DEVI double div_recip(double a, double b, double y) {
  const long long kAbsMask = 0x7fffffffffffffffLL, kMant = 0x000fffffffffffffLL;
  const long long ba = bits_of(a), bbits = bits_of(b);
  long long ab = ba & kAbsMask, bb = bbits & kAbsMask;
  int ea = (int)(ab >> 52), eb = (int)(bb >> 52);
  double q1;
  bool ok;
  if (ab == 0) {  // 0 / b = +-0 for finite non-zero b
    q1 = double_of((ba ^ bbits) & (long long)0x8000000000000000ULL);
    ok = eb >= 1 && eb <= 2046;
  } else {
    double q = a * y;
    double r = fma(-q, b, a);
    q1 = fma(r, y, q);
    double r1 = fma(-q1, b, a);
    long long qb = bits_of(q1) & kAbsMask, rb = bits_of(r1) & kAbsMask;
    int eq = (int)(qb >> 52);
    int et = eb + eq - 1076;  // exponent of |b| * ulp(q1) / 2
    ok = ea >= 64 && ea <= 1980 && eb >= 64 && eb <= 1980 && eq >= 64 && eq <= 1980 && et >= 1 && et <= 2046;
    long long thr = (bb & kMant) | ((long long)et << 52);
    ok = ok && ((qb & kMant) != 0 ? rb < thr : rb == 0);
  }
  if (!__all_sync(__activemask(), ok)) {
    if (!ok) q1 = a / b;
  }
  return q1;
}

// a / b for a divisor used once.
DEVI double div_seeded(double a, double b) { return div_recip(a, b, recip_seed(b)); }

// RN(1e-30 + x) without an FP64 addition where that is exact by inspection:
// +-0 gives the constant 1e-30, and for |x| >= 2^-45 (biased exponent >= 978)
// the sum rounds back to x (1e-30 is below half an ulp of x, also of the
// binade under x when x is a negative power of two).  Tiny non-zero x, Inf and
// NaN take the addition (decided per warp; the addition is volatile so that it
// is not hoisted above the vote and issued for every lane).
DEVI double add_1em30(double x) {
  long long b = bits_of(x);
  unsigned e = (unsigned)((unsigned long long)b >> 52) & 0x7ffu;
  bool zero = (b << 1) == 0;
  bool keep = e >= 978u && e <= 2046u;
  bool fast = zero || keep;
  double r = zero ? 1.0e-30 : x;
  if (__all_sync(__activemask(), fast)) return r;
  if (!fast) asm volatile("add.rn.f64 %0, %1, %2;" : "=d"(r) : "d"(1.0e-30), "d"(x));
  return r;
}

}  // namespace fp64
}  // namespace mom5
