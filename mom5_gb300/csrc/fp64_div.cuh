// Correctly rounded FP64 division with few FP64 instructions, and the exact
// shortcut of the limiters' 1e-30 + x.  GB300 issues FP64 at 1/64 of the FP32
// rate, so the exact schemes are bound by their FP64 instruction count; a
// quotient here costs four FP64 instructions (the product with a reciprocal
// built in FP32, its Markstein correction and one residual for its proof), and
// a lane whose result cannot be proven correctly rounded takes the division
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
// hi + lo as a double, on the integer pipe, for normal FP32 values with
// |lo| < 2^-20 |hi|: the significands are aligned on hi's exponent and added as
// integers (exact when lo's lowest bit is not below hi's 53-bit grid, else lo
// is truncated to it; one bit may be lost when the sum carries into the next
// binade).  Other inputs give a finite or NaN value of no use, which the
// division's proof then rejects.
DEVI double join_f32(float hi, float lo) {
  const unsigned bh = __float_as_uint(hi), bl = __float_as_uint(lo);
  const int eh = (int)((bh >> 23) & 0xffu), el = (int)((bl >> 23) & 0xffu);
  long long m = (long long)((bh & 0x7fffffu) | 0x800000u) << 29;  // hi's significand, bit 52 set
  const long long ml = el ? (long long)((bl & 0x7fffffu) | 0x800000u) : 0;
  const int sh = eh - el - 29;  // lo's significand is ml * 2^-sh units of m's lowest bit
  long long al = 0;
  if (sh >= 0 && sh < 40) al = ml >> sh;
  else if (sh < 0 && sh > -30) al = ml << -sh;
  m = ((bh ^ bl) & 0x80000000u) ? m - al : m + al;
  int e = eh + 896;  // FP64 biased exponent of hi
  if (m >= (1LL << 53)) {
    m >>= 1;
    ++e;
  } else if (m < (1LL << 52)) {
    m <<= 1;
    --e;
  }
  return double_of(((long long)(bh & 0x80000000u) << 32) | ((long long)e << 52) | (m & 0x000fffffffffffffLL));
}

// Approximate reciprocal of b with no FP64 instruction.  b is split into FP32
// terms bh + bl (its truncation to FP32 and the next 24 bits of the remaining
// significand); y0 = rcp.approx(bh) (at most one FP32 ulp of error); the
// residual e = 1 - bh*y0 - bl*y0 by two FP32 FMAs (rounding errors near 2^-46);
// and y = y0 + y0*e joined into a double on the integer pipe, the first-order
// Newton-Raphson correction carried in FP32.  |y*b - 1| is then about
// (2^-22)^2 plus the FP32 roundings, below 2^-42, for 2^-103 <= |b| < 2^127
// (other b give an unusable y, which the division's proof rejects).
DEVI double recip_seed(double b) {
  const unsigned hi = (unsigned)__double2hiint(b), lo = (unsigned)__double2loint(b);
  const unsigned sign = hi & 0x80000000u, E = (hi & 0x7fffffffu) >> 20;
  const float bh = f32_trunc(b);
  // remaining 29 significand bits: (lo & 0x1fffffff) * 2^-29 * 2^(E - 1046), sign of b
  const float low = __uint2float_rz(lo & 0x1fffffffu) * 0x1p-29f;
  const float scale = (E >= 920u && E <= 1150u) ? __uint_as_float((E - 919u) << 23) : 0.0f;
  const float bl = __uint_as_float(__float_as_uint(low * scale) | sign);
  float y0;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y0) : "f"(bh));
  float e = fmaf(-bh, y0, 1.0f);
  e = fmaf(-bl, y0, e);
  return join_f32(y0, y0 * e);
}

// a / b from an approximate reciprocal y of b (Markstein's correction:
// P. Markstein, IBM J. Res. Dev. 34(1), 1990; J.-M. Muller et al., Handbook of
// Floating-Point Arithmetic, ch. 5): q = RN(a*y), r = RN(a - b*q) (one FMA),
// q1 = RN(q + r*y).  For y within 2^-40 of 1/b (relative), q1 is within about
// 2^-80 of a/b before its rounding.  It is then proven correctly rounded at run time: with
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

// Two-term reciprocal yh + yl of b for a divisor shared by many quotients:
// yh = recip_seed(b) and yl = yh*(1 - b*yh) (two FP64 instructions), so that
// yh + yl is within about 2^-84 of 1/b (relative; the square of yh's error)
// where recip_seed is usable, else unusable.
DEVI void recip_pair(double b, double& yh, double& yl) {
  yh = recip_seed(b);
  yl = yh * fma(-b, yh, 1.0);
}

// a / b from a two-term reciprocal (recip_pair): q1 = RN(a*yh + RN(a*yl))
// (N. Brisebarre, J.-M. Muller, S. K. Raina, IEEE Trans. Computers 53(8),
// 2004) is within about 2^-84 of a/b before its rounding; it is proven
// correctly rounded as in div_recip, else the lane takes the division
// instruction.  Three FP64 instructions.
DEVI double div_pair(double a, double b, double yh, double yl) {
  const long long kAbsMask = 0x7fffffffffffffffLL, kMant = 0x000fffffffffffffLL;
  const long long ba = bits_of(a), bbits = bits_of(b);
  long long ab = ba & kAbsMask, bb = bbits & kAbsMask;
  int ea = (int)(ab >> 52), eb = (int)(bb >> 52);
  double q1;
  bool ok;
  if (ab == 0) {
    q1 = double_of((ba ^ bbits) & (long long)0x8000000000000000ULL);
    ok = eb >= 1 && eb <= 2046;
  } else {
    q1 = fma(a, yh, a * yl);
    double r1 = fma(-q1, b, a);
    long long qb = bits_of(q1) & kAbsMask, rb = bits_of(r1) & kAbsMask;
    int eq = (int)(qb >> 52);
    int et = eb + eq - 1076;
    ok = ea >= 64 && ea <= 1980 && eb >= 64 && eb <= 1980 && eq >= 64 && eq <= 1980 && et >= 1 && et <= 2046;
    long long thr = (bb & kMant) | ((long long)et << 52);
    ok = ok && ((qb & kMant) != 0 ? rb < thr : rb == 0);
  }
  if (!__all_sync(__activemask(), ok)) {
    if (!ok) q1 = a / b;
  }
  return q1;
}

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
