// IEEE 754 binary64 multiply and add, round to nearest / ties to even, in
// 64-bit integer arithmetic.  GB300 issues FP64 at 2 lanes per clock per SM
// (one warp instruction per ~64 cycles on each scheduler) while its integer
// and FP32 pipes idle in the FP64-bound S-map solve; these routines move part
// of that arithmetic to those pipes.  They return exactly the IEEE result,
// the same bits as __dmul_rn / __dadd_rn.
//
// Method (the textbook one; e.g. Muller et al., Handbook of Floating-Point
// Arithmetic, ch. 7-8):
//   multiply: the 53-bit significands' exact 106-bit product, normalised by
//     at most one bit, rounded on its guard bit and the OR of the rest;
//   add: significands widened to 63 bits (10 guard bits), the smaller one
//     aligned with the bits shifted out ORed into its lowest bit, added or
//     subtracted, normalised (at most one bit of cancellation when the
//     exponents differ by 2 or more; exact otherwise), rounded.
// The fast path takes normal operands whose result is normal and non-zero;
// zeros, subnormals, infinities, NaNs and results outside the normal range
// go to the hardware instruction.
#pragma once

namespace fedm {

namespace soft {
constexpr unsigned long long SIGN = 0x8000000000000000ULL;
constexpr unsigned long long FRAC = 0x000FFFFFFFFFFFFFULL;
constexpr unsigned long long HIDDEN = 0x0010000000000000ULL;
}  // namespace soft

__device__ __forceinline__ double soft_mul(double a, double b)
{
  using namespace soft;
  const unsigned long long ua = (unsigned long long)__double_as_longlong(a);
  const unsigned long long ub = (unsigned long long)__double_as_longlong(b);
  const int ea = (int)((ua >> 52) & 0x7FF), eb = (int)((ub >> 52) & 0x7FF);
  if (ea == 0 || eb == 0 || ea == 0x7FF || eb == 0x7FF)
    return __dmul_rn(a, b);
  const unsigned long long ma = (ua & FRAC) | HIDDEN, mb = (ub & FRAC) | HIDDEN;
  const unsigned long long lo = ma * mb, hi = __umul64hi(ma, mb);
  // product in [2^104, 2^106)
  int e = ea + eb - 1023;
  unsigned long long m;
  bool round, sticky;
  if (hi >> 41) {  // >= 2^105: significand = bits 105..53
    m = (hi << 11) | (lo >> 53);
    round = (lo >> 52) & 1;
    sticky = (lo & ((1ULL << 52) - 1)) != 0;
    e += 1;
  } else {  // significand = bits 104..52
    m = (hi << 12) | (lo >> 52);
    round = (lo >> 51) & 1;
    sticky = (lo & ((1ULL << 51) - 1)) != 0;
  }
  m += (round && (sticky || (m & 1))) ? 1 : 0;
  if (m >> 53) {  // rounded up to 2^53
    m >>= 1;
    e += 1;
  }
  if (e <= 0 || e >= 0x7FF)
    return __dmul_rn(a, b);
  return __longlong_as_double((long long)(((ua ^ ub) & SIGN) | ((unsigned long long)e << 52) | (m & FRAC)));
}

__device__ __forceinline__ double soft_add(double a, double b)
{
  using namespace soft;
  unsigned long long ua = (unsigned long long)__double_as_longlong(a);
  unsigned long long ub = (unsigned long long)__double_as_longlong(b);
  int ea = (int)((ua >> 52) & 0x7FF), eb = (int)((ub >> 52) & 0x7FF);
  if (ea == 0 || eb == 0 || ea == 0x7FF || eb == 0x7FF)
    return __dadd_rn(a, b);
  if ((ua & ~SIGN) < (ub & ~SIGN)) {  // |a| >= |b| from here on
    const unsigned long long t = ua;
    ua = ub;
    ub = t;
    const int te = ea;
    ea = eb;
    eb = te;
  }
  const int d = ea - eb;
  const unsigned long long ma = ((ua & FRAC) | HIDDEN) << 10;  // leading one at bit 62
  unsigned long long mb = ((ub & FRAC) | HIDDEN) << 10;
  if (d >= 64)
    mb = 1;  // entirely below the guard bits: sticky only
  else if (d > 0)
    mb = (mb >> d) | ((mb << (64 - d)) != 0 ? 1ULL : 0ULL);
  int e = ea;
  unsigned long long m;
  if (((ua ^ ub) & SIGN) == 0) {
    m = ma + mb;
    if (m >> 63) {
      m = (m >> 1) | (m & 1);
      e += 1;
    }
  } else {
    m = ma - mb;
    if (m == 0)
      return __dadd_rn(a, b);  // exact zero: +0
    const int lz = __clzll((long long)m) - 1;
    m <<= lz;
    e -= lz;
  }
  // significand = bits 62..10, round bit 9, sticky bits 8..0
  unsigned long long mant = m >> 10;
  const bool round = (m >> 9) & 1, sticky = (m & 0x1FF) != 0;
  mant += (round && (sticky || (mant & 1))) ? 1 : 0;
  if (mant >> 53) {
    mant >>= 1;
    e += 1;
  }
  if (e <= 0 || e >= 0x7FF)
    return __dadd_rn(a, b);
  return __longlong_as_double((long long)((ua & SIGN) | ((unsigned long long)e << 52) | (mant & FRAC)));
}

}  // namespace fedm
