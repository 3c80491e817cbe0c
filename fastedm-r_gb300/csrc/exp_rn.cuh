// exp(x) built only from IEEE round-to-nearest operations, so every IEEE
// device or host that evaluates the same sequence returns the same bits.
// Method: Cody-Waite argument reduction x = k*ln2 + r with ln2 split into a
// 32-significant-bit head (k*head is exact) and a tail, |r| <= ln2/2; e^r by
// its degree-13 Taylor polynomial in Horner form with fused multiply-adds
// (truncation below 5e-18 relative); scaling by 2^k from exponent bits.
// Constants are ln 2, 1/ln 2 and 1/i! rounded to double.
#pragma once

namespace fedm {

__device__ __forceinline__ double pow2i(int k)
{
  return __longlong_as_double((long long)(k + 1023) << 52);
}

__device__ inline double exp_rn(double x)
{
  if (!(x == x))
    return x;
  if (x > 709.782712893384)
    return __longlong_as_double(0x7ff0000000000000LL);
  if (x < -745.1332191019412)
    return 0.0;
  const double k = rint(__dmul_rn(x, 0x1.71547652b82fep+0));
  double r = __fma_rn(-k, 0x1.62e42ff000000p-1, x);
  r = __fma_rn(-k, -0x1.718432a1b0e26p-35, r);
  double p = 0x1.6124613a86d09p-33;
  p = __fma_rn(p, r, 0x1.1eed8eff8d898p-29);
  p = __fma_rn(p, r, 0x1.ae64567f544e4p-26);
  p = __fma_rn(p, r, 0x1.27e4fb7789f5cp-22);
  p = __fma_rn(p, r, 0x1.71de3a556c734p-19);
  p = __fma_rn(p, r, 0x1.a01a01a01a01ap-16);
  p = __fma_rn(p, r, 0x1.a01a01a01a01ap-13);
  p = __fma_rn(p, r, 0x1.6c16c16c16c17p-10);
  p = __fma_rn(p, r, 0x1.1111111111111p-7);
  p = __fma_rn(p, r, 0x1.5555555555555p-5);
  p = __fma_rn(p, r, 0x1.5555555555555p-3);
  p = __fma_rn(p, r, 0.5);
  p = __fma_rn(p, r, 1.0);
  p = __fma_rn(p, r, 1.0);
  int ki = (int)k;
  if (ki < -1021) {
    p = __dmul_rn(p, pow2i(-600));
    ki += 600;
  } else if (ki > 1023) {
    p = __dmul_rn(p, 2.0);
    ki -= 1;
  }
  return __dmul_rn(p, pow2i(ki));
}

} // namespace fedm
