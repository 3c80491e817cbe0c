// Host check of soft_f64.cuh: its integer multiply and add against the host's
// IEEE binary64 arithmetic (round to nearest even) on random operands drawn
// to stress alignment, cancellation, carries, ties and the range limits.
// Built and run by tests/test_soft_f64_cpu.py; prints "mismatches N".
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#define __device__
#define __forceinline__ inline
static inline long long __double_as_longlong(double x) { long long v; std::memcpy(&v, &x, 8); return v; }
static inline double __longlong_as_double(long long v) { double x; std::memcpy(&x, &v, 8); return x; }
static inline unsigned long long __umul64hi(unsigned long long a, unsigned long long b)
{
  return (unsigned long long)(((unsigned __int128)a * b) >> 64);
}
static inline int __clzll(long long x) { return x == 0 ? 64 : __builtin_clzll((unsigned long long)x); }
static double __dmul_rn(double a, double b) { volatile double r = a * b; return r; }
static double __dadd_rn(double a, double b) { volatile double r = a + b; return r; }

#include "../../fastedm-r_gb300/csrc/soft_f64.cuh"
using fedm::soft_add;
using fedm::soft_mul;

static uint64_t state = 0x9E3779B97F4A7C15ULL;
static uint64_t next()
{
  state ^= state << 13;
  state ^= state >> 7;
  state ^= state << 17;
  return state;
}

// A double with a random sign and significand and an exponent drawn from one
// of several regimes.
static double draw(int regime, int e_ref)
{
  uint64_t f = next() & 0x000FFFFFFFFFFFFFULL;
  const uint64_t r = next();
  if ((r & 7) == 0)
    f &= ~((1ULL << (r >> 58)) - 1);  // trailing zeros: exact products, ties
  if ((r & 15) == 1)
    f |= (1ULL << 52) - (1ULL << ((r >> 58) & 31));  // runs of ones: carries
  int e;
  switch (regime) {
    case 0: e = 1 + (int)(next() % 2046); break;                            // anywhere
    case 1: e = 1023 + (int)(next() % 64) - 32; break;                      // near 1
    case 2: e = e_ref + (int)(next() % 7) - 3; if (e < 1) e = 1; if (e > 2046) e = 2046; break;  // close exponents
    case 3: e = (next() & 1) ? 1 + (int)(next() % 60) : 2046 - (int)(next() % 60); break;  // range limits
    default: e = e_ref + (int)(next() % 120) - 60; if (e < 1) e = 1; if (e > 2046) e = 2046; break;
  }
  uint64_t bits = ((next() & 1) << 63) | ((uint64_t)e << 52) | f;
  if ((next() & 255) == 0)
    bits &= 0x800FFFFFFFFFFFFFULL;  // occasional subnormal / zero: fallback path
  double x;
  std::memcpy(&x, &bits, 8);
  return x;
}

int main(int argc, char** argv)
{
  const long long n = argc > 1 ? atoll(argv[1]) : 20000000LL;
  long long bad = 0;
  for (long long i = 0; i < n; i++) {
    const int regime = (int)(i % 5);
    const double a = draw(regime == 2 || regime == 4 ? 0 : regime, 1023);
    const int ea = (int)((__double_as_longlong(a) >> 52) & 0x7FF);
    double b = draw(regime, ea);
    if (regime == 2 && (i & 3) == 0)  // near-cancellation: b close to -a
      b = -__longlong_as_double(__double_as_longlong(a) + (long long)(next() % 5) - 2);
    const double pm = soft_mul(a, b), hm = a * b;
    const double pa = soft_add(a, b), ha = a + b;
    if (__double_as_longlong(pm) != __double_as_longlong(hm) || __double_as_longlong(pa) != __double_as_longlong(ha)) {
      if (bad < 10)
        std::printf("a=%a b=%a mul %a/%a add %a/%a\n", a, b, pm, hm, pa, ha);
      bad++;
    }
  }
  std::printf("mismatches %lld of %lld\n", bad, n);
  return bad != 0;
}
