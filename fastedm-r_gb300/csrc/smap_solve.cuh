// FP64 solvers for the S-map normal equations, written with explicit
// round-to-nearest multiply and add intrinsics so that every translation unit
// (with or without FMA contraction) computes the same bits.
//
// svd_solve restates Eigen 3.3's JacobiSVD of a square matrix (two-sided
// Jacobi sweeps over (p, q) pairs with a 2x2 real SVD, singular values made
// positive and sorted, rank threshold diagSize * epsilon) followed by
// SVDBase::solve, which is what the reference calls
// (EDM-Developers/fastEDM-r src/edm.cpp:780-782).  Eigen is MPL2; only its
// published algorithm is followed.
#pragma once

#include <cfloat>

namespace fedm {

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dvd(double a, double b) { return __ddiv_rn(a, b); }
// 1.0 / a, correctly rounded (IEEE round-to-nearest): the same bits as
// dvd(1.0, a).
__device__ __forceinline__ double rcp(double a) { return __drcp_rn(a); }

// a / b correctly rounded -- the same bits as dvd(a, b) -- given y = rcp(b),
// for divisions that share a divisor.  Markstein's method (P. Markstein,
// "Computation of elementary functions on the IBM RISC System/6000
// processor", IBM J. Res. Develop. 34(1), 1990): q0 = a y is within 1.5 ulp
// of a/b; one correction q1 = q0 + (a - b q0) y makes it faithful; the
// remainder a - b q1 of a faithful quotient is exact, and q1 + (a - b q1) y
// rounds to a/b (Markstein's theorem, y being within half an ulp of 1/b).
// All products and remainders stay normal while both exponents lie within
// +-500; other operands (zero, tiny, huge, not finite) take the division.
// One multiply and four FMAs against the division's longer sequence;
// tests/division_check.cu compares it with dvd on random pairs over every
// exponent range.
__device__ __forceinline__ double dvd_r(double a, double b, double y)
{
  const unsigned ea = (unsigned)(__double2hiint(a) >> 20) & 0x7ffu;
  const unsigned eb = (unsigned)(__double2hiint(b) >> 20) & 0x7ffu;
  if (ea - 523u > 1000u || eb - 523u > 1000u)
    return __ddiv_rn(a, b);
  const double q0 = __dmul_rn(a, y);
  const double r0 = __fma_rn(-b, q0, a);
  const double q1 = __fma_rn(r0, y, q0);
  const double r1 = __fma_rn(-b, q1, a);
  return __fma_rn(r1, y, q1);
}

// The Jacobi sweep's magnitude tests run on integers, off the FP64 pipe.
// mag_bits(x) is |x| as its bit pattern, whose integer order is the order of
// the magnitudes; NaN maps to -1 so, like a floating-point comparison with
// NaN, it never exceeds a threshold and never wins a maximum.
__device__ __forceinline__ long long mag_bits(double x)
{
  const long long b = __double_as_longlong(x) & 0x7fffffffffffffffLL;
  return b > 0x7ff0000000000000LL ? -1 : b;
}

// Bits of fmax(DBL_MIN, 2 DBL_EPSILON * m) for m = mag_bits of a finite
// m >= 0: the product is a power-of-two scaling, exact (exponent field less
// 51) unless it falls below DBL_MIN, where the maximum is DBL_MIN.
__device__ __forceinline__ long long jacobi_threshold_bits(long long m)
{
  constexpr long long TINY = 1LL << 52;  // bits of DBL_MIN
  return m >= (52LL << 52) ? m - (51LL << 52) : TINY;
}

struct Rot
{
  double c, s;
};

// rows p, q <- J [row p; row q], J = [c s; -s c]
__device__ __forceinline__ void rot_rows(double* A, int n, int p, int q, Rot j)
{
  for (int i = 0; i < n; i++) {
    const double x = A[p * n + i], y = A[q * n + i];
    A[p * n + i] = add(mul(j.c, x), mul(j.s, y));
    A[q * n + i] = add(mul(-j.s, x), mul(j.c, y));
  }
}

// cols p, q <- [col p, col q] J^T  (Eigen's applyOnTheRight)
__device__ __forceinline__ void rot_cols(double* A, int n, int p, int q, Rot j)
{
  const double c = j.c, s = -j.s;
  for (int i = 0; i < n; i++) {
    const double x = A[i * n + p], y = A[i * n + q];
    A[i * n + p] = add(mul(c, x), mul(s, y));
    A[i * n + q] = add(mul(-s, x), mul(c, y));
  }
}

// ops counts the FP64 add/sub/mul/div/sqrt operations performed.
__device__ inline void jacobi_2x2(const double* W, int n, int p, int q, Rot& jl, Rot& jr, int& ops)
{
  ops += 18;
  const double tiny = DBL_MIN;
  const double m00 = W[p * n + p], m01 = W[p * n + q], m10 = W[q * n + p], m11 = W[q * n + q];
  Rot r1;
  const double t = add(m00, m11), d = sub(m10, m01);
  if (fabs(d) < tiny) {
    r1.s = 0;
    r1.c = 1;
  } else {
    const double u = dvd(t, d);
    const double tmp = __dsqrt_rn(add(1.0, mul(u, u)));
    r1.s = rcp(tmp);
    r1.c = dvd_r(u, tmp, r1.s);
    ops += 6;
  }
  const double n00 = add(mul(r1.c, m00), mul(r1.s, m10));
  const double n01 = add(mul(r1.c, m01), mul(r1.s, m11));
  const double n11 = add(mul(-r1.s, m01), mul(r1.c, m11));
  const double deno = mul(2.0, fabs(n01));
  if (deno < tiny) {
    jr.c = 1;
    jr.s = 0;
  } else {
    const double tau = dvd(sub(n00, n11), deno);
    const double w = __dsqrt_rn(add(mul(tau, tau), 1.0));
    const double tt = rcp(tau > 0 ? add(tau, w) : sub(tau, w));
    const double sign_t = tt > 0 ? 1.0 : -1.0;
    const double nn = rcp(__dsqrt_rn(add(mul(tt, tt), 1.0)));
    // Eigen forms -sign_t * (n01 / |n01|) * |tt| * nn left to right; the
    // first two products are exact sign changes (n01 is finite and nonzero
    // here), so only the last multiply rounds.
    const bool neg = (sign_t > 0) == (n01 > 0);
    jr.s = mul(neg ? -fabs(tt) : fabs(tt), nn);
    jr.c = nn;
    ops += 12;
  }
  const double jtc = jr.c, jts = -jr.s;
  jl.c = sub(mul(r1.c, jtc), mul(r1.s, jts));
  jl.s = add(mul(r1.c, jts), mul(r1.s, jtc));
}

// Solves A x = b in the pseudo-inverse sense.  W holds A (n x n, destroyed);
// U, V: n*n scratch; sv, tmp: n scratch.  ops accumulates the number of FP64
// add/sub/mul/div/sqrt operations performed (the solve's algorithmic work).
__device__ inline void svd_solve(double* W, double* U, double* V, double* sv, double* tmp, const double* b, double* x,
                                 int n, int& ops)
{
  const double tiny = DBL_MIN, eps = DBL_EPSILON;
  double scale = 0;
  for (int i = 0; i < n * n; i++)
    scale = fmax(scale, fabs(W[i]));
  if (!isfinite(scale)) {
    for (int i = 0; i < n; i++)
      x[i] = 0;
    return;
  }
  if (scale == 0)
    scale = 1;
  const double yscale = rcp(scale);
  for (int i = 0; i < n * n; i++) {
    W[i] = dvd_r(W[i], scale, yscale);
    U[i] = 0;
    V[i] = 0;
  }
  ops += n * n;
  for (int i = 0; i < n; i++)
    U[i * n + i] = V[i * n + i] = 1;
  long long maxDiag = 0;  // as mag_bits
  for (int i = 0; i < n; i++)
    maxDiag = max(maxDiag, mag_bits(W[i * n + i]));
  bool finished = false;
  int sweeps = 0;
  while (!finished && sweeps < 100) {
    finished = true;
    sweeps++;
    for (int p = 1; p < n; p++) {
      for (int q = 0; q < p; q++) {
        // fmax(tiny, precision * maxDiag), precision = 2 DBL_EPSILON
        const long long threshold = jacobi_threshold_bits(maxDiag);
        if (mag_bits(W[p * n + q]) > threshold || mag_bits(W[q * n + p]) > threshold) {
          finished = false;
          Rot jl, jr;
          jacobi_2x2(W, n, p, q, jl, jr, ops);
          ops += 24 * n;
          rot_rows(W, n, p, q, jl);
          rot_cols(U, n, p, q, Rot{ jl.c, -jl.s });
          rot_cols(W, n, p, q, jr);
          rot_cols(V, n, p, q, jr);
          maxDiag = max(maxDiag, max(mag_bits(W[p * n + p]), mag_bits(W[q * n + q])));
        }
      }
    }
  }
  for (int i = 0; i < n; i++) {
    const double a = W[i * n + i];
    sv[i] = fabs(a);
    if (a < 0)
      for (int r = 0; r < n; r++)
        U[r * n + i] = -U[r * n + i];
  }
  for (int i = 0; i < n; i++)
    sv[i] = mul(sv[i], scale);
  ops += n + 2;
  int nonzero = n;
  for (int i = 0; i < n; i++) {
    int pos = i;
    double mx = sv[i];
    for (int j = i + 1; j < n; j++)
      if (sv[j] > mx) {
        mx = sv[j];
        pos = j;
      }
    if (mx == 0) {
      nonzero = i;
      break;
    }
    if (pos != i) {
      const double s0 = sv[i];
      sv[i] = sv[pos];
      sv[pos] = s0;
      for (int r = 0; r < n; r++) {
        const double u0 = U[r * n + i];
        U[r * n + i] = U[r * n + pos];
        U[r * n + pos] = u0;
        const double v0 = V[r * n + i];
        V[r * n + i] = V[r * n + pos];
        V[r * n + pos] = v0;
      }
    }
  }
  const double thr = fmax(mul(sv[0], mul((double)(n > 1 ? n : 1), eps)), tiny);
  int i = nonzero - 1;
  while (i >= 0 && sv[i] < thr)
    --i;
  const int rank = i + 1;
  for (int cc = 0; cc < rank; cc++) {
    double s = 0;
    for (int r = 0; r < n; r++)
      s = add(s, mul(U[r * n + cc], b[r]));
    tmp[cc] = mul(rcp(sv[cc]), s);
  }
  for (int r = 0; r < n; r++) {
    double s = 0;
    for (int cc = 0; cc < rank; cc++)
      s = add(s, mul(V[r * n + cc], tmp[cc]));
    x[r] = s;
  }
  ops += rank * (2 * n + 2) + 2 * n * rank;
}

__device__ inline void svd_solve(double* W, double* U, double* V, double* sv, double* tmp, const double* b, double* x,
                                 int n)
{
  int ops = 0;
  svd_solve(W, U, V, sv, tmp, b, x, n, ops);
}

} // namespace fedm
