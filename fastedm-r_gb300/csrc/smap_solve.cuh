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

// True for 2^27 <= |a| < 2^511.  There, evaluated in double,
// sqrt(1 + a*a) is |a| exactly: a*a >= 2^54 has an ulp of at least 4, so
// adding 1 rounds back to a*a; and the square root of a correctly rounded
// square rounds to |a|, because the square's relative rounding error (at
// most 2^-53) moves its square root by less than half an ulp of |a|.  The
// upper bound keeps a*a finite.  Checked against the plain evaluation on
// 10^8 random values over the whole range.
__device__ __forceinline__ bool hypot_is_abs(double a)
{
  const unsigned e = ((unsigned)__double2hiint(a) >> 20) & 0x7ffu;
  return e - (1023u + 27u) <= 483u;
}

// True when every lane of the warp that runs this call together (its
// coalesced threads, as cooperative_groups::coalesced_threads() forms them)
// passes c.  The FP64 pipe takes a warp instruction in the same time however
// many of its lanes are active, so a shortcut pays only when the whole
// group takes it; lanes that could take it run the full sequence, whose
// results are the same.
__device__ __forceinline__ bool all_lanes(bool c)
{
  return __all_sync(__activemask(), c) != 0;
}

// Eigen's real_2x2_jacobi_svd on the block [m00 m01; m10 m11]: the left
// rotation jl and the right rotation jr (as Eigen's JacobiRotation c, s).
// ops counts the FP64 operations of the reference's sequence.
//
// Shortcuts that return the reference's values:
//  - a symmetric block (|m10 - m01| < DBL_MIN) takes the identity as its
//    first rotation, whose products return m00, m01, m11 and make
//    jl = jr^T;
//  - for 2^27 <= |u| < 2^511, tmp = sqrt(1 + u^2) is |u| (hypot_is_abs),
//    so the first rotation is c = u/|u| = +-1, s = 1/|u|;
//  - for 2^27 <= |tau| < 2^511, w = sqrt(tau^2 + 1) is |tau|, tau +- w is
//    2 tau (exact), t = 1/(2 tau), and t^2 <= 2^-56 makes 1 + t^2 round
//    to 1, so n = 1/sqrt(1 + t^2) = 1 and the rotation is c = 1, s = +-|t|.
// Both large cases are the rule in later sweeps, where the block is nearly
// symmetric (|u| ~ 1/epsilon) and nearly diagonal (large |tau|); a warp
// takes them when all of its lanes at the call qualify (all_lanes).  Where the
// shortcut's result is a zero, only its sign can differ from the
// reference's; the signs of zeros in the work matrix and the accumulators
// reach no output of the solve (every sum there starts from +0).
__device__ __forceinline__ void jacobi_2x2_vals(double m00, double m01, double m10, double m11, double& jlc,
                                                double& jls, double& jrc, double& jrs, int& ops)
{
  const double tiny = DBL_MIN;
  ops += 18;
  double r1c, r1s, n00, n01, n11;
  bool r1_id = false, r1_unit = false;
  const double d = sub(m10, m01);
  if (fabs(d) < tiny) {
    r1c = 1;
    r1s = 0;
    r1_id = true;
    n00 = m00;
    n01 = m01;
    n11 = m11;
  } else {
    const double t = add(m00, m11);
    const double u = dvd(t, d);
    ops += 6;
    if (all_lanes(hypot_is_abs(u))) {
      // c = u / |u| = +-1: its products are exact sign changes
      r1s = rcp(fabs(u));
      r1c = u < 0 ? -1.0 : 1.0;
      r1_unit = true;
      const bool cn = u < 0;
      n00 = add(cn ? -m00 : m00, mul(r1s, m10));
      n01 = add(cn ? -m01 : m01, mul(r1s, m11));
      n11 = add(mul(-r1s, m01), cn ? -m11 : m11);
    } else {
      const double tmp = __dsqrt_rn(add(1.0, mul(u, u)));
      r1s = rcp(tmp);
      r1c = dvd_r(u, tmp, r1s);
      n00 = add(mul(r1c, m00), mul(r1s, m10));
      n01 = add(mul(r1c, m01), mul(r1s, m11));
      n11 = add(mul(-r1s, m01), mul(r1c, m11));
    }
  }
  const double deno = mul(2.0, fabs(n01));
  if (deno < tiny) {
    jrc = 1;
    jrs = 0;
  } else {
    const double tau = dvd(sub(n00, n11), deno);
    ops += 12;
    // Eigen forms -sign_t * (n01 / |n01|) * |tt| * nn left to right; the
    // first two products are exact sign changes (n01 is finite and nonzero
    // here), so only the last multiply rounds.
    if (all_lanes(hypot_is_abs(tau))) {
      const double tt = rcp(mul(2.0, tau));
      const bool neg = (tt > 0) == (n01 > 0);
      jrs = neg ? -fabs(tt) : fabs(tt);
      jrc = 1.0;
    } else {
      const double w = __dsqrt_rn(add(mul(tau, tau), 1.0));
      const double tt = rcp(tau > 0 ? add(tau, w) : sub(tau, w));
      const double nn = rcp(__dsqrt_rn(add(mul(tt, tt), 1.0)));
      const bool neg = (tt > 0) == (n01 > 0);
      jrs = mul(neg ? -fabs(tt) : fabs(tt), nn);
      jrc = nn;
    }
  }
  const double jtc = jrc, jts = -jrs;
  if (r1_id) {
    jlc = jtc;
    jls = jts;
  } else if (r1_unit) {
    const bool cn = r1c < 0;
    jlc = sub(cn ? -jtc : jtc, mul(r1s, jts));
    jls = add(cn ? -jts : jts, mul(r1s, jtc));
  } else {
    jlc = sub(mul(r1c, jtc), mul(r1s, jts));
    jls = add(mul(r1c, jts), mul(r1s, jtc));
  }
}

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

// ops counts the FP64 add/sub/mul/div/sqrt operations of the reference's
// sequence.
__device__ __forceinline__ void jacobi_2x2(const double* W, int n, int p, int q, Rot& jl, Rot& jr, int& ops)
{
  jacobi_2x2_vals(W[p * n + p], W[p * n + q], W[q * n + p], W[q * n + q], jl.c, jl.s, jr.c, jr.s, ops);
}

// Columns p, q of a rotation accumulator (U or V, started as the identity)
// <- [col p, col q] [c -s; s c], in the first sweep.  Before the first
// sweep's rotation (p, q) column q can be nonzero only in rows < p, and
// column p only in row p (q = 0) or rows <= p (q > 0): rotations come in
// the order (1,0), (2,0), (2,1), (3,0), ... and each leaves both of its
// columns nonzero in the union of their rows.  A lane that skipped an
// earlier rotation has fewer nonzero rows, never more.  Products by those
// zeros are left out: c*x + s*0 is c*x for nonzero c*x, and a zero's sign
// reaches no output of the solve.
__device__ __forceinline__ void rot_cols_first(double* A, int n, int p, int q, double c, double s)
{
  if (q > 0) {
    for (int i = 0; i < p; i++) {
      const double x = A[i * n + p], y = A[i * n + q];
      A[i * n + p] = add(mul(c, x), mul(s, y));
      A[i * n + q] = add(mul(-s, x), mul(c, y));
    }
  } else {
    for (int i = 0; i < p; i++) {
      const double y = A[i * n + q];
      A[i * n + p] = mul(s, y);
      A[i * n + q] = mul(c, y);
    }
  }
  const double x = A[p * n + p];
  A[p * n + p] = mul(c, x);
  A[p * n + q] = mul(-s, x);
}

// Solves A x = b in the pseudo-inverse sense.  W holds A (n x n, destroyed);
// U, V: n*n scratch; sv, tmp: n scratch.  ops accumulates the number of FP64
// add/sub/mul/div/sqrt operations of the reference's sequence (the solve's
// algorithmic work); the exact shortcuts of jacobi_2x2_vals and
// rot_cols_first leave some of them out without changing a result.
__device__ inline void svd_solve(double* W, double* U, double* V, double* sv, double* tmp, const double* b, double* x,
                                 int n, int& ops)
{
  const double tiny = DBL_MIN, eps = DBL_EPSILON;
  // scale = max |W_ij| (fmax over the entries from 0, so a NaN never wins),
  // taken on the magnitudes' bit patterns
  long long smax = 0;
  for (int i = 0; i < n * n; i++)
    smax = max(smax, mag_bits(W[i]));
  if (smax >= 0x7ff0000000000000LL) {
    for (int i = 0; i < n; i++)
      x[i] = 0;
    return;
  }
  const double scale = smax == 0 ? 1.0 : __longlong_as_double(smax);
  const double yscale = rcp(scale);
  // W / scale; the two entries of a symmetric pair have the same quotient
  for (int i = 0; i < n; i++) {
    W[i * n + i] = dvd_r(W[i * n + i], scale, yscale);
    for (int j = i + 1; j < n; j++) {
      const double a = W[i * n + j], b = W[j * n + i];
      const double qa = dvd_r(a, scale, yscale);
      W[i * n + j] = qa;
      W[j * n + i] = __double_as_longlong(a) == __double_as_longlong(b) ? qa : dvd_r(b, scale, yscale);
    }
  }
  for (int i = 0; i < n * n; i++) {
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
          rot_cols(W, n, p, q, jr);
          if (sweeps == 1) {
            rot_cols_first(U, n, p, q, jl.c, jl.s);
            rot_cols_first(V, n, p, q, jr.c, -jr.s);
          } else {
            rot_cols(U, n, p, q, Rot{ jl.c, -jl.s });
            rot_cols(V, n, p, q, jr);
          }
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
