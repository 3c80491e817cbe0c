// The JacobiSVD restatement of smap_solve.cuh for a compile-time size N,
// fully unrolled so the work matrix lives in registers.  The two rotation
// accumulators U and V are reached through accessors (StridedMat: a
// per-thread slice of shared memory interleaved across threads; or a matrix
// held in registers).  Every floating-point operation and
// its order are those of svd_solve(): the results are the same bits.
#pragma once

#include <cfloat>

#include "smap_solve.cuh"

namespace fedm {

// N x N matrix of one thread stored element-major across `stride` threads:
// element (i, j) at base[(i * N + j) * stride], so a warp touching the same
// element reads consecutive doubles.
template<int N>
struct StridedMat
{
  double* base;
  int stride;
  __device__ __forceinline__ double& operator()(int i, int j) const { return base[(i * N + j) * stride]; }
};

// ops accumulates the FP64 add/sub/mul/div/sqrt operations performed, with
// the same rules as svd_solve.
template<int N, class M, class MV>
__device__ __forceinline__ void svd_solve_nm(double (&W)[N][N], const double (&b)[N], double (&x)[N], const M& U,
                                             const MV& V, int& ops)
{
  const double tiny = DBL_MIN, eps = DBL_EPSILON;
  double scale = 0;
#pragma unroll
  for (int i = 0; i < N; i++)
#pragma unroll
    for (int j = 0; j < N; j++)
      scale = fmax(scale, fabs(W[i][j]));
  if (!isfinite(scale)) {
#pragma unroll
    for (int i = 0; i < N; i++)
      x[i] = 0;
    return;
  }
  if (scale == 0)
    scale = 1;
  const double yscale = rcp(scale);
#pragma unroll
  for (int i = 0; i < N; i++)
#pragma unroll
    for (int j = 0; j < N; j++) {
      W[i][j] = dvd_r(W[i][j], scale, yscale);
      U(i, j) = i == j ? 1.0 : 0.0;
      V(i, j) = i == j ? 1.0 : 0.0;
    }
  ops += N * N;
  long long maxDiag = 0;  // as mag_bits
#pragma unroll
  for (int i = 0; i < N; i++)
    maxDiag = max(maxDiag, mag_bits(W[i][i]));
  bool finished = false;
  int sweeps = 0;
  while (!finished && sweeps < 100) {
    finished = true;
    sweeps++;
#pragma unroll
    for (int p = 1; p < N; p++) {
#pragma unroll
      for (int q = 0; q < p; q++) {
        // fmax(tiny, precision * maxDiag), precision = 2 DBL_EPSILON
        const long long threshold = jacobi_threshold_bits(maxDiag);
        if (mag_bits(W[p][q]) > threshold || mag_bits(W[q][p]) > threshold) {
          finished = false;
          ops += 18 + 24 * N;
          // real_2x2_jacobi_svd on rows/cols p, q
          const double m00 = W[p][p], m01 = W[p][q], m10 = W[q][p], m11 = W[q][q];
          double r1c, r1s;
          const double t = add(m00, m11), d = sub(m10, m01);
          if (fabs(d) < tiny) {
            r1s = 0;
            r1c = 1;
          } else {
            const double u = dvd(t, d);
            const double tmp = __dsqrt_rn(add(1.0, mul(u, u)));
            r1s = rcp(tmp);
            r1c = dvd_r(u, tmp, r1s);
            ops += 6;
          }
          const double n00 = add(mul(r1c, m00), mul(r1s, m10));
          const double n01 = add(mul(r1c, m01), mul(r1s, m11));
          const double n11 = add(mul(-r1s, m01), mul(r1c, m11));
          const double deno = mul(2.0, fabs(n01));
          double jrc, jrs;
          if (deno < tiny) {
            jrc = 1;
            jrs = 0;
          } else {
            const double tau = dvd(sub(n00, n11), deno);
            const double w = __dsqrt_rn(add(mul(tau, tau), 1.0));
            const double tt = rcp(tau > 0 ? add(tau, w) : sub(tau, w));
            const double sign_t = tt > 0 ? 1.0 : -1.0;
            const double nn = rcp(__dsqrt_rn(add(mul(tt, tt), 1.0)));
            // -sign_t * (n01 / |n01|) * |tt| is an exact sign change
            const bool neg = (sign_t > 0) == (n01 > 0);
            jrs = mul(neg ? -fabs(tt) : fabs(tt), nn);
            jrc = nn;
            ops += 12;
          }
          const double jtc = jrc, jts = -jrs;
          const double jlc = sub(mul(r1c, jtc), mul(r1s, jts));
          const double jls = add(mul(r1c, jts), mul(r1s, jtc));
          // W.applyOnTheLeft(p, q, jl)
#pragma unroll
          for (int i = 0; i < N; i++) {
            const double xv = W[p][i], yv = W[q][i];
            W[p][i] = add(mul(jlc, xv), mul(jls, yv));
            W[q][i] = add(mul(-jls, xv), mul(jlc, yv));
          }
          // U.applyOnTheRight(p, q, jl^T): rotation (c, -s) applied transposed
          {
            const double c = jlc, s = jls;  // transpose of (jlc, -jls)
#pragma unroll
            for (int i = 0; i < N; i++) {
              const double xv = U(i, p), yv = U(i, q);
              U(i, p) = add(mul(c, xv), mul(s, yv));
              U(i, q) = add(mul(-s, xv), mul(c, yv));
            }
          }
          // W.applyOnTheRight(p, q, jr) and V.applyOnTheRight(p, q, jr)
          {
            const double c = jrc, s = -jrs;
#pragma unroll
            for (int i = 0; i < N; i++) {
              const double xv = W[i][p], yv = W[i][q];
              W[i][p] = add(mul(c, xv), mul(s, yv));
              W[i][q] = add(mul(-s, xv), mul(c, yv));
            }
#pragma unroll
            for (int i = 0; i < N; i++) {
              const double xv = V(i, p), yv = V(i, q);
              V(i, p) = add(mul(c, xv), mul(s, yv));
              V(i, q) = add(mul(-s, xv), mul(c, yv));
            }
          }
          maxDiag = max(maxDiag, max(mag_bits(W[p][p]), mag_bits(W[q][q])));
        }
      }
    }
  }
  double sv[N];
#pragma unroll
  for (int i = 0; i < N; i++) {
    const double a = W[i][i];
    sv[i] = fabs(a);
    if (a < 0) {
#pragma unroll
      for (int r = 0; r < N; r++)
        U(r, i) = -U(r, i);
    }
  }
#pragma unroll
  for (int i = 0; i < N; i++)
    sv[i] = mul(sv[i], scale);
  ops += N + 2;
  int nonzero = N;
  bool stop = false;
#pragma unroll
  for (int i = 0; i < N; i++) {
    if (!stop) {
      int pos = i;
      double mx = sv[i];
#pragma unroll
      for (int j = i + 1; j < N; j++)
        if (sv[j] > mx) {
          mx = sv[j];
          pos = j;
        }
      if (mx == 0) {
        nonzero = i;
        stop = true;
      } else if (pos != i) {
#pragma unroll
        for (int j = i + 1; j < N; j++) {
          if (pos == j) {
            const double s0 = sv[i];
            sv[i] = sv[j];
            sv[j] = s0;
#pragma unroll
            for (int r = 0; r < N; r++) {
              const double u0 = U(r, i);
              U(r, i) = U(r, j);
              U(r, j) = u0;
              const double v0 = V(r, i);
              V(r, i) = V(r, j);
              V(r, j) = v0;
            }
          }
        }
      }
    }
  }
  const double thr = fmax(mul(sv[0], mul((double)(N > 1 ? N : 1), eps)), tiny);
  int rank = 0;
#pragma unroll
  for (int i = 0; i < N; i++)
    if (i < nonzero && !(sv[i] < thr))
      rank = i + 1;
  // rank() walks down from nonzero-1 while sv < thr; with sv sorted in
  // decreasing order that is the count of leading entries >= thr
  double tmp[N];
#pragma unroll
  for (int cc = 0; cc < N; cc++) {
    if (cc < rank) {
      double s = 0;
#pragma unroll
      for (int r = 0; r < N; r++)
        s = add(s, mul(U(r, cc), b[r]));
      tmp[cc] = mul(rcp(sv[cc]), s);
    }
  }
#pragma unroll
  for (int r = 0; r < N; r++) {
    double s = 0;
#pragma unroll
    for (int cc = 0; cc < N; cc++)
      if (cc < rank)
        s = add(s, mul(V(r, cc), tmp[cc]));
    x[r] = s;
  }
  ops += rank * (2 * N + 2) + 2 * N * rank;
}

} // namespace fedm
