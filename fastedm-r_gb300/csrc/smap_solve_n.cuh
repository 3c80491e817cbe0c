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

// Columns p, q of the accumulator M <- [col p, col q] [c -s; s c].
template<int N, class M>
__device__ __forceinline__ void rot_cols_m(const M& A, int p, int q, double c, double s)
{
#pragma unroll
  for (int i = 0; i < N; i++) {
    const double xv = A(i, p), yv = A(i, q);
    A(i, p) = add(mul(c, xv), mul(s, yv));
    A(i, q) = add(mul(-s, xv), mul(c, yv));
  }
}

// The same rotation in the first sweep, skipping the rows that are still
// zero (the rule of rot_cols_first in smap_solve.cuh).
template<int N, class M>
__device__ __forceinline__ void rot_cols_first_m(const M& A, int p, int q, double c, double s)
{
#pragma unroll
  for (int i = 0; i < N; i++) {
    if (i < p) {
      if (q > 0) {
        const double xv = A(i, p), yv = A(i, q);
        A(i, p) = add(mul(c, xv), mul(s, yv));
        A(i, q) = add(mul(-s, xv), mul(c, yv));
      } else {
        const double yv = A(i, q);
        A(i, p) = mul(s, yv);
        A(i, q) = mul(c, yv);
      }
    } else if (i == p) {
      const double xv = A(p, p);
      A(p, p) = mul(c, xv);
      A(p, q) = mul(-s, xv);
    }
  }
}

// ops accumulates the FP64 add/sub/mul/div/sqrt operations of the
// reference's sequence, with the same rules as svd_solve.
template<int N, class M, class MV>
__device__ __forceinline__ void svd_solve_nm(double (&W)[N][N], const double (&b)[N], double (&x)[N], const M& U,
                                             const MV& V, int& ops)
{
  const double tiny = DBL_MIN, eps = DBL_EPSILON;
  // scale = max |W_ij|, on the magnitudes' bit patterns (as svd_solve)
  long long smax = 0;
#pragma unroll
  for (int i = 0; i < N; i++)
#pragma unroll
    for (int j = 0; j < N; j++)
      smax = max(smax, mag_bits(W[i][j]));
  if (smax >= 0x7ff0000000000000LL) {
#pragma unroll
    for (int i = 0; i < N; i++)
      x[i] = 0;
    return;
  }
  const double scale = smax == 0 ? 1.0 : __longlong_as_double(smax);
  const double yscale = rcp(scale);
#pragma unroll
  for (int i = 0; i < N; i++) {
    W[i][i] = dvd_r(W[i][i], scale, yscale);
#pragma unroll
    for (int j = i + 1; j < N; j++) {
      const double a = W[i][j], b = W[j][i];
      const double qa = dvd_r(a, scale, yscale);
      W[i][j] = qa;
      W[j][i] = __double_as_longlong(a) == __double_as_longlong(b) ? qa : dvd_r(b, scale, yscale);
    }
  }
#pragma unroll
  for (int i = 0; i < N; i++)
#pragma unroll
    for (int j = 0; j < N; j++) {
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
          ops += 24 * N;
          // real_2x2_jacobi_svd on rows/cols p, q
          double jlc, jls, jrc, jrs;
          jacobi_2x2_vals(W[p][p], W[p][q], W[q][p], W[q][q], jlc, jls, jrc, jrs, ops);
          // W.applyOnTheLeft(p, q, jl)
#pragma unroll
          for (int i = 0; i < N; i++) {
            const double xv = W[p][i], yv = W[q][i];
            W[p][i] = add(mul(jlc, xv), mul(jls, yv));
            W[q][i] = add(mul(-jls, xv), mul(jlc, yv));
          }
          // W.applyOnTheRight(p, q, jr)
          {
            const double c = jrc, s = -jrs;
#pragma unroll
            for (int i = 0; i < N; i++) {
              const double xv = W[i][p], yv = W[i][q];
              W[i][p] = add(mul(c, xv), mul(s, yv));
              W[i][q] = add(mul(-s, xv), mul(c, yv));
            }
          }
          // U.applyOnTheRight(p, q, jl^T) and V.applyOnTheRight(p, q, jr):
          // column rotations by (c, s) = (jlc, jls) and (jrc, -jrs); in the
          // first sweep only the rows that can be nonzero (rot_cols_first)
          if (sweeps == 1) {
            rot_cols_first_m<N>(U, p, q, jlc, jls);
            rot_cols_first_m<N>(V, p, q, jrc, -jrs);
          } else {
            rot_cols_m<N>(U, p, q, jlc, jls);
            rot_cols_m<N>(V, p, q, jrc, -jrs);
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
