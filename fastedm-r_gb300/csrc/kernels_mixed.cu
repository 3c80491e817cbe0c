// Mixed-precision neighbour search and forecast (the CCM hot path).
//
// Work item = one task x 512 prediction points, taken from a global queue in
// decreasing library size.  A 256-thread CTA stages 1024 library rows of the
// centred FP32 manifold in shared memory at a time; every thread scores them
// against two prediction points and keeps, per point, the C smallest squared
// FP32 distances (sorted, registers) plus up to two exact zeros.
//
// Certification.  With u = 2^-24, the FP32 squared distance s of a pair obeys
// sqrt(s)/sqrt(1+g) - e <= D <= sqrt(s)/sqrt(1-g) + e, where D is the exact
// distance of the FP64 rows, g = (Ea+2)*2^-23 bounds the accumulation and
// e = 2^-21 * R (R = largest centred row norm) bounds the input rounding.
// The k-th true distance is at most hi = sqrt(s_k)/sqrt(1-g) + e, so every
// true neighbour has s <= T = ((hi + e) * sqrt(1+g))^2 (widened by 1e-14).
// If the C-th kept value exceeds T, every entry at or under T is in the list;
// otherwise the point is handed to the exact kernels.  Entries under T are
// re-scored in FP64 with the reference's operation order
// (src/distances.cpp:194-225), so neighbour distances and their
// (distance, index) order are the FP64 bits.  A positive FP32 distance implies
// a positive FP64 one; FP32 zeros are re-scored and dropped when the FP64
// distance is zero too (src/distances.cpp:218).
#include <cfloat>
#include <climits>

#include "exp_rn.cuh"
#include "kernels.h"
#include "smap_solve.cuh"

namespace fedm {

namespace {

constexpr double MISS = 1.0e+100;
constexpr int TPB = 256;
constexpr int TILE = 1024;
constexpr int ZCAP = 2;

template<int C>
__device__ __forceinline__ void topc_insert(float (&D)[C], int (&I)[C], float dv, int iv)
{
  bool ins = false;
#pragma unroll
  for (int j = 0; j < C; j++) {
    const bool s = ins || dv < D[j];
    const float td = D[j];
    const int ti = I[j];
    D[j] = s ? dv : td;
    I[j] = s ? iv : ti;
    dv = s ? td : dv;
    iv = s ? ti : iv;
    ins = s;
  }
}

template<int C>
__device__ __forceinline__ float pick(const float (&D)[C], int j)
{
  float v = D[0];
#pragma unroll
  for (int q = 1; q < C; q++)
    v = (q == j) ? D[q] : v;
  return v;
}

__device__ __forceinline__ void note_rc_m(const GroupParams& g, int task, int code)
{
  if (code)
    atomicMax(&g.task_rc[task], code);
}

// FP64 distance of library row `row` to the prediction row values y
// (src/distances.cpp:194-225 without missing values or panels).
template<int EA>
__device__ __forceinline__ double fp64_sq(const GroupParams& g, int row, const double (&y)[EA])
{
  const double* x = g.F + (size_t)row * EA;
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < EA; j++) {
    const double df = sub(x[j], y[j]);
    s = add(s, mul(df, df));
  }
  return s;
}

template<int EA, int C>
__device__ void finalize_point(const GroupParams& g, const MixedRun& m, const DevTask& T, long long p, int prow,
                               const float (&D)[C], const int (&I)[C], int z, const int (&zi)[ZCAP])
{
  const int k = T.k;
  int lc = 0;
#pragma unroll
  for (int j = 0; j < C; j++)
    lc += D[j] < INFINITY ? 1 : 0;
  bool fallback = z > ZCAP;
  double thr = INFINITY;
  if (!fallback && lc >= k) {
    const double sq = sqrt((double)pick(D, k - 1));
    const double hi = sq / sqrt(1.0 - m.gamma) + m.err_abs;
    const double td = (hi * (1.0 + 1e-14) + m.err_abs) * sqrt(1.0 + m.gamma);
    thr = td * td * (1.0 + 1e-14);
    if (lc == C && !((double)D[C - 1] > thr))
      fallback = true;
  }
  if (fallback) {
    const int slot = atomicAdd(m.fb_count, 1);
    if (slot < m.fb_cap)
      m.fb_list[slot] = p;
    return;
  }
  double y[EA];
#pragma unroll
  for (int j = 0; j < EA; j++)
    y[j] = g.Fp[(size_t)prow * EA + j];
  double cd[C + ZCAP];
  int ci[C + ZCAP];
  int nc = 0;
#pragma unroll
  for (int j = 0; j < C; j++) {
    if (j < lc && (double)D[j] <= thr) {
      const double s = fp64_sq<EA>(g, g.lib_rows[T.lib_off + I[j]], y);
      cd[nc] = __dsqrt_rn(s);
      ci[nc] = I[j];
      nc++;
    }
  }
  int zvalid = 0;
#pragma unroll
  for (int j = 0; j < ZCAP; j++) {
    if (j < z) {
      const double s = fp64_sq<EA>(g, g.lib_rows[T.lib_off + zi[j]], y);
      if (s != 0) {
        cd[nc] = __dsqrt_rn(s);
        ci[nc] = zi[j];
        nc++;
        zvalid++;
      }
    }
  }
  const int numValid = T.n_lib - z + zvalid;
  const int keff = k < numValid ? k : numValid;
  if (keff <= 0) {
    // src/edm.cpp:602-606: no forecast; rc(0) SUCCESS, later thetas untouched
    if (g.n_thetas > 1)
      note_rc_m(g, T.task, 8000);
    if (g.kused)
      g.kused[p] = INT_MIN;
    return;
  }
  // (distance, library index) order among the candidates
  for (int a = 1; a < nc; a++) {
    const double dv = cd[a];
    const int iv = ci[a];
    int b = a - 1;
    while (b >= 0 && (cd[b] > dv || (cd[b] == dv && ci[b] > iv))) {
      cd[b + 1] = cd[b];
      ci[b + 1] = ci[b];
      b--;
    }
    cd[b + 1] = dv;
    ci[b + 1] = iv;
  }
  if (keff == numValid) {
    // every valid neighbour, in library order (src/edm.cpp:615-616)
    for (int a = 1; a < keff; a++) {
      const double dv = cd[a];
      const int iv = ci[a];
      int b = a - 1;
      while (b >= 0 && ci[b] > iv) {
        cd[b + 1] = cd[b];
        ci[b + 1] = ci[b];
        b--;
      }
      cd[b + 1] = dv;
      ci[b + 1] = iv;
    }
  }
  atomicMin(&g.task_kmin[T.task], keff);
  atomicMax(&g.task_kmax[T.task], keff);
  if (g.kused)
    g.kused[p] = keff;
  if (m.nn_idx) {
    for (int j = 0; j < keff; j++) {
      m.nn_idx[p * m.kslots + j] = ci[j];
      m.nn_dist[p * m.kslots + j] = cd[j];
    }
  }
  int rows[C + ZCAP];
  for (int j = 0; j < keff; j++)
    rows[j] = g.lib_rows[T.lib_off + ci[j]];

  if (g.algorithm == 0) {
    // simplex (src/edm.cpp:707-735)
    double minD = cd[0];
    for (int j = 1; j < keff; j++)
      minD = cd[j] < minD ? cd[j] : minD;
    for (int t = 0; t < g.n_thetas; t++) {
      const double theta = g.thetas[t];
      double sumw = 0.0;
      for (int j = 0; j < keff; j++)
        sumw = add(sumw, exp_rn(mul(-theta, dvd(cd[j], minD))));
      double r = 0.0;
      for (int j = 0; j < keff; j++) {
        const double w = exp_rn(mul(-theta, dvd(cd[j], minD)));
        r = add(r, mul(g.lib_target[rows[j]], dvd(w, sumw)));
      }
      g.pred[(size_t)t * g.total_points + p] = r;
    }
    return;
  }
  // S-map (src/edm.cpp:737-814): weighted normal equations, LDL^T when well
  // conditioned, else the JacobiSVD restatement the exact path uses.
  constexpr int n = EA + 1;
  double mean = 0;
  for (int j = 0; j < keff; j++)
    mean = add(mean, cd[j]);
  mean = dvd(mean, (double)keff);
  for (int t = 0; t < g.n_thetas; t++) {
    const double theta = g.thetas[t];
    double A[n * n], bv[n], xs[n];
    for (int a = 0; a < n; a++) {
      for (int b = a; b < n; b++) {
        double s = 0;
        for (int i = 0; i < keff; i++) {
          const double w = exp_rn(mul(-theta, dvd(cd[i], mean)));
          const double xa = a == 0 ? w : mul(w, g.F[(size_t)rows[i] * EA + a - 1]);
          const double xb = b == 0 ? w : mul(w, g.F[(size_t)rows[i] * EA + b - 1]);
          s = add(s, mul(xa, xb));
        }
        A[a * n + b] = s;
        A[b * n + a] = s;
      }
      double s = 0;
      for (int i = 0; i < keff; i++) {
        const double w = exp_rn(mul(-theta, dvd(cd[i], mean)));
        const double xa = a == 0 ? w : mul(w, g.F[(size_t)rows[i] * EA + a - 1]);
        s = add(s, mul(xa, mul(w, g.lib_target[rows[i]])));
      }
      bv[a] = s;
    }
    double L[n * n];
    for (int i = 0; i < n * n; i++)
      L[i] = A[i];
    if (!ldlt_solve(L, bv, xs, n, 1e-7)) {
      double U[n * n], V[n * n], sv[n], tmp[n];
      svd_solve(A, U, V, sv, tmp, bv, xs, n);
    }
    double r = xs[0];
    for (int j = 0; j < EA; j++)
      r = add(r, mul(y[j], xs[j + 1]));
    if (g.coeffs && T.save_coeffs && t == g.n_thetas - 1)
      for (int j = 0; j < n; j++)
        g.coeffs[(size_t)p * n + j] = fabs(xs[j]) < 1.0e-11 ? MISS : xs[j];
    g.pred[(size_t)t * g.total_points + p] = r;
  }
}

template<int EA, int C>
__global__ void __launch_bounds__(TPB, 2) knn_mixed_kernel(GroupParams g, MixedRun m)
{
  constexpr int S = EA <= 4 ? 4 : 8;
  __shared__ __align__(16) float tile[TILE * S];
  __shared__ int s_item;
  const int tid = threadIdx.x;
  for (;;) {
    __syncthreads();
    if (tid == 0)
      s_item = atomicAdd(m.counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= m.n_items)
      return;
    const int2 it = m.items[item];
    const DevTask T = g.tasks[it.x];
    const int pi0 = it.y + tid, pi1 = it.y + tid + TPB;
    const bool a0 = pi0 < T.n_pred, a1 = pi1 < T.n_pred;
    const int prow0 = a0 ? g.pred_rows[T.pred_off + pi0] : 0;
    const int prow1 = a1 ? g.pred_rows[T.pred_off + pi1] : 0;
    float2 ny[EA];
#pragma unroll
    for (int j = 0; j < EA; j++)
      ny[j] = make_float2(a0 ? -m.Fp32[(size_t)prow0 * S + j] : -1e30f, a1 ? -m.Fp32[(size_t)prow1 * S + j] : -1e30f);
    float D0[C], D1[C];
    int I0[C], I1[C];
#pragma unroll
    for (int j = 0; j < C; j++) {
      D0[j] = D1[j] = INFINITY;
      I0[j] = I1[j] = -1;
    }
    int z0 = 0, z1 = 0;
    int zi0[ZCAP], zi1[ZCAP];
#pragma unroll
    for (int j = 0; j < ZCAP; j++)
      zi0[j] = zi1[j] = -1;
    for (int t0 = 0; t0 < T.n_lib; t0 += TILE) {
      const int cnt = min(TILE, T.n_lib - t0);
      __syncthreads();
      for (int i = tid; i < cnt; i += TPB) {
        const int row = g.lib_rows[T.lib_off + t0 + i];
        const float4* src = reinterpret_cast<const float4*>(m.F32 + (size_t)row * S);
        float4* dst = reinterpret_cast<float4*>(tile + i * S);
        dst[0] = src[0];
        if (S == 8)
          dst[1] = src[1];
      }
      __syncthreads();
#pragma unroll 2
      for (int i = 0; i < cnt; i++) {
        const float* xr = tile + i * S;
        float2 df = __fadd2_rn(make_float2(xr[0], xr[0]), ny[0]);
        float2 acc = __fmul2_rn(df, df);
#pragma unroll
        for (int j = 1; j < EA; j++) {
          df = __fadd2_rn(make_float2(xr[j], xr[j]), ny[j]);
          acc = __ffma2_rn(df, df, acc);
        }
        if (acc.x < D0[C - 1] || acc.y < D1[C - 1]) {
          const int li = t0 + i;
          if (acc.x < D0[C - 1]) {
            if (acc.x == 0.f) {
              if (z0 < ZCAP)
                zi0[z0] = li;
              z0++;
            } else {
              topc_insert<C>(D0, I0, acc.x, li);
            }
          }
          if (acc.y < D1[C - 1]) {
            if (acc.y == 0.f) {
              if (z1 < ZCAP)
                zi1[z1] = li;
              z1++;
            } else {
              topc_insert<C>(D1, I1, acc.y, li);
            }
          }
        }
      }
    }
    if (a0)
      finalize_point<EA, C>(g, m, T, T.point_base + pi0, prow0, D0, I0, z0, zi0);
    if (a1)
      finalize_point<EA, C>(g, m, T, T.point_base + pi1, prow1, D1, I1, z1, zi1);
  }
}

template<int EA, int C>
void launch_one(const GroupParams& g, const MixedRun& m, int num_sms, cudaStream_t s)
{
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, knn_mixed_kernel<EA, C>, TPB, 0);
  if (per_sm < 1)
    per_sm = 1;
  long long blocks = (long long)num_sms * per_sm;
  if (blocks > m.n_items)
    blocks = m.n_items;
  if (blocks < 1)
    blocks = 1;
  knn_mixed_kernel<EA, C><<<(int)blocks, TPB, 0, s>>>(g, m);
}

template<int C>
void launch_c(const GroupParams& g, const MixedRun& m, int num_sms, cudaStream_t s)
{
  switch (g.Ea) {
    case 1: launch_one<1, C>(g, m, num_sms, s); break;
    case 2: launch_one<2, C>(g, m, num_sms, s); break;
    case 3: launch_one<3, C>(g, m, num_sms, s); break;
    case 4: launch_one<4, C>(g, m, num_sms, s); break;
    case 5: launch_one<5, C>(g, m, num_sms, s); break;
    case 6: launch_one<6, C>(g, m, num_sms, s); break;
    case 7: launch_one<7, C>(g, m, num_sms, s); break;
    case 8: launch_one<8, C>(g, m, num_sms, s); break;
    default: break;
  }
}

__global__ void center_kernel(const double* F, long long n, int Ea, const double* c, float* F32, int stride)
{
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n * stride;
       i += (long long)gridDim.x * blockDim.x) {
    const long long r = i / stride;
    const int j = (int)(i - r * stride);
    F32[i] = j < Ea ? (float)(F[r * Ea + j] - c[j]) : 0.f;
  }
}

} // namespace

void launch_knn_mixed(const GroupParams& g, const MixedRun& m, int C, int num_sms, cudaStream_t s)
{
  if (m.n_items <= 0)
    return;
  if (C <= 8)
    launch_c<8>(g, m, num_sms, s);
  else
    launch_c<16>(g, m, num_sms, s);
}

void center_to_f32(const double* F, long long n, int Ea, const double* center, float* F32, int stride,
                   cudaStream_t s)
{
  long long total = n * stride;
  long long b = (total + 255) / 256;
  if (b > 8192)
    b = 8192;
  if (b < 1)
    b = 1;
  center_kernel<<<(int)b, 256, 0, s>>>(F, n, Ea, center, F32, stride);
}

} // namespace fedm
