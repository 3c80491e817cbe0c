// Differentiable S-map: forecast, one-step MSE and its gradient with respect
// to theta and to per-lag embedding weights w (no counterpart in the
// reference, which has no gradients).  The forward pass is the reference's
// S-map over every library neighbour (src/edm.cpp:737-814 with k = all) on
// coordinates z = w * m; at w = 1 the distances are the reference's bits.
//
// Per prediction point p (one warp, library rows lane-strided):
//   pass 1  d_i = |z_i - z_p| (zero distances excluded, src/distances.cpp:218),
//           mu = mean d, dmu/dw_j = mean (z_ij - z_pj)(m_ij - m_pj) / d_i
//   pass 2  a_i^2 = exp(-2 theta d_i / mu), A = sum a^2 u u^T, b = sum a^2 u t
//           with u_i = [1, z_i]; c = A^+ b, g = A^+ v (v = [1, z_p]), by the
//           JacobiSVD restatement; yhat = v.c
//   pass 3  s_i = g.u_i, e_i = t_i - u_i.c and the sums
//           Q = sum a^2 s e d, R_j = sum a^2 s e dd_i/dw_j,
//           S_j = sum a^2 e m_ij, T_j = sum a^2 s m_ij
//   dyhat/dtheta = -(2/mu) Q
//   dyhat/dw_j  = m_pj c_{j+1} - (2 theta/mu) R_j + (2 theta dmu/dw_j/mu^2) Q
//                 + g_{j+1} S_j - c_{j+1} T_j
// (from dyhat = dv.c + g.(db - dA c), A symmetric).  Each point writes r,
// yhat, dyhat/dtheta and dyhat/dw; the host composes the objective's
// gradient (MSE or rho) from them in a fixed order.
//
// Only the distances follow the reference's rounding: the sums over the
// library are lane-strided and warp-reduced, so the forecast agrees with the
// reference's k = all S-map to reduction-order rounding, not bit for bit.
// The passes therefore use what the FP64 pipe does cheaply: one reciprocal
// of d per row instead of a division per lag, a2 = exp(-2 theta d / mu) in
// one call, and fused multiply-adds for the normal equations and the
// adjoint sums.
//
// The FP64 pipe bounds the kernel, and HBM has room: the grid is persistent
// (one warp per point at a time, points strided over the warps) and each
// warp owns a slice of device memory for its point's per-row values.  At
// cache level 2 pass 1 stores d_i, 1/d_i and the products
// (z_ij - z_pj)(m_ij - m_pj), and pass 2 (reading d_i) stores a_i^2, so that
// pass 3 reads them instead of recomputing the distance, the exponential and
// the products;
// at level 1 (a library too large for level 2's budget) only d_i and a_i^2
// are kept; at level 0 (larger still) every pass recomputes.  The scaled
// library z = w * m is formed once per call.  The cached values are the ones
// the passes would recompute, so every level gives the same bits.
#include <algorithm>
#include <cfloat>

#include "kernels.h"
#include "smap_solve.cuh"

namespace fedm {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int GRAD_NT = 128;  // threads per CTA: four warps, one point each at a time

__device__ __forceinline__ double wsum(double v)
{
  for (int o = 16; o > 0; o >>= 1)
    v += __shfl_xor_sync(FULL, v, o);
  return v;
}

// z = w * m for every library row: the product pass 1 forms for its
// distance, so the distances keep their bits
__global__ void scale_rows_kernel(const double* lib, const double* w, long long n, int ea, double* z)
{
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    z[i] = mul(w[i % ea], lib[i]);
}

// Doubles per library row of a warp's cache slice at each level.
template<int EA, int CACHE>
__host__ __device__ constexpr int cache_per_row() { return CACHE == 2 ? 3 + EA : CACHE == 1 ? 2 : 0; }

// The three passes for prediction point pnt, by one warp.  cache: this
// warp's slice, n_lib rows per array: d, a^2 (level >= 1), then 1/d and the
// EA products (level 2).
template<int EA, int CACHE>
__device__ __forceinline__ void grad_point(const AdjointParams& a, long long pnt, int lane, double* cache)
{
  const int nl = a.n_lib;
  constexpr int n = EA + 1;
  constexpr int NA = n * (n + 1) / 2;
  double w[EA], y[EA], zp[EA];
#pragma unroll
  for (int j = 0; j < EA; j++) {
    w[j] = a.w[j];
    y[j] = a.pred[(size_t)pnt * EA + j];
    zp[j] = mul(w[j], y[j]);
  }
  // the distance of row i in the reference's operation order (unfused), so
  // at w = 1 it is the same bits as src/distances.cpp:176-225; 0 for an
  // excluded (zero) distance
  auto distance = [&](int i, double* diff) {
    const double* z = a.z + (size_t)i * EA;
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < EA; j++) {
      diff[j] = sub(z[j], zp[j]);
      s = add(s, mul(diff[j], diff[j]));
    }
    return s != 0 ? __dsqrt_rn(s) : 0.0;
  };
  // pass 1: distances, their mean and its derivative
  double sd = 0, dmu[EA];
  int cnt = 0;
#pragma unroll
  for (int j = 0; j < EA; j++)
    dmu[j] = 0;
  for (int i = lane; i < a.n_lib; i += 32) {
    const double* m = a.lib + (size_t)i * EA;
    double diff[EA];
    const double d = distance(i, diff);
    if constexpr (CACHE >= 1)
      cache[i] = d;
    if (d != 0) {
      const double inv = __drcp_rn(d);
      sd += d;
      cnt++;
      if constexpr (CACHE == 2)
        cache[2 * nl + i] = inv;
#pragma unroll
      for (int j = 0; j < EA; j++) {
        const double q = diff[j] * (m[j] - y[j]);
        if constexpr (CACHE == 2)
          cache[(3 + j) * nl + i] = q;
        dmu[j] = fma(q, inv, dmu[j]);
      }
    }
  }
  const double total = wsum(sd);
  const double nv = (double)__reduce_add_sync(FULL, cnt);
  const double mu = total / nv;
  const double c2 = -2.0 * a.theta / mu;  // a^2 = exp(c2 d)
#pragma unroll
  for (int j = 0; j < EA; j++)
    dmu[j] = wsum(dmu[j]) / nv;
  // pass 2: normal equations
  double A[NA], b[n];
#pragma unroll
  for (int e = 0; e < NA; e++)
    A[e] = 0;
#pragma unroll
  for (int e = 0; e < n; e++)
    b[e] = 0;
  for (int i = lane; i < a.n_lib; i += 32) {
    double d;
    if constexpr (CACHE >= 1) {
      d = cache[i];
    } else {
      double diff[EA];
      d = distance(i, diff);
    }
    if (d == 0)
      continue;
    const double a2 = exp(c2 * d);
    if constexpr (CACHE >= 1)
      cache[nl + i] = a2;
    const double* z = a.z + (size_t)i * EA;
    double u[n];
    u[0] = 1.0;
#pragma unroll
    for (int j = 0; j < EA; j++)
      u[j + 1] = z[j];
    const double t = a.lib_t[i];
    int e = 0;
#pragma unroll
    for (int r = 0; r < n; r++) {
      const double au = a2 * u[r];
#pragma unroll
      for (int c = r; c < n; c++) {
        A[e] = fma(au, u[c], A[e]);
        e++;
      }
      b[r] = fma(au, t, b[r]);
    }
  }
#pragma unroll
  for (int e = 0; e < NA; e++)
    A[e] = wsum(A[e]);
#pragma unroll
  for (int e = 0; e < n; e++)
    b[e] = wsum(b[e]);
  double c[n], gv[n];
  {
    // every lane solves the same system (identical inputs, identical bits)
    double W[n * n], U[n * n], V[n * n], sv[n], tmp[n], v[n];
    int e = 0;
    for (int r = 0; r < n; r++)
      for (int cc = r; cc < n; cc++) {
        W[r * n + cc] = A[e];
        W[cc * n + r] = A[e];
        e++;
      }
    svd_solve(W, U, V, sv, tmp, b, c, n);
    e = 0;
    for (int r = 0; r < n; r++)
      for (int cc = r; cc < n; cc++) {
        W[r * n + cc] = A[e];
        W[cc * n + r] = A[e];
        e++;
      }
    v[0] = 1.0;
#pragma unroll
    for (int j = 0; j < EA; j++)
      v[j + 1] = zp[j];
    svd_solve(W, U, V, sv, tmp, v, gv, n);
  }
  double yhat = c[0];
#pragma unroll
  for (int j = 0; j < EA; j++)
    yhat += zp[j] * c[j + 1];
  const double r = yhat - a.pred_t[pnt];
  double* out = a.out + (size_t)pnt * (EA + 3);
  if (!a.backward) {
    if (lane == 0) {
      out[0] = r;
      out[1] = yhat;
    }
    return;
  }
  // pass 3: adjoint sums
  double Q = 0, R[EA], S[EA], Tt[EA];
#pragma unroll
  for (int j = 0; j < EA; j++)
    R[j] = S[j] = Tt[j] = 0;
  for (int i = lane; i < a.n_lib; i += 32) {
    const double* m = a.lib + (size_t)i * EA;
    const double* z = a.z + (size_t)i * EA;
    double q[EA], d, a2, inv;
    if constexpr (CACHE == 2) {
      d = cache[i];
      if (d == 0)
        continue;
      a2 = cache[nl + i];
      inv = cache[2 * nl + i];
#pragma unroll
      for (int j = 0; j < EA; j++)
        q[j] = cache[(3 + j) * nl + i];
    } else {
      double diff[EA];
      if constexpr (CACHE == 1) {
        d = cache[i];
        if (d == 0)
          continue;
        a2 = cache[nl + i];
#pragma unroll
        for (int j = 0; j < EA; j++)
          diff[j] = sub(z[j], zp[j]);
      } else {
        d = distance(i, diff);
        if (d == 0)
          continue;
        a2 = exp(c2 * d);
      }
      inv = __drcp_rn(d);
#pragma unroll
      for (int j = 0; j < EA; j++)
        q[j] = diff[j] * (m[j] - y[j]);
    }
    double u[n];
    u[0] = 1.0;
#pragma unroll
    for (int j = 0; j < EA; j++)
      u[j + 1] = z[j];
    double su = 0, uc = 0;
#pragma unroll
    for (int k = 0; k < n; k++) {
      su = fma(gv[k], u[k], su);
      uc = fma(u[k], c[k], uc);
    }
    const double ei = a.lib_t[i] - uc;
    const double ae = a2 * ei, as = a2 * su;
    const double ase = as * ei;
    Q = fma(ase, d, Q);
    const double ased = ase * inv;
#pragma unroll
    for (int j = 0; j < EA; j++) {
      R[j] = fma(ased, q[j], R[j]);
      S[j] = fma(ae, m[j], S[j]);
      Tt[j] = fma(as, m[j], Tt[j]);
    }
  }
  Q = wsum(Q);
#pragma unroll
  for (int j = 0; j < EA; j++) {
    R[j] = wsum(R[j]);
    S[j] = wsum(S[j]);
    Tt[j] = wsum(Tt[j]);
  }
  if (lane == 0) {
    out[0] = r;
    out[1] = yhat;
    out[2] = -(2 / mu) * Q;
#pragma unroll
    for (int j = 0; j < EA; j++)
      out[3 + j] = y[j] * c[j + 1] - (2 * a.theta / mu) * R[j] + (2 * a.theta * dmu[j] / (mu * mu)) * Q +
                   gv[j + 1] * S[j] - c[j + 1] * Tt[j];
  }
}

template<int EA, int CACHE>
__global__ void __launch_bounds__(GRAD_NT, 3) smap_grad_kernel(AdjointParams a)
{
  const int lane = threadIdx.x & 31;
  const long long warp = (long long)blockIdx.x * (GRAD_NT / 32) + (threadIdx.x >> 5);
  const long long warps = (long long)gridDim.x * (GRAD_NT / 32);
  double* cache = CACHE ? a.cache + warp * cache_per_row<EA, CACHE>() * (long long)a.n_lib : nullptr;
  for (long long pnt = warp; pnt < a.n_pred; pnt += warps)
    grad_point<EA, CACHE>(a, pnt, lane, cache);
}

template<int EA, int CACHE>
void launch_grad_level(const AdjointParams& a, int num_sms, cudaStream_t s)
{
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, smap_grad_kernel<EA, CACHE>, GRAD_NT, 0);
  long long blocks = (long long)num_sms * std::max(per_sm, 1);
  blocks = std::min(blocks, (long long)(a.n_pred + GRAD_NT / 32 - 1) / (GRAD_NT / 32));
  if (CACHE)
    blocks = std::min(blocks, a.cache_warps / (GRAD_NT / 32));
  if (blocks < 1)
    return;
  smap_grad_kernel<EA, CACHE><<<(int)blocks, GRAD_NT, 0, s>>>(a);
}

template<int EA>
void launch_grad(const AdjointParams& a, int num_sms, cudaStream_t s)
{
  if (a.cache && a.cache_level == 2)
    launch_grad_level<EA, 2>(a, num_sms, s);
  else if (a.cache && a.cache_level == 1)
    launch_grad_level<EA, 1>(a, num_sms, s);
  else
    launch_grad_level<EA, 0>(a, num_sms, s);
}

} // namespace

int grad_cache_warps(int e_actual, int num_sms)
{
  int per_sm = 0;
  switch (e_actual) {
#define FEDM_GRAD_OCC(E)                                                                                     \
  case E: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, smap_grad_kernel<E, 2>, GRAD_NT, 0); break;
    FEDM_GRAD_OCC(1) FEDM_GRAD_OCC(2) FEDM_GRAD_OCC(3) FEDM_GRAD_OCC(4)
    FEDM_GRAD_OCC(5) FEDM_GRAD_OCC(6) FEDM_GRAD_OCC(7) FEDM_GRAD_OCC(8)
#undef FEDM_GRAD_OCC
    default: break;
  }
  return num_sms * std::max(per_sm, 1) * (GRAD_NT / 32);
}

void launch_smap_grad(const AdjointParams& a, int num_sms, cudaStream_t s)
{
  if (a.n_pred <= 0 || a.n_lib <= 0)
    return;
  const long long n = (long long)a.n_lib * a.e_actual;
  const int zb = (int)std::min<long long>((n + 255) / 256, (long long)num_sms * 8);
  scale_rows_kernel<<<zb, 256, 0, s>>>(a.lib, a.w, n, a.e_actual, a.z);
  switch (a.e_actual) {
    case 1: launch_grad<1>(a, num_sms, s); break;
    case 2: launch_grad<2>(a, num_sms, s); break;
    case 3: launch_grad<3>(a, num_sms, s); break;
    case 4: launch_grad<4>(a, num_sms, s); break;
    case 5: launch_grad<5>(a, num_sms, s); break;
    case 6: launch_grad<6>(a, num_sms, s); break;
    case 7: launch_grad<7>(a, num_sms, s); break;
    case 8: launch_grad<8>(a, num_sms, s); break;
    default: break;
  }
}

} // namespace fedm
