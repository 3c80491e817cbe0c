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
// adjoint sums.  The weights are recomputed in pass 3, not stored.
#include <cfloat>

#include "kernels.h"
#include "smap_solve.cuh"

namespace fedm {

namespace {

constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ double wsum(double v)
{
  for (int o = 16; o > 0; o >>= 1)
    v += __shfl_xor_sync(FULL, v, o);
  return v;
}

template<int EA>
__global__ void __launch_bounds__(128) smap_grad_kernel(AdjointParams a)
{
  constexpr int n = EA + 1;
  constexpr int NA = n * (n + 1) / 2;
  const int lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  const int pnt = blockIdx.x * wpb + (threadIdx.x >> 5);
  if (pnt >= a.n_pred)
    return;
  double w[EA], y[EA], zp[EA];
#pragma unroll
  for (int j = 0; j < EA; j++) {
    w[j] = a.w[j];
    y[j] = a.pred[(size_t)pnt * EA + j];
    zp[j] = mul(w[j], y[j]);
  }
  // pass 1: distances, their mean and its derivative
  double sd = 0, dmu[EA];
  int cnt = 0;
#pragma unroll
  for (int j = 0; j < EA; j++)
    dmu[j] = 0;
  for (int i = lane; i < a.n_lib; i += 32) {
    const double* m = a.lib + (size_t)i * EA;
    // distance in the reference's operation order (unfused), so at w = 1 it
    // is the same bits as src/distances.cpp:176-225
    double diff[EA], s = 0.0;
#pragma unroll
    for (int j = 0; j < EA; j++) {
      diff[j] = sub(mul(w[j], m[j]), zp[j]);
      s = add(s, mul(diff[j], diff[j]));
    }
    if (s != 0) {
      const double d = __dsqrt_rn(s);
      const double inv = __drcp_rn(d);
      sd += d;
      cnt++;
#pragma unroll
      for (int j = 0; j < EA; j++)
        dmu[j] = fma(diff[j] * (m[j] - y[j]), inv, dmu[j]);
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
    const double* m = a.lib + (size_t)i * EA;
    double u[n], s = 0.0;
    u[0] = 1.0;
#pragma unroll
    for (int j = 0; j < EA; j++) {
      u[j + 1] = mul(w[j], m[j]);
      const double df = sub(u[j + 1], zp[j]);
      s = add(s, mul(df, df));
    }
    if (s == 0)
      continue;
    const double a2 = exp(c2 * __dsqrt_rn(s));
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
    double u[n], diff[EA], s = 0.0;
    u[0] = 1.0;
#pragma unroll
    for (int j = 0; j < EA; j++) {
      u[j + 1] = mul(w[j], m[j]);
      diff[j] = sub(u[j + 1], zp[j]);
      s = add(s, mul(diff[j], diff[j]));
    }
    if (s == 0)
      continue;
    const double d = __dsqrt_rn(s);
    const double a2 = exp(c2 * d);
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
    const double ased = ase * __drcp_rn(d);
#pragma unroll
    for (int j = 0; j < EA; j++) {
      R[j] = fma(ased, diff[j] * (m[j] - y[j]), R[j]);
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

} // namespace

void launch_smap_grad(const AdjointParams& a, cudaStream_t s)
{
  const int blocks = (a.n_pred + 3) / 4;
  if (blocks <= 0)
    return;
  switch (a.e_actual) {
    case 1: smap_grad_kernel<1><<<blocks, 128, 0, s>>>(a); break;
    case 2: smap_grad_kernel<2><<<blocks, 128, 0, s>>>(a); break;
    case 3: smap_grad_kernel<3><<<blocks, 128, 0, s>>>(a); break;
    case 4: smap_grad_kernel<4><<<blocks, 128, 0, s>>>(a); break;
    case 5: smap_grad_kernel<5><<<blocks, 128, 0, s>>>(a); break;
    case 6: smap_grad_kernel<6><<<blocks, 128, 0, s>>>(a); break;
    case 7: smap_grad_kernel<7><<<blocks, 128, 0, s>>>(a); break;
    case 8: smap_grad_kernel<8><<<blocks, 128, 0, s>>>(a); break;
    default: break;
  }
}

} // namespace fedm
