// Device pieces shared by the mixed-precision CCM kernels (kernels_mixed.cu,
// kernels_wide.cu, kernels_one16.cu): work-item scan with FP32 candidate
// lists, the FP64 re-rank that settles a point's neighbour list, and the
// shared-memory hand-off primitives (mbarriers with bounded waits).
// Everything sits in an anonymous namespace, so each translation unit has
// its own copy.
#pragma once

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
// s0: the panel penalty the reference adds first (0, or idw for a row of
// another panel; src/distances.cpp:180-181).
template<int EA>
__device__ __forceinline__ double fp64_sq(const GroupParams& g, int row, const double (&y)[EA], double s0 = 0.0)
{
  const double* x = g.F + (size_t)row * EA;
  double s = s0;
#pragma unroll
  for (int j = 0; j < EA; j++) {
    const double df = sub(x[j], y[j]);
    s = add(s, mul(df, df));
  }
  return s;
}

// FP64 operations of exp_rn: one multiply, fifteen fused multiply-adds (two
// flops each) and the final scaling multiply.
constexpr int EXP_OPS = 32;

// Candidates of one point, handed to the out-of-line FP64 stage.
template<int C>
struct Cand
{
  float D[C];
  int I[C];
  int z;
  int zi[ZCAP];
};

// Settles one point's neighbour list from its FP32 candidates: certifies the
// list against the error margin (else queues the point and its bound for
// knn_refine_kernel), re-scores the candidates in FP64 in the reference's operation
// order, orders them by (distance, library index) -- library order when
// every valid neighbour is used -- and applies the k rules of
// src/edm.cpp:565-639.  Returns true with keff, rows (library manifold rows)
// and cd (their FP64 distances) set when a forecast follows; false when the
// point went on the fallback list or has no valid neighbour.  ops
// accumulates the FP64 operations.
template<int EA, int C>
__device__ __forceinline__ bool prepare_point(const GroupParams& g, const MixedRun& m, const DevTask& T, long long p,
                                              int prow, const Cand<C>& cand, int& keff, int (&rows)[C + ZCAP],
                                              double (&cd)[C + ZCAP], int& ops)
{
  const float(&D)[C] = cand.D;
  const int(&I)[C] = cand.I;
  const int z = cand.z;
  const int(&zi)[ZCAP] = cand.zi;
  const int k = T.k;  // list capacity (the requested k, or the library size for k = all)
  int lc = 0;
#pragma unroll
  for (int j = 0; j < C; j++)
    lc += D[j] < INFINITY ? 1 : 0;
  bool fallback = z > ZCAP;
  // With k kept non-zero values the bound exists even when the list has to
  // fall back (too many zeros, or the C-th value inside it): every row with
  // a non-zero FP32 value is a valid FP64 neighbour, so the k-th true
  // distance is at most the k-th kept row's.  With fewer, the library holds
  // fewer than k non-zero rows and the bound is +inf.
  double thr = INFINITY;
  if (lc >= k) {
    const double sq = sqrt((double)pick(D, k - 1));
    const double hi = sq / sqrt(1.0 - m.gamma) + m.err_abs;
    const double td = (hi * (1.0 + 1e-14) + m.err_abs) * sqrt(1.0 + m.gamma);
    thr = td * td * (1.0 + 1e-14);
    if (lc == C && !((double)D[C - 1] > thr))
      fallback = true;
  }
  if (fallback) {
    // knn_refine_kernel re-scans the library for the rows under thr
    const int slot = atomicAdd(m.fb_count, 1);
    if (slot < m.fb_cap) {
      m.fb_list[slot] = p;
      m.fb_thr[slot] = thr;
    }
    return false;
  }
  double y[EA];
#pragma unroll
  for (int j = 0; j < EA; j++)
    y[j] = g.Fp[(size_t)prow * EA + j];
  // panels with a finite penalty: the reference starts a row of another
  // panel at 0 + idw * 1 = idw, a row of the point's panel at 0
  const bool pen = g.panel_mode && g.idw > 0;
  const int ppan = pen ? g.panel[prow] : 0;
  auto start = [&](int row) { return pen && g.panel[row] != ppan ? g.idw : 0.0; };
  int ci[C + ZCAP];
  int nc = 0;
#pragma unroll
  for (int j = 0; j < C; j++) {
    if (j < lc && (double)D[j] <= thr) {
      const int row = g.lib_rows[T.lib_off + I[j]];
      const double s = fp64_sq<EA>(g, row, y, start(row));
      cd[nc] = __dsqrt_rn(s);
      ci[nc] = I[j];
      nc++;
    }
  }
  int zvalid = 0;
#pragma unroll
  for (int j = 0; j < ZCAP; j++) {
    if (j < z) {
      const int row = g.lib_rows[T.lib_off + zi[j]];
      const double s = fp64_sq<EA>(g, row, y, start(row));
      if (s != 0) {
        cd[nc] = __dsqrt_rn(s);
        ci[nc] = zi[j];
        nc++;
        zvalid++;
      }
    }
  }
  ops += nc * (3 * EA + 1 + (pen ? 2 : 0));
  const int numValid = T.n_lib - z + zvalid;
  const int kr = T.k_req < 0 ? numValid : T.k_req;
  keff = kr < numValid ? kr : numValid;
  if (keff <= 0) {
    // src/edm.cpp:602-606: no forecast; rc(0) SUCCESS, later thetas untouched
    if (g.n_thetas > 1)
      note_rc_m(g, T.task, 8000);
    if (g.kused)
      g.kused[p] = INT_MIN;
    return false;
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
  for (int j = 0; j < keff; j++)
    rows[j] = g.lib_rows[T.lib_off + ci[j]];
  return true;
}

template<int C>
__device__ __forceinline__ void offer(float (&D)[C], int (&I)[C], int& z, int (&zi)[ZCAP], float v, int li)
{
  if (v < D[C - 1]) {
    if (v == 0.f) {
      if (z < ZCAP)
        zi[z] = li;
      z++;
    } else {
      topc_insert<C>(D, I, v, li);
    }
  }
}

// Barrier of the 256 scanning threads: the whole CTA in knn_mixed_kernel,
// named barrier 1 in the warp-specialised kernel (whose solver warps never
// take part in it).
template<bool NAMED>
__device__ __forceinline__ void scan_sync()
{
  if constexpr (NAMED)
    asm volatile("bar.sync 1, %0;" ::"n"(TPB) : "memory");
  else
    __syncthreads();
}

// FP32 scan of one work item: thread tid scores the task's library against
// prediction points first + tid and first + tid + 256 and copies their
// candidate lists to c0 / c1 at the end (the lists live in private arrays
// during the scan, so they stay in registers whatever the caller does with
// c0 / c1).
template<int EA, int C, bool NAMED>
__device__ __forceinline__ void scan_item(const GroupParams& g, const MixedRun& m, const DevTask& T, int first,
                                          int tid, float2* tile, Cand<C>& c0, Cand<C>& c1, int& prow0, int& prow1,
                                          bool& a0, bool& a1)
{
  constexpr int S = EA <= 4 ? 4 : 8;  // row stride of the float manifold
  const int pi0 = first + tid, pi1 = first + tid + TPB;
  a0 = pi0 < T.n_pred;
  a1 = pi1 < T.n_pred;
  prow0 = a0 ? g.pred_rows[T.pred_off + pi0] : 0;
  prow1 = a1 ? g.pred_rows[T.pred_off + pi1] : 0;
  // negated prediction coordinates, duplicated in both halves; an idle slot
  // sits at 1e30 so its squared distances overflow to +inf and never enter
  float2 na[EA], nb[EA];
#pragma unroll
  for (int j = 0; j < EA; j++) {
    const float va = a0 ? -m.Fp32[(size_t)prow0 * S + j] : -1e30f;
    const float vb = a1 ? -m.Fp32[(size_t)prow1 * S + j] : -1e30f;
    na[j] = make_float2(va, va);
    nb[j] = make_float2(vb, vb);
  }
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
    const int npairs = (cnt + 1) >> 1;
    scan_sync<NAMED>();
    for (int i = tid; i < 2 * npairs; i += TPB) {
      float* dst = reinterpret_cast<float*>(tile + (i >> 1) * EA) + (i & 1);
      if (i < cnt) {
        const float* src = m.F32 + (size_t)g.lib_rows[T.lib_off + t0 + i] * S;
#pragma unroll
        for (int j = 0; j < EA; j++)
          dst[2 * j] = src[j];
      } else {
#pragma unroll
        for (int j = 0; j < EA; j++)
          dst[2 * j] = 1e30f;  // padding row: never a candidate
      }
    }
    scan_sync<NAMED>();
#pragma unroll 2
    for (int ip = 0; ip < npairs; ip++) {
      const float2* xr = tile + ip * EA;
      float2 x = xr[0];
      float2 da = __fadd2_rn(x, na[0]);
      float2 db = __fadd2_rn(x, nb[0]);
      float2 sa = __fmul2_rn(da, da);
      float2 sb = __fmul2_rn(db, db);
#pragma unroll
      for (int j = 1; j < EA; j++) {
        x = xr[j];
        da = __fadd2_rn(x, na[j]);
        db = __fadd2_rn(x, nb[j]);
        sa = __ffma2_rn(da, da, sa);
        sb = __ffma2_rn(db, db, sb);
      }
      if (fminf(sa.x, sa.y) < D0[C - 1] || fminf(sb.x, sb.y) < D1[C - 1]) {
        const int li = t0 + 2 * ip;
        offer<C>(D0, I0, z0, zi0, sa.x, li);
        offer<C>(D0, I0, z0, zi0, sa.y, li + 1);
        offer<C>(D1, I1, z1, zi1, sb.x, li);
        offer<C>(D1, I1, z1, zi1, sb.y, li + 1);
      }
    }
  }
#pragma unroll
  for (int j = 0; j < C; j++) {
    c0.D[j] = D0[j];
    c0.I[j] = I0[j];
    c1.D[j] = D1[j];
    c1.I[j] = I1[j];
  }
  c0.z = z0;
  c1.z = z1;
#pragma unroll
  for (int j = 0; j < ZCAP; j++) {
    c0.zi[j] = zi0[j];
    c1.zi[j] = zi1[j];
  }
}

__device__ __forceinline__ void add_ops(const MixedRun& m, unsigned long long ops)
{
  // called by whole warps
  if (m.fp64_ops) {
    for (int o = 16; o > 0; o >>= 1)
      ops += __shfl_xor_sync(0xffffffffu, ops, o);
    if ((threadIdx.x & 31) == 0)
      atomicAdd(m.fp64_ops, ops);
  }
}

// Adds the warp's count of scored (prediction, library row) pairs to the
// run's counter; called by whole warps.
__device__ __forceinline__ void add_scanned(const MixedRun& m, unsigned long long n)
{
  if (m.scanned) {
    for (int o = 16; o > 0; o >>= 1)
      n += __shfl_xor_sync(0xffffffffu, n, o);
    if ((threadIdx.x & 31) == 0)
      atomicAdd(m.scanned, n);
  }
}

template<int C>
struct Job
{
  Cand<C> c;
  long long p;  // global point id, -1 for an idle slot
  int prow;
};

constexpr unsigned long long WAIT_NS = 5000000000ULL;

__device__ __forceinline__ unsigned long long globaltimer_ns()
{
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, int count)
{
  const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(unsigned long long* bar)
{
  const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(a) : "memory");
}

// Waits for the completion of the phase with the given parity; false after
// WAIT_NS nanoseconds (or 2^30 polls) without it.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, int parity)
{
  const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
  unsigned long long t0 = 0;
  for (unsigned n = 0; n < (1u << 30); n++) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok)
      return true;
    if ((n & 31) == 0) {
      const unsigned long long t = globaltimer_ns();
      if (t0 == 0)
        t0 = t;
      else if (t - t0 > WAIT_NS)
        return false;
    }
  }
  return false;
}

// AND of v over the N threads of named barrier ID (a barrier as well), so a
// role takes the same branch on every thread even if one thread's wait ran out.
template<int ID, int N>
__device__ __forceinline__ bool group_and(bool v)
{
  unsigned r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 q, %1, 0;\n\tbar.red.and.pred p, %2, %3, q;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(r)
      : "r"((unsigned)v), "n"(ID), "n"(N)
      : "memory");
  return r != 0;
}

constexpr size_t SMEM_LIMIT = 227 * 1024;


template<int EA>
__device__ __noinline__ int smap_point_local(const GroupParams& g, long long p, int prow, bool save, int keff,
                                             const int* rows, const double* cd);
template<int EA>
__device__ __noinline__ int smap_point_sm(const GroupParams& g, long long p, int prow, bool save, int keff,
                                          const int* rows, const double* cd, double* uv, int uv_stride);

// Returns the number of FP64 add/sub/mul/div/sqrt operations it performed.
// uv, when given, is this thread's shared-memory slice for the S-map solver's
// rotation accumulators (2 (EA+1)^2 doubles, interleaved with stride
// uv_stride).
template<int EA, int C, int ALG, bool UVS = false>
__device__ __noinline__ int finalize_point(const GroupParams& g, const MixedRun& m, const DevTask& T, long long p,
                                           int prow, const Cand<C>& cand, double* uv = nullptr, int uv_stride = 0)
{
  int keff = 0, ops = 0;
  int rows[C + ZCAP];
  double cd[C + ZCAP];
  if (!prepare_point<EA, C>(g, m, T, p, prow, cand, keff, rows, cd, ops))
    return ops;
  if constexpr (ALG == 0) {
    // simplex (src/edm.cpp:707-735)
    double minD = cd[0];
    for (int j = 1; j < keff; j++)
      minD = cd[j] < minD ? cd[j] : minD;
    double rel[C + ZCAP], tg[C + ZCAP];
    const double ymin = rcp(minD);
    for (int j = 0; j < keff; j++) {
      rel[j] = dvd_r(cd[j], minD, ymin);
      tg[j] = g.lib_target[rows[j]];
    }
    for (int t = 0; t < g.n_thetas; t++) {
      const double theta = g.thetas[t];
      double w[C + ZCAP];
      double sumw = 0.0;
      for (int j = 0; j < keff; j++) {
        w[j] = exp_rn(mul(-theta, rel[j]));
        sumw = add(sumw, w[j]);
      }
      double r = 0.0;
      const double ysum = rcp(sumw);
      for (int j = 0; j < keff; j++)
        r = add(r, mul(tg[j], dvd_r(w[j], sumw, ysum)));
      g.pred[(size_t)t * g.total_points + p] = r;
    }
    return ops + keff + g.n_thetas * keff * (EXP_OPS + 5);
  }
  else {
    if constexpr (UVS)
      return ops + smap_point_sm<EA>(g, p, prow, T.save_coeffs != 0, keff, rows, cd, uv, uv_stride);
    else
      return ops + smap_point_local<EA>(g, p, prow, T.save_coeffs != 0, keff, rows, cd);
  }
}

// The same forecast with the solver's matrices in per-thread local memory;
// used inside the scan kernel, whose register budget (two 256-thread CTAs
// per SM) leaves no room for them.  Identical operations and bits.
template<int EA>
__device__ __noinline__ int smap_point_local(const GroupParams& g, long long p, int prow, bool save, int keff,
                                             const int* rows, const double* cd)
{
  constexpr int n = EA + 1;
  // mean; per theta: weights and the normal equations per neighbour, the
  // forecast (the SVD counts its own)
  int ops = keff + 1 + g.n_thetas * (keff * (EXP_OPS + 2 + n + n * (n + 1) + 2 * n) + 2 * EA);
  double y[EA];
#pragma unroll
  for (int j = 0; j < EA; j++)
    y[j] = g.Fp[(size_t)prow * EA + j];
  double mean = 0;
  for (int j = 0; j < keff; j++)
    mean = add(mean, cd[j]);
  mean = dvd(mean, (double)keff);
  const double ymean = rcp(mean);
  for (int t = 0; t < g.n_thetas; t++) {
    const double theta = g.thetas[t];
    double W[n * n], bv[n], xs[n], U[n * n], V[n * n], sv[n], tmp[n];
    for (int e = 0; e < n * n; e++)
      W[e] = 0;
    for (int a = 0; a < n; a++)
      bv[a] = 0;
    for (int i = 0; i < keff; i++) {
      const double w = exp_rn(mul(-theta, dvd_r(cd[i], mean, ymean)));
      const int row = rows[i];
      double xr[n];
      xr[0] = w;
#pragma unroll
      for (int j = 1; j < n; j++)
        xr[j] = mul(w, g.F[(size_t)row * EA + j - 1]);
      const double yl = mul(w, g.lib_target[row]);
#pragma unroll
      for (int a = 0; a < n; a++) {
#pragma unroll
        for (int b = a; b < n; b++)
          W[a * n + b] = add(W[a * n + b], mul(xr[a], xr[b]));
        bv[a] = add(bv[a], mul(xr[a], yl));
      }
    }
    for (int a = 0; a < n; a++)
      for (int b = 0; b < a; b++)
        W[a * n + b] = W[b * n + a];
    svd_solve(W, U, V, sv, tmp, bv, xs, n, ops);
    double r = xs[0];
#pragma unroll
    for (int j = 0; j < EA; j++)
      r = add(r, mul(y[j], xs[j + 1]));
    if (g.coeffs && save && t == g.n_thetas - 1) {
      for (int j = 0; j < n; j++)
        g.coeffs[(size_t)p * n + j] = fabs(xs[j]) < 1.0e-11 ? MISS : xs[j];
    }
    g.pred[(size_t)t * g.total_points + p] = r;
  }
  return ops;
}

} // namespace

} // namespace fedm
