// Mixed-precision neighbour search and forecast (the CCM hot path).
//
// Work item = one task x 512 prediction points (256 in the one-point form of
// kernels_wide.cu), taken from a global queue in decreasing library size.  A
// 256-thread CTA stages 1024 library rows of the centred FP32 manifold in
// shared memory at a time; every thread scores them against two prediction
// points and keeps, per point, the C smallest squared FP32 distances (sorted,
// registers) plus up to two exact zeros.
//
// Certification.  With u = 2^-24, the FP32 squared distance s of a pair obeys
// sqrt(s)/sqrt(1+g) - e <= D <= sqrt(s)/sqrt(1-g) + e, where D is the exact
// distance of the FP64 rows, g = (Ea+2)*2^-23 bounds the FP32 subtraction,
// squares and accumulation ((Ea+3)u suffices), and e bounds the input
// rounding: each centred coordinate A_i reaches FP32 as A_i(1+d), |d| <=
// u(1+2^-29) (the FP64 centring adds 2^-53), so the difference vector moves
// by at most u(1+2^-29)(|A|+|B|) <= 2u(1+2^-29) R with R >= every centred row
// norm (the engine takes 1.01 times the norm of its bounding box's farthest
// corner).  The engine sets e = 2^-22 R, twice that bound.
// The k-th true distance is at most hi = sqrt(s_k)/sqrt(1-g) + e, so every
// true neighbour has s <= T = ((hi + e) * sqrt(1+g))^2 (widened by 1e-14).
// If the C-th kept value exceeds T, every entry at or under T is in the list;
// otherwise the point goes on a fallback list with its T, and
// knn_refine_kernel re-scans the library for the rows under T (the exact
// kernels take a point with more than 1024 of them).  Entries under T are
// re-scored in FP64 with the reference's operation order
// (src/distances.cpp:194-225), so neighbour distances and their
// (distance, index) order are the FP64 bits.  A positive FP32 distance implies
// a positive FP64 one; FP32 zeros are re-scored and dropped when the FP64
// distance is zero too (src/distances.cpp:218).
#include "mixed_common.cuh"
#include "smap_solve_n.cuh"

namespace fedm {

namespace {


template<int EA, int C, int ALG>
__global__ void __launch_bounds__(TPB, 2) knn_mixed_kernel(GroupParams g, MixedRun m)
{
  // library rows staged as interleaved pairs: tile[pair][dim] = (row 2i, row 2i+1)
  __shared__ __align__(16) float2 tile[(TILE / 2) * EA];
  __shared__ int s_item;
  const int tid = threadIdx.x;
  unsigned long long ops = 0;
  for (;;) {
    __syncthreads();
    if (tid == 0)
      s_item = m.item_begin + atomicAdd(m.counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= m.item_end) {
      add_ops(m, ops);  // every thread of the CTA leaves here together
      return;
    }
    const int2 it = m.items[item];
    const DevTask T = g.tasks[it.x];
    Cand<C> c0, c1;
    int prow0, prow1;
    bool a0, a1;
    scan_item<EA, C, false>(g, m, T, it.y, tid, tile, c0, c1, prow0, prow1, a0, a1);
    if (a0) {
      const Cand<C> c = c0;
      ops += finalize_point<EA, C, ALG>(g, m, T, T.point_base + it.y + tid, prow0, c);
    }
    if (a1) {
      const Cand<C> c = c1;
      ops += finalize_point<EA, C, ALG>(g, m, T, T.point_base + it.y + tid + TPB, prow1, c);
    }
  }
}

// ---------------------------------------------------------------------------
// Warp-specialised S-map kernel.  Warps 0-7 scan (FP32 pipe) and warps 8.. run
// the FP64 re-rank and JacobiSVD solve (FP64 pipe) of the previous item, so the
// two pipes work at the same time.  The scan warps hand each item's 512
// candidate lists over through two shared-memory job buffers guarded by
// mbarriers ("full": 256 scanner arrivals; "empty": one arrival per solver
// thread).  Every wait is bounded: past WAIT_NS the waiter sets m.error and
// leaves, so a broken hand-off ends the kernel with an error instead of a hang.


template<int EA, int C>
__host__ __device__ constexpr size_t ws_base_bytes()
{
  return (size_t)(TILE / 2) * EA * sizeof(float2) + 2 * (size_t)(2 * TPB) * sizeof(Job<C>);
}

// The solver threads' U and V (2 (EA+1)^2 doubles each) go to shared memory
// when they fit beside the tile and the job buffers (E_a = 4: 100 KB for 256
// solver threads); otherwise the solver keeps them in local memory.
template<int EA, int C, int SW>
__host__ __device__ constexpr bool ws_uv_in_smem()
{
  return ws_base_bytes<EA, C>() + (size_t)2 * (EA + 1) * (EA + 1) * 32 * SW * sizeof(double) + 1024 <= SMEM_LIMIT;
}

template<int EA, int C, int SW>
__host__ __device__ constexpr size_t ws_smem_bytes()
{
  return ws_base_bytes<EA, C>() +
         (ws_uv_in_smem<EA, C, SW>() ? (size_t)2 * (EA + 1) * (EA + 1) * 32 * SW * sizeof(double) : 0);
}

template<int EA, int C, int SW>
__global__ void __launch_bounds__(TPB + 32 * SW, 1) knn_smap_ws_kernel(GroupParams g, MixedRun m)
{
  constexpr int NS = 32 * SW;  // solver threads
  constexpr int JOBS = 2 * TPB;
  extern __shared__ __align__(16) unsigned char smem[];
  float2* tile = reinterpret_cast<float2*>(smem);
  Job<C>* jobs = reinterpret_cast<Job<C>*>(smem + (size_t)(TILE / 2) * EA * sizeof(float2));
  double* uv_all = reinterpret_cast<double*>(smem + ws_base_bytes<EA, C>());
  __shared__ unsigned long long full_bar[2], empty_bar[2];
  __shared__ DevTask s_task[2];
  __shared__ int s_end[2];
  __shared__ int s_item;
  const int tid = threadIdx.x;
  if (tid == 0) {
    mbar_init(&full_bar[0], TPB);
    mbar_init(&full_bar[1], TPB);
    mbar_init(&empty_bar[0], NS);
    mbar_init(&empty_bar[1], NS);
  }
  __syncthreads();
  unsigned long long ops = 0;
  if (tid < TPB) {
    for (int it = 0;; it++) {
      const int b = it & 1, k = it >> 1;
      scan_sync<true>();  // everyone has read the previous s_item
      if (tid == 0)
        s_item = m.item_begin + atomicAdd(m.counter, 1);
      scan_sync<true>();
      const int item = s_item;
      // buffer b is free once the solvers finished its previous use (the
      // first use waits on the phase before the barrier's first one, which
      // counts as complete)
      if (!group_and<1, TPB>(mbar_wait(&empty_bar[b], (k & 1) ^ 1))) {
        if (tid == 0)
          atomicExch(m.error, 1);
        break;
      }
      if (item >= m.item_end) {
        if (tid == 0)
          s_end[b] = 1;
        mbar_arrive(&full_bar[b]);
        break;
      }
      const int2 iv = m.items[item];
      const DevTask T = g.tasks[iv.x];
      if (tid == 0) {
        s_task[b] = T;
        s_end[b] = 0;
      }
      Job<C>& j0 = jobs[b * JOBS + tid];
      Job<C>& j1 = jobs[b * JOBS + tid + TPB];
      int prow0, prow1;
      bool a0, a1;
      Cand<C> c0, c1;
      scan_item<EA, C, true>(g, m, T, iv.y, tid, tile, c0, c1, prow0, prow1, a0, a1);
      j0.c = c0;
      j0.p = a0 ? T.point_base + iv.y + tid : -1;
      j0.prow = prow0;
      j1.c = c1;
      j1.p = a1 ? T.point_base + iv.y + tid + TPB : -1;
      j1.prow = prow1;
      mbar_arrive(&full_bar[b]);
    }
  } else {
    const int st = tid - TPB;
    constexpr bool UVS = ws_uv_in_smem<EA, C, SW>();
    double* uv = UVS ? uv_all + st : nullptr;
    for (int it = 0;; it++) {
      const int b = it & 1, k = it >> 1;
      if (!group_and<2, NS>(mbar_wait(&full_bar[b], k & 1))) {
        if (st == 0)
          atomicExch(m.error, 1);
        break;
      }
      if (s_end[b])
        break;
      const DevTask T = s_task[b];
      for (int j = st; j < JOBS; j += NS) {
        const Job<C>& jb = jobs[b * JOBS + j];
        if (jb.p >= 0)
          ops += finalize_point<EA, C, 1, UVS>(g, m, T, jb.p, jb.prow, jb.c, uv, NS);
      }
      mbar_arrive(&empty_bar[b]);
    }
  }
  add_ops(m, ops);  // both roles leave their loops as whole warps
}

// The same forecast with the normal matrix in registers and the solver's
// rotation accumulators in the caller's shared-memory slice (the
// warp-specialised kernel's solver threads).  Identical operations and bits.
template<int EA>
__device__ __noinline__ int smap_point_sm(const GroupParams& g, long long p, int prow, bool save, int keff,
                                          const int* rows, const double* cd, double* uv, int uv_stride)
{
  constexpr int n = EA + 1;
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
  const StridedMat<n> U{ uv, uv_stride }, V{ uv + n * n * uv_stride, uv_stride };
  for (int t = 0; t < g.n_thetas; t++) {
    const double theta = g.thetas[t];
    double W[n][n], bv[n], xs[n];
#pragma unroll
    for (int a = 0; a < n; a++) {
      bv[a] = 0;
#pragma unroll
      for (int b = 0; b < n; b++)
        W[a][b] = 0;
    }
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
          W[a][b] = add(W[a][b], mul(xr[a], xr[b]));
        bv[a] = add(bv[a], mul(xr[a], yl));
      }
    }
#pragma unroll
    for (int a = 0; a < n; a++)
#pragma unroll
      for (int b = 0; b < a; b++)
        W[a][b] = W[b][a];
    svd_solve_nm<n>(W, bv, xs, U, V, ops);
    double r = xs[0];
#pragma unroll
    for (int j = 0; j < EA; j++)
      r = add(r, mul(y[j], xs[j + 1]));
    if (g.coeffs && save && t == g.n_thetas - 1) {
#pragma unroll
      for (int j = 0; j < n; j++)
        g.coeffs[(size_t)p * n + j] = fabs(xs[j]) < 1.0e-11 ? MISS : xs[j];
    }
    g.pred[(size_t)t * g.total_points + p] = r;
  }
  return ops;
}

template<int EA, int C, int ALG>
void launch_one(const GroupParams& g, const MixedRun& m, int num_sms, cudaStream_t s)
{
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, knn_mixed_kernel<EA, C, ALG>, TPB, 0);
  if (m.ctas_per_sm > 0 && per_sm > m.ctas_per_sm)
    per_sm = m.ctas_per_sm;
  if (per_sm < 1)
    per_sm = 1;
  long long blocks = (long long)num_sms * per_sm;
  if (blocks > m.item_end - m.item_begin)
    blocks = m.item_end - m.item_begin;
  if (blocks < 1)
    blocks = 1;
  knn_mixed_kernel<EA, C, ALG><<<(int)blocks, TPB, 0, s>>>(g, m);
}

template<int EA, int C, int SW>
void launch_ws(const GroupParams& g, const MixedRun& m, int num_sms, cudaStream_t s)
{
  const size_t smem = ws_smem_bytes<EA, C, SW>();
  cudaFuncSetAttribute(knn_smap_ws_kernel<EA, C, SW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, knn_smap_ws_kernel<EA, C, SW>, TPB + 32 * SW, smem);
  if (per_sm < 1)
    per_sm = 1;
  long long blocks = (long long)num_sms * per_sm;
  if (blocks > m.item_end - m.item_begin)
    blocks = m.item_end - m.item_begin;
  if (blocks < 1)
    blocks = 1;
  knn_smap_ws_kernel<EA, C, SW><<<(int)blocks, TPB + 32 * SW, smem, s>>>(g, m);
}

template<int EA, int C, int ALG>
void launch_ea(const GroupParams& g, const MixedRun& m, int num_sms, cudaStream_t s)
{
  if constexpr (ALG == 1) {
    if (m.form == MIXED_WS4)
      return launch_ws<EA, C, 4>(g, m, num_sms, s);
    if (m.form == MIXED_WS8)
      return launch_ws<EA, C, 8>(g, m, num_sms, s);
  }
  launch_one<EA, C, ALG>(g, m, num_sms, s);
}

template<int C, int ALG>
void launch_c(const GroupParams& g, const MixedRun& m, int num_sms, cudaStream_t s)
{
  switch (g.Ea) {
    case 1: launch_ea<1, C, ALG>(g, m, num_sms, s); break;
    case 2: launch_ea<2, C, ALG>(g, m, num_sms, s); break;
    case 3: launch_ea<3, C, ALG>(g, m, num_sms, s); break;
    case 4: launch_ea<4, C, ALG>(g, m, num_sms, s); break;
    case 5: launch_ea<5, C, ALG>(g, m, num_sms, s); break;
    case 6: launch_ea<6, C, ALG>(g, m, num_sms, s); break;
    case 7: launch_ea<7, C, ALG>(g, m, num_sms, s); break;
    case 8: launch_ea<8, C, ALG>(g, m, num_sms, s); break;
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
  if (m.item_end <= m.item_begin)
    return;
  if (g.algorithm == 1) {
    if (C <= 8)
      launch_c<8, 1>(g, m, num_sms, s);
    else
      launch_c<16, 1>(g, m, num_sms, s);
  } else {
    if (C <= 8)
      launch_c<8, 0>(g, m, num_sms, s);
    else
      launch_c<16, 0>(g, m, num_sms, s);
  }
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
