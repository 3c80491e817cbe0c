// Mixed-precision neighbour search and forecast for wide embeddings:
// E_a = 9..16 (dt columns double E_a, so E = 5..8 with dt lands here) and up
// to 30 neighbours.  The kernel is knn_mixed_kernel's with one prediction
// point per thread and 32 candidate slots, so the lists still fit in
// registers: a 256-thread CTA takes a work item of 256 points, stages 512
// library rows of the centred FP32 manifold (row stride 16 floats) per tile
// as interleaved pairs, and every thread scores two rows against its point
// per packed step.  Certification, the FP64 re-rank in the reference's
// operation order and the forecast are finalize_point's, so neighbours and
// forecasts are the FP64 path's bits.
#include "mixed_common.cuh"

namespace fedm {

namespace {

constexpr int WTILE = 512;  // library rows per tile: 32 KB of shared memory at E_a = 16
constexpr int WC = 32;      // candidate slots per point
constexpr int WS = 16;      // row stride of the float manifold

template<int EA>
__device__ __forceinline__ void scan_item_wide(const GroupParams& g, const MixedRun& m, const DevTask& T, int first,
                                               int tid, float2* tile, Cand<WC>& c0, int& prow0, bool& a0)
{
  const int pi0 = first + tid;
  a0 = pi0 < T.n_pred;
  prow0 = a0 ? g.pred_rows[T.pred_off + pi0] : 0;
  // negated prediction coordinates, duplicated in both halves; an idle slot
  // sits at 1e30 so its squared distances overflow to +inf and never enter
  float2 na[EA];
#pragma unroll
  for (int j = 0; j < EA; j++) {
    const float va = a0 ? -m.Fp32[(size_t)prow0 * WS + j] : -1e30f;
    na[j] = make_float2(va, va);
  }
  float D0[WC];
  int I0[WC];
#pragma unroll
  for (int j = 0; j < WC; j++) {
    D0[j] = INFINITY;
    I0[j] = -1;
  }
  int z0 = 0;
  int zi0[ZCAP];
#pragma unroll
  for (int j = 0; j < ZCAP; j++)
    zi0[j] = -1;
  for (int t0 = 0; t0 < T.n_lib; t0 += WTILE) {
    const int cnt = min(WTILE, T.n_lib - t0);
    const int npairs = (cnt + 1) >> 1;
    __syncthreads();
    for (int i = tid; i < 2 * npairs; i += TPB) {
      float* dst = reinterpret_cast<float*>(tile + (i >> 1) * EA) + (i & 1);
      if (i < cnt) {
        const float* src = m.F32 + (size_t)g.lib_rows[T.lib_off + t0 + i] * WS;
#pragma unroll
        for (int j = 0; j < EA; j++)
          dst[2 * j] = src[j];
      } else {
#pragma unroll
        for (int j = 0; j < EA; j++)
          dst[2 * j] = 1e30f;  // padding row: never a candidate
      }
    }
    __syncthreads();
#pragma unroll 2
    for (int ip = 0; ip < npairs; ip++) {
      const float2* xr = tile + ip * EA;
      float2 d = __fadd2_rn(xr[0], na[0]);
      float2 sa = __fmul2_rn(d, d);
#pragma unroll
      for (int j = 1; j < EA; j++) {
        d = __fadd2_rn(xr[j], na[j]);
        sa = __ffma2_rn(d, d, sa);
      }
      if (fminf(sa.x, sa.y) < D0[WC - 1]) {
        const int li = t0 + 2 * ip;
        offer<WC>(D0, I0, z0, zi0, sa.x, li);
        offer<WC>(D0, I0, z0, zi0, sa.y, li + 1);
      }
    }
  }
#pragma unroll
  for (int j = 0; j < WC; j++) {
    c0.D[j] = D0[j];
    c0.I[j] = I0[j];
  }
  c0.z = z0;
#pragma unroll
  for (int j = 0; j < ZCAP; j++)
    c0.zi[j] = zi0[j];
}

template<int EA, int ALG>
__global__ void __launch_bounds__(TPB, 2) knn_wide_kernel(GroupParams g, MixedRun m)
{
  __shared__ __align__(16) float2 tile[(WTILE / 2) * EA];
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
    Cand<WC> c0;
    int prow0;
    bool a0;
    scan_item_wide<EA>(g, m, T, it.y, tid, tile, c0, prow0, a0);
    if (a0) {
      const Cand<WC> c = c0;
      ops += finalize_point<EA, WC, ALG>(g, m, T, T.point_base + it.y + tid, prow0, c);
    }
  }
}

template<int EA, int ALG>
void launch_wide(const GroupParams& g, const MixedRun& m, int num_sms, cudaStream_t s)
{
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, knn_wide_kernel<EA, ALG>, TPB, 0);
  if (per_sm < 1)
    per_sm = 1;
  long long blocks = (long long)num_sms * per_sm;
  if (blocks > m.item_end - m.item_begin)
    blocks = m.item_end - m.item_begin;
  if (blocks < 1)
    blocks = 1;
  knn_wide_kernel<EA, ALG><<<(int)blocks, TPB, 0, s>>>(g, m);
}

template<int ALG>
void launch_wide_alg(const GroupParams& g, const MixedRun& m, int num_sms, cudaStream_t s)
{
  switch (g.Ea) {
    case 9: launch_wide<9, ALG>(g, m, num_sms, s); break;
    case 10: launch_wide<10, ALG>(g, m, num_sms, s); break;
    case 11: launch_wide<11, ALG>(g, m, num_sms, s); break;
    case 12: launch_wide<12, ALG>(g, m, num_sms, s); break;
    case 13: launch_wide<13, ALG>(g, m, num_sms, s); break;
    case 14: launch_wide<14, ALG>(g, m, num_sms, s); break;
    case 15: launch_wide<15, ALG>(g, m, num_sms, s); break;
    case 16: launch_wide<16, ALG>(g, m, num_sms, s); break;
    default: break;
  }
}

} // namespace

void launch_knn_wide(const GroupParams& g, const MixedRun& m, int num_sms, cudaStream_t s)
{
  if (m.item_end <= m.item_begin)
    return;
  if (g.algorithm == 1)
    launch_wide_alg<1>(g, m, num_sms, s);
  else
    launch_wide_alg<0>(g, m, num_sms, s);
}

} // namespace fedm
