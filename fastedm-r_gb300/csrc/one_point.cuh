// One prediction point per thread: the scan, the work-item kernel and its
// launcher, shared by kernels_wide.cu (k <= 6 at E_a <= 8, and the wide
// embeddings) and kernels_one16.cu (7 <= k <= 14 at E_a <= 8).
// A 256-thread CTA takes a work item of 256 points, stages library rows of
// the centred FP32 manifold per tile as interleaved pairs, and every thread
// scores two rows against its point per packed step.  Certification, the
// FP64 re-rank in the reference's operation order and the forecast are
// finalize_point's, so neighbours and forecasts are the FP64 path's bits.
#pragma once

#include "mixed_common.cuh"

namespace fedm {

namespace {

// One point per thread: C candidate slots, float manifold row stride RS,
// TR library rows per shared-memory tile, NT threads per CTA.  PEN: panels
// with a finite penalty (panelWeight = idw > 0): a library row of another
// panel than the point's scores idw more (src/distances.cpp:180-181), with
// the tile's panel ids staged in tpan.  The FP32 value then carries one more
// rounded addition, within the certification's accumulation bound, and
// sqrt(idw + x^2) is 1-Lipschitz in x, so the input-rounding term holds too.
//
// Spatially ordered libraries (T.box_off >= 0): the rows come in the order
// m.scan_pos (library positions sorted by a Morton key of their
// coordinates), in tiles of TR rows whose boxes (the union of their
// BOX_ROWS-row sub-tiles' boxes) are known.  The CTA visits the tiles that
// overlap the box of its 256 points first, then the others, and skips a
// tile for a point when a lower bound on the FP32 value of any of its rows
// is not below the point's current C-th value: the scan would reject every
// such row (offer keeps values below D[C-1], which only decreases).  The
// bound is formed like the scan's value, from the distance to the box per
// coordinate with the same rounded subtraction, square and fused
// multiply-add sequence; each step is monotone, so no row of the tile can
// score below it.  A tile no point needs is not staged.  The kept list is
// therefore the same C smallest values as a scan of every row (with ties
// at the C-th value settled by the certification as before), and positions
// are the list's, so the re-rank and its ties are unchanged.
template<int EA, int C, int RS, int TR, int NT, bool PEN = false>
__device__ __forceinline__ void scan_item_one(const GroupParams& g, const MixedRun& m, const DevTask& T, int first,
                                              int tid, float2* tile, int* tpan, int* tpos, float* wbox, Cand<C>& c0,
                                              int& prow0, bool& a0, int& pi, unsigned long long& scanned)
{
  // the slot's point: list order, or the task's lane order (points close
  // in the manifold on neighbouring lanes, so that a warp's candidate
  // lists and solver rotations diverge less)
  const int slot = first + tid;
  a0 = slot < T.n_pred;
  pi = (a0 && T.perm_off >= 0) ? g.perm[T.perm_off + slot] : slot;
  prow0 = a0 ? g.pred_rows[T.pred_off + pi] : 0;
  // negated prediction coordinates, duplicated in both halves; an idle slot
  // sits at 1e30 so its squared distances overflow to +inf and never enter
  float2 na[EA];
#pragma unroll
  for (int j = 0; j < EA; j++) {
    const float va = a0 ? -m.Fp32[(size_t)prow0 * RS + j] : -1e30f;
    na[j] = make_float2(va, va);
  }
  float D0[C];
  int I0[C];
#pragma unroll
  for (int j = 0; j < C; j++) {
    D0[j] = INFINITY;
    I0[j] = -1;
  }
  int z0 = 0;
  int zi0[ZCAP];
#pragma unroll
  for (int j = 0; j < ZCAP; j++)
    zi0[j] = -1;
  const float pen = PEN ? (float)g.idw : 0.f;
  const int ppan = PEN && a0 ? g.panel[prow0] : 0;
  if (T.box_off >= 0) {
    // the box of the CTA's points: per warp, then combined into wbox[0..2EA)
    constexpr int NW = NT / 32;
    const int lane = tid & 31, w = tid >> 5;
#pragma unroll
    for (int j = 0; j < EA; j++) {
      float lo = a0 ? -na[j].x : INFINITY, hi = a0 ? -na[j].x : -INFINITY;
      for (int o = 16; o > 0; o >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
      }
      if (lane == 0) {
        wbox[(w + 1) * 2 * EA + j] = lo;
        wbox[(w + 1) * 2 * EA + EA + j] = hi;
      }
    }
    __syncthreads();
    if (tid < EA) {
      float lo = wbox[2 * EA + tid], hi = wbox[2 * EA + EA + tid];
      for (int q = 2; q <= NW; q++) {
        lo = fminf(lo, wbox[q * 2 * EA + tid]);
        hi = fmaxf(hi, wbox[q * 2 * EA + EA + tid]);
      }
      wbox[tid] = lo;
      wbox[EA + tid] = hi;
    }
    __syncthreads();
    constexpr int SPT = TR / BOX_ROWS;
    const int ntile = (T.n_lib + TR - 1) / TR;
    const int nsub = (T.n_lib + BOX_ROWS - 1) / BOX_ROWS;
    for (int pass = 0; pass < 2; pass++) {
      for (int tt = 0; tt < ntile; tt++) {
        // the tile's box (the union of its sub-tiles'), whether it overlaps
        // the points' box, and this thread's lower bound on the scan's value
        // for any row of it
        bool overlap = true;
        float lb = 0.f;
#pragma unroll
        for (int j = 0; j < EA; j++) {
          float tlo = INFINITY, thi = -INFINITY;
#pragma unroll
          for (int u = 0; u < SPT; u++) {
            const int sb = tt * SPT + u;
            if (sb < nsub) {
              const float2 b = m.boxes[(size_t)(T.box_off + sb) * EA + j];
              tlo = fminf(tlo, b.x);
              thi = fmaxf(thi, b.y);
            }
          }
          overlap = overlap && tlo <= wbox[EA + j] && thi >= wbox[j];
          const float p = -na[j].x;
          const float d = p < tlo ? __fadd_rn(tlo, na[j].x) : (p > thi ? __fadd_rn(thi, na[j].x) : 0.f);
          lb = j == 0 ? __fmul_rn(d, d) : __fmaf_rn(d, d, lb);
        }
        if (overlap != (pass == 0))
          continue;  // the same for every thread of the CTA
        const bool need = a0 && lb < D0[C - 1];
        if (!__syncthreads_or(need))
          continue;
        const int t0 = tt * TR;
        const int cnt = min(TR, T.n_lib - t0);
        const int npairs = (cnt + 1) >> 1;
        for (int i = tid; i < 2 * npairs; i += NT) {
          float* dst = reinterpret_cast<float*>(tile + (i >> 1) * EA) + (i & 1);
          if (i < cnt) {
            const int pos = m.scan_pos[T.lib_off + t0 + i];
            const int row = g.lib_rows[T.lib_off + pos];
            const float* src = m.F32 + (size_t)row * RS;
#pragma unroll
            for (int j = 0; j < EA; j++)
              dst[2 * j] = src[j];
            tpos[i] = pos;
            if constexpr (PEN)
              tpan[i] = g.panel[row];
          } else {
#pragma unroll
            for (int j = 0; j < EA; j++)
              dst[2 * j] = 1e30f;  // padding row: never a candidate
            tpos[i] = 0;
            if constexpr (PEN)
              tpan[i] = 0;
          }
        }
        __syncthreads();
        if (need) {
          // the tile's sub-tiles in turn, each skipped when the bound from
          // its own box is not below the point's current C-th value (which
          // only decreases as the scan goes on)
          const float2* sbox = m.boxes + (size_t)(T.box_off + tt * SPT) * EA;
#pragma unroll 1
          for (int u = 0; u < SPT; u++) {
            const int r0 = u * BOX_ROWS;
            if (r0 >= cnt)
              break;
            const int rn = min(BOX_ROWS, cnt - r0);
            if constexpr (SPT > 1) {
              float lbu = 0.f;
#pragma unroll
              for (int j = 0; j < EA; j++) {
                const float2 b = sbox[u * EA + j];
                const float p = -na[j].x;
                const float d = p < b.x ? __fadd_rn(b.x, na[j].x) : (p > b.y ? __fadd_rn(b.y, na[j].x) : 0.f);
                lbu = j == 0 ? __fmul_rn(d, d) : __fmaf_rn(d, d, lbu);
              }
              if (!(lbu < D0[C - 1]))
                continue;
            }
            scanned += (unsigned long long)rn;
#pragma unroll 2
            for (int ip = r0 >> 1; ip < (r0 + rn + 1) >> 1; ip++) {
              const float2* xr = tile + ip * EA;
              float2 d = __fadd2_rn(xr[0], na[0]);
              float2 sa = __fmul2_rn(d, d);
#pragma unroll
              for (int j = 1; j < EA; j++) {
                d = __fadd2_rn(xr[j], na[j]);
                sa = __ffma2_rn(d, d, sa);
              }
              if constexpr (PEN) {
                const int2 pp = reinterpret_cast<const int2*>(tpan)[ip];
                sa = __fadd2_rn(sa, make_float2(pp.x != ppan ? pen : 0.f, pp.y != ppan ? pen : 0.f));
              }
              if (fminf(sa.x, sa.y) < D0[C - 1]) {
                const int2 lp = reinterpret_cast<const int2*>(tpos)[ip];
                offer<C>(D0, I0, z0, zi0, sa.x, lp.x);
                offer<C>(D0, I0, z0, zi0, sa.y, lp.y);
              }
            }
          }
        }
      }
    }
  } else {
  for (int t0 = 0; t0 < T.n_lib; t0 += TR) {
    const int cnt = min(TR, T.n_lib - t0);
    const int npairs = (cnt + 1) >> 1;
    __syncthreads();
    for (int i = tid; i < 2 * npairs; i += NT) {
      float* dst = reinterpret_cast<float*>(tile + (i >> 1) * EA) + (i & 1);
      if (i < cnt) {
        const int row = g.lib_rows[T.lib_off + t0 + i];
        const float* src = m.F32 + (size_t)row * RS;
#pragma unroll
        for (int j = 0; j < EA; j++)
          dst[2 * j] = src[j];
        if constexpr (PEN)
          tpan[i] = g.panel[row];
      } else {
#pragma unroll
        for (int j = 0; j < EA; j++)
          dst[2 * j] = 1e30f;  // padding row: never a candidate
        if constexpr (PEN)
          tpan[i] = 0;  // any panel: the padding row's value is +inf
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
      if constexpr (PEN) {
        const int2 pp = reinterpret_cast<const int2*>(tpan)[ip];
        sa = __fadd2_rn(sa, make_float2(pp.x != ppan ? pen : 0.f, pp.y != ppan ? pen : 0.f));
      }
      if (fminf(sa.x, sa.y) < D0[C - 1]) {
        const int li = t0 + 2 * ip;
        offer<C>(D0, I0, z0, zi0, sa.x, li);
        offer<C>(D0, I0, z0, zi0, sa.y, li + 1);
      }
    }
    scanned += a0 ? (unsigned long long)cnt : 0ull;
  }
  }
#pragma unroll
  for (int j = 0; j < C; j++) {
    c0.D[j] = D0[j];
    c0.I[j] = I0[j];
  }
  c0.z = z0;
#pragma unroll
  for (int j = 0; j < ZCAP; j++)
    c0.zi[j] = zi0[j];
}

template<int EA, int C, int RS, int TR, int ALG, int OCC, int NT = TPB, bool PEN = false>
__global__ void __launch_bounds__(NT, OCC) knn_one_kernel(GroupParams g, MixedRun m)
{
  __shared__ __align__(16) float2 tile[(TR / 2) * EA];
  __shared__ __align__(8) int tpan[PEN ? TR : 2];
  __shared__ __align__(8) int tpos[TR];
  __shared__ float wbox[(NT / 32 + 1) * 2 * EA];
  __shared__ int s_item;
  const int tid = threadIdx.x;
  unsigned long long ops = 0, scanned = 0;
  for (;;) {
    __syncthreads();
    if (tid == 0)
      s_item = m.item_begin + atomicAdd(m.counter, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= m.item_end) {
      add_ops(m, ops);  // every thread of the CTA leaves here together
      add_scanned(m, scanned);
      return;
    }
    const int2 it = m.items[item];
    const DevTask T = g.tasks[it.x];
    Cand<C> c0;
    int prow0, pi0;
    bool a0;
    scan_item_one<EA, C, RS, TR, NT, PEN>(g, m, T, it.y, tid, tile, tpan, tpos, wbox, c0, prow0, a0, pi0, scanned);
    if constexpr (ALG == 2) {
      // S-map lists for smap_list_kernel: settle the neighbours, write them
      const long long slot = (long long)(item - m.item_begin) * NT + tid;
      int keff = 0, iops = 0;
      int rows[C + ZCAP];
      double cd[C + ZCAP];
      if (a0) {
        const Cand<C> c = c0;
        if (!prepare_point<EA, C>(g, m, T, T.point_base + pi0, prow0, c, keff, rows, cd, iops))
          keff = 0;
      }
      m.l_keff[slot] = keff;
#pragma unroll
      for (int j = 0; j < SPLIT_SLOTS; j++)
        if (j < keff) {
          m.l_rows[j * m.l_slots + slot] = rows[j];
          m.l_dist[j * m.l_slots + slot] = cd[j];
        }
      ops += iops;
    } else if (a0) {
      const Cand<C> c = c0;
      ops += finalize_point<EA, C, ALG>(g, m, T, T.point_base + pi0, prow0, c);
    }
  }
}

template<int EA, int C, int RS, int TR, int ALG, int OCC, int NT = TPB, bool PEN = false>
void launch_one(const GroupParams& g, const MixedRun& m, int num_sms, cudaStream_t s)
{
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, knn_one_kernel<EA, C, RS, TR, ALG, OCC, NT, PEN>, NT, 0);
  if (m.ctas_per_sm > 0 && per_sm > m.ctas_per_sm)
    per_sm = m.ctas_per_sm;
  if (per_sm < 1)
    per_sm = 1;
  long long blocks = (long long)num_sms * per_sm;
  if (blocks > m.item_end - m.item_begin)
    blocks = m.item_end - m.item_begin;
  if (blocks < 1)
    blocks = 1;
  knn_one_kernel<EA, C, RS, TR, ALG, OCC, NT, PEN><<<(int)blocks, NT, 0, s>>>(g, m);
}

// The one-point forms by E_a: MIXED_ONE6 (eight candidate slots, six CTAs
// per SM), MIXED_ONE16 (sixteen slots, four CTAs per SM) and the wide form
// (E_a 9..16, 32 slots, 512-row tiles, two CTAs per SM).
constexpr int WTILE = 512;  // wide form: library rows per tile, 32 KB of shared memory at E_a = 16
constexpr int WC = 32;      // wide form: candidate slots per point
constexpr int WS = 16;      // wide form: row stride of the float manifold

template<int ALG, bool PEN>
void launch_one6_t(const GroupParams& g, const MixedRun& m, int num_sms, cudaStream_t s)
{
  constexpr int OCC = 6;
  switch (g.Ea) {
    case 1: launch_one<1, 8, 4, 1024, ALG, OCC, TPB, PEN>(g, m, num_sms, s); break;
    case 2: launch_one<2, 8, 4, 1024, ALG, OCC, TPB, PEN>(g, m, num_sms, s); break;
    case 3: launch_one<3, 8, 4, 1024, ALG, OCC, TPB, PEN>(g, m, num_sms, s); break;
    case 4: launch_one<4, 8, 4, 1024, ALG, OCC, TPB, PEN>(g, m, num_sms, s); break;
    case 5: launch_one<5, 8, 8, 1024, ALG, OCC, TPB, PEN>(g, m, num_sms, s); break;
    case 6: launch_one<6, 8, 8, 1024, ALG, OCC, TPB, PEN>(g, m, num_sms, s); break;
    case 7: launch_one<7, 8, 8, 1024, ALG, OCC, TPB, PEN>(g, m, num_sms, s); break;
    case 8: launch_one<8, 8, 8, 1024, ALG, OCC, TPB, PEN>(g, m, num_sms, s); break;
    default: break;
  }
}

template<int ALG, bool PEN>
void launch_one16_t(const GroupParams& g, const MixedRun& m, int num_sms, cudaStream_t s)
{
  constexpr int OCC = 4;
  switch (g.Ea) {
    case 1: launch_one<1, 16, 4, 1024, ALG, OCC, TPB, PEN>(g, m, num_sms, s); break;
    case 2: launch_one<2, 16, 4, 1024, ALG, OCC, TPB, PEN>(g, m, num_sms, s); break;
    case 3: launch_one<3, 16, 4, 1024, ALG, OCC, TPB, PEN>(g, m, num_sms, s); break;
    case 4: launch_one<4, 16, 4, 1024, ALG, OCC, TPB, PEN>(g, m, num_sms, s); break;
    case 5: launch_one<5, 16, 8, 1024, ALG, OCC, TPB, PEN>(g, m, num_sms, s); break;
    case 6: launch_one<6, 16, 8, 1024, ALG, OCC, TPB, PEN>(g, m, num_sms, s); break;
    case 7: launch_one<7, 16, 8, 1024, ALG, OCC, TPB, PEN>(g, m, num_sms, s); break;
    case 8: launch_one<8, 16, 8, 1024, ALG, OCC, TPB, PEN>(g, m, num_sms, s); break;
    default: break;
  }
}

template<int ALG, bool PEN>
void launch_wide_t(const GroupParams& g, const MixedRun& m, int num_sms, cudaStream_t s)
{
  switch (g.Ea) {
    case 9: launch_one<9, WC, WS, WTILE, ALG, 2, TPB, PEN>(g, m, num_sms, s); break;
    case 10: launch_one<10, WC, WS, WTILE, ALG, 2, TPB, PEN>(g, m, num_sms, s); break;
    case 11: launch_one<11, WC, WS, WTILE, ALG, 2, TPB, PEN>(g, m, num_sms, s); break;
    case 12: launch_one<12, WC, WS, WTILE, ALG, 2, TPB, PEN>(g, m, num_sms, s); break;
    case 13: launch_one<13, WC, WS, WTILE, ALG, 2, TPB, PEN>(g, m, num_sms, s); break;
    case 14: launch_one<14, WC, WS, WTILE, ALG, 2, TPB, PEN>(g, m, num_sms, s); break;
    case 15: launch_one<15, WC, WS, WTILE, ALG, 2, TPB, PEN>(g, m, num_sms, s); break;
    case 16: launch_one<16, WC, WS, WTILE, ALG, 2, TPB, PEN>(g, m, num_sms, s); break;
    default: break;
  }
}

} // namespace

} // namespace fedm
