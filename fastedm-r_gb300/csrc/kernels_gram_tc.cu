// FAST precision, S-map with every library row as a neighbour (k = all), on
// the tensor cores: the weighted normal equations of every (point, theta)
//
//   G[(p, theta), c] = sum_i w2(p, theta, i) P[i, c],   w2 = exp(-2 theta d / mean d),
//   P[i, .] = (u_a u_b for a <= b, u_a t_i),  u = [1, m_i]
//
// are one GEMM, M = points x thetas, N = (E_a+1)(E_a+2)/2 + E_a+1 (<= 32
// here), K = library rows.  The sums must stay near FP64 accuracy (the
// normal equations are solved in FP64 afterwards), so the GEMM runs on
// exact integer slices (the Ozaki scheme, K. Ozaki et al., "Error-free
// transformations of matrix multiplication by using fast routines of matrix
// multiplication and its applications", Numer. Algorithms 59, 2012):
//
//   a' = w2 / 2^E_r = sum_{s<5} alpha_s 2^(-8(s+1)), alpha_s in [0, 256]
//       (E_r: the row's largest weight, so a' <= 1; 40 bits of it are kept)
//   b' = P / 2^F_c  = sum_{t<5} beta_t 2^(-8(t+1)),  beta_t in [-256, 256]
//       (F_c: the column's largest magnitude; 40 bits are kept)
//
// Integers of at most 8 significant bits are exact in bf16 and their
// products exact in FP32.  Pairs (s, t) with s + t <= 4 (zero-based) are
// kept: 15 of them, in five groups of equal s + t whose products share a
// scale.  Only the leading digits reach 256 (alpha_s <= 255 and |beta_t| <=
// 128 after them), so a group's products over one 64-row block sum to at
// most 64 (4 x 2^15 + 2^16) < 2^24 -- exact in the FP32 TMEM accumulator.
// After every block the five accumulators are read back (tcgen05.ld) and
// added, shifted by 8 (4 - g) bits, into one int64 per term, exact while the
// library stays under ~30 000 rows.  Only the slice truncation is
// approximate: 2^-40 of the row's largest weight and 2^-41 of the column's
// largest product.
//
// One CTA of 256 threads takes 128 rows (TMEM lanes); two threads share a
// row, each generating the weight digits of half of every 64-row block and
// reading back part of the accumulators (two CTAs, 16 warps, per SM: shared
// memory and TMEM allow no more CTAs).  Per block the CTA writes the five
// weight slices of its 128 x 64 tile to shared memory, takes the block's
// 20 KB of library-side slices (precomputed in the MMA's shared-memory
// layout) with one cp.async.bulk, issues 60 tcgen05.mma (M = 128, N = 32,
// K = 16, bf16 in, FP32 in TMEM) from one thread and reads the five
// accumulators back.  Every wait is bounded; on a
// timeout the CTA sets the error flag, and TMEM is always freed.
#include <cuda_bf16.h>

#include <algorithm>
#include <cfloat>
#include <climits>
#include <cstdint>

#include "kernels.h"

namespace fedm {

namespace {

constexpr int TC_M = 128;        // rows per tile (TMEM lanes)
constexpr int TC_NT = 256;       // threads per CTA: two per row
constexpr int TC_KB = 64;        // library rows per block
constexpr int TC_KS = 4;         // 16-row MMA K-steps per block
constexpr int TC_SA = 5;         // weight slices
constexpr int TC_SB = 5;         // product slices
constexpr int TC_G = 5;          // accumulator groups (s + t = 0..4)
constexpr int TC_N = 32;         // MMA N (terms, padded)
constexpr int TC_TMEM_COLS = 256;
constexpr uint32_t A_TILE = TC_M * 16 * 2;    // 4 KB: one K-step of one weight slice
constexpr uint32_t B_TILE = TC_N * 16 * 2;    // 1 KB: one K-step of one product slice
constexpr uint32_t A_BYTES = TC_SA * TC_KS * A_TILE;  // 80 KB
constexpr uint32_t B_BYTES = TC_SB * TC_KS * B_TILE;  // 20 KB
constexpr uint32_t TC_SMEM = A_BYTES + B_BYTES + 64;
constexpr unsigned long long TC_WAIT_NS = 2000000000ull;  // a wait gives up after 2 s

// Byte offset of element (row, k) of a K-major tile in the no-swizzle
// canonical layout: core matrices of 8 rows x 16 bytes, the two core
// matrices of a row group 128 bytes apart along K (leading byte offset),
// row groups 256 bytes apart (stride byte offset).
__host__ __device__ constexpr uint32_t core_off(int row, int k)
{
  return (uint32_t)((row >> 3) * 256 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start address, leading and stride byte
// offsets (in 16-byte units), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr)
{
  uint64_t d = (uint64_t)((addr & 0x3FFFF) >> 4);
  d |= (uint64_t)(128 >> 4) << 16;
  d |= (uint64_t)(256 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator, bf16 A and B, both
// K-major, N = TC_N, M = TC_M.
constexpr uint32_t TC_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TC_N >> 3) << 17) |
                              ((uint32_t)(TC_M >> 4) << 24);

__device__ __forceinline__ unsigned long long tc_now_ns()
{
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Waits for the phase of the given parity; false after TC_WAIT_NS (or 2^30
// polls) without it.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity)
{
  unsigned long long t0 = 0;
  for (unsigned n = 0; n < (1u << 30); n++) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok)
      return true;
    if ((n & 63) == 0) {
      const unsigned long long t = tc_now_ns();
      if (t0 == 0)
        t0 = t;
      else if (t - t0 > TC_WAIT_NS)
        return false;
    }
  }
  return false;
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16])
{
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
        "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32])
{
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
      "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
        "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]),
        "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
        "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// The product slices of one task's library: per block of 64 rows, the
// TC_SB x TC_KS tiles in the MMA's layout, 20 KB contiguous.  Pass 1 finds
// each column's largest magnitude (as the bits of |P|, whose integer order
// is the order of the magnitudes).
template<int EA>
__global__ void gram_tc_colmax_kernel(GroupParams g, GramTC t)
{
  constexpr int n = EA + 1;
  const GramTask& K = t.tasks[blockIdx.y];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < K.n_lib; i += gridDim.x * blockDim.x) {
    const int row = g.lib_rows[K.lib_off + i];
    double u[n];
    u[0] = 1.0;
#pragma unroll
    for (int j = 1; j < n; j++)
      u[j] = g.F[(size_t)row * EA + j - 1];
    const double tg = g.lib_target[row];
    int e = 0;
#pragma unroll
    for (int a = 0; a < n; a++) {
#pragma unroll
      for (int b = a; b < n; b++) {
        atomicMax(&t.colmax[blockIdx.y * TC_N + e], (unsigned long long)__double_as_longlong(fabs(u[a] * u[b])));
        e++;
      }
      atomicMax(&t.colmax[blockIdx.y * TC_N + n * (n + 1) / 2 + a],
                (unsigned long long)__double_as_longlong(fabs(u[a] * tg)));
    }
  }
}

template<int EA>
__global__ void gram_tc_slices_kernel(GroupParams g, GramTC t)
{
  constexpr int n = EA + 1, NA = n * (n + 1) / 2, NP = NA + n;
  const GramTask& K = t.tasks[blockIdx.y];
  const int nrows = K.n_blocks * TC_KB;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nrows; i += gridDim.x * blockDim.x) {
    double v[TC_N];
#pragma unroll
    for (int c = 0; c < TC_N; c++)
      v[c] = 0;
    if (i < K.n_lib) {
      const int row = g.lib_rows[K.lib_off + i];
      double u[n];
      u[0] = 1.0;
#pragma unroll
      for (int j = 1; j < n; j++)
        u[j] = g.F[(size_t)row * EA + j - 1];
      const double tg = g.lib_target[row];
      int e = 0;
#pragma unroll
      for (int a = 0; a < n; a++) {
#pragma unroll
        for (int b = a; b < n; b++)
          v[e++] = u[a] * u[b];
        v[NA + a] = u[a] * tg;
      }
    }
    unsigned char* blk = t.bslices + (size_t)(K.b_off + i / TC_KB) * B_BYTES;
    const int kb = i % TC_KB, ks = kb / 16, k = kb % 16;
#pragma unroll
    for (int c = 0; c < TC_N; c++) {
      double b = 0;
      if (c < NP) {
        const double mx = __longlong_as_double((long long)t.colmax[blockIdx.y * TC_N + c]);
        const int F = mx > 0 ? ilogb(mx) + 1 : 0;  // 2^F > the column's largest magnitude
        b = scalbn(v[c], -F);                       // exact; |b| < 1
      }
#pragma unroll
      for (int s = 0; s < TC_SB; s++) {
        const double d = rint(b * 256.0);  // |d| <= 256 (first digit), <= 128 after
        b = b * 256.0 - d;                  // exact
        *(__nv_bfloat16*)(blk + (s * TC_KS + ks) * B_TILE + core_off(c, k)) = __double2bfloat16(d);
      }
    }
  }
}

__global__ void __launch_bounds__(TC_NT, 2) gram_tc_kernel(GramTC t)
{
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  unsigned char* sA = tc_smem;
  unsigned char* sB = tc_smem + A_BYTES;
  unsigned long long* bars = (unsigned long long*)(tc_smem + A_BYTES + B_BYTES);  // [0] B copy, [1] MMAs
  uint32_t* tmem_slot = (uint32_t*)(bars + 2);
  const int tid = threadIdx.x;
  const int lrow = tid & (TC_M - 1);  // the tile row (TMEM lane) of this thread: (warp % 4) * 32 + lane
  const int half = tid >> 7;          // which half of each block's 64 library rows it generates
  const GramTile tile = t.tiles[blockIdx.x];
  const GramTask& K = t.tasks[tile.task];
  const int row = tile.row0 + lrow;  // the task's row (point-major, theta fastest)
  const bool active = lrow < tile.n_rows;
  // this row's weights: exp(c2 d) with c2 = -2 theta / mean, scaled by the
  // row's largest weight exp(c2 dmin)
  int q = 0;
  float c2 = 0.f, rscale = 1.f;
  int rexp = 0;
  if (active) {
    q = K.q0 + row / t.n_thetas;
    const int th = row % t.n_thetas;
    c2 = (float)(-2.0 * t.thetas[th] / t.means[q]);
    const float mx = t.dmin[q] < INFINITY ? expf(__fmul_rn(c2, t.dmin[q])) : 0.f;
    if (mx > 0.f)
      rexp = ilogbf(mx) + 1;  // 2^rexp > mx
    rscale = scalbnf(1.f, -rexp);
  }
  const float* rq = t.rdist + (size_t)q * t.max_nlib;
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[0])) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[1])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (tid < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "n"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const uint32_t lane_base = tmem + ((uint32_t)(((tid >> 5) & 3) * 32) << 16);
  long long acc[TC_N];
#pragma unroll
  for (int c = 0; c < TC_N; c++)
    acc[c] = 0;
  bool ok = true;
  for (int b = 0; b < K.n_blocks && ok; b++) {
    const uint32_t parity = (uint32_t)(b & 1);
    if (tid == 0) {
      // the block's product slices: one bulk copy, completion counted in bytes
      const unsigned char* src = t.bslices + (size_t)(K.b_off + b) * B_BYTES;
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&bars[0])),
                   "r"(B_BYTES)
                   : "memory");
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
              smem_u32(sB)),
          "l"(src), "r"(B_BYTES), "r"(smem_u32(&bars[0]))
          : "memory");
    }
    // the five weight slices of this row for its half of the block's 64
    // library rows
    const int i0 = b * TC_KB;
#pragma unroll 1
    for (int k8 = half * (TC_KB / 2); k8 < (half + 1) * (TC_KB / 2); k8 += 8) {
      // eight distances; rows start on 16-byte boundaries (the stride is a
      // multiple of four), so a full group is two vector loads
      float d8[8];
      if (active && i0 + k8 + 8 <= K.n_lib) {
        const float4 lo = *reinterpret_cast<const float4*>(rq + i0 + k8);
        const float4 hi = *reinterpret_cast<const float4*>(rq + i0 + k8 + 4);
        d8[0] = lo.x; d8[1] = lo.y; d8[2] = lo.z; d8[3] = lo.w;
        d8[4] = hi.x; d8[5] = hi.y; d8[6] = hi.z; d8[7] = hi.w;
      } else {
#pragma unroll
        for (int j = 0; j < 8; j++)
          d8[j] = (active && i0 + k8 + j < K.n_lib) ? rq[i0 + k8 + j] : -1.f;
      }
      uint32_t packed[TC_SA][4];
#pragma unroll
      for (int j = 0; j < 8; j += 2) {
        float a2[2];
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const float d = d8[j + h];
          // exact scaling by a power of two; -1 marks a row that is no neighbour
          const float w = d >= 0.f ? expf(__fmul_rn(c2, d)) * rscale : 0.f;
          a2[h] = fminf(w, 1.f);
        }
        float digit[TC_SA][2];
#pragma unroll
        for (int h = 0; h < 2; h++) {
          float a = a2[h];
#pragma unroll
          for (int s = 0; s < TC_SA; s++) {
            const float dg = floorf(a * 256.f);  // in [0, 256]
            a = a * 256.f - dg;                  // exact
            digit[s][h] = dg;
          }
        }
#pragma unroll
        for (int s = 0; s < TC_SA; s++) {
          const __nv_bfloat162 pr = __floats2bfloat162_rn(digit[s][0], digit[s][1]);
          packed[s][j / 2] = *reinterpret_cast<const uint32_t*>(&pr);
        }
      }
      const int ks = k8 / 16, k = k8 % 16;
#pragma unroll
      for (int s = 0; s < TC_SA; s++) {
        uint4 v;
        v.x = packed[s][0];
        v.y = packed[s][1];
        v.z = packed[s][2];
        v.w = packed[s][3];
        *reinterpret_cast<uint4*>(sA + (s * TC_KS + ks) * A_TILE + core_off(lrow, k)) = v;
      }
    }
    // the weight tiles (generic proxy) must be visible to the tensor core
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      ok = mbar_wait_bounded(smem_u32(&bars[0]), parity);
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (ok) {
#pragma unroll
        for (int gsum = 0; gsum < TC_G; gsum++) {
          bool first = true;
#pragma unroll
          for (int s = 0; s < TC_SA; s++) {
            const int tt = gsum - s;
            if (tt < 0 || tt >= TC_SB)
              continue;
#pragma unroll
            for (int ks = 0; ks < TC_KS; ks++) {
              const uint64_t ad = sdesc(smem_u32(sA + (s * TC_KS + ks) * A_TILE));
              const uint64_t bd = sdesc(smem_u32(sB + (tt * TC_KS + ks) * B_TILE));
              asm volatile(
                  "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                  "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem + gsum * TC_N),
                  "l"(ad), "l"(bd), "r"(TC_IDESC), "r"(first ? 0 : 1)
                  : "memory");
              first = false;
            }
          }
        }
      }
      // completion of the MMAs issued above (or of none) arrives on bars[1]
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(&bars[1]))
                   : "memory");
    }
    const bool done = mbar_wait_bounded(smem_u32(&bars[1]), parity);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    ok = __syncthreads_and(done && (tid != 0 || ok)) != 0;
    if (!ok)
      break;
    // the first half of the threads reads groups 0..2, the second 3..4
#pragma unroll
    for (int gsum = 0; gsum < TC_G; gsum++) {
      if ((gsum < 3) != (half == 0))
        continue;
      const int sh = 8 * (TC_G - 1 - gsum);
#pragma unroll
      for (int c0 = 0; c0 < TC_N; c0 += 16) {
        uint32_t v[16];
        tmem_ld16(lane_base + gsum * TC_N + c0, v);
#pragma unroll
        for (int c = 0; c < 16; c++)
          acc[c0 + c] += (long long)(int)__uint_as_float(v[c]) << sh;
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();  // the tiles and accumulators are reused by the next block
  }
  if (!ok && tid == 0)
    atomicExch(t.error, 1);
  // the second half hands its partial sums to the first through shared
  // memory (the weight tiles are free: every MMA has completed)
  long long* part = reinterpret_cast<long long*>(sA);
  if (ok && half == 1) {
#pragma unroll
    for (int c = 0; c < TC_N; c++)
      part[c * TC_M + lrow] = acc[c];
  }
  __syncthreads();
  if (ok && half == 0) {
#pragma unroll
    for (int c = 0; c < TC_N; c++)
      acc[c] += part[c * TC_M + lrow];
  }
  if (ok && active && half == 0) {
    // acc holds sum_g S_g 2^(8 (4 - g)); the slices' scales make the sum
    // acc 2^-48 2^rexp 2^F_c
    double* out = t.G + ((size_t)K.q0 * t.n_thetas + row) * TC_N;
#pragma unroll
    for (int c = 0; c < TC_N; c++) {
      if (c < t.np) {
        const double mx = __longlong_as_double((long long)t.colmax[tile.task * TC_N + c]);
        const int F = mx > 0 ? ilogb(mx) + 1 : 0;
        out[c] = scalbn((double)acc[c], rexp + F - 48);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (tid < 32)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(TC_TMEM_COLS) : "memory");
}

} // namespace

int gram_tc_columns() { return TC_N; }
long long gram_tc_block_bytes() { return B_BYTES; }
int gram_tc_block_rows() { return TC_KB; }
int gram_tc_tile_rows() { return TC_M; }

bool gram_tc_supported(int Ea) { return Ea >= 1 && Ea <= 5; }

void launch_gram_tc_slices(const GroupParams& g, const GramTC& t, int n_tasks, int max_lib, cudaStream_t s)
{
  if (n_tasks <= 0)
    return;
  const dim3 grid((unsigned)std::max(1, std::min(1024, (max_lib + TC_KB + 127) / 128)), (unsigned)n_tasks);
  switch (g.Ea) {
    case 1:
      gram_tc_colmax_kernel<1><<<grid, 128, 0, s>>>(g, t);
      gram_tc_slices_kernel<1><<<grid, 128, 0, s>>>(g, t);
      break;
    case 2:
      gram_tc_colmax_kernel<2><<<grid, 128, 0, s>>>(g, t);
      gram_tc_slices_kernel<2><<<grid, 128, 0, s>>>(g, t);
      break;
    case 3:
      gram_tc_colmax_kernel<3><<<grid, 128, 0, s>>>(g, t);
      gram_tc_slices_kernel<3><<<grid, 128, 0, s>>>(g, t);
      break;
    case 4:
      gram_tc_colmax_kernel<4><<<grid, 128, 0, s>>>(g, t);
      gram_tc_slices_kernel<4><<<grid, 128, 0, s>>>(g, t);
      break;
    case 5:
      gram_tc_colmax_kernel<5><<<grid, 128, 0, s>>>(g, t);
      gram_tc_slices_kernel<5><<<grid, 128, 0, s>>>(g, t);
      break;
    default: break;
  }
}

void launch_gram_tc(const GramTC& t, int n_tiles, cudaStream_t s)
{
  if (n_tiles <= 0)
    return;
  cudaFuncSetAttribute(gram_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM);
  gram_tc_kernel<<<n_tiles, TC_NT, TC_SMEM, s>>>(t);
}

} // namespace fedm
