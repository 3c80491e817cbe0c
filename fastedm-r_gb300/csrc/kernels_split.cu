// The split S-map of the mixed path (MIXED_SPLIT; E_a <= 4, k <= 6).
//
// The fused S-map kernel (knn_one_kernel, ALG = 1) runs its FP32 scan at six
// CTAs per SM, 40 registers, and every thread then solves its own point's
// JacobiSVD with the work matrix and both rotation accumulators in local
// memory: ~1.2 KB of stack per thread, ~280 MB over the GPU's resident
// threads, more than L2 holds, so the solver's spills reach DRAM.
//
// Split, the scan (knn_one_kernel, ALG = 2) certifies and re-ranks each
// point's candidates as before and writes the settled neighbour list (rows
// and FP64 distances, at most six) to a list buffer; smap_list_kernel makes
// the forecasts from the lists with W, U and V in registers (no stack), at a
// few warps per SM -- the FP64 pipe, a small fraction of the FP32 rate on
// this GPU, needs few warps to stay busy.  The engine runs the scan of one
// chunk of work items beside the solves of the previous chunk on a second
// stream.  Every operation and its order are those of smap_point_local, so
// forecasts and coefficients are the same bits.
#include "one_point.cuh"
#include "smap_solve_n.cuh"

namespace fedm {

namespace {

// N x N matrix of one thread held in registers (every index is a
// compile-time constant once svd_solve_nm is unrolled).  For E_a <= 3 both
// rotation accumulators live in registers; at E_a = 4 they sit in shared
// memory, interleaved across the CTA's threads (conflict-free: a warp's
// threads touch 32 consecutive doubles), and only W stays in registers,
// which keeps the kernel within its registers without spilling.
template<int N>
struct RegMat
{
  mutable double a[N][N];
  __device__ __forceinline__ double& operator()(int i, int j) const { return a[i][j]; }
};

constexpr int SOLVE_NT = 64;  // threads per solver CTA

template<int EA>
__host__ __device__ constexpr bool uv_in_registers() { return EA <= 3; }

template<int EA>
__host__ __device__ constexpr size_t solve_smem()
{
  return uv_in_registers<EA>() ? 0 : (size_t)2 * (EA + 1) * (EA + 1) * SOLVE_NT * sizeof(double);
}

template<int EA>
__global__ void __launch_bounds__(SOLVE_NT) smap_list_kernel(GroupParams g, SolveRun r)
{
  constexpr int n = EA + 1;
  extern __shared__ double uv_smem[];
  const long long slots = (long long)(r.item_end - r.item_begin) * TPB;
  unsigned long long ops = 0;
  for (long long slot = (long long)blockIdx.x * SOLVE_NT + threadIdx.x; slot < slots;
       slot += (long long)gridDim.x * SOLVE_NT) {
    const int keff = r.l_keff[slot];
    if (keff <= 0)
      continue;
    const int2 it = r.items[r.item_begin + (int)(slot / TPB)];
    const DevTask& T = g.tasks[it.x];
    const int si = it.y + (int)(slot % TPB);  // the scan's slot order
    const int i = T.perm_off >= 0 ? g.perm[T.perm_off + si] : si;
    const long long p = T.point_base + i;
    const int prow = g.pred_rows[T.pred_off + i];
    int rows[SPLIT_SLOTS];
    double cd[SPLIT_SLOTS];
#pragma unroll
    for (int j = 0; j < SPLIT_SLOTS; j++)
      if (j < keff) {
        rows[j] = r.l_rows[j * r.l_slots + slot];
        cd[j] = r.l_dist[j * r.l_slots + slot];
      }
    // smap_point_local's operations in its order (src/edm.cpp:737-814)
    int pops = keff + 1 + g.n_thetas * (keff * (EXP_OPS + 2 + n + n * (n + 1) + 2 * n) + 2 * EA);
    double y[EA];
#pragma unroll
    for (int j = 0; j < EA; j++)
      y[j] = g.Fp[(size_t)prow * EA + j];
    double mean = 0;
#pragma unroll
    for (int j = 0; j < SPLIT_SLOTS; j++)
      if (j < keff)
        mean = add(mean, cd[j]);
    mean = dvd(mean, (double)keff);
    const double ymean = rcp(mean);
    const bool save = g.coeffs && T.save_coeffs;
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
#pragma unroll
      for (int q = 0; q < SPLIT_SLOTS; q++) {
        if (q < keff) {
          const double w = exp_rn(mul(-theta, dvd_r(cd[q], mean, ymean)));
          const int row = rows[q];
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
      }
#pragma unroll
      for (int a = 0; a < n; a++)
#pragma unroll
        for (int b = 0; b < a; b++)
          W[a][b] = W[b][a];
      if constexpr (uv_in_registers<EA>()) {
        RegMat<n> U, V;
        svd_solve_nm<n>(W, bv, xs, U, V, pops);
      } else {
        const StridedMat<n> U{ uv_smem + threadIdx.x, SOLVE_NT }, V{ uv_smem + n * n * SOLVE_NT + threadIdx.x,
                                                                    SOLVE_NT };
        svd_solve_nm<n>(W, bv, xs, U, V, pops);
      }
      double fc = xs[0];
#pragma unroll
      for (int j = 0; j < EA; j++)
        fc = add(fc, mul(y[j], xs[j + 1]));
      if (save && t == g.n_thetas - 1) {
#pragma unroll
        for (int j = 0; j < n; j++)
          g.coeffs[(size_t)p * n + j] = fabs(xs[j]) < 1.0e-11 ? MISS : xs[j];
      }
      g.pred[(size_t)t * g.total_points + p] = fc;
    }
    ops += pops;
  }
  if (r.fp64_ops) {
    for (int o = 16; o > 0; o >>= 1)
      ops += __shfl_xor_sync(0xffffffffu, ops, o);
    if ((threadIdx.x & 31) == 0)
      atomicAdd(r.fp64_ops, ops);
  }
}

template<int EA>
void launch_solve(const GroupParams& g, const SolveRun& r, int num_sms, int ctas_per_sm, cudaStream_t s)
{
  const long long slots = (long long)(r.item_end - r.item_begin) * TPB;
  long long blocks = (long long)num_sms * (ctas_per_sm > 0 ? ctas_per_sm : 1);
  const long long need = (slots + SOLVE_NT - 1) / SOLVE_NT;
  if (blocks > need)
    blocks = need;
  if (blocks < 1)
    return;
  constexpr size_t smem = solve_smem<EA>();
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(smap_list_kernel<EA>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  smap_list_kernel<EA><<<(int)blocks, SOLVE_NT, smem, s>>>(g, r);
}

// The list scan: knn_one_kernel's default S-map shape (eight candidate
// slots, 1024-row tiles), writing lists instead of forecasts.
template<int EA>
void launch_scan(const GroupParams& g, const MixedRun& m, int num_sms, cudaStream_t s)
{
  launch_one<EA, 8, EA <= 4 ? 4 : 8, 1024, 2, 6>(g, m, num_sms, s);
}

} // namespace

void launch_smap_scan_lists(const GroupParams& g, const MixedRun& m, int num_sms, cudaStream_t s)
{
  if (m.item_end <= m.item_begin)
    return;
  switch (g.Ea) {
    case 1: launch_scan<1>(g, m, num_sms, s); break;
    case 2: launch_scan<2>(g, m, num_sms, s); break;
    case 3: launch_scan<3>(g, m, num_sms, s); break;
    case 4: launch_scan<4>(g, m, num_sms, s); break;
    default: break;
  }
}

void launch_smap_lists(const GroupParams& g, const SolveRun& r, int num_sms, int ctas_per_sm, cudaStream_t s)
{
  if (r.item_end <= r.item_begin)
    return;
  switch (g.Ea) {
    case 1: launch_solve<1>(g, r, num_sms, ctas_per_sm, s); break;
    case 2: launch_solve<2>(g, r, num_sms, ctas_per_sm, s); break;
    case 3: launch_solve<3>(g, r, num_sms, ctas_per_sm, s); break;
    case 4: launch_solve<4>(g, r, num_sms, ctas_per_sm, s); break;
    default: break;
  }
}

} // namespace fedm
