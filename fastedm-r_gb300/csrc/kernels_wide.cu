// Mixed-precision neighbour search and forecast with one prediction point
// per thread (knn_mixed_kernel has two):
//   * wide embeddings, E_a = 9..16 (dt columns double E_a, so E = 5..8 with
//     dt lands here), up to 30 neighbours: 32 candidate slots, 512-row tiles
//     of a float manifold with row stride 16;
//   * simplex and S-map at E_a <= 8, k <= 6 with six CTAs per SM (40
//     registers): more warps to hide the scan's and the FP64 solve's
//     latency (the default form).
// The kernel itself is one_point.cuh's knn_one_kernel.
#include "one_point.cuh"

namespace fedm {

namespace {

constexpr int WTILE = 512;  // wide form: library rows per tile, 32 KB of shared memory at E_a = 16
constexpr int WC = 32;      // wide form: candidate slots per point
constexpr int WS = 16;      // wide form: row stride of the float manifold

template<int EA, int ALG>
void launch_wide(const GroupParams& g, const MixedRun& m, int num_sms, cudaStream_t s)
{
  launch_one<EA, WC, WS, WTILE, ALG, 2>(g, m, num_sms, s);
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

template<int ALG>
void launch_one6(const GroupParams& g, const MixedRun& m, int num_sms, cudaStream_t s)
{
  constexpr int OCC = 6;
  switch (g.Ea) {
    case 1: launch_one<1, 8, 4, 1024, ALG, OCC>(g, m, num_sms, s); break;
    case 2: launch_one<2, 8, 4, 1024, ALG, OCC>(g, m, num_sms, s); break;
    case 3: launch_one<3, 8, 4, 1024, ALG, OCC>(g, m, num_sms, s); break;
    case 4: launch_one<4, 8, 4, 1024, ALG, OCC>(g, m, num_sms, s); break;
    case 5: launch_one<5, 8, 8, 1024, ALG, OCC>(g, m, num_sms, s); break;
    case 6: launch_one<6, 8, 8, 1024, ALG, OCC>(g, m, num_sms, s); break;
    case 7: launch_one<7, 8, 8, 1024, ALG, OCC>(g, m, num_sms, s); break;
    case 8: launch_one<8, 8, 8, 1024, ALG, OCC>(g, m, num_sms, s); break;
    default: break;
  }
}

void launch_mixed_one(const GroupParams& g, const MixedRun& m, int num_sms, cudaStream_t s)
{
  if (m.item_end <= m.item_begin)
    return;
  if (g.algorithm == 1)
    launch_one6<1>(g, m, num_sms, s);
  else
    launch_one6<0>(g, m, num_sms, s);
}

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
