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

void launch_mixed_one(const GroupParams& g, const MixedRun& m, int num_sms, cudaStream_t s)
{
  if (m.item_end <= m.item_begin)
    return;
  if (g.algorithm == 1)
    launch_one6_t<1, false>(g, m, num_sms, s);
  else
    launch_one6_t<0, false>(g, m, num_sms, s);
}

void launch_knn_wide(const GroupParams& g, const MixedRun& m, int num_sms, cudaStream_t s)
{
  if (m.item_end <= m.item_begin)
    return;
  if (g.algorithm == 1)
    launch_wide_t<1, false>(g, m, num_sms, s);
  else
    launch_wide_t<0, false>(g, m, num_sms, s);
}

} // namespace fedm
