// The one-point-per-thread form for 7 <= k <= 14 at E_a <= 8: 16 candidate
// slots per point, 1024-row tiles, four 256-thread CTAs per SM.  The
// autotuner weighs it against knn_mixed_kernel (two points per thread) for
// each (algorithm, E_a, k); both give the FP64 path's bits.
#include "one_point.cuh"

namespace fedm {

void launch_mixed_one16(const GroupParams& g, const MixedRun& m, int num_sms, cudaStream_t s)
{
  if (m.item_end <= m.item_begin)
    return;
  if (g.algorithm == 1)
    launch_one16_t<1, false>(g, m, num_sms, s);
  else
    launch_one16_t<0, false>(g, m, num_sms, s);
}

} // namespace fedm
