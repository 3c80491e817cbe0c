// The one-point-per-thread form for 7 <= k <= 14 at E_a <= 8: 16 candidate
// slots per point, 1024-row tiles, four 256-thread CTAs per SM.  The
// autotuner weighs it against knn_mixed_kernel (two points per thread) for
// each (algorithm, E_a, k); both give the FP64 path's bits.
#include "one_point.cuh"

namespace fedm {

namespace {

template<int ALG>
void launch_one16(const GroupParams& g, const MixedRun& m, int num_sms, cudaStream_t s)
{
  constexpr int OCC = 4;
  switch (g.Ea) {
    case 1: launch_one<1, 16, 4, 1024, ALG, OCC>(g, m, num_sms, s); break;
    case 2: launch_one<2, 16, 4, 1024, ALG, OCC>(g, m, num_sms, s); break;
    case 3: launch_one<3, 16, 4, 1024, ALG, OCC>(g, m, num_sms, s); break;
    case 4: launch_one<4, 16, 4, 1024, ALG, OCC>(g, m, num_sms, s); break;
    case 5: launch_one<5, 16, 8, 1024, ALG, OCC>(g, m, num_sms, s); break;
    case 6: launch_one<6, 16, 8, 1024, ALG, OCC>(g, m, num_sms, s); break;
    case 7: launch_one<7, 16, 8, 1024, ALG, OCC>(g, m, num_sms, s); break;
    case 8: launch_one<8, 16, 8, 1024, ALG, OCC>(g, m, num_sms, s); break;
    default: break;
  }
}

} // namespace

void launch_mixed_one16(const GroupParams& g, const MixedRun& m, int num_sms, cudaStream_t s)
{
  if (m.item_end <= m.item_begin)
    return;
  if (g.algorithm == 1)
    launch_one16<1>(g, m, num_sms, s);
  else
    launch_one16<0>(g, m, num_sms, s);
}

} // namespace fedm
