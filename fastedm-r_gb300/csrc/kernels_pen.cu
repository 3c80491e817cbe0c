// The one-point mixed kernels for panels with a finite penalty
// (panelWeight = idw > 0, src/distances.cpp:180-181): knn_one_kernel with
// PEN set, in all three one-point forms (eight or sixteen candidate slots at
// E_a <= 8, the wide form at E_a 9..16).  The penalty enters the FP32 scan
// per pair (one_point.cuh) and the FP64 re-rank as the reference's first
// term (prepare_point), so neighbours and forecasts are the FP64 path's
// bits.  A translation unit of its own so that it compiles beside the
// unpenalised forms.
#include "one_point.cuh"

namespace fedm {

void launch_mixed_pen(const GroupParams& g, const MixedRun& m, int C, int num_sms, cudaStream_t s)
{
  if (m.item_end <= m.item_begin)
    return;
  const bool smap = g.algorithm == 1;
  if (g.Ea > 8) {
    if (smap)
      launch_wide_t<1, true>(g, m, num_sms, s);
    else
      launch_wide_t<0, true>(g, m, num_sms, s);
  } else if (C == 16) {
    if (smap)
      launch_one16_t<1, true>(g, m, num_sms, s);
    else
      launch_one16_t<0, true>(g, m, num_sms, s);
  } else {
    if (smap)
      launch_one6_t<1, true>(g, m, num_sms, s);
    else
      launch_one6_t<0, true>(g, m, num_sms, s);
  }
}

} // namespace fedm
