// Manifold rows on the device (src/manifold.cpp:82-238): one thread per
// observation fills its row of the lagged manifold for one E -- the E lags
// of x (or co_x for coprediction), then with dt the E time differences, then
// the extras (lagged ones per lag, unlagged ones once) -- from the series
// uploaded once per call.  The lag search walks back from the row through
// the observation numbers, skipping missing observations and stopping at the
// row's panel boundary and at an overshoot, as the host generator
// (host.cpp: Generator::find_obs/fill_row) does; the dt columns are one
// subtraction and one multiply, unfused, so every row is the host's bits.
#include <climits>

#include "kernels.h"

namespace fedm {

namespace {

constexpr int OBS_MISSING = INT_MIN;
constexpr double VAL_MISSING = 1.0e+100;

// Observation number a + b in two's complement (the reference's builds wrap
// when a is the missing marker).
__device__ __forceinline__ int add_wrap(int a, long long b)
{
  return (int)((unsigned)a + (unsigned)(long long)b);
}

// src/manifold.cpp:82-123: walk k in the given direction to the observation
// numbered target within panel_id's rows.
__device__ bool find_obs(const ManifoldParams& s, int target, int& k, int direction, int panel_id)
{
  while (k >= 0 && k < s.n) {
    if (s.panel) {
      const int pk = s.panel[k];
      if (pk == OBS_MISSING) {
        k += direction;
        continue;
      }
      if (panel_id != pk)
        return false;
    }
    const int o = s.obs[k];
    if (o == OBS_MISSING) {
      k += direction;
      continue;
    }
    if (o == target)
      return true;
    if (direction > 0 ? o > target : o < target)
      return false;
    k += direction;
  }
  return false;
}

__global__ void manifold_kernel(ManifoldParams s, double* F)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < s.n; i += gridDim.x * blockDim.x) {
    double* out = F + (size_t)i * s.Ea;
    const int pid = s.panel ? s.panel[i] : -1;
    const int ti = s.target_row[i];
    const double tPred = (s.with_dt && ti >= 0) ? s.t[ti] : VAL_MISSING;
    int lagged = i, prev = i, k = i - 1;
    const int start = s.obs[i];
    for (int j = 0; j < s.E; j++) {
      bool found = j == 0;
      if (!found && find_obs(s, add_wrap(start, -(long long)j * s.tau), k, -1, pid)) {
        found = true;
        lagged = k;
      }
      out[j] = found ? s.x[lagged] : VAL_MISSING;
      if (s.with_dt) {
        double v = VAL_MISSING;
        if (found) {
          const double now = s.t[lagged];
          if (j == 0 || s.reldt) {
            if (now != VAL_MISSING && tPred != VAL_MISSING)
              v = __dmul_rn(s.w, __dsub_rn(tPred, now));
          } else {
            const double nxt = s.t[prev];
            if (nxt != VAL_MISSING && now != VAL_MISSING)
              v = __dmul_rn(s.w, __dsub_rn(nxt, now));
          }
        }
        out[s.E + j] = v;
      }
      for (int e = 0; e < s.num_extras; e++) {
        const double v = found ? s.extras[(size_t)e * s.n + lagged] : VAL_MISSING;
        if (e < s.num_extras_lagged)
          out[s.E + s.Edt + e * s.E + j] = v;
        else if (j == 0)
          out[s.E + s.Edt + s.num_extras_lagged * s.E + (e - s.num_extras_lagged)] = v;
      }
      prev = lagged;
    }
  }
}

} // namespace

void launch_manifold(const ManifoldParams& p, double* F, int num_sms, cudaStream_t s)
{
  if (p.n <= 0)
    return;
  constexpr int NT = 256;
  long long blocks = ((long long)p.n + NT - 1) / NT;
  if (blocks > (long long)num_sms * 8)
    blocks = (long long)num_sms * 8;
  manifold_kernel<<<(int)blocks, NT, 0, s>>>(p, F);
}

} // namespace fedm
