// Wasserstein distance between a library point and a prediction point, as
// the reference's wasserstein_distances computes it
// (EDM-Developers/fastEDM-r src/distances.cpp:270-527): the cost matrix of
// wasserstein_cost_matrix, then the optimal-transport cost with uniform
// masses 1/len_i and 1/len_j that wasserstein() takes from EMD_wrap
// (src/vendor/EMD_wrapper.h:34-117, POT's network simplex).
//
// The transport problem is solved here by successive shortest paths (an
// exact min-cost-flow method: Dijkstra with node potentials on the residual
// graph), with the masses scaled to integers: every source sends len_j
// units, every sink takes len_i units, len_i * len_j units in all.  The
// cost is summed as EMD_wrap sums it, flow * cost over the arcs from the
// last to the first.  Where the optimal plan is unique and the lengths are
// equal (a permutation with flows 1/n) that sum has the reference's bits.
// Often the plan is not unique -- costs that are sums of absolute
// differences of one-dimensional values tie across many permutations -- and
// the network simplex's pivot order picks one of the optimal plans; the
// same total summed over another plan differs in the last bits.  For
// unequal lengths the network simplex's flows also carry roundings of their
// own.  Either way the distances agree with the reference's to a few ulps.
//
// This header is included by kernels_exact.cu, which is built with
// --fmad=false: every product and sum rounds separately, as in the
// reference.
#pragma once

#include <cfloat>

#include "kernels.h"

namespace fedm {

// Optimal-transport cost of the n1 x n2 row-major cost matrix D with masses
// 1/n1 and 1/n2.  status becomes nonzero if the solver's bounded loop runs
// out (never expected: every augmentation moves at least one unit).
__device__ __noinline__ double emd_uniform(const double* D, int n1, int n2, int& status)
{
  const int V = n1 + n2;
  int sup[WASS_EMAX], dem[WASS_EMAX], prev[2 * WASS_EMAX];
  short f[WASS_EMAX * WASS_EMAX];
  double pot[2 * WASS_EMAX], dist[2 * WASS_EMAX];
  for (int i = 0; i < n1; i++)
    sup[i] = n2;
  for (int j = 0; j < n2; j++)
    dem[j] = n1;
  for (int a = 0; a < n1 * n2; a++)
    f[a] = 0;
  // potentials that make every forward reduced cost D + pot_i - pot_j >= 0
  for (int i = 0; i < n1; i++)
    pot[i] = 0.0;
  for (int j = 0; j < n2; j++) {
    double m = D[j];
    for (int i = 1; i < n1; i++)
      m = fmin(m, D[i * n2 + j]);
    pot[n1 + j] = m;
  }
  int remaining = n1 * n2;
  for (int it = 0; remaining > 0; it++) {
    if (it > n1 * n2 + 4) {
      status = 1;
      return 0.0;
    }
    unsigned done = 0;
    for (int v = 0; v < V; v++) {
      dist[v] = (v < n1 && sup[v] > 0) ? 0.0 : INFINITY;
      prev[v] = -1;
    }
    for (int step = 0; step < V; step++) {
      int u = -1;
      double du = INFINITY;
      for (int v = 0; v < V; v++)
        if (!((done >> v) & 1u) && dist[v] < du) {
          du = dist[v];
          u = v;
        }
      if (u < 0)
        break;
      done |= 1u << u;
      if (u < n1) {
        // forward arcs u -> sink j (unbounded)
        for (int j = 0; j < n2; j++) {
          const int v = n1 + j;
          if ((done >> v) & 1u)
            continue;
          const double nd = du + ((D[u * n2 + j] + pot[u]) - pot[v]);
          if (nd < dist[v]) {
            dist[v] = nd;
            prev[v] = u;
          }
        }
      } else {
        // backward arcs sink j -> source i where flow can be returned
        const int j = u - n1;
        for (int i = 0; i < n1; i++) {
          if (((done >> i) & 1u) || f[i * n2 + j] == 0)
            continue;
          const double nd = du + ((pot[u] - D[i * n2 + j]) - pot[i]);
          if (nd < dist[i]) {
            dist[i] = nd;
            prev[i] = u;
          }
        }
      }
    }
    int t = -1;
    double dtmin = INFINITY;
    for (int j = 0; j < n2; j++)
      if (dem[j] > 0 && dist[n1 + j] < dtmin) {
        dtmin = dist[n1 + j];
        t = j;
      }
    if (t < 0) {
      status = 1;
      return 0.0;
    }
    // potentials: reduced costs stay nonnegative (nodes beyond the sink's
    // distance, or unreached, move by the sink's distance)
    for (int v = 0; v < V; v++)
      pot[v] += fmin(dist[v], dtmin);
    // bottleneck along the path back from the sink
    int delta = dem[t];
    int v = n1 + t;
    while (prev[v] >= 0) {
      const int u = prev[v];
      if (v < n1)
        delta = min(delta, (int)f[v * n2 + (u - n1)]);
      v = u;
    }
    const int s = v;
    delta = min(delta, sup[s]);
    v = n1 + t;
    while (prev[v] >= 0) {
      const int u = prev[v];
      if (v >= n1)
        f[u * n2 + (v - n1)] += delta;
      else
        f[v * n2 + (u - n1)] -= delta;
      v = u;
    }
    sup[s] -= delta;
    dem[t] -= delta;
    remaining -= delta;
  }
  // EMD_wrap's sum: flow * cost over the arcs, last arc first
  const double L = (double)(n1 * n2);
  double cost = 0.0;
  for (int a = n1 * n2 - 1; a >= 0; a--)
    if (f[a] > 0)
      cost += ((double)f[a] / L) * D[a];
  return cost;
}

// The cost matrix of wasserstein_cost_matrix (src/distances.cpp:296-411)
// for library point x and prediction point y (rows of the manifold, E_a
// values each), and its transport cost.  The reference reads each point as
// a column-major rows x E matrix over the row's leading rows * E values
// (rows = 1 + [dt] + lagged extras), the unlagged extras after it; a column
// with a missing entry is left out (missing distance 0) or costs the missing
// distance.  pen is the panel term (idw or the id weight), added when
// has_pen.  Returns false where the reference keeps no distance: no
// columns, or a cost that is zero or not normal.
__device__ __noinline__ bool wasserstein_pair(const double* x, const double* y, int E, int rows, int n_unlagged,
                                              bool has_dt, double aspect_ratio, double missing_distance,
                                              bool has_pen, double pen, double& out, int& status)
{
  constexpr double MISS_W = 1.0e+100;
  const bool skip = missing_distance == 0;
  unsigned mx = 0, my = 0;
  for (int c = 0; c < E; c++)
    for (int r = 0; r < rows; r++) {
      if (x[c * rows + r] == MISS_W)
        mx |= 1u << c;
      if (y[c * rows + r] == MISS_W)
        my |= 1u << c;
    }
  const int li = skip ? E - __popc(mx) : E, lj = skip ? E - __popc(my) : E;
  if (li <= 0 || lj <= 0)
    return false;
  double gamma = 1.0;
  if (has_dt) {
    // the aspect ratio of the library point's curve (src/distances.cpp:340-362)
    double minData = DBL_MAX, maxData = DBL_MIN, maxTime = 0.0;
    for (int c = 0; c < E; c++) {
      const double v = x[c * rows], tv = x[c * rows + 1];
      if (v != MISS_W) {
        if (v < minData)
          minData = v;
        if (v > maxData)
          maxData = v;
      }
      if (tv != MISS_W && tv > maxTime)
        maxTime = tv;
    }
    const double eps = 1e-6;
    gamma = aspect_ratio * (maxData - minData + eps) / (maxTime + eps);
  }
  double unlagged = 0.0;
  for (int e = 0; e < n_unlagged; e++) {
    const double xe = x[E * rows + e], ye = y[E * rows + e];
    if (xe == MISS_W || ye == MISS_W)
      unlagged += missing_distance;
    else
      unlagged += fabs(xe - ye);
  }
  if (has_pen)
    unlagged += pen;
  // column-major li x lj, as the reference fills it
  double C[WASS_EMAX * WASS_EMAX];
  for (int a = 0; a < li * lj; a++)
    C[a] = unlagged;
  for (int k = 0; k < rows; k++) {
    int n = 0;
    for (int nn = 0; nn < E; nn++) {
      if (skip && ((mx >> nn) & 1u))
        continue;
      int m = 0;
      for (int mm = 0; mm < E; mm++) {
        if (skip && ((my >> mm) & 1u))
          continue;
        double dist;
        if (((mx >> nn) | (my >> mm)) & 1u)
          dist = missing_distance;
        else
          dist = fabs(x[nn * rows + k] - y[mm * rows + k]);
        if (has_dt && k == 1)
          dist *= gamma;
        C[m * li + n] += dist;
        m++;
      }
      n++;
    }
  }
  // EMD_wrap reads the flat buffer as a row-major li x lj matrix
  const double d = emd_uniform(C, li, lj, status);
  // std::isnormal: the exponent field is neither 0 (zero, subnormal) nor
  // all ones (infinity, NaN)
  const unsigned ex = ((unsigned)__double2hiint(d) >> 20) & 0x7ffu;
  if (d != 0 && ex != 0u && ex != 0x7ffu) {
    out = d;
    return true;
  }
  return false;
}

} // namespace fedm
