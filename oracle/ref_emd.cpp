// Test infrastructure: the reference's own transport solver, compiled in
// place from the reference checkout (src/vendor/EMD_wrapper.h and the
// network simplex it includes, header-only, from POT) by oracle/Makefile into
// oracle/_ref/.  It exists only where the checkout does, and serves only to
// check the oracle's restatement of the Wasserstein cost
// (tests/test_oracle_wasserstein.py, tests/golden/make_wasserstein_goldens.py).
#include <vector>

#include "EMD_wrapper.h"

extern "C" double ref_emd_uniform(const double* D, int n1, int n2, int* ret)
{
  // src/distances.cpp:455-470: masses 1/len_i and 1/len_j, 10000 iterations
  std::vector<double> w1(n1, 1.0 / n1), w2(n2, 1.0 / n2), d(D, D + (size_t)n1 * n2);
  double cost = 0;
  *ret = EMD_wrap(n1, n2, w1.data(), w2.data(), d.data(), &cost, 10000);
  return cost;
}
