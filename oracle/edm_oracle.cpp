/*
 * edm_oracle.cpp -- TEST INFRASTRUCTURE ONLY (see edm_oracle.h).
 *
 * A plain, single-source C++ restatement of fastEDM's prediction path.  Every
 * function cites the reference file:line it follows (paths relative to the
 * reference project root).  Arithmetic is kept in the reference's order and
 * the file is compiled with -ffp-contract=off so no FMA is introduced.
 * Reductions that the reference delegates to Eigen (mean, sum, products,
 * JacobiSVD) are written as plain sequential loops / a restatement of Eigen
 * 3.3's published two-sided Jacobi SVD.
 */
#include "edm_oracle.h"

#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <numeric>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace {

// src/manifold.h:6-8
const double MISSING_D = 1.0e+100;
const int MISSING_I = INT_MIN;

// src/common.h:3-13
enum : int
{
  SUCCESS = 0,
  BREAK_HIT = 1,
  INSUFFICIENT_UNIQUE = 503,
  INVALID_ALGORITHM = 400,
  UNKNOWN_ERROR = 8000
};

enum class Algorithm
{
  Simplex,
  SMap
};
enum class Distance
{
  MeanAbsoluteError,
  Euclidean,
  Wasserstein
};

// Wrapping int addition: the reference adds offsets to MISSING_I observation
// numbers in a few places (src/manifold.cpp:183,255,290); two's complement
// wrap is what those builds do in practice.
inline int wrap_add(int a, long long b)
{
  return (int)(uint32_t)((uint32_t)a + (uint32_t)(int64_t)b);
}

// ------------------------------------------------------------------- exp
// The reference calls std::exp (src/edm.cpp:723,745).  For bit-level
// comparison with the GPU library the oracle can instead evaluate the same
// IEEE-only exp formula the device uses: Cody-Waite reduction with a 32-bit
// head of ln 2, a degree-13 Taylor polynomial with fused multiply-adds and an
// exact 2^k scaling.  Mode 0 (default) = std::exp, mode 1 = that formula.
int g_exp_mode = 0;
// Benchmark sampling only: predict every g_pred_stride-th row of each task's
// prediction set (1 = all rows, the reference's behaviour).
int g_pred_stride = 1;

// Order of the floating-point sums that the reference leaves to Eigen and to
// its compiler.  Quantification only: it measures how far the reference's
// own builds spread.  0, the default, is the plain sequential unfused order,
// which the GPU library reproduces bit for bit.  Bits:
//   1, 2  Eigen's vectorised order with packets of 2 (SSE2, NEON) or 4 (AVX)
//         doubles, in the S-map's three Eigen reductions (src/edm.cpp:745,
//         781-782): mean(d) (Redux.h, linear vectorised traversal), X^T X
//         (a coefficient-wise lazy product, each entry such a reduction,
//         below Eigen's threshold rows+cols+depth < 20; else a GEMM whose
//         depth is blocked, GEMM_KC rows per block, each block summed in
//         order) and X^T y (a row-major GEMV: one packet accumulator per
//         row, then the horizontal sum and the scalar tail);
//   4     the multiply-adds of those products fused (Eigen's pmadd on FMA
//         targets);
//   8     the reference's own scalar loops contracted to FMA, as GCC's
//         default -ffp-contract=fast does on aarch64: the distance sums
//         (src/distances.cpp:211-215), the simplex sum (src/edm.cpp:729) and
//         the S-map forecast (src/edm.cpp:793-797).
int g_sum_mode = 0;
const int GEMM_KC = 256;

inline double mac(double a, double b, double c, bool fused)
{
  return fused ? std::fma(a, b, c) : a * b + c;
}

// Horizontal sum of one packet: l0 + l1, or (l0 + l2) + (l1 + l3).
inline double predux(const double* l, int P)
{
  return P == 2 ? l[0] + l[1] : (l[0] + l[2]) + (l[1] + l[3]);
}

// Eigen's linear vectorised reduction of v[0..n) (or of the products
// a[i*sa] * b[i*sb] when a is given) with packets of P and no aligned
// prefix: two packet accumulators over blocks of 2P, combined, one more
// packet if it fits, the horizontal sum, then the remaining scalars.
double packet_reduce(const double* v, const double* a, int sa, const double* b, int sb, int n, int P, bool fused)
{
  auto term = [&](int i) { return a ? a[(size_t)i * sa] * b[(size_t)i * sb] : v[i]; };
  auto acc = [&](double c, int i) { return a ? mac(a[(size_t)i * sa], b[(size_t)i * sb], c, fused) : c + v[i]; };
  const int aligned = n / P * P, aligned2 = n / (2 * P) * (2 * P);
  if (aligned == 0) {
    double r = term(0);
    for (int i = 1; i < n; i++)
      r = acc(r, i);
    return r;
  }
  double p0[4], p1[4];
  for (int l = 0; l < P; l++)
    p0[l] = term(l);
  if (aligned > P) {
    for (int l = 0; l < P; l++)
      p1[l] = term(P + l);
    for (int i = 2 * P; i < aligned2; i += 2 * P)
      for (int l = 0; l < P; l++) {
        p0[l] = acc(p0[l], i + l);
        p1[l] = acc(p1[l], i + P + l);
      }
    for (int l = 0; l < P; l++)
      p0[l] = p0[l] + p1[l];
    if (aligned > aligned2)
      for (int l = 0; l < P; l++)
        p0[l] = acc(p0[l], aligned2 + l);
  }
  double r = predux(p0, P);
  for (int i = aligned; i < n; i++)
    r = acc(r, i);
  return r;
}

// Row-major GEMV order: one packet accumulator from zero over the full
// packets, the horizontal sum, then the scalar tail.
double gemv_dot(const double* a, int sa, const double* b, int sb, int n, int P, bool fused)
{
  double l[4] = { 0, 0, 0, 0 };
  const int aligned = n / P * P;
  for (int i = 0; i < aligned; i += P)
    for (int q = 0; q < P; q++)
      l[q] = mac(a[(size_t)(i + q) * sa], b[(size_t)(i + q) * sb], l[q], fused);
  double r = predux(l, P);
  for (int i = aligned; i < n; i++)
    r = mac(a[(size_t)i * sa], b[(size_t)i * sb], r, fused);
  return r;
}

// GEMM order: the depth in blocks of GEMM_KC, each summed in order into a
// register from zero, the blocks added to the result in turn.
double blocked_dot(const double* a, int sa, const double* b, int sb, int n, bool fused)
{
  double r = 0;
  for (int i0 = 0; i0 < n; i0 += GEMM_KC) {
    double c = 0;
    for (int i = i0; i < std::min(n, i0 + GEMM_KC); i++)
      c = mac(a[(size_t)i * sa], b[(size_t)i * sb], c, fused);
    r = r + c;
  }
  return r;
}

double pow2i(int k)
{
  uint64_t b = (uint64_t)(k + 1023) << 52;
  double d;
  std::memcpy(&d, &b, 8);
  return d;
}

double exp_rn(double x)
{
  if (!(x == x))
    return x;
  if (x > 709.782712893384)
    return INFINITY;
  if (x < -745.1332191019412)
    return 0.0;
  const double k = std::rint(x * 0x1.71547652b82fep+0);
  double r = std::fma(-k, 0x1.62e42ff000000p-1, x);
  r = std::fma(-k, -0x1.718432a1b0e26p-35, r);
  static const double c[14] = { 1.0, 1.0, 0.5, 0x1.5555555555555p-3, 0x1.5555555555555p-5, 0x1.1111111111111p-7,
                                0x1.6c16c16c16c17p-10, 0x1.a01a01a01a01ap-13, 0x1.a01a01a01a01ap-16,
                                0x1.71de3a556c734p-19, 0x1.27e4fb7789f5cp-22, 0x1.ae64567f544e4p-26,
                                0x1.1eed8eff8d898p-29, 0x1.6124613a86d09p-33 };
  double p = c[13];
  for (int i = 12; i >= 0; i--)
    p = std::fma(p, r, c[i]);
  int ki = (int)k;
  if (ki < -1021) {
    p = p * pow2i(-600);
    ki += 600;
  } else if (ki > 1023) {
    p = p * 2.0;
    ki -= 1;
  }
  return p * pow2i(ki);
}

inline double edm_exp(double x)
{
  return g_exp_mode ? exp_rn(x) : std::exp(x);
}

// ---------------------------------------------------------------- stats.cpp
double seq_sum(const std::vector<double>& v)
{
  double s = 0.0;
  for (double a : v)
    s += a;
  return s;
}

// src/stats.cpp:96-101 (n-1 denominator)
double standard_deviation(const std::vector<double>& v)
{
  double mean = seq_sum(v) / (double)v.size();
  double ss = 0.0;
  for (double a : v) {
    double c = a - mean;
    ss += c * c;
  }
  return std::sqrt(ss / (double)((long long)v.size() - 1));
}

std::vector<double> remove_missing(const std::vector<double>& v)
{
  std::vector<double> out;
  for (double a : v)
    if (a != MISSING_D)
      out.push_back(a);
  return out;
}

// src/stats.cpp:103-108
double default_missing_distance(const std::vector<double>& x)
{
  auto xo = remove_missing(x);
  double sd = standard_deviation(xo);
  return 2 / std::sqrt(3.14159265358979323846) * sd;
}

// src/stats.cpp:64-82 (centred sums; MISSING if either SD < 1e-9)
double correlation(const std::vector<double>& y1, const std::vector<double>& y2)
{
  size_t n = y1.size();
  double m1 = seq_sum(y1) / (double)n, m2 = seq_sum(y2) / (double)n;
  double s11 = 0, s22 = 0, s12 = 0;
  for (size_t i = 0; i < n; i++) {
    double a = y1[i] - m1, b = y2[i] - m2;
    s11 += a * a;
    s22 += b * b;
    s12 += a * b;
  }
  double sd1 = std::sqrt(s11), sd2 = std::sqrt(s22);
  if (sd1 < 1e-9 || sd2 < 1e-9)
    return MISSING_D;
  return s12 / (sd1 * sd2);
}

// src/stats.cpp:84-94
double mean_absolute_error(const std::vector<double>& y1, const std::vector<double>& y2)
{
  double s = 0;
  for (size_t i = 0; i < y1.size(); i++)
    s += std::abs(y1[i] - y2[i]);
  double mae = s / (double)y1.size();
  return mae < 1e-8 ? 0 : mae;
}

// src/stats.cpp:10-28
double median(std::vector<double> u)
{
  if (u.size() % 2 == 0) {
    auto it1 = u.begin() + u.size() / 2 - 1;
    auto it2 = u.begin() + u.size() / 2;
    std::nth_element(u.begin(), it1, u.end());
    double e1 = *it1;
    std::nth_element(u.begin(), it2, u.end());
    double e2 = *it2;
    return (e1 + e2) / 2;
  }
  auto it = u.begin() + u.size() / 2;
  std::nth_element(u.begin(), it, u.end());
  return *it;
}

// src/stats.cpp:30-47 (1-based ranks)
std::vector<int> rank_of(const std::vector<double>& v)
{
  std::vector<std::pair<double, int>> s(v.size());
  for (size_t i = 0; i < v.size(); i++)
    s[i] = { v[i], (int)i };
  std::sort(s.begin(), s.end());
  std::vector<int> r(v.size());
  for (size_t i = 0; i < s.size(); i++)
    r[s[i].second] = (int)i + 1;
  return r;
}

// ------------------------------------------------ vendor/mersennetwister.h
// MT19937-64 (Matsumoto & Nishimura) in the reference's "left/next" form:
// init leaves left=1 so the first draw tempers the raw seed word
// (src/vendor/mersennetwister.h:88-146).
struct MT64
{
  uint64_t s[312];
  size_t left;
  int next;

  void init(uint64_t seed)
  {
    s[0] = seed;
    for (int j = 1; j < 312; j++)
      s[j] = 6364136223846793005ULL * (s[j - 1] ^ (s[j - 1] >> 62)) + (uint64_t)j;
    left = 1;
    next = 0;
  }
  static uint64_t twist(uint64_t u, uint64_t v)
  {
    return (((u & 0xFFFFFFFF80000000ULL) | (v & 0x7FFFFFFFULL)) >> 1) ^ ((v & 1ULL) ? 0xB5026F5AA96619E9ULL : 0ULL);
  }
  void next_state()
  {
    left = 311;
    next = 0;
    int i = 0;
    for (; i < 156; i++)
      s[i] = s[i + 156] ^ twist(s[i], s[i + 1]);
    for (; i < 311; i++)
      s[i] = s[i - 156] ^ twist(s[i], s[i + 1]);
    s[311] = s[155] ^ twist(s[311], s[0]);
  }
  static uint64_t temper(uint64_t y)
  {
    y ^= (y >> 29) & 0x5555555555555555ULL;
    y ^= (y << 17) & 0x71D67FFFEDA60000ULL;
    y ^= (y << 37) & 0xFFF7EEE000000000ULL;
    y ^= (y >> 43);
    return y;
  }
  double real2()
  {
    if (left-- == 0)
      next_state();
    return (double)(temper(s[next++]) >> 11) * (1.0 / 9007199254740992.0);
  }
};

// ---------------------------------------------------- manifold.h / .cpp
// src/manifold.cpp:7-18
double gcd(double a, double b)
{
  if (a < b)
    return gcd(b, a);
  if (std::fabs(b) < 0.001)
    return a;
  return gcd(b, a - std::floor(a / b) * b);
}

struct Generator
{
  std::vector<double> t, x, xmap, co_x;
  std::vector<std::vector<double>> extras;
  std::vector<int> panelIDs;
  int tau = 1, p = 0, num_extras = 0, num_extras_lagged = 0;
  bool dt = false, reldt = false, allow_missing = false, panel_mode = false, xmap_mode = false;
  std::vector<int> obs;
  double dtWeight = 0;

  // src/manifold.h:85-127
  Generator(const std::vector<double>& t_, const std::vector<double>& x_, int tau_, int p_,
            const std::vector<double>& xmap_, const std::vector<double>& co_x_, const std::vector<int>& panel_,
            const std::vector<std::vector<double>>& extras_, int numExtrasLagged, bool dt_, bool reldt_,
            bool allowMissing, double dtWeight_)
    : t(t_), x(x_), xmap(xmap_), co_x(co_x_), extras(extras_), panelIDs(panel_), tau(tau_), p(p_),
      num_extras((int)extras_.size()), num_extras_lagged(numExtrasLagged), dt(dt_), reldt(reldt_),
      allow_missing(allowMissing), panel_mode(!panel_.empty()), xmap_mode(!xmap_.empty()), dtWeight(dtWeight_)
  {
    if ((dt_ || reldt_) && dtWeight_ == 0.0) {
      dt = true;
      reldt = false;
      setup_observation_numbers();
      double w = default_dt_weight();
      if (w > 0) {
        dt = dt_;
        reldt = reldt_;
        dtWeight = w;
      } else {
        dt = false;
        reldt = false;
        dtWeight = 0;
      }
    }
    setup_observation_numbers();
  }

  int numObs() const { return (int)t.size(); }
  int E_dt(int E) const { return (dt || reldt) * E; }
  int E_extras(int E) const { return num_extras + num_extras_lagged * (E - 1); }
  int E_actual(int E) const { return E + E_dt(E) + E_extras(E); }

  // src/manifold.h:53-67
  double default_dt_weight() const
  {
    double xSD = standard_deviation(remove_missing(x));
    std::vector<double> d(t.size());
    for (int i = 0; i < numObs(); i++)
      d[i] = get_dt(i);
    double dtSD = standard_deviation(remove_missing(d));
    if (dtSD == 0.0)
      return -1;
    return xSD / dtSD;
  }

  // src/manifold.cpp:20-48
  double calculate_time_increment() const
  {
    double unit = -1;
    for (int i = 1; i < numObs(); i++) {
      double diff = t[i] - t[i - 1];
      if (diff <= 0 || t[i] == MISSING_D || t[i - 1] == MISSING_D)
        continue;
      if (unit < 0) {
        unit = diff;
        continue;
      }
      unit = gcd(diff, unit);
    }
    return unit;
  }

  // src/manifold.cpp:50-80
  void setup_observation_numbers()
  {
    obs.clear();
    if (!(dt || reldt)) {
      double unit = calculate_time_increment();
      double minT = *std::min_element(t.begin(), t.end());
      for (int i = 0; i < numObs(); i++)
        obs.push_back(t[i] != MISSING_D ? (int)std::round((t[i] - minT) / unit) : MISSING_I);
    } else {
      int countUp = 0;
      for (int i = 0; i < numObs(); i++) {
        if (t[i] != MISSING_D && (allow_missing || x[i] != MISSING_D))
          obs.push_back(countUp++);
        else
          obs.push_back(MISSING_I);
      }
    }
  }

  // src/manifold.cpp:82-123
  bool find_observation_num(int target, int& k, int direction, int panel) const
  {
    while (k >= 0 && k < (int)obs.size()) {
      if (panel_mode) {
        if (panelIDs[k] == MISSING_I) {
          k += direction;
          continue;
        }
        if (panel != panelIDs[k])
          return false;
      }
      if (obs[k] == MISSING_I) {
        k += direction;
        continue;
      }
      if (obs[k] == target)
        return true;
      if (direction > 0 && obs[k] > target)
        return false;
      if (direction < 0 && obs[k] < target)
        return false;
      k += direction;
    }
    return false;
  }

  // src/manifold.cpp:281-312
  double get_target(int i, bool copred, bool predSet, int& targetIndex) const
  {
    int panel = panel_mode ? panelIDs[i] : -1;
    bool use_co_x = copred && predSet;
    if (p != 0) {
      int target = wrap_add(obs[targetIndex], p);
      int direction = p > 0 ? 1 : -1;
      if (!find_observation_num(target, targetIndex, direction, panel))
        targetIndex = -1;
    }
    if (targetIndex < 0)
      return MISSING_D;
    if (use_co_x)
      return co_x[targetIndex];
    if (xmap_mode)
      return xmap[targetIndex];
    return x[targetIndex];
  }

  // src/manifold.cpp:240-279
  double get_dt(int i) const
  {
    double tNow = t[i];
    if (tNow == MISSING_D)
      return MISSING_D;
    int target = wrap_add(obs[i], -(long long)tau);
    int lagged = i - 1;
    int panel = panel_mode ? panelIDs[i] : -1;
    double tPrev;
    if (find_observation_num(target, lagged, -1, panel))
      tPrev = t[lagged];
    else
      return MISSING_D;
    if (!reldt)
      return tNow - tPrev;
    int ti = i;
    get_target(i, false, true, ti);
    if (ti < 0)
      return MISSING_D;
    return t[ti] - tPrev;
  }

  // src/manifold.cpp:156-238
  void fill_in_point(int i, int E, bool copred, bool predSet, double w, double* point) const
  {
    int panel = panel_mode ? panelIDs[i] : -1;
    bool use_co_x = copred && predSet;
    double tPred = 0;
    if (dt || reldt) {
      int ti = i;
      get_target(i, copred, predSet, ti);
      tPred = (ti >= 0) ? t[ti] : MISSING_D;
    }
    int laggedIndex = i;
    int start = obs[i];
    int k = i - 1;
    int prevLaggedIndex = laggedIndex;
    int Edt = E_dt(E);
    for (int j = 0; j < E; j++) {
      bool found = (j == 0);
      if (!found) {
        int target = wrap_add(start, -(long long)j * tau);
        if (find_observation_num(target, k, -1, panel)) {
          found = true;
          laggedIndex = k;
        }
      }
      if (!found)
        point[j] = MISSING_D;
      else if (use_co_x)
        point[j] = co_x[laggedIndex];
      else
        point[j] = x[laggedIndex];

      if (dt || reldt) {
        if (!found) {
          point[j + E] = MISSING_D;
        } else {
          double tNow = t[laggedIndex];
          if (j == 0 || reldt) {
            point[E + j] = (tNow != MISSING_D && tPred != MISSING_D) ? w * (tPred - tNow) : MISSING_D;
          } else {
            double tNext = t[prevLaggedIndex];
            point[E + j] = (tNext != MISSING_D && tNow != MISSING_D) ? w * (tNext - tNow) : MISSING_D;
          }
        }
      }
      for (int e = 0; e < num_extras; e++) {
        double v = found ? extras[e][laggedIndex] : MISSING_D;
        if (e < num_extras_lagged)
          point[E + Edt + e * E + j] = v;
        else if (j == 0)
          point[E + Edt + num_extras_lagged * E + (e - num_extras_lagged)] = v;
      }
      prevLaggedIndex = laggedIndex;
    }
  }

  // src/manifold.cpp:314-360
  std::vector<bool> generate_usable(int maxE, bool copred) const
  {
    std::vector<bool> usable(t.size());
    int sz = E_actual(maxE);
    std::vector<double> point(std::max(sz, 1));
    for (int i = 0; i < numObs(); i++) {
      if (t[i] == MISSING_D || (panel_mode && panelIDs[i] == MISSING_I)) {
        usable[i] = false;
        continue;
      }
      fill_in_point(i, maxE, copred, copred, 1.0, point.data());
      bool ok;
      if (allow_missing) {
        ok = false;
        for (int j = 0; j < sz; j++)
          if (point[j] != MISSING_D) {
            ok = true;
            break;
          }
      } else {
        ok = true;
        for (int j = 0; j < sz; j++)
          if (point[j] == MISSING_D) {
            ok = false;
            break;
          }
      }
      usable[i] = ok;
    }
    return usable;
  }
};

// src/manifold.h:140-286 (eager and lazy forms hold identical values)
struct Manifold
{
  const Generator* gen;
  std::vector<double> flat, targets, targetTimes, pointTimes;
  std::vector<int> panels, rows;
  int numPoints = 0, E_x = 0, E_actual = 0;
  bool predSet, copred;

  Manifold(const Generator& g, int E, const std::vector<bool>& filter, bool predictionSet, bool copredictMode)
    : gen(&g), predSet(predictionSet), copred(copredictMode)
  {
    E_x = E;
    E_actual = g.E_actual(E);
    bool every = filter.empty();
    for (int i = 0; i < g.numObs(); i++) {
      if (every || filter[i]) {
        int ti = i;
        double target = g.get_target(i, copredictMode, predictionSet, ti);
        if (!predictionSet && target == MISSING_D)
          continue;  // src/manifold.h:186-189
        rows.push_back(i);
        pointTimes.push_back(g.t[i]);
        targets.push_back(target);
        targetTimes.push_back(target != MISSING_D ? g.t[ti] : MISSING_D);
        if (g.panel_mode)
          panels.push_back(g.panelIDs[i]);
      }
    }
    numPoints = (int)rows.size();
    flat.assign((size_t)numPoints * E_actual, 0.0);
    for (int i = 0; i < numPoints; i++)
      g.fill_in_point(rows[i], E_x, copred, predSet, g.dtWeight, &flat[(size_t)i * E_actual]);
  }
  double operator()(int i, int j) const { return flat[(size_t)i * E_actual + j]; }
  int panel(int i) const { return panels[i]; }
};

// --------------------------------------------------------------- Options
struct Options
{
  bool copredict = false, forceCompute = true, saveTargets = false, savePrediction = false, saveSMAPCoeffs = false;
  int k = 0, nthreads = 1, library = 0;
  double missingdistance = 0;
  bool panelMode = false;
  double idw = 0;
  std::map<std::pair<int, int>, float> idWeights;
  std::vector<double> thetas;
  Algorithm algorithm = Algorithm::Simplex;
  int taskNum = 0, numTasks = 0, configNum = 0;
  Distance distance = Distance::Euclidean;
  double aspectRatio = 0;
  bool lowMemoryMode = false, useOnlyPastToPredictFuture = false, hasMissing = false;
};

struct DistanceIndexPairs
{
  std::vector<int> inds;
  std::vector<double> dists;
};

// src/distances.cpp:151-229 (eager) and :69-149 (lazy).  All metrics are
// Metric::Diff because run_command never builds a categorical one
// (src/r.cpp:241-244).  The lazy form has no past-only rule.
DistanceIndexPairs lp_distances(int Mp_i, const Options& opts, const Manifold& M, const Manifold& Mp)
{
  DistanceIndexPairs out;
  const bool skipOtherPanels = opts.panelMode && (opts.idw < 0);
  const bool skipFuture = opts.useOnlyPastToPredictFuture && !opts.lowMemoryMode;
  const bool l1 = opts.distance == Distance::MeanAbsoluteError;
  const bool hasMissing = opts.lowMemoryMode ? true : opts.hasMissing;
  for (int i = 0; i < M.numPoints; i++) {
    if (skipOtherPanels && M.panel(i) != Mp.panel(Mp_i))
      continue;
    if (skipFuture && M.targetTimes[i] > Mp.pointTimes[Mp_i])
      continue;
    double d = 0.0;
    if (opts.panelMode && opts.idw > 0) {
      d += opts.idw * (M.panel(i) != Mp.panel(Mp_i));
    } else if (opts.panelMode && !opts.idWeights.empty()) {
      d += opts.idWeights.at(std::pair<int, int>(M.panel(i), Mp.panel(Mp_i)));
    }
    for (int j = 0; j < M.E_actual; j++) {
      double a = M(i, j), b = Mp(Mp_i, j), dij;
      if (hasMissing && (a == MISSING_D || b == MISSING_D)) {
        if (opts.missingdistance == 0) {
          d = MISSING_D;
          break;
        }
        dij = opts.missingdistance;
      } else {
        dij = a - b;
      }
      if (l1)
        d += std::abs(dij) / M.E_actual;
      else
        d = mac(dij, dij, d, g_sum_mode & 8);
    }
    if (d != 0 && d != MISSING_D) {
      out.dists.push_back(l1 ? d : std::sqrt(d));
      out.inds.push_back(i);
    }
  }
  return out;
}

// ------------------------------------------------ Wasserstein distance
// src/distances.cpp:270-527.  The cost matrix is restated step by step; the
// transport cost that the reference takes from EMD_wrap
// (src/vendor/EMD_wrapper.h:34-117, POT's network simplex, vendored) is
// computed here by an independent exact method: an optimal assignment by the
// Hungarian method (Kuhn-Munkres with potentials, O(N^3)), directly for equal
// lengths n (flows 1/n) and, for unequal lengths, on the problem with every
// source repeated len_j times and every sink len_i times (flows in units of
// 1/(len_i len_j)).  EMD_wrap sums flow * cost over the arcs from the last
// (i = n1-1, j = n2-1) to the first; the same sum is formed here.  For equal
// lengths and a unique optimal plan that reproduces EMD_wrap's bits (its
// network simplex carries the flows 1/n exactly).  Where several plans are
// optimal the two solvers may return different ones, whose sums differ in
// the last bits; for unequal lengths EMD_wrap's flows carry roundings of
// their own, a few ulps from the exact fractions.

// Minimum-cost perfect assignment of an N x N cost matrix (row-major);
// returns the column of each row.
std::vector<int> hungarian(const std::vector<double>& cost, int N)
{
  const long double INF = std::numeric_limits<long double>::infinity();
  std::vector<long double> u(N + 1, 0), v(N + 1, 0), minv(N + 1);
  std::vector<int> p(N + 1, 0), way(N + 1, 0);
  std::vector<char> used(N + 1);
  for (int i = 1; i <= N; i++) {
    p[0] = i;
    int j0 = 0;
    std::fill(minv.begin(), minv.end(), INF);
    std::fill(used.begin(), used.end(), 0);
    do {
      used[j0] = 1;
      const int i0 = p[j0];
      long double delta = INF;
      int j1 = 0;
      for (int j = 1; j <= N; j++)
        if (!used[j]) {
          const long double cur = (long double)cost[(size_t)(i0 - 1) * N + (j - 1)] - u[i0] - v[j];
          if (cur < minv[j]) {
            minv[j] = cur;
            way[j] = j0;
          }
          if (minv[j] < delta) {
            delta = minv[j];
            j1 = j;
          }
        }
      for (int j = 0; j <= N; j++)
        if (used[j]) {
          u[p[j]] += delta;
          v[j] -= delta;
        } else {
          minv[j] -= delta;
        }
      j0 = j1;
    } while (p[j0] != 0);
    do {
      const int j1 = way[j0];
      p[j0] = p[j1];
      j0 = j1;
    } while (j0);
  }
  std::vector<int> col(N);
  for (int j = 1; j <= N; j++)
    col[p[j] - 1] = j - 1;
  return col;
}

// Transport cost of the n1 x n2 row-major cost matrix D with masses 1/n1
// and 1/n2 (src/distances.cpp:455-470 calling EMD_wrap).
double emd_uniform(const double* D, int n1, int n2)
{
  std::vector<long long> f((size_t)n1 * n2, 0);
  long long L;
  if (n1 == n2) {
    std::vector<double> c(D, D + (size_t)n1 * n2);
    const std::vector<int> col = hungarian(c, n1);
    for (int i = 0; i < n1; i++)
      f[(size_t)i * n2 + col[i]] = 1;
    L = n1;
  } else {
    const int N = n1 * n2;  // source i repeated n2 times, sink j n1 times
    std::vector<double> c((size_t)N * N);
    for (int a = 0; a < N; a++)
      for (int b = 0; b < N; b++)
        c[(size_t)a * N + b] = D[(size_t)(a / n2) * n2 + (b / n1)];
    const std::vector<int> col = hungarian(c, N);
    for (int a = 0; a < N; a++)
      f[(size_t)(a / n2) * n2 + col[a] / n1] += 1;
    L = N;
  }
  double cost = 0;
  for (long long a = (long long)n1 * n2 - 1; a >= 0; a--) {
    const double flow = (double)f[a] / (double)L;
    cost += flow * D[a];
  }
  return cost;
}

// src/distances.cpp:296-411: the cost matrix between library point i of M
// and prediction point j of Mp.  The reference maps each point's leading
// rows * E values as a column-major rows x E matrix (rows = 1 + [dt] +
// lagged extras), the unlagged extras after it.
std::vector<double> wasserstein_cost_matrix(const Manifold& M, const Manifold& Mp, int i, int j, const Options& opts,
                                            int& len_i, int& len_j)
{
  const Generator& g = *M.gen;
  const int E = M.E_x;
  const bool skipMissing = opts.missingdistance == 0;
  const int rows = 1 + (g.E_dt(E) > 0 ? 1 : 0) + g.num_extras_lagged;
  const double* x = &M.flat[(size_t)i * M.E_actual];
  const double* y = &Mp.flat[(size_t)j * Mp.E_actual];
  auto at = [&](const double* v, int r, int c) { return v[(size_t)c * rows + r]; };
  std::vector<bool> xm(E, false), ym(E, false);
  for (int c = 0; c < E; c++)
    for (int r = 0; r < rows; r++) {
      if (at(x, r, c) == MISSING_D)
        xm[c] = true;
      if (at(y, r, c) == MISSING_D)
        ym[c] = true;
    }
  if (skipMissing) {
    len_i = E - (int)std::count(xm.begin(), xm.end(), true);
    len_j = E - (int)std::count(ym.begin(), ym.end(), true);
  } else {
    len_i = E;
    len_j = E;
  }
  double gamma = 1.0;
  if (g.E_dt(E) > 0) {
    double minData = std::numeric_limits<double>::max();
    double maxData = std::numeric_limits<double>::min();
    double maxTime = 0.0;
    for (int t = 0; t < E; t++) {
      if (at(x, 0, t) != MISSING_D) {
        if (at(x, 0, t) < minData)
          minData = at(x, 0, t);
        if (at(x, 0, t) > maxData)
          maxData = at(x, 0, t);
      }
      if (at(x, 1, t) != MISSING_D && at(x, 1, t) > maxTime)
        maxTime = at(x, 1, t);
    }
    const double epsilon = 1e-6;
    gamma = opts.aspectRatio * (maxData - minData + epsilon) / (maxTime + epsilon);
  }
  double unlaggedDist = 0.0;
  const int numUnlagged = g.num_extras - g.num_extras_lagged;
  for (int e = 0; e < numUnlagged; e++) {
    const double xe = x[(size_t)rows * E + e], ye = y[(size_t)rows * E + e];
    if (xe == MISSING_D || ye == MISSING_D)
      unlaggedDist += opts.missingdistance;
    else
      unlaggedDist += std::abs(xe - ye);
  }
  if (opts.panelMode && opts.idw > 0) {
    unlaggedDist += opts.idw * (M.panel(i) != Mp.panel(j));
  } else if (opts.panelMode && !opts.idWeights.empty()) {
    unlaggedDist += opts.idWeights.at(std::pair<int, int>(M.panel(i), Mp.panel(j)));
  }
  std::vector<double> C((size_t)std::max(0, len_i * len_j), unlaggedDist);  // column-major len_i x len_j
  for (int k = 0; k < rows; k++) {
    int n = 0;
    for (int nn = 0; nn < E; nn++) {
      if (skipMissing && xm[nn])
        continue;
      int m = 0;
      for (int mm = 0; mm < E; mm++) {
        if (skipMissing && ym[mm])
          continue;
        double dist;
        if (xm[nn] || ym[mm])
          dist = opts.missingdistance;
        else
          dist = std::abs(at(x, k, nn) - at(y, k, mm));
        if (g.E_dt(E) > 0 && k == 1)
          dist *= gamma;
        C[(size_t)m * len_i + n] += dist;
        m++;
      }
      n++;
    }
  }
  return C;
}

// src/distances.cpp:488-527
DistanceIndexPairs wasserstein_distances(int Mp_i, const Options& opts, const Manifold& M, const Manifold& Mp)
{
  DistanceIndexPairs out;
  const bool skipOtherPanels = opts.panelMode && (opts.idw < 0);
  for (int i = 0; i < M.numPoints; i++) {
    if (skipOtherPanels && M.panel(i) != Mp.panel(Mp_i))
      continue;
    int len_i, len_j;
    std::vector<double> C = wasserstein_cost_matrix(M, Mp, i, Mp_i, opts, len_i, len_j);
    if (len_i > 0 && len_j > 0) {
      // EMD_wrap reads the buffer as a row-major len_i x len_j matrix
      const double d = emd_uniform(C.data(), len_i, len_j);
      if (d != 0 && std::isnormal(d)) {
        out.dists.push_back(d);
        out.inds.push_back(i);
      }
    }
  }
  return out;
}

// src/edm.cpp:652-681: first k in (distance, position) order.
DistanceIndexPairs k_nearest_neighbours(const DistanceIndexPairs& pn, int k)
{
  std::vector<int> idx(pn.inds.size());
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return pn.dists[a] < pn.dists[b]; });
  DistanceIndexPairs out;
  for (int i = 0; i < k; i++) {
    out.inds.push_back(pn.inds[idx[i]]);
    out.dists.push_back(pn.dists[idx[i]]);
  }
  return out;
}

// -------------------------------------------- Jacobi SVD (Eigen restatement)
// Restates Eigen 3.3/3.4 JacobiSVD<MatrixXd>::compute for a square matrix
// (no QR preconditioner applies) followed by SVDBase::solve with the default
// threshold diagSize*epsilon.  Eigen is MPL2; only its published algorithm
// is followed here.
struct Rot
{
  double c, s;
};

// rows p,q <- J * [row p; row q] with J = [c s; -s c]
void rot_rows(std::vector<double>& A, int n, int p, int q, Rot j)
{
  for (int i = 0; i < n; i++) {
    double x = A[p * n + i], y = A[q * n + i];
    A[p * n + i] = j.c * x + j.s * y;
    A[q * n + i] = -j.s * x + j.c * y;
  }
}
// cols p,q <- [col p, col q] * J
void rot_cols(std::vector<double>& A, int n, int p, int q, Rot j)
{
  // applyOnTheRight uses the transposed rotation on the column pair.
  Rot t{ j.c, -j.s };
  for (int i = 0; i < n; i++) {
    double x = A[i * n + p], y = A[i * n + q];
    A[i * n + p] = t.c * x + t.s * y;
    A[i * n + q] = -t.s * x + t.c * y;
  }
}

bool make_jacobi(double x, double y, double z, Rot& r)
{
  const double tiny = std::numeric_limits<double>::min();
  double deno = 2 * std::abs(y);
  if (deno < tiny) {
    r.c = 1;
    r.s = 0;
    return false;
  }
  double tau = (x - z) / deno;
  double w = std::sqrt(tau * tau + 1);
  double t = tau > 0 ? 1 / (tau + w) : 1 / (tau - w);
  double sign_t = t > 0 ? 1 : -1;
  double n = 1 / std::sqrt(t * t + 1);
  r.s = -sign_t * (y / std::abs(y)) * std::abs(t) * n;
  r.c = n;
  return true;
}

void real_2x2_jacobi_svd(const std::vector<double>& W, int n, int p, int q, Rot& jl, Rot& jr)
{
  const double tiny = std::numeric_limits<double>::min();
  double m00 = W[p * n + p], m01 = W[p * n + q], m10 = W[q * n + p], m11 = W[q * n + q];
  Rot r1;
  double t = m00 + m11;
  double d = m10 - m01;
  if (std::abs(d) < tiny) {
    r1.s = 0;
    r1.c = 1;
  } else {
    double u = t / d;
    double tmp = std::sqrt(1 + u * u);
    r1.s = 1 / tmp;
    r1.c = u / tmp;
  }
  // m.applyOnTheLeft(0, 1, r1)
  double n00 = r1.c * m00 + r1.s * m10, n01 = r1.c * m01 + r1.s * m11;
  double n11 = -r1.s * m01 + r1.c * m11;
  make_jacobi(n00, n01, n11, jr);
  // jl = r1 * jr.transpose()
  Rot jt{ jr.c, -jr.s };
  jl.c = r1.c * jt.c - r1.s * jt.s;
  jl.s = r1.c * jt.s + r1.s * jt.c;
}

// Solves (A) x = b for symmetric n x n A in the least-squares/pseudo-inverse
// sense exactly as JacobiSVD(A, ThinU|ThinV).solve(b).
std::vector<double> jacobi_svd_solve(const std::vector<double>& A, int n, const std::vector<double>& b)
{
  const double tiny = std::numeric_limits<double>::min();
  const double eps = std::numeric_limits<double>::epsilon();
  const double precision = 2 * eps;
  double scale = 0;
  for (double a : A)
    scale = std::max(scale, std::abs(a));
  if (!std::isfinite(scale))
    return std::vector<double>(n, 0.0);  // Eigen flags InvalidInput; rank 0
  if (scale == 0)
    scale = 1;
  std::vector<double> W(n * n), U(n * n, 0.0), V(n * n, 0.0);
  for (int i = 0; i < n * n; i++)
    W[i] = A[i] / scale;
  for (int i = 0; i < n; i++)
    U[i * n + i] = V[i * n + i] = 1;
  double maxDiag = 0;
  for (int i = 0; i < n; i++)
    maxDiag = std::max(maxDiag, std::abs(W[i * n + i]));
  bool finished = false;
  while (!finished) {
    finished = true;
    for (int p = 1; p < n; p++) {
      for (int q = 0; q < p; q++) {
        double threshold = std::max(tiny, precision * maxDiag);
        if (std::abs(W[p * n + q]) > threshold || std::abs(W[q * n + p]) > threshold) {
          finished = false;
          Rot jl, jr;
          real_2x2_jacobi_svd(W, n, p, q, jl, jr);
          rot_rows(W, n, p, q, jl);
          rot_cols(U, n, p, q, Rot{ jl.c, -jl.s });  // U.applyOnTheRight(p,q,jl.transpose())
          rot_cols(W, n, p, q, jr);
          rot_cols(V, n, p, q, jr);
          maxDiag = std::max(maxDiag, std::max(std::abs(W[p * n + p]), std::abs(W[q * n + q])));
        }
      }
    }
  }
  std::vector<double> sv(n);
  for (int i = 0; i < n; i++) {
    double a = W[i * n + i];
    sv[i] = std::abs(a);
    if (a < 0)
      for (int r = 0; r < n; r++)
        U[r * n + i] = -U[r * n + i];
  }
  for (int i = 0; i < n; i++)
    sv[i] *= scale;
  int nonzero = n;
  for (int i = 0; i < n; i++) {
    int pos = i;
    double mx = sv[i];
    for (int j = i + 1; j < n; j++)
      if (sv[j] > mx) {
        mx = sv[j];
        pos = j;
      }
    if (mx == 0) {
      nonzero = i;
      break;
    }
    if (pos != i) {
      std::swap(sv[i], sv[pos]);
      for (int r = 0; r < n; r++) {
        std::swap(U[r * n + i], U[r * n + pos]);
        std::swap(V[r * n + i], V[r * n + pos]);
      }
    }
  }
  // rank(): threshold = diagSize * epsilon
  double thr = std::max(sv[0] * ((double)std::max(1, n) * eps), tiny);
  int i = nonzero - 1;
  while (i >= 0 && sv[i] < thr)
    --i;
  int rank = i + 1;
  std::vector<double> tmp(rank), x(n, 0.0);
  for (int c = 0; c < rank; c++) {
    double s = 0;
    for (int r = 0; r < n; r++)
      s += U[r * n + c] * b[r];
    tmp[c] = (1.0 / sv[c]) * s;  // diag(sv)^-1 * tmp
  }
  for (int r = 0; r < n; r++) {
    double s = 0;
    for (int c = 0; c < rank; c++)
      s += V[r * n + c] * tmp[c];
    x[r] = s;
  }
  return x;
}

// ------------------------------------------------------------- edm.cpp
struct TaskOut
{
  int numThetas = 0, numPredictions = 0, numCoeffCols = 0;
  std::vector<double> predictions, coeffs;
  std::vector<int> rc, kUsed;
  std::vector<DistanceIndexPairs> nn;
};

// src/edm.cpp:707-735
void simplex_prediction(int Mp_i, int t, const Options& opts, const Manifold& M, const std::vector<double>& dists,
                        const std::vector<int>& inds, TaskOut& o)
{
  int k = (int)inds.size();
  double minDist = *std::min_element(dists.begin(), dists.end());
  std::vector<double> w(k);
  double sumw = 0.0;
  const double theta = opts.thetas[t];
  for (int j = 0; j < k; j++) {
    w[j] = edm_exp(-theta * (dists[j] / minDist));
    sumw = sumw + w[j];
  }
  double r = 0.0;
  for (int j = 0; j < k; j++)
    r = mac(M.targets[inds[j]], w[j] / sumw, r, g_sum_mode & 8);
  o.predictions[(size_t)t * o.numPredictions + Mp_i] = r;
  o.rc[(size_t)t * o.numPredictions + Mp_i] = SUCCESS;
}

// src/edm.cpp:737-814
void smap_prediction(int Mp_i, int t, const Options& opts, const Manifold& M, const Manifold& Mp,
                     const std::vector<double>& dists, const std::vector<int>& inds, TaskOut& o)
{
  int k = (int)inds.size();
  int Ea = M.E_actual, n = Ea + 1;
  const int P = (g_sum_mode & 1) ? 2 : ((g_sum_mode & 2) ? 4 : 0);
  const bool fused = (g_sum_mode & 4) != 0;
  double mean = 0;
  if (P) {
    mean = packet_reduce(dists.data(), nullptr, 0, nullptr, 0, k, P, false);
  } else {
    for (double d : dists)
      mean += d;
  }
  mean /= (double)k;
  std::vector<double> w(k);
  for (int i = 0; i < k; i++)
    w[i] = edm_exp(-opts.thetas[t] * (dists[i] / mean));
  std::vector<double> X((size_t)k * n), y(k);
  for (int i = 0; i < k; i++) {
    X[(size_t)i * n] = w[i];
    for (int j = 1; j < n; j++)
      X[(size_t)i * n + j] = w[i] * M(inds[i], j - 1);
    y[i] = w[i] * M.targets[inds[i]];
  }
  std::vector<double> XtX((size_t)n * n), Xty(n);
  for (int a = 0; a < n; a++) {
    for (int b = 0; b < n; b++) {
      double s = 0;
      if (P && k + n + k < 20)
        s = packet_reduce(nullptr, &X[a], n, &X[b], n, k, P, fused);
      else if (P)
        s = blocked_dot(&X[a], n, &X[b], n, k, fused);
      else
        for (int i = 0; i < k; i++)
          s += X[(size_t)i * n + a] * X[(size_t)i * n + b];
      XtX[(size_t)a * n + b] = s;
    }
    double s = 0;
    if (P)
      s = gemv_dot(&X[a], n, y.data(), 1, k, P, fused);
    else
      for (int i = 0; i < k; i++)
        s += X[(size_t)i * n + a] * y[i];
    Xty[a] = s;
  }
  std::vector<double> ics = jacobi_svd_solve(XtX, n, Xty);
  double r = ics[0];
  for (int j = 0; j < Ea; j++) {
    double yj = Mp(Mp_i, j);
    if (yj != MISSING_D)
      r = mac(yj, ics[j + 1], r, g_sum_mode & 8);
  }
  if (opts.saveSMAPCoeffs && t == (int)opts.thetas.size() - 1) {
    for (int j = 0; j < n; j++)
      o.coeffs[(size_t)Mp_i * n + j] = std::abs(ics[j]) < 1.0e-11 ? MISSING_D : ics[j];
  }
  o.predictions[(size_t)t * o.numPredictions + Mp_i] = r;
  o.rc[(size_t)t * o.numPredictions + Mp_i] = SUCCESS;
}

// src/edm.cpp:565-639
void make_prediction(int Mp_i, const Options& opts, const Manifold& M, const Manifold& Mp, TaskOut& o, bool keepNN)
{
  // src/edm.cpp:578-582
  DistanceIndexPairs pn = opts.distance == Distance::Wasserstein ? wasserstein_distances(Mp_i, opts, M, Mp)
                                                                  : lp_distances(Mp_i, opts, M, Mp);
  int numValid = (int)pn.inds.size();
  int k = opts.k;
  if (k > numValid) {
    if (opts.forceCompute) {
      k = numValid;
    } else {
      o.rc[Mp_i] = INSUFFICIENT_UNIQUE;
      return;
    }
  }
  if (k == 0 || numValid == 0) {
    o.rc[Mp_i] = opts.forceCompute ? SUCCESS : INSUFFICIENT_UNIQUE;
    return;
  }
  DistanceIndexPairs knn;
  if (k < 0 || k == numValid)
    knn = pn;  // whole valid list, library order (src/edm.cpp:613-617)
  else
    knn = k_nearest_neighbours(pn, k);
  o.kUsed[Mp_i] = (int)knn.inds.size();
  if (keepNN)
    o.nn[Mp_i] = knn;
  if (opts.algorithm == Algorithm::Simplex) {
    for (int t = 0; t < (int)opts.thetas.size(); t++)
      simplex_prediction(Mp_i, t, opts, M, knn.dists, knn.inds, o);
  } else {
    for (int t = 0; t < (int)opts.thetas.size(); t++)
      smap_prediction(Mp_i, t, opts, M, Mp, knn.dists, knn.inds, o);
  }
}

struct PredStats
{
  int library, E;
  double theta, mae, rho;
};

struct PredictionResult
{
  int rc = 0;
  int numThetas = 0, numPredictions = 0, numCoeffCols = 0;
  std::vector<double> predictions, coeffs;
  bool hasPredictions = false, hasCoeffs = false;
  std::vector<PredStats> stats;
  std::vector<bool> predictionRows;
  int kMin = MISSING_I, kMax = MISSING_I;
  bool copredict = false;
};

void run_predictions(const Options& opts, const Manifold& M, const Manifold& Mp, TaskOut& o, bool keepNN)
{
  int np = Mp.numPoints;
  int nt = std::max(1, opts.nthreads);
  if (nt == 1 || np < 64) {
    for (int i = 0; i < np; i++)
      make_prediction(i, opts, M, Mp, o, keepNN);
    return;
  }
  // Per-prediction parallelism like the reference's workerPool
  // (src/edm.cpp:367-392); results are independent of the thread count.
  std::vector<std::thread> th;
  std::atomic<int> next{ 0 };
  for (int w = 0; w < nt; w++) {
    th.emplace_back([&] {
      for (;;) {
        int s = next.fetch_add(16);
        if (s >= np)
          break;
        int e = std::min(np, s + 16);
        for (int i = s; i < e; i++)
          make_prediction(i, opts, M, Mp, o, keepNN);
      }
    });
  }
  for (auto& t : th)
    t.join();
}

// src/edm.cpp:285-548
PredictionResult edm_task(const Generator& gen, Options opts, int E, const std::vector<bool>& libraryRows,
                          const std::vector<bool>& predictionRows, TaskOut* keep = nullptr)
{
  Manifold M(gen, E, libraryRows, false, opts.copredict);
  Manifold Mp(gen, E, predictionRows, true, opts.copredict);
  TaskOut o;
  o.numThetas = (int)opts.thetas.size();
  o.numPredictions = Mp.numPoints;
  o.numCoeffCols = M.E_actual + 1;
  o.predictions.assign((size_t)o.numThetas * o.numPredictions, MISSING_D);
  o.coeffs.assign((size_t)o.numPredictions * o.numCoeffCols, MISSING_D);
  o.rc.assign((size_t)o.numThetas * o.numPredictions, UNKNOWN_ERROR);
  o.kUsed.assign(o.numPredictions, MISSING_I);
  if (keep)
    o.nn.resize(o.numPredictions);
  run_predictions(opts, M, Mp, o, keep != nullptr);

  PredictionResult pred;
  for (int t = 0; t < o.numThetas; t++) {
    PredStats s;
    s.library = opts.library;
    s.E = M.E_actual;
    s.theta = opts.thetas[t];
    std::vector<double> y1, y2;
    for (int i = 0; i < Mp.numPoints; i++) {
      double pr = o.predictions[(size_t)t * o.numPredictions + i];
      if (Mp.targets[i] != MISSING_D && pr != MISSING_D) {
        y1.push_back(Mp.targets[i]);
        y2.push_back(pr);
      }
    }
    if (!y1.empty()) {
      s.mae = mean_absolute_error(y1, y2);
      s.rho = correlation(y1, y2);
    } else {
      s.mae = MISSING_D;
      s.rho = MISSING_D;
    }
    pred.stats.push_back(s);
  }
  // *max_element over an empty range is undefined in the reference; no
  // predictions is reported as SUCCESS here.
  pred.rc = o.rc.empty() ? SUCCESS : *std::max_element(o.rc.begin(), o.rc.end());
  if (opts.savePrediction) {
    pred.hasPredictions = true;
    pred.predictions.resize(o.numPredictions);
    for (int i = 0; i < o.numPredictions; i++)
      pred.predictions[i] = o.predictions[(size_t)(o.numThetas - 1) * o.numPredictions + i];
  }
  if (opts.saveSMAPCoeffs) {
    pred.hasCoeffs = true;
    pred.coeffs = o.coeffs;
  }
  pred.predictionRows = predictionRows;
  std::vector<int> ku;
  for (int v : o.kUsed)
    if (v != MISSING_I)
      ku.push_back(v);
  if (!ku.empty()) {
    pred.kMin = *std::min_element(ku.begin(), ku.end());
    pred.kMax = *std::max_element(ku.begin(), ku.end());
  }
  pred.copredict = opts.copredict;
  pred.numThetas = o.numThetas;
  pred.numPredictions = o.numPredictions;
  pred.numCoeffCols = o.numCoeffCols;
  if (keep)
    *keep = std::move(o);
  return pred;
}

// ------------------------------------------- library_prediction_split.h
struct Splitter
{
  bool explore, full, shuffle;
  int crossfold, numObsUsable;
  std::vector<bool> usable, lib, pred;
  std::vector<int> crossfoldGroup;
  MT64 rng;

  // src/library_prediction_split.h:28-48 (the R caller passes no Stata state)
  Splitter(bool e, bool f, bool s, int cf, const std::vector<bool>& u, int seed)
    : explore(e), full(f), shuffle(s), crossfold(cf), usable(u)
  {
    rng.init((uint64_t)(unsigned long long)seed);
    numObsUsable = (int)std::count(u.begin(), u.end(), true);
    if (crossfold > 0)
      setup_crossfold_groups();
  }

  // src/library_prediction_split.h:72-101
  void setup_crossfold_groups()
  {
    std::vector<int> uRank;
    if (shuffle) {
      std::vector<double> u;
      for (int i = 0; i < numObsUsable; i++)
        u.push_back(rng.real2());
      uRank = rank_of(u);
    }
    int sizeOfEachFold = (int)std::round(((float)numObsUsable) / crossfold);
    int obsNum = 0;
    crossfoldGroup.assign(usable.size(), 0);
    for (size_t i = 0; i < usable.size(); i++) {
      if (usable[i]) {
        crossfoldGroup[i] = shuffle ? uRank[obsNum] % crossfold : obsNum / sizeOfEachFold;
        obsNum++;
      } else {
        crossfoldGroup[i] = -1;
      }
    }
  }

  // src/library_prediction_split.h:104-120
  int next_library_size(int iter) const
  {
    if (crossfold > 0) {
      int n = 0;
      for (int o = 0; o < numObsUsable; o++)
        if ((o + 1) % crossfold != (iter - 1))
          n++;
      return n;
    }
    if (full)
      return numObsUsable;
    return numObsUsable / 2;
  }

  // src/library_prediction_split.h:145-157
  void update(int library, int iter)
  {
    if (explore && full) {
      lib = usable;
      pred = usable;
    } else if (explore && crossfold > 0) {
      lib.assign(usable.size(), false);
      pred.assign(usable.size(), false);
      for (size_t i = 0; i < usable.size(); i++)
        if (usable[i]) {
          bool inPred = crossfoldGroup[i] == (iter - 1);
          lib[i] = !inPred;
          pred[i] = inPred;
        }
    } else if (explore) {
      half_split();
    } else {
      fixed_size_library(library);
    }
  }

  // src/library_prediction_split.h:180-229
  void half_split()
  {
    lib.assign(usable.size(), false);
    pred.assign(usable.size(), false);
    if (shuffle) {
      std::vector<double> u;
      for (int i = 0; i < numObsUsable; i++)
        u.push_back(rng.real2());
      double med = median(u);
      int o = 0;
      for (size_t i = 0; i < usable.size(); i++)
        if (usable[i]) {
          bool l = u[o] < med;
          lib[i] = l;
          pred[i] = !l;
          o++;
        }
    } else {
      int librarySize = numObsUsable / 2;
      int o = 0;
      for (size_t i = 0; i < usable.size(); i++)
        if (usable[i]) {
          bool l = o < librarySize;
          lib[i] = l;
          pred[i] = !l;
          o++;
        }
    }
  }

  // src/library_prediction_split.h:231-286
  void fixed_size_library(int library)
  {
    lib.assign(usable.size(), false);
    pred = usable;
    if (shuffle) {
      std::vector<double> u;
      for (int i = 0; i < numObsUsable; i++)
        u.push_back(rng.real2());
      double cutoff = 1.0;
      if (library < (int)u.size()) {
        std::vector<double> c(u);
        std::nth_element(c.begin(), c.begin() + library, c.end());
        cutoff = c[library];
      }
      int o = 0;
      for (size_t i = 0; i < usable.size(); i++)
        if (usable[i]) {
          lib[i] = u[o] < cutoff;
          o++;
        }
    } else {
      int o = 0;
      for (size_t i = 0; i < usable.size(); i++)
        if (usable[i]) {
          lib[i] = o < library;
          o++;
        }
    }
  }
};

// ------------------------------------------------------------ run_command
std::vector<double> clean(const double* v, int n)
{
  // src/r.cpp:64-71: every non-normal value (NaN, Inf, 0, subnormal) is MISSING
  std::vector<double> out(v, v + n);
  for (double& a : out)
    if (!std::isnormal(a))
      a = MISSING_D;
  return out;
}

struct Prepared
{
  std::unique_ptr<Generator> gen;
  Options opts;
  bool explore = true;
  std::vector<int> Es, libraries;
};

// src/r.cpp:119-246 (inputs, options and the generator)
Prepared prepare(const oracle_args* a)
{
  Prepared P;
  Options& opts = P.opts;
  opts.nthreads = a->num_threads;
  opts.copredict = false;
  opts.forceCompute = true;
  opts.saveSMAPCoeffs = a->save_smap_coeffs;
  opts.missingdistance = a->missing_distance;
  opts.lowMemoryMode = a->low_memory;
  opts.useOnlyPastToPredictFuture = a->predict_with_past;
  if (a->n_thetas > 0)
    opts.thetas.assign(a->thetas, a->thetas + a->n_thetas);
  else
    opts.thetas = { 1.0 };
  P.Es.assign(a->Es, a->Es + a->nE);
  if (a->libs)
    P.libraries.assign(a->libs, a->libs + a->n_libs);
  opts.algorithm = a->algorithm == 1 ? Algorithm::SMap : Algorithm::Simplex;
  opts.distance = Distance::Euclidean;

  int n = a->n;
  std::vector<double> t = clean(a->t, n), x = clean(a->x, n);
  for (int i = 0; i < n; i++)
    if (t[i] == MISSING_D)
      x[i] = MISSING_D;
  std::vector<double> xmap;
  if (a->y) {
    xmap = clean(a->y, n);
    P.explore = false;
  }
  opts.idw = a->panel_weight;
  std::vector<int> panelIDs;
  if (a->panel) {
    panelIDs.assign(a->panel, a->panel + n);
    opts.panelMode = true;
    if (a->panel_weights) {
      std::vector<int> uniq(panelIDs);
      uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
      int m = a->n_panel_weights;
      for (int i = 0; i < (int)uniq.size(); i++)
        for (int j = 0; j < (int)uniq.size(); j++)
          if (i < m && j < m)
            opts.idWeights[{ uniq[i], uniq[j] }] = (float)a->panel_weights[i + (size_t)j * m];
      opts.idw = 0;
    }
  }
  std::vector<double> co_x;
  if (a->co_x)
    co_x = clean(a->co_x, n);
  std::vector<std::vector<double>> ex;
  for (int e = 0; e < a->num_extras; e++)
    ex.push_back(clean(a->extras + (size_t)e * n, n));
  P.gen.reset(new Generator(t, x, a->tau, a->p, xmap, co_x, panelIDs, ex, 0, a->dt, a->reldt, a->allow_missing,
                            a->dt_weight));
  opts.hasMissing = a->allow_missing;
  if (a->allow_missing && opts.missingdistance == 0)
    opts.missingdistance = default_missing_distance(x);
  return P;
}

struct ResultStore
{
  oracle_result r;
  std::vector<int> sE, sL, cE, cL;
  std::vector<double> sT, sR, sM, cT, cR, cM, preds, copreds, coeffs;
};

double to_na(double v) { return v != MISSING_D ? v : NAN; }

// src/r.cpp:73-105 (rowMajor=false form, reading the buffer in column order)
std::vector<double> to_R_matrix(const std::vector<double>& v, int r, int c, const std::vector<bool>& filter)
{
  std::vector<double> m((size_t)r * c, NAN);
  size_t obs = 0;
  for (int j = 0; j < c; j++)
    for (int i = 0; i < r; i++) {
      if (!filter.empty() && !filter[i])
        continue;
      m[(size_t)j * r + i] = obs < v.size() ? to_na(v[obs]) : NAN;
      obs++;
    }
  return m;
}


struct TaskSpec
{
  int E, k, library;
  bool copredict, savePrediction, saveSMAPCoeffs;
  std::vector<bool> lib, pred;
};

// src/edm.cpp:90-212
std::vector<TaskSpec> configure(const oracle_args* a, const Prepared& P, const Generator& gen,
                                const std::vector<bool>& usable, const std::vector<int>& libraries)
{
  std::vector<TaskSpec> out;
  const bool explore = P.explore;
  const int maxE = P.Es.back();
  const bool copredictMode = !gen.co_x.empty();
  Splitter splitter(explore, a->full, a->shuffle, a->crossfold, usable, a->seed);
  int numLibraries = explore ? 1 : (int)libraries.size();
  int numIters = a->num_reps > a->crossfold ? a->num_reps : a->crossfold;
  std::vector<bool> cousable;
  if (copredictMode)
    cousable = gen.generate_usable(maxE, true);
  bool newSplit = true;
  int librarySize = 0;
  for (int iter = 1; iter <= numIters; iter++) {
    if (explore) {
      newSplit = true;
      librarySize = splitter.next_library_size(iter);
    }
    for (int i = 0; i < (int)P.Es.size(); i++) {
      int E = P.Es[i];
      for (int l = 0; l == 0 || l < (int)libraries.size(); l++) {
        if (!explore)
          newSplit = true;
        int library = explore ? librarySize : libraries[l];
        int kAdj;
        if (a->k > 0)
          kAdj = a->k;
        else if (a->k < 0)
          kAdj = -1;
        else {
          int isSMap = P.opts.algorithm == Algorithm::SMap;
          int defK = gen.E_actual(E) + 1 + isSMap;
          kAdj = defK < library ? defK : library;
        }
        bool lastConfig = (E == maxE) && (l + 1 == numLibraries);
        TaskSpec t;
        t.E = E;
        t.k = kAdj;
        t.library = library;
        t.copredict = false;
        if (explore)
          t.savePrediction = a->save_predictions && ((iter == a->num_reps) || (a->crossfold > 0)) && lastConfig;
        else
          t.savePrediction = a->save_predictions && (iter == a->num_reps) && lastConfig;
        t.saveSMAPCoeffs = a->save_smap_coeffs;
        if (newSplit) {
          splitter.update(library, iter);
          newSplit = false;
        }
        t.lib = splitter.lib;
        t.pred = splitter.pred;
        out.push_back(t);
        if (copredictMode) {
          TaskSpec c = t;
          c.copredict = true;
          if (explore)
            c.savePrediction =
              a->save_copredictions && ((iter == a->num_reps) || (a->crossfold > 0)) && lastConfig;
          else
            c.savePrediction = a->save_copredictions && (iter == a->num_reps) && lastConfig;
          c.saveSMAPCoeffs = false;
          c.pred = cousable;
          out.push_back(c);
        }
      }
    }
  }
  return out;
}

} // namespace

extern "C" {

void oracle_set_exp_mode(int mode)
{
  g_exp_mode = mode;
}

void oracle_set_sum_mode(int mode)
{
  g_sum_mode = mode & 15;
}

void oracle_set_pred_stride(int stride)
{
  g_pred_stride = stride > 1 ? stride : 1;
}

double oracle_exp(double x)
{
  return exp_rn(x);
}

void oracle_mt_real2(unsigned long long seed, long long count, double* out)
{
  MT64 m;
  m.init(seed);
  for (long long i = 0; i < count; i++)
    out[i] = m.real2();
}

int oracle_usable(const oracle_args* a, int maxE, int copredict, unsigned char* usable_out)
{
  Prepared P = prepare(a);
  auto u = P.gen->generate_usable(maxE, copredict != 0);
  for (int i = 0; i < a->n; i++)
    usable_out[i] = u[i];
  return 0;
}

oracle_result* oracle_run_command(const oracle_args* a)
{
  auto* S = new ResultStore();
  oracle_result& R = S->r;
  std::memset(&R, 0, sizeof(R));
  R.internal = S;
  R.kmin = R.kmax = MISSING_I;
  R.missing_distance = NAN;
  R.dt_weight = NAN;
  try {
    Prepared P = prepare(a);
    Generator& gen = *P.gen;
    Options opts = P.opts;
    int maxE = P.Es.back();
    std::vector<bool> usable = gen.generate_usable(maxE, false);
    int numUsable = (int)std::count(usable.begin(), usable.end(), true);
    if (numUsable == 0) {
      R.rc = UNKNOWN_ERROR;
      return &R;
    }
    std::vector<int> libraries = P.libraries;
    if (!P.explore && libraries.empty())
      libraries = { numUsable };

    // src/edm.cpp:90-212 configure_tasks, executed in order (run_tasks)
    std::vector<TaskSpec> specs = configure(a, P, gen, usable, libraries);
    std::vector<PredictionResult> results;
    for (TaskSpec& ts : specs) {
      if (g_pred_stride > 1) {
        int c = 0;
        for (size_t r = 0; r < ts.pred.size(); r++)
          if (ts.pred[r] && (c++ % g_pred_stride) != 0)
            ts.pred[r] = false;
      }
      Options o2 = opts;
      o2.k = ts.k;
      o2.library = ts.library;
      o2.copredict = ts.copredict;
      o2.savePrediction = ts.savePrediction;
      o2.saveSMAPCoeffs = ts.saveSMAPCoeffs;
      results.push_back(edm_task(gen, o2, ts.E, ts.lib, ts.pred));
    }

    // src/r.cpp:348-457 result marshalling
    int rc = 0, kMin = 0, kMax = 0;
    for (size_t f = 0; f < results.size(); f++) {
      const PredictionResult& pr = results[f];
      if (f == 0 || pr.kMin < kMin)
        kMin = pr.kMin;
      if (f == 0 || pr.kMax > kMax)
        kMax = pr.kMax;
      for (const auto& s : pr.stats) {
        if (!pr.copredict) {
          S->sE.push_back(s.E);
          S->sL.push_back(s.library);
          S->sT.push_back(to_na(s.theta));
          S->sR.push_back(to_na(s.rho));
          S->sM.push_back(to_na(s.mae));
        } else {
          S->cE.push_back(s.E);
          S->cL.push_back(s.library);
          S->cT.push_back(to_na(s.theta));
          S->cR.push_back(to_na(s.rho));
          S->cM.push_back(to_na(s.mae));
        }
      }
      if (pr.rc > rc)
        rc = pr.rc;
      int nrow = (int)pr.predictionRows.size();
      if (pr.hasPredictions) {
        // The reference reads numThetas columns from a buffer holding only
        // the last theta (src/r.cpp:394-399); only that first column is defined.
        auto m = to_R_matrix(pr.predictions, nrow, 1, pr.predictionRows);
        if (!pr.copredict) {
          S->preds = m;
          R.pred_rows = nrow;
          R.pred_cols = 1;
        } else {
          S->copreds = m;
          R.copred_rows = nrow;
          R.copred_cols = 1;
        }
      }
      if (pr.hasCoeffs) {
        S->coeffs = to_R_matrix(pr.coeffs, nrow, pr.numCoeffCols, pr.predictionRows);
        R.coeff_rows = nrow;
        R.coeff_cols = pr.numCoeffCols;
      }
    }
    R.rc = rc;
    R.kmin = kMin;
    R.kmax = kMax;
    R.n_stats = (int)S->sE.size();
    R.stat_E = S->sE.data();
    R.stat_library = S->sL.data();
    R.stat_theta = S->sT.data();
    R.stat_rho = S->sR.data();
    R.stat_mae = S->sM.data();
    R.n_costats = (int)S->cE.size();
    R.costat_E = S->cE.data();
    R.costat_library = S->cL.data();
    R.costat_theta = S->cT.data();
    R.costat_rho = S->cR.data();
    R.costat_mae = S->cM.data();
    if (a->save_predictions && !S->preds.empty())
      R.predictions = S->preds.data();
    if (a->save_copredictions && !S->copreds.empty())
      R.copredictions = S->copreds.data();
    if (a->save_smap_coeffs && !S->coeffs.empty())
      R.coeffs = S->coeffs.data();
    if (a->allow_missing)
      R.missing_distance = opts.missingdistance;
    if (a->dt || a->reldt)
      R.dt_weight = gen.dtWeight;
  } catch (...) {
    // src/r.cpp:459-467
    R.rc = UNKNOWN_ERROR;
  }
  return &R;
}

// Differentiable S-map reference gradient (no counterpart in the fastEDM
// reference): S-map over every library neighbour on coordinates z = w * m,
// MSE over prediction points, and dMSE/dtheta, dMSE/dw by the adjoint of the
// weighted normal equations (c = A^+ b, g = A^+ v, dyhat = dv.c +
// g.(db - dA c)), evaluated sequentially in FP64.  Distances follow
// src/distances.cpp:176-225 (zero distances excluded); weights
// src/edm.cpp:744-745; the solve is the JacobiSVD restatement above.
int oracle_smap_grad(const double* lib, const double* lib_t, int n_lib, const double* pred, const double* pred_t,
                     int n_pred, int E, double theta, const double* w, double* mse, double* dtheta, double* dw,
                     double* yhat_out)
{
  const int n = E + 1;
  double se = 0, gt = 0;
  std::vector<double> gw(E, 0.0), d(n_lib), a2(n_lib), dmu(E);
  for (int p = 0; p < n_pred; p++) {
    const double* y = pred + (size_t)p * E;
    std::vector<double> zp(E);
    for (int j = 0; j < E; j++)
      zp[j] = w[j] * y[j];
    double sum = 0;
    int cnt = 0;
    std::fill(dmu.begin(), dmu.end(), 0.0);
    for (int i = 0; i < n_lib; i++) {
      const double* m = lib + (size_t)i * E;
      double s = 0;
      for (int j = 0; j < E; j++) {
        const double df = w[j] * m[j] - zp[j];
        s += df * df;
      }
      d[i] = s != 0 ? std::sqrt(s) : -1.0;
      if (s != 0) {
        sum += d[i];
        cnt++;
        for (int j = 0; j < E; j++)
          dmu[j] += (w[j] * m[j] - zp[j]) * (m[j] - y[j]) / d[i];
      }
    }
    const double mu = sum / cnt;
    for (int j = 0; j < E; j++)
      dmu[j] /= cnt;
    std::vector<double> A((size_t)n * n, 0.0), b(n, 0.0), u(n);
    for (int i = 0; i < n_lib; i++) {
      if (d[i] < 0)
        continue;
      const double aw = edm_exp(-theta * (d[i] / mu));
      a2[i] = aw * aw;
      u[0] = 1;
      for (int j = 0; j < E; j++)
        u[j + 1] = w[j] * lib[(size_t)i * E + j];
      for (int r = 0; r < n; r++) {
        for (int c = 0; c < n; c++)
          A[(size_t)r * n + c] += a2[i] * u[r] * u[c];
        b[r] += a2[i] * u[r] * lib_t[i];
      }
    }
    std::vector<double> v(n);
    v[0] = 1;
    for (int j = 0; j < E; j++)
      v[j + 1] = zp[j];
    std::vector<double> c = jacobi_svd_solve(A, n, b), g = jacobi_svd_solve(A, n, v);
    double yh = c[0];
    for (int j = 0; j < E; j++)
      yh += zp[j] * c[j + 1];
    if (yhat_out)
      yhat_out[p] = yh;
    const double r = yh - pred_t[p];
    se += r * r;
    if (!dtheta)
      continue;
    double Q = 0;
    std::vector<double> R(E, 0.0), S(E, 0.0), T(E, 0.0);
    for (int i = 0; i < n_lib; i++) {
      if (d[i] < 0)
        continue;
      const double* m = lib + (size_t)i * E;
      u[0] = 1;
      for (int j = 0; j < E; j++)
        u[j + 1] = w[j] * m[j];
      double su = 0, uc = 0;
      for (int k = 0; k < n; k++) {
        su += g[k] * u[k];
        uc += u[k] * c[k];
      }
      const double ei = lib_t[i] - uc;
      Q += a2[i] * su * ei * d[i];
      for (int j = 0; j < E; j++) {
        R[j] += a2[i] * su * ei * ((w[j] * m[j] - zp[j]) * (m[j] - y[j]) / d[i]);
        S[j] += a2[i] * ei * m[j];
        T[j] += a2[i] * su * m[j];
      }
    }
    gt += 2 * r * (-(2 / mu) * Q);
    for (int j = 0; j < E; j++)
      gw[j] += 2 * r *
               (y[j] * c[j + 1] - (2 * theta / mu) * R[j] + (2 * theta * dmu[j] / (mu * mu)) * Q + g[j + 1] * S[j] -
                c[j + 1] * T[j]);
  }
  *mse = se / n_pred;
  if (dtheta) {
    *dtheta = gt / n_pred;
    for (int j = 0; j < E; j++)
      dw[j] = gw[j] / n_pred;
  }
  return 0;
}

int oracle_plan(const oracle_args* a, int max_tasks, int* n_tasks, int* task_E, int* task_k, int* task_library,
                int* task_copredict, unsigned char* lib_masks, unsigned char* pred_masks)
{
  try {
    Prepared P = prepare(a);
    std::vector<bool> usable = P.gen->generate_usable(P.Es.back(), false);
    int numUsable = (int)std::count(usable.begin(), usable.end(), true);
    std::vector<int> libraries = P.libraries;
    if (!P.explore && libraries.empty())
      libraries = { numUsable };
    auto specs = configure(a, P, *P.gen, usable, libraries);
    *n_tasks = (int)specs.size();
    for (int i = 0; i < (int)specs.size() && i < max_tasks; i++) {
      task_E[i] = specs[i].E;
      task_k[i] = specs[i].k;
      task_library[i] = specs[i].library;
      task_copredict[i] = specs[i].copredict;
      for (int r = 0; r < a->n; r++) {
        lib_masks[(size_t)i * a->n + r] = specs[i].lib[r];
        pred_masks[(size_t)i * a->n + r] = specs[i].pred[r];
      }
    }
    return 0;
  } catch (...) {
    return UNKNOWN_ERROR;
  }
}

void oracle_free_result(oracle_result* r)
{
  if (r)
    delete (ResultStore*)r->internal;
}

static Options task_options(const Prepared& P, const oracle_args* a, const oracle_task_io* io)
{
  Options opts = P.opts;
  opts.k = io->k;
  opts.copredict = io->copredict != 0;
  opts.forceCompute = io->force_compute != 0;
  opts.distance = io->distance == 0   ? Distance::MeanAbsoluteError
                  : io->distance == 2 ? Distance::Wasserstein
                                      : Distance::Euclidean;
  opts.aspectRatio = io->aspect_ratio;
  opts.saveSMAPCoeffs = true;
  opts.library = 0;
  return opts;
}

double oracle_emd_uniform(const double* D, int n1, int n2)
{
  return emd_uniform(D, n1, n2);
}

int oracle_task_sizes(const oracle_args* a, oracle_task_io* io)
{
  try {
    Prepared P = prepare(a);
    std::vector<bool> lib(a->n), pred(a->n);
    for (int i = 0; i < a->n; i++) {
      lib[i] = io->library_rows[i];
      pred[i] = io->prediction_rows[i];
    }
    Options opts = task_options(P, a, io);
    Manifold M(*P.gen, io->E, lib, false, opts.copredict);
    Manifold Mp(*P.gen, io->E, pred, true, opts.copredict);
    io->n_lib = M.numPoints;
    io->n_pred = Mp.numPoints;
    io->e_actual = M.E_actual;
    long long total = 0;
    TaskOut o;
    o.numThetas = (int)opts.thetas.size();
    o.numPredictions = Mp.numPoints;
    o.predictions.assign((size_t)o.numThetas * o.numPredictions, MISSING_D);
    o.coeffs.assign((size_t)o.numPredictions * (M.E_actual + 1), MISSING_D);
    o.rc.assign((size_t)o.numThetas * o.numPredictions, UNKNOWN_ERROR);
    o.kUsed.assign(o.numPredictions, MISSING_I);
    o.nn.resize(o.numPredictions);
    opts.algorithm = Algorithm::Simplex;  // sizes only need the neighbour lists
    run_predictions(opts, M, Mp, o, true);
    for (auto& d : o.nn)
      total += (long long)d.inds.size();
    io->total_nn = (int)total;
    io->missing_distance_used = opts.missingdistance;
    io->dt_weight_used = P.gen->dtWeight;
    return 0;
  } catch (...) {
    return UNKNOWN_ERROR;
  }
}

int oracle_task_run(const oracle_args* a, oracle_task_io* io)
{
  try {
    Prepared P = prepare(a);
    std::vector<bool> lib(a->n), pred(a->n);
    for (int i = 0; i < a->n; i++) {
      lib[i] = io->library_rows[i];
      pred[i] = io->prediction_rows[i];
    }
    Options opts = task_options(P, a, io);
    TaskOut o;
    PredictionResult pr = edm_task(*P.gen, opts, io->E, lib, pred, &o);
    Manifold M(*P.gen, io->E, lib, false, opts.copredict);
    Manifold Mp(*P.gen, io->E, pred, true, opts.copredict);
    int np = o.numPredictions, nt = o.numThetas, nc = o.numCoeffCols;
    std::copy(o.predictions.begin(), o.predictions.end(), io->predictions);
    std::copy(o.coeffs.begin(), o.coeffs.end(), io->coeffs);
    std::copy(o.rc.begin(), o.rc.end(), io->rc);
    std::copy(o.kUsed.begin(), o.kUsed.end(), io->kused);
    int pos = 0;
    for (int i = 0; i < np; i++) {
      io->nn_offsets[i] = pos;
      for (size_t j = 0; j < o.nn[i].inds.size(); j++) {
        io->nn_idx[pos] = o.nn[i].inds[j];
        io->nn_dist[pos] = o.nn[i].dists[j];
        pos++;
      }
    }
    io->nn_offsets[np] = pos;
    for (int t = 0; t < nt; t++) {
      io->stats_rho[t] = pr.stats[t].rho;
      io->stats_mae[t] = pr.stats[t].mae;
    }
    if (io->lib_point_rows)
      std::copy(M.rows.begin(), M.rows.end(), io->lib_point_rows);
    if (io->pred_point_rows)
      std::copy(Mp.rows.begin(), Mp.rows.end(), io->pred_point_rows);
    if (io->lib_manifold)
      std::copy(M.flat.begin(), M.flat.end(), io->lib_manifold);
    if (io->pred_manifold)
      std::copy(Mp.flat.begin(), Mp.flat.end(), io->pred_manifold);
    if (io->lib_targets)
      std::copy(M.targets.begin(), M.targets.end(), io->lib_targets);
    if (io->pred_targets)
      std::copy(Mp.targets.begin(), Mp.targets.end(), io->pred_targets);
    (void)nc;
    return pr.rc;
  } catch (...) {
    return UNKNOWN_ERROR;
  }
}

} // extern "C"
