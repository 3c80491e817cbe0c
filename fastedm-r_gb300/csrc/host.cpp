// Host side: series preparation, manifold rows, splitter, task list.
#include "host.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <numeric>
#include <thread>

namespace fedm {

namespace {

inline int add_wrap(int a, long long b)
{
  // Observation numbers can be MISSING_I (INT_MIN) when these offsets are
  // applied; the reference's builds wrap in two's complement.
  return (int)(uint32_t)((uint32_t)a + (uint32_t)(int64_t)b);
}

double gcd_tol(double a, double b)
{
  // src/manifold.cpp:7-18 (float GCD with a 1e-3 tolerance)
  for (;;) {
    if (a < b)
      std::swap(a, b);
    if (std::fabs(b) < 0.001)
      return a;
    double r = a - std::floor(a / b) * b;
    a = b;
    b = r;
  }
}

template<class F>
void parallel_rows(int n, int threads, F&& f)
{
  threads = std::max(1, std::min(threads, (n + 4095) / 4096));
  if (threads <= 1) {
    f(0, n);
    return;
  }
  std::vector<std::thread> th;
  int chunk = (n + threads - 1) / threads;
  for (int w = 0; w < threads; w++) {
    int b = w * chunk, e = std::min(n, b + chunk);
    if (b < e)
      th.emplace_back([&f, b, e] { f(b, e); });
  }
  for (auto& t : th)
    t.join();
}

} // namespace

std::vector<double> clean_vector(const double* v, int n)
{
  std::vector<double> out(v, v + n);
  for (double& a : out)
    if (!std::isnormal(a))
      a = MISSING_D;
  return out;
}

double sd_observed(const std::vector<double>& v)
{
  double s = 0;
  long long m = 0;
  for (double a : v)
    if (a != MISSING_D) {
      s += a;
      m++;
    }
  double mean = s / (double)m;
  double ss = 0;
  for (double a : v)
    if (a != MISSING_D) {
      double c = a - mean;
      ss += c * c;
    }
  return std::sqrt(ss / (double)(m - 1));
}

double Generator::calc_time_increment() const
{
  // src/manifold.cpp:20-48
  double unit = -1;
  for (int i = 1; i < n; i++) {
    double d = t[i] - t[i - 1];
    if (d <= 0 || t[i] == MISSING_D || t[i - 1] == MISSING_D)
      continue;
    unit = unit < 0 ? d : gcd_tol(d, unit);
  }
  return unit;
}

void Generator::setup_obs()
{
  // src/manifold.cpp:50-80
  obs.assign(n, MISSING_I);
  if (!(dt || reldt)) {
    double unit = calc_time_increment();
    double minT = n ? *std::min_element(t.begin(), t.end()) : 0;
    for (int i = 0; i < n; i++)
      if (t[i] != MISSING_D)
        obs[i] = (int)std::round((t[i] - minT) / unit);
  } else {
    int c = 0;
    for (int i = 0; i < n; i++)
      if (t[i] != MISSING_D && (allow_missing || x[i] != MISSING_D))
        obs[i] = c++;
  }
}

void Generator::init(double requested_dt_weight)
{
  num_extras = (int)extras.size();
  panel_mode = !panel.empty();
  xmap_mode = !xmap.empty();
  dt_weight = requested_dt_weight;
  bool want_dt = dt, want_reldt = reldt;
  if ((want_dt || want_reldt) && requested_dt_weight == 0.0) {
    // src/manifold.h:110-124: measure dt with plain dt mode, then rescale
    dt = true;
    reldt = false;
    setup_obs();
    std::vector<double> dts(n);
    for (int i = 0; i < n; i++)
      dts[i] = dt_of(i);
    double xsd = sd_observed(x), dtsd = sd_observed(dts);
    double w = (dtsd == 0.0) ? -1 : xsd / dtsd;
    if (w > 0) {
      dt = want_dt;
      reldt = want_reldt;
      dt_weight = w;
    } else {
      dt = reldt = false;
      dt_weight = 0;
    }
  }
  setup_obs();
}

bool Generator::find_obs(int target, int& k, int direction, int panel_id) const
{
  while (k >= 0 && k < n) {
    if (panel_mode) {
      if (panel[k] == MISSING_I) {
        k += direction;
        continue;
      }
      if (panel_id != panel[k])
        return false;
    }
    int o = obs[k];
    if (o == MISSING_I) {
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

int Generator::target_row(int i) const
{
  int ti = i;
  if (p != 0) {
    int pid = panel_mode ? panel[i] : -1;
    if (!find_obs(add_wrap(obs[ti], p), ti, p > 0 ? 1 : -1, pid))
      ti = -1;
  }
  return ti;
}

double Generator::dt_of(int i) const
{
  double now = t[i];
  if (now == MISSING_D)
    return MISSING_D;
  int k = i - 1;
  int pid = panel_mode ? panel[i] : -1;
  if (!find_obs(add_wrap(obs[i], -(long long)tau), k, -1, pid))
    return MISSING_D;
  double prev = t[k];
  if (!reldt)
    return now - prev;
  int ti = target_row(i);
  if (ti < 0)
    return MISSING_D;
  return t[ti] - prev;
}

void Generator::fill_row(int i, int E, bool use_co_x, double w, int target_i, double* out) const
{
  const bool with_dt = dt || reldt;
  const int Edt = E_dt(E);
  const int pid = panel_mode ? panel[i] : -1;
  const double tPred = (with_dt && target_i >= 0) ? t[target_i] : MISSING_D;
  const std::vector<double>& src = use_co_x ? co_x : x;
  int lagged = i, prev = i, k = i - 1;
  const int start = obs[i];
  for (int j = 0; j < E; j++) {
    bool found = (j == 0);
    if (!found && find_obs(add_wrap(start, -(long long)j * tau), k, -1, pid)) {
      found = true;
      lagged = k;
    }
    out[j] = found ? src[lagged] : MISSING_D;
    if (with_dt) {
      double v = MISSING_D;
      if (found) {
        double now = t[lagged];
        if (j == 0 || reldt) {
          if (now != MISSING_D && tPred != MISSING_D)
            v = w * (tPred - now);
        } else {
          double nxt = t[prev];
          if (nxt != MISSING_D && now != MISSING_D)
            v = w * (nxt - now);
        }
      }
      out[E + j] = v;
    }
    for (int e = 0; e < num_extras; e++) {
      double v = found ? extras[e][lagged] : MISSING_D;
      if (e < num_extras_lagged)
        out[E + Edt + e * E + j] = v;
      else if (j == 0)
        out[E + Edt + num_extras_lagged * E + (e - num_extras_lagged)] = v;
    }
    prev = lagged;
  }
}

std::vector<uint8_t> Generator::usable(int maxE, bool copredict, int threads) const
{
  std::vector<uint8_t> u(n, 0);
  const int Ea = E_actual(maxE);
  parallel_rows(n, threads, [&](int b, int e) {
    std::vector<double> row(std::max(Ea, 1));
    for (int i = b; i < e; i++) {
      if (t[i] == MISSING_D || (panel_mode && panel[i] == MISSING_I))
        continue;
      fill_row(i, maxE, copredict, 1.0, target_row(i), row.data());
      bool ok;
      if (allow_missing) {
        ok = false;
        for (int j = 0; j < Ea && !ok; j++)
          ok = row[j] != MISSING_D;
      } else {
        ok = true;
        for (int j = 0; j < Ea && ok; j++)
          ok = row[j] != MISSING_D;
      }
      u[i] = ok;
    }
  });
  return u;
}

RowTables build_row_tables(const Generator& g)
{
  RowTables r;
  r.target_row.resize(g.n);
  r.lib_target.resize(g.n);
  r.co_target.resize(g.n);
  r.lib_target_time.resize(g.n);
  r.point_time = g.t;
  const std::vector<double>& tv = g.xmap_mode ? g.xmap : g.x;
  for (int i = 0; i < g.n; i++) {
    int ti = g.target_row(i);
    r.target_row[i] = ti;
    r.lib_target[i] = ti >= 0 ? tv[ti] : MISSING_D;
    r.co_target[i] = (ti >= 0 && !g.co_x.empty()) ? g.co_x[ti] : MISSING_D;
    r.lib_target_time[i] = r.lib_target[i] != MISSING_D ? g.t[ti] : MISSING_D;
  }
  return r;
}

std::vector<double> build_manifold(const Generator& g, const RowTables& rt, int E, bool use_co_x, int threads)
{
  const int Ea = g.E_actual(E);
  std::vector<double> F((size_t)g.n * Ea);
  parallel_rows(g.n, threads, [&](int b, int e) {
    for (int i = b; i < e; i++)
      g.fill_row(i, E, use_co_x, g.dt_weight, rt.target_row[i], &F[(size_t)i * Ea]);
  });
  return F;
}

// ------------------------------------------------------------------ Mt64
void Mt64::init(uint64_t seed)
{
  s[0] = seed;
  for (int j = 1; j < 312; j++)
    s[j] = 6364136223846793005ULL * (s[j - 1] ^ (s[j - 1] >> 62)) + (uint64_t)j;
  left = 1;  // the first draw tempers the seed word itself
  next = 0;
}

void Mt64::refill()
{
  auto mix = [](uint64_t u, uint64_t v) {
    return (((u & 0xFFFFFFFF80000000ULL) | (v & 0x7FFFFFFFULL)) >> 1) ^ ((v & 1ULL) ? 0xB5026F5AA96619E9ULL : 0ULL);
  };
  for (int i = 0; i < 156; i++)
    s[i] = s[i + 156] ^ mix(s[i], s[i + 1]);
  for (int i = 156; i < 311; i++)
    s[i] = s[i - 156] ^ mix(s[i], s[i + 1]);
  s[311] = s[155] ^ mix(s[311], s[0]);
  left = 312;
  next = 0;
}

void Mt64::skip(long long count)
{
  while (count > 0) {
    if (left == 0)
      refill();
    const long long take = count < left ? count : left;
    left -= (int)take;
    next += (int)take;
    count -= take;
  }
}

uint64_t Mt64::next53()
{
  if (left == 0)
    refill();
  left--;
  uint64_t y = s[next++];
  y ^= (y >> 29) & 0x5555555555555555ULL;
  y ^= (y << 17) & 0x71D67FFFEDA60000ULL;
  y ^= (y << 37) & 0xFFF7EEE000000000ULL;
  y ^= (y >> 43);
  return y >> 11;
}

double Mt64::real2()
{
  return (double)next53() * (1.0 / 9007199254740992.0);
}

// -------------------------------------------------------------- Splitter
Splitter::Splitter(bool explore, bool full, bool shuffle, int crossfold, const std::vector<uint8_t>& usable,
                   int seed)
  : explore_(explore), full_(full), shuffle_(shuffle), crossfold_(crossfold), usable_(usable)
{
  rng_.init((uint64_t)(unsigned long long)(long long)seed);
  num_usable_ = (int)std::count(usable.begin(), usable.end(), (uint8_t)1);
  if (crossfold > 0) {
    // src/library_prediction_split.h:72-101
    std::vector<int> rank;
    if (shuffle) {
      draw();
      std::vector<int> order(num_usable_);
      std::iota(order.begin(), order.end(), 0);
      std::sort(order.begin(), order.end(), [&](int a, int b) {
        return u_[a] < u_[b] || (u_[a] == u_[b] && a < b);
      });
      rank.assign(num_usable_, 0);
      for (int r = 0; r < num_usable_; r++)
        rank[order[r]] = r + 1;
    }
    int fold_size = (int)std::round(((float)num_usable_) / crossfold);
    fold_.assign(usable.size(), -1);
    int o = 0;
    for (size_t i = 0; i < usable.size(); i++)
      if (usable[i]) {
        fold_[i] = shuffle ? rank[o] % crossfold : o / fold_size;
        o++;
      }
  }
}

void Splitter::draw()
{
  u_.resize(num_usable_);
  for (int i = 0; i < num_usable_; i++)
    u_[i] = rng_.real2();
}

int Splitter::next_library_size(int iter) const
{
  // src/library_prediction_split.h:104-120
  if (crossfold_ > 0) {
    int c = 0;
    for (int o = 0; o < num_usable_; o++)
      c += ((o + 1) % crossfold_ != (iter - 1));
    return c;
  }
  return full_ ? num_usable_ : num_usable_ / 2;
}

void Splitter::defer_fixed_size(Mt64& snapshot)
{
  // the state a shuffled fixed_size_library split starts from; the stream is
  // then advanced past its num_usable draws
  snapshot = rng_;
  rng_.skip(num_usable_);
}

void Splitter::update(int library, int iter)
{
  const size_t n = usable_.size();
  lib_.assign(n, 0);
  pred_.assign(n, 0);
  if (explore_ && full_) {
    lib_ = usable_;
    pred_ = usable_;
  } else if (explore_ && crossfold_ > 0) {
    for (size_t i = 0; i < n; i++)
      if (usable_[i]) {
        bool p = fold_[i] == iter - 1;
        lib_[i] = !p;
        pred_[i] = p;
      }
  } else if (explore_) {
    // src/library_prediction_split.h:180-229
    if (shuffle_) {
      draw();
      std::vector<double> c(u_);
      double med;
      if (c.size() % 2 == 0) {
        std::nth_element(c.begin(), c.begin() + c.size() / 2 - 1, c.end());
        double e1 = c[c.size() / 2 - 1];
        std::nth_element(c.begin(), c.begin() + c.size() / 2, c.end());
        med = (e1 + c[c.size() / 2]) / 2;
      } else {
        std::nth_element(c.begin(), c.begin() + c.size() / 2, c.end());
        med = c[c.size() / 2];
      }
      int o = 0;
      for (size_t i = 0; i < n; i++)
        if (usable_[i]) {
          bool l = u_[o++] < med;
          lib_[i] = l;
          pred_[i] = !l;
        }
    } else {
      int half = num_usable_ / 2, o = 0;
      for (size_t i = 0; i < n; i++)
        if (usable_[i]) {
          bool l = o++ < half;
          lib_[i] = l;
          pred_[i] = !l;
        }
    }
  } else {
    // src/library_prediction_split.h:231-286
    pred_ = usable_;
    if (shuffle_) {
      draw();
      double cutoff = 1.0;
      if (library < (int)u_.size()) {
        std::vector<double> c(u_);
        std::nth_element(c.begin(), c.begin() + library, c.end());
        cutoff = c[library];
      }
      int o = 0;
      for (size_t i = 0; i < n; i++)
        if (usable_[i])
          lib_[i] = u_[o++] < cutoff;
    } else {
      int o = 0;
      for (size_t i = 0; i < n; i++)
        if (usable_[i])
          lib_[i] = o++ < library;
    }
  }
}

// ------------------------------------------------------- configure_tasks
void select_library(Mt64& state, int library, const std::vector<int>& urows, const std::vector<double>& lib_target,
                    std::vector<int>& out, SplitScratch& sc)
{
  const int nu = (int)urows.size();
  sc.u.resize(nu);
  sc.hist.assign(4096, 0);
  for (int o = 0; o < nu; o++)
    sc.u[o] = state.next53();
  uint64_t cutoff = 1ULL << 53;  // getReal2() < 1.0 always
  if (library < nu) {
    // histogram of the top 12 bits, then nth_element inside the bucket that
    // holds the order statistic
    for (int o = 0; o < nu; o++)
      sc.hist[sc.u[o] >> 41]++;
    int b = 0, below = 0;
    while (below + sc.hist[b] <= library)
      below += sc.hist[b++];
    sc.c.clear();
    for (int o = 0; o < nu; o++)
      if ((int)(sc.u[o] >> 41) == b)
        sc.c.push_back(sc.u[o]);
    std::nth_element(sc.c.begin(), sc.c.begin() + (library - below), sc.c.end());
    cutoff = sc.c[library - below];
  }
  out.clear();
  out.reserve(std::min(library, nu));
  for (int o = 0; o < nu; o++)
    if (sc.u[o] < cutoff && lib_target[urows[o]] != MISSING_D)
      out.push_back(urows[o]);
}

SplitProducer::SplitProducer(TaskPlan& plan, const std::vector<double>& lib_target, int threads)
    : plan_(plan), target_(lib_target)
{
  const LazySplits& lz = plan.lazy;
  const int n = (int)lz.library.size();
  snaps_.resize(n);
  done_.assign(n, 0);
  split_of_mask_.assign(plan.masks.size(), -1);
  for (int j = 0; j < n; j++)
    split_of_mask_[lz.mask[j]] = j;
  threads_.emplace_back([this] { sequence(); });
  const int workers = std::max(1, std::min(threads - 2, n));
  for (int w = 0; w < workers; w++)
    threads_.emplace_back([this] { work(); });
}

SplitProducer::~SplitProducer()
{
  stop_ = true;
  {
    std::lock_guard<std::mutex> lk(mu_);
  }
  cv_snap_.notify_all();
  cv_done_.notify_all();
  for (auto& t : threads_)
    t.join();
}

void SplitProducer::sequence()
{
  const LazySplits& lz = plan_.lazy;
  Mt64 s = lz.start;
  const int n = (int)lz.library.size();
  for (int j = 0; j < n && !stop_; j++) {
    snaps_[j] = s;
    {
      std::lock_guard<std::mutex> lk(mu_);
      snapped_.store(j + 1);
    }
    cv_snap_.notify_all();
    s.skip(lz.num_usable);
  }
}

void SplitProducer::work()
{
  const LazySplits& lz = plan_.lazy;
  const int n = (int)lz.library.size();
  SplitScratch sc;
  std::vector<int> out;
  for (;;) {
    const int j = next_.fetch_add(1);
    if (j >= n)
      return;
    {
      std::unique_lock<std::mutex> lk(mu_);
      cv_snap_.wait(lk, [&] { return stop_.load() || snapped_.load() > j; });
      if (stop_)
        return;
    }
    Mt64 st = snaps_[j];
    select_library(st, lz.library[j], lz.urows, target_, out, sc);
    {
      std::lock_guard<std::mutex> lk(mu_);
      plan_.lib_lists[lz.mask[j]].swap(out);
      plan_.lists_ready[lz.mask[j]] = 1;
      done_[j] = 1;
    }
    cv_done_.notify_all();
  }
}

void SplitProducer::wait(int mask)
{
  const int j = mask < (int)split_of_mask_.size() ? split_of_mask_[mask] : -1;
  if (j < 0)
    return;
  std::unique_lock<std::mutex> lk(mu_);
  cv_done_.wait(lk, [&] { return stop_.load() || done_[j] != 0; });
}

TaskPlan configure_tasks(const Generator& g, const Options& opts, const std::vector<int>& Es,
                         const std::vector<int>& libraries, int k, int num_reps, int crossfold, bool explore,
                         bool full, bool shuffle, bool save_predictions, bool save_copredictions,
                         bool save_smap_coeffs, bool copredict_mode, const std::vector<uint8_t>& usable,
                         const std::vector<uint8_t>& cousable, int seed, const std::vector<double>* lib_target,
                         int threads, bool lazy_lists)
{
  TaskPlan plan;
  Splitter sp(explore, full, shuffle, crossfold, usable, seed);
  const int num_libraries = explore ? 1 : (int)libraries.size();
  const int num_iters = num_reps > crossfold ? num_reps : crossfold;
  const int maxE = Es.back();
  const bool deferred = lib_target != nullptr && !explore && shuffle;
  struct Deferred
  {
    Mt64 state;
    int library;
    int mask;
  };
  std::vector<Deferred> splits;
  int cousable_mask = -1;
  if (copredict_mode) {
    plan.masks.push_back(cousable);
    cousable_mask = 0;
  }
  int usable_mask = -1;
  bool new_split = true;
  int library_size = 0, lib_mask = -1, pred_mask = -1;
  for (int iter = 1; iter <= num_iters; iter++) {
    if (explore) {
      new_split = true;
      library_size = sp.next_library_size(iter);
    }
    for (int E : Es) {
      for (int l = 0; l == 0 || l < (int)libraries.size(); l++) {
        if (!explore)
          new_split = true;
        const int library = explore ? library_size : libraries[l];
        Task t;
        t.E = E;
        if (k > 0)
          t.k = k;
        else if (k < 0)
          t.k = -1;
        else {
          int def = g.E_actual(E) + 1 + (opts.algorithm == 1);
          t.k = def < library ? def : library;
        }
        const bool last = (E == maxE) && (l + 1 == num_libraries);
        const bool last_iter = explore ? ((iter == num_reps) || (crossfold > 0)) : (iter == num_reps);
        t.save_prediction = save_predictions && last_iter && last;
        t.save_coeffs = save_smap_coeffs;
        if (new_split) {
          new_split = false;
          if (deferred && lazy_lists) {
            // src/library_prediction_split.h:231-270 (shuffle branch), left
            // to a SplitProducer: only the first split's stream state is kept
            if (!plan.lazy.active) {
              plan.lazy.active = true;
              plan.lazy.start = sp.stream();
              plan.lazy.num_usable = sp.num_usable();
            }
            plan.masks.emplace_back();
            lib_mask = (int)plan.masks.size() - 1;
            plan.lazy.library.push_back(library);
            plan.lazy.mask.push_back(lib_mask);
            if (usable_mask < 0) {
              plan.masks.push_back(usable);
              usable_mask = (int)plan.masks.size() - 1;
            }
            pred_mask = usable_mask;
          } else if (deferred) {
            // src/library_prediction_split.h:231-270 (shuffle branch), run
            // later from a snapshot of the stream
            Deferred d;
            sp.defer_fixed_size(d.state);
            d.library = library;
            plan.masks.emplace_back();
            d.mask = lib_mask = (int)plan.masks.size() - 1;
            splits.push_back(d);
            if (usable_mask < 0) {
              plan.masks.push_back(usable);
              usable_mask = (int)plan.masks.size() - 1;
            }
            pred_mask = usable_mask;
          } else {
            sp.update(library, iter);
            plan.masks.push_back(sp.lib());
            lib_mask = (int)plan.masks.size() - 1;
            // cross-mapping prediction sets are all usable rows: reuse one mask
            if (!(!explore && pred_mask >= 0 && plan.masks[pred_mask] == sp.pred())) {
              plan.masks.push_back(sp.pred());
              pred_mask = (int)plan.masks.size() - 1;
            }
          }
        }
        t.library = library;
        t.lib_mask = lib_mask;
        t.pred_mask = pred_mask;
        t.copredict = false;
        plan.tasks.push_back(t);
        if (copredict_mode) {
          Task c = t;
          c.copredict = true;
          c.pred_mask = cousable_mask;
          c.save_prediction = save_copredictions && last_iter && last;
          c.save_coeffs = false;
          plan.tasks.push_back(c);
        }
      }
    }
  }
  if (plan.lazy.active) {
    plan.lib_lists.resize(plan.masks.size());
    plan.lists_ready.assign(plan.masks.size(), 0);
    for (int i = 0; i < (int)usable.size(); i++)
      if (usable[i])
        plan.lazy.urows.push_back(i);
  }
  if (!splits.empty()) {
    plan.lib_lists.resize(plan.masks.size());
    plan.lists_ready.assign(plan.masks.size(), 0);
    std::vector<int> urows;
    for (int i = 0; i < (int)usable.size(); i++)
      if (usable[i])
        urows.push_back(i);
    std::atomic<size_t> next{ 0 };
    auto worker = [&] {
      SplitScratch sc;
      for (;;) {
        const size_t j = next.fetch_add(1);
        if (j >= splits.size())
          break;
        Deferred& d = splits[j];
        select_library(d.state, d.library, urows, *lib_target, plan.lib_lists[d.mask], sc);
        plan.lists_ready[d.mask] = 1;
      }
    };
    const int nt = std::max(1, std::min<int>(threads, (int)splits.size()));
    std::vector<std::thread> pool;
    for (int w = 1; w < nt; w++)
      pool.emplace_back(worker);
    worker();
    for (auto& th : pool)
      th.join();
  }
  return plan;
}

} // namespace fedm
