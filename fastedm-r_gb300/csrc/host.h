// Host side of the GB300 EDM library: series preparation, lagged-manifold
// construction, the library/prediction splitter and task configuration.
// Semantics follow the reference (EDM-Developers/fastEDM-r) file:line cited
// at each declaration; the layout is batched: one manifold per embedding
// dimension E over all rows, tasks are row-index lists into it.
#pragma once

#include <atomic>
#include <climits>
#include <condition_variable>
#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/fastedm_gb300.h"

namespace fedm {

constexpr double MISSING_D = 1.0e+100;  // src/manifold.h:6
constexpr int MISSING_I = INT_MIN;      // src/manifold.h:8

enum Rc : int
{
  RC_SUCCESS = 0,
  RC_BREAK_HIT = 1,
  RC_INVALID_ALGORITHM = 400,
  RC_INSUFFICIENT_UNIQUE = 503,
  RC_NOT_IMPLEMENTED = 908,
  RC_UNKNOWN_ERROR = 8000
};

struct Error
{
  int rc;
  std::string what;
};

// The observed series after run_command's cleaning (src/r.cpp:171-246) and
// the ManifoldGenerator state (src/manifold.h:38-170).
class Generator
{
public:
  int n = 0;
  std::vector<double> t, x, xmap, co_x;
  std::vector<std::vector<double>> extras;
  std::vector<int> panel;
  int tau = 1, p = 0, num_extras = 0, num_extras_lagged = 0;
  bool dt = false, reldt = false, allow_missing = false, panel_mode = false, xmap_mode = false;
  std::vector<int> obs;
  double dt_weight = 0;

  // src/manifold.h:85-127 (default dt weight = sd(x)/sd(dt), manifold.h:53-67)
  void init(double requested_dt_weight);

  int E_dt(int E) const { return (dt || reldt) ? E : 0; }
  int E_extras(int E) const { return num_extras + num_extras_lagged * (E - 1); }
  int E_actual(int E) const { return E + E_dt(E) + E_extras(E); }

  // src/manifold.cpp:82-123
  bool find_obs(int target, int& k, int direction, int panel_id) const;
  // Row of the forecast target at horizon p, or -1 (src/manifold.cpp:281-303)
  int target_row(int i) const;
  // One manifold row (src/manifold.cpp:156-238)
  void fill_row(int i, int E, bool use_co_x, double w, int target_i, double* out) const;
  // src/manifold.cpp:314-360
  std::vector<uint8_t> usable(int maxE, bool copredict, int threads) const;
  // src/manifold.cpp:240-279
  double dt_of(int i) const;

private:
  void setup_obs();
  double calc_time_increment() const;
};

// Per-row quantities shared by every task (src/manifold.h:172-197).
struct RowTables
{
  std::vector<int> target_row;
  std::vector<double> lib_target;      // x (explore) or xmap (cross-map)
  std::vector<double> co_target;       // co_x at the target row
  std::vector<double> lib_target_time; // t at the target row, MISSING if target missing
  std::vector<double> point_time;      // t
};

RowTables build_row_tables(const Generator& g);

// Manifold of every row for embedding dimension E, row-major [n x E_actual].
std::vector<double> build_manifold(const Generator& g, const RowTables& rt, int E, bool use_co_x, int threads);

// MT19937-64 in the reference's form (src/vendor/mersennetwister.h:58-171).
struct Mt64
{
  uint64_t s[312];
  int left;
  int next;
  void init(uint64_t seed);
  void refill();
  double real2();
  // The 53-bit integer behind real2(): real2() == next53() * 2^-53 exactly.
  uint64_t next53();
  // Advances the stream by `count` draws without producing them (refills
  // only); the next real2() returns the value it would have returned after
  // `count` calls.
  void skip(long long count);
};

// src/library_prediction_split.h:17-286
class Splitter
{
public:
  Splitter(bool explore, bool full, bool shuffle, int crossfold, const std::vector<uint8_t>& usable, int seed);
  int next_library_size(int iter) const;
  void update(int library, int iter);
  void defer_fixed_size(Mt64& snapshot);
  const Mt64& stream() const { return rng_; }
  int num_usable() const { return num_usable_; }
  const std::vector<uint8_t>& lib() const { return lib_; }
  const std::vector<uint8_t>& pred() const { return pred_; }

private:
  bool explore_, full_, shuffle_;
  int crossfold_, num_usable_;
  std::vector<uint8_t> usable_, lib_, pred_;
  std::vector<int> fold_;
  std::vector<double> u_;
  Mt64 rng_;
  void draw();
};

struct Options
{
  int algorithm = 0;  // 0 simplex, 1 smap
  int distance = 1;   // 0 L1 (mean absolute error), 1 L2, 2 Wasserstein
  double aspect_ratio = 0;  // Wasserstein with dt: weight of the time axis
  bool force_compute = true;
  double missing_distance = 0;
  bool has_missing = false;
  bool panel_mode = false;
  double idw = 0;
  bool has_id_weights = false;
  std::map<std::pair<int, int>, float> id_weights;
  std::vector<double> thetas;
  bool low_memory = false;
  bool past_only = false;
};

// One configured task (the arguments an edm_task closure captures,
// src/edm.cpp:186-189).
struct Task
{
  int E = 0;
  int k = 0;        // kAdj: >0 neighbours, -1 all
  int library = 0;  // reported library size (src/edm.cpp:444)
  bool copredict = false;
  int lib_mask = 0;  // index into TaskPlan::masks
  int pred_mask = 0;
  bool save_prediction = false;
  bool save_coeffs = false;
};

// Shuffled fixed-size CCM splits whose row lists are left to a SplitProducer:
// the MT19937-64 state at the first split (each split then consumes
// num_usable draws), and per split, in stream order, its library size and
// mask id.
struct LazySplits
{
  bool active = false;
  Mt64 start{};
  int num_usable = 0;
  std::vector<int> library;
  std::vector<int> mask;
  std::vector<int> urows;  // the usable rows, in order
};

struct TaskPlan
{
  std::vector<Task> tasks;
  std::vector<std::vector<uint8_t>> masks;
  // Library row lists (mask rows whose target is observed) computed by the
  // parallel CCM splitter; lists_ready[id] marks the mask ids they replace.
  std::vector<std::vector<int>> lib_lists;
  std::vector<uint8_t> lists_ready;
  LazySplits lazy;
};

// One shuffled fixed-size split (src/library_prediction_split.h:231-270):
// draws num_usable uniforms from `state`, takes the library-th order
// statistic as the cutoff and returns, in `out`, the usable rows under it
// whose target is observed.  The uniforms are compared as the 53-bit
// integers behind getReal2 (same order, same cutoff test).
struct SplitScratch
{
  std::vector<uint64_t> u, c;
  std::vector<int> hist;
};
void select_library(Mt64& state, int library, const std::vector<int>& urows, const std::vector<double>& lib_target,
                    std::vector<int>& out, SplitScratch& scratch);

// Produces the row lists of plan.lazy on background threads while the
// caller runs the GPU work of earlier tasks: one thread walks the stream and
// snapshots it at each split, the others select each split's library from
// its snapshot.  wait(mask) blocks until that mask's list is in
// plan.lib_lists; the destructor stops and joins the threads.
class SplitProducer
{
public:
  SplitProducer(TaskPlan& plan, const std::vector<double>& lib_target, int threads);
  ~SplitProducer();
  SplitProducer(const SplitProducer&) = delete;
  SplitProducer& operator=(const SplitProducer&) = delete;
  void wait(int mask);

private:
  TaskPlan& plan_;
  const std::vector<double>& target_;
  std::vector<Mt64> snaps_;
  std::vector<int> split_of_mask_;
  std::vector<uint8_t> done_;
  std::atomic<int> snapped_{ 0 };
  std::atomic<int> next_{ 0 };
  std::atomic<bool> stop_{ false };
  std::mutex mu_;
  std::condition_variable cv_snap_, cv_done_;
  std::vector<std::thread> threads_;
  void sequence();
  void work();
};

// src/edm.cpp:90-212 configure_tasks
// With `lib_target` given, the shuffled fixed-size library splits of cross
// mapping (src/library_prediction_split.h:231-270) are produced as row lists
// by a parallel pass: one sequential sweep advances the MT19937-64 state and
// snapshots it at each split, then threads regenerate each split's uniforms,
// select the cutoff and emit the rows.  Without it every split is a mask.
TaskPlan configure_tasks(const Generator& g, const Options& opts, const std::vector<int>& Es,
                         const std::vector<int>& libraries, int k, int num_reps, int crossfold, bool explore,
                         bool full, bool shuffle, bool save_predictions, bool save_copredictions,
                         bool save_smap_coeffs, bool copredict_mode, const std::vector<uint8_t>& usable,
                         const std::vector<uint8_t>& cousable, int seed,
                         const std::vector<double>* lib_target = nullptr, int threads = 1,
                         bool lazy_lists = false);

// Cleans one input vector: every non-normal value becomes MISSING_D
// (src/r.cpp:64-71).
std::vector<double> clean_vector(const double* v, int n);

double sd_observed(const std::vector<double>& v);  // stats.cpp:96-101 on non-missing values

} // namespace fedm
