// C++ engine behind the C ABI: one context per GPU, the run_command
// pipeline and the single-task seam.
#pragma once

#include <array>
#include <map>
#include <memory>
#include <set>
#include <string>
#include <tuple>
#include <vector>

#include "host.h"
#include "kernels.h"

namespace fedm {

struct DevBuf
{
  void* p = nullptr;
  size_t cap = 0;
};

class Context
{
public:
  int device = 0;
  int num_sms = 1;
  cudaStream_t stream = nullptr;
  int precision = FEDM_PRECISION_MIXED;
  int (*keep_going)(void) = nullptr;
  // Kernel form of the mixed path (MixedForm in kernels.h); the environment
  // variable FEDM_MIXED_KERNEL (one6, fused2, ws4, ws8, split, one16)
  // overrides it when the context is created.
  int mixed_form = MIXED_ONE6;     // for k <= 6
  int mixed_form16 = MIXED_ONE16;  // for 7 <= k <= 14
  // With autotune on (the default; FEDM_AUTOTUNE=0 or a named form turns it
  // off) the form for E_a <= 8, k <= 14 is chosen per (algorithm, E_a, k) by
  // timing the candidates on the first batch large enough to measure.
  bool autotune = true;
  // Cap on resident CTAs per SM of the mixed kernels' persistent grids (0:
  // as many as fit), so that calls from other contexts can share the SMs;
  // FEDM_CTAS_PER_SM sets it when the context is created.
  int ctas_per_sm = 0;
  // Order of the mixed kernels' work items: 1 (default) largest and
  // smallest library alternately, so that scan-heavy and solve-heavy items
  // share the SMs; 0 largest first (FEDM_ITEM_ORDER=interleave|lpt).
  // Per-panel sub-tasks (independent panels) always go largest first.
  int item_order = 1;
  // Manifolds built on host threads and uploaded (FEDM_HOST_MANIFOLD=1)
  // instead of on the device; the same bits.
  bool host_manifold = false;
  // The series behind the manifolds now held in the context's buffers (the
  // device manifolds F_E, their pinned host copies and the uploaded series).
  // A later call whose manifold inputs are the same bits -- easy_edm()'s
  // sequence of edm() calls on one series -- takes those manifolds instead
  // of uploading the series and building them again; a call on another
  // series replaces the record.  FEDM_SERIES_CACHE=0 turns it off.
  struct SeriesCache
  {
    bool valid = false;
    std::vector<double> scalars, x, co_x, extras, point_time;
    std::vector<int> obs, target_row, panel;
    bool uploaded = false;                   // the series_* buffers hold it
    std::set<std::pair<int, bool>> built;    // (E, co_x) manifolds built from it
  } series;
  bool series_cache = true;
  // The task seam's sizes pass (fedm_run_task with null outputs) keeps its
  // task's outputs and timing here; the outputs pass that follows with the
  // same inputs (the same bytes) copies them instead of running the task
  // again.  Opaque to the header (engine.cpp's TaskMemo).
  std::shared_ptr<void> task_memo;
  // Lane order of the one-point mixed kernels: 1 (default) points of a work
  // item in Morton order of their first four manifold coordinates (three
  // when E_a < 4), 2 of their first three, 0 list order
  // (FEDM_POINT_ORDER=morton|morton3|list); per-panel sub-tasks keep list
  // order.  Results do not depend on it.
  int point_order = 1;
  // the lane orders computed during the current call, by (list, first row,
  // rows, manifold): a CCM call's batches share its prediction list
  std::map<std::tuple<const void*, int, int, const void*>, std::vector<int>> lane_orders;
  // lane orders kept across calls on the same series (the simplex and the
  // S-map call of one workflow order the same prediction lists alike), by
  // series generation, host manifold, key dimensions and the list's rows
  struct KeptLaneOrder
  {
    long long gen;
    const void* F;
    int dims;
    std::vector<int> rows, order;
  };
  std::vector<KeptLaneOrder> kept_lane_orders;
  // Spatially ordered library scans of the one-point mixed kernels (lists
  // of 2 048 to 262 144 rows, scanned in a Morton order of their rows with
  // tiles that no point of a work item can use skipped; the same bits):
  // on by default, FEDM_PRUNE=0 turns it off.  spatial_ranks: per manifold
  // buffer, every row's rank in that order, with the series generation it
  // was computed for (series_gen changes whenever the manifold buffers may
  // hold another series, so ranks are reused only across calls on the same
  // series).
  bool prune = true;
  long long series_gen = 0;
  std::map<const void*, std::pair<long long, std::vector<int>>> spatial_ranks;
  // The split S-map (MIXED_SPLIT): a second stream for the solves, the
  // scan's and the solver's resident CTAs per SM (FEDM_SPLIT_SCAN_CTAS,
  // FEDM_SPLIT_SOLVE_CTAS) and the points per chunk of the pipeline.
  cudaStream_t stream2 = nullptr;
  int split_scan_ctas = 3;
  int split_solve_ctas = 2;
  long long split_chunk_points = 4 << 20;
  // FAST precision: the k = all S-map's normal equations on the tensor cores
  // (E_a <= 5); FEDM_GRAM_TC=0 keeps the double-float SIMT kernel.
  bool gram_tc = true;
  // Differentiable S-map: the highest per-warp cache level its kernel may
  // use (FEDM_GRAD_CACHE=0..2; every level gives the same bits).
  int grad_cache_max = 2;
  std::map<std::array<int, 3>, int> tuned_forms;
  std::string last_error;
  fedm_timing timing{};

  explicit Context(int dev);
  ~Context();
  void reset_timing();
  // Grow-only named device buffers (the context's memory pool).
  void* buf(const std::string& name, size_t bytes);
  // The same for an optional buffer: null (and the pool unchanged) when the
  // device cannot provide it.
  void* try_buf(const std::string& name, size_t bytes);
  // Grow-only named pinned host buffers, for uploads that need no staging;
  // the caller must not refill one while a copy from it is in flight.
  void* host_buf(const std::string& name, size_t bytes);
  void upload(void* dst, const void* src, size_t bytes);
  void download(void* dst, const void* src, size_t bytes);
  void check(const char* what);

private:
  std::map<std::string, DevBuf> bufs_, host_bufs_;
};

// Everything run_command returns, in host memory.
struct CommandResult
{
  int rc = 0;
  std::vector<int> sE, sL, cE, cL;
  std::vector<double> sT, sR, sM, cT, cR, cM;
  int kmin = MISSING_I, kmax = MISSING_I;
  std::vector<double> preds, copreds, coeffs;  // R matrices (column-major)
  // saveManifolds: per task in task order, the library and prediction
  // manifolds, row-major and concatenated
  std::vector<int> man_rows, pman_rows, man_cols;
  std::vector<double> man, pman;
  int pred_rows = 0, pred_cols = 0, copred_rows = 0, copred_cols = 0, coeff_rows = 0, coeff_cols = 0;
  double missing_distance = 0, dt_weight = 0;
  bool has_missing_distance = false, has_dt_weight = false;
};

CommandResult run_command(Context& ctx, const fedm_args& a);

// Host-only pieces of the path (no device involved).
void host_usable(const fedm_args& a, int maxE, int copredict, unsigned char* out);
int host_manifold(const fedm_args& a, int E, int copredict, double* out);
int host_plan(const fedm_args& a, int max_tasks, int* task_E, int* task_k, int* task_library, int* task_copredict,
              unsigned char* lib_masks, unsigned char* pred_masks);
int run_task(Context& ctx, const fedm_args& a, fedm_task_io& io);
// Differentiable S-map (all library neighbours, per-lag weights w): the
// objective (0: MSE of the forecasts, 1: their rho with the targets) and,
// when dtheta is not null, its gradient.  predictions may be null.
int smap_grad(Context& ctx, const double* lib, const double* lib_t, int n_lib, const double* pred,
              const double* pred_t, int n_pred, int e_actual, double theta, const double* w, int objective,
              double* value, double* predictions, double* dtheta, double* dw);

} // namespace fedm
