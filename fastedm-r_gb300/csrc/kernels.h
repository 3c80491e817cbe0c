// Device-side data layout and kernel launchers.
//
// HBM layout of one run (all FP64 unless noted):
//   F_E      [n_rows x Ea]   lagged manifold of every row for one E
//   coF_E    [n_rows x Ea]   the coprediction manifold (co_x lags)
//   F32_E    [n_rows x Ea]   float copy for the mixed-precision scan
//   row tables [n_rows]      library target, coprediction target, target
//                            time, point time, panel id
//   lib_rows / pred_rows     int32 row lists, one slice per task
//   pred     [n_thetas x P]  forecasts, theta-major over the point space
//   coeffs   [P x (Ea+1)]    S-map coefficients of the last theta
// A "point" is one (task, prediction row); P counts them over all tasks.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

namespace fedm {

struct GramTC;

struct DevTask
{
  long long point_base;  // first global point id of this task
  int lib_off, n_lib;    // slice of lib_rows
  int pred_off, n_pred;  // slice of pred_rows
  int k;                 // neighbour slots the list kernels keep
  int k_req;             // k as requested (kAdj): >0, 0 or -1 (all valid)
  int task;              // index of the task's rc / k / stats slots
  int save_coeffs;
  int all_mode;          // k < 0 or k >= n_lib: every valid neighbour, library order
  int mixed;             // handled by the mixed-precision kernel
  int perm_off;          // one-point mixed kernels: point i of a work item's
                         // slot order is GroupParams::perm[perm_off + slot]
                         // (-1: slot order is list order)
  int box_off;           // one-point mixed kernels: -1, or the library is
                         // scanned in the spatial order MixedRun::scan_pos
                         // [lib_off + i] (positions in the list), whose
                         // 512-row sub-tiles have bounding boxes at
                         // MixedRun::boxes[(box_off + s) * E_a + j]
};

// Rows per sub-tile of the bounding boxes of a spatially ordered library.
constexpr int BOX_ROWS = 512;

// Largest E (columns of a point) the Wasserstein distance takes.
constexpr int WASS_EMAX = 16;

struct GroupParams
{
  // inputs
  const double* F;
  const double* Fp;
  const float* F32;
  const double* lib_target;
  const double* pred_target;
  const double* lib_target_time;
  const double* point_time;
  const int* panel;
  const int* panel_dense;  // dense panel index per row (id weights matrix)
  const float* id_w;       // [n_pid x n_pid] id weights, NaN = no entry
  int n_pid;
  const int* lib_rows;
  const int* pred_rows;
  const DevTask* tasks;
  const int* perm;         // lane orders of the one-point mixed kernels (DevTask::perm_off)
  int n_tasks;
  int Ea;
  int n_thetas;
  const double* thetas;
  int algorithm;  // 0 simplex, 1 smap
  int l1;
  int has_missing;
  double missing_distance;
  int panel_mode;
  double idw;
  int skip_other_panels;
  int has_id_weights;
  int past_only;
  int force_compute;
  // Wasserstein distance (src/distances.cpp:270-527) instead of L1/L2: a
  // point is read as a column-major w_rows x w_E matrix (w_rows = 1 + [dt]
  // + lagged extras) followed by w_unlagged unlagged extras
  int wasserstein;
  int w_E, w_rows, w_unlagged, w_dt;
  double aspect_ratio;
  long long total_points;  // size of the point space of the whole run
  // outputs
  double* pred;            // [n_thetas x total_points]
  double* coeffs;          // [total_points x (Ea+1)] or null
  int* kused;              // [total_points] or null
  int* task_rc;            // per task: max return code
  int* task_kmin;
  int* task_kmax;
  int* err_flag;           // set on a device-detected fault (missing id weight)
};

// Point statuses written by the neighbour kernels.
enum : int
{
  PT_OK = 0,
  PT_EARLY_SUCCESS = 1,  // k == 0 or no valid neighbour: rc SUCCESS, no forecast
  PT_INSUFFICIENT = 2,   // the same without forceCompute: rc 503
  PT_SKIP = 3,           // point belongs to the other (all / finite k) path
  PT_REDO = 4            // knn_refine_kernel could not settle the point: knn_exact_kernel runs it
};

struct ChunkBuffers
{
  long long p_begin, p_end;  // point range of this chunk
  int kcap;                  // neighbour slots per point
  int* nn_idx;               // [chunk x kcap]
  double* nn_dist;           // [chunk x kcap]
  int* nn_count;             // [chunk] k used
  int* status;               // [chunk]
  double* scratch;           // smap_nn solver scratch, or all-mode distances [chunk x max_nlib]
  long long scratch_doubles; // its size
  double* gram;              // all-mode S-map solver scratch, [chunk x n_thetas x slab]
  const long long* plist;    // optional: chunk point q is plist[q] (p_begin = 0, p_end = count)
  int redo_only;             // knn_exact_kernel runs only the points whose status is PT_REDO
};

// Exact FP64 kernels (reference operation order, no FMA contraction).
void launch_knn_exact(const GroupParams& g, const ChunkBuffers& c, int num_sms, cudaStream_t s);
void launch_simplex_nn(const GroupParams& g, const ChunkBuffers& c, cudaStream_t s);
void launch_smap_nn(const GroupParams& g, const ChunkBuffers& c, int num_sms, cudaStream_t s);
// ev0 / ev1 (optional) are recorded around the forecast kernels, after the
// distance pass.  With tc (FAST precision, E_a <= 5) the forecasts take the
// tensor-core path: rdist, means and dmin are filled, tc->G computed and
// solved.
void launch_all_mode(const GroupParams& g, const ChunkBuffers& c, int num_sms, long long max_nlib, cudaStream_t s,
                     const float2* gram_terms = nullptr, float* rdist = nullptr, double* means = nullptr,
                     cudaEvent_t ev0 = nullptr, cudaEvent_t ev1 = nullptr, const GramTC* tc = nullptr,
                     int tc_tiles = 0, float* dmin = nullptr);
// FAST precision, k = all S-map (E_a <= 8): per library-pool row the
// n(n+1)/2 + n Gram and right-hand-side products as float pairs; *bad is set
// when a product is not below 1e30 in magnitude.  launch_all_mode then also
// takes rdist [chunk x max_nlib] floats and means [chunk] doubles of scratch.
int gram_terms_per_row(int Ea);
void launch_gram_terms(const GroupParams& g, long long pool_size, float2* P, int* bad, cudaStream_t s);
void launch_stats(const GroupParams& g, const DevTask* tasks_host_unused, int n_tasks, double* rho, double* mae,
                  cudaStream_t s);
long long all_mode_slab(int Ea);  // doubles of solver scratch per (point, theta)
long long smap_nn_scratch_doubles(int num_sms, int n, int kcap);

// In-kernel forms of the mixed path (E_a <= 8).  ONE6 applies to k <= 6
// (8 candidate slots); other k use FUSED2.  WS4 / WS8 are S-map forms; the
// simplex then uses ONE6.
enum MixedForm
{
  MIXED_FUSED2 = 0,  // knn_mixed_kernel: two points per thread, two CTAs per SM
  MIXED_ONE6 = 1,    // knn_one_kernel: one point per thread, six CTAs per SM (40 registers)
  MIXED_WS4 = 2,     // S-map: knn_smap_ws_kernel, 8 scan warps, 4 FP64 solver warps
  MIXED_WS8 = 3,     // S-map: knn_smap_ws_kernel, 8 scan warps, 8 FP64 solver warps
  MIXED_WIDE = 4,    // knn_one_kernel's wide form (E_a 9..16), chosen by E_a; reported in timings only
  MIXED_ONE16 = 5,   // 7 <= k <= 14: knn_one_kernel with 16 candidate slots, four CTAs per SM
  MIXED_SPLIT = 6    // S-map, k <= 6: scan writes neighbour lists, smap_list_kernel solves in registers
};

// Mixed-precision neighbour scan for the common case (L2, no missing values,
// no panels, no past-only rule, finite k): FP32 candidate distances on a
// centred float copy of the manifold with a proven error margin, an FP64
// re-rank of every candidate inside the margin (reference operation order,
// so neighbour distances are the FP64 bits), then the forecast.  Points it
// cannot certify are appended to `fb_list` for the exact kernels.
struct MixedRun
{
  const float* F32;    // centred float library manifold, row stride 4 or 8
  const float* Fp32;   // centred float prediction manifold (same centre)
  const int2* items;   // (task, first prediction index) blocks of 512 points
  int n_items;
  int* counter;        // work-queue head
  double err_abs;      // bound on | ||fl32 diff|| - ||exact diff|| | from input rounding
  double gamma;        // relative bound of the FP32 accumulation
  long long* fb_list;  // points to recompute exactly
  double* fb_thr;      // per listed point: the certified bound on its neighbours' FP32 values (+inf: none)
  int* fb_count;
  int fb_cap;
  int* nn_idx;         // optional [total_points x kslots] final neighbour lists
  double* nn_dist;
  int kslots;
  unsigned long long* fp64_ops;  // optional: FP64 operations of the re-rank and forecast stage
  int* error;          // set when a bounded wait of the warp-specialised kernel ran out
  int form;            // kernel form (MixedForm)
  int ctas_per_sm;     // cap on resident CTAs per SM for the persistent grid (0: as many as fit)
  int item_begin;      // first item of this launch (the queue head starts here)
  int item_end;        // one past the last item of this launch
  // S-map lists (the scan of the split S-map, MIXED_SPLIT): per point slot
  // (item - item_begin) * 256 + thread, the neighbours a forecast uses
  int* l_keff;         // [slots] neighbours used; 0: no forecast to make
  int* l_rows;         // [L x slots] their library manifold rows
  double* l_dist;      // [L x slots] their FP64 distances
  long long l_slots;   // slots of the list buffers (the stride of l_rows / l_dist)
  // spatially ordered libraries (DevTask::box_off): positions in scan order,
  // the sub-tiles' (min, max) per coordinate, and a count of the
  // (prediction, library row) pairs the one-point scan actually scored
  const int* scan_pos;
  const float2* boxes;
  unsigned long long* scanned;
};

// Spatial scan orders of library lists (list l at pool offset lists[l].x,
// lists[l].y entries): its positions sorted by the bucket rank[row] >> sh
// of their rows (nb buckets, nb <= 8192), into scan_pos at the same offsets.
void launch_spatial_order(const int* lib_rows, const int* rank, int sh, int nb, const int2* lists, int n_lists,
                          int* scan_pos, cudaStream_t s);

// Bounding boxes of BOX_ROWS-row sub-tiles of spatially ordered libraries:
// sub-tile s covers positions [t.y, t.y + t.z) of the scan order of the list
// at pool offset t.x (rows lib_rows[t.x + scan_pos[t.x + i]]); boxes[s * ea
// + j] = (min, max) of coordinate j of the float manifold (row stride rs).
void launch_tile_boxes(const int* lib_rows, const int* scan_pos, const float* F32, int rs, int ea, const int4* subtiles,
                       int n_subtiles, float2* boxes, cudaStream_t s);

void launch_knn_mixed(const GroupParams& g, const MixedRun& m, int C, int num_sms, cudaStream_t s);

// The split S-map (E_a <= 4, k <= 6; kernels_split.cu).  The scan
// (knn_one_kernel's list form: FP32 scan, certification, FP64 re-rank)
// writes every point's neighbour list; smap_list_kernel then makes the
// forecasts with the whole JacobiSVD in registers, a few warps per SM,
// alongside the next chunk's scan on another stream.  Bits are those of the
// fused form.
constexpr int SPLIT_SLOTS = 6;  // neighbours a list holds (k <= 6)
constexpr int SPLIT_MAX_EA = 4;
struct SolveRun
{
  const int2* items;   // the scan's work items
  int item_begin, item_end;
  const int* l_keff;
  const int* l_rows;
  const double* l_dist;
  long long l_slots;
  unsigned long long* fp64_ops;  // optional: FP64 operations of the solves
};
void launch_smap_scan_lists(const GroupParams& g, const MixedRun& m, int num_sms, cudaStream_t s);

// FAST precision, k = all S-map, E_a <= 5 (kernels_gram_tc.cu): the
// weighted normal equations of every (point, theta) as one GEMM on the
// tensor cores (tcgen05), on exact bf16 slices of the weights and of the
// library-side products, then the FP64 solve (all_smap_gram_kernel).
struct GramTask
{
  int lib_off, n_lib;  // the task's library list (slice of lib_rows)
  int n_blocks;        // 64-row blocks of it
  int b_off;           // its first block in GramTC::bslices
  int q0;              // its first point of the chunk (chunk index; rows = points x thetas)
};
struct GramTile
{
  int task, row0, n_rows;  // 128 rows (or fewer) of one task's (point, theta) rows
};
struct GramTC
{
  const GramTask* tasks;
  const GramTile* tiles;
  unsigned long long* colmax;  // [tasks x 32] largest |product| per column, as bits
  unsigned char* bslices;      // product slices, 20 KB per block
  const float* rdist;          // [chunk x max_nlib] FP32 distances, -1: not a neighbour
  const float* dmin;           // [chunk] smallest distance
  const double* means;         // [chunk] mean distance
  const double* thetas;
  int n_thetas;
  long long max_nlib;
  int np;                      // terms: (E_a+1)(E_a+2)/2 + E_a+1
  double* G;                   // [chunk x n_thetas x 32] the sums
  int* error;                  // set when a bounded wait ran out
};
bool gram_tc_supported(int Ea);
int gram_tc_columns();
long long gram_tc_block_bytes();
int gram_tc_block_rows();
int gram_tc_tile_rows();
void launch_gram_tc_slices(const GroupParams& g, const GramTC& t, int n_tasks, int max_lib, cudaStream_t s);
void launch_gram_tc(const GramTC& t, int n_tiles, cudaStream_t s);
void launch_smap_lists(const GroupParams& g, const SolveRun& r, int num_sms, int ctas_per_sm, cudaStream_t s);

// Points the mixed kernels could not certify (ChunkBuffers::plist): the rows
// whose FP32 value is within the certified bound, scored in FP64 and ranked
// (knn_refine_kernel); a point with too many such rows is left PT_REDO.
struct RefineRun
{
  const float* F32;   // centred float library manifold (MixedRun::F32)
  const float* Fp32;  // centred float prediction manifold
  int rs;             // row stride of both
  const double* thr;  // [chunk] the bound of chunk point q
  int* redo_count;    // points marked PT_REDO
};
void launch_knn_refine(const GroupParams& g, const ChunkBuffers& c, const RefineRun& r, int num_sms, cudaStream_t s);

// The mixed path for E_a = 9..16 and up to 30 neighbours (knn_one_kernel:
// one point per thread, 32 candidate slots, work items of 256 points, float
// manifold row stride 16).
void launch_knn_wide(const GroupParams& g, const MixedRun& m, int num_sms, cudaStream_t s);

// Simplex or S-map (E_a <= 8, k <= 6) in the MIXED_ONE6 form; work items of
// 256 points.
void launch_mixed_one(const GroupParams& g, const MixedRun& m, int num_sms, cudaStream_t s);

// The same for 7 <= k <= 14 (MIXED_ONE16, kernels_one16.cu).
void launch_mixed_one16(const GroupParams& g, const MixedRun& m, int num_sms, cudaStream_t s);

// The lagged manifold of every observation for one E, built on the device
// from the series (kernels_manifold.cu): row-major [n x Ea], the host
// generator's bits.
struct ManifoldParams
{
  const double* t;           // observation times
  const double* x;           // x, or co_x for a coprediction manifold
  const double* extras;      // [num_extras x n]
  const int* panel;          // panel ids, null without panels
  const int* obs;            // observation numbers (INT_MIN: missing)
  const int* target_row;     // row of each row's forecast target, -1 if none
  int n, E, Edt, Ea, tau, num_extras, num_extras_lagged;
  int with_dt, reldt;
  double w;                  // dt weight
};
void launch_manifold(const ManifoldParams& p, double* F, int num_sms, cudaStream_t s);

// Panels with a finite penalty (panel_mode, idw > 0): the one-point form for
// E_a and C (8 or 16 slots; the wide form at E_a > 8) with the penalty in
// the scan (kernels_pen.cu).
void launch_mixed_pen(const GroupParams& g, const MixedRun& m, int C, int num_sms, cudaStream_t s);

// Differentiable S-map over every library neighbour (kernels_adjoint.cu).
struct AdjointParams
{
  const double* lib;     // [n_lib x e_actual] library manifold
  const double* lib_t;   // [n_lib] library targets
  const double* pred;    // [n_pred x e_actual] prediction manifold
  const double* pred_t;  // [n_pred] prediction targets
  const double* w;       // [e_actual] per-lag embedding weights
  double theta;
  int n_lib, n_pred, e_actual;
  int backward;          // 0: r, yhat only; 1: also dyhat/dtheta and dyhat/dw
  double* out;           // [n_pred x (e_actual + 3)]
  double* z;             // [n_lib x e_actual] scratch: the library scaled by w
  double* cache;         // [cache_warps x per-row doubles x n_lib] per-warp row values, or null
  long long cache_warps; // warps that own a slice of cache (the grid is capped to them)
  int cache_level;       // 2: d, a^2, 1/d and e_actual products per row; 1: d and a^2
};
// Warps of a full persistent grid of the cached adjoint kernel (the levels
// share one register budget, so one figure serves all of them).
int grad_cache_warps(int e_actual, int num_sms);
void launch_smap_grad(const AdjointParams& a, int num_sms, cudaStream_t s);
void center_to_f32(const double* F, long long n, int Ea, const double* center, float* F32, int stride,
                   cudaStream_t s);

} // namespace fedm
