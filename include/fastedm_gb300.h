/*
 * fastedm_gb300.h -- C ABI of the GB300 (sm_103a) implementation of fastEDM's
 * prediction path: lagged manifolds, pairwise distances with exact
 * k-nearest-neighbour selection, simplex and S-map forecasts, and the
 * convergent-cross-mapping library-size x replicate loop.
 *
 * The ABI takes plain pointers and sizes only.  Every entry point returns an
 * int status from the reference's return-code table (src/common.h:3-13 of
 * EDM-Developers/fastEDM-r): 0 SUCCESS, 1 BREAK_HIT, 400 INVALID_ALGORITHM,
 * 503 INSUFFICIENT_UNIQUE, 908 NOT_IMPLEMENTED, 8000 UNKNOWN_ERROR.  CUDA
 * failures map to 8000 with a message in fedm_last_error().  No C++
 * exception crosses this boundary.  One context is not re-entrant; distinct
 * contexts may be used from distinct threads.
 */
#ifndef FASTEDM_GB300_H
#define FASTEDM_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define FEDM_SUCCESS 0
#define FEDM_BREAK_HIT 1
#define FEDM_INVALID_ALGORITHM 400
#define FEDM_INSUFFICIENT_UNIQUE 503
#define FEDM_NOT_IMPLEMENTED 908
#define FEDM_UNKNOWN_ERROR 8000

/* Arithmetic of the distance / neighbour step.
 *  FEDM_PRECISION_FP64:  every distance in FP64 in the reference's operation
 *                        order ("plain FP64 GPU form").
 *  FEDM_PRECISION_MIXED: FP32 candidate distances with a proven error margin,
 *                        then an FP64 re-rank of every candidate inside the
 *                        margin, so neighbour sets, distances and forecasts
 *                        are the same bits as FP64.  Falls back to FP64
 *                        where its preconditions (no missing values, L2
 *                        distances, no panel weights) do not hold.
 *  FEDM_PRECISION_FAST:  MIXED, and the S-map with every library row as a
 *                        neighbour (k = all, E_actual <= 8, no missing
 *                        values) takes its weights in FP32 and accumulates
 *                        its normal equations in double-float arithmetic
 *                        before the FP64 solve: forecasts agree with FP64 to
 *                        about 1e-7 relative instead of bit for bit. */
#define FEDM_PRECISION_FP64 0
#define FEDM_PRECISION_MIXED 1
#define FEDM_PRECISION_FAST 2

typedef struct fedm_ctx fedm_ctx;

/* Opens a context on CUDA device `device` (its own stream and memory pool).
 * Replaces the reference's process-global thread pools (src/edm.cpp:79-88). */
int fedm_create(int device, fedm_ctx** out);
void fedm_destroy(fedm_ctx* ctx);
const char* fedm_last_error(const fedm_ctx* ctx);
/* Selects FEDM_PRECISION_*; the default is FEDM_PRECISION_MIXED. */
int fedm_set_precision(fedm_ctx* ctx, int precision);
/* Caps the resident CTAs per SM of the context's persistent mixed-path
 * kernels (0, the default: as many as fit).  Contexts used from concurrent
 * host threads can then share the SMs: an FP64-bound S-map call leaves most
 * issue slots idle, which a concurrent FP32-bound simplex call can fill
 * (e.g. S-map 5 and simplex 1 of the six CTAs per SM). */
int fedm_set_ctas_per_sm(fedm_ctx* ctx, int ctas);
/* Optional cancellation callback, polled between GPU chunks (the
 * reference's keep_going(), src/edm.cpp:572-591).  Returning 0 stops the run
 * with FEDM_BREAK_HIT. */
int fedm_set_keep_going(fedm_ctx* ctx, int (*keep_going)(void));

/* Arguments of the reference's run_command (src/r.cpp:107-117) after
 * edm()'s normalisation (R/edm.R:241-322).  NA is passed as NaN.  Optional
 * arrays are NULL. */
typedef struct fedm_args {
  int n;
  const double* t;
  const double* x;
  const double* y;          /* xmap variable; NULL => explore mode          */
  const int* panel;         /* panel ids, NA = INT_MIN; NULL => no panels    */
  const double* co_x;       /* coprediction variable; NULL => none           */
  int num_extras;
  const double* extras;     /* num_extras * n; extra e starts at e*n         */
  const int* Es;
  int nE;
  int tau;
  const double* thetas;
  int n_thetas;
  const int* libs;          /* NULL => library = NULL in R                   */
  int n_libs;
  int k;                    /* 0 default, -1 all (k = Inf in R)              */
  int algorithm;            /* 0 simplex, 1 smap                             */
  int num_reps;
  int p;
  int crossfold;
  int full;
  int shuffle;
  int seed;
  int save_predictions;
  int save_copredictions;
  int save_manifolds;
  int save_smap_coeffs;
  int dt;
  int reldt;
  double dt_weight;
  int allow_missing;
  double missing_distance;
  double panel_weight;      /* -1 => panelWeight = Inf (skip other panels)   */
  const double* panel_weights; /* n_panel_weights^2, column-major           */
  int n_panel_weights;
  int num_threads;          /* host threads for manifold construction        */
  int low_memory;
  int predict_with_past;
} fedm_args;

/* The list run_command returns (src/r.cpp:420-457), flattened.  NA is NaN
 * (doubles) or INT_MIN (ints).  Matrices are column-major like R's. */
typedef struct fedm_result {
  int rc;
  int n_stats;
  const int* stat_E;
  const int* stat_library;
  const double* stat_theta;
  const double* stat_rho;
  const double* stat_mae;
  int n_costats;
  const int* costat_E;
  const int* costat_library;
  const double* costat_theta;
  const double* costat_rho;
  const double* costat_mae;
  int kmin;
  int kmax;
  int pred_rows, pred_cols;
  const double* predictions;
  int copred_rows, copred_cols;
  const double* copredictions;
  int coeff_rows, coeff_cols;
  const double* coeffs;
  double missing_distance;  /* NaN unless allow_missing                       */
  double dt_weight;         /* NaN unless dt or reldt                         */
  void* internal;
  /* save_manifolds (src/r.cpp:406-409, 440-443): per task, in task order,
   * the library manifold (manifold_rows[f] x manifold_cols[f]: the task's
   * library rows whose target is observed) and the prediction manifold
   * (pred_manifold_rows[f] x manifold_cols[f]), each row-major with NA as
   * NaN, concatenated in task order in manifolds / pred_manifolds.
   * n_manifolds is 0 without save_manifolds. */
  int n_manifolds;
  const int* manifold_rows;
  const int* pred_manifold_rows;
  const int* manifold_cols;
  const double* manifolds;
  const double* pred_manifolds;
} fedm_result;

/* Replaces run_command -> launch_tasks -> edm_task (src/r.cpp:107-468,
 * src/edm.cpp:256-283, src/edm.cpp:285-548): all tasks of the call (every
 * E x library size x replicate/fold, and the coprediction tasks) are
 * configured on the host with the reference's splitter and RNG and executed
 * as batched GPU launches.  *out must be released with fedm_free_result. */
int fedm_run_command(fedm_ctx* ctx, const fedm_args* args, fedm_result** out);
void fedm_free_result(fedm_result* r);

/* One prediction task on explicit masks, the seam of edm_task /
 * af_make_prediction (src/edm.cpp:285-548, decl :66-71): library rows
 * `library_rows`, prediction rows `prediction_rows` (n bytes each).  The
 * first call (buffers NULL) fills the sizes; the second fills the
 * caller-allocated outputs:
 *   predictions[n_thetas*n_pred] (theta-major), coeffs[n_pred*(e_actual+1)],
 *   rc[n_thetas*n_pred], kused[n_pred], nn_offsets[n_pred+1],
 *   nn_idx[total_nn], nn_dist[total_nn], stats_rho[n_thetas],
 *   stats_mae[n_thetas]
 * nn_idx are indices into the task's library manifold (rows kept after
 * dropping missing targets), in the order make_prediction uses them
 * (src/edm.cpp:608-619). */
typedef struct fedm_task_io {
  const unsigned char* library_rows;
  const unsigned char* prediction_rows;
  int E;
  int k;
  int copredict;
  int distance;       /* 0 mean absolute error (L1), 1 Euclidean (L2),
                         2 Wasserstein (src/distances.cpp:270-527; the
                         reference's Distance enum, src/common.h:37-42;
                         E <= 16)                                           */
  int force_compute;
  int n_pred, n_lib, e_actual, total_nn;
  double* predictions;
  double* coeffs;
  int* rc;
  int* kused;
  int* nn_offsets;
  int* nn_idx;
  double* nn_dist;
  double* stats_rho;
  double* stats_mae;
  double aspect_ratio; /* Wasserstein with dt: Options::aspectRatio
                          (src/distances.cpp:361), 0 as R sets it           */
} fedm_task_io;

int fedm_run_task(fedm_ctx* ctx, const fedm_args* args, fedm_task_io* io);

/* Timing of the last fedm_run_command / fedm_run_task, from CUDA events on
 * the context's stream: device time from the first kernel of each batch
 * (inputs already uploaded) to its statistics, time of the dominant
 * distance/neighbour kernel and its launch count, and the host wall time of
 * the whole call (ms). */
typedef struct fedm_timing {
  double device_ms;
  double knn_kernel_ms;
  int knn_launches;
  double host_ms;
  long long distance_pairs;  /* (prediction, library) pairs examined        */
  long long predictions;     /* (prediction point, theta) forecasts made    */
  long long h2d_bytes;
  long long d2h_bytes;
  int fallback_points;       /* mixed path: points whose candidate list could
                                not be certified (re-run by the refine and,
                                if needed, the exact FP64 search)            */
  int kernel_launches;       /* kernels this library launched                */
  long long fp64_ops;        /* mixed path: FP64 add/sub/mul/div/sqrt of the
                                re-rank and forecast stage (exp = 32)        */
  double list_wait_ms;       /* host time blocked on CCM library lists that
                                the background splitter had not finished     */
  double setup_ms;           /* host time preparing task batches before their
                                first kernel (row pools, uploads)            */
  double finish_ms;          /* host time after each batch's statistics
                                (downloads, per-task results)                */
  int exact_points;          /* of fallback_points, those the bounded FP32
                                re-scan could not settle (full FP64 search)  */
  int mixed_form;            /* kernel form of the last mixed launch: 0
                                two points per thread, 1 one point per
                                thread at six CTAs per SM, 2 / 3 warp-
                                specialised S-map (4 / 8 solver warps),
                                4 the wide form (E_actual 9..16), 5 one
                                point per thread with 16 candidate slots
                                (7 <= k <= 14); -1 none                      */
  int autotune_probes;       /* timed form probes of the autotuner          */
  double prep_ms;            /* host time before the first batch: argument
                                handling, usable rows, task plan, row tables */
  double manifold_ms;        /* host time building and uploading manifolds  */
  long long scan_flops;      /* 3 * E_actual per (prediction, library) pair
                                the neighbour kernels scan (per-panel pairs
                                under independent panels)                    */
  double forecast_kernel_ms; /* k = all: time of the forecast kernels after
                                the distance pass (CUDA events)              */
  int forecast_launches;     /* their launches                               */
  int tensor_core_tiles;     /* FAST k = all S-map: 128-row tiles whose
                                normal equations ran on the tensor cores     */
  int manifold_builds;       /* manifolds built (and their series uploaded)
                                by this call                                 */
  int manifolds_reused;      /* manifolds taken from the context's buffers,
                                built by an earlier call on the same series  */
  long long scanned_pairs;   /* one-point mixed kernels: (prediction, library)
                                pairs actually scored; spatially ordered
                                libraries skip tiles no point can use        */
  int grad_cache_level;      /* differentiable S-map: per-warp cache level of
                                its kernel (2: distances, weights, 1/d and
                                per-lag products; 1: distances and weights;
                                0: none)                                     */
} fedm_timing;

int fedm_last_timing(const fedm_ctx* ctx, fedm_timing* out);

/* Host-side pieces of the path; they touch no GPU.
 *  fedm_host_usable:   the usable-row mask of run_command
 *                      (src/r.cpp:256-257 -> src/manifold.cpp:314-360).
 *  fedm_host_manifold: the lagged manifold row of every observation for E
 *                      (src/manifold.cpp:156-238), [n x e_actual]; out may
 *                      be NULL to query e_actual.
 *  fedm_host_mt_real2: the splitter's MT19937-64 stream
 *                      (src/vendor/mersennetwister.h:137-146).
 *  fedm_host_plan:     configure_tasks' task list (src/edm.cpp:90-212): per
 *                      task E, k, reported library size, coprediction flag
 *                      and library / prediction masks ([max_tasks x n]).
 *                      *n_tasks is always set. */
int fedm_host_usable(const fedm_args* args, int maxE, int copredict, unsigned char* out);
int fedm_host_manifold(const fedm_args* args, int E, int copredict, double* out, int* e_actual);
int fedm_host_mt_real2(unsigned long long seed, long long count, double* out);
int fedm_host_plan(const fedm_args* args, int max_tasks, int* n_tasks, int* task_E, int* task_k, int* task_library,
                   int* task_copredict, unsigned char* lib_masks, unsigned char* pred_masks);

/* Differentiable S-map over every library neighbour (k = all) with per-lag
 * embedding weights w: coordinates z = w * m enter both the distances and the
 * local regression.  No counterpart in the reference (it has no gradients);
 * at w = 1 the forward pass is the reference's S-map with k = all
 * (src/edm.cpp:737-814).  Host arrays: lib_manifold [n_lib x e_actual],
 * lib_targets [n_lib], pred_manifold [n_pred x e_actual], pred_targets
 * [n_pred], w [e_actual]; 1 <= e_actual <= 8.
 *  fedm_smap_fwd: mse = mean (yhat - target)^2 over prediction points;
 *                 predictions [n_pred] (may be NULL).
 *  fedm_smap_bwd: mse and its gradient dmse_dtheta, dmse_dw [e_actual],
 *                 from the adjoint of the weighted normal equations.
 *                 Nothing of size n_pred x n_lib is stored: each resident
 *                 warp keeps its current point's per-row values (distance,
 *                 weight, 1/d, per-lag products) in a slice of device
 *                 memory that the context holds for later calls, up to
 *                 8 GB; where that cannot be had, a smaller cache or none
 *                 is used, with the same results. */
int fedm_smap_fwd(fedm_ctx* ctx, const double* lib_manifold, const double* lib_targets, int n_lib,
                  const double* pred_manifold, const double* pred_targets, int n_pred, int e_actual, double theta,
                  const double* w, double* mse, double* predictions);
int fedm_smap_bwd(fedm_ctx* ctx, const double* lib_manifold, const double* lib_targets, int n_lib,
                  const double* pred_manifold, const double* pred_targets, int n_pred, int e_actual, double theta,
                  const double* w, double* mse, double* dmse_dtheta, double* dmse_dw);
/*  fedm_smap_grad: the same forward and backward pass for a chosen
 *                 objective: 0 the MSE (as fedm_smap_bwd), 1 rho, the
 *                 correlation of forecasts and targets computed as
 *                 src/stats.cpp:64-80 does (NaN, with NaN gradients, when
 *                 either has a root sum of squared deviations below 1e-9).
 *                 value, dvalue_dtheta, dvalue_dw [e_actual]; predictions
 *                 [n_pred] may be NULL. */
int fedm_smap_grad(fedm_ctx* ctx, const double* lib_manifold, const double* lib_targets, int n_lib,
                   const double* pred_manifold, const double* pred_targets, int n_pred, int e_actual, double theta,
                   const double* w, int objective, double* value, double* dvalue_dtheta, double* dvalue_dw,
                   double* predictions);

/* Allocation-free prediction for one task on caller-owned device buffers.
 * No counterpart in the reference: it exists for callers that cannot let a
 * library allocate GPU memory -- hosts that hand the process a fixed device
 * memory budget (the allocator belongs to someone else, so an unplanned
 * cudaMalloc fails or fragments it) and latency-sensitive pipelines that
 * avoid cudaMalloc/cudaFree because both can synchronise the device.
 *
 * Inputs (device pointers): lib_manifold [n_lib x e_actual] and lib_targets
 * [n_lib] (library rows whose target is observed, as edm_task's M),
 * pred_manifold [n_pred x e_actual]; thetas is a HOST array of n_thetas,
 * read before the call returns (its values travel as a kernel parameter).
 * Outputs (device pointers): predictions [n_thetas x n_pred] (theta-major,
 * MISSING = 1e100 where no forecast is made), kused [n_pred] (may be NULL).
 * algorithm 0 simplex, 1 S-map; 1 <= k (k >= n_lib uses every valid library
 * row, in library order); exact FP64 path, L2 distance, no missing values,
 * panels or past-only rule; work is queued on `stream` (a cudaStream_t, NULL
 * = legacy default stream) and the call returns before it finishes.  The
 * return value reports argument and launch errors only: a point without a
 * forecast (no valid neighbour) shows as MISSING in predictions and INT_MIN
 * in kused, as in edm_task's outputs.
 *
 * Working memory is one file-scope __device__ array of
 * FEDM_STATIC_SCRATCH_BYTES (32 MiB) that every GPU loading the library holds
 * until exit.  Limits: n_lib <= FEDM_STATIC_MAX_LIB, n_pred <=
 * FEDM_STATIC_MAX_PRED, k <= FEDM_STATIC_MAX_K, e_actual <= FEDM_STATIC_MAX_E,
 * n_thetas <= FEDM_STATIC_MAX_THETAS; larger requests return
 * FEDM_NOT_IMPLEMENTED with a message on stderr.  The first call on a device
 * looks the array's device address up (cudaGetSymbolAddress) with that device
 * current; make that first call before any stream capture.  The address is
 * kept for the life of the process, so the library must not be used across
 * a cudaDeviceReset.  All calls on a device share the array and it keeps the
 * last call's contents (each call re-initialises what it reads): calls that
 * overlap on the GPU race and must be serialised by the caller. */
#define FEDM_STATIC_SCRATCH_BYTES (32 << 20)
#define FEDM_STATIC_MAX_LIB (1 << 20)
#define FEDM_STATIC_MAX_PRED 65536
#define FEDM_STATIC_MAX_K 32
#define FEDM_STATIC_MAX_E 7
#define FEDM_STATIC_MAX_THETAS 64
int fedm_predict_static(const double* lib_manifold, const double* lib_targets, int n_lib,
                        const double* pred_manifold, int n_pred, int e_actual, int k, int algorithm,
                        const double* thetas, int n_thetas, double* predictions, int* kused, void* stream);

/* Measured arithmetic peak of this GPU in TFLOP/s (2 flops per fused
 * multiply-add): kind 0 FP32 FFMA, 1 FP64 DFMA, 2 packed FP32 FFMA2, 3 FP64
 * multiply and add issued separately (1 flop per instruction; the rate of
 * FP64 work that keeps an unfused operation order).  A diagnostic for
 * roofline fractions; it has no counterpart in the reference. */
int fedm_measure_peak(fedm_ctx* ctx, int kind, double* tflops);

#ifdef __cplusplus
}
#endif
#endif
