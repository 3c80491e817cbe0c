/*
 * edm_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of fastEDM's prediction path (the reference's src/edm.cpp,
 * src/manifold.{h,cpp}, src/distances.cpp, src/stats.cpp,
 * src/library_prediction_split.h and src/vendor/mersennetwister.h, driven the
 * way src/r.cpp:107-468 run_command drives them).  It exists to check the
 * GB300 library; nothing in the product links it.  Only tests/, bench.py's CPU
 * baseline leg and __graft_entry__.smoke() may load it.
 *
 * Parity pin: the restatement is checked against the golden rho values of the
 * reference's own test suite (tests/testthat/test-ci.R) to 1e-4, the
 * tolerance that suite uses.  Eigen (RcppEigen, unpinned version) is absent,
 * so its JacobiSVD / reductions are restated from Eigen 3.3/3.4's published
 * algorithm; S-map results are pinned only through those rho goldens.
 */
#ifndef FASTEDM_ORACLE_H
#define FASTEDM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Arguments of run_command (src/r.cpp:107-117) after edm()'s normalisation
 * (R/edm.R:241-322).  NA values are passed as NaN.  Optional arrays are NULL. */
typedef struct oracle_args {
  int n;
  const double* t;
  const double* x;
  const double* y;          /* xmap target; NULL => explore mode            */
  const int* panel;         /* panel ids (NA = INT_MIN); NULL => no panels  */
  const double* co_x;       /* coprediction variable; NULL => none          */
  int num_extras;
  const double* extras;     /* num_extras * n, extra e at extras[e*n]       */
  const int* Es;
  int nE;
  int tau;
  const double* thetas;
  int n_thetas;
  const int* libs;          /* NULL => R's library = NULL                   */
  int n_libs;
  int k;
  int algorithm;            /* 0 simplex, 1 smap                            */
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
  double panel_weight;
  const double* panel_weights; /* n_panel_weights^2, R column-major        */
  int n_panel_weights;
  int num_threads;
  int low_memory;
  int predict_with_past;
} oracle_args;

/* The R list that run_command returns (src/r.cpp:420-457), flattened.
 * MISSING values are reported as NaN (R's NA). */
typedef struct oracle_result {
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
  int kmin; /* INT_MIN => NA */
  int kmax;
  int pred_rows, pred_cols;       /* R matrices, column-major               */
  const double* predictions;      /* NULL if not saved                      */
  int copred_rows, copred_cols;
  const double* copredictions;
  int coeff_rows, coeff_cols;
  const double* coeffs;
  double missing_distance;
  double dt_weight;
  void* internal;
} oracle_result;

oracle_result* oracle_run_command(const oracle_args* args);
void oracle_free_result(oracle_result* r);

/* One edm_task (src/edm.cpp:285-548) on explicit library / prediction masks,
 * exposing the neighbour lists that make_prediction (src/edm.cpp:565-639)
 * selects.  Inputs are already NaN-cleaned by the caller exactly like
 * run_command does (the 'args' generator fields are used; Es[0] is E).
 * Outputs (caller-allocated, sizes from oracle_task_sizes):
 *   predictions[n_thetas * Np], coeffs[Np * (E_actual+1)], rc[n_thetas * Np],
 *   kused[Np], nn_offsets[Np+1], nn_idx[total], nn_dist[total],
 *   stats_rho[n_thetas], stats_mae[n_thetas].
 * 'copredict' selects the coprediction manifold for the prediction set. */
typedef struct oracle_task_io {
  const unsigned char* library_rows;    /* [n] */
  const unsigned char* prediction_rows; /* [n] */
  int E;
  int k;
  int copredict;
  int distance; /* 0 MAE (L1), 1 Euclidean, 2 Wasserstein */
  int force_compute;
  int n_pred, n_lib, e_actual, total_nn; /* filled by oracle_task_sizes */
  double* predictions;
  double* coeffs;
  int* rc;
  int* kused;
  int* nn_offsets;
  int* nn_idx;
  double* nn_dist;
  double* stats_rho;
  double* stats_mae;
  int* lib_point_rows;  /* [n_lib] original row of each library point      */
  int* pred_point_rows; /* [n_pred]                                         */
  double* lib_manifold; /* [n_lib * e_actual] or NULL                       */
  double* pred_manifold;/* [n_pred * e_actual] or NULL                      */
  double* lib_targets;  /* [n_lib] or NULL                                  */
  double* pred_targets; /* [n_pred] or NULL                                 */
  double missing_distance_used;
  double dt_weight_used;
  double aspect_ratio;  /* Wasserstein with dt (Options::aspectRatio)       */
} oracle_task_io;

/* The Wasserstein distance's transport cost of an n1 x n2 row-major cost
 * matrix with masses 1/n1 and 1/n2 (what the reference takes from
 * EMD_wrap, src/distances.cpp:455-470). */
double oracle_emd_uniform(const double* D, int n1, int n2);

/* First pass: fills n_pred, n_lib, e_actual and total_nn. */
int oracle_task_sizes(const oracle_args* args, oracle_task_io* io);
/* Second pass: fills the output arrays. Returns the task's max rc. */
int oracle_task_run(const oracle_args* args, oracle_task_io* io);

/* The task list configure_tasks builds (src/edm.cpp:90-212): per task E,
 * kAdj, reported library size, coprediction flag and the library /
 * prediction membership masks ([max_tasks x n] each).  *n_tasks is always
 * set; at most max_tasks entries are written. */
int oracle_plan(const oracle_args* args, int max_tasks, int* n_tasks, int* task_E, int* task_k, int* task_library,
                int* task_copredict, unsigned char* lib_masks, unsigned char* pred_masks);

/* Differentiable S-map check (no counterpart in the reference): MSE over
 * prediction points of S-map with every library neighbour on coordinates
 * z = w * m, and (dtheta non-NULL) dMSE/dtheta, dMSE/dw[E]; yhat may be NULL. */
int oracle_smap_grad(const double* lib, const double* lib_t, int n_lib, const double* pred, const double* pred_t,
                     int n_pred, int E, double theta, const double* w, double* mse, double* dtheta, double* dw,
                     double* yhat);

/* The usable-row mask run_command computes (src/r.cpp:256-257). */
int oracle_usable(const oracle_args* args, int maxE, int copredict, unsigned char* usable_out);

/* 0 (default): weights use std::exp like the reference.  1: weights use the
 * IEEE-only exp formula the GPU library evaluates, for bit-level parity. */
void oracle_set_exp_mode(int mode);
/* Summation orders the reference leaves to Eigen and its compiler, to
 * measure the spread of the reference's own builds: 0 (default) plain
 * sequential unfused sums; bit 1 / 2 Eigen's vectorised order with packets
 * of 2 / 4 doubles in the S-map's mean(d), X^T X and X^T y; bit 4 those
 * products' multiply-adds fused; bit 8 the scalar loops (distances, simplex
 * sum, S-map forecast) contracted to FMA. */
void oracle_set_sum_mode(int mode);
/* Benchmark sampling: predict only every stride-th row of each prediction
 * set (1, the default, is the reference's behaviour). */
void oracle_set_pred_stride(int stride);
double oracle_exp(double x);

/* MT19937-64 stream as the splitter consumes it (getReal2). */
void oracle_mt_real2(unsigned long long seed, long long count, double* out);

#ifdef __cplusplus
}
#endif
#endif
