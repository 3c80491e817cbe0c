// extern "C" boundary: plain pointers in, return codes out, no exceptions.
#include <cmath>
#include <cstring>
#include <new>

#include "engine.h"

namespace fedm {
double measure_peak(int kind, int num_sms, cudaStream_t s);
}

using fedm::CommandResult;
using fedm::Context;

struct fedm_ctx
{
  Context* c;
};

namespace {

struct ResultBox
{
  fedm_result r;
  CommandResult data;
};

template<class F>
int guarded(fedm_ctx* ctx, F&& f)
{
  try {
    return f();
  } catch (const fedm::Error& e) {
    if (ctx && ctx->c)
      ctx->c->last_error = e.what;
    return e.rc;
  } catch (const std::bad_alloc&) {
    if (ctx && ctx->c)
      ctx->c->last_error = "host allocation failed";
    return FEDM_UNKNOWN_ERROR;
  } catch (...) {
    if (ctx && ctx->c)
      ctx->c->last_error = "unknown error";
    return FEDM_UNKNOWN_ERROR;
  }
}

} // namespace

extern "C" {

int fedm_create(int device, fedm_ctx** out)
{
  if (!out)
    return FEDM_UNKNOWN_ERROR;
  *out = nullptr;
  try {
    auto* h = new fedm_ctx{ new Context(device) };
    *out = h;
    return FEDM_SUCCESS;
  } catch (...) {
    return FEDM_UNKNOWN_ERROR;
  }
}

void fedm_destroy(fedm_ctx* ctx)
{
  if (ctx) {
    delete ctx->c;
    delete ctx;
  }
}

const char* fedm_last_error(const fedm_ctx* ctx)
{
  return (ctx && ctx->c) ? ctx->c->last_error.c_str() : "no context";
}

int fedm_set_precision(fedm_ctx* ctx, int precision)
{
  if (!ctx || (precision != FEDM_PRECISION_FP64 && precision != FEDM_PRECISION_MIXED &&
               precision != FEDM_PRECISION_FAST))
    return FEDM_UNKNOWN_ERROR;
  ctx->c->precision = precision;
  return FEDM_SUCCESS;
}

int fedm_set_ctas_per_sm(fedm_ctx* ctx, int ctas)
{
  if (!ctx || ctas < 0)
    return FEDM_UNKNOWN_ERROR;
  ctx->c->ctas_per_sm = ctas;
  return FEDM_SUCCESS;
}

int fedm_set_keep_going(fedm_ctx* ctx, int (*keep_going)(void))
{
  if (!ctx)
    return FEDM_UNKNOWN_ERROR;
  ctx->c->keep_going = keep_going;
  return FEDM_SUCCESS;
}

int fedm_run_command(fedm_ctx* ctx, const fedm_args* args, fedm_result** out)
{
  if (!ctx || !args || !out)
    return FEDM_UNKNOWN_ERROR;
  *out = nullptr;
  auto* box = new (std::nothrow) ResultBox();
  if (!box)
    return FEDM_UNKNOWN_ERROR;
  std::memset(&box->r, 0, sizeof(box->r));
  box->r.internal = box;
  int rc = guarded(ctx, [&] {
    box->data = fedm::run_command(*ctx->c, *args);
    return FEDM_SUCCESS;
  });
  CommandResult& d = box->data;
  fedm_result& r = box->r;
  if (rc != FEDM_SUCCESS) {
    d = CommandResult{};
    d.rc = rc == FEDM_BREAK_HIT ? FEDM_BREAK_HIT : (rc ? rc : FEDM_UNKNOWN_ERROR);
  }
  r.rc = d.rc;
  r.n_stats = (int)d.sE.size();
  r.stat_E = d.sE.data();
  r.stat_library = d.sL.data();
  r.stat_theta = d.sT.data();
  r.stat_rho = d.sR.data();
  r.stat_mae = d.sM.data();
  r.n_costats = (int)d.cE.size();
  r.costat_E = d.cE.data();
  r.costat_library = d.cL.data();
  r.costat_theta = d.cT.data();
  r.costat_rho = d.cR.data();
  r.costat_mae = d.cM.data();
  r.kmin = d.kmin;
  r.kmax = d.kmax;
  r.pred_rows = d.pred_rows;
  r.pred_cols = d.pred_cols;
  r.predictions = (args->save_predictions && !d.preds.empty()) ? d.preds.data() : nullptr;
  r.copred_rows = d.copred_rows;
  r.copred_cols = d.copred_cols;
  r.copredictions = (args->save_copredictions && !d.copreds.empty()) ? d.copreds.data() : nullptr;
  r.coeff_rows = d.coeff_rows;
  r.coeff_cols = d.coeff_cols;
  r.coeffs = (args->save_smap_coeffs && !d.coeffs.empty()) ? d.coeffs.data() : nullptr;
  r.missing_distance = d.has_missing_distance ? d.missing_distance : NAN;
  r.dt_weight = d.has_dt_weight ? d.dt_weight : NAN;
  r.n_manifolds = (int)d.man_rows.size();
  r.manifold_rows = d.man_rows.data();
  r.pred_manifold_rows = d.pman_rows.data();
  r.manifold_cols = d.man_cols.data();
  r.manifolds = d.man.data();
  r.pred_manifolds = d.pman.data();
  *out = &r;
  return rc;
}

void fedm_free_result(fedm_result* r)
{
  if (r)
    delete (ResultBox*)r->internal;
}

int fedm_run_task(fedm_ctx* ctx, const fedm_args* args, fedm_task_io* io)
{
  if (!ctx || !args || !io || !io->library_rows || !io->prediction_rows)
    return FEDM_UNKNOWN_ERROR;
  return guarded(ctx, [&] { return fedm::run_task(*ctx->c, *args, *io); });
}

int fedm_last_timing(const fedm_ctx* ctx, fedm_timing* out)
{
  if (!ctx || !out)
    return FEDM_UNKNOWN_ERROR;
  *out = ctx->c->timing;
  return FEDM_SUCCESS;
}

int fedm_host_usable(const fedm_args* args, int maxE, int copredict, unsigned char* out)
{
  if (!args || !out)
    return FEDM_UNKNOWN_ERROR;
  return guarded(nullptr, [&] {
    fedm::host_usable(*args, maxE, copredict, out);
    return FEDM_SUCCESS;
  });
}

int fedm_host_manifold(const fedm_args* args, int E, int copredict, double* out, int* e_actual)
{
  if (!args || !e_actual)
    return FEDM_UNKNOWN_ERROR;
  return guarded(nullptr, [&] {
    *e_actual = fedm::host_manifold(*args, E, copredict, out);
    return FEDM_SUCCESS;
  });
}

int fedm_host_mt_real2(unsigned long long seed, long long count, double* out)
{
  if (!out || count < 0)
    return FEDM_UNKNOWN_ERROR;
  fedm::Mt64 m;
  m.init(seed);
  for (long long i = 0; i < count; i++)
    out[i] = m.real2();
  return FEDM_SUCCESS;
}

int fedm_host_plan(const fedm_args* args, int max_tasks, int* n_tasks, int* task_E, int* task_k, int* task_library,
                   int* task_copredict, unsigned char* lib_masks, unsigned char* pred_masks)
{
  if (!args || !n_tasks)
    return FEDM_UNKNOWN_ERROR;
  return guarded(nullptr, [&] {
    *n_tasks = fedm::host_plan(*args, max_tasks, task_E, task_k, task_library, task_copredict, lib_masks, pred_masks);
    return FEDM_SUCCESS;
  });
}

int fedm_smap_fwd(fedm_ctx* ctx, const double* lib_manifold, const double* lib_targets, int n_lib,
                  const double* pred_manifold, const double* pred_targets, int n_pred, int e_actual, double theta,
                  const double* w, double* mse, double* predictions)
{
  if (!ctx || !lib_manifold || !lib_targets || !pred_manifold || !pred_targets || !w || !mse)
    return FEDM_UNKNOWN_ERROR;
  return guarded(ctx, [&] {
    return fedm::smap_grad(*ctx->c, lib_manifold, lib_targets, n_lib, pred_manifold, pred_targets, n_pred, e_actual,
                           theta, w, 0, mse, predictions, nullptr, nullptr);
  });
}

int fedm_smap_bwd(fedm_ctx* ctx, const double* lib_manifold, const double* lib_targets, int n_lib,
                  const double* pred_manifold, const double* pred_targets, int n_pred, int e_actual, double theta,
                  const double* w, double* mse, double* dmse_dtheta, double* dmse_dw)
{
  if (!ctx || !lib_manifold || !lib_targets || !pred_manifold || !pred_targets || !w || !mse || !dmse_dtheta ||
      !dmse_dw)
    return FEDM_UNKNOWN_ERROR;
  return guarded(ctx, [&] {
    return fedm::smap_grad(*ctx->c, lib_manifold, lib_targets, n_lib, pred_manifold, pred_targets, n_pred, e_actual,
                           theta, w, 0, mse, nullptr, dmse_dtheta, dmse_dw);
  });
}

int fedm_smap_grad(fedm_ctx* ctx, const double* lib_manifold, const double* lib_targets, int n_lib,
                   const double* pred_manifold, const double* pred_targets, int n_pred, int e_actual, double theta,
                   const double* w, int objective, double* value, double* dvalue_dtheta, double* dvalue_dw,
                   double* predictions)
{
  if (!ctx || !lib_manifold || !lib_targets || !pred_manifold || !pred_targets || !w || !value ||
      !dvalue_dtheta || !dvalue_dw)
    return FEDM_UNKNOWN_ERROR;
  return guarded(ctx, [&] {
    return fedm::smap_grad(*ctx->c, lib_manifold, lib_targets, n_lib, pred_manifold, pred_targets, n_pred, e_actual,
                           theta, w, objective, value, predictions, dvalue_dtheta, dvalue_dw);
  });
}

int fedm_measure_peak(fedm_ctx* ctx, int kind, double* tflops)
{
  if (!ctx || !tflops || kind < 0 || kind > 3)
    return FEDM_UNKNOWN_ERROR;
  return guarded(ctx, [&] {
    *tflops = fedm::measure_peak(kind, ctx->c->num_sms, ctx->c->stream);
    return FEDM_SUCCESS;
  });
}

} // extern "C"
