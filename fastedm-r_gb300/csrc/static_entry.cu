// fedm_predict_static: one neighbour search + forecast on caller-owned device
// buffers that allocates no device memory.
//
// Some callers cannot let a library allocate GPU memory.  Embedding hosts that
// hand the process a fixed device-memory budget (an R session or a service
// whose allocator owns the GPU) see an unplanned cudaMalloc fail or fragment
// their pool.  Latency-sensitive pipelines avoid cudaMalloc/cudaFree because
// both can synchronise the device and stall unrelated streams.  This entry
// point serves them: its working memory (neighbour lists, statuses, index
// lists, the task descriptor) lives in one file-scope __device__ array of
// fixed size, FEDM_STATIC_SCRATCH_BYTES, that every GPU which loads the
// library holds until the process exits.
//
// The array is shared by every call on a device and keeps the previous
// call's contents; each call re-initialises everything it reads.  Calls that
// overlap on the GPU (on two streams, or from two host threads) race on it
// and must be serialised by the caller.
#include <cuda_runtime.h>

#include <climits>
#include <cstdio>
#include <mutex>

#include "../../include/fastedm_gb300.h"
#include "kernels.h"

namespace fedm {

namespace {

constexpr size_t kScratchBytes = (size_t)FEDM_STATIC_SCRATCH_BYTES;

__device__ __align__(256) unsigned char g_static_scratch[kScratchBytes];

// Device address of g_static_scratch per device, looked up once per device
// with that device current (in host code the symbol name is only a handle).
std::mutex g_mu;
void* g_addr[64] = {};

void* scratch_address(int device, int& rc)
{
  std::lock_guard<std::mutex> lock(g_mu);
  if (device < 0 || device >= 64) {
    rc = FEDM_UNKNOWN_ERROR;
    return nullptr;
  }
  if (!g_addr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess || !p) {
      std::fprintf(stderr, "fedm_predict_static: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
      rc = FEDM_UNKNOWN_ERROR;
      return nullptr;
    }
    g_addr[device] = p;
  }
  rc = FEDM_SUCCESS;
  return g_addr[device];
}

// Everything a call needs besides the caller's buffers, passed by value as
// a kernel parameter: the host's copies may be gone once the call returns.
struct StaticInit
{
  DevTask task;
  int flags[4];  // task rc, kmin, kmax, error flag
  int n_thetas;
  double thetas[FEDM_STATIC_MAX_THETAS];
};

// Writes the task descriptor, the flags, the thetas and the identity row
// lists into the scratch array, and starts the forecasts as MISSING and
// kused as INT_MIN like edm_task's buffers (src/edm.cpp:345-361).
__global__ void static_init_kernel(StaticInit in, DevTask* d_task, int* d_flags, double* d_thetas, int* lib_rows,
                                   int n_lib, int* pred_rows, int n_pred, double* pred, long long n_forecasts,
                                   int* kused)
{
  const long long i0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long stride = (long long)gridDim.x * blockDim.x;
  if (i0 == 0) {
    *d_task = in.task;
    for (int j = 0; j < 4; j++)
      d_flags[j] = in.flags[j];
  }
  for (long long i = i0; i < in.n_thetas; i += stride)
    d_thetas[i] = in.thetas[i];
  for (long long i = i0; i < n_lib; i += stride)
    lib_rows[i] = (int)i;
  for (long long i = i0; i < n_pred; i += stride) {
    pred_rows[i] = (int)i;
    if (kused)
      kused[i] = INT_MIN;
  }
  for (long long i = i0; i < n_forecasts; i += stride)
    pred[i] = 1.0e+100;
}

size_t align256(size_t v)
{
  return (v + 255) & ~(size_t)255;
}

} // namespace

} // namespace fedm

extern "C" int fedm_predict_static(const double* lib_manifold, const double* lib_targets, int n_lib,
                                   const double* pred_manifold, int n_pred, int e_actual, int k, int algorithm,
                                   const double* thetas, int n_thetas, double* predictions, int* kused,
                                   void* stream)
{
  using namespace fedm;
  if (!lib_manifold || !lib_targets || !pred_manifold || !thetas || !predictions || n_lib < 0 || n_pred < 0 ||
      e_actual < 1 || n_thetas < 1 || (algorithm != 0 && algorithm != 1) || k < 1)
    return FEDM_UNKNOWN_ERROR;
  if (n_lib > FEDM_STATIC_MAX_LIB || n_pred > FEDM_STATIC_MAX_PRED || k > FEDM_STATIC_MAX_K ||
      e_actual > FEDM_STATIC_MAX_E || n_thetas > FEDM_STATIC_MAX_THETAS) {
    std::fprintf(stderr,
                 "fedm_predict_static: size beyond the static scratch limits (n_lib %d/%d, n_pred %d/%d, k %d/%d, "
                 "e_actual %d/%d, n_thetas %d/%d)\n",
                 n_lib, FEDM_STATIC_MAX_LIB, n_pred, FEDM_STATIC_MAX_PRED, k, FEDM_STATIC_MAX_K, e_actual,
                 FEDM_STATIC_MAX_E, n_thetas, FEDM_STATIC_MAX_THETAS);
    return FEDM_NOT_IMPLEMENTED;
  }
  if (n_pred == 0)
    return FEDM_SUCCESS;
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess)
    return FEDM_UNKNOWN_ERROR;
  int rc = 0;
  unsigned char* base = (unsigned char*)scratch_address(device, rc);
  if (!base)
    return rc;
  int num_sms = 1;
  cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, device);
  cudaStream_t s = (cudaStream_t)stream;

  // carve the scratch: task, counters, thetas, index lists, neighbour lists
  size_t off = 0;
  auto take = [&](size_t bytes) {
    unsigned char* p = base + off;
    off += align256(bytes);
    return p;
  };
  DevTask* d_task = (DevTask*)take(sizeof(DevTask));
  int* d_flags = (int*)take(4 * sizeof(int));  // task rc, kmin, kmax, error flag
  double* d_thetas = (double*)take((size_t)n_thetas * 8);
  int* d_lib_rows = (int*)take((size_t)(n_lib > 0 ? n_lib : 1) * 4);
  int* d_pred_rows = (int*)take((size_t)n_pred * 4);
  int* d_count = (int*)take((size_t)n_pred * 4);
  int* d_status = (int*)take((size_t)n_pred * 4);
  int* d_nn_idx = (int*)take((size_t)n_pred * k * 4);
  double* d_nn_dist = (double*)take((size_t)n_pred * k * 8);
  double* d_solver = (double*)take(8);
  if (off > kScratchBytes)
    return FEDM_NOT_IMPLEMENTED;  // cannot happen within the stated limits

  StaticInit init{};
  DevTask& task = init.task;
  task.point_base = 0;
  task.lib_off = 0;
  task.n_lib = n_lib;
  task.pred_off = 0;
  task.n_pred = n_pred;
  task.k = k;
  task.k_req = k;
  task.task = 0;
  task.save_coeffs = 0;
  task.all_mode = 0;
  task.mixed = 0;
  task.perm_off = -1;
  init.flags[0] = 0;
  init.flags[1] = INT_MAX;
  init.flags[2] = INT_MIN;
  init.flags[3] = 0;
  init.n_thetas = n_thetas;
  for (int t = 0; t < n_thetas; t++)
    init.thetas[t] = thetas[t];
  const long long np = (long long)n_pred * n_thetas;
  long long span = np > n_lib ? np : n_lib;
  const int blocks = (int)((span + 255) / 256 < 1024 ? (span + 255) / 256 : 1024);
  static_init_kernel<<<blocks, 256, 0, s>>>(init, d_task, d_flags, d_thetas, d_lib_rows, n_lib, d_pred_rows, n_pred,
                                            predictions, np, kused);

  GroupParams g{};
  g.F = lib_manifold;
  g.Fp = pred_manifold;
  g.lib_target = lib_targets;
  // no prediction targets (statistics are not computed here) and no time
  // tables: the kernels read those only for rho/MAE and under the past-only
  // rule, both off here (g.past_only = 0)
  g.pred_target = nullptr;
  g.lib_target_time = nullptr;
  g.point_time = nullptr;
  g.past_only = 0;
  g.lib_rows = d_lib_rows;
  g.pred_rows = d_pred_rows;
  g.tasks = d_task;
  g.n_tasks = 1;
  g.Ea = e_actual;
  g.n_thetas = n_thetas;
  g.thetas = d_thetas;
  g.algorithm = algorithm;
  g.force_compute = 1;
  g.total_points = n_pred;
  g.pred = predictions;
  g.kused = kused;
  g.task_rc = d_flags;
  g.task_kmin = d_flags + 1;
  g.task_kmax = d_flags + 2;
  g.err_flag = d_flags + 3;
  ChunkBuffers c{};
  c.p_begin = 0;
  c.p_end = n_pred;
  c.kcap = k;
  c.nn_idx = d_nn_idx;
  c.nn_dist = d_nn_dist;
  c.nn_count = d_count;
  c.status = d_status;
  c.scratch = d_solver;
  c.scratch_doubles = 1;
  launch_knn_exact(g, c, num_sms, s);
  if (algorithm == 0)
    launch_simplex_nn(g, c, s);
  else
    launch_smap_nn(g, c, num_sms, s);
  return cudaGetLastError() == cudaSuccess ? FEDM_SUCCESS : FEDM_UNKNOWN_ERROR;
}
