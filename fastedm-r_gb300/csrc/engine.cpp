// The run_command pipeline on one GB300.
//
// Host: clean the series, build the generator, configure every task with
// the reference's splitter (src/edm.cpp:90-212), build one manifold per E for
// all rows, turn each task's masks into row lists.  Device: one batched
// launch sequence per (E, coprediction) group over the point space of all
// its tasks, chunked to bound scratch memory; rho/MAE per (task, theta) on the
// device; only the statistics and the saved forecasts come back.
#include "engine.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <thread>
#include <unordered_map>

namespace fedm {

// Device helpers (kernels_util.cu).
void fill_f64(double* p, long long n, double v, cudaStream_t s);
void fill_i32(int* p, long long n, int v, cudaStream_t s);

namespace {

void ck(cudaError_t e, const char* what)
{
  if (e != cudaSuccess)
    throw Error{ RC_UNKNOWN_ERROR, std::string(what) + ": " + cudaGetErrorString(e) };
}

double now_ms()
{
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

} // namespace

// ------------------------------------------------------------------ Context
Context::Context(int dev) : device(dev)
{
  ck(cudaSetDevice(dev), "cudaSetDevice");
  ck(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
  ck(cudaStreamCreateWithFlags(&stream2, cudaStreamNonBlocking), "cudaStreamCreate");
  ck(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute");
  if (const char* v = std::getenv("FEDM_MIXED_KERNEL")) {
    static const std::pair<const char*, int> forms[] = {
      { "one6", MIXED_ONE6 }, { "fused2", MIXED_FUSED2 }, { "ws4", MIXED_WS4 }, { "ws8", MIXED_WS8 },
      { "one16", MIXED_ONE16 }, { "split", MIXED_SPLIT }
    };
    for (const auto& f : forms)
      if (std::strcmp(v, f.first) == 0) {
        // a named form is used as given: one16 names the 7 <= k <= 14 form,
        // fused2 both, the others the k <= 6 form
        if (f.second == MIXED_ONE16 || f.second == MIXED_FUSED2)
          mixed_form16 = f.second;
        if (f.second != MIXED_ONE16)
          mixed_form = f.second;
        autotune = false;
      }
  }
  if (const char* v = std::getenv("FEDM_AUTOTUNE"))
    if (std::strcmp(v, "0") == 0)
      autotune = false;
  if (const char* v = std::getenv("FEDM_CTAS_PER_SM"))
    ctas_per_sm = std::max(0, std::atoi(v));
  if (const char* v = std::getenv("FEDM_SPLIT_SCAN_CTAS"))
    split_scan_ctas = std::max(1, std::atoi(v));
  if (const char* v = std::getenv("FEDM_SPLIT_SOLVE_CTAS"))
    split_solve_ctas = std::max(1, std::atoi(v));
  if (const char* v = std::getenv("FEDM_SPLIT_CHUNK_POINTS"))
    split_chunk_points = std::max(256LL, std::atoll(v));
  if (const char* v = std::getenv("FEDM_GRAM_TC"))
    gram_tc = std::strcmp(v, "0") != 0;
  if (const char* v = std::getenv("FEDM_GRAD_CACHE"))
    grad_cache_max = std::min(2, std::max(0, std::atoi(v)));
  if (const char* v = std::getenv("FEDM_ITEM_ORDER"))
    item_order = std::strcmp(v, "lpt") == 0 ? 0 : 1;
  if (const char* v = std::getenv("FEDM_HOST_MANIFOLD"))
    host_manifold = std::strcmp(v, "1") == 0;
  if (const char* v = std::getenv("FEDM_SERIES_CACHE"))
    series_cache = std::strcmp(v, "0") != 0;
  if (const char* v = std::getenv("FEDM_PRUNE"))
    prune = std::strcmp(v, "0") != 0;
  if (const char* v = std::getenv("FEDM_POINT_ORDER"))
    point_order = std::strcmp(v, "list") == 0 ? 0 : (std::strcmp(v, "morton3") == 0 ? 2 : 1);
  reset_timing();
}

void Context::reset_timing()
{
  timing = fedm_timing{};
  timing.mixed_form = -1;
  lane_orders.clear();  // list and manifold addresses are reused by later calls
}

namespace {

// Spreads the low 10 bits of v to every third bit (a Morton code of three
// coordinates).
uint32_t spread3(uint32_t v)
{
  v &= 0x3ff;
  v = (v | (v << 16)) & 0x030000ff;
  v = (v | (v << 8)) & 0x0300f00f;
  v = (v | (v << 4)) & 0x030c30c3;
  v = (v | (v << 2)) & 0x09249249;
  return v;
}

// Spreads the low 8 bits of v to every fourth bit (a Morton code of four
// coordinates).
uint32_t spread4(uint32_t v)
{
  v &= 0xff;
  v = (v | (v << 12)) & 0x000f000f;
  v = (v | (v << 6)) & 0x03030303;
  v = (v | (v << 3)) & 0x11111111;
  return v;
}

// Slot order of the rows rows[0..n): the Morton order of their first three
// manifold coordinates (F row-major, Ea columns), quantised to 10 bits over
// the rows' range -- or, with dims = 4, of their first four at 8 bits (at
// E_a = 4 that keys every coordinate; CCM's S-map step is 1.2% shorter than
// with three).  Ties keep list order: the sort key is (Morton key, list
// position).  Long lists are split over host threads: ranges and keys per
// thread, a stable split on the key's top byte, then each of the 256
// buckets sorted alone -- the order of one global sort.
std::vector<int> morton_lane_order(const double* F, int Ea, const int* rows, int n, int dims = 3)
{
  const int D = std::min(Ea, dims);
  const int bits = dims == 4 ? 8 : 10;
  const int hw = std::max(1, std::min(16, (int)std::thread::hardware_concurrency()));
  const int nt = std::max(1, std::min(hw, n / 16384));
  auto par = [nt](auto&& fn) {
    std::vector<std::thread> pool;
    for (int w = 1; w < nt; w++)
      pool.emplace_back(fn, w);
    fn(0);
    for (auto& t : pool)
      t.join();
  };
  auto first = [&](int w) { return (long long)n * w / nt; };
  std::vector<double> tlo((size_t)nt * 4, INFINITY), thi((size_t)nt * 4, -INFINITY);
  par([&](int w) {
    double l[4] = { INFINITY, INFINITY, INFINITY, INFINITY }, h[4] = { -INFINITY, -INFINITY, -INFINITY, -INFINITY };
    for (long long i = first(w); i < first(w + 1); i++)
      for (int j = 0; j < D; j++) {
        const double v = F[(size_t)rows[i] * Ea + j];
        l[j] = std::min(l[j], v);
        h[j] = std::max(h[j], v);
      }
    for (int j = 0; j < 4; j++) {
      tlo[(size_t)w * 4 + j] = l[j];
      thi[(size_t)w * 4 + j] = h[j];
    }
  });
  const double top = (double)((1 << bits) - 1);
  double lo[4] = { 0, 0, 0, 0 }, scale[4] = { 0, 0, 0, 0 };
  for (int j = 0; j < D; j++) {
    double l = INFINITY, h = -INFINITY;
    for (int w = 0; w < nt; w++) {
      l = std::min(l, tlo[(size_t)w * 4 + j]);
      h = std::max(h, thi[(size_t)w * 4 + j]);
    }
    lo[j] = l;
    scale[j] = h > l ? top / (h - l) : 0.0;
  }
  // packed (Morton key, list position), and per thread the count of each top byte
  std::vector<uint64_t> a(n), b(n);
  std::vector<int> pos((size_t)nt * 256, 0);
  par([&](int w) {
    int* cnt = &pos[(size_t)w * 256];
    for (long long i = first(w); i < first(w + 1); i++) {
      uint32_t k = 0;
      for (int j = 0; j < D; j++) {
        const double q = (F[(size_t)rows[i] * Ea + j] - lo[j]) * scale[j];
        const uint32_t qv = q >= 0 ? (uint32_t)std::min(top, q) : 0;  // NaN: 0
        k |= dims == 4 ? spread4(qv) << (3 - j) : spread3(qv) << (2 - j);
      }
      a[i] = ((uint64_t)k << 32) | (uint32_t)i;
      cnt[k >> 24]++;
    }
  });
  std::vector<int> start(257, 0);
  int acc = 0;
  for (int d = 0; d < 256; d++) {
    start[d] = acc;
    for (int w = 0; w < nt; w++) {
      const int c = pos[(size_t)w * 256 + d];
      pos[(size_t)w * 256 + d] = acc;
      acc += c;
    }
  }
  start[256] = acc;
  par([&](int w) {
    int* p = &pos[(size_t)w * 256];
    for (long long i = first(w); i < first(w + 1); i++)
      b[p[a[i] >> 56]++] = a[i];
  });
  std::atomic<int> next{ 0 };
  par([&](int) {
    for (int d; (d = next++) < 256;)
      std::sort(b.begin() + start[d], b.begin() + start[d + 1]);
  });
  std::vector<int> order(n);
  for (int i = 0; i < n; i++)
    order[i] = (int)(uint32_t)b[i];
  return order;
}

} // namespace

namespace {

// Every manifold row's place in a Morton order of its first four
// coordinates, at the resolution of cells: the coordinates are quantised
// over the range of the rows that have them all (5 bits each for four, 7
// for three, 10 for two or one), and a row's rank is the number of rows in
// cells of smaller Morton index, so the rows of one cell share it.  A cell
// histogram and its prefix sums give it in O(n), without a sort; rows with a
// missing or non-finite coordinate come last.  Computed once per manifold
// and call.
const std::vector<int>& spatial_rank(Context& ctx, const double* F, int n, int Ea)
{
  auto it = ctx.spatial_ranks.find(F);
  if (it != ctx.spatial_ranks.end() && it->second.first == ctx.series_gen)
    return it->second.second;
  const int D = std::min(Ea, 4);
  const int bits = D == 4 ? 5 : (D == 3 ? 7 : 10);
  double lo[4] = { INFINITY, INFINITY, INFINITY, INFINITY }, hi[4] = { -INFINITY, -INFINITY, -INFINITY, -INFINITY };
  std::vector<uint8_t> ok(n, 1);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < D; j++) {
      const double v = F[(size_t)i * Ea + j];
      if (v == MISSING_D || !std::isfinite(v)) {
        ok[i] = 0;
        break;
      }
      lo[j] = std::min(lo[j], v);
      hi[j] = std::max(hi[j], v);
    }
  const double top = (double)((1 << bits) - 1);
  double scale[4];
  for (int j = 0; j < D; j++)
    scale[j] = hi[j] > lo[j] ? top / (hi[j] - lo[j]) : 0.0;
  auto spread2 = [](uint32_t v) {
    v &= 0x3ff;
    v = (v | (v << 8)) & 0x00ff00ff;
    v = (v | (v << 4)) & 0x0f0f0f0f;
    v = (v | (v << 2)) & 0x33333333;
    v = (v | (v << 1)) & 0x55555555;
    return v;
  };
  const size_t ncell = (size_t)1 << (bits * D);
  std::vector<uint32_t> cell(n);
  std::vector<int> cnt(ncell + 1, 0);
  int nok = 0;
  for (int i = 0; i < n; i++) {
    if (!ok[i])
      continue;
    uint32_t q[4] = { 0, 0, 0, 0 };
    for (int j = 0; j < D; j++)
      q[j] = (uint32_t)std::min(top, std::max(0.0, std::floor((F[(size_t)i * Ea + j] - lo[j]) * scale[j])));
    uint32_t key;
    if (D == 4)
      key = spread4(q[0]) | (spread4(q[1]) << 1) | (spread4(q[2]) << 2) | (spread4(q[3]) << 3);
    else if (D == 3)
      key = spread3(q[0]) | (spread3(q[1]) << 1) | (spread3(q[2]) << 2);
    else if (D == 2)
      key = spread2(q[0]) | (spread2(q[1]) << 1);
    else
      key = q[0];
    cell[i] = key;
    cnt[key + 1]++;
    nok++;
  }
  for (size_t c = 0; c < ncell; c++)
    cnt[c + 1] += cnt[c];
  std::vector<int> rank(n);
  for (int i = 0; i < n; i++)
    rank[i] = ok[i] ? cnt[cell[i]] : nok;
  auto& slot = ctx.spatial_ranks[F];
  slot.first = ctx.series_gen;
  slot.second = std::move(rank);
  return slot.second;
}

} // namespace

Context::~Context()
{
  cudaSetDevice(device);
  if (stream)
    cudaStreamSynchronize(stream);
  if (stream2)
    cudaStreamSynchronize(stream2);
  for (auto& kv : bufs_)
    if (kv.second.p)
      cudaFree(kv.second.p);
  for (auto& kv : host_bufs_)
    if (kv.second.p)
      cudaFreeHost(kv.second.p);
  if (stream)
    cudaStreamDestroy(stream);
  if (stream2)
    cudaStreamDestroy(stream2);
}

void* Context::host_buf(const std::string& name, size_t bytes)
{
  DevBuf& b = host_bufs_[name];
  if (bytes == 0)
    bytes = 16;
  if (b.cap < bytes) {
    if (b.p) {
      ck(cudaStreamSynchronize(stream), "sync before realloc");
      ck(cudaFreeHost(b.p), "cudaFreeHost");
      b.p = nullptr;
      b.cap = 0;
    }
    size_t want = bytes + bytes / 8;
    ck(cudaHostAlloc(&b.p, want, cudaHostAllocDefault), ("cudaHostAlloc " + name).c_str());
    b.cap = want;
  }
  return b.p;
}

void* Context::buf(const std::string& name, size_t bytes)
{
  DevBuf& b = bufs_[name];
  if (bytes == 0)
    bytes = 16;
  if (b.cap < bytes) {
    if (b.p) {
      ck(cudaStreamSynchronize(stream), "sync before realloc");
      ck(cudaFree(b.p), "cudaFree");
      b.p = nullptr;
      b.cap = 0;
    }
    size_t want = bytes + bytes / 8;
    ck(cudaMalloc(&b.p, want), ("cudaMalloc " + name).c_str());
    b.cap = want;
  }
  return b.p;
}

void* Context::try_buf(const std::string& name, size_t bytes)
{
  auto it = bufs_.find(name);
  if (it != bufs_.end() && it->second.cap >= bytes)
    return it->second.p;
  void* p = nullptr;
  if (cudaMalloc(&p, bytes) != cudaSuccess) {
    cudaGetLastError();  // an allocation failure leaves the context usable
    return nullptr;
  }
  if (it != bufs_.end() && it->second.p) {
    ck(cudaStreamSynchronize(stream), "sync before realloc");
    ck(cudaFree(it->second.p), "cudaFree");
  }
  bufs_[name] = DevBuf{ p, bytes };
  return p;
}

void Context::upload(void* dst, const void* src, size_t bytes)
{
  if (bytes) {
    ck(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream), "H2D");
    timing.h2d_bytes += (long long)bytes;
  }
}

void Context::download(void* dst, const void* src, size_t bytes)
{
  if (bytes) {
    ck(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, stream), "D2H");
    timing.d2h_bytes += (long long)bytes;
  }
}

void Context::check(const char* what)
{
  ck(cudaGetLastError(), what);
}

namespace {

// ------------------------------------------------------------ preparation
struct Prepared
{
  Generator gen;
  Options opts;
  bool explore = true;
  std::vector<int> Es, libraries;
};

void prepare(const fedm_args& a, Prepared& P)
{
  // src/r.cpp:119-246
  Options& o = P.opts;
  o.missing_distance = a.missing_distance;
  o.low_memory = a.low_memory;
  o.past_only = a.predict_with_past;
  if (a.n_thetas > 0 && a.thetas)
    o.thetas.assign(a.thetas, a.thetas + a.n_thetas);
  else
    o.thetas = { 1.0 };
  if (a.nE <= 0 || !a.Es)
    throw Error{ RC_UNKNOWN_ERROR, "no E values" };
  if (a.n <= 0 || !a.t || !a.x)
    throw Error{ RC_UNKNOWN_ERROR, "empty series" };
  P.Es.assign(a.Es, a.Es + a.nE);
  for (int E : P.Es)
    if (E <= 0)
      throw Error{ RC_UNKNOWN_ERROR, "E must be positive" };
  if (a.libs)
    P.libraries.assign(a.libs, a.libs + a.n_libs);
  if (a.algorithm != 0 && a.algorithm != 1)
    throw Error{ RC_INVALID_ALGORITHM, "unknown algorithm" };
  o.algorithm = a.algorithm;
  o.distance = 1;
  Generator& g = P.gen;
  g.n = a.n;
  g.t = clean_vector(a.t, a.n);
  g.x = clean_vector(a.x, a.n);
  for (int i = 0; i < a.n; i++)
    if (g.t[i] == MISSING_D)
      g.x[i] = MISSING_D;
  if (a.y) {
    g.xmap = clean_vector(a.y, a.n);
    P.explore = false;
  }
  o.idw = a.panel_weight;
  if (a.panel) {
    g.panel.assign(a.panel, a.panel + a.n);
    o.panel_mode = true;
    if (a.panel_weights) {
      std::vector<int> uniq(g.panel);
      uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
      const int m = a.n_panel_weights;
      for (int i = 0; i < (int)uniq.size(); i++)
        for (int j = 0; j < (int)uniq.size(); j++)
          if (i < m && j < m)
            o.id_weights[{ uniq[i], uniq[j] }] = (float)a.panel_weights[i + (size_t)j * m];
      o.has_id_weights = !o.id_weights.empty();
      o.idw = 0;
    }
  }
  if (a.co_x)
    g.co_x = clean_vector(a.co_x, a.n);
  for (int e = 0; e < a.num_extras; e++)
    g.extras.push_back(clean_vector(a.extras + (size_t)e * a.n, a.n));
  g.tau = a.tau;
  g.p = a.p;
  g.num_extras_lagged = 0;
  g.dt = a.dt;
  g.reldt = a.reldt;
  g.allow_missing = a.allow_missing;
  g.init(a.dt_weight);
  o.has_missing = a.allow_missing;
  if (a.allow_missing && o.missing_distance == 0) {
    // src/stats.cpp:103-108 on the cleaned x
    o.missing_distance = 2 / std::sqrt(3.14159265358979323846) * sd_observed(g.x);
  }
}

int host_threads(const fedm_args& a)
{
  int hw = (int)std::thread::hardware_concurrency();
  int t = std::max(a.num_threads, hw > 0 ? hw : 1);
  return std::min(t, 64);
}

// Device copies of the per-row tables, shared by every group of a run.
struct DevRows
{
  double* lib_target;
  double* co_target;
  double* lib_target_time;
  double* point_time;
  int* panel;
  int* panel_dense;
  float* id_w;
  int n_pid;
  int n_rows;
  const int* panel_host;  // the generator's panel ids (host), null without panels
};

DevRows upload_rows(Context& ctx, const Generator& g, const RowTables& rt, const Options& o)
{
  DevRows d{};
  const size_t n = (size_t)g.n;
  d.n_rows = g.n;
  d.lib_target = (double*)ctx.buf("lib_target", n * 8);
  d.co_target = (double*)ctx.buf("co_target", n * 8);
  d.lib_target_time = (double*)ctx.buf("lib_target_time", n * 8);
  d.point_time = (double*)ctx.buf("point_time", n * 8);
  ctx.upload(d.lib_target, rt.lib_target.data(), n * 8);
  ctx.upload(d.co_target, rt.co_target.data(), n * 8);
  ctx.upload(d.lib_target_time, rt.lib_target_time.data(), n * 8);
  ctx.upload(d.point_time, rt.point_time.data(), n * 8);
  if (g.panel_mode) {
    d.panel = (int*)ctx.buf("panel", n * 4);
    ctx.upload(d.panel, g.panel.data(), n * 4);
    d.panel_host = g.panel.data();
    if (o.has_id_weights) {
      std::vector<int> ids(g.panel);
      std::sort(ids.begin(), ids.end());
      ids.erase(std::unique(ids.begin(), ids.end()), ids.end());
      std::unordered_map<int, int> dense;
      for (int i = 0; i < (int)ids.size(); i++)
        dense[ids[i]] = i;
      std::vector<int> pd(n);
      for (size_t i = 0; i < n; i++)
        pd[i] = dense[g.panel[i]];
      const int m = (int)ids.size();
      std::vector<float> w((size_t)m * m, NAN);
      for (int a = 0; a < m; a++)
        for (int b = 0; b < m; b++) {
          auto it = o.id_weights.find({ ids[a], ids[b] });
          if (it != o.id_weights.end())
            w[(size_t)a * m + b] = it->second;
        }
      d.panel_dense = (int*)ctx.buf("panel_dense", n * 4);
      d.id_w = (float*)ctx.buf("id_w", w.size() * 4);
      ctx.upload(d.panel_dense, pd.data(), n * 4);
      ctx.upload(d.id_w, w.data(), w.size() * 4);
      d.n_pid = m;
    }
  }
  return d;
}

// Outcome of one task.
struct TaskOut
{
  int rc = 0;
  int kmin = MISSING_I, kmax = MISSING_I;
  std::vector<double> rho, mae;
  std::vector<double> pred_last;  // saved forecasts (last theta), one per prediction row of the task
  std::vector<double> coeffs;     // [n_pred x (Ea+1)]
  // detail (single-task seam only)
  std::vector<double> pred_all;   // [n_thetas x n_pred]
  std::vector<int> kused;         // [n_pred]
  std::vector<int> nn_offsets, nn_idx;
  std::vector<double> nn_dist;
};

struct GroupJob
{
  int Ea = 0;
  const double* dF = nullptr;   // library manifold on the device
  const double* dFp = nullptr;  // prediction manifold on the device
  const double* hF = nullptr;   // host copies, row-major [n x Ea] (mixed-path margin, lane order)
  const double* hFp = nullptr;
  bool copredict = false;
  std::vector<int> task_ids;    // indices into the run's task list
  std::vector<const std::vector<int>*> lib_lists, pred_lists;
  bool detail = false;          // keep per-point outputs and neighbour lists
  bool knn_for_all = false;     // route all-neighbour tasks through the list path
  // optional: rows containing every library list of the job (the usable rows
  // for lazily produced CCM lists); the mixed path's bounding box is then
  // taken over it once instead of over each list
  const std::vector<int>* lib_superset = nullptr;
  // Wasserstein distance: the layout of a point (see GroupParams)
  int w_E = 0, w_rows = 1, w_unlagged = 0;
  bool w_dt = false;
};

// A point of E columns for the Wasserstein distance: the rows of the
// reference's column-major view and the unlagged extras after it
// (src/distances.cpp:316-320, 364-366).
void set_wasserstein_shape(GroupJob& job, const Generator& g, int E)
{
  job.w_E = E;
  job.w_dt = g.E_dt(E) > 0;
  job.w_rows = 1 + (job.w_dt ? 1 : 0) + g.num_extras_lagged;
  job.w_unlagged = g.num_extras - g.num_extras_lagged;
}

constexpr int KCAP_MAX = 16384;
constexpr int MIX_KMAX = 14;        // neighbours the mixed kernel serves (slots C = 16)
constexpr int MIX_POINTS = 512;     // prediction points per mixed work item
constexpr int WIDE_EA = 16;         // widest embedding of the mixed path (knn_one_kernel's wide form above 8)
constexpr int WIDE_KMAX = 30;       // neighbours the wide kernel serves (slots C = 32)
constexpr int WIDE_POINTS = 256;    // prediction points per wide work item
constexpr size_t LAZY_FIRST_BATCH = 64;  // first task batch of a group with lazily produced CCM lists
constexpr long long FB_CAP = 1 << 24;

// Whether the mixed kernel's preconditions hold for a group (see
// kernels_mixed.cu): L2, no missing values in any used row, no id weights,
// a panel penalty only between 1e-30 and 1e30 (a normal FP32 number whose
// sum with a squared distance cannot overflow; served by the one-point
// forms), independent panels only through per-panel sub-tasks, no
// past-only rule, Ea <= 16.  Also returns the per-column centre and the
// largest centred row norm.
bool mixed_eligible(const Context& ctx, const Options& o, const GroupJob& job, bool panel_split,
                    std::vector<double>& center, double& R)
{
  if (ctx.precision == FEDM_PRECISION_FP64 || o.distance != 1 || o.has_missing || o.low_memory || o.past_only ||
      !o.force_compute || job.Ea > WIDE_EA || job.Ea < 1 || !job.hF || !job.hFp)
    return false;
  // id weights change the distances per pair of panels; independent panels
  // are served when every task is split into per-panel sub-tasks
  if (o.panel_mode && (o.has_id_weights || (o.idw > 0 && !(o.idw >= 1e-30 && o.idw <= 1e30)) ||
                       (o.idw < 0 && !panel_split)))
    return false;
  const int Ea = job.Ea;
  std::vector<double> lo(Ea, INFINITY), hi(Ea, -INFINITY);
  // bounding box of the listed rows, split over host threads for long lists
  // (minimum and maximum do not depend on the split)
  const int hw = std::max(1, std::min(16, (int)std::thread::hardware_concurrency()));
  auto scan = [&](const double* F, const std::vector<int>& rows) {
    const long long n = (long long)rows.size();
    const int nt = (int)std::max<long long>(1, std::min<long long>(hw, n / 16384));
    std::vector<std::vector<double>> tlo(nt, lo), thi(nt, hi);
    std::vector<uint8_t> ok(nt, 1);
    auto work = [&](int w) {
      for (long long q = n * w / nt; q < n * (w + 1) / nt; q++) {
        const double* row = &F[(size_t)rows[q] * Ea];
        for (int j = 0; j < Ea; j++) {
          const double v = row[j];
          if (v == MISSING_D || !std::isfinite(v)) {
            ok[w] = 0;
            return;
          }
          tlo[w][j] = std::min(tlo[w][j], v);
          thi[w][j] = std::max(thi[w][j], v);
        }
      }
    };
    std::vector<std::thread> pool;
    for (int w = 1; w < nt; w++)
      pool.emplace_back(work, w);
    work(0);
    for (auto& th : pool)
      th.join();
    for (int w = 0; w < nt; w++) {
      if (!ok[w])
        return false;
      for (int j = 0; j < Ea; j++) {
        lo[j] = std::min(lo[j], tlo[w][j]);
        hi[j] = std::max(hi[j], thi[w][j]);
      }
    }
    return true;
  };
  std::vector<const std::vector<int>*> seen_l, seen_p;
  if (job.lib_superset && !scan(job.hF, *job.lib_superset))
    return false;
  for (size_t i = 0; i < job.lib_lists.size(); i++) {
    if (!job.lib_superset && std::find(seen_l.begin(), seen_l.end(), job.lib_lists[i]) == seen_l.end()) {
      seen_l.push_back(job.lib_lists[i]);
      if (!scan(job.hF, *job.lib_lists[i]))
        return false;
    }
    if (std::find(seen_p.begin(), seen_p.end(), job.pred_lists[i]) == seen_p.end()) {
      seen_p.push_back(job.pred_lists[i]);
      if (!scan(job.hFp, *job.pred_lists[i]))
        return false;
    }
  }
  center.assign(Ea, 0.0);
  for (int j = 0; j < Ea; j++)
    if (lo[j] <= hi[j])
      center[j] = 0.5 * (lo[j] + hi[j]);
  double r2 = 0;
  for (int j = 0; j < Ea; j++) {
    const double a = std::max(std::fabs(lo[j] - center[j]), std::fabs(hi[j] - center[j]));
    r2 += a * a;
  }
  R = std::sqrt(r2) * 1.01;
  return std::isfinite(R) && R < 1e15;
}

void run_group(Context& ctx, const Options& o, const std::vector<Task>& tasks, const DevRows& rows,
               GroupJob& job, std::vector<TaskOut>& outs)
{
  const int nT = (int)job.task_ids.size();
  if (nT == 0)
    return;
  const double t_enter = now_ms();
  const int Ea = job.Ea, n = Ea + 1;
  const int nth = (int)o.thetas.size();
  cudaStream_t s = ctx.stream;

  // Independent panels (panelWeight = Inf): a point's neighbours come from
  // its own panel only (src/distances.cpp:167-169), so every task runs as
  // sub-tasks, one per run of same-panel prediction rows, each scanning the
  // task's library rows of that panel.  A sub-list keeps library order, so
  // positions, ties and the k rules are those of the whole list; rho/MAE,
  // k and the outputs stay per task.
  const bool split = o.panel_mode && o.idw < 0 && rows.panel_host != nullptr;
  std::vector<double> center;
  double R = 0;
  const bool mixed_group = mixed_eligible(ctx, o, job, split, center, R);

  // task tables and row pools: offsets first, then the distinct lists copied
  // in parallel into pinned host buffers, uploaded without staging.  dt has
  // one entry per task (statistics, outputs); dk one per kernel task (the
  // tasks themselves, or their per-panel sub-tasks), in point order.
  std::vector<DevTask> dt(nT);
  std::unordered_map<const std::vector<int>*, int> lib_off, pred_off;
  std::vector<const std::vector<int>*> lib_src, pred_src;
  long long lib_total = 0, pred_total = 0;
  long long P = 0, max_nlib_all = 1;
  int kcap = 1, kmix = 0;
  bool any_finite = false, any_all = false, any_coeffs = false, any_mixed = false;
  struct PanelLists
  {
    std::unordered_map<int, int> of_panel;
    std::vector<std::vector<int>> rows, pos;  // per panel: library rows, their positions in the list
  };
  std::unordered_map<const std::vector<int>*, PanelLists> panel_lists;
  const std::vector<int> no_rows;
  struct KTask
  {
    int parent;
    const std::vector<int>* L;    // library rows scanned
    const std::vector<int>* pos;  // their positions in the task's list (null: the list itself)
    int pstart, plen;             // slice of the task's prediction rows
  };
  std::vector<KTask> kt;
  for (int j = 0; j < nT; j++) {
    const Task& t = tasks[job.task_ids[j]];
    const std::vector<int>* L = job.lib_lists[j];
    const std::vector<int>* Pl = job.pred_lists[j];
    auto it2 = pred_off.find(Pl);
    if (it2 == pred_off.end()) {
      it2 = pred_off.emplace(Pl, (int)pred_total).first;
      pred_src.push_back(Pl);
      pred_total += (long long)Pl->size();
    }
    DevTask& d = dt[j];
    d.point_base = P;
    d.lib_off = 0;
    d.n_lib = (int)L->size();
    d.pred_off = it2->second;
    d.n_pred = (int)Pl->size();
    d.k = t.k;
    d.k_req = t.k;
    d.task = j;
    d.save_coeffs = t.save_coeffs || job.detail;
    d.all_mode = (t.k < 0 || t.k >= d.n_lib) ? 1 : 0;
    if (d.all_mode && job.knn_for_all && d.n_lib <= KCAP_MAX) {
      d.all_mode = 0;
      d.k = std::max(d.n_lib, 0);
    }
    if (!d.all_mode && d.k > KCAP_MAX)
      throw Error{ RC_NOT_IMPLEMENTED, "k above the supported maximum of 16384 neighbours" };
    d.mixed = (mixed_group && !d.all_mode && d.k >= 1 && d.k <= (Ea > 8 ? WIDE_KMAX : MIX_KMAX)) ? 1 : 0;
    if (d.all_mode) {
      any_all = true;
      max_nlib_all = std::max<long long>(max_nlib_all, d.n_lib);
    } else if (d.mixed) {
      any_mixed = true;
      kmix = std::max(kmix, d.k);
      kcap = std::max(kcap, d.k);  // fallback points use the exact list path
    } else {
      any_finite = true;
      kcap = std::max(kcap, d.k);
    }
    any_coeffs |= (bool)d.save_coeffs && o.algorithm == 1;
    P += d.n_pred;
    if (!split) {
      kt.push_back(KTask{ j, L, nullptr, 0, d.n_pred });
      continue;
    }
    auto pit = panel_lists.find(L);
    if (pit == panel_lists.end()) {
      pit = panel_lists.emplace(L, PanelLists{}).first;
      PanelLists& pl = pit->second;
      for (int q = 0; q < (int)L->size(); q++) {
        const int pn = rows.panel_host[(*L)[q]];
        auto f = pl.of_panel.find(pn);
        if (f == pl.of_panel.end()) {
          f = pl.of_panel.emplace(pn, (int)pl.rows.size()).first;
          pl.rows.emplace_back();
          pl.pos.emplace_back();
        }
        pl.rows[f->second].push_back((*L)[q]);
        pl.pos[f->second].push_back(q);
      }
    }
    const PanelLists& pl = pit->second;
    for (int i = 0; i < d.n_pred;) {
      const int pn = rows.panel_host[(*Pl)[i]];
      int e = i + 1;
      while (e < d.n_pred && rows.panel_host[(*Pl)[e]] == pn)
        e++;
      auto f = pl.of_panel.find(pn);
      if (f == pl.of_panel.end())
        kt.push_back(KTask{ j, &no_rows, &no_rows, i, e - i });
      else
        kt.push_back(KTask{ j, &pl.rows[f->second], &pl.pos[f->second], i, e - i });
      i = e;
    }
  }
  const int nK = (int)kt.size();
  std::vector<DevTask> dk(nK);
  std::vector<long long> kbase(nK);
  for (int q = 0; q < nK; q++) {
    const KTask& kq = kt[q];
    auto it = lib_off.find(kq.L);
    if (it == lib_off.end()) {
      it = lib_off.emplace(kq.L, (int)lib_total).first;
      lib_src.push_back(kq.L);
      lib_total += (long long)kq.L->size();
    }
    DevTask d = dt[kq.parent];
    d.point_base += kq.pstart;
    d.pred_off += kq.pstart;
    d.n_pred = kq.plen;
    d.lib_off = it->second;
    d.n_lib = (int)kq.L->size();
    dk[q] = d;
    kbase[q] = d.point_base;
  }
  for (const DevTask& d : dk)
    ctx.timing.scan_flops += 3LL * Ea * d.n_pred * (long long)d.n_lib;
  // lane orders of the one-point mixed kernels: per kernel task, its
  // prediction rows in Morton order of their coordinates (computed once per
  // list and call, or taken from an earlier call on the same series).  Not for per-panel sub-tasks: their small libraries make
  // every item solve-bound alike, and on 512 independent panels the orders
  // gained no device time while their host cost lowered the end-to-end rate
  // by 5%.
  std::vector<int> perm_pool;
  for (int j = 0; j < nK; j++) {
    dk[j].perm_off = -1;
    dk[j].box_off = -1;
  }
  if (mixed_group && !split && ctx.point_order >= 1 && Ea <= 16) {
    std::map<std::tuple<const void*, int, int, const void*>, int> offs;
    for (int j = 0; j < nK; j++) {
      if (!dk[j].mixed || dk[j].n_pred < 64)
        continue;
      const std::vector<int>* Pl = job.pred_lists[kt[j].parent];
      const auto key = std::make_tuple((const void*)Pl, kt[j].pstart, kt[j].plen, (const void*)job.hFp);
      auto it = offs.find(key);
      if (it == offs.end()) {
        auto c = ctx.lane_orders.find(key);
        if (c == ctx.lane_orders.end()) {
          const int dims = ctx.point_order == 1 && Ea >= 4 ? 4 : 3;
          const int* rows = Pl->data() + kt[j].pstart;
          const int len = kt[j].plen;
          const std::vector<int>* kept = nullptr;
          for (const auto& e : ctx.kept_lane_orders)
            if (e.gen == ctx.series_gen && e.F == (const void*)job.hFp && e.dims == dims && (int)e.rows.size() == len &&
                std::memcmp(e.rows.data(), rows, (size_t)len * sizeof(int)) == 0) {
              kept = &e.order;
              break;
            }
          if (kept) {
            c = ctx.lane_orders.emplace(key, *kept).first;
          } else {
            c = ctx.lane_orders.emplace(key, morton_lane_order(job.hFp, Ea, rows, len, dims)).first;
            // keep it for later calls on this series (at most 32 lists)
            auto& kl = ctx.kept_lane_orders;
            kl.erase(std::remove_if(kl.begin(), kl.end(),
                                    [&](const Context::KeptLaneOrder& e) { return e.gen != ctx.series_gen; }),
                     kl.end());
            if (kl.size() >= 32)
              kl.erase(kl.begin());
            kl.push_back(Context::KeptLaneOrder{ ctx.series_gen, (const void*)job.hFp, dims,
                                                 std::vector<int>(rows, rows + len), c->second });
          }
        }
        it = offs.emplace(key, (int)perm_pool.size()).first;
        perm_pool.insert(perm_pool.end(), c->second.begin(), c->second.end());
      }
      dk[j].perm_off = it->second;
    }
  }
  // spatially ordered scans of the one-point mixed kernels (one_point.cuh):
  // each library list of PRUNE_MIN..PRUNE_MAX rows that a mixed kernel task
  // scans gets an order of its positions by the spatial rank of their rows
  // (a counting sort on the rank's top 12 bits, on the device: tiles of
  // 1 024 rows then hold rows of a compact region) and BOX_ROWS-row
  // sub-tiles whose boxes a kernel computes once the float manifold exists
  constexpr int PRUNE_MIN = 2048, PRUNE_MAX = 1 << 18;
  std::vector<int4> subtiles;
  std::vector<const std::vector<int>*> scan_src;
  std::unordered_map<const std::vector<int>*, int> box_of;
  if (mixed_group && !split && ctx.prune && job.hF) {
    for (int q = 0; q < nK; q++) {
      const std::vector<int>* L = kt[q].L;
      if (!dk[q].mixed || (int)L->size() < PRUNE_MIN || (int)L->size() > PRUNE_MAX)
        continue;
      auto it = box_of.find(L);
      if (it == box_of.end()) {
        it = box_of.emplace(L, (int)subtiles.size()).first;
        scan_src.push_back(L);
        const int off = lib_off[L];
        for (int st = 0; st < (int)L->size(); st += BOX_ROWS)
          subtiles.push_back(make_int4(off, st, std::min<int>(BOX_ROWS, (int)L->size() - st), 0));
      }
      dk[q].box_off = it->second;
    }
  }
  // library position of slot v of point p in its task's list (detail mode)
  auto task_pos = [&](long long p, int v) {
    if (!split)
      return v;
    const int q = (int)(std::upper_bound(kbase.begin(), kbase.end(), p) - kbase.begin()) - 1;
    return (*kt[q].pos)[v];
  };
  // the all-mode distance rows' stride, a multiple of four so that rows of
  // FP32 distances start on 16-byte boundaries
  max_nlib_all = (max_nlib_all + 3) & ~3LL;
  if (Ea + 32 * (n + 1) + n * (n + 1) / 2 + n > 24000 && any_all && o.algorithm == 1)
    throw Error{ RC_NOT_IMPLEMENTED, "embedding too wide for the all-neighbour S-map" };

  DevTask* d_tasks = (DevTask*)ctx.buf("tasks", std::max<size_t>(dk.size(), 1) * sizeof(DevTask));
  DevTask* d_ptasks = (DevTask*)ctx.buf("ptasks", dt.size() * sizeof(DevTask));
  if (lib_total > INT_MAX || pred_total > INT_MAX)
    throw Error{ RC_NOT_IMPLEMENTED, "row pool of a task batch above 2^31 rows" };
  // an upload from these buffers by an earlier call that ended in an error
  // may still be queued; normally the stream is idle here
  ck(cudaStreamSynchronize(s), "sync");
  auto fill_pool = [&](const std::vector<const std::vector<int>*>& src, long long total, const char* name) {
    int* h = (int*)ctx.host_buf(name, (size_t)std::max<long long>(total, 1) * 4);
    const int nth_copy = (int)std::min<long long>(8, std::max<long long>(1, total >> 20));
    auto copy_range = [&](int w) {
      long long off = 0;
      for (size_t l = 0; l < src.size(); l++) {
        if ((int)(l % nth_copy) == w && !src[l]->empty())
          std::memcpy(h + off, src[l]->data(), src[l]->size() * 4);
        off += (long long)src[l]->size();
      }
    };
    std::vector<std::thread> pool;
    for (int w = 1; w < nth_copy; w++)
      pool.emplace_back(copy_range, w);
    copy_range(0);
    for (auto& th : pool)
      th.join();
    return h;
  };
  const int* h_lib = fill_pool(lib_src, lib_total, "lib_pool");
  const int* h_pred = fill_pool(pred_src, pred_total, "pred_pool");
  int* d_lib = (int*)ctx.buf("lib_pool", (size_t)std::max<long long>(lib_total, 1) * 4);
  int* d_pred = (int*)ctx.buf("pred_pool", (size_t)std::max<long long>(pred_total, 1) * 4);
  double* d_thetas = (double*)ctx.buf("thetas", nth * 8);
  ctx.upload(d_tasks, dk.data(), dk.size() * sizeof(DevTask));
  ctx.upload(d_ptasks, dt.data(), dt.size() * sizeof(DevTask));
  int* d_perm = (int*)ctx.buf("perm_pool", std::max<size_t>(perm_pool.size(), 1) * 4);
  if (!perm_pool.empty())
    ctx.upload(d_perm, perm_pool.data(), perm_pool.size() * 4);
  ctx.upload(d_lib, h_lib, (size_t)lib_total * 4);
  ctx.upload(d_pred, h_pred, (size_t)pred_total * 4);
  // the spatial scan orders, at the lists' offsets in the library pool: a
  // counting sort per list on the device, on the top bits of each row's
  // spatial rank (at most 4 096 buckets)
  int* d_scan = nullptr;
  int2* d_lists = nullptr;
  int* d_rank = nullptr;
  int scan_sh = 0, scan_nb = 0;
  if (!scan_src.empty()) {
    const std::vector<int>& rank = spatial_rank(ctx, job.hF, rows.n_rows, Ea);
    while ((rows.n_rows >> scan_sh) >= 4096)
      scan_sh++;
    scan_nb = (rows.n_rows >> scan_sh) + 1;
    std::vector<int2> lists;
    lists.reserve(scan_src.size());
    for (const std::vector<int>* L : scan_src)
      lists.push_back(make_int2(lib_off[L], (int)L->size()));
    d_rank = (int*)ctx.buf("spatial_rank", (size_t)std::max(rows.n_rows, 1) * 4);
    d_lists = (int2*)ctx.buf("scan_lists", lists.size() * sizeof(int2));
    ctx.upload(d_rank, rank.data(), (size_t)rows.n_rows * 4);
    ctx.upload(d_lists, lists.data(), lists.size() * sizeof(int2));
    d_scan = (int*)ctx.buf("scan_pool", (size_t)std::max<long long>(lib_total, 1) * 4);
  }
  ctx.upload(d_thetas, o.thetas.data(), nth * 8);

  GroupParams g{};
  g.F = job.dF;
  g.Fp = job.dFp;
  g.lib_target = rows.lib_target;
  g.pred_target = job.copredict ? rows.co_target : rows.lib_target;
  g.lib_target_time = rows.lib_target_time;
  g.point_time = rows.point_time;
  g.panel = rows.panel;
  g.panel_dense = rows.panel_dense;
  g.id_w = rows.id_w;
  g.n_pid = rows.n_pid;
  g.lib_rows = d_lib;
  g.pred_rows = d_pred;
  g.tasks = d_tasks;
  g.perm = d_perm;
  g.n_tasks = nK;
  g.Ea = Ea;
  g.n_thetas = nth;
  g.thetas = d_thetas;
  g.algorithm = o.algorithm;
  g.l1 = o.distance == 0;
  // the lazy (lowMemory) distance always tests for missing values and has
  // no past-only rule (src/distances.cpp:69-149)
  g.has_missing = o.has_missing || o.low_memory;
  g.missing_distance = o.missing_distance;
  g.panel_mode = o.panel_mode;
  g.idw = o.idw;
  g.skip_other_panels = o.panel_mode && o.idw < 0;
  g.has_id_weights = o.has_id_weights;
  g.past_only = o.past_only && !o.low_memory;
  g.force_compute = o.force_compute;
  g.wasserstein = o.distance == 2;
  g.w_E = job.w_E;
  g.w_rows = job.w_rows;
  g.w_unlagged = job.w_unlagged;
  g.w_dt = job.w_dt ? 1 : 0;
  g.aspect_ratio = o.aspect_ratio;
  g.total_points = P;
  g.pred = (double*)ctx.buf("pred", (size_t)std::max<long long>(P, 1) * nth * 8);
  fill_f64(g.pred, P * nth, MISSING_D, s);
  if (any_coeffs) {
    g.coeffs = (double*)ctx.buf("coeffs", (size_t)std::max<long long>(P, 1) * n * 8);
    fill_f64(g.coeffs, P * n, MISSING_D, s);
  }
  if (job.detail) {
    g.kused = (int*)ctx.buf("kused", (size_t)std::max<long long>(P, 1) * 4);
    fill_i32(g.kused, P, MISSING_I, s);
  }
  g.task_rc = (int*)ctx.buf("task_rc", nT * 4);
  g.task_kmin = (int*)ctx.buf("task_kmin", nT * 4);
  g.task_kmax = (int*)ctx.buf("task_kmax", nT * 4);
  g.err_flag = (int*)ctx.buf("err_flag", 4);
  fill_i32(g.task_rc, nT, 0, s);
  fill_i32(g.task_kmin, nT, INT_MAX, s);
  fill_i32(g.task_kmax, nT, INT_MIN, s);
  fill_i32(g.err_flag, 1, 0, s);

  cudaEvent_t gs, ge;
  ck(cudaEventCreate(&gs), "event");
  ck(cudaEventCreate(&ge), "event");
  ck(cudaEventRecord(gs, s), "event");
  ctx.timing.setup_ms += now_ms() - t_enter;
  ctx.timing.kernel_launches += 6;  // fills

  // FAST precision: the k = all S-map accumulates its normal equations in
  // double-float arithmetic from a per-row table of products
  const float2* gram_terms = nullptr;
  if (ctx.precision == FEDM_PRECISION_FAST && any_all && o.algorithm == 1 && Ea <= 8 && !o.has_missing &&
      !o.low_memory && o.distance == 1) {
    const long long pool = lib_total;
    const long long bytes = pool * gram_terms_per_row(Ea) * (long long)sizeof(float2);
    if (pool > 0 && bytes <= (2LL << 30)) {
      float2* P = (float2*)ctx.buf("gram_terms", (size_t)bytes);
      int* bad = (int*)ctx.buf("gram_bad", 4);
      fill_i32(bad, 1, 0, s);
      launch_gram_terms(g, pool, P, bad, s);
      ctx.check("gram terms");
      int hbad = 0;
      ctx.download(&hbad, bad, 4);
      ck(cudaStreamSynchronize(s), "sync");
      if (!hbad)
        gram_terms = P;
      ctx.timing.kernel_launches += 2;
    }
  }

  // FAST precision on the tensor cores: the product slices of every
  // all-mode task's library, once per batch
  GramTC tc{};
  std::vector<GramTask> gt_tasks;
  std::vector<int> gt_of;  // kernel task -> its GramTask (-1: none)
  if (gram_terms && ctx.gram_tc && gram_tc_supported(Ea)) {
    bool fits = true;
    gt_of.assign(nK, -1);
    long long blocks = 0;
    int max_lib = 0;
    for (int j = 0; j < nK; j++)
      if (dk[j].all_mode) {
        if (dk[j].n_lib > 30000)
          fits = false;  // the int64 sums stay exact below ~32 000 rows
        GramTask t{};
        t.lib_off = dk[j].lib_off;
        t.n_lib = dk[j].n_lib;
        t.n_blocks = (dk[j].n_lib + gram_tc_block_rows() - 1) / gram_tc_block_rows();
        t.b_off = (int)blocks;
        blocks += t.n_blocks;
        max_lib = std::max(max_lib, dk[j].n_lib);
        gt_of[j] = (int)gt_tasks.size();
        gt_tasks.push_back(t);
      }
    if (fits && !gt_tasks.empty() && blocks > 0) {
      const int nA = (int)gt_tasks.size();
      tc.tasks = (const GramTask*)ctx.buf("gt_tasks", gt_tasks.size() * sizeof(GramTask));
      tc.colmax = (unsigned long long*)ctx.buf("gt_colmax", (size_t)nA * gram_tc_columns() * 8);
      tc.bslices = (unsigned char*)ctx.buf("gt_slices", (size_t)blocks * gram_tc_block_bytes());
      tc.error = (int*)ctx.buf("gt_error", 4);
      ctx.upload((void*)tc.tasks, gt_tasks.data(), gt_tasks.size() * sizeof(GramTask));
      ck(cudaMemsetAsync(tc.colmax, 0, (size_t)nA * gram_tc_columns() * 8, s), "memset");
      fill_i32(tc.error, 1, 0, s);
      launch_gram_tc_slices(g, tc, nA, max_lib, s);
      ctx.check("gram slices");
      ctx.timing.kernel_launches += 3;
    } else {
      gt_tasks.clear();
    }
  }

  // chunking: neighbour lists, statuses and the all-mode Gram buffer
  const long long budget = 2LL << 30;
  long long per_point = (long long)kcap * 12 + 8;
  if (any_all)
    per_point += max_nlib_all * 8;  // the point's distances
  if (any_all && o.algorithm == 1)
    per_point += (long long)nth * all_mode_slab(Ea) * 8;
  long long chunk = std::max<long long>(1, std::min<long long>(std::max<long long>(P, 1), budget / per_point));
  ChunkBuffers c{};
  c.kcap = kcap;
  c.nn_idx = (int*)ctx.buf("nn_idx", (size_t)chunk * kcap * 4);
  c.nn_dist = (double*)ctx.buf("nn_dist", (size_t)chunk * kcap * 8);
  c.nn_count = (int*)ctx.buf("nn_count", (size_t)chunk * 4);
  c.status = (int*)ctx.buf("status", (size_t)chunk * 4);
  if (any_all && o.algorithm == 1)
    c.gram = (double*)ctx.buf("gram", (size_t)chunk * nth * all_mode_slab(Ea) * 8);
  long long scratch = 1;
  if (any_all)
    scratch = std::max(scratch, chunk * max_nlib_all);
  if ((any_finite || any_mixed) && o.algorithm == 1)
    scratch = std::max(scratch, smap_nn_scratch_doubles(ctx.num_sms, n, kcap));
  c.scratch = (double*)ctx.buf("scratch", (size_t)scratch * 8);
  c.scratch_doubles = scratch;

  // detail mode: per-point neighbour lists gathered from every path
  std::vector<std::vector<int>> pt_idx;
  std::vector<std::vector<double>> pt_dist;
  if (job.detail) {
    pt_idx.resize(P);
    pt_dist.resize(P);
  }
  std::vector<int> h_cnt, h_idx, h_status;
  std::vector<double> h_dist;
  std::vector<long long> h_plist;
  auto gather_detail = [&](long long cl) {
    h_cnt.resize(cl);
    h_status.resize(cl);
    h_idx.resize((size_t)cl * kcap);
    h_dist.resize((size_t)cl * kcap);
    ctx.download(h_cnt.data(), c.nn_count, cl * 4);
    ctx.download(h_status.data(), c.status, cl * 4);
    ctx.download(h_idx.data(), c.nn_idx, (size_t)cl * kcap * 4);
    ctx.download(h_dist.data(), c.nn_dist, (size_t)cl * kcap * 8);
    ck(cudaStreamSynchronize(s), "sync");
    for (long long q = 0; q < cl; q++) {
      const long long p = c.plist ? h_plist[q] : c.p_begin + q;
      if (h_status[q] != PT_OK)
        continue;
      pt_idx[p].assign(h_idx.begin() + q * kcap, h_idx.begin() + q * kcap + h_cnt[q]);
      pt_dist[p].assign(h_dist.begin() + q * kcap, h_dist.begin() + q * kcap + h_cnt[q]);
      for (int& v : pt_idx[p])
        v = task_pos(p, v);
    }
  };

  cudaEvent_t e0, e1, f0, f1;
  ck(cudaEventCreate(&e0), "event");
  ck(cudaEventCreate(&e1), "event");
  ck(cudaEventCreate(&f0), "event");
  ck(cudaEventCreate(&f1), "event");
  float knn_ms = 0;
  auto timed = [&](auto&& launch) {
    ck(cudaEventRecord(e0, s), "event");
    launch();
    ck(cudaEventRecord(e1, s), "event");
    ctx.check("neighbour kernel");
    ck(cudaEventSynchronize(e1), "sync");
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    knn_ms += ms;
    ctx.timing.knn_launches++;
  };
  auto exact_pass = [&](bool with_list_path, bool with_all, const RefineRun* refine = nullptr) {
    ctx.timing.kernel_launches += 1;  // status fill
    if (with_list_path) {
      if (refine) {
        // uncertified mixed points: the rows under their bound, then the
        // exact search for the points that bound does not settle
        timed([&] {
          launch_knn_refine(g, c, *refine, ctx.num_sms, s);
          c.redo_only = 1;
          launch_knn_exact(g, c, ctx.num_sms, s);
          c.redo_only = 0;
        });
        ctx.timing.kernel_launches += 1;
      } else {
        timed([&] { launch_knn_exact(g, c, ctx.num_sms, s); });
      }
      if (o.algorithm == 0)
        launch_simplex_nn(g, c, s);
      else
        launch_smap_nn(g, c, ctx.num_sms, s);
      ctx.check("forecast");
      ctx.timing.kernel_launches += 1;
    }
    if (with_all) {
      float* rdist = nullptr;
      double* means = nullptr;
      float* dmin = nullptr;
      int tiles = 0;
      if (gram_terms) {
        rdist = (float*)ctx.buf("df_rdist", (size_t)(c.p_end - c.p_begin) * max_nlib_all * 4);
        means = (double*)ctx.buf("df_means", (size_t)(c.p_end - c.p_begin) * 8);
      }
      if (!gt_tasks.empty()) {
        // the chunk's rows ((point, theta), theta fastest) of every all-mode
        // task, in tiles of 128
        const long long cl = c.p_end - c.p_begin;
        std::vector<GramTile> tl;
        for (int j = 0; j < nK; j++) {
          if (gt_of[j] < 0)
            continue;
          const long long a = std::max(dk[j].point_base, c.p_begin);
          const long long b = std::min(dk[j].point_base + dk[j].n_pred, c.p_end);
          GramTask& t = gt_tasks[gt_of[j]];
          t.q0 = (int)(a - c.p_begin);
          if (b <= a)
            continue;
          const long long rows = (b - a) * nth;
          for (long long r = 0; r < rows; r += gram_tc_tile_rows())
            tl.push_back(GramTile{ gt_of[j], (int)r, (int)std::min<long long>(gram_tc_tile_rows(), rows - r) });
        }
        tiles = (int)tl.size();
        ctx.timing.tensor_core_tiles += tiles;
        ctx.upload((void*)tc.tasks, gt_tasks.data(), gt_tasks.size() * sizeof(GramTask));
        tc.tiles = (const GramTile*)ctx.buf("gt_tiles", std::max<size_t>(tl.size(), 1) * sizeof(GramTile));
        ctx.upload((void*)tc.tiles, tl.data(), tl.size() * sizeof(GramTile));
        dmin = (float*)ctx.buf("df_dmin", (size_t)cl * 4);
        tc.rdist = rdist;
        tc.dmin = dmin;
        tc.means = means;
        tc.thetas = g.thetas;
        tc.n_thetas = nth;
        tc.max_nlib = max_nlib_all;
        tc.np = n * (n + 1) / 2 + n;
        tc.G = (double*)ctx.buf("gt_G", (size_t)cl * nth * gram_tc_columns() * 8);
      }
      launch_all_mode(g, c, ctx.num_sms, max_nlib_all, s, gram_terms, rdist, means, f0, f1, tiles ? &tc : nullptr,
                      tiles, dmin);
      ctx.check("all_mode");
      ck(cudaEventSynchronize(f1), "sync");
      float ms = 0;
      cudaEventElapsedTime(&ms, f0, f1);
      ctx.timing.forecast_kernel_ms += ms;
      ctx.timing.forecast_launches += 1;
      ctx.timing.kernel_launches += o.algorithm == 1 ? (gram_terms ? (tiles ? 4 : 3) : (Ea <= 8 ? 3 : 2)) : 1;
    }
  };

  // 1. mixed-precision kernel for the tasks it serves
  if (any_mixed) {
    const bool wide = Ea > 8;
    const int S = Ea <= 4 ? 4 : (Ea <= 8 ? 8 : 16);
    const int C = wide ? 32 : (kmix <= 6 ? 8 : 16);
    // one point per thread: for k <= 6 the default form (and the simplex's
    // when the S-map uses the warp-specialised kernel); for 7 <= k <= 14 the
    // MIXED_ONE16 form
    auto is_one = [&](int form) {
      if (wide)
        return false;
      if (C == 16)
        return form == MIXED_ONE16;
      const bool ws = o.algorithm == 1 && (form == MIXED_WS4 || form == MIXED_WS8);
      return form != MIXED_FUSED2 && form != MIXED_ONE16 && !ws;
    };
    // panels with a finite penalty: the one-point forms only
    const bool pen = o.panel_mode && o.idw > 0;
    // the split S-map serves E_a <= 4 with at most six neighbours
    const bool split_ok =
      o.algorithm == 1 && !wide && !pen && C == 8 && kmix <= SPLIT_SLOTS && Ea <= SPLIT_MAX_EA;
    auto points_per_item = [&](int form) { return (wide || is_one(form)) ? WIDE_POINTS : MIX_POINTS; };
    const long long nrows = (long long)rows.n_rows;
    double* d_center = (double*)ctx.buf("center", Ea * 8);
    ctx.upload(d_center, center.data(), Ea * 8);
    float* F32 = (float*)ctx.buf("F32", (size_t)nrows * S * 4);
    center_to_f32(job.dF, nrows, Ea, d_center, F32, S, s);
    float* Fp32 = F32;
    if (job.dFp != job.dF) {
      Fp32 = (float*)ctx.buf("Fp32", (size_t)nrows * S * 4);
      center_to_f32(job.dFp, nrows, Ea, d_center, Fp32, S, s);
    }
    std::vector<int> order;
    for (int j = 0; j < nK; j++)
      if (dk[j].mixed)
        order.push_back(j);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return dk[a].n_lib > dk[b].n_lib; });
    // interleaved: the largest, smallest, second largest, second smallest,
    // ... library, so that scan-heavy and solve-heavy items share the SMs;
    // per-panel sub-tasks keep decreasing size (all of them are
    // solve-heavy, and interleaving cost 3% of device time on 512
    // independent panels)
    if (ctx.item_order == 1 && !split && order.size() > 2) {
      std::vector<int> mix;
      mix.reserve(order.size());
      for (size_t lo = 0, hi = order.size(); lo < hi;) {
        mix.push_back(order[lo++]);
        if (lo < hi)
          mix.push_back(order[--hi]);
      }
      order.swap(mix);
    }
    // work items of the tasks in this order, up to the task that takes the
    // count of points past max_points
    auto items_of = [&](int per_item, long long max_points) {
      std::vector<int2> it;
      long long covered = 0;
      for (int j : order) {
        if (covered >= max_points)
          break;
        for (int b = 0; b < dk[j].n_pred; b += per_item)
          it.push_back(make_int2(j, b));
        covered += dk[j].n_pred;
      }
      return it;
    };
    long long mixed_points = 0;
    size_t max_items = 1;
    for (int j : order) {
      mixed_points += dk[j].n_pred;
      max_items += (dk[j].n_pred + WIDE_POINTS - 1) / WIDE_POINTS;
    }
    MixedRun m{};
    m.F32 = F32;
    m.Fp32 = Fp32;
    m.items = (const int2*)ctx.buf("items", max_items * sizeof(int2));  // 256-point items: the longest list
    // queue head, fallback count, FP64 operation count (8 B), hand-off
    // error, points left to the exact search by knn_refine_kernel
    m.counter = (int*)ctx.buf("mix_counter", 32);
    m.fb_count = m.counter + 1;
    m.fp64_ops = (unsigned long long*)(m.counter + 2);
    m.error = m.counter + 4;
    m.scanned = (unsigned long long*)(m.counter + 6);
    fill_i32(m.counter, 8, 0, s);
    m.form = ctx.mixed_form;
    m.fb_cap = (int)std::min<long long>(std::max<long long>(P, 1), FB_CAP);
    m.fb_list = (long long*)ctx.buf("fb_list", (size_t)m.fb_cap * 8);
    m.fb_thr = (double*)ctx.buf("fb_thr", (size_t)m.fb_cap * 8);
    m.gamma = (Ea + 2) * std::ldexp(1.0, -23);
    // input-rounding term of the certification (kernels_mixed.cu): twice the
    // proven 2u(1 + 2^-29) R
    m.err_abs = std::ldexp(R, -22) + 1e-21;
    if (job.detail) {
      m.nn_idx = (int*)ctx.buf("mix_nn_idx", (size_t)std::max<long long>(P, 1) * C * 4);
      m.nn_dist = (double*)ctx.buf("mix_nn_dist", (size_t)std::max<long long>(P, 1) * C * 8);
    }
    ctx.timing.kernel_launches += (job.dFp != job.dF ? 2 : 1) + 1;  // centring, counter fill
    if (d_scan) {
      // the lists' spatial orders, then the boxes of their sub-tiles from the
      // float manifold (inside the timed span)
      launch_spatial_order(d_lib, d_rank, scan_sh, scan_nb, d_lists, (int)scan_src.size(), d_scan, s);
      ctx.check("spatial_order_kernel");
      ctx.timing.kernel_launches += 1;
      int4* d_sub = (int4*)ctx.buf("subtiles", subtiles.size() * sizeof(int4));
      float2* d_boxes = (float2*)ctx.buf("boxes", subtiles.size() * Ea * sizeof(float2));
      ctx.upload(d_sub, subtiles.data(), subtiles.size() * sizeof(int4));
      launch_tile_boxes(d_lib, d_scan, F32, S, Ea, d_sub, (int)subtiles.size(), d_boxes, s);
      ctx.check("tile_box_kernel");
      ctx.timing.kernel_launches += 1;
      m.scan_pos = d_scan;
      m.boxes = d_boxes;
    }
    m.kslots = C;
    m.ctas_per_sm = ctx.ctas_per_sm;
    // The split S-map: the items in chunks; the scan of a chunk writes its
    // neighbour lists into one of three list buffers on the main stream,
    // and the solves of that chunk run on the second stream while the next
    // chunk is scanned.  A buffer is rescanned only after its solves are
    // done; the main stream waits for the last solve.
    constexpr int SPLIT_BUFS = 3;
    cudaEvent_t scan_ev[SPLIT_BUFS] = {}, solve_ev[SPLIT_BUFS] = {}, split_done = nullptr;
    auto split_pipeline = [&]() {
      const int ib0 = m.item_begin, ie0 = m.item_end;
      const long long items = ie0 - ib0;
      if (items <= 0)
        return;
      long long nchunks = std::max<long long>(4, (items * WIDE_POINTS + ctx.split_chunk_points - 1) /
                                                     ctx.split_chunk_points);
      nchunks = std::min(nchunks, items);
      const long long per_chunk = (items + nchunks - 1) / nchunks;
      const long long lslots = per_chunk * WIDE_POINTS;
      int* keff = (int*)ctx.buf("split_keff", (size_t)SPLIT_BUFS * lslots * 4);
      int* lrows = (int*)ctx.buf("split_rows", (size_t)SPLIT_BUFS * SPLIT_SLOTS * lslots * 4);
      double* ldist = (double*)ctx.buf("split_dist", (size_t)SPLIT_BUFS * SPLIT_SLOTS * lslots * 8);
      if (!split_done) {
        for (int b = 0; b < SPLIT_BUFS; b++) {
          ck(cudaEventCreateWithFlags(&scan_ev[b], cudaEventDisableTiming), "event");
          ck(cudaEventCreateWithFlags(&solve_ev[b], cudaEventDisableTiming), "event");
        }
        ck(cudaEventCreateWithFlags(&split_done, cudaEventDisableTiming), "event");
      }
      for (long long c = 0; c * per_chunk < items; c++) {
        const int b = (int)(c % SPLIT_BUFS);
        if (c >= SPLIT_BUFS)
          ck(cudaStreamWaitEvent(s, solve_ev[b], 0), "wait");
        MixedRun mc = m;
        mc.item_begin = (int)(ib0 + c * per_chunk);
        mc.item_end = (int)std::min<long long>(ie0, ib0 + (c + 1) * per_chunk);
        mc.l_keff = keff + b * lslots;
        mc.l_rows = lrows + (size_t)b * SPLIT_SLOTS * lslots;
        mc.l_dist = ldist + (size_t)b * SPLIT_SLOTS * lslots;
        mc.l_slots = lslots;
        mc.ctas_per_sm = ctx.ctas_per_sm > 0 ? std::min(ctx.ctas_per_sm, ctx.split_scan_ctas) : ctx.split_scan_ctas;
        ck(cudaMemsetAsync(m.counter, 0, 4, s), "memset");  // the queue head
        launch_smap_scan_lists(g, mc, ctx.num_sms, s);
        ck(cudaEventRecord(scan_ev[b], s), "event");
        ck(cudaStreamWaitEvent(ctx.stream2, scan_ev[b], 0), "wait");
        const SolveRun r{ m.items, mc.item_begin, mc.item_end, mc.l_keff, mc.l_rows, mc.l_dist, lslots, m.fp64_ops };
        launch_smap_lists(g, r, ctx.num_sms, ctx.split_solve_ctas, ctx.stream2);
        ck(cudaEventRecord(solve_ev[b], ctx.stream2), "event");
        ctx.timing.kernel_launches += 2;
      }
      ck(cudaEventRecord(split_done, ctx.stream2), "event");
      ck(cudaStreamWaitEvent(s, split_done, 0), "wait");
    };
    auto launch_form = [&](int form) {
      m.form = form;
      if (pen)
        launch_mixed_pen(g, m, C, ctx.num_sms, s);
      else if (wide)
        launch_knn_wide(g, m, ctx.num_sms, s);
      else if (form == MIXED_SPLIT && split_ok)
        split_pipeline();
      else if (is_one(form) && C == 16)
        launch_mixed_one16(g, m, ctx.num_sms, s);
      else if (is_one(form))
        launch_mixed_one(g, m, ctx.num_sms, s);
      else
        launch_knn_mixed(g, m, C, ctx.num_sms, s);
    };
    auto run_items = [&](const std::vector<int2>& it) {
      ctx.upload((void*)m.items, it.data(), it.size() * sizeof(int2));
      m.n_items = (int)it.size();
      m.item_begin = 0;
      m.item_end = m.n_items;
    };
    int form = C == 16 ? ctx.mixed_form16 : ctx.mixed_form;
    if (pen)
      form = C == 16 ? MIXED_ONE16 : MIXED_ONE6;
    if (!wide && !pen && ctx.autotune) {
      // Autotuner: every form gives the same bits, so the first batch of
      // each (algorithm, E_a, k) with enough points times each candidate
      // form on the same leading tasks (about two waves of the default
      // form) and the context keeps the fastest.  Each candidate first runs
      // once on one work item, untimed, so that module loading and the
      // clock ramp of a first launch fall outside the timing; then two
      // rounds in alternating order, the minimum per candidate.  The probes
      // write the values the real run writes again; the counters are reset
      // after.
      const std::array<int, 3> key{ o.algorithm, Ea, kmix };
      auto hit = ctx.tuned_forms.find(key);
      const long long probe_points = 2LL * ctx.num_sms * 6 * WIDE_POINTS;
      if (hit != ctx.tuned_forms.end()) {
        form = hit->second;
      } else if (mixed_points >= probe_points) {
        std::vector<int> cands{ MIXED_ONE6, MIXED_FUSED2 };
        if (C == 16)
          cands = { MIXED_ONE16, MIXED_FUSED2 };
        else if (o.algorithm == 1)
          cands.push_back(MIXED_WS8);

        std::vector<float> best(cands.size(), INFINITY);
        for (int f : cands) {
          fill_i32(m.counter, 8, 0, s);
          std::vector<int2> one_item = items_of(points_per_item(f), 1);
          one_item.resize(1);
          run_items(one_item);
          launch_form(f);
          ctx.timing.kernel_launches += 2;
        }
        cudaEvent_t p0, p1;
        ck(cudaEventCreate(&p0), "event");
        ck(cudaEventCreate(&p1), "event");
        for (int round = 0; round < 2; round++)
          for (size_t c = 0; c < cands.size(); c++) {
            const size_t ci = round == 0 ? c : cands.size() - 1 - c;
            const int f = cands[ci];
            fill_i32(m.counter, 8, 0, s);
            run_items(items_of(points_per_item(f), probe_points));
            ck(cudaEventRecord(p0, s), "event");
            launch_form(f);
            ck(cudaEventRecord(p1, s), "event");
            ctx.check("autotune probe");
            ck(cudaEventSynchronize(p1), "sync");
            int herr = 0;
            ctx.download(&herr, m.error, 4);
            ck(cudaStreamSynchronize(s), "sync");
            float ms = 0;
            cudaEventElapsedTime(&ms, p0, p1);
            if (!herr)
              best[ci] = std::min(best[ci], ms);
            ctx.timing.autotune_probes++;
            ctx.timing.kernel_launches += 2;
          }
        cudaEventDestroy(p0);
        cudaEventDestroy(p1);
        size_t bi = 0;  // ties keep the earlier candidate
        for (size_t c = 1; c < cands.size(); c++)
          if (best[c] < best[bi])
            bi = c;
        if (best[bi] < INFINITY)
          form = cands[bi];
        fill_i32(m.counter, 8, 0, s);
        ctx.tuned_forms[key] = form;
      }
    }
    if (form == MIXED_SPLIT && !split_ok)
      form = MIXED_ONE6;  // a context fixed to the split form, on a shape it does not serve
    if (wide)
      ctx.timing.mixed_form = MIXED_WIDE;
    else if (form == MIXED_SPLIT)
      ctx.timing.mixed_form = MIXED_SPLIT;
    else if (is_one(form))
      ctx.timing.mixed_form = C == 16 ? MIXED_ONE16 : MIXED_ONE6;
    else
      ctx.timing.mixed_form = (o.algorithm == 1 && (form == MIXED_WS4 || form == MIXED_WS8)) ? form : MIXED_FUSED2;
    run_items(items_of(points_per_item(form), LLONG_MAX));
    timed([&] { launch_form(form); });
    int nfb = 0, herr = 0;
    unsigned long long nops = 0;
    ctx.download(&nfb, m.fb_count, 4);
    unsigned long long nscan = 0;
    ctx.download(&nops, m.fp64_ops, 8);
    ctx.download(&nscan, m.scanned, 8);
    ctx.download(&herr, m.error, 4);
    ck(cudaStreamSynchronize(s), "sync");
    if (herr)
      throw Error{ RC_UNKNOWN_ERROR, "mixed S-map kernel: scan/solve hand-off timed out" };
    ctx.timing.fallback_points += nfb;
    ctx.timing.fp64_ops += (long long)nops;
    ctx.timing.scanned_pairs += (long long)nscan;
    if (split_done) {
      for (int b = 0; b < SPLIT_BUFS; b++) {
        cudaEventDestroy(scan_ev[b]);
        cudaEventDestroy(solve_ev[b]);
      }
      cudaEventDestroy(split_done);
    }
    if (job.detail) {
      std::vector<int> ku(P), mi((size_t)P * C);
      std::vector<double> md((size_t)P * C);
      ctx.download(ku.data(), g.kused, P * 4);
      ctx.download(mi.data(), m.nn_idx, (size_t)P * C * 4);
      ctx.download(md.data(), m.nn_dist, (size_t)P * C * 8);
      ck(cudaStreamSynchronize(s), "sync");
      for (int j = 0; j < nK; j++)
        if (dk[j].mixed)
          for (long long p = dk[j].point_base; p < dk[j].point_base + dk[j].n_pred; p++)
            if (ku[p] != MISSING_I) {
              pt_idx[p].assign(mi.begin() + p * C, mi.begin() + p * C + ku[p]);
              pt_dist[p].assign(md.begin() + p * C, md.begin() + p * C + ku[p]);
              if (kt[j].pos)
                for (int& v : pt_idx[p])
                  v = (*kt[j].pos)[v];
            }
    }
    if (nfb > m.fb_cap) {
      // too many uncertified points: run every mixed task exactly
      for (auto& d : dk)
        d.mixed = 0;
      ctx.upload(d_tasks, dk.data(), dk.size() * sizeof(DevTask));
      fill_f64(g.pred, P * nth, MISSING_D, s);
      if (g.coeffs)
        fill_f64(g.coeffs, P * n, MISSING_D, s);
      if (g.kused)
        fill_i32(g.kused, P, MISSING_I, s);
      fill_i32(g.task_rc, nT, 0, s);
      fill_i32(g.task_kmin, nT, INT_MAX, s);
      fill_i32(g.task_kmax, nT, INT_MIN, s);
      for (auto& v : pt_idx)
        v.clear();
      for (auto& v : pt_dist)
        v.clear();
      any_finite = true;
    } else if (nfb > 0) {
      h_plist.resize(nfb);
      std::vector<double> h_thr(nfb);
      ctx.download(h_plist.data(), m.fb_list, (size_t)nfb * 8);
      ctx.download(h_thr.data(), m.fb_thr, (size_t)nfb * 8);
      ck(cudaStreamSynchronize(s), "sync");
      // in point order, so that consecutive points share a task and
      // knn_refine_kernel's CTAs can stage each library tile once for all
      // their points
      {
        std::vector<int> ord(nfb);
        std::iota(ord.begin(), ord.end(), 0);
        std::sort(ord.begin(), ord.end(), [&](int u, int v) { return h_plist[u] < h_plist[v]; });
        std::vector<long long> sp(nfb);
        std::vector<double> st(nfb);
        for (int q = 0; q < nfb; q++) {
          sp[q] = h_plist[ord[q]];
          st[q] = h_thr[ord[q]];
        }
        h_plist.swap(sp);
        ctx.upload(m.fb_list, h_plist.data(), (size_t)nfb * 8);
        ctx.upload(m.fb_thr, st.data(), (size_t)nfb * 8);
        ck(cudaStreamSynchronize(s), "sync");
      }
      for (long long b = 0; b < nfb; b += chunk) {
        c.p_begin = 0;
        c.p_end = std::min<long long>(nfb - b, chunk);
        c.plist = m.fb_list + b;
        fill_i32(c.status, c.p_end, PT_SKIP, s);
        const RefineRun rr{ F32, Fp32, S, m.fb_thr + b, m.counter + 5 };
        exact_pass(true, false, &rr);
        if (job.detail) {
          std::vector<long long> keep(h_plist.begin() + b, h_plist.begin() + b + c.p_end);
          std::swap(keep, h_plist);
          gather_detail(c.p_end);
          std::swap(keep, h_plist);
        }
      }
      c.plist = nullptr;
      int nredo = 0;
      ctx.download(&nredo, m.counter + 5, 4);
      ck(cudaStreamSynchronize(s), "sync");
      ctx.timing.exact_points += nredo;
    }
  }

  // 2. exact kernels over the point space for the other tasks
  if (any_finite || any_all) {
    for (long long b = 0; b < P; b += chunk) {
      if (ctx.keep_going && !ctx.keep_going())
        throw Error{ RC_BREAK_HIT, "cancelled" };
      c.p_begin = b;
      c.p_end = std::min(P, b + chunk);
      c.plist = nullptr;
      const long long cl = c.p_end - c.p_begin;
      fill_i32(c.status, cl, PT_SKIP, s);
      exact_pass(any_finite, any_all);
      if (job.detail && any_finite)
        gather_detail(cl);
    }
  }
  ctx.timing.knn_kernel_ms += knn_ms;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(f0);
  cudaEventDestroy(f1);

  // statistics
  double* d_rho = (double*)ctx.buf("rho", (size_t)nT * nth * 8);
  double* d_mae = (double*)ctx.buf("mae", (size_t)nT * nth * 8);
  GroupParams gt = g;  // per task, not per kernel task
  gt.tasks = d_ptasks;
  gt.n_tasks = nT;
  launch_stats(gt, nullptr, nT, d_rho, d_mae, s);
  ctx.check("stats");
  ctx.timing.kernel_launches += 1;
  ck(cudaEventRecord(ge, s), "event");
  ck(cudaEventSynchronize(ge), "sync");
  {
    float ms = 0;
    cudaEventElapsedTime(&ms, gs, ge);
    ctx.timing.device_ms += ms;
  }
  cudaEventDestroy(gs);
  cudaEventDestroy(ge);
  const double t_fin = now_ms();
  std::vector<int> rc(nT), kmin(nT), kmax(nT);
  std::vector<double> rho((size_t)nT * nth), mae((size_t)nT * nth);
  int err = 0;
  ctx.download(rc.data(), g.task_rc, nT * 4);
  ctx.download(kmin.data(), g.task_kmin, nT * 4);
  ctx.download(kmax.data(), g.task_kmax, nT * 4);
  ctx.download(rho.data(), d_rho, rho.size() * 8);
  ctx.download(mae.data(), d_mae, mae.size() * 8);
  ctx.download(&err, g.err_flag, 4);
  ck(cudaStreamSynchronize(s), "sync");
  if (err)
    throw Error{ RC_UNKNOWN_ERROR, "panel weight missing for a compared pair of panels" };
  if (!gt_tasks.empty()) {
    int terr = 0;
    ctx.download(&terr, tc.error, 4);
    ck(cudaStreamSynchronize(s), "sync");
    if (terr)
      throw Error{ RC_UNKNOWN_ERROR, "tensor-core normal equations: a bounded wait ran out" };
  }
  for (int j = 0; j < nT; j++) {
    TaskOut& to = outs[job.task_ids[j]];
    const Task& t = tasks[job.task_ids[j]];
    to.rc = rc[j];
    to.kmin = kmin[j] == INT_MAX ? MISSING_I : kmin[j];
    to.kmax = kmax[j] == INT_MIN ? MISSING_I : kmax[j];
    to.rho.assign(rho.begin() + (size_t)j * nth, rho.begin() + (size_t)(j + 1) * nth);
    to.mae.assign(mae.begin() + (size_t)j * nth, mae.begin() + (size_t)(j + 1) * nth);
    const long long base = dt[j].point_base;
    const int np = dt[j].n_pred;
    if (t.save_prediction || job.detail) {
      to.pred_last.resize(np);
      ctx.download(to.pred_last.data(), g.pred + (size_t)(nth - 1) * P + base, (size_t)np * 8);
    }
    if (job.detail) {
      to.pred_all.resize((size_t)nth * np);
      for (int th = 0; th < nth; th++)
        ctx.download(to.pred_all.data() + (size_t)th * np, g.pred + (size_t)th * P + base, (size_t)np * 8);
      to.kused.resize(np);
      ctx.download(to.kused.data(), g.kused + base, (size_t)np * 4);
      to.nn_offsets.assign(np + 1, 0);
      for (int i = 0; i < np; i++) {
        const auto& li = pt_idx[base + i];
        const auto& ld = pt_dist[base + i];
        to.nn_idx.insert(to.nn_idx.end(), li.begin(), li.end());
        to.nn_dist.insert(to.nn_dist.end(), ld.begin(), ld.end());
        to.nn_offsets[i + 1] = (int)to.nn_idx.size();
      }
    }
    if ((t.save_coeffs || job.detail) && o.algorithm == 1 && g.coeffs) {
      to.coeffs.resize((size_t)np * n);
      ctx.download(to.coeffs.data(), g.coeffs + (size_t)base * n, (size_t)np * n * 8);
    } else if (t.save_coeffs || job.detail) {
      to.coeffs.assign((size_t)np * n, MISSING_D);
    }
  }
  ck(cudaStreamSynchronize(s), "sync");
  ctx.timing.finish_ms += now_ms() - t_fin;
}

double na(double v)
{
  return v != MISSING_D ? v : NAN;
}

// src/r.cpp:73-105 (column-major read of the buffer, NA where filtered)
std::vector<double> to_R_matrix(const std::vector<double>& v, int r, int c, const std::vector<uint8_t>& filter)
{
  std::vector<double> m((size_t)r * c, NAN);
  size_t k = 0;
  for (int j = 0; j < c; j++)
    for (int i = 0; i < r; i++) {
      if (!filter.empty() && !filter[i])
        continue;
      m[(size_t)j * r + i] = k < v.size() ? na(v[k]) : NAN;
      k++;
    }
  return m;
}

std::vector<int> rows_of(const std::vector<uint8_t>& mask)
{
  std::vector<int> r;
  for (int i = 0; i < (int)mask.size(); i++)
    if (mask[i])
      r.push_back(i);
  return r;
}

// Library manifold rows: the mask's rows whose target is observed
// (src/manifold.h:186-189).
std::vector<int> lib_rows_of(const std::vector<uint8_t>& mask, const RowTables& rt)
{
  std::vector<int> r;
  for (int i = 0; i < (int)mask.size(); i++)
    if (mask[i] && rt.lib_target[i] != MISSING_D)
      r.push_back(i);
  return r;
}

// The manifolds of one call, per (E, coprediction): on the device, and
// their host copies (row-major [n x Ea]).
struct Manifolds
{
  std::map<std::pair<int, bool>, const double*> host;
  std::map<std::pair<int, bool>, std::vector<double>> host_store;  // host-built copies
  std::map<std::pair<int, bool>, double*> dev;
  // the series on the device for manifold_kernel, uploaded at the first build
  bool series = false;
  double *x = nullptr, *co_x = nullptr, *extras = nullptr;
  int *obs = nullptr, *target_row = nullptr;
};

template<class T>
bool same_bits(const std::vector<T>& a, const std::vector<T>& b)
{
  return a.size() == b.size() && (a.empty() || std::memcmp(a.data(), b.data(), a.size() * sizeof(T)) == 0);
}

// Checks the context's record of the series behind its manifold buffers
// against this call's manifold inputs (every array and setting that
// manifold_kernel and the host build read), bit for bit.  When they differ
// the record takes this call's inputs and forgets its manifolds.
void sync_series(Context& ctx, const Generator& g, const RowTables& rt)
{
  auto& c = ctx.series;
  if (!ctx.series_cache || ctx.host_manifold) {
    c = Context::SeriesCache{};
    ctx.series_gen++;
    ctx.spatial_ranks.clear();
    return;
  }
  std::vector<double> scalars = { (double)g.n, (double)g.tau, g.dt ? 1.0 : 0.0, g.reldt ? 1.0 : 0.0, g.dt_weight,
                                  (double)g.num_extras, (double)g.num_extras_lagged, g.panel_mode ? 1.0 : 0.0 };
  std::vector<double> extras;
  for (const auto& e : g.extras)
    extras.insert(extras.end(), e.begin(), e.end());
  static const std::vector<int> none;
  const std::vector<int>& panel = g.panel_mode ? g.panel : none;
  if (c.valid && same_bits(c.scalars, scalars) && same_bits(c.x, g.x) && same_bits(c.co_x, g.co_x) &&
      same_bits(c.extras, extras) && same_bits(c.point_time, rt.point_time) && same_bits(c.obs, g.obs) &&
      same_bits(c.target_row, rt.target_row) && same_bits(c.panel, panel))
    return;
  ctx.series_gen++;
  ctx.spatial_ranks.clear();
  c.valid = true;
  c.scalars = std::move(scalars);
  c.x = g.x;
  c.co_x = g.co_x;
  c.extras = std::move(extras);
  c.point_time = rt.point_time;
  c.obs = g.obs;
  c.target_row = rt.target_row;
  c.panel = panel;
  c.uploaded = false;
  c.built.clear();
}

// The manifold for E (co: of co_x) on the device, built once per call.  By
// default manifold_kernel builds it from the series and the host copy comes
// back into a pinned buffer of the context; FEDM_HOST_MANIFOLD=1 builds it
// on host threads and uploads it.  Both give the same bits.
double* device_manifold(Context& ctx, Manifolds& M, const Generator& g, const RowTables& rt, const DevRows& rows, int E,
                        bool co, int threads)
{
  auto key = std::make_pair(E, co);
  auto it = M.dev.find(key);
  if (it != M.dev.end())
    return it->second;
  const double t0 = now_ms();
  const int Ea = g.E_actual(E);
  const size_t count = (size_t)g.n * Ea;
  const std::string name = "F_" + std::to_string(E) + (co ? "_co" : "");
  double* d = (double*)ctx.buf(name, std::max<size_t>(count, 1) * 8);
  if (ctx.series.valid && ctx.series.built.count(key)) {
    // built by an earlier call on the same series: the buffers still hold
    // it (only this function writes them, and the same size never
    // reallocates)
    M.host[key] = (const double*)ctx.host_buf("host_" + name, std::max<size_t>(count, 1) * 8);
    M.dev[key] = d;
    ctx.timing.manifolds_reused += 1;
    ctx.timing.manifold_ms += now_ms() - t0;
    return d;
  }
  ctx.timing.manifold_builds += 1;
  if (ctx.host_manifold) {
    auto& h = M.host_store[key];
    h = build_manifold(g, rt, E, co, threads);
    ctx.upload(d, h.data(), h.size() * 8);
    M.host[key] = h.data();
  } else {
    const size_t n = (size_t)g.n;
    if (!M.series) {
      // uploaded once per series: a call on the series the buffers hold
      // (ctx.series) skips the copies
      const bool have = ctx.series.valid && ctx.series.uploaded;
      M.x = (double*)ctx.buf("series_x", n * 8);
      if (!have)
        ctx.upload(M.x, g.x.data(), n * 8);
      if (!g.co_x.empty()) {
        M.co_x = (double*)ctx.buf("series_co_x", n * 8);
        if (!have)
          ctx.upload(M.co_x, g.co_x.data(), n * 8);
      }
      if (g.num_extras > 0) {
        M.extras = (double*)ctx.buf("series_extras", (size_t)g.num_extras * n * 8);
        for (int e = 0; e < g.num_extras && !have; e++)
          ctx.upload(M.extras + (size_t)e * n, g.extras[e].data(), n * 8);
      }
      M.obs = (int*)ctx.buf("series_obs", n * 4);
      M.target_row = (int*)ctx.buf("series_target_row", n * 4);
      if (!have) {
        ctx.upload(M.obs, g.obs.data(), n * 4);
        ctx.upload(M.target_row, rt.target_row.data(), n * 4);
      }
      ctx.series.uploaded = ctx.series.valid;
      M.series = true;
    }
    ManifoldParams p{};
    p.t = rows.point_time;
    p.x = co ? M.co_x : M.x;
    p.extras = M.extras;
    p.panel = g.panel_mode ? rows.panel : nullptr;
    p.obs = M.obs;
    p.target_row = M.target_row;
    p.n = g.n;
    p.E = E;
    p.Edt = g.E_dt(E);
    p.Ea = Ea;
    p.tau = g.tau;
    p.num_extras = g.num_extras;
    p.num_extras_lagged = g.num_extras_lagged;
    p.with_dt = (g.dt || g.reldt) ? 1 : 0;
    p.reldt = g.reldt ? 1 : 0;
    p.w = g.dt_weight;
    launch_manifold(p, d, ctx.num_sms, ctx.stream);
    ctx.check("manifold_kernel");
    ctx.timing.kernel_launches += 1;
    double* h = (double*)ctx.host_buf("host_" + name, std::max<size_t>(count, 1) * 8);
    ctx.download(h, d, count * 8);
    ck(cudaStreamSynchronize(ctx.stream), "manifold download");
    M.host[key] = h;
    if (ctx.series.valid)
      ctx.series.built.insert(key);
  }
  M.dev[key] = d;
  ctx.timing.manifold_ms += now_ms() - t0;
  return d;
}

} // namespace

// ------------------------------------------------------------ run_command
CommandResult run_command(Context& ctx, const fedm_args& a)
{
  CommandResult R;
  const double t0 = now_ms();
  ctx.reset_timing();
  ck(cudaSetDevice(ctx.device), "cudaSetDevice");
  Prepared P;
  prepare(a, P);
  const Generator& gen = P.gen;
  const Options& o = P.opts;
  const int threads = host_threads(a);
  const int maxE = P.Es.back();
  std::vector<uint8_t> usable = gen.usable(maxE, false, threads);
  const int numUsable = (int)std::count(usable.begin(), usable.end(), (uint8_t)1);
  if (numUsable == 0) {
    R.rc = RC_UNKNOWN_ERROR;  // src/r.cpp:259-266
    return R;
  }
  std::vector<int> libraries = P.libraries;
  if (!P.explore && libraries.empty())
    libraries = { numUsable };
  const bool copredict_mode = !gen.co_x.empty();
  std::vector<uint8_t> cousable;
  if (copredict_mode)
    cousable = gen.usable(maxE, true, threads);
  RowTables rt = build_row_tables(gen);
  sync_series(ctx, gen, rt);
  // CCM library splits are left lazy: a SplitProducer computes their row
  // lists on background threads while the GPU runs earlier task batches
  TaskPlan plan = configure_tasks(gen, o, P.Es, libraries, a.k, a.num_reps, a.crossfold, P.explore, a.full,
                                  a.shuffle, a.save_predictions, a.save_copredictions, a.save_smap_coeffs,
                                  copredict_mode, usable, cousable, a.seed, &rt.lib_target, threads, true);
  std::unique_ptr<SplitProducer> producer;
  if (plan.lazy.active)
    producer = std::make_unique<SplitProducer>(plan, rt.lib_target, threads);
  DevRows drows = upload_rows(ctx, gen, rt, o);
  ctx.timing.prep_ms += now_ms() - t0;

  // row lists per mask (shared by every task that uses the mask); lazy
  // library lists are taken when their batch runs
  std::vector<std::vector<int>> lib_lists(plan.masks.size()), pred_lists(plan.masks.size());
  std::vector<uint8_t> lib_done(plan.masks.size(), 0), pred_done(plan.masks.size(), 0);
  auto take_lib_list = [&](int mask) {
    if (lib_done[mask])
      return;
    if (producer) {
      const double tw = now_ms();
      producer->wait(mask);
      ctx.timing.list_wait_ms += now_ms() - tw;
    }
    if (!plan.lists_ready.empty() && plan.lists_ready[mask])
      lib_lists[mask].swap(plan.lib_lists[mask]);
    else
      lib_lists[mask] = lib_rows_of(plan.masks[mask], rt);
    lib_done[mask] = 1;
  };
  for (const Task& t : plan.tasks) {
    if (!producer)
      take_lib_list(t.lib_mask);
    if (!pred_done[t.pred_mask]) {
      pred_lists[t.pred_mask] = rows_of(plan.masks[t.pred_mask]);
      pred_done[t.pred_mask] = 1;
    }
  }

  std::vector<TaskOut> outs(plan.tasks.size());
  Manifolds M;
  // groups: (E, copredict) in first-appearance order
  std::vector<std::pair<int, bool>> order;
  for (const Task& t : plan.tasks) {
    auto key = std::make_pair(t.E, t.copredict);
    if (std::find(order.begin(), order.end(), key) == order.end())
      order.push_back(key);
  }
  for (auto key : order) {
    GroupJob job;
    job.Ea = gen.E_actual(key.first);
    job.copredict = key.second;
    job.dF = device_manifold(ctx, M, gen, rt, drows, key.first, false, threads);
    job.dFp = key.second ? device_manifold(ctx, M, gen, rt, drows, key.first, true, threads) : job.dF;
    job.hF = M.host[std::make_pair(key.first, false)];
    job.hFp = key.second ? M.host[std::make_pair(key.first, true)] : job.hF;
    std::vector<int> ids;
    for (int i = 0; i < (int)plan.tasks.size(); i++)
      if (plan.tasks[i].E == key.first && plan.tasks[i].copredict == key.second)
        ids.push_back(i);
    if (producer)
      job.lib_superset = &plan.lazy.urows;
    // With lazy lists the group runs in task batches in plan order
    // (replicates outermost, so every batch spans all library sizes), each
    // waiting only for its own lists.  Batches double from LAZY_FIRST_BATCH
    // tasks: the GPU starts after a few splits, and the splitter, far faster
    // per task than the GPU, stays ahead.
    size_t per = producer ? LAZY_FIRST_BATCH : ids.size();
    for (size_t b0 = 0; b0 < ids.size(); b0 += per, per *= 2) {
      // src/edm.cpp:572-591: the caller may stop the run between batches
      if (ctx.keep_going && !ctx.keep_going())
        throw Error{ RC_BREAK_HIT, "cancelled" };
      job.task_ids.clear();
      job.lib_lists.clear();
      job.pred_lists.clear();
      for (size_t q = b0; q < std::min(ids.size(), b0 + per); q++) {
        const Task& t = plan.tasks[ids[q]];
        take_lib_list(t.lib_mask);
        job.task_ids.push_back(ids[q]);
        job.lib_lists.push_back(&lib_lists[t.lib_mask]);
        job.pred_lists.push_back(&pred_lists[t.pred_mask]);
      }
      run_group(ctx, o, plan.tasks, drows, job, outs);
    }
  }

  // src/r.cpp:348-457 marshalling, in task order
  int rc = 0, kMin = 0, kMax = 0;
  long long npred = 0, pairs = 0;
  for (size_t f = 0; f < plan.tasks.size(); f++) {
    const Task& t = plan.tasks[f];
    const TaskOut& to = outs[f];
    if (f == 0 || to.kmin < kMin)
      kMin = to.kmin;
    if (f == 0 || to.kmax > kMax)
      kMax = to.kmax;
    const int Ea = gen.E_actual(t.E);
    for (size_t th = 0; th < o.thetas.size(); th++) {
      if (!t.copredict) {
        R.sE.push_back(Ea);
        R.sL.push_back(t.library);
        R.sT.push_back(na(o.thetas[th]));
        R.sR.push_back(na(to.rho[th]));
        R.sM.push_back(na(to.mae[th]));
      } else {
        R.cE.push_back(Ea);
        R.cL.push_back(t.library);
        R.cT.push_back(na(o.thetas[th]));
        R.cR.push_back(na(to.rho[th]));
        R.cM.push_back(na(to.mae[th]));
      }
    }
    if (to.rc > rc)
      rc = to.rc;
    const std::vector<uint8_t>& pm = plan.masks[t.pred_mask];
    const int nrow = (int)pm.size();
    if (t.save_prediction) {
      // only the first of the numThetas columns the reference reads is
      // defined (src/r.cpp:394-399 reads past a one-theta buffer)
      auto m = to_R_matrix(to.pred_last, nrow, 1, pm);
      if (!t.copredict) {
        R.preds = m;
        R.pred_rows = nrow;
        R.pred_cols = 1;
      } else {
        R.copreds = m;
        R.copred_rows = nrow;
        R.copred_cols = 1;
      }
    }
    if (t.save_coeffs && !t.copredict) {
      R.coeffs = to_R_matrix(to.coeffs, nrow, Ea + 1, pm);
      R.coeff_rows = nrow;
      R.coeff_cols = Ea + 1;
    }
    if (a.save_manifolds) {
      // src/edm.cpp:473-475, src/r.cpp:406-409: the task's library manifold
      // (library rows whose target is observed) and prediction manifold
      // (co_x lags for coprediction), row-major, MISSING as NA
      auto append = [&](const double* F, const std::vector<int>& rows, std::vector<double>& out) {
        for (int r : rows)
          for (int j = 0; j < Ea; j++)
            out.push_back(na(F[(size_t)r * Ea + j]));
      };
      append(M.host[std::make_pair(t.E, false)], lib_lists[t.lib_mask], R.man);
      append(M.host[std::make_pair(t.E, t.copredict)], pred_lists[t.pred_mask], R.pman);
      R.man_rows.push_back((int)lib_lists[t.lib_mask].size());
      R.pman_rows.push_back((int)pred_lists[t.pred_mask].size());
      R.man_cols.push_back(Ea);
    }
    npred += (long long)pred_lists[t.pred_mask].size() * (long long)o.thetas.size();
    pairs += (long long)pred_lists[t.pred_mask].size() * (long long)lib_lists[t.lib_mask].size();
  }
  R.rc = rc;
  R.kmin = kMin;
  R.kmax = kMax;
  if (a.allow_missing) {
    R.has_missing_distance = true;
    R.missing_distance = o.missing_distance;
  }
  if (a.dt || a.reldt) {
    R.has_dt_weight = true;
    R.dt_weight = gen.dt_weight;
  }
  ctx.timing.host_ms = now_ms() - t0;
  ctx.timing.predictions = npred;
  ctx.timing.distance_pairs = pairs;
  return R;
}

// ------------------------------------------------------ differentiable S-map
int smap_grad(Context& ctx, const double* lib, const double* lib_t, int n_lib, const double* pred,
              const double* pred_t, int n_pred, int e_actual, double theta, const double* w, int objective,
              double* value, double* predictions, double* dtheta, double* dw)
{
  if (objective != 0 && objective != 1)
    throw Error{ RC_UNKNOWN_ERROR, "objective must be 0 (MSE) or 1 (rho)" };
  if (e_actual < 1 || e_actual > 8)
    throw Error{ RC_NOT_IMPLEMENTED, "differentiable S-map supports 1 <= E_actual <= 8" };
  if (n_lib < 1 || n_pred < 1)
    throw Error{ RC_UNKNOWN_ERROR, "empty library or prediction set" };
  ctx.reset_timing();
  const double t0 = now_ms();
  ck(cudaSetDevice(ctx.device), "cudaSetDevice");
  cudaStream_t s = ctx.stream;
  const size_t E = (size_t)e_actual;
  AdjointParams a{};
  double* d_lib = (double*)ctx.buf("adj_lib", (size_t)n_lib * E * 8);
  double* d_lt = (double*)ctx.buf("adj_lib_t", (size_t)n_lib * 8);
  double* d_pred = (double*)ctx.buf("adj_pred", (size_t)n_pred * E * 8);
  double* d_pt = (double*)ctx.buf("adj_pred_t", (size_t)n_pred * 8);
  double* d_w = (double*)ctx.buf("adj_w", E * 8);
  double* d_out = (double*)ctx.buf("adj_out", (size_t)n_pred * (E + 3) * 8);
  ctx.upload(d_lib, lib, (size_t)n_lib * E * 8);
  ctx.upload(d_lt, lib_t, (size_t)n_lib * 8);
  ctx.upload(d_pred, pred, (size_t)n_pred * E * 8);
  ctx.upload(d_pt, pred_t, (size_t)n_pred * 8);
  ctx.upload(d_w, w, E * 8);
  a.lib = d_lib;
  a.lib_t = d_lt;
  a.pred = d_pred;
  a.pred_t = d_pt;
  a.w = d_w;
  a.theta = theta;
  a.n_lib = n_lib;
  a.n_pred = n_pred;
  a.e_actual = e_actual;
  a.backward = dtheta != nullptr;
  a.out = d_out;
  a.z = (double*)ctx.buf("adj_z", (size_t)n_lib * E * 8);
  // per-warp slices for the per-row values of passes 1 and 2, within a
  // budget: the highest cache level for which a full persistent grid, or at
  // least half of one, fits; else none
  {
    constexpr size_t GRAD_CACHE_BUDGET = (size_t)8 << 30;
    const long long full = grad_cache_warps(e_actual, ctx.num_sms);
    for (int level = ctx.grad_cache_max; level >= 1 && !a.cache; level--) {
      const size_t per_row = level == 2 ? 3 + E : 2;
      const long long fit = (long long)(GRAD_CACHE_BUDGET / ((size_t)n_lib * per_row * 8));
      if (std::min(full, fit) * 2 >= full) {
        a.cache = (double*)ctx.try_buf("adj_cache", (size_t)std::min(full, fit) * per_row * n_lib * 8);
        if (a.cache) {
          a.cache_warps = std::min(full, fit);
          a.cache_level = level;
        }
      }
    }
  }
  cudaEvent_t e0, e1;
  ck(cudaEventCreate(&e0), "event");
  ck(cudaEventCreate(&e1), "event");
  ck(cudaEventRecord(e0, s), "event");
  launch_smap_grad(a, ctx.num_sms, s);
  ctx.check("smap_grad");
  ck(cudaEventRecord(e1, s), "event");
  std::vector<double> out((size_t)n_pred * (E + 3));
  ctx.download(out.data(), d_out, out.size() * 8);
  ck(cudaStreamSynchronize(s), "sync");
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  // fixed-order host reductions over prediction points; per point the
  // kernel gives r = yhat - target, yhat, dyhat/dtheta and dyhat/dw
  auto o = [&](int p) { return &out[(size_t)p * (E + 3)]; };
  if (predictions)
    for (int p = 0; p < n_pred; p++)
      predictions[p] = o(p)[1];
  // dvalue/dyhat_p for the chosen objective
  std::vector<double> dv(n_pred);
  if (objective == 0) {
    // MSE = mean r^2, dMSE/dyhat_p = 2 r_p / n
    double se = 0;
    for (int p = 0; p < n_pred; p++) {
      se += o(p)[0] * o(p)[0];
      dv[p] = 2 * o(p)[0] / n_pred;
    }
    *value = se / n_pred;
  } else {
    // rho as src/stats.cpp:64-80 computes it (centred sums; no value when
    // either series is constant), and
    // drho/dyhat_p = ((t_p - tbar) - (Sxy / Sxx)(yhat_p - ybar)) / sqrt(Sxx Syy)
    double ybar = 0, tbar = 0;
    for (int p = 0; p < n_pred; p++) {
      ybar += o(p)[1];
      tbar += pred_t[p];
    }
    ybar /= n_pred;
    tbar /= n_pred;
    double sxx = 0, syy = 0, sxy = 0;
    for (int p = 0; p < n_pred; p++) {
      const double a = o(p)[1] - ybar, b = pred_t[p] - tbar;
      sxx += a * a;
      syy += b * b;
      sxy += a * b;
    }
    const double sdx = std::sqrt(sxx), sdy = std::sqrt(syy);
    if (sdx < 1e-9 || sdy < 1e-9) {
      *value = NAN;
      std::fill(dv.begin(), dv.end(), NAN);
    } else {
      *value = sxy / (sdx * sdy);
      for (int p = 0; p < n_pred; p++)
        dv[p] = ((pred_t[p] - tbar) - (sxy / sxx) * (o(p)[1] - ybar)) / (sdx * sdy);
    }
  }
  if (dtheta) {
    double gt = 0;
    std::vector<double> gw(E, 0.0);
    for (int p = 0; p < n_pred; p++) {
      gt += dv[p] * o(p)[2];
      for (size_t j = 0; j < E; j++)
        gw[j] += dv[p] * o(p)[3 + j];
    }
    *dtheta = gt;
    for (size_t j = 0; j < E; j++)
      dw[j] = gw[j];
  }
  ctx.timing.device_ms = ms;
  ctx.timing.knn_kernel_ms = ms;
  ctx.timing.knn_launches = 1;
  ctx.timing.kernel_launches = 2;  // the scaled library, the passes
  ctx.timing.grad_cache_level = a.cache ? a.cache_level : 0;
  ctx.timing.distance_pairs = (long long)n_pred * n_lib * (a.cache ? 1 : dtheta ? 3 : 2);
  ctx.timing.predictions = n_pred;
  ctx.timing.host_ms = now_ms() - t0;
  return RC_SUCCESS;
}

// ------------------------------------------------------ host-only helpers
void host_usable(const fedm_args& a, int maxE, int copredict, unsigned char* out)
{
  Prepared P;
  prepare(a, P);
  auto u = P.gen.usable(maxE, copredict != 0, host_threads(a));
  std::copy(u.begin(), u.end(), out);
}

int host_manifold(const fedm_args& a, int E, int copredict, double* out)
{
  Prepared P;
  prepare(a, P);
  RowTables rt = build_row_tables(P.gen);
  if (out) {
    auto F = build_manifold(P.gen, rt, E, copredict != 0, host_threads(a));
    std::copy(F.begin(), F.end(), out);
  }
  return P.gen.E_actual(E);
}

int host_plan(const fedm_args& a, int max_tasks, int* task_E, int* task_k, int* task_library, int* task_copredict,
              unsigned char* lib_masks, unsigned char* pred_masks)
{
  Prepared P;
  prepare(a, P);
  const Generator& gen = P.gen;
  const int threads = host_threads(a);
  std::vector<uint8_t> usable = gen.usable(P.Es.back(), false, threads);
  const int numUsable = (int)std::count(usable.begin(), usable.end(), (uint8_t)1);
  std::vector<int> libraries = P.libraries;
  if (!P.explore && libraries.empty())
    libraries = { numUsable };
  const bool co = !gen.co_x.empty();
  std::vector<uint8_t> cousable;
  if (co)
    cousable = gen.usable(P.Es.back(), true, threads);
  // every row counts as having a target here, so the splitter's row lists
  // are exactly the membership masks; the lists come from the same lazy
  // SplitProducer that run_command uses
  std::vector<double> all_targets(gen.n, 0.0);
  TaskPlan plan = configure_tasks(gen, P.opts, P.Es, libraries, a.k, a.num_reps, a.crossfold, P.explore, a.full,
                                  a.shuffle, a.save_predictions, a.save_copredictions, a.save_smap_coeffs, co,
                                  usable, cousable, a.seed, &all_targets, threads, true);
  std::unique_ptr<SplitProducer> producer;
  if (plan.lazy.active && max_tasks > 0)
    producer = std::make_unique<SplitProducer>(plan, all_targets, threads);
  for (int i = 0; i < (int)plan.tasks.size() && i < max_tasks; i++) {
    const Task& t = plan.tasks[i];
    if (producer)
      producer->wait(t.lib_mask);
    task_E[i] = t.E;
    task_k[i] = t.k;
    task_library[i] = t.library;
    task_copredict[i] = t.copredict;
    unsigned char* lm = lib_masks + (size_t)i * a.n;
    if (!plan.lists_ready.empty() && plan.lists_ready[t.lib_mask]) {
      std::fill(lm, lm + a.n, 0);
      for (int r : plan.lib_lists[t.lib_mask])
        lm[r] = 1;
    } else {
      std::copy(plan.masks[t.lib_mask].begin(), plan.masks[t.lib_mask].end(), lm);
    }
    std::copy(plan.masks[t.pred_mask].begin(), plan.masks[t.pred_mask].end(), pred_masks + (size_t)i * a.n);
  }
  return (int)plan.tasks.size();
}

// ------------------------------------------------------ single-task seam
namespace {

// Outputs of the task seam's sizes pass, for the outputs pass that follows.
struct TaskMemo
{
  std::string key;
  TaskOut out;
  int n_pred = 0, n_lib = 0, e_actual = 0;
  bool force_compute = true;
  int n_thetas = 0;
  fedm_timing timing{};
};

// Every input of a task on the seam, as bytes: the arguments' scalars (with
// their pointers cleared) and the contents of their arrays, the task's masks
// and settings, and the context's precision.  Equal keys give equal outputs.
std::string task_key(const Context& ctx, const fedm_args& a, const fedm_task_io& io)
{
  std::string k;
  auto put = [&](const void* p, size_t bytes) {
    k.append(reinterpret_cast<const char*>(&bytes), sizeof bytes);
    if (p && bytes)
      k.append(static_cast<const char*>(p), bytes);
  };
  const size_t n = (size_t)std::max(a.n, 0);
  fedm_args s{};
  std::memcpy(&s, &a, sizeof s);
  s.t = s.x = s.y = s.co_x = s.extras = s.thetas = s.panel_weights = nullptr;
  s.panel = s.Es = s.libs = nullptr;
  put(&s, sizeof s);
  put(a.t, n * 8);
  put(a.x, n * 8);
  put(a.y, a.y ? n * 8 : 0);
  put(a.panel, a.panel ? n * 4 : 0);
  put(a.co_x, a.co_x ? n * 8 : 0);
  put(a.extras, a.extras ? (size_t)std::max(a.num_extras, 0) * n * 8 : 0);
  put(a.Es, a.Es ? (size_t)std::max(a.nE, 0) * 4 : 0);
  put(a.thetas, a.thetas ? (size_t)std::max(a.n_thetas, 0) * 8 : 0);
  put(a.libs, a.libs ? (size_t)std::max(a.n_libs, 0) * 4 : 0);
  put(a.panel_weights, a.panel_weights ? (size_t)std::max(a.n_panel_weights, 0) * a.n_panel_weights * 8 : 0);
  put(io.library_rows, io.library_rows ? n : 0);
  put(io.prediction_rows, io.prediction_rows ? n : 0);
  const int sc[6] = { io.E, io.k, io.copredict, io.distance, io.force_compute, ctx.precision };
  put(sc, sizeof sc);
  put(&io.aspect_ratio, sizeof io.aspect_ratio);
  return k;
}

int write_task_outputs(const TaskOut& to, fedm_task_io& io, int nth, bool force_compute);

} // namespace

int run_task(Context& ctx, const fedm_args& a, fedm_task_io& io)
{
  const double t0 = now_ms();
  const bool sizes_only = io.predictions == nullptr;
  std::string key = task_key(ctx, a, io);
  if (!sizes_only && ctx.task_memo) {
    // the outputs pass after a sizes pass on the same inputs
    std::shared_ptr<TaskMemo> memo = std::static_pointer_cast<TaskMemo>(ctx.task_memo);
    ctx.task_memo.reset();
    if (memo->key == key) {
      ctx.timing = memo->timing;
      ctx.timing.host_ms += now_ms() - t0;
      io.n_pred = memo->n_pred;
      io.n_lib = memo->n_lib;
      io.e_actual = memo->e_actual;
      io.total_nn = memo->out.nn_offsets.empty() ? 0 : memo->out.nn_offsets.back();
      return write_task_outputs(memo->out, io, memo->n_thetas, memo->force_compute);
    }
  }
  ctx.task_memo.reset();
  ctx.reset_timing();
  ck(cudaSetDevice(ctx.device), "cudaSetDevice");
  Prepared P;
  prepare(a, P);
  Options o = P.opts;
  o.distance = io.distance == 0 ? 0 : io.distance == 2 ? 2 : 1;
  o.aspect_ratio = io.aspect_ratio;
  o.force_compute = io.force_compute != 0;
  if (o.distance == 2 && (io.E < 1 || io.E > WASS_EMAX))
    throw Error{ RC_NOT_IMPLEMENTED, "the Wasserstein distance takes 1 <= E <= 16" };
  // (the task seam routes all-neighbour tasks through knn_exact_kernel, the
  // only kernel with a Wasserstein instance)
  const Generator& gen = P.gen;
  const int threads = host_threads(a);
  RowTables rt = build_row_tables(gen);
  sync_series(ctx, gen, rt);
  std::vector<uint8_t> lm(io.library_rows, io.library_rows + a.n), pm(io.prediction_rows, io.prediction_rows + a.n);
  for (auto& v : lm)
    v = v ? 1 : 0;
  for (auto& v : pm)
    v = v ? 1 : 0;
  std::vector<int> L = lib_rows_of(lm, rt), Pl = rows_of(pm);
  const int Ea = gen.E_actual(io.E);
  const int nth = (int)o.thetas.size();
  Task t;
  t.E = io.E;
  t.k = io.k;
  t.copredict = io.copredict != 0;
  t.save_coeffs = true;
  std::vector<Task> tasks{ t };
  std::vector<TaskOut> outs(1);
  {
    // the sizes pass runs the task too: total_nn is the length of the
    // neighbour lists make_prediction keeps, known only after the search
    DevRows drows = upload_rows(ctx, gen, rt, o);
    Manifolds M;
    GroupJob job;
    job.Ea = Ea;
    job.copredict = t.copredict;
    job.dF = device_manifold(ctx, M, gen, rt, drows, io.E, false, threads);
    job.dFp = t.copredict ? device_manifold(ctx, M, gen, rt, drows, io.E, true, threads) : job.dF;
    job.hF = M.host[std::make_pair(io.E, false)];
    job.hFp = t.copredict ? M.host[std::make_pair(io.E, true)] : job.hF;
    job.task_ids = { 0 };
    job.lib_lists = { &L };
    job.pred_lists = { &Pl };
    job.detail = true;
    job.knn_for_all = true;
    set_wasserstein_shape(job, gen, io.E);
    run_group(ctx, o, tasks, drows, job, outs);
  }
  TaskOut& to = outs[0];
  io.n_pred = (int)Pl.size();
  io.n_lib = (int)L.size();
  io.e_actual = Ea;
  io.total_nn = to.nn_offsets.empty() ? 0 : to.nn_offsets.back();
  ctx.timing.host_ms = now_ms() - t0;
  ctx.timing.predictions = (long long)Pl.size() * nth;
  ctx.timing.distance_pairs = (long long)Pl.size() * (long long)L.size();
  if (sizes_only) {
    auto memo = std::make_shared<TaskMemo>();
    memo->key = std::move(key);
    memo->out = std::move(to);
    memo->n_pred = io.n_pred;
    memo->n_lib = io.n_lib;
    memo->e_actual = io.e_actual;
    memo->force_compute = o.force_compute;
    memo->n_thetas = nth;
    memo->timing = ctx.timing;
    ctx.task_memo = memo;
    return RC_SUCCESS;
  }
  return write_task_outputs(to, io, nth, o.force_compute);
}

namespace {

// The task seam's outputs (src/edm.cpp:598-610 and 730-813 for the return
// codes), copied into the caller's buffers.
int write_task_outputs(const TaskOut& to, fedm_task_io& io, int nth, bool force_compute)
{
  const int np = io.n_pred;
  std::copy(to.pred_all.begin(), to.pred_all.end(), io.predictions);
  if (io.coeffs)
    std::copy(to.coeffs.begin(), to.coeffs.end(), io.coeffs);
  // per-point return codes (src/edm.cpp:598-610 and 730-813)
  for (int i = 0; i < np; i++) {
    const bool made = to.kused[i] != MISSING_I;
    for (int th = 0; th < nth; th++) {
      int code = 0;
      if (!made)
        code = th == 0 ? (force_compute ? 0 : 503) : 8000;
      if (io.rc)
        io.rc[(size_t)th * np + i] = code;
    }
    if (io.kused)
      io.kused[i] = to.kused[i];
  }
  if (io.nn_offsets)
    std::copy(to.nn_offsets.begin(), to.nn_offsets.end(), io.nn_offsets);
  if (io.nn_idx)
    std::copy(to.nn_idx.begin(), to.nn_idx.end(), io.nn_idx);
  if (io.nn_dist)
    std::copy(to.nn_dist.begin(), to.nn_dist.end(), io.nn_dist);
  if (io.stats_rho)
    for (int th = 0; th < nth; th++)
      io.stats_rho[th] = to.rho[th];
  if (io.stats_mae)
    for (int th = 0; th < nth; th++)
      io.stats_mae[th] = to.mae[th];
  return to.rc;
}

} // namespace

} // namespace fedm
