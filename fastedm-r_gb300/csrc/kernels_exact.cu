// Exact FP64 kernels: distances, k-nearest-neighbour selection, simplex and
// S-map forecasts, rho/MAE.  Arithmetic follows the reference's operation
// order (EDM-Developers/fastEDM-r src/distances.cpp:151-229,
// src/edm.cpp:652-814, src/stats.cpp:64-94).  This translation unit is built
// with --fmad=false so every a*b+c stays a rounded multiply and a rounded
// add, as in the reference's FP64 loops; sqrt and division are IEEE
// round-to-nearest, so distances are bit-identical to the CPU.
#include <cfloat>
#include <climits>
#include <cstdio>

#include "kernels.h"
#include "exp_rn.cuh"
#include "smap_solve.cuh"
#include "wasserstein.cuh"

namespace fedm {

namespace {

constexpr double MISS = 1.0e+100;
constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ int find_task(const GroupParams& g, long long p)
{
  int lo = 0, hi = g.n_tasks - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (g.tasks[mid].point_base <= p)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// One reference distance (src/distances.cpp:160-226; with WASS the
// Wasserstein distance, :488-527).  Returns false for skipped or invalid
// pairs (zero or missing distance).  The Wasserstein form is a template
// instance of its own, so the L1/L2 kernels keep their registers.
template<bool WASS>
__device__ __forceinline__ bool exact_distance(const GroupParams& g, int lrow, int prow, const double* y, int ppanel,
                                               double ptime, double& out)
{
  if (g.skip_other_panels && g.panel[lrow] != ppanel)
    return false;
  if constexpr (WASS) {
    // src/distances.cpp:488-527: no past-only rule on this path; the panel
    // term joins the unlagged distance
    bool has_pen = false;
    double pen = 0.0;
    if (g.panel_mode && g.idw > 0) {
      has_pen = true;
      pen = g.idw * (double)(g.panel[lrow] != ppanel);
    } else if (g.panel_mode && g.has_id_weights) {
      float w = g.id_w[(size_t)g.panel_dense[lrow] * g.n_pid + g.panel_dense[prow]];
      if (isnan(w)) {
        atomicExch(g.err_flag, 1);  // the reference's map::at throws here
        w = 0.f;
      }
      has_pen = true;
      pen = (double)w;
    }
    int st = 0;
    const bool ok = wasserstein_pair(g.F + (size_t)lrow * g.Ea, y, g.w_E, g.w_rows, g.w_unlagged, g.w_dt != 0,
                                     g.aspect_ratio, g.missing_distance, has_pen, pen, out, st);
    if (st)
      atomicExch(g.err_flag, 1);
    return ok;
  }
  if (g.past_only && g.lib_target_time[lrow] > ptime)
    return false;
  double d = 0.0;
  if (g.panel_mode && g.idw > 0) {
    d += g.idw * (double)(g.panel[lrow] != ppanel);
  } else if (g.panel_mode && g.has_id_weights) {
    float w = g.id_w[(size_t)g.panel_dense[lrow] * g.n_pid + g.panel_dense[prow]];
    if (isnan(w)) {
      atomicExch(g.err_flag, 1);  // the reference's map::at throws here
      w = 0.f;
    }
    d += (double)w;
  }
  const double* x = g.F + (size_t)lrow * g.Ea;
  const int Ea = g.Ea;
  for (int j = 0; j < Ea; j++) {
    double a = x[j], b = y[j], dij;
    if (g.has_missing && (a == MISS || b == MISS)) {
      if (g.missing_distance == 0) {
        d = MISS;
        break;
      }
      dij = g.missing_distance;
    } else {
      dij = a - b;
    }
    if (g.l1)
      d += fabs(dij) / Ea;
    else
      d += dij * dij;
  }
  if (d != 0 && d != MISS) {
    out = g.l1 ? d : sqrt(d);
    return true;
  }
  return false;
}

__device__ __forceinline__ long long point_of(const ChunkBuffers& c, long long q)
{
  return c.plist ? c.plist[q] : c.p_begin + q;
}

__device__ __forceinline__ void note_rc(const GroupParams& g, int task, int code)
{
  if (code)
    atomicMax(&g.task_rc[task], code);
}

// Return codes of a point that made no forecast (src/edm.cpp:598-610): the
// reference writes rc(0, i) only, so with several thetas the untouched
// entries keep UNKNOWN_ERROR and dominate the task's max.
__device__ __forceinline__ void early_rc(const GroupParams& g, int task, int status, int t)
{
  if (t == 0)
    note_rc(g, task, status == PT_EARLY_SUCCESS ? 0 : 503);
  else
    note_rc(g, task, 8000);
}

__device__ __forceinline__ void note_k(const GroupParams& g, int task, long long p, int k)
{
  atomicMin(&g.task_kmin[task], k);
  atomicMax(&g.task_kmax[task], k);
  if (g.kused)
    g.kused[p] = k;
}

// ------------------------------------------------------ neighbour selection
// One warp per prediction point.  The k best (distance, library index)
// pairs are kept sorted in shared memory; a library chunk of 32 is scored in
// parallel and its candidates are inserted in index order, which realises
// the reference's (distance asc, index asc) order (src/edm.cpp:652-681).
template<bool WASS>
__global__ void knn_exact_kernel(GroupParams g, ChunkBuffers c, int warps_per_block, int per_warp_bytes)
{
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  unsigned char* base = smem + (size_t)wib * per_warp_bytes;
  double* sy = (double*)base;
  double* sD = sy + g.Ea;
  int* sI = (int*)(sD + c.kcap);
  const long long nwarps = (long long)gridDim.x * warps_per_block;
  const long long chunk = c.p_end - c.p_begin;
  for (long long q = (long long)blockIdx.x * warps_per_block + wib; q < chunk; q += nwarps) {
    if (c.redo_only && c.status[q] != PT_REDO)
      continue;
    const long long p = point_of(c, q);
    const int ti = find_task(g, p);
    const DevTask T = g.tasks[ti];
    if (T.all_mode || (T.mixed && !c.plist))
      continue;
    const int prow = g.pred_rows[T.pred_off + (int)(p - T.point_base)];
    for (int j = lane; j < g.Ea; j += 32)
      sy[j] = g.Fp[(size_t)prow * g.Ea + j];
    const int ppanel = g.panel ? g.panel[prow] : 0;
    const double ptime = g.past_only ? g.point_time[prow] : 0.0;
    __syncwarp();
    const int k = T.k;
    int count = 0, numValid = 0;
    // capacity for the whole library: every valid neighbour is kept, so the
    // list is simply the valid entries in library order (no ranking needed)
    const bool collect_all = k >= T.n_lib;
    for (int b0 = 0; b0 < T.n_lib && collect_all; b0 += 32) {
      const int i = b0 + lane;
      double d = 0;
      bool valid = false;
      if (i < T.n_lib)
        valid = exact_distance<WASS>(g, g.lib_rows[T.lib_off + i], prow, sy, ppanel, ptime, d);
      const unsigned vm = __ballot_sync(FULL, valid);
      if (valid) {
        const int slot = count + __popc(vm & ((1u << lane) - 1u));
        sD[slot] = d;
        sI[slot] = i;
      }
      count += __popc(vm);
    }
    if (collect_all)
      numValid = count;
    __syncwarp();
    for (int b0 = 0; b0 < T.n_lib && !collect_all; b0 += 32) {
      const int i = b0 + lane;
      double d = 0;
      bool valid = false;
      if (i < T.n_lib)
        valid = exact_distance<WASS>(g, g.lib_rows[T.lib_off + i], prow, sy, ppanel, ptime, d);
      numValid += __popc(__ballot_sync(FULL, valid));
      const double thr = (k <= 0 || count < k) ? DBL_MAX : sD[k - 1];
      unsigned cm = __ballot_sync(FULL, valid && k > 0 && (count < k ? true : d < thr));
      while (cm) {
        const int src = __ffs(cm) - 1;
        cm &= cm - 1;
        const double dd = __shfl_sync(FULL, d, src);
        if (count == k && !(dd < sD[k - 1]))
          continue;
        int cnt = 0;
        for (int e = lane; e < count; e += 32)
          cnt += sD[e] <= dd;
        const int pos = __reduce_add_sync(FULL, cnt);
        const int last = count < k - 1 ? count : k - 1;
        for (int top = last; top > pos; top -= 32) {
          const int e = top - 1 - lane;
          const bool act = e >= pos;
          double vD = 0;
          int vI = 0;
          if (act) {
            vD = sD[e];
            vI = sI[e];
          }
          __syncwarp();
          if (act) {
            sD[e + 1] = vD;
            sI[e + 1] = vI;
          }
          __syncwarp();
        }
        if (lane == 0) {
          sD[pos] = dd;
          sI[pos] = b0 + src;
        }
        count = count + 1 < k ? count + 1 : k;
        __syncwarp();
      }
    }
    // src/edm.cpp:595-617 on the requested k (k_req = -1: all valid)
    int status = PT_OK, keff = T.k_req < 0 ? numValid : T.k_req;
    if (T.k_req > numValid) {
      if (g.force_compute)
        keff = numValid;
      else
        status = PT_INSUFFICIENT;
    }
    if (status == PT_OK && (keff == 0 || numValid == 0))
      status = g.force_compute ? PT_EARLY_SUCCESS : PT_INSUFFICIENT;
    int* oi = c.nn_idx + q * c.kcap;
    double* od = c.nn_dist + q * c.kcap;
    if (status == PT_OK) {
      if (collect_all && keff == numValid) {
        for (int e = lane; e < count; e += 32) {
          oi[e] = sI[e];
          od[e] = sD[e];
        }
      } else if (keff == numValid) {
        // all valid neighbours, in library order (src/edm.cpp:615-616)
        for (int e = lane; e < count; e += 32) {
          int r = 0;
          const int me = sI[e];
          for (int f = 0; f < count; f++)
            r += sI[f] < me;
          oi[r] = me;
          od[r] = sD[e];
        }
      } else {
        for (int e = lane; e < keff; e += 32) {
          oi[e] = sI[e];
          od[e] = sD[e];
        }
      }
    }
    if (lane == 0) {
      c.status[q] = status;
      c.nn_count[q] = keff;
      if (status == PT_OK)
        note_k(g, T.task, p, keff);
      else if (g.kused)
        g.kused[p] = INT_MIN;
    }
    __syncwarp();
  }
}

// ------------------------------------------------ uncertified mixed points
// A point whose FP32 candidate list could not be certified still has a
// certified bound thr: every row among its true neighbours has an FP32
// squared distance, evaluated as the scan evaluates it (difference, square,
// fused accumulation, in coordinate order), of at most thr.  One warp per
// point re-scans the library in FP32, keeps the rows under thr in library
// order, scores them with exact_distance and ranks the valid ones by
// (distance, library index).  Rows outside the kept set have non-zero FP32
// values and count as valid neighbours, the mixed kernels' rule.  The output
// (status, count, lists, k statistics) is knn_exact_kernel's; a point with
// more than REFINE_CAP kept rows, or whose kept rows cannot supply its k, is
// marked PT_REDO and left to knn_exact_kernel.
constexpr int REFINE_CAP = 1024;
constexpr int REFINE_WARPS = 8;
constexpr int REFINE_TILE = 256;  // library rows staged per tile

// FP32 squared distance of a row to the negated point np, in the scan's
// operation order
template<int EA>
__device__ __forceinline__ float refine_sq(const float* x, const float (&np)[EA])
{
  float d = __fadd_rn(x[0], np[0]);
  float sq = __fmul_rn(d, d);
#pragma unroll
  for (int j = 1; j < EA; j++) {
    d = __fadd_rn(x[j], np[j]);
    sq = __fmaf_rn(d, d, sq);
  }
  return sq;
}

// Appends a warp's hits (library indices, in index order) to its list;
// false when the list would overflow (the same answer in every lane).
__device__ __forceinline__ bool refine_append(bool hit, int i, int lane, int* sI, int& count)
{
  const unsigned hm = __ballot_sync(FULL, hit);
  if (count + __popc(hm) > REFINE_CAP)
    return false;
  if (hit)
    sI[count + __popc(hm & ((1u << lane) - 1u))] = i;
  count += __popc(hm);
  return true;
}

// Dynamic shared memory: per warp REFINE_CAP indices and distances, then a
// tile of REFINE_TILE rows at an odd row stride (no bank conflicts when the
// lanes read consecutive rows).
template<int EA>
__host__ __device__ constexpr int refine_tile_stride() { return EA | 1; }
template<int EA>
__host__ __device__ constexpr size_t refine_smem()
{
  return (size_t)REFINE_WARPS * REFINE_CAP * 12 + (size_t)REFINE_TILE * refine_tile_stride<EA>() * 4;
}

// A CTA takes REFINE_WARPS consecutive points of the (point-ordered) list.
// When they all belong to one task -- the usual case -- the CTA stages each
// tile of the library once and every warp scans it from shared memory;
// otherwise each warp gathers its task's rows itself.
template<int EA>
__global__ void __launch_bounds__(32 * REFINE_WARPS) knn_refine_kernel(GroupParams g, ChunkBuffers c, RefineRun r)
{
  constexpr int TS = refine_tile_stride<EA>();
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_task[REFINE_WARPS];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  int* sI = (int*)smem + (size_t)wib * REFINE_CAP;
  double* sD = (double*)(smem + (size_t)REFINE_WARPS * REFINE_CAP * 4) + (size_t)wib * REFINE_CAP;
  float* tile = (float*)(smem + (size_t)REFINE_WARPS * REFINE_CAP * 12);
  const long long chunk = c.p_end - c.p_begin;
  for (long long q0 = (long long)blockIdx.x * REFINE_WARPS; q0 < chunk; q0 += (long long)gridDim.x * REFINE_WARPS) {
    const long long q = q0 + wib;
    const bool has = q < chunk;
    long long p = 0;
    int ti = -1, prow = 0;
    double thr = 0;
    float np[EA];
#pragma unroll
    for (int j = 0; j < EA; j++)
      np[j] = 0.f;
    if (has) {
      p = point_of(c, q);
      ti = find_task(g, p);
      const DevTask& Tq = g.tasks[ti];
      prow = g.pred_rows[Tq.pred_off + (int)(p - Tq.point_base)];
      thr = r.thr[q];
#pragma unroll
      for (int j = 0; j < EA; j++)
        np[j] = -r.Fp32[(size_t)prow * r.rs + j];
    }
    if (lane == 0)
      s_task[wib] = ti;
    __syncthreads();
    const int t0 = s_task[0];  // warp 0 always has a point
    bool same = true;
#pragma unroll
    for (int w = 1; w < REFINE_WARPS; w++)
      same = same && (s_task[w] < 0 || s_task[w] == t0);
    const DevTask T = g.tasks[has ? ti : t0];
    // panels with a finite penalty: the scan's FP32 value of a row of
    // another panel carries idw (one_point.cuh), and so does the value
    // compared with the point's bound here
    const bool pen = g.panel_mode && g.idw > 0;
    const float penf = pen ? (float)g.idw : 0.f;
    const int ppan = pen && has ? g.panel[prow] : 0;
    auto value = [&](float v, int li) {
      return pen && g.panel[g.lib_rows[T.lib_off + li]] != ppan ? __fadd_rn(v, penf) : v;
    };
    int count = 0;
    bool over = false;
    if (same) {
      for (int b0 = 0; b0 < T.n_lib; b0 += REFINE_TILE) {
        const int nrow = min(REFINE_TILE, T.n_lib - b0);
        __syncthreads();  // every warp is done with the previous tile
        for (int e = threadIdx.x; e < nrow * EA; e += blockDim.x) {
          const int i = e / EA, j = e - i * EA;
          tile[i * TS + j] = r.F32[(size_t)g.lib_rows[T.lib_off + b0 + i] * r.rs + j];
        }
        __syncthreads();
        if (has && !over)
          for (int i0 = 0; i0 < nrow; i0 += 32) {
            const int i = i0 + lane;
            const bool hit = i < nrow && (double)value(refine_sq<EA>(tile + i * TS, np), b0 + i) <= thr;
            if (!refine_append(hit, b0 + i, lane, sI, count)) {
              over = true;
              break;
            }
          }
      }
    } else if (has) {
      for (int b0 = 0; b0 < T.n_lib; b0 += 32) {
        const int i = b0 + lane;
        const bool hit = i < T.n_lib &&
                         (double)value(refine_sq<EA>(r.F32 + (size_t)g.lib_rows[T.lib_off + i] * r.rs, np), i) <= thr;
        if (!refine_append(hit, i, lane, sI, count)) {
          over = true;
          break;
        }
      }
    }
    if (has) {
      __syncwarp();
      int status = PT_REDO, keff = 0;
      if (!over) {
        const double* y = g.Fp + (size_t)prow * g.Ea;
        const int ppanel = g.panel ? g.panel[prow] : 0;
        const double ptime = g.past_only ? g.point_time[prow] : 0.0;
        int nvalid = 0;
        for (int e = lane; e < count; e += 32) {
          double d = 0;
          const bool valid = exact_distance<false>(g, g.lib_rows[T.lib_off + sI[e]], prow, y, ppanel, ptime, d);
          sD[e] = valid ? d : -1.0;
          nvalid += valid ? 1 : 0;
        }
        nvalid = __reduce_add_sync(FULL, nvalid);
        __syncwarp();
        const int numValid = T.n_lib - (count - nvalid);
        // src/edm.cpp:595-617, as in knn_exact_kernel
        status = PT_OK;
        keff = T.k_req < 0 ? numValid : T.k_req;
        if (T.k_req > numValid) {
          if (g.force_compute)
            keff = numValid;
          else
            status = PT_INSUFFICIENT;
        }
        if (status == PT_OK && (keff == 0 || numValid == 0))
          status = g.force_compute ? PT_EARLY_SUCCESS : PT_INSUFFICIENT;
        if (status == PT_OK && nvalid < keff)
          status = PT_REDO;
        if (status == PT_OK) {
          // rank among the valid kept rows: (distance, index), or library
          // order when every valid neighbour is used (src/edm.cpp:615-616)
          const bool lib_order = keff == numValid;
          int* oi = c.nn_idx + q * c.kcap;
          double* od = c.nn_dist + q * c.kcap;
          for (int e = lane; e < count; e += 32) {
            const double de = sD[e];
            if (de < 0)
              continue;
            const int ie = sI[e];
            int rank = 0;
            for (int f = 0; f < count; f++) {
              const double df = sD[f];
              if (df < 0)
                continue;
              rank += lib_order ? (sI[f] < ie) : (df < de || (df == de && sI[f] < ie));
            }
            if (rank < keff) {
              oi[rank] = ie;
              od[rank] = de;
            }
          }
        }
      }
      if (lane == 0) {
        c.status[q] = status;
        if (status == PT_REDO)
          atomicAdd(r.redo_count, 1);
        else {
          c.nn_count[q] = keff;
          if (status == PT_OK)
            note_k(g, T.task, p, keff);
          else if (g.kused)
            g.kused[p] = INT_MIN;
        }
      }
      __syncwarp();
    }
    __syncthreads();  // s_task and the tile are reused by the next group
  }
}

// ------------------------------------------------------------- simplex
// src/edm.cpp:707-735, one thread per (point, theta).
__global__ void simplex_nn_kernel(GroupParams g, ChunkBuffers c)
{
  const long long chunk = c.p_end - c.p_begin;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= chunk * g.n_thetas)
    return;
  const int t = (int)(idx / chunk);
  const long long q = idx - (long long)t * chunk;
  const long long p = point_of(c, q);
  const DevTask T = g.tasks[find_task(g, p)];
  if (T.all_mode || (T.mixed && !c.plist))
    return;
  const int st = c.status[q];
  if (st != PT_OK) {
    early_rc(g, T.task, st, t);
    return;
  }
  const int ke = c.nn_count[q];
  const double* dists = c.nn_dist + q * c.kcap;
  const int* inds = c.nn_idx + q * c.kcap;
  double minDist = dists[0];
  for (int j = 1; j < ke; j++)
    minDist = dists[j] < minDist ? dists[j] : minDist;
  const double theta = g.thetas[t];
  double sumw = 0.0;
  for (int j = 0; j < ke; j++)
    sumw = sumw + exp_rn(-theta * (dists[j] / minDist));
  double r = 0.0;
  for (int j = 0; j < ke; j++) {
    // the weight is recomputed rather than stored: identical bits, no
    // per-thread array of k doubles
    const double w = exp_rn(-theta * (dists[j] / minDist));
    r = r + g.lib_target[g.lib_rows[T.lib_off + inds[j]]] * (w / sumw);
  }
  g.pred[(size_t)t * g.total_points + p] = r;
}

// ---------------------------------------------------------------- S-map
// Forecast from coefficients (src/edm.cpp:784-812).
__device__ __forceinline__ void smap_finish(const GroupParams& g, const DevTask& T, long long p, int prow, int t,
                                            const double* ics, int n)
{
  const double* y = g.Fp + (size_t)prow * g.Ea;
  double r = ics[0];
  for (int j = 0; j < g.Ea; j++) {
    const double yj = y[j];
    if (yj != MISS)
      r += yj * ics[j + 1];
  }
  if (g.coeffs && T.save_coeffs && t == g.n_thetas - 1) {
    for (int j = 0; j < n; j++)
      g.coeffs[(size_t)p * n + j] = fabs(ics[j]) < 1.0e-11 ? MISS : ics[j];
  }
  g.pred[(size_t)t * g.total_points + p] = r;
}

constexpr int SMALL_N = 8;
constexpr int KW_LOCAL = 32;  // weights cached per thread (larger k recomputes)

// src/edm.cpp:737-814 for a finite neighbour list, one thread per
// (point, theta).  X^T X and X^T y are summed over the neighbours in order.
__global__ void smap_nn_kernel(GroupParams g, ChunkBuffers c, long long slab)
{
  const long long chunk = c.p_end - c.p_begin;
  const long long nthreads = (long long)gridDim.x * blockDim.x;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int n = g.Ea + 1;
  double lW[SMALL_N * SMALL_N], lU[SMALL_N * SMALL_N], lV[SMALL_N * SMALL_N], lsv[SMALL_N], ltmp[SMALL_N],
    lb[SMALL_N], lx[SMALL_N], wbuf[KW_LOCAL];
  double *W = lW, *U = lU, *V = lV, *sv = lsv, *tmp = ltmp, *bv = lb, *xs = lx;
  if (n > SMALL_N) {
    double* s = c.scratch + tid * slab;
    W = s;
    U = W + n * n;
    V = U + n * n;
    sv = V + n * n;
    tmp = sv + n;
    bv = tmp + n;
    xs = bv + n;
  }
  for (long long idx = tid; idx < chunk * g.n_thetas; idx += nthreads) {
    const int t = (int)(idx / chunk);
    const long long q = idx - (long long)t * chunk;
    const long long p = point_of(c, q);
    const DevTask T = g.tasks[find_task(g, p)];
    if (T.all_mode || (T.mixed && !c.plist))
      continue;
    const int st = c.status[q];
    if (st != PT_OK) {
      early_rc(g, T.task, st, t);
      continue;
    }
    const int ke = c.nn_count[q];
    const double* dists = c.nn_dist + q * c.kcap;
    const int* inds = c.nn_idx + q * c.kcap;
    double mean = 0;
    for (int j = 0; j < ke; j++)
      mean += dists[j];
    mean /= (double)ke;
    const double theta = g.thetas[t];
    // weights once per (point, theta) (src/edm.cpp:744-745); the X entries
    // w * M(row, j) are re-formed where used, which gives the same bits
    for (int i = 0; i < ke && i < KW_LOCAL; i++)
      wbuf[i] = exp_rn(-theta * (dists[i] / mean));
    auto weight = [&](int i) { return i < KW_LOCAL ? wbuf[i] : exp_rn(-theta * (dists[i] / mean)); };
    for (int a = 0; a < n; a++) {
      for (int b = a; b < n; b++) {
        double s = 0;
        for (int i = 0; i < ke; i++) {
          const double w = weight(i);
          const int row = g.lib_rows[T.lib_off + inds[i]];
          const double xa = a == 0 ? w : w * g.F[(size_t)row * g.Ea + a - 1];
          const double xb = b == 0 ? w : w * g.F[(size_t)row * g.Ea + b - 1];
          s += xa * xb;
        }
        W[a * n + b] = s;
        W[b * n + a] = s;
      }
      double s = 0;
      for (int i = 0; i < ke; i++) {
        const double w = weight(i);
        const int row = g.lib_rows[T.lib_off + inds[i]];
        const double xa = a == 0 ? w : w * g.F[(size_t)row * g.Ea + a - 1];
        s += xa * (w * g.lib_target[row]);
      }
      bv[a] = s;
    }
    svd_solve(W, U, V, sv, tmp, bv, xs, n);
    const int prow = g.pred_rows[T.pred_off + (int)(p - T.point_base)];
    smap_finish(g, T, p, prow, t, xs, n);
  }
}

// ------------------------------------------------------ all-neighbour mode
// k = -1 (or k >= library size): every valid neighbour in library order
// (src/edm.cpp:613-617).  all_dist_kernel writes each point's distances to
// its row of the chunk's distance buffer (-1 marks an invalid pair); then
// one thread per (point, theta) reduces them sequentially in library order,
// the order the reference's loops use, so the results are the same bits.
__global__ void all_dist_kernel(GroupParams g, ChunkBuffers c, long long max_nlib, int per_warp_bytes)
{
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  const long long chunk = c.p_end - c.p_begin;
  double* sy = (double*)(smem + (size_t)wib * per_warp_bytes);
  for (long long q = (long long)blockIdx.x * wpb + wib; q < chunk; q += (long long)gridDim.x * wpb) {
    const long long p = point_of(c, q);
    const DevTask T = g.tasks[find_task(g, p)];
    if (!T.all_mode)
      continue;
    const int prow = g.pred_rows[T.pred_off + (int)(p - T.point_base)];
    for (int j = lane; j < g.Ea; j += 32)
      sy[j] = g.Fp[(size_t)prow * g.Ea + j];
    const int ppanel = g.panel ? g.panel[prow] : 0;
    const double ptime = g.past_only ? g.point_time[prow] : 0.0;
    __syncwarp();
    double* dq = c.scratch + q * max_nlib;
    int lcnt = 0;
    for (int i = lane; i < T.n_lib; i += 32) {
      double d;
      const bool ok = exact_distance<false>(g, g.lib_rows[T.lib_off + i], prow, sy, ppanel, ptime, d);
      dq[i] = ok ? d : -1.0;
      lcnt += ok;
    }
    const int cnt = __reduce_add_sync(FULL, lcnt);
    int status = PT_OK;
    if (!g.force_compute && T.k_req > 0 && T.k_req > cnt)
      status = PT_INSUFFICIENT;
    else if (cnt == 0)
      status = g.force_compute ? PT_EARLY_SUCCESS : PT_INSUFFICIENT;
    if (lane == 0) {
      c.status[q] = status;
      c.nn_count[q] = cnt;
      if (status == PT_OK)
        note_k(g, T.task, p, cnt);
      else if (g.kused)
        g.kused[p] = INT_MIN;
    }
    __syncwarp();
  }
}

// One thread per (point, theta), theta fastest: the threads of a warp read
// the same point's distance row and library rows (broadcast loads).
__global__ void all_forecast_kernel(GroupParams g, ChunkBuffers c, long long max_nlib, long long slab)
{
  const long long chunk = c.p_end - c.p_begin;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= chunk * g.n_thetas)
    return;
  const long long q = idx / g.n_thetas;
  const int t = (int)(idx - q * g.n_thetas);
  const long long p = point_of(c, q);
  const DevTask T = g.tasks[find_task(g, p)];
  if (!T.all_mode)
    return;
  const int st = c.status[q];
  if (st != PT_OK) {
    early_rc(g, T.task, st, t);
    return;
  }
  double* dq = c.scratch + q * max_nlib;
  const double theta = g.thetas[t];
  if (g.algorithm == 0) {
    // src/edm.cpp:707-735
    double minDist = DBL_MAX;
    for (int i = 0; i < T.n_lib; i++)
      if (dq[i] >= 0 && dq[i] < minDist)
        minDist = dq[i];
    const double ymin = rcp(minDist);
    double sumw = 0.0;
    // with one theta this thread alone reads the point's distance row, so
    // each weight replaces its distance (weights are positive, the -1 marks
    // of invalid rows stay) and is not evaluated twice
    const bool keep = g.n_thetas == 1;
    for (int i = 0; i < T.n_lib; i++)
      if (dq[i] >= 0) {
        const double w = exp_rn(-theta * dvd_r(dq[i], minDist, ymin));
        sumw = sumw + w;
        if (keep)
          dq[i] = w;
      }
    const double ysum = rcp(sumw);
    double r = 0.0;
    for (int i = 0; i < T.n_lib; i++)
      if (dq[i] >= 0) {
        const double w = keep ? dq[i] : exp_rn(-theta * dvd_r(dq[i], minDist, ymin));
        r = r + g.lib_target[g.lib_rows[T.lib_off + i]] * dvd_r(w, sumw, ysum);
      }
    g.pred[(size_t)t * g.total_points + p] = r;
    return;
  }
  // src/edm.cpp:737-814 over every valid neighbour
  const int n = g.Ea + 1;
  const int ke = c.nn_count[q];
  double mean = 0;
  for (int i = 0; i < T.n_lib; i++)
    if (dq[i] >= 0)
      mean += dq[i];
  mean /= (double)ke;
  double* W = c.gram + idx * slab;  // [n*n] normal matrix, then U, V, sv, tmp, b, x
  double* U = W + n * n;
  double* V = U + n * n;
  double* sv = V + n * n;
  double* tmp = sv + n;
  double* bv = tmp + n;
  double* xs = bv + n;
  for (int e = 0; e < n * n; e++)
    W[e] = 0;
  for (int a = 0; a < n; a++)
    bv[a] = 0;
  for (int i = 0; i < T.n_lib; i++) {
    if (dq[i] < 0)
      continue;
    const double w = exp_rn(-theta * (dq[i] / mean));
    const int row = g.lib_rows[T.lib_off + i];
    const double* fr = g.F + (size_t)row * g.Ea;
    const double yl = w * g.lib_target[row];
    for (int a = 0; a < n; a++) {
      const double xa = a == 0 ? w : w * fr[a - 1];
      for (int b = a; b < n; b++) {
        const double xb = b == 0 ? w : w * fr[b - 1];
        W[a * n + b] += xa * xb;
      }
      bv[a] += xa * yl;
    }
  }
  for (int a = 0; a < n; a++)
    for (int b = 0; b < a; b++)
      W[a * n + b] = W[b * n + a];
  svd_solve(W, U, V, sv, tmp, bv, xs, n);
  const int prow = g.pred_rows[T.pred_off + (int)(p - T.point_base)];
  smap_finish(g, T, p, prow, t, xs, n);
}

// The S-map's weights over every valid neighbour depend on theta only
// through w = exp(-theta * (d / mean)) (src/edm.cpp:744-745).  One thread per
// point forms mean (in library order, as the forecast kernels do) and the
// ratios d / mean in place of the distances, once for every theta; invalid
// rows keep their -1 mark.  Runs only before all_smap_kernel, the last
// reader of the distance rows.
__global__ void all_ratio_kernel(GroupParams g, ChunkBuffers c, long long max_nlib)
{
  const long long chunk = c.p_end - c.p_begin;
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= chunk)
    return;
  const long long p = point_of(c, q);
  const DevTask T = g.tasks[find_task(g, p)];
  if (!T.all_mode || c.status[q] != PT_OK)
    return;
  double* dq = c.scratch + q * max_nlib;
  double mean = 0;
  for (int i = 0; i < T.n_lib; i++)
    if (dq[i] >= 0)
      mean += dq[i];
  mean /= (double)c.nn_count[q];
  const double ymean = rcp(mean);
  for (int i = 0; i < T.n_lib; i++)
    if (dq[i] >= 0)
      dq[i] = dvd_r(dq[i], mean, ymean);
}

// S-map over every valid neighbour for E_a <= 8 (src/edm.cpp:737-814): the
// all_forecast_kernel computation with the normal equations accumulated in
// registers (the same operations in the same order, so the same bits), on
// the ratios d / mean that all_ratio_kernel left in the distance rows.
template<int EA>
__global__ void __launch_bounds__(128) all_smap_kernel(GroupParams g, ChunkBuffers c, long long max_nlib)
{
  constexpr int n = EA + 1;
  const long long chunk = c.p_end - c.p_begin;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= chunk * g.n_thetas)
    return;
  const long long q = idx / g.n_thetas;
  const int t = (int)(idx - q * g.n_thetas);
  const long long p = point_of(c, q);
  const DevTask T = g.tasks[find_task(g, p)];
  if (!T.all_mode)
    return;
  const int st = c.status[q];
  if (st != PT_OK) {
    early_rc(g, T.task, st, t);
    return;
  }
  const double* rq = c.scratch + q * max_nlib;  // d / mean per valid row
  const double theta = g.thetas[t];
  double W[n][n], bv[n];
#pragma unroll
  for (int a = 0; a < n; a++) {
    bv[a] = 0;
#pragma unroll
    for (int b = 0; b < n; b++)
      W[a][b] = 0;
  }
  for (int i = 0; i < T.n_lib; i++) {
    const double r = rq[i];
    if (r < 0)
      continue;
    const double w = exp_rn(-theta * r);
    const int row = g.lib_rows[T.lib_off + i];
    const double* fr = g.F + (size_t)row * EA;
    const double yl = w * g.lib_target[row];
    double xr[n];
    xr[0] = w;
#pragma unroll
    for (int j = 1; j < n; j++)
      xr[j] = w * fr[j - 1];
#pragma unroll
    for (int a = 0; a < n; a++) {
#pragma unroll
      for (int b = a; b < n; b++)
        W[a][b] += xr[a] * xr[b];
      bv[a] += xr[a] * yl;
    }
  }
  double Wl[n * n], U[n * n], V[n * n], sv[n], tmp[n], xs[n];
#pragma unroll
  for (int a = 0; a < n; a++)
#pragma unroll
    for (int b = 0; b < n; b++)
      Wl[a * n + b] = b >= a ? W[a][b] : W[b][a];
  svd_solve(Wl, U, V, sv, tmp, bv, xs, n);
  const int prow = g.pred_rows[T.pred_off + (int)(p - T.point_base)];
  smap_finish(g, T, p, prow, t, xs, n);
}

// ------------------------------------------- k = all S-map, FAST precision
// The normal equations of the k = all S-map are sum_i w_i^2 u_i u_i^T and
// sum_i w_i^2 t_i u_i (u_i = [1, m_i]): per library row a fixed table of
// n(n+1)/2 + n products, scaled by one weight per (point, theta, row).
// gram_terms_kernel writes each pool row's products, rounded to FP64 and
// split into a float pair hi + lo (48 significant bits);
// all_smap_df_kernel computes w^2 = exp(-2 theta d / mean) in FP32 and
// accumulates every entry in double-float arithmetic: the product w^2 * hi
// exactly by TwoProd (an FMA), the sum exactly by Knuth's TwoSum, and the
// rounding errors with w^2 * lo in a float correction term.  The solve is
// the FP64 JacobiSVD of the exact path.  The weights carry FP32 rounding
// (~1e-7 relative); the sums carry ~1e-13.  A term of 1e30 or more, or not
// finite, sets *bad and the caller keeps the exact path.
template<int EA>
__global__ void gram_terms_kernel(GroupParams g, long long pool_size, float2* P, int* bad)
{
  constexpr int n = EA + 1, NP = n * (n + 1) / 2 + n;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= pool_size)
    return;
  const int row = g.lib_rows[i];
  double u[n];
  u[0] = 1.0;
#pragma unroll
  for (int j = 1; j < n; j++)
    u[j] = g.F[(size_t)row * EA + j - 1];
  const double t = g.lib_target[row];
  float2* out = P + (size_t)i * NP;
  int e = 0;
  bool ok = true;
  auto put = [&](double v) {
    const float hi = (float)v;
    const float lo = (float)(v - (double)hi);
    ok = ok && fabs(v) < 1e30;
    out[e++] = make_float2(hi, lo);
  };
#pragma unroll
  for (int a = 0; a < n; a++)
#pragma unroll
    for (int b = a; b < n; b++)
      put(u[a] * u[b]);
#pragma unroll
  for (int a = 0; a < n; a++)
    put(t * u[a]);
  if (!ok)
    atomicExch(bad, 1);
}

// Once per point for every theta: the mean distance (a warp reduction, not
// the reference's sequential sum: this path is not bit-exact anyway) and the
// distances in FP32 (-1: not a neighbour).
__global__ void all_df_prep_kernel(GroupParams g, ChunkBuffers c, long long max_nlib, float* rdist, double* means,
                                   float* dmin)
{
  const int lane = threadIdx.x & 31;
  const long long q = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long chunk = c.p_end - c.p_begin;
  if (q >= chunk)
    return;
  const long long p = point_of(c, q);
  const DevTask T = g.tasks[find_task(g, p)];
  if (dmin && lane == 0)
    dmin[q] = INFINITY;  // no neighbour (set below otherwise)
  if (!T.all_mode || c.status[q] != PT_OK)
    return;
  const double* dq = c.scratch + q * max_nlib;
  float* rq = rdist + q * max_nlib;
  double sum = 0;
  float mn = INFINITY;
  for (int i = lane; i < T.n_lib; i += 32) {
    const double d = dq[i];
    const float f = d >= 0 ? (float)d : -1.f;
    rq[i] = f;
    if (d >= 0) {
      sum += d;
      mn = fminf(mn, f);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    sum += __shfl_xor_sync(FULL, sum, o);
    mn = fminf(mn, __shfl_xor_sync(FULL, mn, o));
  }
  if (lane == 0) {
    means[q] = sum / (double)c.nn_count[q];
    if (dmin)
      dmin[q] = mn;
  }
}

// The solve of the tensor-core sums (kernels_gram_tc.cu): per (point,
// theta), the normal equations from G, the FP64 JacobiSVD, the forecast.
template<int EA>
__global__ void __launch_bounds__(128) all_smap_gram_kernel(GroupParams g, ChunkBuffers c, const double* G)
{
  constexpr int n = EA + 1;
  const long long chunk = c.p_end - c.p_begin;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= chunk * g.n_thetas)
    return;
  const long long q = idx / g.n_thetas;
  const int t = (int)(idx - q * g.n_thetas);
  const long long p = point_of(c, q);
  const DevTask T = g.tasks[find_task(g, p)];
  if (!T.all_mode)
    return;
  const int st = c.status[q];
  if (st != PT_OK) {
    early_rc(g, T.task, st, t);
    return;
  }
  const double* gr = G + (size_t)idx * 32;
  double Wl[n * n], bv[n], U[n * n], V[n * n], sv[n], tmp[n], xs[n];
  int e = 0;
#pragma unroll
  for (int a = 0; a < n; a++)
#pragma unroll
    for (int b = a; b < n; b++) {
      Wl[a * n + b] = gr[e];
      Wl[b * n + a] = gr[e];
      e++;
    }
#pragma unroll
  for (int a = 0; a < n; a++)
    bv[a] = gr[e++];
  svd_solve(Wl, U, V, sv, tmp, bv, xs, n);
  const int prow = g.pred_rows[T.pred_off + (int)(p - T.point_base)];
  smap_finish(g, T, p, prow, t, xs, n);
}

template<int EA>
__global__ void __launch_bounds__(128) all_smap_df_kernel(GroupParams g, ChunkBuffers c, long long max_nlib,
                                                           const float2* P, const float* rdist, const double* means)
{
  constexpr int n = EA + 1, NA = n * (n + 1) / 2, NP = NA + n;
  const long long chunk = c.p_end - c.p_begin;
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= chunk * g.n_thetas)
    return;
  const long long q = idx / g.n_thetas;
  const int t = (int)(idx - q * g.n_thetas);
  const long long p = point_of(c, q);
  const DevTask T = g.tasks[find_task(g, p)];
  if (!T.all_mode)
    return;
  const int st = c.status[q];
  if (st != PT_OK) {
    early_rc(g, T.task, st, t);
    return;
  }
  const float* rq = rdist + q * max_nlib;
  const float c2 = (float)(-2.0 * g.thetas[t] / means[q]);
  float S[NP], Cr[NP];
#pragma unroll
  for (int e = 0; e < NP; e++)
    S[e] = Cr[e] = 0.f;
  const float2* pool = P + (size_t)T.lib_off * NP;
  for (int i = 0; i < T.n_lib; i++) {
    const float d = rq[i];
    if (d < 0.f)
      continue;
    const float om = expf(__fmul_rn(c2, d));
    const float2* pr = pool + (size_t)i * NP;
#pragma unroll
    for (int e = 0; e < NP; e++) {
      const float2 v = pr[e];
      const float prod = __fmul_rn(om, v.x);
      const float perr = __fmaf_rn(om, v.x, -prod);  // om * hi = prod + perr exactly
      const float s = __fadd_rn(S[e], prod);
      const float bp = __fsub_rn(s, S[e]);
      const float ds = __fadd_rn(__fsub_rn(S[e], __fsub_rn(s, bp)), __fsub_rn(prod, bp));  // S + prod = s + ds exactly
      S[e] = s;
      Cr[e] = __fadd_rn(Cr[e], __fadd_rn(ds, __fmaf_rn(om, v.y, perr)));
    }
  }
  double Wl[n * n], bv[n], U[n * n], V[n * n], sv[n], tmp[n], xs[n];
  int e = 0;
#pragma unroll
  for (int a = 0; a < n; a++)
#pragma unroll
    for (int b = a; b < n; b++) {
      const double v = (double)S[e] + (double)Cr[e];
      Wl[a * n + b] = v;
      Wl[b * n + a] = v;
      e++;
    }
#pragma unroll
  for (int a = 0; a < n; a++) {
    bv[a] = (double)S[e] + (double)Cr[e];
    e++;
  }
  svd_solve(Wl, U, V, sv, tmp, bv, xs, n);
  const int prow = g.pred_rows[T.pred_off + (int)(p - T.point_base)];
  smap_finish(g, T, p, prow, t, xs, n);
}

// ----------------------------------------------------------------- stats
// rho and MAE per (task, theta) over forecasts whose target is observed
// (src/edm.cpp:441-467, src/stats.cpp:64-94).  Two passes like the
// reference's centred correlation.
__global__ void stats_kernel(GroupParams g, double* rho, double* mae)
{
  __shared__ double red[5][256];
  const int ti = blockIdx.x / g.n_thetas, t = blockIdx.x % g.n_thetas;
  const DevTask T = g.tasks[ti];
  const double* pr = g.pred + (size_t)t * g.total_points + T.point_base;
  double c = 0, s1 = 0, s2 = 0, sa = 0;
  for (int i = threadIdx.x; i < T.n_pred; i += blockDim.x) {
    const double y1 = g.pred_target[g.pred_rows[T.pred_off + i]], y2 = pr[i];
    if (y1 != MISS && y2 != MISS) {
      c += 1;
      s1 += y1;
      s2 += y2;
      sa += fabs(y1 - y2);
    }
  }
  red[0][threadIdx.x] = c;
  red[1][threadIdx.x] = s1;
  red[2][threadIdx.x] = s2;
  red[3][threadIdx.x] = sa;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int v = 0; v < 4; v++)
        red[v][threadIdx.x] += red[v][threadIdx.x + o];
    __syncthreads();
  }
  const double cnt = red[0][0], m1 = red[1][0] / cnt, m2 = red[2][0] / cnt, sabs = red[3][0];
  __syncthreads();
  double s11 = 0, s22 = 0, s12 = 0;
  for (int i = threadIdx.x; i < T.n_pred; i += blockDim.x) {
    const double y1 = g.pred_target[g.pred_rows[T.pred_off + i]], y2 = pr[i];
    if (y1 != MISS && y2 != MISS) {
      const double a = y1 - m1, b = y2 - m2;
      s11 += a * a;
      s22 += b * b;
      s12 += a * b;
    }
  }
  red[0][threadIdx.x] = s11;
  red[1][threadIdx.x] = s22;
  red[2][threadIdx.x] = s12;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int v = 0; v < 3; v++)
        red[v][threadIdx.x] += red[v][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double r = MISS, m = MISS;
    if (cnt > 0) {
      const double sd1 = sqrt(red[0][0]), sd2 = sqrt(red[1][0]);
      r = (sd1 < 1e-9 || sd2 < 1e-9) ? MISS : red[2][0] / (sd1 * sd2);
      const double v = sabs / cnt;
      m = v < 1e-8 ? 0 : v;
    }
    rho[T.task * g.n_thetas + t] = r;
    mae[T.task * g.n_thetas + t] = m;
  }
}

int knn_warps_per_block(int Ea, int kcap, int& per_warp)
{
  per_warp = ((Ea * 8 + kcap * 12) + 15) / 16 * 16;
  int w = 8;
  while (w > 1 && (long long)w * per_warp > 200 * 1024)
    w >>= 1;
  return w;
}

int all_warps_per_block(int Ea, int& per_warp)
{
  per_warp = (Ea * 8 + 15) / 16 * 16;
  return 8;
}

} // namespace

void launch_knn_exact(const GroupParams& g, const ChunkBuffers& c, int num_sms, cudaStream_t s)
{
  int per_warp;
  const int w = knn_warps_per_block(g.Ea, c.kcap, per_warp);
  const size_t smem = (size_t)w * per_warp;
  auto kern = g.wasserstein ? knn_exact_kernel<true> : knn_exact_kernel<false>;
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const long long chunk = c.p_end - c.p_begin;
  long long blocks = (chunk + w - 1) / w;
  const long long cap = (long long)num_sms * 64;
  if (blocks > cap)
    blocks = cap;
  if (blocks < 1)
    blocks = 1;
  kern<<<(int)blocks, 32 * w, smem, s>>>(g, c, w, per_warp);
}

template<int EA>
void launch_refine_ea(const GroupParams& g, const ChunkBuffers& c, const RefineRun& r, int blocks, cudaStream_t s)
{
  constexpr size_t smem = refine_smem<EA>();
  cudaFuncSetAttribute(knn_refine_kernel<EA>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  knn_refine_kernel<EA><<<blocks, 32 * REFINE_WARPS, smem, s>>>(g, c, r);
}

void launch_knn_refine(const GroupParams& g, const ChunkBuffers& c, const RefineRun& r, int num_sms, cudaStream_t s)
{
  const long long chunk = c.p_end - c.p_begin;
  if (chunk <= 0)
    return;
  long long blocks = (chunk + REFINE_WARPS - 1) / REFINE_WARPS;
  const long long cap = (long long)num_sms * 2;  // 113 KB of shared memory per CTA at E_a = 16
  if (blocks > cap)
    blocks = cap;
  const int b = (int)blocks;
  switch (g.Ea) {
    case 1: launch_refine_ea<1>(g, c, r, b, s); break;
    case 2: launch_refine_ea<2>(g, c, r, b, s); break;
    case 3: launch_refine_ea<3>(g, c, r, b, s); break;
    case 4: launch_refine_ea<4>(g, c, r, b, s); break;
    case 5: launch_refine_ea<5>(g, c, r, b, s); break;
    case 6: launch_refine_ea<6>(g, c, r, b, s); break;
    case 7: launch_refine_ea<7>(g, c, r, b, s); break;
    case 8: launch_refine_ea<8>(g, c, r, b, s); break;
    case 9: launch_refine_ea<9>(g, c, r, b, s); break;
    case 10: launch_refine_ea<10>(g, c, r, b, s); break;
    case 11: launch_refine_ea<11>(g, c, r, b, s); break;
    case 12: launch_refine_ea<12>(g, c, r, b, s); break;
    case 13: launch_refine_ea<13>(g, c, r, b, s); break;
    case 14: launch_refine_ea<14>(g, c, r, b, s); break;
    case 15: launch_refine_ea<15>(g, c, r, b, s); break;
    case 16: launch_refine_ea<16>(g, c, r, b, s); break;
    default: break;
  }
}

void launch_simplex_nn(const GroupParams& g, const ChunkBuffers& c, cudaStream_t s)
{
  const long long total = (c.p_end - c.p_begin) * g.n_thetas;
  if (total <= 0)
    return;
  simplex_nn_kernel<<<(int)((total + 255) / 256), 256, 0, s>>>(g, c);
}

long long smap_nn_scratch_doubles(int num_sms, int n, int kcap)
{
  (void)kcap;
  if (n <= SMALL_N)
    return 0;
  const long long slab = 3LL * n * n + 4LL * n;
  return (long long)num_sms * 4 * 128 * slab;
}

void launch_smap_nn(const GroupParams& g, const ChunkBuffers& c, int num_sms, cudaStream_t s)
{
  const int n = g.Ea + 1;
  const long long slab = 3LL * n * n + 4LL * n;
  const long long total = (c.p_end - c.p_begin) * g.n_thetas;
  if (total <= 0)
    return;
  long long blocks = (total + 127) / 128;
  if (n > SMALL_N) {
    const long long cap = c.scratch_doubles / (128 * slab);
    if (blocks > cap)
      blocks = cap;
  } else if (blocks > (long long)num_sms * 64) {
    blocks = (long long)num_sms * 64;
  }
  if (blocks < 1)
    blocks = 1;
  smap_nn_kernel<<<(int)blocks, 128, 0, s>>>(g, c, slab);
}

long long all_mode_slab(int Ea)
{
  const int n = Ea + 1;
  return 3LL * n * n + 4LL * n;
}

int gram_terms_per_row(int Ea)
{
  const int n = Ea + 1;
  return n * (n + 1) / 2 + n;
}

void launch_gram_terms(const GroupParams& g, long long pool_size, float2* P, int* bad, cudaStream_t s)
{
  if (pool_size <= 0)
    return;
  const int b = (int)((pool_size + 127) / 128);
  switch (g.Ea) {
    case 1: gram_terms_kernel<1><<<b, 128, 0, s>>>(g, pool_size, P, bad); break;
    case 2: gram_terms_kernel<2><<<b, 128, 0, s>>>(g, pool_size, P, bad); break;
    case 3: gram_terms_kernel<3><<<b, 128, 0, s>>>(g, pool_size, P, bad); break;
    case 4: gram_terms_kernel<4><<<b, 128, 0, s>>>(g, pool_size, P, bad); break;
    case 5: gram_terms_kernel<5><<<b, 128, 0, s>>>(g, pool_size, P, bad); break;
    case 6: gram_terms_kernel<6><<<b, 128, 0, s>>>(g, pool_size, P, bad); break;
    case 7: gram_terms_kernel<7><<<b, 128, 0, s>>>(g, pool_size, P, bad); break;
    case 8: gram_terms_kernel<8><<<b, 128, 0, s>>>(g, pool_size, P, bad); break;
    default: break;
  }
}

namespace {

void launch_forecast(const GroupParams& g, const ChunkBuffers& c, long long max_nlib, cudaStream_t s,
                     const float2* gram_terms, float* rdist, double* means, const GramTC* tc, int tc_tiles,
                     float* dmin)
{
  const long long chunk = c.p_end - c.p_begin;
  const long long total = chunk * g.n_thetas;
  const int fb = (int)((total + 127) / 128);
  if (g.algorithm == 1 && tc && tc_tiles > 0 && rdist && means && dmin && gram_tc_supported(g.Ea)) {
    all_df_prep_kernel<<<(int)((chunk * 32 + 127) / 128), 128, 0, s>>>(g, c, max_nlib, rdist, means, dmin);
    launch_gram_tc(*tc, tc_tiles, s);
    switch (g.Ea) {
      case 1: all_smap_gram_kernel<1><<<fb, 128, 0, s>>>(g, c, tc->G); return;
      case 2: all_smap_gram_kernel<2><<<fb, 128, 0, s>>>(g, c, tc->G); return;
      case 3: all_smap_gram_kernel<3><<<fb, 128, 0, s>>>(g, c, tc->G); return;
      case 4: all_smap_gram_kernel<4><<<fb, 128, 0, s>>>(g, c, tc->G); return;
      case 5: all_smap_gram_kernel<5><<<fb, 128, 0, s>>>(g, c, tc->G); return;
      default: break;
    }
  }
  if (g.algorithm == 1 && g.Ea <= 8 && gram_terms && rdist && means) {
    all_df_prep_kernel<<<(int)((chunk * 32 + 127) / 128), 128, 0, s>>>(g, c, max_nlib, rdist, means, nullptr);
    switch (g.Ea) {
      case 1: all_smap_df_kernel<1><<<fb, 128, 0, s>>>(g, c, max_nlib, gram_terms, rdist, means); return;
      case 2: all_smap_df_kernel<2><<<fb, 128, 0, s>>>(g, c, max_nlib, gram_terms, rdist, means); return;
      case 3: all_smap_df_kernel<3><<<fb, 128, 0, s>>>(g, c, max_nlib, gram_terms, rdist, means); return;
      case 4: all_smap_df_kernel<4><<<fb, 128, 0, s>>>(g, c, max_nlib, gram_terms, rdist, means); return;
      case 5: all_smap_df_kernel<5><<<fb, 128, 0, s>>>(g, c, max_nlib, gram_terms, rdist, means); return;
      case 6: all_smap_df_kernel<6><<<fb, 128, 0, s>>>(g, c, max_nlib, gram_terms, rdist, means); return;
      case 7: all_smap_df_kernel<7><<<fb, 128, 0, s>>>(g, c, max_nlib, gram_terms, rdist, means); return;
      case 8: all_smap_df_kernel<8><<<fb, 128, 0, s>>>(g, c, max_nlib, gram_terms, rdist, means); return;
      default: break;
    }
  }
  if (g.algorithm == 1 && g.Ea <= 8) {
    all_ratio_kernel<<<(int)((chunk + 127) / 128), 128, 0, s>>>(g, c, max_nlib);
    switch (g.Ea) {
      case 1: all_smap_kernel<1><<<fb, 128, 0, s>>>(g, c, max_nlib); return;
      case 2: all_smap_kernel<2><<<fb, 128, 0, s>>>(g, c, max_nlib); return;
      case 3: all_smap_kernel<3><<<fb, 128, 0, s>>>(g, c, max_nlib); return;
      case 4: all_smap_kernel<4><<<fb, 128, 0, s>>>(g, c, max_nlib); return;
      case 5: all_smap_kernel<5><<<fb, 128, 0, s>>>(g, c, max_nlib); return;
      case 6: all_smap_kernel<6><<<fb, 128, 0, s>>>(g, c, max_nlib); return;
      case 7: all_smap_kernel<7><<<fb, 128, 0, s>>>(g, c, max_nlib); return;
      case 8: all_smap_kernel<8><<<fb, 128, 0, s>>>(g, c, max_nlib); return;
      default: break;
    }
  }
  all_forecast_kernel<<<fb, 128, 0, s>>>(g, c, max_nlib, all_mode_slab(g.Ea));
}

} // namespace

void launch_all_mode(const GroupParams& g, const ChunkBuffers& c, int num_sms, long long max_nlib, cudaStream_t s,
                     const float2* gram_terms, float* rdist, double* means, cudaEvent_t ev0, cudaEvent_t ev1,
                     const GramTC* tc, int tc_tiles, float* dmin)
{
  int per_warp;
  const int w = all_warps_per_block(g.Ea, per_warp);
  const long long chunk = c.p_end - c.p_begin;
  long long blocks = (chunk + w - 1) / w;
  if (blocks > (long long)num_sms * 64)
    blocks = (long long)num_sms * 64;
  if (blocks < 1)
    blocks = 1;
  // the Wasserstein distance is reached only through the task seam, which
  // sends every task through the neighbour-list path (knn_exact_kernel)
  all_dist_kernel<<<(int)blocks, 32 * w, (size_t)w * per_warp, s>>>(g, c, max_nlib, per_warp);
  if (chunk * g.n_thetas <= 0)
    return;
  if (ev0)
    cudaEventRecord(ev0, s);
  launch_forecast(g, c, max_nlib, s, gram_terms, rdist, means, tc, tc_tiles, dmin);
  if (ev1)
    cudaEventRecord(ev1, s);
}

void launch_stats(const GroupParams& g, const DevTask*, int n_tasks, double* rho, double* mae, cudaStream_t s)
{
  if (n_tasks <= 0)
    return;
  stats_kernel<<<n_tasks * g.n_thetas, 256, 0, s>>>(g, rho, mae);
}

} // namespace fedm
