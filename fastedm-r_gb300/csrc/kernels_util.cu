// Small device helpers: fills, the bounding boxes of spatially ordered
// library sub-tiles, and the peak probes of the roofline.
#include <cuda_runtime.h>

#include "kernels.h"

namespace fedm {

namespace {

// One CTA of 256 threads per sub-tile: each thread takes rows i = tid,
// tid + 256, ... of it and keeps (min, max) per coordinate; a warp-shuffle
// and a shared-memory reduction give the sub-tile's box.  min and max of
// float values are exact, so every row of the sub-tile lies in its box.
__global__ void __launch_bounds__(256) tile_box_kernel(const int* lib_rows, const int* scan_pos, const float* F32,
                                                       int rs, int ea, const int4* subtiles, float2* boxes)
{
  constexpr int EMAX = 16;
  const int4 t = subtiles[blockIdx.x];
  __shared__ float s_lo[8][EMAX], s_hi[8][EMAX];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  float lo[EMAX], hi[EMAX];
#pragma unroll
  for (int j = 0; j < EMAX; j++) {
    lo[j] = INFINITY;
    hi[j] = -INFINITY;
  }
  for (int i = tid; i < t.z; i += 256) {
    const float* r = F32 + (size_t)lib_rows[t.x + scan_pos[t.x + t.y + i]] * rs;
#pragma unroll
    for (int j = 0; j < EMAX; j++)
      if (j < ea) {
        lo[j] = fminf(lo[j], r[j]);
        hi[j] = fmaxf(hi[j], r[j]);
      }
  }
#pragma unroll
  for (int j = 0; j < EMAX; j++) {
    if (j < ea) {
      float a = lo[j], b = hi[j];
      for (int o = 16; o > 0; o >>= 1) {
        a = fminf(a, __shfl_xor_sync(0xffffffffu, a, o));
        b = fmaxf(b, __shfl_xor_sync(0xffffffffu, b, o));
      }
      if (lane == 0) {
        s_lo[w][j] = a;
        s_hi[w][j] = b;
      }
    }
  }
  __syncthreads();
  if (tid < ea) {
    float a = s_lo[0][tid], b = s_hi[0][tid];
    for (int q = 1; q < 8; q++) {
      a = fminf(a, s_lo[q][tid]);
      b = fmaxf(b, s_hi[q][tid]);
    }
    boxes[(size_t)blockIdx.x * ea + tid] = make_float2(a, b);
  }
}

__global__ void fill_f64_kernel(double* p, long long n, double v)
{
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    p[i] = v;
}

__global__ void fill_i32_kernel(int* p, long long n, int v)
{
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    p[i] = v;
}

int grid_for(long long n)
{
  long long b = (n + 255) / 256;
  if (b > 4096)
    b = 4096;
  return b < 1 ? 1 : (int)b;
}

// One CTA of 256 threads per library list (pool offset L.x, L.y entries):
// a counting sort of its positions q by the bucket rank[lib_rows[L.x + q]]
// >> sh (nb buckets), written to scan_pos[L.x ...].  Shared-memory atomics
// make the order within a bucket vary from run to run; the scan that reads
// it gives the same results in any order.
__global__ void __launch_bounds__(256) spatial_order_kernel(const int* lib_rows, const int* rank, int sh, int nb,
                                                            const int2* lists, int* scan_pos)
{
  extern __shared__ int cnt[];  // nb bucket counters, then 256 partial sums
  int* part = cnt + nb;
  const int2 L = lists[blockIdx.x];
  const int tid = threadIdx.x;
  for (int b = tid; b < nb; b += 256)
    cnt[b] = 0;
  __syncthreads();
  for (int q = tid; q < L.y; q += 256)
    atomicAdd(&cnt[rank[lib_rows[L.x + q]] >> sh], 1);
  __syncthreads();
  // exclusive prefix sums: each thread a contiguous chunk of buckets, then
  // the chunks' totals
  const int per = (nb + 255) / 256;
  const int b0 = tid * per, b1 = min(nb, b0 + per);
  int sum = 0;
  for (int b = b0; b < b1; b++)
    sum += cnt[b];
  part[tid] = sum;
  __syncthreads();
  if (tid == 0) {
    int run = 0;
    for (int w = 0; w < 256; w++) {
      const int v = part[w];
      part[w] = run;
      run += v;
    }
  }
  __syncthreads();
  int run = part[tid];
  for (int b = b0; b < b1; b++) {
    const int v = cnt[b];
    cnt[b] = run;
    run += v;
  }
  __syncthreads();
  for (int q = tid; q < L.y; q += 256) {
    const int b = rank[lib_rows[L.x + q]] >> sh;
    scan_pos[L.x + atomicAdd(&cnt[b], 1)] = q;
  }
}

} // namespace

void fill_f64(double* p, long long n, double v, cudaStream_t s)
{
  if (n > 0)
    fill_f64_kernel<<<grid_for(n), 256, 0, s>>>(p, n, v);
}

void fill_i32(int* p, long long n, int v, cudaStream_t s)
{
  if (n > 0)
    fill_i32_kernel<<<grid_for(n), 256, 0, s>>>(p, n, v);
}

void launch_spatial_order(const int* lib_rows, const int* rank, int sh, int nb, const int2* lists, int n_lists,
                          int* scan_pos, cudaStream_t s)
{
  if (n_lists > 0)
    spatial_order_kernel<<<n_lists, 256, (size_t)(nb + 256) * sizeof(int), s>>>(lib_rows, rank, sh, nb, lists,
                                                                                  scan_pos);
}

void launch_tile_boxes(const int* lib_rows, const int* scan_pos, const float* F32, int rs, int ea, const int4* subtiles,
                       int n_subtiles, float2* boxes, cudaStream_t s)
{
  if (n_subtiles > 0 && ea >= 1 && ea <= 16)
    tile_box_kernel<<<n_subtiles, 256, 0, s>>>(lib_rows, scan_pos, F32, rs, ea, subtiles, boxes);
}

} // namespace fedm

// ------------------------------------------------------------ peak probes
// Independent multiply-add chains: FP32 FFMA, packed FP32 FFMA2 and FP64
// DFMA.  Used only to give the roofline its FP32/FP64 denominators.
namespace fedm {

namespace {

__global__ void peak_fp32_kernel(float* out, int iters)
{
  float a[8];
  for (int j = 0; j < 8; j++)
    a[j] = threadIdx.x * 1e-7f + j;
  const float b = 0.999999f, c = 1e-7f;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int j = 0; j < 8; j++)
      a[j] = fmaf(a[j], b, c);
  }
  float s = 0;
  for (int j = 0; j < 8; j++)
    s += a[j];
  if (s == 12345.f)
    out[0] = s;
}

__global__ void peak_fp32x2_kernel(float* out, int iters)
{
  float2 a[4];
  for (int j = 0; j < 4; j++)
    a[j] = make_float2(threadIdx.x * 1e-7f + j, threadIdx.x * 2e-7f + j);
  const float2 b = make_float2(0.999999f, 0.999998f), c = make_float2(1e-7f, 2e-7f);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int j = 0; j < 4; j++)
      a[j] = __ffma2_rn(a[j], b, c);
  }
  float s = 0;
  for (int j = 0; j < 4; j++)
    s += a[j].x + a[j].y;
  if (s == 12345.f)
    out[0] = s;
}

__global__ void peak_fp64_kernel(double* out, int iters)
{
  double a[8];
  for (int j = 0; j < 8; j++)
    a[j] = threadIdx.x * 1e-7 + j;
  const double b = 0.999999, c = 1e-7;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int j = 0; j < 8; j++)
      a[j] = fma(a[j], b, c);
  }
  double s = 0;
  for (int j = 0; j < 8; j++)
    s += a[j];
  if (s == 12345.0)
    out[0] = s;
}

// Separate multiply and add (never contracted): the rate of the FP64 work
// that must keep the reference's unfused operation order.
__global__ void peak_fp64_unfused_kernel(double* out, int iters)
{
  double a[8];
  for (int j = 0; j < 8; j++)
    a[j] = threadIdx.x * 1e-7 + j;
  const double b = 0.999999, c = 1e-7;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int j = 0; j < 8; j++)
      a[j] = __dadd_rn(__dmul_rn(a[j], b), c);
  }
  double s = 0;
  for (int j = 0; j < 8; j++)
    s += a[j];
  if (s == 12345.0)
    out[0] = s;
}

} // namespace

// Returns TFLOP/s (2 flops per multiply-add, fused or not) of the chosen probe.
double measure_peak(int kind, int num_sms, cudaStream_t s)
{
  void* buf = nullptr;
  cudaMalloc(&buf, 64);
  const int threads = 256, blocks = num_sms * 8;
  const int iters = (kind == 1 || kind == 3) ? 2000 : 40000;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = 0;
  for (int rep = 0; rep < 4; rep++) {
    cudaEventRecord(e0, s);
    if (kind == 0)
      peak_fp32_kernel<<<blocks, threads, 0, s>>>((float*)buf, iters);
    else if (kind == 2)
      peak_fp32x2_kernel<<<blocks, threads, 0, s>>>((float*)buf, iters);
    else if (kind == 3)
      peak_fp64_unfused_kernel<<<blocks, threads, 0, s>>>((double*)buf, iters);
    else
      peak_fp64_kernel<<<blocks, threads, 0, s>>>((double*)buf, iters);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    const double flops = 2.0 * 8 * (double)iters * threads * blocks;
    if (rep > 0 && ms > 0)
      best = fmax(best, flops / (ms * 1e-3) / 1e12);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  return best;
}

} // namespace fedm
