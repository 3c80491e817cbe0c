// Small device helpers: fills, and the peak probes of the roofline.
#include <cuda_runtime.h>

namespace fedm {

namespace {

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
