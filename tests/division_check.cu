// Checks the solver's shared-reciprocal division (dvd_r in smap_solve.cuh)
// against IEEE division (__ddiv_rn) bit for bit on random operands: for each
// exponent range +-E given on the command line, 2^32 pairs with random
// mantissas and signs.  Prints one line per range and exits non-zero on any
// difference.  Built and run by tests/test_gpu_division.py.
#include <cstdio>
#include <cstdlib>
#include <cstdint>
#include <cuda_runtime.h>

#include "smap_solve.cuh"

namespace {

__device__ __forceinline__ uint64_t mix(uint64_t x)
{
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdULL;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ULL;
  x ^= x >> 33;
  return x;
}

__device__ __forceinline__ double operand(uint64_t s, int e)
{
  const uint64_t h = mix(s);
  const int ex = (int)(h % (uint64_t)(2 * e + 1)) - e;
  const uint64_t man = mix(h) & ((1ULL << 52) - 1);
  return __longlong_as_double((long long)(((uint64_t)(ex + 1023) << 52) | man | ((h >> 63) << 63)));
}

__global__ void compare(uint64_t seed, long long n, int e, unsigned long long* diff)
{
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double a = operand(seed + 2 * i, e), b = operand(seed + 2 * i + 1, e);
    if (__double_as_longlong(__ddiv_rn(a, b)) != __double_as_longlong(fedm::dvd_r(a, b, fedm::rcp(b))))
      atomicAdd(diff, 1ULL);
  }
}

} // namespace

int main(int argc, char** argv)
{
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0) != cudaSuccess)
    return 2;
  unsigned long long* d = nullptr;
  cudaMalloc(&d, 8);
  unsigned long long total = 0;
  for (int a = 1; a < argc; a++) {
    const int e = std::atoi(argv[a]);
    cudaMemset(d, 0, 8);
    const long long n = 1LL << 32;
    compare<<<sms * 8, 256>>>(0x9e3779b97f4a7c15ULL + (uint64_t)e, n, e, d);
    unsigned long long h = 0;
    if (cudaMemcpy(&h, d, 8, cudaMemcpyDeviceToHost) != cudaSuccess)
      return 2;
    printf("exponents within +-%d: %lld pairs, %llu differ\n", e, n, h);
    total += h;
  }
  cudaFree(d);
  return total == 0 ? 0 : 1;
}
