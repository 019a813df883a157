// Every float x in [2^-120, 2^127): sqrt.approx.f32(x) against the root of x computed in
// double (correctly rounded to 53 bits).  Prints the largest relative error and how many
// x violate r * (1 + 2^-18) >= sqrt(x), the upper bound the cull's prefilter relies on.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <cuda_runtime.h>

__global__ void check(unsigned long long first, unsigned long long count, unsigned int* max_err_bits,
                      unsigned long long* violations)
{
  unsigned long long local_bad = 0;
  float local_max = 0.f;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < count;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const float x = __uint_as_float((unsigned int)(first + i));
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    const double t = sqrt((double)x);
    const double rel = fabs((double)r - t) / t;
    local_max = fmaxf(local_max, (float)rel);
    if ((double)(r * (1.0f + 0x1p-18f)) < t) ++local_bad;
  }
  atomicMax(max_err_bits, __float_as_uint(local_max));  // non-negative floats order as integers
  if (local_bad) atomicAdd(violations, local_bad);
}

int main()
{
  const unsigned int lo = 0x03800000u;  // 2^-120
  const unsigned int hi = 0x7f800000u;  // +inf (exclusive)
  unsigned int* d_max = nullptr;
  unsigned long long* d_bad = nullptr;
  if (cudaMalloc(&d_max, 4) != cudaSuccess || cudaMalloc(&d_bad, 8) != cudaSuccess) return 2;
  cudaMemset(d_max, 0, 4);
  cudaMemset(d_bad, 0, 8);
  check<<<152 * 8, 256>>>(lo, (unsigned long long)(hi - lo), d_max, d_bad);
  unsigned int m = 0;
  unsigned long long bad = 0;
  if (cudaMemcpy(&m, d_max, 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(&bad, d_bad, 8, cudaMemcpyDeviceToHost) != cudaSuccess)
    return 3;
  float me;
  memcpy(&me, &m, 4);
  printf("inputs=%u max_rel_err=%.9g log2=%.3f violations=%llu\n", hi - lo, me, me > 0 ? log2(me) : -999.0, bad);
  return 0;
}
