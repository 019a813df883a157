// fma.rn.f32x2 against two fma.rn.f32: the cull evaluates the lo and hi plane of an axis
// as one packed pair and relies on each half rounding exactly like the scalar FMA chain
// the host test checks.  Seeded pseudo-random triples in four families (any bit pattern,
// normal values over a wide exponent range, near-cancelling c = -a*b, subnormal-heavy);
// prints how many halves differ (NaN results count as equal when both are NaN).
#include <cstdio>
#include <cuda_runtime.h>

__device__ __forceinline__ unsigned long long mix(unsigned long long z)
{
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ float pick(unsigned long long r, int family)
{
  const unsigned int u = (unsigned int)r;
  switch (family) {
    case 0:  // any bit pattern: NaN, infinities, subnormals included
      return __uint_as_float(u);
    case 1: {  // normal values, exponents -40..40
      const unsigned int e = 127u - 40u + (unsigned int)((r >> 32) % 81u);
      return __uint_as_float((u & 0x807fffffu) | (e << 23));
    }
    default: {  // around the subnormal range, exponents -150..-100
      const unsigned int e = (unsigned int)((r >> 32) % 28u);
      return __uint_as_float((u & 0x807fffffu) | (e << 23));
    }
  }
}

__device__ __forceinline__ bool same(float x, float y)
{
  return (__float_as_uint(x) == __float_as_uint(y)) || (x != x && y != y);
}

__global__ void check(unsigned long long count, unsigned long long* mismatches)
{
  unsigned long long bad = 0;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < count;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const int family = (int)(i & 3u);
    float a[2], b[2], c[2];
    for (int h = 0; h < 2; ++h) {
      const unsigned long long s = mix(i * 8u + (unsigned long long)h * 3u);
      const int f = family == 2 ? 1 : family == 3 ? 2 : family;
      a[h] = pick(s, f);
      b[h] = pick(mix(s), f);
      if (family == 2) {  // near-cancelling addend: -(a*b) nudged by a few units
        const float p = a[h] * b[h];
        c[h] = __uint_as_float(__float_as_uint(-p) + (unsigned int)(mix(s + 1) % 7u) - 3u);
      } else {
        c[h] = pick(mix(s + 2), f);
      }
    }
    unsigned long long pa, pb, pc, pd;
    asm("mov.b64 %0, {%1, %2};" : "=l"(pa) : "f"(a[0]), "f"(a[1]));
    asm("mov.b64 %0, {%1, %2};" : "=l"(pb) : "f"(b[0]), "f"(b[1]));
    asm("mov.b64 %0, {%1, %2};" : "=l"(pc) : "f"(c[0]), "f"(c[1]));
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(pd) : "l"(pa), "l"(pb), "l"(pc));
    float d0, d1;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(d0), "=f"(d1) : "l"(pd));
    if (!same(d0, __fmaf_rn(a[0], b[0], c[0]))) ++bad;
    if (!same(d1, __fmaf_rn(a[1], b[1], c[1]))) ++bad;
  }
  if (bad) atomicAdd(mismatches, bad);
}

int main()
{
  const unsigned long long count = 1ull << 28;
  unsigned long long* d_bad = nullptr;
  if (cudaMalloc(&d_bad, 8) != cudaSuccess) return 2;
  cudaMemset(d_bad, 0, 8);
  check<<<152 * 8, 256>>>(count, d_bad);
  unsigned long long bad = 0;
  if (cudaMemcpy(&bad, d_bad, 8, cudaMemcpyDeviceToHost) != cudaSuccess) return 3;
  printf("pairs=%llu mismatches=%llu\n", count, bad);
  return 0;
}
