// xform.cu -- world-matrix propagation of the transform tree on the GPU.
//
// The reference (dp/transform/src/Tree.cpp:133-166) walks its level lists in order and,
// for every (parent, transform) entry whose parent world matrix was recomputed in this
// pass or whose local matrix is dirty, sets world = local * parentWorld and marks the
// world matrix dirty.  Here the host splits the level lists into segments in which no
// entry reads a matrix that another entry of the same segment writes; all entries of a
// segment then run in parallel, one thread per entry.  Small consecutive segments run
// inside one CTA separated by __syncthreads (one launch for the narrow top of the tree);
// wide segments get a grid of their own.  Products use the reference's operation order
// (Matmnt.h:1381-1415), so world matrices are bit-identical to the CPU tree.
#include <cuda_runtime.h>

#include "dpcull_exact.cuh"
#include "dpcull_internal.h"

namespace dpcull {

namespace {

__device__ __forceinline__ void propagate_entry(const XformLaunch& a, uint32_t e)
{
  const uint2 pt = a.entries[e];
  const uint32_t p = pt.x, t = pt.y;
  const bool dw = (a.dirty_world[p >> 5] >> (p & 31)) & 1u;
  const bool dl = (__ldg(a.dirty_local + (t >> 5)) >> (t & 31)) & 1u;
  if (!(dw || dl)) return;
  const float4* L = reinterpret_cast<const float4*>(a.local) + 4 * (size_t)t;
  const float4* P = reinterpret_cast<const float4*>(a.world) + 4 * (size_t)p;
  float4* W = reinterpret_cast<float4*>(a.world) + 4 * (size_t)t;
  const float4 p0 = P[0], p1 = P[1], p2 = P[2], p3 = P[3];
#pragma unroll
  for (int r = 0; r < 4; ++r) W[r] = vec4_mul_mat44(__ldg(L + r), p0, p1, p2, p3);
  atomicOr(a.dirty_world + (t >> 5), 1u << (t & 31));
}

__global__ void xform_segment_kernel(const XformLaunch a, uint32_t begin, uint32_t end)
{
  for (uint32_t e = begin + blockIdx.x * blockDim.x + threadIdx.x; e < end;
       e += gridDim.x * blockDim.x)
    propagate_entry(a, e);
}

// One CTA walks segments [s0, s1); __syncthreads orders the levels (global writes of a
// block are visible to the whole block after the barrier).
__global__ void xform_segments_cta_kernel(const XformLaunch a, uint32_t s0, uint32_t s1)
{
  for (uint32_t s = s0; s < s1; ++s) {
    const uint32_t begin = a.seg[s], end = a.seg[s + 1];
    for (uint32_t e = begin + threadIdx.x; e < end; e += blockDim.x) propagate_entry(a, e);
    __syncthreads();
  }
}

// dst[idx[i]] = src[i] for 64-byte matrices; optionally marks idx[i] in a dirty bit array
// (Tree::updateLocalMatrix, Tree.h:87, on the device copy).
__global__ void scatter_matrices_kernel(float4* dst, const float4* src, const uint32_t* idx,
                                        uint32_t k, uint32_t* dirty)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 4 * k) return;
  const uint32_t m = i >> 2, r = i & 3;
  const uint32_t t = idx[m];
  dst[4 * (size_t)t + r] = src[4 * (size_t)m + r];
  if (dirty && r == 0) atomicOr(dirty + (t >> 5), 1u << (t & 31));
}

// SoA object rows: soa[row][idx[i]] = src[row][i] for the 7 rows (lower xyz, extent xyz,
// transform index), src being 7 planar rows of k entries.
__global__ void scatter_objects_kernel(float* soa, uint32_t cap, const float* src,
                                       const uint32_t* idx, uint32_t k)
{
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= k) return;
  const uint32_t o = idx[i];
#pragma unroll
  for (int r = 0; r < 7; ++r) soa[(size_t)r * cap + o] = src[(size_t)r * k + i];
}

}  // namespace

int launch_xform_cta(const XformLaunch& a, uint32_t s0, uint32_t s1, void* stream)
{
  if (s1 <= s0) return 0;
  xform_segments_cta_kernel<<<1, 1024, 0, static_cast<cudaStream_t>(stream)>>>(a, s0, s1);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_xform_range(const XformLaunch& a, uint32_t begin, uint32_t end, void* stream)
{
  if (end <= begin) return 0;
  const uint32_t n = end - begin;
  const int threads = 256;
  const int grid = (int)((n + threads - 1) / threads);
  xform_segment_kernel<<<grid, threads, 0, static_cast<cudaStream_t>(stream)>>>(a, begin, end);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_scatter_matrices(float* dst, const float* src, const uint32_t* idx, uint32_t k,
                            uint32_t* dirty_bits, void* stream)
{
  if (!k) return 0;
  const uint32_t n = 4 * k;
  scatter_matrices_kernel<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      reinterpret_cast<float4*>(dst), reinterpret_cast<const float4*>(src), idx, k, dirty_bits);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_scatter_objects(float* soa, uint32_t cap, const float* src, const uint32_t* idx,
                           uint32_t k, void* stream)
{
  if (!k) return 0;
  scatter_objects_kernel<<<(k + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      soa, cap, src, idx, k);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace dpcull
