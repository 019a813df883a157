// xform.cu -- world-matrix propagation of the transform tree on the GPU.
//
// The reference (dp/transform/src/Tree.cpp:133-166) walks its level lists in order and,
// for every (parent, transform) entry whose parent world matrix was recomputed in this
// pass or whose local matrix is dirty, sets world = local * parentWorld and marks the
// world matrix dirty.  Here the host splits the level lists into segments in which no
// entry reads a matrix that another entry of the same segment writes; all entries of a
// segment then run in parallel, one thread per entry.  Small consecutive segments run
// inside one CTA separated by __syncthreads (one launch for the narrow top of the tree);
// wide segments get a grid of their own.  dpcull_tree_compute runs all of it as one
// cooperative launch (xform_tree_kernel): the narrow segments in block 0, the wide ones
// over the grid, a bounded grid barrier between the steps.  Products use the reference's
// operation order (Matmnt.h:1381-1415), so world matrices are bit-identical to the CPU
// tree.
#include <algorithm>
#include <atomic>

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

// The same inside the cooperative tree kernel, whose blocks read matrices and dirty bits
// that other blocks wrote earlier in the launch: those reads go to L2 (a matrix can be
// read in one segment and rewritten in a later one, so an L1 line could be stale).
__device__ __forceinline__ void propagate_entry_l2(const XformLaunch& a, uint32_t e)
{
  const uint2 pt = __ldg(a.entries + e);
  const uint32_t p = pt.x, t = pt.y;
  const bool dw = (__ldcg(a.dirty_world + (p >> 5)) >> (p & 31)) & 1u;
  const bool dl = (__ldg(a.dirty_local + (t >> 5)) >> (t & 31)) & 1u;
  if (!(dw || dl)) return;
  const float4* L = reinterpret_cast<const float4*>(a.local) + 4 * (size_t)t;
  const float4* P = reinterpret_cast<const float4*>(a.world) + 4 * (size_t)p;
  float4* W = reinterpret_cast<float4*>(a.world) + 4 * (size_t)t;
  const float4 p0 = __ldcg(P + 0), p1 = __ldcg(P + 1), p2 = __ldcg(P + 2), p3 = __ldcg(P + 3);
#pragma unroll
  for (int r = 0; r < 4; ++r) __stcg(W + r, vec4_mul_mat44(__ldg(L + r), p0, p1, p2, p3));
  atomicOr(a.dirty_world + (t >> 5), 1u << (t & 31));
}

constexpr uint32_t kBarrierSpins = 1u << 22;  // polls of the barrier generation (~0.3 s)

// Grid barrier of a cooperative launch (every block is resident): each block's thread 0
// arrives with one atomic; the last one resets the count and advances the generation the
// others wait on.  A wait is bounded: a block that gives up records kErrWaitTimeout and
// goes on (its results are then not to be trusted, and the host reports the error).
__device__ __forceinline__ void grid_barrier(unsigned int* bar, unsigned int* err)
{
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int* gen = bar + 1;
    const unsigned int g = *gen;
    __threadfence();  // this block's writes before its arrival
    if (atomicAdd(bar, 1u) == gridDim.x - 1) {
      *(volatile unsigned int*)bar = 0u;
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      for (uint32_t spins = 0; *gen == g; ++spins) {
        if (spins == kBarrierSpins) {
          atomicOr(err, kErrWaitTimeout);
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
  }
  __syncthreads();
}

constexpr int kTreeThreads = 256;

__global__ void __launch_bounds__(kTreeThreads)
    xform_tree_kernel(const XformLaunch a, const uint4* sched, uint32_t n_sched, uint32_t words,
                      unsigned int* bar, unsigned int* err)
{
  const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x, gstride = gridDim.x * blockDim.x;
  for (uint32_t i = gtid; i < words; i += gstride) a.dirty_world[i] = 0u;
  grid_barrier(bar, err);
  for (uint32_t k = 0; k < n_sched; ++k) {
    const uint4 L = __ldg(sched + k);
    if (L.x) {  // narrow segments: block 0 alone, a block barrier between them
      if (blockIdx.x == 0) {
        for (uint32_t s = L.y; s < L.z; ++s) {
          const uint32_t begin = __ldg(a.seg + s), end = __ldg(a.seg + s + 1);
          for (uint32_t e = begin + threadIdx.x; e < end; e += blockDim.x) propagate_entry_l2(a, e);
          __syncthreads();
        }
      }
    } else {
      for (uint32_t e = L.y + gtid; e < L.z; e += gstride) propagate_entry_l2(a, e);
    }
    grid_barrier(bar, err);
  }
  // every entry has read its dirty-local bit
  for (uint32_t i = gtid; i < words; i += gstride) a.dirty_local[i] = 0u;
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

int launch_xform_tree(const XformLaunch& a, const uint4* sched, uint32_t n_sched, uint32_t words,
                      uint32_t max_wide, unsigned int* bar, unsigned int* err, int sm_count, void* stream)
{
  static std::atomic<int> occ_cached{0};  // the same on every GB300
  int occ = occ_cached.load(std::memory_order_relaxed);
  if (!occ) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, xform_tree_kernel, kTreeThreads, 0) != cudaSuccess ||
        occ < 1)
      return -1;
    occ_cached.store(occ, std::memory_order_relaxed);
  }
  const uint32_t need = std::max<uint32_t>(1, (std::max(max_wide, words) + kTreeThreads - 1) / kTreeThreads);
  const unsigned grid = std::min<unsigned>((unsigned)(occ * std::max(sm_count, 1)), need);
  XformLaunch la = a;
  void* args[] = {&la, &sched, &n_sched, &words, &bar, &err};
  if (cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(xform_tree_kernel), dim3(grid), dim3(kTreeThreads),
                                  args, 0, static_cast<cudaStream_t>(stream)) != cudaSuccess)
    return -1;
  return 0;
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
