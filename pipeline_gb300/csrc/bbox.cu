// bbox.cu -- world-space bounding box of a culling group (Manager::getBoundingBox).
//
// The reference (dp/culling/src/ManagerBitSet.cpp:268-306) walks the objects in group
// order, builds the 8 world-space corners of each box with the same add chain as the
// cull, and folds them into a box with "replace only if strictly smaller / larger"
// (dp/math/Boxnt.h:245-258).  That fold keeps the first of several equal values (it can
// tell -0 from +0) and skips NaN.  The GPU reduction keeps the fold's order: every
// partial covers a contiguous, ordered range of objects and partials are combined left
// to right, where combine(L, R) takes R's bound only if it is strictly beyond L's.  The
// operator is associative, so the result is bit-identical to the sequential fold.
#include <cfloat>

#include <cuda_runtime.h>

#include "dpcull_exact.cuh"
#include "dpcull_internal.h"

namespace dpcull {

namespace {

constexpr int kBoxThreads = 256;
constexpr int kBoxBlocksMax = 1024;

struct Box6 {
  float lo[3], hi[3];
};

__device__ __forceinline__ void box_init(Box6& b)
{
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    b.lo[i] = FLT_MAX;
    b.hi[i] = -FLT_MAX;
  }
}

__device__ __forceinline__ void box_point(Box6& b, float4 p)
{
  const float c[3] = {p.x, p.y, p.z};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    if (b.lo[i] > c[i]) b.lo[i] = c[i];
    if (b.hi[i] < c[i]) b.hi[i] = c[i];
  }
}

// L covers the earlier objects, R the later ones.
__device__ __forceinline__ void box_combine(Box6& L, const Box6& R)
{
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    if (R.lo[i] < L.lo[i]) L.lo[i] = R.lo[i];
    if (R.hi[i] > L.hi[i]) L.hi[i] = R.hi[i];
  }
}

__device__ __forceinline__ Box6 shfl_down_box(const Box6& b, int d)
{
  Box6 r;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    r.lo[i] = __shfl_down_sync(0xffffffffu, b.lo[i], d);
    r.hi[i] = __shfl_down_sync(0xffffffffu, b.hi[i], d);
  }
  return r;
}

// Ordered warp reduction: lane i combines with lane i+d (its right neighbour range).
__device__ __forceinline__ Box6 warp_reduce_box(Box6 b)
{
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const Box6 r = shfl_down_box(b, d);
    if ((threadIdx.x & 31) + d < 32 && ((threadIdx.x & 31) & (2 * d - 1)) == 0) box_combine(b, r);
  }
  return b;
}

__device__ __forceinline__ void object_corners(Box6& b, const float* soa, size_t cap, uint32_t i,
                                               const float4* mats)
{
  const float lx = soa[i], ly = soa[cap + i], lz = soa[2 * cap + i];
  const float ex = soa[3 * cap + i], ey = soa[4 * cap + i], ez = soa[5 * cap + i];
  const uint32_t mi = reinterpret_cast<const uint32_t*>(soa)[6 * cap + i];
  const float4* M = mats + 4 * (size_t)mi;
  const Obb o = make_obb(lx, ly, lz, ex, ey, ez, __ldg(M), __ldg(M + 1), __ldg(M + 2), __ldg(M + 3));
  const float4 v0 = o.p;
  const float4 v1 = vadd4(v0, o.ex);
  const float4 v2 = vadd4(v0, o.ey);
  const float4 v3 = vadd4(v1, o.ey);
  box_point(b, v0);
  box_point(b, v1);
  box_point(b, v2);
  box_point(b, v3);
  box_point(b, vadd4(v0, o.ez));
  box_point(b, vadd4(v1, o.ez));
  box_point(b, vadd4(v2, o.ez));
  box_point(b, vadd4(v3, o.ez));
}

// Each block owns a contiguous object range; inside it, each warp owns a contiguous
// sub-range processed 32 objects per round (lane j takes object j of the round).
__global__ void __launch_bounds__(kBoxThreads) bbox_kernel(const float* soa, uint32_t cap,
                                                           uint32_t n, const float4* mats,
                                                           float* partials,
                                                           unsigned int* counter, float* out)
{
  __shared__ Box6 warp_box[kBoxThreads / 32];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t per_block = (n + gridDim.x - 1) / gridDim.x;
  const uint32_t b0 = min(n, blockIdx.x * per_block), b1 = min(n, b0 + per_block);
  const uint32_t per_warp = (b1 - b0 + kBoxThreads / 32 - 1) / (kBoxThreads / 32);
  const uint32_t w0 = min(b1, b0 + warp * per_warp), w1 = min(b1, w0 + per_warp);

  Box6 acc;
  box_init(acc);
  for (uint32_t base = w0; base < w1; base += 32) {
    Box6 mine;
    box_init(mine);
    if (base + lane < w1) object_corners(mine, soa, cap, base + lane, mats);
    const Box6 round = warp_reduce_box(mine);
    if (lane == 0) box_combine(acc, round);
  }
  if (lane == 0) warp_box[warp] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    Box6 blk = warp_box[0];
    for (int w = 1; w < kBoxThreads / 32; ++w) box_combine(blk, warp_box[w]);
    for (int i = 0; i < 3; ++i) {
      partials[6 * blockIdx.x + i] = blk.lo[i];
      partials[6 * blockIdx.x + 3 + i] = blk.hi[i];
    }
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    Box6 all;
    box_init(all);
    for (uint32_t b = 0; b < gridDim.x; ++b) {
      Box6 r;
      for (int i = 0; i < 3; ++i) {
        r.lo[i] = __ldcg(partials + 6 * b + i);
        r.hi[i] = __ldcg(partials + 6 * b + 3 + i);
      }
      box_combine(all, r);
    }
    for (int i = 0; i < 3; ++i) {
      out[i] = all.lo[i];
      out[3 + i] = all.hi[i];
    }
    *counter = 0;  // ready for the next launch
  }
}

int box_blocks(uint32_t n)
{
  const uint32_t want = (n + 8191) / 8192;  // about 32 objects per thread
  return (int)(want < 1 ? 1 : (want > kBoxBlocksMax ? kBoxBlocksMax : want));
}

}  // namespace

size_t bbox_partials_needed(uint32_t) { return 6 * (size_t)kBoxBlocksMax; }

int launch_bbox(const float* soa, uint32_t cap, uint32_t n, const float* mats, float* partials,
                unsigned int* counter, float* out8, void* stream)
{
  bbox_kernel<<<box_blocks(n), kBoxThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      soa, cap, n, reinterpret_cast<const float4*>(mats), partials, counter, out8);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace dpcull
