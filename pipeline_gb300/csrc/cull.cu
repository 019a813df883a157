// cull.cu -- frustum-cull kernels of the GB300 culling backend.
//
// One kernel serves both the plain per-call path (one group, one view, a grid of one
// CTA per tile) and the batched persistent path (many groups x many views, a grid of
// resident CTAs that pull work items from an atomic ticket).  A work item is one tile of
// 1024 objects of one scene and one group of up to VPP views:
//   1. stage the views' view-projection matrices in shared memory;
//   2. 128-bit streaming loads of the tile's SoA rows (each thread owns 4 objects);
//   3. per object: gather its world matrix (4 x 128-bit __ldg), build the world-space box
//      exactly as the reference's OBB cache, and run the exact clip test once per view;
//   4. per view: assemble the 32-bit visibility words with warp shuffles, XOR them with
//      the result's previous words (ResultBitSet::updateChanged), write the new words,
//      and place the changed objects in the global ascending list with a single-pass
//      decoupled look-back over the tiles of that scene and view.
// Every wait on another tile is bounded; on expiry the kernel sets an error bit, still
// publishes its status (so no successor waits forever) and the host reports the error.
#include <cuda_runtime.h>

#include "dpcull_exact.cuh"
#include "dpcull_internal.h"

namespace dpcull {

namespace {

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p)
{
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v)
{
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ float4 ld_stream4(const float* p)
{
  return __ldcs(reinterpret_cast<const float4*>(p));
}

__device__ __forceinline__ uint4 ld_stream4u(const float* p)
{
  return __ldcs(reinterpret_cast<const uint4*>(p));
}

__device__ __forceinline__ float comp(const float4& v, int k)
{
  return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w;
}

__device__ __forceinline__ uint32_t compu(const uint4& v, int k)
{
  return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w;
}

__device__ __forceinline__ unsigned long long pack_status(uint32_t epoch, uint32_t flag,
                                                          uint32_t value)
{
  return ((unsigned long long)epoch << 32) | ((unsigned long long)flag << 30) |
         (unsigned long long)(value & 0x3FFFFFFFu);
}

// Warp-cooperative decoupled look-back.  Publishes this tile's aggregate, sums the
// aggregates of its predecessors (32 at a time) until it meets an inclusive prefix,
// publishes its own inclusive prefix and returns the exclusive prefix (lane-uniform).
__device__ uint32_t lookback(unsigned long long* status, uint32_t tile, uint32_t total,
                             uint32_t epoch, uint32_t spin_limit, CullControl* ctl)
{
  const int lane = threadIdx.x & 31;
  if (tile == 0) {
    if (lane == 0) st_relaxed_u64(&status[0], pack_status(epoch, kFlagPrefix, total));
    return 0;
  }
  if (lane == 0) st_relaxed_u64(&status[tile], pack_status(epoch, kFlagAggregate, total));
  uint32_t excl = 0;
  int64_t top = (int64_t)tile - 1;
  uint32_t polls = 0;
  bool timed_out = false;
  for (;;) {
    const int64_t pred = top - lane;
    unsigned long long s;
    for (;;) {
      s = pred >= 0 ? ld_relaxed_u64(&status[pred]) : pack_status(epoch, kFlagPrefix, 0);
      const bool ready = (uint32_t)(s >> 32) == epoch && ((s >> 30) & 3u) != 0;
      if (__all_sync(0xffffffffu, ready)) break;
      // Give up when the budget is spent, or at once when another tile already gave up
      // (then no wait in this launch can be trusted and none may run its full budget).
      if (++polls > spin_limit ||
          ((polls & 255u) == 0 &&
           (*reinterpret_cast<volatile unsigned int*>(&ctl->error) & kErrLookbackTimeout))) {
        timed_out = true;
        break;
      }
      __nanosleep(64);
    }
    if (timed_out) break;
    const uint32_t flag = (uint32_t)(s >> 30) & 3u;
    const uint32_t val = (uint32_t)s & 0x3FFFFFFFu;
    const uint32_t pmask = __ballot_sync(0xffffffffu, flag == kFlagPrefix);
    if (pmask) {
      const int first = __ffs(pmask) - 1;
      excl += __reduce_add_sync(0xffffffffu, lane <= first ? val : 0u);
      break;
    }
    excl += __reduce_add_sync(0xffffffffu, val);
    top -= 32;
  }
  if (timed_out && lane == 0) atomicOr(&ctl->error, kErrLookbackTimeout);
  // Publish even after a timeout so that no successor waits on this tile.
  if (lane == 0) st_relaxed_u64(&status[tile], pack_status(epoch, kFlagPrefix, excl + total));
  return excl;
}

struct CullShared {
  float vp[kMaxViewsPerPass][16];
  uint32_t wtot[kMaxViewsPerPass][kThreads / 32];   // per-warp changed counts
  uint32_t wbase[kMaxViewsPerPass][kThreads / 32];  // per-warp output offsets
  uint32_t item;
};

__device__ __forceinline__ uint32_t find_scene(const CullScene* scenes, uint32_t n, uint32_t item)
{
  uint32_t lo = 0, hi = n;  // last scene with item_begin <= item
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (scenes[mid].item_begin <= item) lo = mid;
    else hi = mid;
  }
  return lo;
}

template <int VPP>
__device__ void process_item(const CullLaunch& a, uint32_t item, uint32_t epoch, CullShared& sh)
{
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const CullScene sc = a.scenes ? a.scenes[find_scene(a.scenes, a.n_scenes, item)] : a.one_scene;
  const uint32_t local = item - sc.item_begin;
  const uint32_t tile = local / sc.n_vgroups;
  const uint32_t vfirst = (local - tile * sc.n_vgroups) * VPP;
  const int nv = (int)min((uint32_t)VPP, sc.n_views - vfirst);
  const CullView* views = a.views ? a.views + sc.view_begin + vfirst : &a.one_view;

  if (tid < nv * 16) sh.vp[tid >> 4][tid & 15] = views[tid >> 4].vp[tid & 15];
  __syncthreads();

  // ---- visibility of my 4 objects in each view ----
  const uint32_t obj0 = tile * kTileObjects + (uint32_t)tid * kObjPerThread;
  const float* soa = sc.soa;
  const size_t cap = sc.cap;
  const float4 lx = ld_stream4(soa + 0 * cap + obj0);
  const float4 ly = ld_stream4(soa + 1 * cap + obj0);
  const float4 lz = ld_stream4(soa + 2 * cap + obj0);
  const float4 ex = ld_stream4(soa + 3 * cap + obj0);
  const float4 ey = ld_stream4(soa + 4 * cap + obj0);
  const float4 ez = ld_stream4(soa + 5 * cap + obj0);
  const uint4 xf = ld_stream4u(soa + 6 * cap + obj0);
  const float4* mats = reinterpret_cast<const float4*>(sc.mats);

  uint32_t nib[VPP];
#pragma unroll
  for (int v = 0; v < VPP; ++v) nib[v] = 0;

#pragma unroll
  for (int k = 0; k < kObjPerThread; ++k) {
    if (obj0 + k < sc.n_objects) {
      const uint32_t mi = compu(xf, k);
      if (mi < sc.n_mats) {
        const float4* M = mats + 4 * (size_t)mi;
        const float4 r0 = __ldg(M + 0), r1 = __ldg(M + 1), r2 = __ldg(M + 2), r3 = __ldg(M + 3);
        const Obb o = make_obb(comp(lx, k), comp(ly, k), comp(lz, k), comp(ex, k), comp(ey, k),
                               comp(ez, k), r0, r1, r2, r3);
#pragma unroll
        for (int v = 0; v < VPP; ++v)
          if (v < nv && obb_visible(o, sh.vp[v])) nib[v] |= 1u << k;
      } else {
        if (atomicOr(&a.ctl->error, kErrBadTransform) == 0) a.ctl->error_info = obj0 + k;
      }
    }
  }

  // ---- words, changed nibbles and per-thread changed counts ----
  const uint32_t word = tile * kTileWords + (uint32_t)(tid >> 3);
  const int shift = (tid & 7) * 4;
  uint32_t chg[VPP];
  uint32_t packed[(VPP + 3) / 4];
#pragma unroll
  for (int q = 0; q < (VPP + 3) / 4; ++q) packed[q] = 0;
#pragma unroll
  for (int v = 0; v < VPP; ++v) {
    chg[v] = 0;
    if (v < nv) {
      uint32_t* bits = views[v].bits;
      const uint32_t prev = bits[word];
      chg[v] = nib[v] ^ ((prev >> shift) & 0xFu);
      uint32_t w = nib[v] << shift;
      w |= __shfl_xor_sync(0xffffffffu, w, 1);
      w |= __shfl_xor_sync(0xffffffffu, w, 2);
      w |= __shfl_xor_sync(0xffffffffu, w, 4);
      if ((tid & 7) == 0 && w != prev) bits[word] = w;
      packed[v >> 2] |= (uint32_t)__popc(chg[v]) << (8 * (v & 3));
    } else {
      // keep the shuffles warp-uniform: nv is uniform, so this branch is too
    }
  }

  // Warp inclusive scan of the packed counts (fields stay below 256: 32 lanes x 4).
  uint32_t incl[(VPP + 3) / 4];
#pragma unroll
  for (int q = 0; q < (VPP + 3) / 4; ++q) {
    uint32_t x = packed[q];
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
      if (lane >= d) x += y;
    }
    incl[q] = x;
  }
  if (lane == 31) {
#pragma unroll
    for (int v = 0; v < VPP; ++v)
      if (v < nv) sh.wtot[v][warp] = (incl[v >> 2] >> (8 * (v & 3))) & 0xFFu;
  }
  __syncthreads();

  // ---- tile totals and look-back: warp v handles view v ----
  if (warp < nv) {
    const int v = warp;
    uint32_t x = lane < kThreads / 32 ? sh.wtot[v][lane] : 0u;
    const uint32_t own = x;
#pragma unroll
    for (int d = 1; d < kThreads / 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
      if (lane >= d) x += y;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, x, kThreads / 32 - 1);
    const uint32_t base = lookback(views[v].status, tile, total, epoch, a.spin_limit, a.ctl);
    if (lane < kThreads / 32) sh.wbase[v][lane] = base + x - own;
    if (lane == 0 && tile == sc.n_tiles - 1) *views[v].n_changed = base + total;
  }
  __syncthreads();

  // ---- ascending changed-object indices ----
#pragma unroll
  for (int v = 0; v < VPP; ++v) {
    if (v < nv && chg[v]) {
      const uint32_t own = (uint32_t)__popc(chg[v]);
      uint32_t off = sh.wbase[v][warp] + ((incl[v >> 2] >> (8 * (v & 3))) & 0xFFu) - own;
      uint32_t* out = views[v].changed;
      uint32_t m = chg[v];
      while (m) {
        const int k = __ffs(m) - 1;
        out[off++] = obj0 + (uint32_t)k;
        m &= m - 1u;
      }
    }
  }
  __syncthreads();  // shared views / totals are reused by the next item
}

template <int VPP>
__global__ void __launch_bounds__(kThreads) cull_kernel(const __grid_constant__ CullLaunch a)
{
  __shared__ CullShared sh;
  CullControl* ctl = a.ctl;
  const uint32_t epoch = *reinterpret_cast<volatile unsigned int*>(&ctl->epoch);
  for (;;) {
    if (threadIdx.x == 0) sh.item = atomicAdd(&ctl->ticket, a.items_per_ticket);
    __syncthreads();
    const uint32_t first = sh.item;
    __syncthreads();
    if (first >= a.n_items) break;
    const uint32_t last = min(first + a.items_per_ticket, a.n_items);
    for (uint32_t item = first; item < last; ++item) process_item<VPP>(a, item, epoch, sh);
  }
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned int prev = atomicAdd(&ctl->done, 1u);
    if (prev == gridDim.x - 1) {
      // Last CTA of the launch: reset the ticket and advance the epoch, so the next
      // launch on this control block needs no memset.
      ctl->ticket = 0;
      ctl->done = 0;
      __threadfence();
      atomicAdd(&ctl->epoch, ctl->stride);
    }
  }
}

template <int VPP>
int launch_vpp(const CullLaunch& a, int grid, cudaStream_t s)
{
  cull_kernel<VPP><<<grid, kThreads, 0, s>>>(a);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <int VPP>
int max_ctas()
{
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, cull_kernel<VPP>, kThreads, 0) != cudaSuccess)
    return 1;
  return n > 0 ? n : 1;
}

// ---- small helper kernels -----------------------------------------------------------

// ResultBitSet::onNotify (dp/culling/src/ResultBitSet.cpp:110-128): the object moved from
// old_index to new_index carries its bit; an unknown old slot counts as visible.
__global__ void move_bit_kernel(uint32_t* bits, uint32_t size_bits, uint32_t old_index,
                                uint32_t new_index)
{
  if (new_index >= size_bits) return;
  const uint32_t b = old_index < size_bits ? (bits[old_index >> 5] >> (old_index & 31)) & 1u : 1u;
  const uint32_t m = 1u << (new_index & 31);
  bits[new_index >> 5] = b ? (bits[new_index >> 5] | m) : (bits[new_index >> 5] & ~m);
}

// GroupBitSet::removeObject moves the last object into the hole: SoA row copy.
__global__ void move_object_kernel(float* soa, uint32_t cap, uint32_t from, uint32_t to)
{
  const int r = threadIdx.x;
  if (r < 7) soa[(size_t)r * cap + to] = soa[(size_t)r * cap + from];
}

}  // namespace

int launch_cull(const CullLaunch& a, int grid, int vpp, void* stream)
{
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  switch (vpp) {
    case 1: return launch_vpp<1>(a, grid, s);
    case 2: return launch_vpp<2>(a, grid, s);
    case 4: return launch_vpp<4>(a, grid, s);
    case 8: return launch_vpp<8>(a, grid, s);
    default: return -1;
  }
}

int cull_max_ctas_per_sm(int vpp)
{
  switch (vpp) {
    case 1: return max_ctas<1>();
    case 2: return max_ctas<2>();
    case 4: return max_ctas<4>();
    case 8: return max_ctas<8>();
    default: return 1;
  }
}

int launch_move_bit(uint32_t* bits, uint32_t size_bits, uint32_t old_index, uint32_t new_index,
                    void* stream)
{
  move_bit_kernel<<<1, 1, 0, static_cast<cudaStream_t>(stream)>>>(bits, size_bits, old_index,
                                                                  new_index);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_move_object(float* soa, uint32_t cap, uint32_t from, uint32_t to, void* stream)
{
  move_object_kernel<<<1, 32, 0, static_cast<cudaStream_t>(stream)>>>(soa, cap, from, to);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace dpcull
