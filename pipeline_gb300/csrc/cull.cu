// cull.cu -- frustum-cull kernels of the GB300 culling backend.
//
// One kernel serves both the plain per-call path (one group, one view, a grid of one
// CTA per tile) and the batched persistent path (many groups x many views, a grid of
// resident CTAs that pull work items from an atomic ticket).  A work item is one tile of
// 1024 objects of one scene and one group of up to VPP views:
//   1. stage the views' view-projection matrices (and their prefilter bounds) in shared
//      memory;
//   2. 128-bit streaming loads of the tile's SoA rows (each thread owns 4 objects);
//   3. per object: gather its world matrix (4 x 128-bit __ldg) and build the world-space
//      box exactly as the reference's OBB cache; per view, the conservative prefilter
//      (dpcull_exact.cuh) decides visible / invisible where the reference's rounded
//      result is certain; the undecided (object, view) pairs of the tile are compacted
//      into a shared-memory queue and run through the exact reference test by all
//      threads together, so no warp idles on a rare exact pair;
//   4. per view: assemble the 32-bit visibility words with warp shuffles, XOR them with
//      the result's previous words (ResultBitSet::updateChanged), write the new words
//      (only where they changed), and write the tile's changed objects, ascending, into
//      the tile's private slot range together with the tile's count.
// A CTA never waits for another.  Two small kernels then turn the per-tile slots into
// the packed ascending changed list: a per-view exclusive scan of the tile counts and a
// gather of the slots (launch_changed_lists).
#include <cuda_runtime.h>

#include "dpcull_exact.cuh"
#include "dpcull_internal.h"

namespace dpcull {

namespace {

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

struct CullShared {
  CullView cv[kMaxViewsPerPass];                     // the item's views (matrices + outputs)
  PfView vn[kMaxViewsPerPass];                       // prefilter view bounds
  uint32_t vis[kMaxViewsPerPass][kTileWords];        // visibility from the exact drain
  uint32_t wtot[kMaxViewsPerPass][kThreads / 32];   // per-warp changed counts
  uint32_t item;
  uint32_t qn;                                       // undecided (object, view) pairs
  uint16_t queue[kTileObjects * kMaxViewsPerPass];   // entry = tile object << 3 | view
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

// Exact visibility of one object of the scene (reference operation order), reloading its
// row and matrix; used for the pairs the prefilter cannot decide.
__device__ __forceinline__ bool exact_visible(const CullScene& sc, uint32_t i, const float* vp)
{
  const float* soa = sc.soa;
  const size_t cap = sc.cap;
  const uint32_t mi = __ldg(reinterpret_cast<const uint32_t*>(soa) + 6 * cap + i);
  const float4* M = reinterpret_cast<const float4*>(sc.mats) + 4 * (size_t)mi;
  const Obb o = make_obb(__ldg(soa + i), __ldg(soa + cap + i), __ldg(soa + 2 * cap + i),
                         __ldg(soa + 3 * cap + i), __ldg(soa + 4 * cap + i),
                         __ldg(soa + 5 * cap + i), __ldg(M + 0), __ldg(M + 1), __ldg(M + 2),
                         __ldg(M + 3));
  return obb_visible(o, vp);
}

template <int VPP, bool PF>
__device__ void process_item(const CullLaunch& a, uint32_t item, CullShared& sh)
{
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const CullScene sc = a.scenes ? a.scenes[find_scene(a.scenes, a.n_scenes, item)] : a.one_scene;
  const uint32_t local = item - sc.item_begin;
  const uint32_t tile = local / sc.n_vgroups;
  const uint32_t vfirst = (local - tile * sc.n_vgroups) * VPP;
  const int nv = (int)min((uint32_t)VPP, sc.n_views - vfirst);
  const CullView* views = a.views ? a.views + sc.view_begin + vfirst : &a.one_view;

  // Stage the views (matrices and output pointers) in shared memory: the per-view work
  // below then never waits on a dependent global load of a descriptor.
  constexpr int kViewWords = (int)(sizeof(CullView) / 4);
  static_assert(sizeof(CullView) % 16 == 0, "CullView is staged as whole words");
  if (tid < nv * kViewWords)
    reinterpret_cast<uint32_t*>(sh.cv)[tid] = reinterpret_cast<const uint32_t*>(views)[tid];
  if (PF) {
    if (tid < VPP * kTileWords) sh.vis[tid / kTileWords][tid % kTileWords] = 0u;
    if (tid == 0) sh.qn = 0u;
  }
  __syncthreads();
  if (PF && tid < nv) sh.vn[tid] = pf_view(sh.cv[tid].vp);
  if (PF) __syncthreads();

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
  uint32_t amb = 0;  // bit 8k + v: object k in view v needs the exact test

  if (PF) {
    // Boxes and their bounds for the 4 objects first (the 16 matrix gathers overlap),
    // then each view's constants are read once for all 4 objects.
    PfObject pb[kObjPerThread];
    uint32_t valid = 0;
#pragma unroll
    for (int k = 0; k < kObjPerThread; ++k) {
      pb[k].da = pf_nan();
      if (obj0 + k < sc.n_objects) {
        const uint32_t mi = compu(xf, k);
        if (mi < sc.n_mats) {
          const float4* M = mats + 4 * (size_t)mi;
          const Obb o = make_obb(comp(lx, k), comp(ly, k), comp(lz, k), comp(ex, k), comp(ey, k),
                                 comp(ez, k), __ldg(M + 0), __ldg(M + 1), __ldg(M + 2), __ldg(M + 3));
          pb[k] = pf_object(o);
          valid |= 1u << k;
        } else if (atomicOr(&a.ctl->error, kErrBadTransform) == 0) {
          a.ctl->error_info = obj0 + k;
        }
      }
    }
#pragma unroll
    for (int v = 0; v < VPP; ++v) {
      if (v < nv) {
        const PfViewRegs vr = pf_load_view(sh.cv[v].vp, sh.vn[v]);
#pragma unroll
        for (int k = 0; k < kObjPerThread; ++k) {
          if (valid & (1u << k)) {
            const int cls = pf_classify(pb[k], vr);
            if (cls == kPfVisible) nib[v] |= 1u << k;
            else if (cls == kPfAmbiguous) amb |= 1u << (8 * k + v);
          }
        }
      }
    }
  } else {
#pragma unroll
    for (int k = 0; k < kObjPerThread; ++k) {
      if (obj0 + k < sc.n_objects) {
        const uint32_t mi = compu(xf, k);
        if (mi < sc.n_mats) {
          const float4* M = mats + 4 * (size_t)mi;
          const Obb o = make_obb(comp(lx, k), comp(ly, k), comp(lz, k), comp(ex, k), comp(ey, k),
                                 comp(ez, k), __ldg(M + 0), __ldg(M + 1), __ldg(M + 2), __ldg(M + 3));
#pragma unroll
          for (int v = 0; v < VPP; ++v)
            if (v < nv && obb_visible(o, sh.cv[v].vp)) nib[v] |= 1u << k;
        } else if (atomicOr(&a.ctl->error, kErrBadTransform) == 0) {
          a.ctl->error_info = obj0 + k;
        }
      }
    }
  }

  if (PF) {
    // ---- compact the undecided pairs of the tile and run them through the exact test ----
    const uint32_t cnt = (uint32_t)__popc(amb);
    uint32_t x = cnt;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
      if (lane >= d) x += y;
    }
    uint32_t base = 0;
    if (lane == 31) base = atomicAdd(&sh.qn, x);
    base = __shfl_sync(0xffffffffu, base, 31);
    uint32_t pos = base + x - cnt;
    while (amb) {
      const int b = __ffs(amb) - 1;
      sh.queue[pos++] =
          (uint16_t)(((uint32_t)(tid * kObjPerThread + (b >> 3)) << 3) | (uint32_t)(b & 7));
      amb &= amb - 1u;
    }
    __syncthreads();
    const uint32_t qn = sh.qn;
    const uint32_t tile0 = tile * kTileObjects;
    for (uint32_t q = tid; q < qn; q += kThreads) {
      const uint32_t e = sh.queue[q];
      const uint32_t o = e >> 3, v = e & 7u;
      if (exact_visible(sc, tile0 + o, sh.cv[v].vp)) atomicOr(&sh.vis[v][o >> 5], 1u << (o & 31));
    }
    __syncthreads();
#pragma unroll
    for (int v = 0; v < VPP; ++v)
      if (v < nv) nib[v] |= (sh.vis[v][tid >> 3] >> ((tid & 7) * 4)) & 0xFu;
  }

  // ---- words, changed nibbles and per-thread changed counts ----
  // All previous words are loaded before any word is stored, so the loads are in flight
  // together (a later view's load could not move above an earlier view's store).
  const uint32_t word = tile * kTileWords + (uint32_t)(tid >> 3);
  uint32_t prevw[VPP];
#pragma unroll
  for (int v = 0; v < VPP; ++v)
    prevw[v] = (v < nv && !(sh.cv[v].flags & kViewNoChanged)) ? sh.cv[v].bits[word] : ~0u;
  const int shift = (tid & 7) * 4;
  uint32_t chg[VPP];
  uint32_t packed[(VPP + 3) / 4];
#pragma unroll
  for (int q = 0; q < (VPP + 3) / 4; ++q) packed[q] = 0;
#pragma unroll
  for (int v = 0; v < VPP; ++v) {
    chg[v] = 0;
    if (v < nv) {  // nv is uniform over the CTA, so the shuffles stay warp-uniform
      uint32_t* bits = sh.cv[v].bits;
      const bool track = !(sh.cv[v].flags & kViewNoChanged);
      const uint32_t prev = prevw[v];
      uint32_t w = nib[v] << shift;
      w |= __shfl_xor_sync(0xffffffffu, w, 1);
      w |= __shfl_xor_sync(0xffffffffu, w, 2);
      w |= __shfl_xor_sync(0xffffffffu, w, 4);
      if ((tid & 7) == 0 && (!track || w != prev)) bits[word] = w;
      if (sh.cv[v].n_visible) {
        const uint32_t cnt = __reduce_add_sync(0xffffffffu, (uint32_t)__popc(nib[v]));
        if (lane == 0 && cnt) atomicAdd(sh.cv[v].n_visible, cnt);
      }
      if (track) {
        chg[v] = nib[v] ^ ((prev >> shift) & 0xFu);
        packed[v >> 2] |= (uint32_t)__popc(chg[v]) << (8 * (v & 3));
      }
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

  // ---- the tile's changed objects, ascending, into its private slots ----
#pragma unroll
  for (int v = 0; v < VPP; ++v) {
    if (v < nv && !(sh.cv[v].flags & kViewNoChanged)) {
      uint32_t before = 0, total = 0;
#pragma unroll
      for (int w = 0; w < kThreads / 32; ++w) {
        const uint32_t t = sh.wtot[v][w];
        before += w < warp ? t : 0u;
        total += t;
      }
      if (tid == 0) sh.cv[v].counts[tile] = total;
      if (chg[v]) {
        const uint32_t own = (uint32_t)__popc(chg[v]);
        uint32_t off = tile * kTileObjects + before + ((incl[v >> 2] >> (8 * (v & 3))) & 0xFFu) - own;
        uint32_t* slots = sh.cv[v].slots;
        uint32_t m = chg[v];
        while (m) {
          const int k = __ffs(m) - 1;
          slots[off++] = obj0 + (uint32_t)k;
          m &= m - 1u;
        }
      }
    }
  }
  __syncthreads();  // shared views / totals are reused by the next item
}

template <int VPP, bool PF>
__global__ void __launch_bounds__(kThreads, 3) cull_kernel(const __grid_constant__ CullLaunch a)
{
  __shared__ CullShared sh;
  CullControl* ctl = a.ctl;
  for (;;) {
    if (threadIdx.x == 0) sh.item = atomicAdd(&ctl->ticket, a.items_per_ticket);
    __syncthreads();
    const uint32_t first = sh.item;
    __syncthreads();
    if (first >= a.n_items) break;
    const uint32_t last = min(first + a.items_per_ticket, a.n_items);
    for (uint32_t item = first; item < last; ++item) process_item<VPP, PF>(a, item, sh);
  }
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned int prev = atomicAdd(&ctl->done, 1u);
    if (prev == gridDim.x - 1) {
      // Last CTA of the launch: reset the ticket for the next launch (no memset needed).
      ctl->ticket = 0;
      ctl->done = 0;
    }
  }
}

// ---- changed-list assembly ----------------------------------------------------------------
constexpr int kScanThreads = 1024;

// One CTA per view: exclusive scan of the tile counts into offsets, total into n_changed.
__global__ void __launch_bounds__(kScanThreads)
    scan_counts_kernel(const CullView* views, const __grid_constant__ CullView one)
{
  __shared__ uint32_t warp_sum[kScanThreads / 32];
  const CullView& v = views ? views[blockIdx.x] : one;
  const uint32_t n = v.n_tiles;
  const uint32_t per = (n + kScanThreads - 1) / kScanThreads;
  const uint32_t b = min(n, threadIdx.x * per), e = min(n, b + per);
  // Independent loads, 8 in flight per thread (the counts were just written by the cull).
  uint32_t s = 0;
  for (uint32_t i = b; i < e; i += 8) {
    uint32_t c[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) c[j] = i + j < e ? __ldcg(v.counts + i + j) : 0u;
#pragma unroll
    for (int j = 0; j < 8; ++j) s += c[j];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = s;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
    if (lane >= d) x += y;
  }
  if (lane == 31) warp_sum[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = warp_sum[lane];
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, d);
      if (lane >= d) w += y;
    }
    warp_sum[lane] = w;  // inclusive over warps
  }
  __syncthreads();
  uint32_t run = (warp ? warp_sum[warp - 1] : 0u) + x - s;
  for (uint32_t i = b; i < e; i += 8) {
    uint32_t c[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) c[j] = i + j < e ? __ldcg(v.counts + i + j) : 0u;
#pragma unroll
    for (int j = 0; j < 8; ++j)
      if (i + j < e) {
        v.offsets[i + j] = run;
        run += c[j];
      }
  }
  if (threadIdx.x == kScanThreads - 1) *v.n_changed = warp_sum[31];
}

// blockIdx.y = view.  Each warp reads the counts and offsets of 32 consecutive tiles in
// one coalesced load, then copies the slot ranges of the non-empty ones, all lanes per
// tile, to their packed positions.
__global__ void gather_changed_kernel(const CullView* views, const __grid_constant__ CullView one)
{
  const CullView& v = views ? views[blockIdx.y] : one;
  const int lane = threadIdx.x & 31;
  const uint32_t warps = blockDim.x / 32;
  for (uint32_t t0 = (blockIdx.x * warps + threadIdx.x / 32) * 32; t0 < v.n_tiles;
       t0 += gridDim.x * warps * 32) {
    const uint32_t t = t0 + lane;
    const uint32_t c = t < v.n_tiles ? __ldcg(v.counts + t) : 0u;
    const uint32_t o = t < v.n_tiles ? __ldcg(v.offsets + t) : 0u;
    uint32_t busy = __ballot_sync(0xffffffffu, c != 0);
    while (busy) {
      const int k = __ffs(busy) - 1;
      busy &= busy - 1u;
      const uint32_t ck = __shfl_sync(0xffffffffu, c, k), ok = __shfl_sync(0xffffffffu, o, k);
      const uint32_t* src = v.slots + (size_t)(t0 + k) * kTileObjects;
      for (uint32_t j = lane; j < ck; j += 32) v.changed[ok + j] = __ldcg(src + j);
    }
  }
}

template <int VPP>
int launch_vpp(const CullLaunch& a, int grid, cudaStream_t s)
{
  if (a.exact_only) cull_kernel<VPP, false><<<grid, kThreads, 0, s>>>(a);
  else cull_kernel<VPP, true><<<grid, kThreads, 0, s>>>(a);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <int VPP>
int max_ctas()
{
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, cull_kernel<VPP, true>, kThreads, 0) != cudaSuccess)
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

int launch_changed_lists(const CullView* views, const CullView& one, uint32_t n_views,
                         uint32_t max_tiles, void* stream)
{
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!n_views) return 0;
  scan_counts_kernel<<<n_views, kScanThreads, 0, s>>>(views, one);
  const uint32_t warps = 8, tiles_per_cta = warps * 32;
  uint32_t gx = (max_tiles + tiles_per_cta - 1) / tiles_per_cta;
  if (gx > 1024) gx = 1024;
  if (gx < 1) gx = 1;
  gather_changed_kernel<<<dim3(gx, n_views), warps * 32, 0, s>>>(views, one);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
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
