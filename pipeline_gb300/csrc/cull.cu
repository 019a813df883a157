// cull.cu -- frustum-cull kernels of the GB300 culling backend.
//
// One kernel serves the plain per-call path (one group, one view) and the batched
// persistent path (many groups x many views).  Every warp works on its own: it pulls work
// items from an atomic ticket, and a work item is 1-8 tiles of 128 objects (one float4 of
// each SoA row per lane; the launch picks the tiles per item) of one scene with one group
// of up to VPP views:
//   1. stage the views (view-projection matrices, output pointers) and their prefilter
//      planes in the warp's shared memory, unless the previous item had the same views;
//   2. per tile: 128-bit streaming loads of the SoA rows (the transform-index row one tile
//      ahead, so the matrix gathers go out with the other rows); per object, gather its
//      world matrix (2 x 256-bit loads when the launch's matrix arrays are 32-byte
//      aligned, else 4 x 128-bit) and build its prefilter box; per view, the conservative
//      prefilter (dpcull_prefilter.h; an axis' lo and hi plane as one fma.rn.f32x2 pair)
//      decides visible / invisible wherever the reference's rounded result is certain; the
//      decided-visible bits go to the item's words in shared memory (one nibble transpose
//      per tile) and the undecided (object, view) pairs to the warp's queue;
//   3. all lanes run the queued pairs through the exact reference test (dpcull_exact.cuh)
//      and set the visible ones in the words;
//   4. per view of the item: XOR with the result's previous words (ResultBitSet::
//      updateChanged), store the new words where they changed and the delta words.
// No warp waits for another.  One small kernel then turns the delta words into the packed
// ascending changed list (launch_changed_lists).
#include <algorithm>
#include <atomic>

#include <cuda_runtime.h>

#include "dpcull_exact.cuh"
#include "dpcull_internal.h"
#include "dpcull_prefilter.h"

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

// Shared memory of one warp: its cached scene and views, the views' prefilter planes, the
// provisional visibility words of its item and the item's undecided pairs.  Warps of a
// CTA never share state, so no CTA barrier is taken per item.
struct WarpShared {
  CullScene sc;                                          // the scene of the warp's last item
  CullView cv[kMaxViewsPerPass];                         // the item's views (matrices + outputs)
  pf::GroupMargin gm;                                    // margin of the staged view group
  uint32_t words[kMaxViewsPerPass][kItemTiles][kTileWords];  // the item's visibility words
  uint16_t queue[kQueueCap];                             // tile << 10 | object << 3 | view
  uint32_t qtail;                                        // the queue's length (slots taken)
  ulonglong2 qp[kMaxViewsPerPass][3][2];                 // per axis: (lo, hi) pairs of x, y | z, w
  float4 zlo[kMaxViewsPerPass];                          // the z-lo planes alone (five-plane test)
  uint32_t far_off;                                      // the group may leave out its z-hi planes
  uint32_t bnd[kBoundWords];                             // Fill: the item's scene-bound keys
};
static_assert(kTileObjects == 32 * kObjPerThread, "a tile is one warp's objects");
static_assert(kItemTiles * kTileWords <= 32, "one word of a view's item per lane");

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

// One 64-byte world matrix (4 rows).  When the matrix array is 32-byte aligned (every
// array this library allocates; bound arrays need only 16) two 256-bit loads replace the
// four 128-bit ones: a gather instruction touches 32 different lines whatever its width,
// so halving the instructions halves the gather's L1 wavefronts.
__device__ __forceinline__ void load_matrix(const float* M, bool wide, float4& r0, float4& r1,
                                            float4& r2, float4& r3)
{
  if (wide) {
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(r0.x), "=f"(r0.y), "=f"(r0.z), "=f"(r0.w), "=f"(r1.x), "=f"(r1.y), "=f"(r1.z), "=f"(r1.w)
        : "l"(M));
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(r2.x), "=f"(r2.y), "=f"(r2.z), "=f"(r2.w), "=f"(r3.x), "=f"(r3.y), "=f"(r3.z), "=f"(r3.w)
        : "l"(M + 8));
  } else {
    const float4* M4 = reinterpret_cast<const float4*>(M);
    r0 = __ldg(M4 + 0);
    r1 = __ldg(M4 + 1);
    r2 = __ldg(M4 + 2);
    r3 = __ldg(M4 + 3);
  }
}

// Exact visibility of one object of the scene (reference operation order), reloading its
// row and matrix; used for the pairs the prefilter cannot decide.
__device__ __forceinline__ bool exact_visible(const CullScene& sc, uint32_t i, const float* vp)
{
  const float* soa = sc.soa;
  const size_t cap = sc.cap;
  const uint32_t mi = __ldg(reinterpret_cast<const uint32_t*>(soa) + 6 * cap + i);
  if (mi >= sc.n_mats) return false;  // reported by the host before any launch
  const float4* M = reinterpret_cast<const float4*>(sc.mats) + 4 * (size_t)mi;
  const Obb o = make_obb(__ldg(soa + i), __ldg(soa + cap + i), __ldg(soa + 2 * cap + i),
                         __ldg(soa + 3 * cap + i), __ldg(soa + 4 * cap + i),
                         __ldg(soa + 5 * cap + i), __ldg(M + 0), __ldg(M + 1), __ldg(M + 2),
                         __ldg(M + 3));
  return obb_visible(o, vp);
}

// The same test from the group's cached OBB of object i (the values make_obb computes, in
// one 64-byte record): two 256-bit loads replace the seven scattered row reloads and the
// matrix gather.
__device__ __forceinline__ bool exact_visible_cached(const CullScene& sc, uint32_t i, const float* vp)
{
  const float* rec = sc.obb + (size_t)kObbFloats * i;
  Obb o;
  asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=f"(o.p.x), "=f"(o.p.y), "=f"(o.p.z), "=f"(o.p.w), "=f"(o.ex.x), "=f"(o.ex.y), "=f"(o.ex.z), "=f"(o.ex.w)
      : "l"(rec));
  asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=f"(o.ey.x), "=f"(o.ey.y), "=f"(o.ey.z), "=f"(o.ey.w), "=f"(o.ez.x), "=f"(o.ez.y), "=f"(o.ez.z), "=f"(o.ez.w)
      : "l"(rec + 8));
  return obb_visible(o, vp);
}

// Stores the reference's cached OBB of object i (Fill launches): 64 bytes, two 256-bit
// stores.
__device__ __forceinline__ void store_obb(const CullScene& sc, uint32_t i, const Obb& o)
{
  float* rec = sc.obb + (size_t)kObbFloats * i;
  asm volatile("st.global.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"l"(rec), "f"(o.p.x), "f"(o.p.y), "f"(o.p.z),
               "f"(o.p.w), "f"(o.ex.x), "f"(o.ex.y), "f"(o.ex.z), "f"(o.ex.w)
               : "memory");
  asm volatile("st.global.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"l"(rec + 8), "f"(o.ey.x), "f"(o.ey.y), "f"(o.ey.z),
               "f"(o.ey.w), "f"(o.ez.x), "f"(o.ez.y), "f"(o.ez.z), "f"(o.ez.w)
               : "memory");
}

// The lane's 4 visibility bits of one view (bit k = object k) into the tile's words of
// that view in the item (warp shuffles; the lanes 0, 8, 16, 24 store).
__device__ __forceinline__ void store_nibble(WarpShared& ws, int v, uint32_t t, uint32_t nib, int lane)
{
  uint32_t w = nib << ((lane & 7) * 4);
  w |= __shfl_xor_sync(0xffffffffu, w, 1);
  w |= __shfl_xor_sync(0xffffffffu, w, 2);
  w |= __shfl_xor_sync(0xffffffffu, w, 4);
  if ((lane & 7) == 0) ws.words[v][t][lane >> 3] = w;
}

// Packed FP32 pairs: each half of fma.rn.f32x2 is one fma.rn.f32, bit for bit.
__device__ __forceinline__ unsigned long long pk2(float lo, float hi)
{
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void upk2(unsigned long long v, float& lo, float& hi)
{
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ unsigned long long fma2(unsigned long long a, unsigned long long b,
                                                   unsigned long long c)
{
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}

// 8x8 transpose of 4-bit elements across the 8 lanes of each lane octet: nibble v of
// octet lane i moves to nibble i of octet lane v.  Three butterfly steps; in step s the
// lanes i and i ^ s swap the off-diagonal s x s blocks.
__device__ __forceinline__ uint32_t transpose_nibbles8(uint32_t x, int lane)
{
#pragma unroll
  for (int s = 1; s <= 4; s <<= 1) {
    const uint32_t hi = s == 1 ? 0xF0F0F0F0u : s == 2 ? 0xFF00FF00u : 0xFFFF0000u;  // nibble bit set
    const bool upper = (lane & s) != 0;
    const uint32_t send = upper ? (x & ~hi) << (4 * s) : (x & hi) >> (4 * s);
    const uint32_t got = __shfl_xor_sync(0xffffffffu, send, s);
    x = (upper ? (x & hi) : (x & ~hi)) | got;
  }
  return x;
}

// Object K of the lane's 4 in one view: its six plane values (each axis' lo and hi plane
// as one fma.rn.f32x2 pair, the FMA chain of pf::plane) and the group decision as bit K of
// `in` (visible) and of `un` (undecided).
template <int K>
__device__ __forceinline__ void decide_object(const unsigned long long (&cx)[kObjPerThread],
                                              const unsigned long long (&cy)[kObjPerThread],
                                              const unsigned long long (&cz)[kObjPerThread],
                                              const ulonglong2& ax0, const ulonglong2& ax1,
                                              const ulonglong2& ay0, const ulonglong2& ay1,
                                              const ulonglong2& az0, const ulonglong2& az1,
                                              const float (&D)[kObjPerThread], const float (&nT)[kObjPerThread],
                                              uint32_t& in, uint32_t& un)
{
  float xl, xh, yl, yh, zl, zh;
  upk2(fma2(cz[K], ax1.x, fma2(cy[K], ax0.y, fma2(cx[K], ax0.x, ax1.y))), xl, xh);
  upk2(fma2(cz[K], ay1.x, fma2(cy[K], ay0.y, fma2(cx[K], ay0.x, ay1.y))), yl, yh);
  upk2(fma2(cz[K], az1.x, fma2(cy[K], az0.y, fma2(cx[K], az0.x, az1.y))), zl, zh);
  pf::decide_bits<1u << K>(xl, xh, yl, yh, zl, zh, D[K], nT[K], in, un);
}

// The same without the z-hi plane (the scene bound cleared it): the z-lo value alone, the
// scalar FMA chain of the packed pair's lo half.
template <int K>
__device__ __forceinline__ void decide_object5(const unsigned long long (&cx)[kObjPerThread],
                                               const unsigned long long (&cy)[kObjPerThread],
                                               const unsigned long long (&cz)[kObjPerThread],
                                               const ulonglong2& ax0, const ulonglong2& ax1,
                                               const ulonglong2& ay0, const ulonglong2& ay1, const float4& zq,
                                               const float (&D)[kObjPerThread], const float (&nT)[kObjPerThread],
                                               uint32_t& in, uint32_t& un)
{
  float xl, xh, yl, yh, c0, c1, c2, dup;
  upk2(fma2(cz[K], ax1.x, fma2(cy[K], ax0.y, fma2(cx[K], ax0.x, ax1.y))), xl, xh);
  upk2(fma2(cz[K], ay1.x, fma2(cy[K], ay0.y, fma2(cx[K], ay0.x, ay1.y))), yl, yh);
  upk2(cx[K], c0, dup);
  upk2(cy[K], c1, dup);
  upk2(cz[K], c2, dup);
  const float zl = __fmaf_rn(c2, zq.z, __fmaf_rn(c1, zq.y, __fmaf_rn(c0, zq.x, zq.w)));
  pf::decide_bits5<1u << K>(xl, xh, yl, yh, zl, D[K], nT[K], in, un);
}

// Prefilter of the lane's 4 boxes in each view of the item; returns the undecided pairs
// (bit layout: und_object / und_view below).  With several views the visible bits collect
// as nibbles (bit 4v + k: object k, view v) and one nibble transpose per tile gives every
// lane one visibility word (view lane & 7, word lane >> 3 of the tile): 3 shuffles per tile
// instead of 3 per view.  The views run last to first and each view's nibbles are shifted
// in below the later views' (no per-view shift by v).  With one view the nibble goes to
// its word directly (the 1-view kernel keeps its registers better that way).  Per pair of
// box and view: 9 paired FMAs for the six plane values, then pf::decide_bits against the
// view group's margin (each box's two thresholds are computed once for all the group's
// views): one comparison and one predicated OR per bit.  Branch-free per pair; the view
// loop is not unrolled (nv is uniform over the warp).  SIX = false: the five-plane test of
// a group whose scene bound cleared every z-hi plane (the same bits: pf::far_plane_clear).
template <int VPP, bool SIX = true>
__device__ __forceinline__ uint32_t classify_views(WarpShared& ws, const pf::Box (&bx)[kObjPerThread],
                                                   int nv, uint32_t t, uint32_t valid, int lane)
{
  static_assert(kObjPerThread == 4, "decide_object is called for objects 0..3");
  // Per box: its centre as (c, c) pairs and its two thresholds against the group margin,
  // once for all views.
  unsigned long long cx[kObjPerThread], cy[kObjPerThread], cz[kObjPerThread];
  float D[kObjPerThread], nT[kObjPerThread];
  const pf::GroupMargin gm = ws.gm;
#pragma unroll
  for (int k = 0; k < kObjPerThread; ++k) {
    cx[k] = pk2(bx[k].cx, bx[k].cx);
    cy[k] = pk2(bx[k].cy, bx[k].cy);
    cz[k] = pk2(bx[k].cz, bx[k].cz);
    float T;
    pf::group_thresholds(bx[k], gm, D[k], T);
    nT[k] = -T;
  }
  uint32_t vis_n = 0, und_n = 0;
#pragma unroll 1
  for (int v = nv - 1; v >= 0; --v) {
    const ulonglong2 ax0 = ws.qp[v][0][0], ax1 = ws.qp[v][0][1];
    const ulonglong2 ay0 = ws.qp[v][1][0], ay1 = ws.qp[v][1][1];
    uint32_t in = VPP == 1 ? 0u : vis_n << 4, un = VPP == 1 ? 0u : und_n << 4;
    if (SIX) {
      const ulonglong2 az0 = ws.qp[v][2][0], az1 = ws.qp[v][2][1];
      decide_object<0>(cx, cy, cz, ax0, ax1, ay0, ay1, az0, az1, D, nT, in, un);
      decide_object<1>(cx, cy, cz, ax0, ax1, ay0, ay1, az0, az1, D, nT, in, un);
      decide_object<2>(cx, cy, cz, ax0, ax1, ay0, ay1, az0, az1, D, nT, in, un);
      decide_object<3>(cx, cy, cz, ax0, ax1, ay0, ay1, az0, az1, D, nT, in, un);
    } else {
      const float4 zq = ws.zlo[v];
      decide_object5<0>(cx, cy, cz, ax0, ax1, ay0, ay1, zq, D, nT, in, un);
      decide_object5<1>(cx, cy, cz, ax0, ax1, ay0, ay1, zq, D, nT, in, un);
      decide_object5<2>(cx, cy, cz, ax0, ax1, ay0, ay1, zq, D, nT, in, un);
      decide_object5<3>(cx, cy, cz, ax0, ax1, ay0, ay1, zq, D, nT, in, un);
    }
    if (VPP == 1) {
      // bit k of un -> bit 8k (the multiply places each bit k at 8k; the mask drops the
      // cross terms); one view per pass, so v == 0
      und_n |= ((un & valid) * 0x204081u) & 0x01010101u;
      store_nibble(ws, v, t, in & valid, lane);
    } else {
      vis_n = in;
      und_n = un;
    }
  }
  if (VPP == 1) return und_n;
  const uint32_t vm = valid * 0x11111111u;  // the lane's valid objects in every view
  const uint32_t w = transpose_nibbles8(vis_n & vm, lane);
  if ((lane & 7) < nv) ws.words[lane & 7][t][lane >> 3] = w;
  return und_n & vm;
}

// Object (within the lane's 4) and view of bit b of classify_views' undecided pairs: bit
// 8k + v with one view per pass, bit 4v + k with several.
template <int VPP>
__device__ __forceinline__ uint32_t und_object(int b) { return VPP == 1 ? (uint32_t)b >> 3 : (uint32_t)b & 3u; }
template <int VPP>
__device__ __forceinline__ uint32_t und_view(int b) { return VPP == 1 ? (uint32_t)b & 7u : (uint32_t)b >> 2; }

// Inclusive warp scan.
__device__ __forceinline__ uint32_t warp_scan(uint32_t x, int lane)
{
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
    if (lane >= d) x += y;
  }
  return x;
}

// Runs the queued undecided pairs through the exact test, all lanes together, and sets
// the visible ones in the item's words.  OBBS: the group's OBB cache is valid.
template <bool OBBS>
__device__ __forceinline__ void drain_queue(WarpShared& ws, const CullScene& sc, uint32_t tile_first,
                                            uint32_t qn, int lane)
{
  __syncwarp();
  for (uint32_t q = lane; q < qn; q += 32) {
    const uint32_t e = ws.queue[q];
    const uint32_t t = e >> 10, o = (e >> 3) & 127u, v = e & 7u;
    const uint32_t i = (tile_first + t) * kTileObjects + o;
    if (OBBS ? exact_visible_cached(sc, i, ws.cv[v].vp) : exact_visible(sc, i, ws.cv[v].vp))
      atomicOr(&ws.words[v][t][o >> 5], 1u << (o & 31));
  }
  __syncwarp();
}

template <uint32_t MODE>
__device__ __forceinline__ void drain(WarpShared& ws, const CullScene& sc, uint32_t tile_first, uint32_t qn,
                                      int lane, bool obbs)
{
  if (MODE == kCacheRead && obbs) drain_queue<true>(ws, sc, tile_first, qn, lane);
  else drain_queue<false>(ws, sc, tile_first, qn, lane);
}

// The lane's undecided pairs of tile t into the warp's queue (drained early only if it
// would overflow).  Each lane with pairs takes its slots with one shared-memory atomicAdd
// on the queue's length, so the pairs of a tile land in lane order only by chance; the
// order does not matter (each pair sets its own bit).  Returns the new queue length.
template <int VPP, uint32_t MODE>
__device__ __forceinline__ uint32_t push_undecided(WarpShared& ws, const CullScene& sc, uint32_t tile_first,
                                                   uint32_t t, uint32_t qn, uint32_t amb, int lane, bool obbs)
{
  const uint32_t cnt = (uint32_t)__popc(amb);
  const uint32_t tot = __reduce_add_sync(0xffffffffu, cnt);
  if (tot) {  // uniform over the warp
    if (qn + tot > (uint32_t)kQueueCap) {
      drain<MODE>(ws, sc, tile_first, qn, lane, obbs);
      qn = 0;
      if (lane == 0) ws.qtail = 0u;
      __syncwarp();
    }
    uint32_t pos = cnt ? atomicAdd(&ws.qtail, cnt) : 0u;
    while (amb) {
      const int b = __ffs(amb) - 1;
      ws.queue[pos++] = (uint16_t)((t << 10) | (((uint32_t)lane * kObjPerThread + und_object<VPP>(b)) << 3) |
                                   und_view<VPP>(b));
      amb &= amb - 1u;
    }
    qn += tot;
  }
  return qn;
}

// The lane's 4 prefilter boxes of a tile from the group's box cache.  The Fill launch that
// validated it found every transform index in range, so only the object count limits which
// boxes are used.
__device__ __forceinline__ uint32_t cached_boxes(const CullScene& sc, uint32_t obj0, pf::Box (&bx)[kObjPerThread])
{
  const size_t cap = sc.cap;
  const float4 cx = ld_stream4(sc.box + 0 * cap + obj0), cy = ld_stream4(sc.box + 1 * cap + obj0);
  const float4 cz = ld_stream4(sc.box + 2 * cap + obj0), r = ld_stream4(sc.box + 3 * cap + obj0);
  const float4 d0 = ld_stream4(sc.box + 4 * cap + obj0);
  uint32_t valid = 0;
#pragma unroll
  for (int k = 0; k < kObjPerThread; ++k) {
    bx[k] = pf::Box{comp(cx, k), comp(cy, k), comp(cz, k), comp(r, k), comp(d0, k)};
    valid |= (uint32_t)(obj0 + k < sc.n_objects) << k;
  }
  return valid;
}

// Stores the lane's 4 prefilter boxes into the group's box cache (Fill launches).
__device__ __forceinline__ void store_boxes(const CullScene& sc, uint32_t obj0, const pf::Box (&bx)[kObjPerThread])
{
  const size_t cap = sc.cap;
  __stcg(reinterpret_cast<float4*>(sc.box + 0 * cap + obj0), make_float4(bx[0].cx, bx[1].cx, bx[2].cx, bx[3].cx));
  __stcg(reinterpret_cast<float4*>(sc.box + 1 * cap + obj0), make_float4(bx[0].cy, bx[1].cy, bx[2].cy, bx[3].cy));
  __stcg(reinterpret_cast<float4*>(sc.box + 2 * cap + obj0), make_float4(bx[0].cz, bx[1].cz, bx[2].cz, bx[3].cz));
  __stcg(reinterpret_cast<float4*>(sc.box + 3 * cap + obj0), make_float4(bx[0].r, bx[1].r, bx[2].r, bx[3].r));
  __stcg(reinterpret_cast<float4*>(sc.box + 4 * cap + obj0), make_float4(bx[0].d0, bx[1].d0, bx[2].d0, bx[3].d0));
}

// Fill launches: the tile's boxes into the item's scene bound (the bound words of the
// cache's state block, see pf::far_plane_clear): per lane over its boxes whose margin is a
// number, then one warp reduction per word; lane 0 keeps the item's running maximum.
__device__ __forceinline__ void gather_bound(WarpShared& ws, const pf::Box (&bx)[kObjPerThread], uint32_t valid,
                                             int lane)
{
  uint32_t key[kBoundWords] = {0u, 0u, 0u, 0u, 0u, 0u, 0u};
#pragma unroll
  for (int k = 0; k < kObjPerThread; ++k) {
    if (((valid >> k) & 1u) && bx[k].d0 == bx[k].d0) {
      const uint32_t x = pf::bound_key(bx[k].cx), y = pf::bound_key(bx[k].cy), z = pf::bound_key(bx[k].cz);
      key[0] = max(key[0], x);
      key[1] = max(key[1], y);
      key[2] = max(key[2], z);
      key[3] = max(key[3], ~x);
      key[4] = max(key[4], ~y);
      key[5] = max(key[5], ~z);
      key[6] = max(key[6], pf::bound_key(bx[k].d0));
    }
  }
#pragma unroll
  for (int w = 0; w < kBoundWords; ++w) {
    const uint32_t m = __reduce_max_sync(0xffffffffu, key[w]);
    if (lane == 0) ws.bnd[w] = max(ws.bnd[w], m);
  }
}

// Classification of one tile into the item's words (visible objects) and queue
// (undecided pairs).  Returns the new queue length.  WIDE: the scene's matrix array is
// 32-byte aligned (two 256-bit loads per matrix).  MODE: the fused kernel computes the
// boxes from the rows and the world matrices, the Fill kernel also stores them (and the
// OBBs), the cached kernel reads them (cache_ok: the scene's cache is valid; if not, every
// pair of the tile goes to the exact test).
template <int VPP, bool PF, bool WIDE, uint32_t MODE>
__device__ __forceinline__ uint32_t classify_tile(const CullLaunch& a, WarpShared& ws, const CullScene& sc,
                                                  uint32_t tile, uint32_t t, uint32_t tile_first,
                                                  uint32_t n_t, int nv, uint32_t qn, int lane, bool cache_ok,
                                                  const uint4 xf_cur, uint4& xf_next)
{
  const uint32_t obj0 = tile * kTileObjects + (uint32_t)lane * kObjPerThread;
  const float* soa = sc.soa;
  const size_t cap = sc.cap;
  if (PF && MODE == kCacheRead) {
    pf::Box bx[kObjPerThread];
    uint32_t amb;
    if (cache_ok) {
      // The next tile's boxes into L1 while this tile is classified (5 x 512 bytes per
      // warp; the loads below of the tile after hit there).
      if (t + 1 < n_t) {
        const float* nb = sc.box + obj0 + kTileObjects;
#pragma unroll
        for (int r = 0; r < kBoxRows; ++r) asm volatile("prefetch.global.L1 [%0];" ::"l"(nb + r * cap));
      }
      const uint32_t valid = cached_boxes(sc, obj0, bx);
      amb = ws.far_off ? classify_views<VPP, false>(ws, bx, nv, t, valid, lane)
                       : classify_views<VPP, true>(ws, bx, nv, t, valid, lane);
    } else {
      // A Stale cache (the host never launches this kernel on one): no visible bit from the
      // prefilter, every pair of the lane's objects to the exact test.
      uint32_t valid = 0;
#pragma unroll
      for (int k = 0; k < kObjPerThread; ++k) valid |= (uint32_t)(obj0 + k < sc.n_objects) << k;
      if (VPP == 1) {
        amb = (valid * 0x204081u) & 0x01010101u;
        store_nibble(ws, 0, t, 0u, lane);
      } else {
        amb = (valid * 0x11111111u) & (nv >= 8 ? 0xFFFFFFFFu : (1u << (4 * nv)) - 1u);
        if ((lane & 7) < nv) ws.words[lane & 7][t][lane >> 3] = 0u;
      }
    }
    return push_undecided<VPP, MODE>(ws, sc, tile_first, t, qn, amb, lane, cache_ok);
  }
  // The transform indices of this tile were loaded one tile ahead, so the matrix gathers
  // below go out together with the other rows; the next tile's indices go out now.
  const uint4 xf = xf_cur;
  if (t + 1 < n_t) xf_next = ld_stream4u(soa + 6 * cap + obj0 + kTileObjects);
  const float4 lx = ld_stream4(soa + 0 * cap + obj0);
  const float4 ly = ld_stream4(soa + 1 * cap + obj0);
  const float4 lz = ld_stream4(soa + 2 * cap + obj0);
  const float4 ex = ld_stream4(soa + 3 * cap + obj0);
  const float4 ey = ld_stream4(soa + 4 * cap + obj0);
  const float4 ez = ld_stream4(soa + 5 * cap + obj0);
  if (PF) {
    // Prefilter boxes of the 4 objects first (their matrix gathers overlap), then each
    // view's planes are read once for all 4 objects.
    pf::Box bx[kObjPerThread];
    uint32_t valid = 0, bad = 0;
#pragma unroll
    for (int k = 0; k < kObjPerThread; ++k) {
      const uint32_t mi = compu(xf, k);
      const bool exists = obj0 + k < sc.n_objects;
      const bool use = exists & (mi < sc.n_mats);
      // A transform index past the matrix array is reported and its object skipped.  With
      // several views one test per tile is cheaper; the 1-view kernel allocates its
      // registers better with the test per object.
      if (VPP > 1) bad |= (uint32_t)(exists & !use) << k;
      else if (exists && !use && atomicOr(&a.ctl->error, kErrBadTransform) == 0) a.ctl->error_info = obj0 + k;
      float4 r0 = make_float4(0.f, 0.f, 0.f, 0.f), r1 = r0, r2 = r0, r3 = r0;
      if (use) load_matrix(sc.mats + 16 * (size_t)mi, WIDE, r0, r1, r2, r3);
      const pf::F4 m0{r0.x, r0.y, r0.z, r0.w}, m1{r1.x, r1.y, r1.z, r1.w};
      const pf::F4 m2{r2.x, r2.y, r2.z, r2.w}, m3{r3.x, r3.y, r3.z, r3.w};
      bx[k] = pf::make_box(comp(lx, k), comp(ly, k), comp(lz, k), comp(ex, k), comp(ey, k),
                           comp(ez, k), m0, m1, m2, m3);
      // Boxes stored in the cache are read by every later launch: the tighter radius pays.
      if (MODE == kCacheFill && sc.box)
        bx[k].r = pf::tight_radius(comp(ex, k), comp(ey, k), comp(ez, k), m0, m1, m2, bx[k].r);
      if (MODE == kCacheFill && use && sc.box)
        store_obb(sc, obj0 + k, make_obb(comp(lx, k), comp(ly, k), comp(lz, k), comp(ex, k), comp(ey, k),
                                         comp(ez, k), r0, r1, r2, r3));
      valid |= (uint32_t)use << k;
    }
    if (VPP > 1 && bad) {
      const uint32_t o = obj0 + (uint32_t)__ffs(bad) - 1u;
      if (atomicOr(&a.ctl->error, kErrBadTransform) == 0) a.ctl->error_info = o;
    }
    if (MODE == kCacheFill && sc.box) {
      store_boxes(sc, obj0, bx);
      gather_bound(ws, bx, valid, lane);
    }
    const uint32_t amb = classify_views<VPP>(ws, bx, nv, t, valid, lane);
    return push_undecided<VPP, MODE>(ws, sc, tile_first, t, qn, amb, lane, false);
  }
  // Exact test only: every pair in the reference's operation order (the box is rebuilt
  // per view from the loaded rows; the matrix reloads hit L1).
  const float4* mats = reinterpret_cast<const float4*>(sc.mats);
  uint32_t use = 0;
#pragma unroll
  for (int k = 0; k < kObjPerThread; ++k) {
    if (obj0 + k < sc.n_objects) {
      if (compu(xf, k) < sc.n_mats) use |= 1u << k;
      else if (atomicOr(&a.ctl->error, kErrBadTransform) == 0) a.ctl->error_info = obj0 + k;
    }
  }
#pragma unroll 1
  for (int v = 0; v < nv; ++v) {
    uint32_t nib = 0;
#pragma unroll
    for (int k = 0; k < kObjPerThread; ++k) {
      if (use & (1u << k)) {
        const float4* M = mats + 4 * (size_t)compu(xf, k);
        const Obb o = make_obb(comp(lx, k), comp(ly, k), comp(lz, k), comp(ex, k), comp(ey, k),
                               comp(ez, k), __ldg(M + 0), __ldg(M + 1), __ldg(M + 2), __ldg(M + 3));
        if (obb_visible(o, ws.cv[v].vp)) nib |= 1u << k;
      }
    }
    store_nibble(ws, v, t, nib, lane);
  }
  return qn;
}

// The final words of the item, per view: the new words (stored only where they changed),
// the delta words (old XOR new, every word) and, for serving launches, the visible count.
// The lanes take (view, word) pairs: a view's words occupy 32 lanes (16 for an item of 2
// to 4 tiles, 4 for a single-tile item), so 1 (2, 8) views go per pass and the 8 views of
// an item take 8 passes (4, 1).  Every
// pass's previous words are loaded before any store, so the loads are in flight together.
template <int VPP>
__device__ __forceinline__ void finish_item(const WarpShared& ws, uint32_t tile_first, uint32_t n_t,
                                            int nv, int lane)
{
  constexpr int kPasses = (VPP * kItemTiles * kTileWords + 31) / 32;
  const uint32_t wpv = n_t * kTileWords;  // the item's words per view
  const int sh = n_t == 1 ? 2 : n_t <= 4 ? 4 : 5;  // lanes per view: 4, 16 or 32
  const uint32_t base = tile_first * kTileWords;
  uint32_t prev[kPasses];
#pragma unroll
  for (int i = 0; i < kPasses; ++i) {
    const uint32_t p = (uint32_t)lane + 32u * i, v = p >> sh, wd = p & ((1u << sh) - 1u);
    const bool act = v < (uint32_t)nv && wd < wpv;
    prev[i] = act && !(ws.cv[v].flags & kViewNoChanged) ? ws.cv[v].bits[base + wd] : 0u;
  }
#pragma unroll
  for (int i = 0; i < kPasses; ++i) {
    const uint32_t p = (uint32_t)lane + 32u * i, v = p >> sh, wd = p & ((1u << sh) - 1u);
    if (v < (uint32_t)nv && wd < wpv) {
      const CullView& cv = ws.cv[v];
      const uint32_t w = (&ws.words[v][0][0])[wd];
      if (cv.flags & kViewNoChanged) {
        cv.bits[base + wd] = w;
      } else {
        const uint32_t d = w ^ prev[i];
        if (d) cv.bits[base + wd] = w;
        cv.delta[base + wd] = d;
      }
      if (cv.copy_bits) cv.copy_bits[base + wd] = w;
    }
  }
  if (ws.cv[0].n_visible) {  // serving launches count every view's visible objects
    const bool mine = (uint32_t)lane < wpv;
#pragma unroll
    for (int v = 0; v < VPP; ++v) {
      if (v < nv && ws.cv[v].n_visible) {
        const uint32_t w = mine ? (&ws.words[v][0][0])[lane] : 0u;
        const uint32_t cnt = __reduce_add_sync(0xffffffffu, (uint32_t)__popc(w));
        if (lane == 0 && cnt) atomicAdd(ws.cv[v].n_visible, cnt);
      }
    }
  }
}

// One work item (up to kItemTiles tiles of 128 objects x one group of up to VPP views)
// by one warp.  ws.sc and `vkey` cache the warp's current scene and staged view group
// across items.
template <int VPP, bool PF, bool WIDE, uint32_t MODE>
__device__ __forceinline__ void warp_item(const CullLaunch& a, uint32_t item, WarpShared& ws,
                                          uint32_t& vkey)
{
  const int lane = threadIdx.x & 31;
  __syncwarp();  // the previous item's reads of the shared state are done
  if ((uint64_t)(item - ws.sc.item_begin) >=
      (uint64_t)tile_groups_of(ws.sc.n_tiles, ws.sc.n_big, a.item_tiles) * ws.sc.n_vgroups) {
    const CullScene* src = a.scenes ? a.scenes + find_scene(a.scenes, a.n_scenes, item) : &a.one_scene;
    constexpr int kSceneWords = (int)(sizeof(CullScene) / 4);
    if (lane < kSceneWords) reinterpret_cast<uint32_t*>(&ws.sc)[lane] = reinterpret_cast<const uint32_t*>(src)[lane];
    __syncwarp();
  }
  const CullScene& sc = ws.sc;
  if (WIDE && ((uintptr_t)sc.mats & 31u)) {  // the launch's alignment promise does not hold:
    if (lane == 0 && atomicOr(&a.ctl->error, kErrMisaligned) == 0) a.ctl->error_info = item;
    return;                                  // report it, load nothing
  }
  const uint32_t local = item - sc.item_begin;
  const uint32_t group = local / sc.n_vgroups;
  const uint32_t vfirst = (local - group * sc.n_vgroups) * VPP;
  const int nv = (int)min((uint32_t)VPP, sc.n_views - vfirst);
  const bool big = group < sc.n_big;  // else one of the scene's single-tile items
  const uint32_t tile_first = big ? group * a.item_tiles : sc.n_big * a.item_tiles + (group - sc.n_big);
  const uint32_t n_t = big ? min(a.item_tiles, sc.n_tiles - tile_first) : 1u;
  // The cached kernel reads the scene's cache state once per item (it does not change
  // during a launch); the other kernels load the first tile's transform indices while the
  // views are staged.
  const bool cache_ok = PF && MODE == kCacheRead && sc.box && __ldcg(sc.box_state) == kBoxValid;
  uint4 xf_first = make_uint4(0u, 0u, 0u, 0u);
  if (!(PF && MODE == kCacheRead))
    xf_first = ld_stream4u(sc.soa + 6 * (size_t)sc.cap + tile_first * kTileObjects + (uint32_t)lane * kObjPerThread);

  // Stage the views (matrices and output pointers) and their prefilter planes in the
  // warp's shared memory when the view group changes; consecutive items of one scene
  // keep them.
  const uint32_t key = sc.view_begin + vfirst;
  if (key != vkey) {
    constexpr int kViewWords = (int)(sizeof(CullView) / 4);
    static_assert(sizeof(CullView) % 16 == 0, "CullView is staged as whole words");
    const uint32_t* src = reinterpret_cast<const uint32_t*>(a.views ? a.views + key : &a.one_view);
    for (int i = lane; i < nv * kViewWords; i += 32) reinterpret_cast<uint32_t*>(ws.cv)[i] = src[i];
    __syncwarp();
    if (PF) {
      pf::GroupMargin m{0.f, 0.f};
      pf::Planes pl;
      if (lane < nv) {
        pf::group_view(ws.cv[lane].vp, pl, m);
        for (int ax = 0; ax < 3; ++ax) {
          const pf::F4 lo = pl.q[ax][0], hi = pl.q[ax][1];
          ws.qp[lane][ax][0] = make_ulonglong2(pk2(lo.x, hi.x), pk2(lo.y, hi.y));
          ws.qp[lane][ax][1] = make_ulonglong2(pk2(lo.z, hi.z), pk2(lo.w, hi.w));
        }
        if (MODE == kCacheRead) ws.zlo[lane] = make_float4(pl.q[2][0].x, pl.q[2][0].y, pl.q[2][0].z, pl.q[2][0].w);
      }
      // the group margin: the largest over the views (lanes past nv contribute zeros)
#pragma unroll
      for (int d = 1; d < kMaxViewsPerPass; d <<= 1)
        m = pf::merge(m, pf::GroupMargin{__shfl_xor_sync(0xffffffffu, m.k, d), __shfl_xor_sync(0xffffffffu, m.g, d)});
      if (lane == 0) ws.gm = m;
      if (MODE == kCacheRead) {
        // Five planes when the scene bound clears the z-hi plane of every view of the group
        // (read only where the cache is valid: cache_ok guards every use).
        bool clear = false;
        if (lane < nv && sc.box) {
          float lo[3], hi[3];
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            hi[k] = pf::bound_value(__ldcg(sc.box_state + 1 + k));
            lo[k] = pf::bound_value(~__ldcg(sc.box_state + 4 + k));
          }
          clear = pf::far_plane_clear(pl.q[2][1], lo, hi, pf::bound_value(__ldcg(sc.box_state + 7)), m);
        }
        const uint32_t all = nv >= 32 ? ~0u : (1u << nv) - 1u;
        const uint32_t got = __ballot_sync(0xffffffffu, clear);
        if (lane == 0) ws.far_off = (got & all) == all ? 1u : 0u;
      }
    }
    __syncwarp();
    vkey = key;
  }

  if (PF && MODE == kCacheFill) {  // the item's scene bound starts empty
    if (lane < kBoundWords) ws.bnd[lane] = 0u;
    __syncwarp();
  }
  uint32_t qn = 0;
  if (lane == 0) ws.qtail = 0u;
  __syncwarp();
  uint4 xf = xf_first;
  for (uint32_t t = 0; t < n_t; ++t) {
    uint4 xf_next = make_uint4(0u, 0u, 0u, 0u);
    qn = classify_tile<VPP, PF, WIDE, MODE>(a, ws, sc, tile_first + t, t, tile_first, n_t, nv, qn, lane, cache_ok, xf,
                                            xf_next);
    xf = xf_next;
  }
  if (PF && qn) drain<MODE>(ws, sc, tile_first, qn, lane, cache_ok);
  else __syncwarp();
  finish_item<VPP>(ws, tile_first, n_t, nv, lane);
  if (PF && MODE == kCacheFill && sc.box) {  // the item's bound into the scene's
    __syncwarp();
    if (lane < kBoundWords && ws.bnd[lane]) atomicMax(sc.box_state + 1 + lane, ws.bnd[lane]);
  }
}

// The changed list of a view whose delta words fit one chunk, by one CTA (defined with the
// changed-list assembly below).
__device__ void emit_small_view(const CullView& v);

// The kernels that transform the boxes hold 80 registers (3 CTAs of 256 threads per SM);
// the one that reads the box cache needs fewer and runs at 4.
template <int VPP, bool PF, bool WIDE, uint32_t MODE>
__global__ void __launch_bounds__(kThreads, MODE == kCacheRead ? 4 : 3) cull_kernel(const __grid_constant__ CullLaunch a)
{
  __shared__ WarpShared wsh[kThreads / 32];
  WarpShared& ws = wsh[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  CullControl* ctl = a.ctl;
  // The changed-list kernel after this one may start launching once every CTA of this
  // grid runs (it waits for this grid's completion before it reads anything).
  asm volatile("griddepcontrol.launch_dependents;");
  if (threadIdx.x % 32 == 0) {
    ws.sc.item_begin = 0;  // no scene cached: the first item looks its scene up
    ws.sc.n_tiles = 0;
    ws.sc.n_big = 0;
    ws.sc.n_vgroups = 1;
  }
  uint32_t vkey = ~0u;
  // Each warp claims its own tickets; the next claim is issued before the current items
  // are processed, so its round trip overlaps them.
  uint32_t first = 0;
  if (lane == 0) first = atomicAdd(&ctl->ticket, a.items_per_ticket);
  first = __shfl_sync(0xffffffffu, first, 0);
  while (first < a.n_items) {
    uint32_t next = 0;
    if (lane == 0) next = atomicAdd(&ctl->ticket, a.items_per_ticket);
    const uint32_t last = min(first + a.items_per_ticket, a.n_items);
    for (uint32_t item = first; item < last; ++item) warp_item<VPP, PF, WIDE, MODE>(a, item, ws, vkey);
    first = __shfl_sync(0xffffffffu, next, 0);
  }
  __shared__ bool last_cta;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();  // this CTA's stores (words, cached boxes) before its count
    last_cta = atomicAdd(&ctl->done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last_cta) {
    // Last CTA of the launch: every other CTA has finished.  A Fill launch validates the
    // caches it stored (not after finding a bad transform index); then the ticket is reset
    // for the next launch (no memset needed).
    if (PF && MODE == kCacheFill && *(volatile unsigned int*)&ctl->error == 0u) {
      const uint32_t ns = a.scenes ? a.n_scenes : 1u;
      for (uint32_t i = threadIdx.x; i < ns; i += blockDim.x) {
        const CullScene& sc = a.scenes ? a.scenes[i] : a.one_scene;
        if (sc.box) *sc.box_state = kBoxValid;
      }
    }
    if (threadIdx.x == 0) {
      ctl->ticket = 0;
      ctl->done = 0;
    }
    // Small launches: the changed lists too (every CTA's delta words are visible: each
    // fenced its stores before counting itself done).
    for (uint32_t v = 0; v < a.emit_views; ++v) emit_small_view(a.views ? a.views[v] : a.one_view);
  }
}

// ---- changed-list assembly ----------------------------------------------------------------
// One pass over a view's delta words in chunks of kEmitChunk words, one block each: the
// blocks of a view take their chunks in the order they start (a ticket), count their
// chunk's changed objects and publish the count, then add the earlier chunks' counts
// (published by blocks that started before them, so the wait always ends) and write every
// changed index, ascending.  The view's last block clears the counts for the next launch.
// Each warp owns 1024 consecutive words of its block's chunk, read in 8 rounds of one
// coalesced uint4 per lane, and writes each round's changed indices after a warp scan, so
// the lanes of a warp store into one stretch of the list.  Blocks of 256 threads with at
// most 64 registers: 4 per SM, so the 16M-object stress views (62 chunks x 8 views) run in
// one wave.  The small-launch path in the cull's last CTA (emit_small_view) keeps chunks
// of kDeltaChunk words, 16 per thread.
constexpr int kScanThreads = 256;
constexpr int kEmitRounds = 8;                                        // uint4 rounds per warp
constexpr uint32_t kEmitWarpWords = 32u * 4u * kEmitRounds;           // 1024
constexpr uint32_t kEmitChunk = kScanThreads / 32 * kEmitWarpWords;   // 8192 words per block
static_assert(kEmitChunk % kDeltaChunk == 0, "a view's emit chunks fit its scratch counts");
static_assert(kEmitChunk == kEmitChunkWords, "the host sizes the pass with kEmitChunkWords");
constexpr int kWordsPerThread = kDeltaChunk / kScanThreads;
static_assert(kWordsPerThread % 4 == 0, "whole uint4 loads");
constexpr uint32_t kSpinLimit = 1u << 20;  // polls of an earlier chunk's count (~0.1 s)

// The thread's delta words (n_words is a multiple of 4, the arrays 16-byte aligned).
__device__ __forceinline__ void load_delta(const CullView& v, uint32_t b, uint32_t (&w)[kWordsPerThread])
{
#pragma unroll
  for (int j = 0; j < kWordsPerThread; j += 4) {
    uint4 q = make_uint4(0u, 0u, 0u, 0u);
    if (b + j < v.n_words) q = __ldcg(reinterpret_cast<const uint4*>(v.delta + b + j));
    w[j] = q.x;
    w[j + 1] = q.y;
    w[j + 2] = q.z;
    w[j + 3] = q.w;
  }
}

// Block-wide exclusive scan of one value per thread; the block total goes to *total.
__device__ __forceinline__ uint32_t block_scan(uint32_t x, uint32_t* wsum, uint32_t* total)
{
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t incl = warp_scan(x, lane);
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    const uint32_t w = lane < kScanThreads / 32 ? wsum[lane] : 0u;
    const uint32_t wi = warp_scan(w, lane);
    if (lane < kScanThreads / 32) wsum[lane] = wi - w;
    if (lane == 31) *total = wi;
  }
  __syncthreads();
  return wsum[warp] + incl - x;
}

// A warp's 8 rounds of delta words from word `base` (n_words is a multiple of 4 and the
// array 16-byte aligned, so a round's uint4 is whole or past the end).
__device__ __forceinline__ void load_rounds(const uint32_t* delta, uint32_t n_words, uint32_t base, int lane,
                                            uint4 (&q)[kEmitRounds])
{
#pragma unroll
  for (int k = 0; k < kEmitRounds; ++k) {
    const uint32_t i = base + (uint32_t)k * 128u + 4u * (uint32_t)lane;
    q[k] = i < n_words ? __ldcg(reinterpret_cast<const uint4*>(delta + i)) : make_uint4(0u, 0u, 0u, 0u);
  }
}

// The set bits of one delta word as object indices at out[p], out[p + 1], ...
__device__ __forceinline__ void emit_word(uint32_t m, uint32_t word, uint32_t* changed, uint32_t* copy, uint32_t& p)
{
  while (m) {
    const uint32_t obj = word * 32u + (uint32_t)(__ffs(m) - 1);
    changed[p] = obj;
    if (copy) copy[p] = obj;
    ++p;
    m &= m - 1u;
  }
}

// grid = (chunks of kEmitChunk words, views), or (blocks of all views) with first_block
__global__ void __launch_bounds__(kScanThreads, 4)
    emit_changed_kernel(const CullView* views, const __grid_constant__ CullView one, unsigned int* err,
                        const uint32_t* first_block, uint32_t n_views)
{
  __shared__ uint32_t woff[kScanThreads / 32];
  __shared__ uint32_t wbefore[kScanThreads / 32];
  __shared__ uint32_t tot;
  __shared__ uint32_t chunk;
  __shared__ bool last;
  // Launched as a programmatic dependent of the cull.  The view (written before the cull
  // started) and the chunk ticket (cleared by the previous launch) do not depend on it, so
  // the block reads and takes them while the cull's last CTAs run; then it waits for the
  // cull's grid and its memory.
  uint32_t vi = blockIdx.y, bx = blockIdx.x;
  if (first_block) {  // the last view whose first block is at or before this one
    uint32_t lo = 0, hi = n_views;
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (__ldg(first_block + mid) <= blockIdx.x) lo = mid;
      else hi = mid;
    }
    vi = lo;
    bx = blockIdx.x - __ldg(first_block + lo);
  }
  const CullView& v = views ? views[vi] : one;
  if (v.flags & kViewNoChanged) return;  // uniform
  const uint32_t n_words = v.n_words;
  const uint32_t n_chunks = (n_words + kEmitChunk - 1) / kEmitChunk;
  if (bx >= n_chunks) {  // uniform; only the view's first n_chunks blocks take tickets
    asm volatile("griddepcontrol.wait;" ::: "memory");
    if (bx == 0 && threadIdx.x == 0) {
      *v.n_changed = 0;
      if (v.copy_count) *v.copy_count = 0;
    }
    return;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t* state = v.chunk_tot;  // per chunk: its count + 1 once published
  uint32_t* ticket = state + n_chunks;
  uint32_t* done = ticket + 1;
  const uint32_t* delta = v.delta;
  if (threadIdx.x == 0) chunk = atomicAdd(ticket, 1u);
  __syncthreads();
  const uint32_t c = chunk;
  asm volatile("griddepcontrol.wait;" ::: "memory");
  uint4 q[kEmitRounds];
  load_rounds(delta, n_words, c * kEmitChunk + (uint32_t)warp * kEmitWarpWords, lane, q);
  uint32_t cnt[kEmitRounds];
  uint32_t mine = 0;
#pragma unroll
  for (int k = 0; k < kEmitRounds; ++k) {
    cnt[k] = (uint32_t)(__popc(q[k].x) + __popc(q[k].y) + __popc(q[k].z) + __popc(q[k].w));
    mine += cnt[k];
  }
  const uint32_t wtot = __reduce_add_sync(0xffffffffu, mine);
  if (lane == 0) woff[warp] = wtot;
  __syncthreads();
  if (warp == 0) {
    const uint32_t x = lane < kScanThreads / 32 ? woff[lane] : 0u;
    const uint32_t incl = warp_scan(x, lane);
    if (lane < kScanThreads / 32) woff[lane] = incl - x;
    if (lane == 31) tot = incl;
  }
  __syncthreads();
  const uint32_t count = tot;
  if (threadIdx.x == 0) atomicExch(state + c, count + 1u);
  // Changed objects of the earlier chunks: their blocks took earlier tickets, so they are
  // running or done and publish without waiting for anything.
  uint32_t before = 0;
  bool gave_up = false;
  for (uint32_t i = threadIdx.x; i < c; i += kScanThreads) {
    uint32_t x = *(volatile const uint32_t*)(state + i);
    for (uint32_t spins = 0; x == 0u; ++spins) {
      if (spins == kSpinLimit) {
        gave_up = true;
        x = 1u;
        break;
      }
      __nanosleep(64);
      x = *(volatile const uint32_t*)(state + i);
    }
    before += x - 1u;
  }
  if (gave_up) atomicOr(err, kErrWaitTimeout);
  const uint32_t wb = __reduce_add_sync(0xffffffffu, before);
  if (lane == 0) wbefore[warp] = wb;
  __syncthreads();
  uint32_t base = 0;
#pragma unroll
  for (int i = 0; i < kScanThreads / 32; ++i) base += wbefore[i];
  if (threadIdx.x == 0 && c == n_chunks - 1) {
    const uint32_t n = base + count;
    *v.n_changed = n;
    if (v.copy_count) *v.copy_count = n;
  }
  // This block has read every count it needs; the count of finished blocks tells the last
  // one (its return value is waited for only after the writes).
  uint32_t finished = 0;
  if (threadIdx.x == 0) finished = atomicAdd(done, 1u);
  uint32_t* const changed = v.changed;
  uint32_t* const copy = v.copy_changed;
  uint32_t pos = base + woff[warp];
  const uint32_t wbase = c * kEmitChunk + (uint32_t)warp * kEmitWarpWords + 4u * (uint32_t)lane;
#pragma unroll
  for (int k = 0; k < kEmitRounds; ++k) {
    const uint32_t incl = warp_scan(cnt[k], lane);
    uint32_t p = pos + incl - cnt[k];
    pos += __shfl_sync(0xffffffffu, incl, 31);
    const uint32_t wd = wbase + (uint32_t)k * 128u;
    emit_word(q[k].x, wd, changed, copy, p);
    emit_word(q[k].y, wd + 1u, changed, copy, p);
    emit_word(q[k].z, wd + 2u, changed, copy, p);
    emit_word(q[k].w, wd + 3u, changed, copy, p);
  }
  // The last block past its reads clears the counts, the ticket and the block count.
  if (threadIdx.x == 0) last = finished == n_chunks - 1;
  __syncthreads();
  if (last) {
    for (uint32_t i = threadIdx.x; i < n_chunks; i += kScanThreads) state[i] = 0u;
    if (threadIdx.x == 0) {
      *ticket = 0u;
      *done = 0u;
    }
  }
}

// One view's changed list from its delta words, all in one chunk: chunk count and block
// scan in one block (the cull kernel's last CTA, kScanThreads threads).
static_assert(kThreads == kScanThreads, "the cull kernel's CTA runs the block scan");
__device__ void emit_small_view(const CullView& v)
{
  __shared__ uint32_t wsum[kScanThreads / 32];
  __shared__ uint32_t tot;
  if (v.flags & kViewNoChanged) return;  // uniform
  const uint32_t b = threadIdx.x * kWordsPerThread;
  uint32_t w[kWordsPerThread];
  load_delta(v, b, w);
  uint32_t s = 0;
#pragma unroll
  for (int j = 0; j < kWordsPerThread; ++j) s += (uint32_t)__popc(w[j]);
  uint32_t pos = block_scan(s, wsum, &tot);
  if (threadIdx.x == 0) {
    *v.n_changed = tot;
    if (v.copy_count) *v.copy_count = tot;
  }
#pragma unroll
  for (int j = 0; j < kWordsPerThread; ++j) {
    uint32_t m = w[j];
    while (m) {
      const int k = __ffs(m) - 1;
      const uint32_t obj = (b + (uint32_t)j) * 32u + (uint32_t)k;
      v.changed[pos] = obj;
      if (v.copy_changed) v.copy_changed[pos] = obj;
      ++pos;
      m &= m - 1u;
    }
  }
  __syncthreads();  // wsum and tot are used again for the next view
}

template <int VPP, bool WIDE>
void launch_pf(const CullLaunch& a, int grid, cudaStream_t s)
{
  if (a.cache_mode == kCacheRead) cull_kernel<VPP, true, WIDE, kCacheRead><<<grid, kThreads, 0, s>>>(a);
  else if (a.cache_mode == kCacheFill) cull_kernel<VPP, true, WIDE, kCacheFill><<<grid, kThreads, 0, s>>>(a);
  else cull_kernel<VPP, true, WIDE, kCacheNone><<<grid, kThreads, 0, s>>>(a);
}

template <int VPP>
int launch_vpp(const CullLaunch& a, int grid, cudaStream_t s)
{
  if (a.exact_only) cull_kernel<VPP, false, false, kCacheNone><<<grid, kThreads, 0, s>>>(a);
  else if (a.wide_mats) launch_pf<VPP, true>(a, grid, s);
  else launch_pf<VPP, false>(a, grid, s);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

template <int VPP, uint32_t MODE>
int max_ctas()
{
  static std::atomic<int> cached{0};  // the same on every GB300: threads that race store the same value
  const int known = cached.load(std::memory_order_relaxed);
  if (known) return known;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, cull_kernel<VPP, true, true, MODE>, kThreads, 0) !=
      cudaSuccess)
    return 1;
  n = n > 0 ? n : 1;
  cached.store(n, std::memory_order_relaxed);
  return n;
}

template <int VPP>
int max_ctas_mode(uint32_t mode)
{
  return mode == kCacheRead ? max_ctas<VPP, kCacheRead>() : mode == kCacheFill ? max_ctas<VPP, kCacheFill>()
                                                                               : max_ctas<VPP, kCacheNone>();
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

// grid = (blocks, results): copies each result's words and changed list (its length read
// here, on the device) into the snapshot buffers.
__global__ void snapshot_kernel(const ResultCopy* copies)
{
  const ResultCopy c = copies[blockIdx.y];
  const uint32_t count = *c.n_changed;
  if (blockIdx.x == 0 && threadIdx.x == 0) *c.dst_count = count;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < c.n_words; i += stride)
    c.dst_bits[i] = __ldcg(c.bits + i);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride)
    c.dst_changed[i] = __ldcg(c.changed + i);
}

// A plan's views from their pinned host slot into device memory (the first node of the
// plan's graph): a kernel reads the host buffer directly, which starts the cull sooner
// than a copy-engine transfer of the same ~1 KB would.
__global__ void copy_words_kernel(uint32_t* dst, const uint32_t* src, uint32_t n)
{
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = src[i];
}

// The same 16 bytes per thread, with a grid of one uint4 per thread: every read of host
// memory is in flight at once (each is a round trip to the host).
__global__ void copy_quads_kernel(uint4* dst, const uint4* src, uint32_t n)
{
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = src[i];
}

// GroupBitSet::removeObject moves the last object into the hole: SoA row copy.
__global__ void move_object_kernel(float* soa, uint32_t cap, uint32_t from, uint32_t to)
{
  const int r = threadIdx.x;
  if (r < 7) soa[(size_t)r * cap + to] = soa[(size_t)r * cap + from];
}

}  // namespace

int launch_cull(const CullLaunch& args, int grid, int vpp, void* stream)
{
  if (args.item_tiles < 1 || args.item_tiles > (uint32_t)kItemTiles) return -1;
  CullLaunch a = args;
  if (!a.scenes) a.wide_mats = ((uintptr_t)a.one_scene.mats & 31u) == 0 ? 1u : 0u;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  switch (vpp) {
    case 1: return launch_vpp<1>(a, grid, s);
    case 2: return launch_vpp<2>(a, grid, s);
    case 4: return launch_vpp<4>(a, grid, s);
    case 8: return launch_vpp<8>(a, grid, s);
    default: return -1;
  }
}

int cull_max_ctas_per_sm(int vpp, uint32_t mode)
{
  switch (vpp) {
    case 1: return max_ctas_mode<1>(mode);
    case 2: return max_ctas_mode<2>(mode);
    case 4: return max_ctas_mode<4>(mode);
    case 8: return max_ctas_mode<8>(mode);
    default: return 1;
  }
}

int launch_changed_lists(const CullView* views, const CullView& one, uint32_t n_views,
                         uint32_t max_words, unsigned int* err, void* stream, const uint32_t* first_block,
                         uint32_t n_blocks)
{
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!n_views) return 0;
  const uint32_t chunks = std::max<uint32_t>(1, (max_words + kEmitChunk - 1) / kEmitChunk);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = first_block ? dim3(n_blocks) : dim3(chunks, n_views);
  cfg.blockDim = dim3(kScanThreads);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (cudaLaunchKernelEx(&cfg, emit_changed_kernel, views, one, err, first_block, n_views) != cudaSuccess) return -1;
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_copy_words(uint32_t* dst, const uint32_t* src, size_t n_words, void* stream)
{
  if (!n_words) return 0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (n_words % 4 == 0 && ((uintptr_t)dst & 15u) == 0 && ((uintptr_t)src & 15u) == 0) {
    const size_t n = n_words / 4;
    const unsigned blocks = (unsigned)std::min<size_t>(1024, (n + 255) / 256);
    copy_quads_kernel<<<blocks, 256, 0, s>>>(reinterpret_cast<uint4*>(dst), reinterpret_cast<const uint4*>(src),
                                             (uint32_t)n);
  } else {
    const unsigned blocks = (unsigned)std::min<size_t>(1024, (n_words + 255) / 256);
    copy_words_kernel<<<blocks, 256, 0, s>>>(dst, src, (uint32_t)n_words);
  }
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_move_bit(uint32_t* bits, uint32_t size_bits, uint32_t old_index, uint32_t new_index,
                    void* stream)
{
  move_bit_kernel<<<1, 1, 0, static_cast<cudaStream_t>(stream)>>>(bits, size_bits, old_index,
                                                                  new_index);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_snapshot(const ResultCopy* copies, uint32_t n, uint32_t max_len, void* stream)
{
  if (!n) return 0;
  const uint32_t blocks = std::max<uint32_t>(1, std::min<uint32_t>(256, (max_len + 4095) / 4096));
  snapshot_kernel<<<dim3(blocks, n), 256, 0, static_cast<cudaStream_t>(stream)>>>(copies);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_move_object(float* soa, uint32_t cap, uint32_t from, uint32_t to, void* stream)
{
  move_object_kernel<<<1, 32, 0, static_cast<cudaStream_t>(stream)>>>(soa, cap, from, to);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace dpcull
