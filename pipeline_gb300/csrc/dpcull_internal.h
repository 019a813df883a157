// dpcull_internal.h -- shared host/device definitions of the GB300 culling backend.
//
// Data layout in HBM (one allocation per culling group):
//   lower.x | lower.y | lower.z | extent.x | extent.y | extent.z   float[cap] each
//   transform index                                                  uint32[cap]
// cap is the object count rounded up to a whole tile (kTileObjects), so every 128-bit
// load of a tile stays inside the allocation.  World matrices are Mat44f rows
// (4 x float4, row-major, row-vector convention) gathered by transform index.
// A result (one group x one view) owns its visibility bit array (bit i of word i/32 is
// object i, the ResultBitSet layout, padded to whole tiles), its changed-object list and
// its scratch: the delta words (bit i set where object i changed; the cull writes every
// word) and one changed count per chunk of kDeltaChunk delta words (with a ticket and a
// block count).  One small kernel, a single pass, turns the delta words into the packed
// ascending list.  A tile is the 128 objects of one warp.
#pragma once

#include <cstddef>
#include <cstdint>

struct dpcull_ctx_s;

#if defined(__CUDACC__)
#define DPCULL_HD_CONST __host__ __device__ constexpr
#else
#define DPCULL_HD_CONST constexpr
#endif

namespace dpcull {

constexpr int kThreads = 256;                      // threads per CTA (8 independent warps)
constexpr int kWarpsPerCta = kThreads / 32;
constexpr int kObjPerThread = 4;                   // one float4 of each SoA row
constexpr int kTileObjects = 32 * kObjPerThread;   // 128 objects per tile (one warp)
constexpr int kTileWords = kTileObjects / 32;      // 4 bit-array words per tile and view
constexpr int kItemTiles = 8;                      // tiles per work item (one warp, one view group)
constexpr int kQueueCap = 1024;                    // undecided pairs a warp holds before a drain
constexpr uint32_t kDeltaChunk = 4096;             // delta words per changed-list chunk

// Work items of a scene: groups of item_tiles (1..kItemTiles) tiles x view groups.
DPCULL_HD_CONST uint32_t items_of(uint32_t n_tiles, uint32_t n_vgroups, uint32_t item_tiles)
{
  return (n_tiles + item_tiles - 1) / item_tiles * n_vgroups;
}

// With a tail: the scene's first n_big tile groups have item_tiles tiles (the last of them
// may be short), every tile after them is a group of its own.  Any n_big from 0 to
// ceil(n_tiles / item_tiles) covers every tile once; the launch hands the items out in
// order, so single-tile items at the end of a launch shorten the time the warps that
// finish first wait for the last ones.
DPCULL_HD_CONST uint32_t tile_groups_of(uint32_t n_tiles, uint32_t n_big, uint32_t item_tiles)
{
  return n_big + (n_tiles > n_big * item_tiles ? n_tiles - n_big * item_tiles : 0u);
}

// Tiles per work item for a launch of `tile_groups` (tiles x view groups) on `sm_count`
// SMs: long items amortise each warp's exact drain, short ones keep every warp busy when
// the launch is small.
inline uint32_t item_tiles_for(uint64_t tile_groups, int sm_count)
{
  const uint64_t warps = (uint64_t)(sm_count > 0 ? sm_count : 1) * 24;
  if (tile_groups >= warps * 16) return kItemTiles;
  if (tile_groups >= warps * 8) return 4;
  if (tile_groups >= warps * 4) return 2;
  return 1;
}
constexpr int kMaxViewsPerPass = 8;                // views evaluated per object load
constexpr uint32_t kMaxObjects = (1u << 30) - 1;   // keeps every index and count in 32 bits

// Chunk counts of a view with n_words visibility words.
DPCULL_HD_CONST size_t chunks_of(size_t n_words) { return (n_words + kDeltaChunk - 1) / kDeltaChunk; }

// Error bits reported through CullControl::error.
constexpr uint32_t kErrBadTransform = 1u;   // transform index >= matrix count
constexpr uint32_t kErrMisaligned = 2u;     // a wide launch met a matrix array not 32-byte aligned
constexpr uint32_t kErrWaitTimeout = 4u;    // a changed-list block gave up waiting for an earlier
                                            // count, or a tree block at a grid barrier

// Box cache of a group (the counterpart of the reference's OBB cache, GroupCPU::updateOBBs,
// dp/culling/cpu/src/ManagerImpl.cpp:114-162): per object the prefilter box of
// dpcull_prefilter.h -- centre x, y, z, radius, margin -- in 5 planar rows of `cap` floats,
// and the reference's cached OBB (point and three axes, computed in its operation order:
// one 64-byte record per object) for the exact test of the pairs the prefilter leaves
// undecided.  Its state word is Valid once a Fill launch has stored the boxes of the
// group's current objects and matrices; the host resets it to Stale (in stream order)
// whenever they change.  Three kernels (CacheMode): the fused one computes every box from
// the rows and the world matrices, the Fill one also stores them and validates the cache,
// the cached one reads them -- and should it meet a group whose cache is Stale, it sends
// all of that group's pairs to the exact test instead, so its results never depend on the
// host's choice of kernel.
constexpr uint32_t kBoxStale = 0u;
constexpr uint32_t kBoxValid = 1u;
// The cache's state block: the state word, then the scene bound that the Fill launch
// gathers with atomicMax (dpcull_prefilter.h bound_key): the largest centre x, y, z, the
// complements of the smallest, the largest margin d0.  All zero when the cache goes stale.
constexpr int kBoundWords = 7;
constexpr size_t kCacheStateBytes = 32;
static_assert((1 + kBoundWords) * 4 <= (int)kCacheStateBytes, "state word and bound fit the block");
constexpr int kBoxRows = 5;
constexpr int kObbFloats = 16;
enum CacheMode : uint32_t { kCacheNone = 0u, kCacheFill = 1u, kCacheRead = 2u };

struct CullScene {
  const float* soa;        // base of the group's SoA block
  const float* mats;       // [n_mats][16]
  float* box;              // prefilter-box cache [kBoxRows][cap], or nullptr (not cached)
  float* obb;              // OBB cache [cap][kObbFloats] (present with box)
  uint32_t* box_state;     // the caches' state word (kBoxStale / kBoxValid) and scene bound
  uint32_t cap;            // SoA row stride (objects)
  uint32_t n_objects;
  uint32_t n_mats;
  uint32_t view_begin;     // first CullView of this scene
  uint32_t n_views;
  uint32_t n_vgroups;      // ceil(n_views / views per pass)
  uint32_t n_tiles;
  uint32_t item_begin;     // first work item of this scene (scene_items)
  uint32_t n_big;          // tile groups of item_tiles tiles; the tiles after them are one per item
};

// Host: the item layout of a launch over `n` scenes with `item_tiles` tiles per item.
// The launch's last `tail` (tile x view group) units become single-tile items (walking
// from the last scene back); every other scene keeps items of item_tiles tiles.  Sets
// every scene's n_big and item_begin; returns the launch's item count.
inline uint32_t lay_out_items(CullScene* scenes, size_t n, uint32_t item_tiles, uint64_t tail)
{
  for (size_t k = n; k-- > 0;) {
    CullScene& s = scenes[k];
    const uint64_t per = s.n_vgroups ? s.n_vgroups : 1u;
    uint32_t singles = 0;
    if (item_tiles > 1 && tail) {
      const uint64_t want = (tail + per - 1) / per;
      singles = want < s.n_tiles ? (uint32_t)want : s.n_tiles;
      tail -= (uint64_t)singles * per < tail ? (uint64_t)singles * per : tail;
    }
    s.n_big = singles ? (s.n_tiles - singles) / item_tiles : (s.n_tiles + item_tiles - 1) / item_tiles;
  }
  uint32_t items = 0;
  for (size_t k = 0; k < n; ++k) {
    scenes[k].item_begin = items;
    items += tile_groups_of(scenes[k].n_tiles, scenes[k].n_big, item_tiles) * scenes[k].n_vgroups;
  }
  return items;
}

// Single-tile units at the end of a launch: about two per warp that can be resident.
inline uint64_t tail_units(int sm_count) { return (uint64_t)(sm_count > 0 ? sm_count : 1) * 64u; }

struct alignas(16) CullView {   // 144 bytes; staged whole into shared memory by the cull
  float vp[16];
  uint32_t* bits;        // previous visibility on entry, new visibility on exit
  uint32_t* changed;     // ascending changed-object list
  uint32_t* n_changed;   // its length
  uint32_t* delta;       // scratch: old XOR new visibility, n_words words
  uint32_t* chunk_tot;   // scratch, zero between launches: per chunk of kDeltaChunk delta
                        // words its changed objects + 1 once counted, then a ticket and a
                        // block count (chunks_of(n_words) + 2 words)
  uint32_t n_words;      // visibility words of the view (whole tiles)
  uint32_t flags;        // kViewNoChanged: write the visibility words only
  uint32_t* n_visible;   // optional: number of visible objects (accumulated)
  // Optional second copies of the results (a plan's asynchronous reads): every new word,
  // the changed list and its length, written beside bits / changed / n_changed.
  uint32_t* copy_bits;
  uint32_t* copy_changed;
  uint32_t* copy_count;
};
static_assert(sizeof(CullView) == 144, "CullView is 144 bytes");

// CullView::flags: no previous visibility and no changed list (bits are overwritten;
// changed / n_changed / delta / chunk_tot are not used).
constexpr uint32_t kViewNoChanged = 1u;

struct CullControl {
  unsigned int ticket;     // next work item
  unsigned int done;       // CTAs finished
  unsigned int error;      // sticky kErr* bits
  unsigned int error_info; // first offending index
  unsigned int bar_count;  // the tree kernel's grid barrier: blocks arrived,
  unsigned int bar_gen;    // and its generation
};

struct CullLaunch {
  const CullScene* scenes;   // device array, or nullptr to use `one_scene`
  const CullView* views;     // device array, or nullptr to use `one_view`
  uint32_t n_scenes;
  uint32_t n_items;
  uint32_t items_per_ticket; // items a warp claims per ticket (the "tiles per ticket" knob)
  uint32_t item_tiles;       // tiles per work item, 1..kItemTiles
  uint32_t exact_only;       // 1 = skip the conservative prefilter (every pair exact)
  uint32_t wide_mats;        // 1 = every scene's matrix array is 32-byte aligned (256-bit
                             // matrix loads); set by launch_cull itself for `one_scene`
  uint32_t cache_mode;       // CacheMode: the fused, Fill or cached kernel (the host's choice)
  uint32_t emit_views;       // > 0: every view's delta words fit one chunk, and the launch's
                             // last CTA builds the changed lists of these views itself
  CullControl* ctl;
  CullScene one_scene;
  CullView one_view;
};

// Launchers (cull.cu).  vpp = views per pass (1, 2, 4 or 8).
int launch_cull(const CullLaunch& args, int grid, int vpp, void* stream);
// CTAs of the cull kernel of this kind (CacheMode) that fit on one SM.
int cull_max_ctas_per_sm(int vpp, uint32_t mode);
// Changed-list assembly after a cull launch over `n_views` views (device array `views`,
// or the single `one` when views is null): one pass over the delta words that counts each
// chunk, sums the earlier chunks' counts and emits every changed index into the packed
// ascending list.  max_words bounds n_words; a block that gives up waiting for an earlier
// chunk's count sets kErrWaitTimeout in *err.
int launch_changed_lists(const CullView* views, const CullView& one, uint32_t n_views,
                         uint32_t max_words, unsigned int* err, void* stream,
                         const uint32_t* first_block = nullptr, uint32_t n_blocks = 0);
// Delta words per block of the changed-list pass.  With `first_block` (device, n_views + 1
// entries: view v's blocks are [first_block[v], first_block[v + 1]), at least one each)
// the pass runs n_blocks blocks in one dimension, so views with fewer chunks than the
// largest take no idle blocks; without it, max_words' chunks x n_views.
constexpr uint32_t kEmitChunkWords = 8192;
inline uint32_t emit_blocks_of(uint32_t n_words)
{
  const uint32_t c = (n_words + kEmitChunkWords - 1) / kEmitChunkWords;
  return c ? c : 1u;
}
// Launches of at most this many views whose delta words fit one chunk build their changed
// lists in the cull kernel's last CTA (CullLaunch::emit_views): no second kernel.
constexpr uint32_t kFusedEmitViews = 4;
inline uint32_t fused_emit_views(uint32_t n_views, uint32_t max_words)
{
  return (n_views <= kFusedEmitViews && max_words <= kDeltaChunk) ? n_views : 0u;
}

// Transform propagation (xform.cu).
struct XformLaunch {
  const uint2* entries;      // (parent, transform) in level order
  const uint32_t* seg;       // segment offsets into entries
  const float* local;        // [cap][16]
  float* world;              // [cap][16]
  uint32_t* dirty_local;
  uint32_t* dirty_world;
};
// Segments [s0, s1) inside one CTA (narrow levels), or entries [begin, end) of one wide
// segment over a grid.
int launch_xform_cta(const XformLaunch& a, uint32_t s0, uint32_t s1, void* stream);
int launch_xform_range(const XformLaunch& a, uint32_t begin, uint32_t end, void* stream);
// The whole propagation in one cooperative launch: clears the dirty-world bits, runs the
// schedule (x = 1: segments [y, z) of narrow levels in block 0, one __syncthreads each;
// x = 0: entries [y, z) of one wide segment over the grid) with a grid barrier after each
// step, then clears the dirty-local bits.  `words`: dirty bit words; `max_wide`: entries of
// the widest segment (sizes the grid).  A block that gives up waiting at a barrier sets
// kErrWaitTimeout in *err.  Returns -1 if the device cannot run the launch.
int launch_xform_tree(const XformLaunch& a, const uint4* sched, uint32_t n_sched, uint32_t words,
                      uint32_t max_wide, unsigned int* bar, unsigned int* err, int sm_count, void* stream);
int launch_scatter_matrices(float* dst, const float* src, const uint32_t* idx, uint32_t k,
                            uint32_t* dirty_bits, void* stream);
int launch_scatter_objects(float* soa, uint32_t cap, const float* src, const uint32_t* idx,
                           uint32_t k, void* stream);

// Sets the calling thread's dpcull_last_error() message; returns code (api.cu).
int record_error(int code, const char* msg);
// CUDA ordinal and SM count of a context (api.cu).
void ctx_info(::dpcull_ctx_s* ctx, int* device, int* sm_count);

// Bounding box (bbox.cu): partials has room for bbox_partials_needed() floats.
size_t bbox_partials_needed(uint32_t n_objects);
int launch_bbox(const float* soa, uint32_t cap, uint32_t n, const float* mats, float* partials,
                unsigned int* counter, float* out8, void* stream);

// n_words 32-bit words from src (device memory, or page-locked host memory, which the
// kernel reads directly) to dst (device memory).
int launch_copy_words(uint32_t* dst, const uint32_t* src, size_t n_words, void* stream);

// Result remap on object removal (api helpers in cull.cu).
int launch_move_bit(uint32_t* bits, uint32_t size_bits, uint32_t old_index, uint32_t new_index,
                    void* stream);
int launch_move_object(float* soa, uint32_t cap, uint32_t from, uint32_t to, void* stream);

// Snapshot of a result for an asynchronous read: its visibility words, its changed list
// (length read on the device) and that length.
struct ResultCopy {
  const uint32_t* bits;
  const uint32_t* changed;
  const uint32_t* n_changed;
  uint32_t* dst_bits;
  uint32_t* dst_changed;
  uint32_t* dst_count;
  uint32_t n_words;
  uint32_t pad;
};
// One launch over `n` results (device array `copies`).
int launch_snapshot(const ResultCopy* copies, uint32_t n, uint32_t max_len, void* stream);

}  // namespace dpcull
