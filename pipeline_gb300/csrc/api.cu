// api.cu -- the C ABI (include/dpcull.h) over the GB300 culling kernels.
//
// Host-side bookkeeping mirrors the reference's state classes:
//   * Group  ~ GroupBitSet (dp/culling/GroupBitSet.h:40-104): object count, incarnation
//     (bumped on every add / remove), matrices; objects and matrices live in HBM.
//   * Result ~ ResultBitSet (dp/culling/ResultBitSet.h:38-67): visibility bits sized
//     lazily at cull time when the group's incarnation changed, new bits visible.
//   * Tree   ~ dp::transform::Tree (dp/transform/Tree.h:42-129): the level lists are
//     kept as hazard-free segments, matrices and dirty bits live in HBM.
// Indices are validated on the host before any launch (a bad transform index is an
// error code, never a device fault); kernels check again and raise an error bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cerrno>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include <sys/stat.h>

#include "../../include/dpcull.h"
#include "dpcull_internal.h"

using namespace dpcull;

namespace {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...)
{
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* what)
{
  return fail(DPCULL_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CU(call)                                        \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

size_t round_up(size_t x, size_t m) { return (x + m - 1) / m * m; }
uint32_t tiles_of(size_t n) { return (uint32_t)((n + kTileObjects - 1) / kTileObjects); }

struct Group {
  bool alive = false;
  size_t n = 0, cap = 0;
  float* soa = nullptr;             // 7 rows x cap
  std::vector<uint32_t> xform;      // host mirror of transform indices (validation)
  uint32_t max_xform = 0;
  bool max_dirty = false;
  float* mats = nullptr;
  size_t n_mats = 0, mats_cap = 0;  // mats_cap = 0 for bound (not owned) matrices
  uint64_t incarnation = 0;
  std::vector<uint32_t> results;
  float* box_scratch = nullptr;     // partials + counter + output
  // Box cache (see CullScene::box): prefilter boxes (kBoxRows x cap floats) and OBBs
  // (cap x kObbFloats), allocated with the rows, and the state word.  A group whose matrices
  // are device memory the library neither owns nor sees change (cache_volatile) is never
  // cached; one bound to a tree of this context goes stale at every compute of that tree.
  float* cache = nullptr;
  float* obb = nullptr;
  uint32_t* cache_state = nullptr;
  bool cache_volatile = false;
  int tree = -1;
  // Host record of the cache, which picks the kernel: launches since it went stale, and
  // whether a Fill launch has stored it since.  The cached kernel is only launched when
  // `filled`; the kernels themselves read the device state word.
  uint32_t cache_launches = 0;
  bool cache_filled = false;
};

struct Result {
  bool alive = false;
  uint32_t group = 0;
  size_t size_bits = 0;             // ResultBitSet::m_results.getSize()
  uint64_t incarnation = ~0ull;     // ResultBitSet.cpp:43
  uint32_t* bits = nullptr;
  size_t words_cap = 0;
  uint32_t* changed = nullptr;
  size_t changed_cap = 0;
  uint32_t* n_changed = nullptr;
  uint32_t* delta = nullptr;        // words_cap: old XOR new visibility (changed-list scratch)
  uint32_t* chunk_tot = nullptr;    // chunks_of(words_cap): changed objects per chunk
  uint32_t n_words = 0;             // visibility words of the group at the last prepare
  uint32_t last_changed = 0;        // length of the changed list at the last read
};

struct TreeLaunch {
  bool single_cta;
  uint32_t a, b;  // segment range (single CTA) or entry range (grid)
};

struct Tree {
  bool alive = false;
  size_t cap = 0, words = 0;
  float* local = nullptr;
  float* world = nullptr;
  uint32_t* dirty_local = nullptr;
  uint32_t* dirty_world = nullptr;
  uint2* entries = nullptr;
  size_t entries_cap = 0;
  uint32_t* seg = nullptr;
  size_t seg_cap = 0;
  std::vector<TreeLaunch> schedule;
  // The schedule of the cooperative tree kernel (launch_xform_tree): narrow segments only
  // up to two entries per thread of block 0, anything wider over the grid.
  uint4* d_sched = nullptr;
  size_t sched_cap = 0;
  uint32_t n_sched = 0, max_wide = 0;
};

struct Plan {
  bool alive = false;
  std::vector<uint32_t> groups;
  std::vector<uint64_t> incarnations;
  std::vector<uint32_t> results;
  std::vector<CullScene> scenes;
  std::vector<CullView> views;
  CullScene* d_scenes = nullptr;
  CullView* d_views = nullptr;
  CullView* h_views[2] = {nullptr, nullptr};   // pinned, double buffered
  cudaGraphExec_t exec[3][2] = {};        // per kernel (CacheMode) and view slot, captured on first use
  cudaEvent_t done[2] = {nullptr, nullptr};
  cudaEvent_t kt[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // cull kernel begin / end
  bool pending[2] = {false, false};
  bool fresh[2] = {false, false};      // slot holds matrices from set_views
  std::vector<uint32_t> all_groups;    // every job's group (empty ones included)
  std::vector<uint32_t> all_results;   // every job's results, in job and view order
  uint32_t* h_counts = nullptr;        // pinned: changed counts of the snapshot (read_async),
                                       // then the device error word pair
  uint32_t* h_rcounts = nullptr;       // pinned: changed counts read by dpcull_plan_read, apart
                                       // from a pending snapshot's, which it must not overwrite
  // Asynchronous reads (dpcull_plan_snapshot / _read_async).  Once the first one is asked
  // for, every launch also writes its results into the copy buffer of its slot (the views'
  // copy pointers), and a read copies a launch's buffer to the host on copy_stream while
  // the next launch runs.  Slot layout: the results' changed counts (one word each), then
  // per result its words and its changed list (snap_bits / snap_changed offsets).
  bool copies = false;                 // the buffers exist and the views point at them
  uint32_t* cbuf[2] = {nullptr, nullptr};
  bool copied[2] = {false, false};     // the slot's buffer holds its last launch's results
  bool copying[2] = {false, false};    // the slot's views carry the copy pointers
  bool read_pending[2] = {false, false};  // copies out of the slot issued, not yet waited for
  int snap_slot = -1;                  // the slot the pending snapshot reads
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t snap_ev = nullptr, counts_ev = nullptr;
  cudaEvent_t copies_ev[2] = {nullptr, nullptr};
  bool snap_pending = false;           // snapshot taken (dpcull_plan_snapshot), not yet read
  ResultCopy* d_copies = nullptr;      // per slot, one per result: live results -> slot buffer
  size_t snap_words = 0;               // words per slot buffer
  uint32_t snap_max_len = 0;
  std::vector<size_t> snap_bits, snap_changed;  // offsets into a slot buffer
  std::vector<size_t> snap_sizes;      // each result's size at set-up
  std::vector<int> view_result;        // result index (in all_results) of each launched view
  std::vector<uint64_t> all_incarnations;
  int next = 0;
  dpcull_tuning tuning{};
  uint32_t n_items = 0;
  uint32_t item_tiles = kItemTiles;
  int grid = 0;
  uint32_t* d_emit_first = nullptr;    // the changed-list pass's first block of each view
  uint32_t emit_blocks = 0;            // (emit_blocks_of per view; n_views + 1 entries)
};

}  // namespace

struct dpcull_ctx_s {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  CullControl* ctl = nullptr;
  unsigned int* h_err = nullptr;     // pinned: ctl->error, error_info, one scratch word
  int sm_count = 0;
  uint64_t launches = 0;
  uint64_t mode_launches[3] = {0, 0, 0};  // cull kernels by CacheMode
  uint64_t device_bytes = 0;
  bool exact_only = false;            // prefilter disabled (testing / ablation)
  bool box_cache = true;              // groups keep their boxes between culls
  // Upload staging for scatter updates: pinned host and device buffers, grown on demand.
  unsigned char* stage_h = nullptr;
  unsigned char* stage_d = nullptr;
  size_t stage_cap = 0;
  cudaEvent_t stage_ev = nullptr;
  bool stage_pending = false;
  std::vector<Group> groups;
  std::vector<Result> results;
  std::vector<Tree> trees;
  std::vector<Plan> plans;
  std::map<std::string, dpcull_tuning> tune_cache;
};

namespace {

int dalloc(dpcull_ctx c, void** p, size_t bytes)
{
  *p = nullptr;
  if (!bytes) return DPCULL_OK;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(DPCULL_ERR_NO_MEMORY, "cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
  }
  c->device_bytes += bytes;
  return DPCULL_OK;
}

void dfree(dpcull_ctx c, void* p, size_t bytes)
{
  if (p) {
    cudaFree(p);
    c->device_bytes -= bytes;
  }
}

Group* get_group(dpcull_ctx c, dpcull_group g)
{
  if (!c || g >= c->groups.size() || !c->groups[g].alive) return nullptr;
  return &c->groups[g];
}

Result* get_result(dpcull_ctx c, dpcull_result r)
{
  if (!c || r >= c->results.size() || !c->results[r].alive) return nullptr;
  return &c->results[r];
}

Tree* get_tree(dpcull_ctx c, dpcull_tree t)
{
  if (!c || t >= c->trees.size() || !c->trees[t].alive) return nullptr;
  return &c->trees[t];
}

Plan* get_plan(dpcull_ctx c, dpcull_plan p)
{
  if (!c || p >= c->plans.size() || !c->plans[p].alive) return nullptr;
  return &c->plans[p];
}

size_t soa_bytes(size_t cap) { return 7 * cap * sizeof(float); }
size_t cache_bytes(size_t cap) { return (size_t)(kBoxRows + kObbFloats) * cap * sizeof(float); }

// The group's objects or matrices changed: its cached boxes are stale (in stream order, so
// launches already queued still read the old state).
int cache_stale(dpcull_ctx c, Group& g)
{
  g.cache_launches = 0;
  g.cache_filled = false;
  if (g.cache_state) CU(cudaMemsetAsync(g.cache_state, 0, kCacheStateBytes, c->stream));
  return DPCULL_OK;
}

// Grows the SoA block to hold n objects (copying the existing rows).
int group_reserve(dpcull_ctx c, Group& g, size_t n)
{
  if (n <= g.cap && g.soa) return DPCULL_OK;
  size_t cap = round_up(std::max<size_t>(n, 1), kTileObjects);
  if (g.cap) cap = std::max(cap, round_up(g.cap + g.cap / 2, kTileObjects));
  float* soa = nullptr;
  int rc = dalloc(c, (void**)&soa, soa_bytes(cap));
  if (rc) return rc;
  CU(cudaMemsetAsync(soa, 0, soa_bytes(cap), c->stream));
  float* cache = nullptr;
  rc = dalloc(c, (void**)&cache, cache_bytes(cap));
  if (rc) {
    dfree(c, soa, soa_bytes(cap));
    return rc;
  }
  if (g.soa && g.n)
    for (int r = 0; r < 7; ++r)
      CU(cudaMemcpyAsync(soa + (size_t)r * cap, g.soa + (size_t)r * g.cap, g.n * sizeof(float),
                         cudaMemcpyDeviceToDevice, c->stream));
  if (g.soa) {
    CU(cudaStreamSynchronize(c->stream));
    dfree(c, g.soa, soa_bytes(g.cap));
    dfree(c, g.cache, cache_bytes(g.cap));
  }
  g.soa = soa;
  g.cache = cache;
  g.obb = cache + (size_t)kBoxRows * cap;  // 64-byte aligned: cap is a multiple of 128
  g.cap = cap;
  return cache_stale(c, g);
}

// Uploads k planar objects into rows starting at object `at` (contiguous).
int upload_rows(dpcull_ctx c, Group& g, size_t at, size_t k, const float* lower,
                const float* extent, const uint32_t* xform)
{
  if (!k) return DPCULL_OK;
  for (int r = 0; r < 3; ++r) {
    CU(cudaMemcpyAsync(g.soa + (size_t)r * g.cap + at, lower + (size_t)r * k, k * sizeof(float),
                       cudaMemcpyHostToDevice, c->stream));
    CU(cudaMemcpyAsync(g.soa + (size_t)(3 + r) * g.cap + at, extent + (size_t)r * k,
                       k * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  }
  CU(cudaMemcpyAsync(g.soa + (size_t)6 * g.cap + at, xform, k * sizeof(uint32_t),
                     cudaMemcpyHostToDevice, c->stream));
  return DPCULL_OK;
}

uint32_t group_max_xform(Group& g)
{
  if (g.max_dirty) {
    uint32_t m = 0;
    for (size_t i = 0; i < g.n; ++i) m = std::max(m, g.xform[i]);
    g.max_xform = m;
    g.max_dirty = false;
  }
  return g.max_xform;
}

int check_cull_ready(Group& g)
{
  if (g.n > kMaxObjects) return fail(DPCULL_ERR_INVALID_ARGUMENT, "group has %zu objects (max %u)", g.n, kMaxObjects);
  if (g.n && !g.mats) return fail(DPCULL_ERR_STATE, "group has objects but no matrices");
  if (g.n && group_max_xform(g) >= g.n_mats)
    return fail(DPCULL_ERR_OUT_OF_RANGE, "transform index %u >= matrix count %zu", group_max_xform(g),
                g.n_mats);
  return DPCULL_OK;
}

__global__ void resize_bits_kernel(uint32_t* bits, size_t old_bits, size_t new_bits, size_t words)
{
  // ResultBitSet.cpp:65-79: keep [0, min(old,new)), set [old, new) visible, clear >= new.
  for (size_t w = blockIdx.x * (size_t)blockDim.x + threadIdx.x; w < words;
       w += (size_t)gridDim.x * blockDim.x) {
    uint32_t v = bits[w];
    for (int b = 0; b < 32; ++b) {
      const size_t i = w * 32 + b;
      if (i >= new_bits) v &= ~(1u << b);
      else if (i >= old_bits) v |= 1u << b;
    }
    bits[w] = v;
  }
}

// Capacity for a group of n objects, and the ResultBitSet resize on incarnation change.
int result_prepare(dpcull_ctx c, Result& r, Group& g)
{
  const uint32_t tiles = tiles_of(g.n);
  const size_t words = std::max<size_t>((size_t)tiles * kTileWords, 32);
  if (words > r.words_cap) {
    uint32_t* nb = nullptr;
    int rc = dalloc(c, (void**)&nb, words * 4);
    if (rc) return rc;
    CU(cudaMemsetAsync(nb, 0, words * 4, c->stream));
    if (r.bits) {
      CU(cudaMemcpyAsync(nb, r.bits, r.words_cap * 4, cudaMemcpyDeviceToDevice, c->stream));
      CU(cudaStreamSynchronize(c->stream));
      dfree(c, r.bits, r.words_cap * 4);
    }
    r.bits = nb;
    CU(cudaStreamSynchronize(c->stream));
    dfree(c, r.delta, r.words_cap * 4);
    dfree(c, r.chunk_tot, (chunks_of(r.words_cap) + 2) * 4);
    r.delta = r.chunk_tot = nullptr;
    r.words_cap = words;
    rc = dalloc(c, (void**)&r.delta, words * 4);
    // the chunk counts, ticket and block count of the changed-list pass: zero between launches
    if (!rc) rc = dalloc(c, (void**)&r.chunk_tot, (chunks_of(words) + 2) * 4);
    if (rc) return rc;
    CU(cudaMemsetAsync(r.chunk_tot, 0, (chunks_of(words) + 2) * 4, c->stream));
  }
  const size_t chcap = std::max<size_t>(g.n, 1);
  if (chcap > r.changed_cap) {
    CU(cudaStreamSynchronize(c->stream));
    dfree(c, r.changed, r.changed_cap * 4);
    r.changed = nullptr;
    size_t want = std::max(chcap, r.changed_cap + r.changed_cap / 2);
    int rc = dalloc(c, (void**)&r.changed, want * 4);
    if (rc) return rc;
    r.changed_cap = want;
  }
  r.n_words = tiles * kTileWords;
  if (r.incarnation != g.incarnation) {
    r.incarnation = g.incarnation;
    const size_t old = r.size_bits;
    r.size_bits = g.n;
    resize_bits_kernel<<<(unsigned)std::min<size_t>((r.words_cap + 255) / 256, 4096), 256, 0,
                         c->stream>>>(r.bits, old, g.n, r.words_cap);
    CU(cudaGetLastError());
    c->launches++;
  }
  return DPCULL_OK;
}

CullScene scene_of(Group& g, uint32_t view_begin, uint32_t n_views, uint32_t vpp,
                   uint32_t item_begin)
{
  CullScene s{};
  s.soa = g.soa;
  s.mats = g.mats;
  s.box = g.cache_volatile ? nullptr : g.cache;  // the launch builder may still drop it
  s.obb = g.obb;
  s.box_state = g.cache_state;
  s.cap = (uint32_t)g.cap;
  s.n_objects = (uint32_t)g.n;
  s.n_mats = (uint32_t)std::min<size_t>(g.n_mats, 0xFFFFFFFFu);
  s.view_begin = view_begin;
  s.n_views = n_views;
  s.n_vgroups = (n_views + vpp - 1) / vpp;
  s.n_tiles = tiles_of(g.n);
  s.item_begin = item_begin;
  return s;
}

CullView view_of(Result& r, const float* vp)
{
  CullView v{};
  memcpy(v.vp, vp, sizeof v.vp);
  v.bits = r.bits;
  v.changed = r.changed;
  v.n_changed = r.n_changed;
  v.delta = r.delta;
  v.chunk_tot = r.chunk_tot;
  v.n_words = r.n_words;
  return v;
}

// Copies n host ranges into the context's pinned staging buffer (after the previous
// staged copy has left it) and sends them to the device staging buffer in one
// asynchronous copy; dev[i] receives the device address of part i.  The caller's host
// memory may be reused as soon as this returns.
int stage_upload(dpcull_ctx c, int n, const void* const* src, const size_t* bytes, unsigned char** dev)
{
  size_t off[8], total = 0;
  for (int i = 0; i < n; ++i) {
    off[i] = total;
    total += (bytes[i] + 255) & ~size_t(255);
  }
  if (total > c->stage_cap) {
    CU(cudaStreamSynchronize(c->stream));
    if (c->stage_h) cudaFreeHost(c->stage_h);
    if (c->stage_d) dfree(c, c->stage_d, c->stage_cap);
    c->stage_h = c->stage_d = nullptr;
    const size_t cap = std::max(total, 2 * c->stage_cap);
    c->stage_cap = 0;
    if (cudaMallocHost((void**)&c->stage_h, cap) != cudaSuccess) {
      cudaGetLastError();
      return fail(DPCULL_ERR_NO_MEMORY, "pinned staging allocation failed");
    }
    int rc = dalloc(c, (void**)&c->stage_d, cap);
    if (rc) return rc;
    c->stage_cap = cap;
    c->stage_pending = false;
  }
  if (!c->stage_ev) CU(cudaEventCreateWithFlags(&c->stage_ev, cudaEventDisableTiming));
  // Sources in page-locked memory go to the device directly (one DMA each, no host copy);
  // the call returns once they have landed (after the context's earlier work), so the
  // caller may reuse its buffers at once, as with the staged path.
  bool pinned = true;
  for (int i = 0; i < n && pinned; ++i) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, src[i]) != cudaSuccess || at.type != cudaMemoryTypeHost) {
      cudaGetLastError();
      pinned = false;
    }
  }
  if (pinned) {
    for (int i = 0; i < n; ++i) {
      dev[i] = c->stage_d + off[i];
      CU(cudaMemcpyAsync(dev[i], src[i], bytes[i], cudaMemcpyHostToDevice, c->stream));
    }
    CU(cudaEventRecord(c->stage_ev, c->stream));
    CU(cudaEventSynchronize(c->stage_ev));
    c->stage_pending = false;
    return DPCULL_OK;
  }
  if (c->stage_pending) CU(cudaEventSynchronize(c->stage_ev));
  for (int i = 0; i < n; ++i) {
    memcpy(c->stage_h + off[i], src[i], bytes[i]);
    dev[i] = c->stage_d + off[i];
  }
  CU(cudaMemcpyAsync(c->stage_d, c->stage_h, total, cudaMemcpyHostToDevice, c->stream));
  CU(cudaEventRecord(c->stage_ev, c->stream));
  c->stage_pending = true;
  return DPCULL_OK;
}

// Queues the copy of the device error word pair to c->h_err[0..1]; device_errors_read
// reports it after the next synchronisation of the stream, so a read of results and its
// error check share one round trip.
cudaError_t enqueue_error_read(dpcull_ctx c)
{
  return cudaMemcpyAsync(c->h_err, &c->ctl->error, 2 * sizeof(unsigned int), cudaMemcpyDeviceToHost,
                         c->stream);
}

int device_errors_read(dpcull_ctx c)
{
  const unsigned int err = c->h_err[0], info = c->h_err[1];
  if (err) {
    CU(cudaMemsetAsync(&c->ctl->error, 0, 2 * sizeof(unsigned int), c->stream));
    CU(cudaStreamSynchronize(c->stream));
    if (err & kErrBadTransform)
      return fail(DPCULL_ERR_OUT_OF_RANGE, "object %u has a transform index past the matrix array", info);
    if (err & kErrMisaligned)
      return fail(DPCULL_ERR_STATE, "work item %u: a matrix array moved off its 32-byte alignment", info);
    if (err & kErrWaitTimeout)
      return fail(DPCULL_ERR_CUDA,
                  "a bounded device wait gave up (a changed-list chunk count or a tree grid barrier): "
                  "results incomplete");
  }
  return DPCULL_OK;
}

int check_device_errors(dpcull_ctx c)
{
  CU(enqueue_error_read(c));
  CU(cudaStreamSynchronize(c->stream));
  return device_errors_read(c);
}

int default_vpp(uint32_t max_views)
{
  return max_views <= 1 ? 1 : max_views <= 2 ? 2 : max_views <= 4 ? 4 : 8;
}

// Builds scenes/views for a job list; returns n_items.
int build_batch(dpcull_ctx c, const dpcull_job* jobs, size_t n_jobs, uint32_t vpp,
                std::vector<CullScene>& scenes, std::vector<CullView>& views, uint32_t* n_items,
                std::vector<uint32_t>* groups_out, std::vector<uint32_t>* results_out,
                uint32_t* item_tiles_out)
{
  scenes.clear();
  views.clear();
  uint32_t items = 0;
  for (size_t j = 0; j < n_jobs; ++j) {
    Group* g = get_group(c, jobs[j].group);
    if (!g) return fail(DPCULL_ERR_INVALID_ARGUMENT, "job %zu: bad group", j);
    if (!jobs[j].n_views || !jobs[j].results || !jobs[j].vps)
      return fail(DPCULL_ERR_INVALID_ARGUMENT, "job %zu: needs views, results and matrices", j);
    int rc = check_cull_ready(*g);
    if (rc) return rc;
    if (g->n == 0) {
      for (uint32_t v = 0; v < jobs[j].n_views; ++v) {
        Result* r = get_result(c, jobs[j].results[v]);
        if (!r || r->group != jobs[j].group) return fail(DPCULL_ERR_INVALID_ARGUMENT, "job %zu: bad result", j);
        rc = result_prepare(c, *r, *g);
        if (rc) return rc;
        CU(cudaMemsetAsync(r->n_changed, 0, 4, c->stream));
      }
      continue;
    }
    const uint32_t vb = (uint32_t)views.size();
    for (uint32_t v = 0; v < jobs[j].n_views; ++v) {
      Result* r = get_result(c, jobs[j].results[v]);
      if (!r || r->group != jobs[j].group) return fail(DPCULL_ERR_INVALID_ARGUMENT, "job %zu: bad result", j);
      rc = result_prepare(c, *r, *g);
      if (rc) return rc;
      views.push_back(view_of(*r, jobs[j].vps + 16 * (size_t)v));
      if (results_out) results_out->push_back(jobs[j].results[v]);
    }
    CullScene s = scene_of(*g, vb, jobs[j].n_views, vpp, 0);
    scenes.push_back(s);
    if (groups_out) groups_out->push_back(jobs[j].group);
  }
  // A cache is stored by one scene of a launch, so a group in several jobs of one launch
  // is culled without it (as is every group with the cache switched off or the prefilter
  // disabled).
  std::map<const uint32_t*, int> uses;
  for (const CullScene& sc : scenes) uses[sc.box_state]++;
  for (CullScene& sc : scenes)
    if (uses[sc.box_state] > 1 || c->exact_only || !c->box_cache) sc.box = nullptr;
  uint64_t tile_groups = 0;
  for (auto& s : scenes) tile_groups += (uint64_t)s.n_tiles * s.n_vgroups;
  const uint32_t it = item_tiles_for(tile_groups, c->sm_count);
  items = lay_out_items(scenes.data(), scenes.size(), it, tail_units(c->sm_count));
  *n_items = items;
  if (item_tiles_out) *item_tiles_out = it;
  return DPCULL_OK;
}

int persistent_grid(dpcull_ctx c, uint32_t vpp, uint32_t ctas_per_sm, uint32_t n_items,
                    uint32_t per_ticket, CacheMode mode)
{
  int occ = cull_max_ctas_per_sm((int)vpp, mode);
  int per_sm = ctas_per_sm ? std::min<int>((int)ctas_per_sm, occ) : occ;
  const long long per_cta = (long long)per_ticket * kWarpsPerCta;  // each warp claims its own
  long long want = ((long long)n_items + per_cta - 1) / per_cta;
  long long grid = std::min<long long>((long long)c->sm_count * per_sm, want);
  return (int)std::max<long long>(grid, 1);
}

uint32_t max_words_of(const std::vector<CullScene>& scenes);

// The kernel for a launch over these scenes (groups[i] is scene i's group): the cached one
// when every scene's cache has been stored since it last went stale, the Fill one when
// every scene has been culled since (so a group whose objects or matrices change every
// frame is never stored), the fused one otherwise -- and whenever some scene has no cache
// or the context has the cache switched off (a plan keeps the box pointers it was
// created with, so the switch is read here, at every launch).
CacheMode batch_mode(dpcull_ctx c, const std::vector<uint32_t>& groups, const std::vector<CullScene>& scenes)
{
  if (scenes.empty() || !c->box_cache || c->exact_only) return kCacheNone;
  bool all_filled = true, all_culled = true;
  for (size_t i = 0; i < scenes.size(); ++i) {
    if (!scenes[i].box) return kCacheNone;
    const Group& g = c->groups[groups[i]];
    all_filled &= g.cache_filled;
    all_culled &= g.cache_launches > 0;
  }
  return all_filled ? kCacheRead : all_culled ? kCacheFill : kCacheNone;
}

// Records a launch in the host record of every cached group it culled (count: also in
// the context's launch counts by kind).
void note_launch(dpcull_ctx c, const std::vector<uint32_t>& groups, const std::vector<CullScene>& scenes,
                 CacheMode mode, bool count = true)
{
  if (count) c->mode_launches[mode]++;
  for (size_t i = 0; i < scenes.size(); ++i)
    if (scenes[i].box) {
      Group& g = c->groups[groups[i]];
      g.cache_launches++;
      if (mode == kCacheFill) g.cache_filled = true;
    }
}

// The cull over all scenes and views, then the changed-list assembly of every view.
// d_scenes is the device copy of `scenes`.  k0 / k1 (optional, timing events, stream
// capture only) are recorded right before and after the cull kernel on the capture's side
// stream `side`: their event-record nodes hang off the graph beside the kernels instead of
// sitting between them (between them they cost ~4.6 us per step and break the changed-list
// pass's programmatic launch).  The caller joins `side` back before ending the capture.
int launch_batch(dpcull_ctx c, const CullScene* d_scenes, const CullView* d_views,
                 const std::vector<CullScene>& scenes, uint32_t n_views, uint32_t n_items,
                 uint32_t item_tiles, const dpcull_tuning& t, cudaStream_t s,
                 cudaEvent_t k0 = nullptr, cudaEvent_t k1 = nullptr, CacheMode mode = kCacheNone,
                 cudaStream_t side = nullptr, cudaEvent_t fork = nullptr, const uint32_t* emit_first = nullptr,
                 uint32_t emit_blocks = 0)
{
  if (n_views > 65535) return fail(DPCULL_ERR_INVALID_ARGUMENT, "at most 65535 views per launch");
  const uint32_t max_words = max_words_of(scenes);
  CullLaunch a{};
  a.scenes = d_scenes;
  a.views = d_views;
  a.n_scenes = (uint32_t)scenes.size();
  a.wide_mats = 1;  // 256-bit matrix loads only if every scene's array allows them
  for (const CullScene& sc : scenes)
    if ((uintptr_t)sc.mats & 31u) a.wide_mats = 0;
  a.n_items = n_items;
  a.item_tiles = item_tiles;
  a.items_per_ticket = std::max<uint32_t>(1, t.tiles_per_ticket);
  a.exact_only = c->exact_only ? 1u : 0u;
  a.cache_mode = mode;
  a.emit_views = fused_emit_views(n_views, max_words);
  a.ctl = c->ctl;
  const int grid = persistent_grid(c, t.views_per_pass, t.ctas_per_sm, n_items, a.items_per_ticket, mode);
  if (k0) {  // after everything the cull waits for
    CU(cudaEventRecord(fork, s));
    CU(cudaStreamWaitEvent(side, fork, 0));
    CU(cudaEventRecordWithFlags(k0, side, cudaEventRecordExternal));
  }
  if (launch_cull(a, grid, (int)t.views_per_pass, s)) return cuda_fail(cudaGetLastError(), "cull launch");
  if (k1) {  // after the cull
    CU(cudaEventRecord(fork, s));
    CU(cudaStreamWaitEvent(side, fork, 0));
    CU(cudaEventRecordWithFlags(k1, side, cudaEventRecordExternal));
  }
  CullView none{};
  if (!a.emit_views && launch_changed_lists(d_views, none, n_views, max_words, &c->ctl->error, s, emit_first,
                                            emit_blocks))
    return cuda_fail(cudaGetLastError(), "changed-list launch");
  c->launches += a.emit_views ? 1 : 2;
  return DPCULL_OK;
}

uint32_t max_words_of(const std::vector<CullScene>& scenes)
{
  uint32_t m = 1;
  for (auto& s : scenes) m = std::max(m, s.n_tiles * (uint32_t)kTileWords);
  return m;
}

bool valid_vpp(uint32_t v) { return v == 1 || v == 2 || v == 4 || v == 8; }

std::string tune_key(const std::vector<CullScene>& scenes, const std::vector<CullView>& views)
{
  uint64_t objs = 0;
  uint32_t maxv = 0;
  bool cached = !scenes.empty();
  for (auto& s : scenes) {
    objs += s.n_objects;
    maxv = std::max(maxv, s.n_views);
    cached = cached && s.box;
  }
  const int bucket = objs ? (int)std::floor(std::log2((double)objs)) : 0;
  char buf[112];
  // "w1024": tunings of the kernel whose warp items are up to 1024 objects; "bc": of the kernel
  // that reads the box caches (the steady state of a plan whose scenes all keep one)
  snprintf(buf, sizeof buf, "w%d_n2^%d_v%zu_maxv%u_s%zu%s", kItemTiles * kTileObjects, bucket, views.size(), maxv,
           scenes.size(),
           cached ? "_bc" : "");
  return buf;
}

std::string tune_cache_path()
{
  const char* p = getenv("DPCULL_TUNE_CACHE");
  if (p && *p) return p;
  const char* home = getenv("HOME");
  return std::string(home && *home ? home : "/tmp") + "/.cache/dpcull_tune.json";
}

void tune_cache_load(dpcull_ctx c)
{
  FILE* f = fopen(tune_cache_path().c_str(), "r");
  if (!f) return;
  char line[512];
  while (fgets(line, sizeof line, f)) {
    char key[128];
    unsigned a, b, d;
    // one JSON object per line: {"key": "...", "views_per_pass": a, "tiles_per_ticket": b, "ctas_per_sm": d}
    if (sscanf(line, " {\"key\": \"%127[^\"]\", \"views_per_pass\": %u, \"tiles_per_ticket\": %u, \"ctas_per_sm\": %u",
               key, &a, &b, &d) == 4 && valid_vpp(a))
      c->tune_cache[key] = dpcull_tuning{a, b, d, 0};
  }
  fclose(f);
}

void tune_cache_store(const std::string& key, const dpcull_tuning& t)
{
  std::string path = tune_cache_path();
  const size_t slash = path.find_last_of('/');
  if (slash != std::string::npos && slash > 0) mkdir(path.substr(0, slash).c_str(), 0755);
  FILE* f = fopen(path.c_str(), "a");
  if (!f) return;
  fprintf(f, "{\"key\": \"%s\", \"views_per_pass\": %u, \"tiles_per_ticket\": %u, \"ctas_per_sm\": %u}\n",
          key.c_str(), t.views_per_pass, t.tiles_per_ticket, t.ctas_per_sm);
  fclose(f);
}

}  // namespace

int dpcull::record_error(int code, const char* msg) { return fail(code, "%s", msg); }

void dpcull::ctx_info(dpcull_ctx_s* c, int* device, int* sm_count)
{
  *device = c->device;
  *sm_count = c->sm_count;
}

// ===================================================================================
extern "C" {

const char* dpcull_last_error(void) { return g_last_error.c_str(); }
uint32_t dpcull_version(void) { return (1u << 16) | 0u; }

int dpcull_ctx_create(int device, void* stream, dpcull_ctx* out)
{
  if (!out) return fail(DPCULL_ERR_INVALID_ARGUMENT, "out is null");
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    return fail(DPCULL_ERR_CUDA, "no CUDA device available (%s)", cudaGetErrorString(e));
  }
  if (device < 0 || device >= n) return fail(DPCULL_ERR_INVALID_ARGUMENT, "device %d of %d", device, n);
  CU(cudaSetDevice(device));
  dpcull_ctx c = new dpcull_ctx_s();
  c->device = device;
  if (stream) {
    c->stream = static_cast<cudaStream_t>(stream);
  } else {
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      delete c;
      return cuda_fail(e, "cudaStreamCreate");
    }
    c->own_stream = true;
  }
  cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
  int rc = dalloc(c, (void**)&c->ctl, sizeof(CullControl));
  if (rc) {
    delete c;
    return rc;
  }
  CullControl init{};
  e = cudaMemcpy(c->ctl, &init, sizeof init, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMallocHost((void**)&c->h_err, 4 * sizeof(unsigned int));
  if (e != cudaSuccess) {
    dpcull_ctx_destroy(c);
    return cuda_fail(e, "context set-up");
  }
  tune_cache_load(c);
  *out = c;
  return DPCULL_OK;
}

int dpcull_ctx_destroy(dpcull_ctx c)
{
  if (!c) return fail(DPCULL_ERR_INVALID_ARGUMENT, "null context");
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (dpcull_plan p = 0; p < c->plans.size(); ++p)
    if (c->plans[p].alive) dpcull_plan_destroy(c, p);
  for (dpcull_tree t = 0; t < c->trees.size(); ++t)
    if (c->trees[t].alive) dpcull_tree_destroy(c, t);
  for (dpcull_result r = 0; r < c->results.size(); ++r)
    if (c->results[r].alive) dpcull_result_destroy(c, r);
  for (dpcull_group g = 0; g < c->groups.size(); ++g)
    if (c->groups[g].alive) dpcull_group_destroy(c, g);
  if (c->ctl) cudaFree(c->ctl);
  if (c->h_err) cudaFreeHost(c->h_err);
  if (c->stage_h) cudaFreeHost(c->stage_h);
  if (c->stage_d) cudaFree(c->stage_d);
  if (c->stage_ev) cudaEventDestroy(c->stage_ev);
  if (c->own_stream) cudaStreamDestroy(c->stream);
  delete c;
  return DPCULL_OK;
}

int dpcull_ctx_synchronize(dpcull_ctx c)
{
  if (!c) return fail(DPCULL_ERR_INVALID_ARGUMENT, "null context");
  CU(cudaStreamSynchronize(c->stream));
  return check_device_errors(c);
}

void* dpcull_ctx_stream(dpcull_ctx c) { return c ? (void*)c->stream : nullptr; }
uint64_t dpcull_ctx_kernel_launches(dpcull_ctx c) { return c ? c->launches : 0; }
uint64_t dpcull_ctx_device_bytes(dpcull_ctx c) { return c ? c->device_bytes : 0; }

int dpcull_ctx_cull_launches(dpcull_ctx c, uint64_t out[3])
{
  if (!c || !out) return fail(DPCULL_ERR_INVALID_ARGUMENT, "null context or output");
  for (int k = 0; k < 3; ++k) out[k] = c->mode_launches[k];
  return DPCULL_OK;
}

int dpcull_ctx_set_prefilter(dpcull_ctx c, int enabled)
{
  if (!c) return fail(DPCULL_ERR_INVALID_ARGUMENT, "null context");
  c->exact_only = !enabled;
  return DPCULL_OK;
}

int dpcull_ctx_set_box_cache(dpcull_ctx c, int enabled)
{
  if (!c) return fail(DPCULL_ERR_INVALID_ARGUMENT, "null context");
  c->box_cache = enabled != 0;
  return DPCULL_OK;
}

// ---- groups ------------------------------------------------------------------------
int dpcull_group_create(dpcull_ctx c, dpcull_group* out)
{
  if (!c || !out) return fail(DPCULL_ERR_INVALID_ARGUMENT, "null argument");
  c->groups.emplace_back();
  Group& g = c->groups.back();
  g.alive = true;
  int rc = dalloc(c, (void**)&g.box_scratch, (bbox_partials_needed(0) + 16) * sizeof(float));
  if (rc) {
    g.alive = false;
    return rc;
  }
  CU(cudaMemsetAsync(g.box_scratch, 0, (bbox_partials_needed(0) + 16) * sizeof(float), c->stream));
  rc = dalloc(c, (void**)&g.cache_state, kCacheStateBytes);
  if (rc) {
    dfree(c, g.box_scratch, (bbox_partials_needed(0) + 16) * sizeof(float));
    g = Group();
    return rc;
  }
  CU(cudaMemsetAsync(g.cache_state, 0, kCacheStateBytes, c->stream));
  *out = (dpcull_group)(c->groups.size() - 1);
  return DPCULL_OK;
}

int dpcull_group_destroy(dpcull_ctx c, dpcull_group gh)
{
  Group* g = get_group(c, gh);
  if (!g) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad group %u", gh);
  cudaStreamSynchronize(c->stream);
  for (uint32_t r : g->results)
    if (get_result(c, r)) dpcull_result_destroy(c, r);
  dfree(c, g->soa, soa_bytes(g->cap));
  dfree(c, g->cache, cache_bytes(g->cap));
  dfree(c, g->cache_state, kCacheStateBytes);
  if (g->mats_cap) dfree(c, g->mats, g->mats_cap * 64);
  dfree(c, g->box_scratch, (bbox_partials_needed(0) + 16) * sizeof(float));
  *g = Group();
  return DPCULL_OK;
}

int dpcull_group_set_objects(dpcull_ctx c, dpcull_group gh, size_t n, const float* lower,
                             const float* extent, const uint32_t* xform)
{
  Group* g = get_group(c, gh);
  if (!g) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad group %u", gh);
  if (n && (!lower || !extent || !xform)) return fail(DPCULL_ERR_INVALID_ARGUMENT, "null object arrays");
  if (n > kMaxObjects) return fail(DPCULL_ERR_INVALID_ARGUMENT, "%zu objects (max %u)", n, kMaxObjects);
  int rc = group_reserve(c, *g, n);
  if (rc) return rc;
  // Rows past the new count must read as zero (padding of the last tile).
  if (n < g->n)
    for (int r = 0; r < 7; ++r)
      CU(cudaMemsetAsync(g->soa + (size_t)r * g->cap + n, 0, (g->n - n) * sizeof(float), c->stream));
  rc = upload_rows(c, *g, 0, n, lower, extent, xform);
  if (rc) return rc;
  g->xform.assign(xform, xform + n);
  g->max_dirty = true;
  g->n = n;
  g->incarnation += n ? n : 1;  // clearObjects + addObject x n
  rc = cache_stale(c, *g);
  if (rc) return rc;
  CU(cudaStreamSynchronize(c->stream));
  return DPCULL_OK;
}

int dpcull_group_append_objects(dpcull_ctx c, dpcull_group gh, size_t k, const float* lower,
                                const float* extent, const uint32_t* xform)
{
  Group* g = get_group(c, gh);
  if (!g) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad group %u", gh);
  if (!k) return DPCULL_OK;
  if (!lower || !extent || !xform) return fail(DPCULL_ERR_INVALID_ARGUMENT, "null object arrays");
  if (g->n + k > kMaxObjects) return fail(DPCULL_ERR_INVALID_ARGUMENT, "too many objects");
  int rc = group_reserve(c, *g, g->n + k);
  if (rc) return rc;
  rc = upload_rows(c, *g, g->n, k, lower, extent, xform);
  if (rc) return rc;
  g->xform.insert(g->xform.end(), xform, xform + k);
  for (size_t i = 0; i < k; ++i) g->max_xform = std::max(g->max_xform, xform[i]);
  g->n += k;
  g->incarnation += k;
  rc = cache_stale(c, *g);
  if (rc) return rc;
  CU(cudaStreamSynchronize(c->stream));
  return DPCULL_OK;
}

int dpcull_group_update_objects(dpcull_ctx c, dpcull_group gh, size_t k, const uint32_t* index,
                                const float* lower, const float* extent, const uint32_t* xform)
{
  Group* g = get_group(c, gh);
  if (!g) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad group %u", gh);
  if (!k) return DPCULL_OK;
  if (!index || !lower || !extent || !xform) return fail(DPCULL_ERR_INVALID_ARGUMENT, "null arrays");
  for (size_t i = 0; i < k; ++i)
    if (index[i] >= g->n) return fail(DPCULL_ERR_OUT_OF_RANGE, "object index %u >= %zu", index[i], g->n);
  std::vector<float> rows(7 * k);
  for (int r = 0; r < 3; ++r) {
    memcpy(&rows[r * k], lower + r * k, k * 4);
    memcpy(&rows[(3 + r) * k], extent + r * k, k * 4);
  }
  memcpy(&rows[6 * k], xform, k * 4);
  const void* src[2] = {rows.data(), index};
  const size_t bytes[2] = {rows.size() * 4, k * 4};
  unsigned char* dev[2];
  int rc = stage_upload(c, 2, src, bytes, dev);
  if (rc) return rc;
  if (launch_scatter_objects(g->soa, (uint32_t)g->cap, reinterpret_cast<float*>(dev[0]),
                             reinterpret_cast<uint32_t*>(dev[1]), (uint32_t)k, c->stream))
    return cuda_fail(cudaGetLastError(), "update objects");
  c->launches++;
  for (size_t i = 0; i < k; ++i) g->xform[index[i]] = xform[i];
  g->max_dirty = true;
  return cache_stale(c, *g);
}

int dpcull_group_remove_object(dpcull_ctx c, dpcull_group gh, size_t index)
{
  Group* g = get_group(c, gh);
  if (!g) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad group %u", gh);
  if (index >= g->n) return fail(DPCULL_ERR_STATE, "object does not belong to this group");
  const size_t last = g->n - 1;
  if (index != last) {
    if (launch_move_object(g->soa, (uint32_t)g->cap, (uint32_t)last, (uint32_t)index, c->stream))
      return cuda_fail(cudaGetLastError(), "move object");
    c->launches++;
    g->xform[index] = g->xform[last];
  }
  for (int r = 0; r < 7; ++r)
    CU(cudaMemsetAsync(g->soa + (size_t)r * g->cap + last, 0, sizeof(float), c->stream));
  g->xform.pop_back();
  g->max_dirty = true;
  g->n = last;
  // Event(old = new size, new = hole) to every result (GroupBitSet.cpp:108).
  for (uint32_t rh : g->results) {
    Result* r = get_result(c, rh);
    if (!r || !r->bits) continue;
    if (launch_move_bit(r->bits, (uint32_t)r->size_bits, (uint32_t)g->n, (uint32_t)index, c->stream))
      return cuda_fail(cudaGetLastError(), "move bit");
    c->launches++;
  }
  g->incarnation++;
  return cache_stale(c, *g);
}

int dpcull_group_count(dpcull_ctx c, dpcull_group gh, size_t* n)
{
  Group* g = get_group(c, gh);
  if (!g || !n) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad group %u", gh);
  *n = g->n;
  return DPCULL_OK;
}

static int ensure_owned_mats(dpcull_ctx c, Group& g, size_t count)
{
  if (g.mats_cap >= count && g.mats_cap) return DPCULL_OK;
  CU(cudaStreamSynchronize(c->stream));
  if (g.mats_cap) dfree(c, g.mats, g.mats_cap * 64);
  g.mats = nullptr;
  g.mats_cap = 0;
  const size_t cap = std::max<size_t>(count, 1);
  int rc = dalloc(c, (void**)&g.mats, cap * 64);
  if (rc) return rc;
  g.mats_cap = cap;
  return DPCULL_OK;
}

int dpcull_group_set_matrices(dpcull_ctx c, dpcull_group gh, const void* matrices, size_t count,
                              size_t stride)
{
  Group* g = get_group(c, gh);
  if (!g) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad group %u", gh);
  if (count && (!matrices || stride < 64)) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad matrix array");
  if (count > 0xFFFFFFFFull) return fail(DPCULL_ERR_INVALID_ARGUMENT, "too many matrices");
  int rc = ensure_owned_mats(c, *g, count);
  if (rc) return rc;
  if (count) {
    if (stride == 64) {
      CU(cudaMemcpyAsync(g->mats, matrices, count * 64, cudaMemcpyHostToDevice, c->stream));
    } else {
      CU(cudaMemcpy2DAsync(g->mats, 64, matrices, stride, 64, count, cudaMemcpyHostToDevice, c->stream));
    }
  }
  g->n_mats = count;
  g->cache_volatile = false;
  g->tree = -1;
  rc = cache_stale(c, *g);
  if (rc) return rc;
  CU(cudaStreamSynchronize(c->stream));
  return DPCULL_OK;
}

int dpcull_group_update_matrices(dpcull_ctx c, dpcull_group gh, size_t k, const uint32_t* index,
                                 const void* matrices, size_t stride)
{
  Group* g = get_group(c, gh);
  if (!g) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad group %u", gh);
  if (!k) return DPCULL_OK;
  if (!index || !matrices || stride < 64) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad arguments");
  if (!g->mats_cap) return fail(DPCULL_ERR_STATE, "group matrices are bound, not owned");
  std::vector<float> packed(16 * k);
  for (size_t i = 0; i < k; ++i) {
    if (index[i] >= g->n_mats) return fail(DPCULL_ERR_OUT_OF_RANGE, "matrix %u >= %zu", index[i], g->n_mats);
    memcpy(&packed[16 * i], (const char*)matrices + (size_t)index[i] * stride, 64);
  }
  const void* src[2] = {packed.data(), index};
  const size_t bytes[2] = {64 * k, 4 * k};
  unsigned char* dev[2];
  int rc = stage_upload(c, 2, src, bytes, dev);
  if (rc) return rc;
  if (launch_scatter_matrices(g->mats, reinterpret_cast<float*>(dev[0]), reinterpret_cast<uint32_t*>(dev[1]),
                              (uint32_t)k, nullptr, c->stream))
    return cuda_fail(cudaGetLastError(), "update matrices");
  c->launches++;
  return cache_stale(c, *g);
}

int dpcull_group_bind_device_matrices(dpcull_ctx c, dpcull_group gh, const float* dev, size_t count)
{
  Group* g = get_group(c, gh);
  if (!g) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad group %u", gh);
  if (count && (!dev || ((uintptr_t)dev & 15))) return fail(DPCULL_ERR_INVALID_ARGUMENT, "device matrices must be 16-byte aligned");
  CU(cudaStreamSynchronize(c->stream));
  if (g->mats_cap) dfree(c, g->mats, g->mats_cap * 64);
  g->mats = const_cast<float*>(dev);
  g->mats_cap = 0;
  g->n_mats = count;
  // The world matrices of a tree of this context go stale at each compute of that tree;
  // any other device memory may change without the library seeing it: never cached.
  g->tree = -1;
  for (size_t t = 0; t < c->trees.size(); ++t)
    if (c->trees[t].alive && c->trees[t].world == dev) g->tree = (int)t;
  g->cache_volatile = g->tree < 0;
  return cache_stale(c, *g);
}

int dpcull_group_bounding_box(dpcull_ctx c, dpcull_group gh, float lower[3], float upper[3])
{
  Group* g = get_group(c, gh);
  if (!g || !lower || !upper) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad arguments");
  float box[8] = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX, 0, 0};
  if (g->n) {
    int rc = check_cull_ready(*g);
    if (rc) return rc;
    float* partials = g->box_scratch;
    unsigned int* counter = reinterpret_cast<unsigned int*>(g->box_scratch + bbox_partials_needed(0));
    float* out = g->box_scratch + bbox_partials_needed(0) + 8;
    if (launch_bbox(g->soa, (uint32_t)g->cap, (uint32_t)g->n, g->mats, partials, counter, out, c->stream))
      return cuda_fail(cudaGetLastError(), "bbox launch");
    c->launches++;
    CU(cudaMemcpyAsync(box, out, 6 * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
  }
  // Box3f(lower, upper) of the folded corners (Boxnt.h:214-231): init, then two updates.
  for (int i = 0; i < 3; ++i) {
    float lo = FLT_MAX, hi = -FLT_MAX;
    const float p0 = box[i], p1 = box[3 + i];
    if (lo > p0) lo = p0;
    if (hi < p0) hi = p0;
    if (lo > p1) lo = p1;
    if (hi < p1) hi = p1;
    lower[i] = lo;
    upper[i] = hi;
  }
  return DPCULL_OK;
}

// ---- results -----------------------------------------------------------------------
int dpcull_result_create(dpcull_ctx c, dpcull_group gh, dpcull_result* out)
{
  Group* g = get_group(c, gh);
  if (!g || !out) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad group %u", gh);
  c->results.emplace_back();
  Result& r = c->results.back();
  r.alive = true;
  r.group = gh;
  int rc = dalloc(c, (void**)&r.n_changed, 4);
  if (rc) {
    r.alive = false;
    return rc;
  }
  CU(cudaMemsetAsync(r.n_changed, 0, 4, c->stream));
  const dpcull_result h = (dpcull_result)(c->results.size() - 1);
  c->groups[gh].results.push_back(h);
  *out = h;
  return DPCULL_OK;
}

int dpcull_result_destroy(dpcull_ctx c, dpcull_result rh)
{
  Result* r = get_result(c, rh);
  if (!r) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad result %u", rh);
  cudaStreamSynchronize(c->stream);
  dfree(c, r->bits, r->words_cap * 4);
  dfree(c, r->changed, r->changed_cap * 4);
  dfree(c, r->n_changed, 4);
  dfree(c, r->delta, r->words_cap * 4);
  dfree(c, r->chunk_tot, (chunks_of(r->words_cap) + 2) * 4);
  if (r->group < c->groups.size()) {
    auto& v = c->groups[r->group].results;
    v.erase(std::remove(v.begin(), v.end(), rh), v.end());
  }
  *r = Result();
  return DPCULL_OK;
}

int dpcull_cull(dpcull_ctx c, dpcull_group gh, dpcull_result rh, const float vp[16])
{
  Group* g = get_group(c, gh);
  Result* r = get_result(c, rh);
  if (!g || !r || !vp) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad group, result or matrix");
  if (r->group != gh) return fail(DPCULL_ERR_INVALID_ARGUMENT, "result %u belongs to another group", rh);
  int rc = check_cull_ready(*g);
  if (rc) return rc;
  rc = result_prepare(c, *r, *g);
  if (rc) return rc;
  if (g->n == 0) {
    CU(cudaMemsetAsync(r->n_changed, 0, 4, c->stream));
    return DPCULL_OK;
  }
  CullLaunch a{};
  a.scenes = nullptr;
  a.views = nullptr;
  a.n_scenes = 1;
  a.items_per_ticket = 1;
  a.exact_only = c->exact_only ? 1u : 0u;
  a.ctl = c->ctl;
  a.one_scene = scene_of(*g, 0, 1, 1, 0);
  if (c->exact_only || !c->box_cache) a.one_scene.box = nullptr;
  const std::vector<uint32_t> groups{gh};
  const std::vector<CullScene> scenes{a.one_scene};
  const CacheMode mode = batch_mode(c, groups, scenes);
  a.cache_mode = mode;
  a.one_view = view_of(*r, vp);
  a.item_tiles = item_tiles_for(a.one_scene.n_tiles, c->sm_count);
  a.n_items = lay_out_items(&a.one_scene, 1, a.item_tiles, tail_units(c->sm_count));
  a.emit_views = fused_emit_views(1, a.one_view.n_words);
  const int grid = persistent_grid(c, 1, 0, a.n_items, 1, mode);
  if (launch_cull(a, grid, 1, c->stream)) return cuda_fail(cudaGetLastError(), "cull launch");
  if (!a.emit_views && launch_changed_lists(nullptr, a.one_view, 1, a.one_view.n_words, &c->ctl->error, c->stream))
    return cuda_fail(cudaGetLastError(), "changed-list launch");
  c->launches += a.emit_views ? 1 : 2;
  note_launch(c, groups, scenes, mode);
  return DPCULL_OK;
}

// The visibility words (bits: null skips them) and the changed list (n_changed: null skips
// it; changed: null reads the length only) of one result, in one round trip in the common
// case: the count, the error word and a prefix of the list sized from the last read
// travel together (entries past the count are left unspecified); a second copy only when
// the list outgrew the prefix.  The callers check the words' capacity.
static int result_read(dpcull_ctx c, Result* r, uint32_t* bits, uint32_t* changed, size_t cap,
                       size_t* n_changed)
{
  const size_t words = (r->size_bits + 31) / 32;
  if (bits && words) CU(cudaMemcpyAsync(bits, r->bits, words * 4, cudaMemcpyDeviceToHost, c->stream));
  size_t spec = 0;
  if (n_changed) {
    spec = changed ? std::min<size_t>(cap, std::max<size_t>(4096, r->last_changed + r->last_changed / 2)) : 0;
    CU(cudaMemcpyAsync(c->h_err + 2, r->n_changed, 4, cudaMemcpyDeviceToHost, c->stream));
    if (spec) CU(cudaMemcpyAsync(changed, r->changed, spec * 4, cudaMemcpyDeviceToHost, c->stream));
  }
  CU(enqueue_error_read(c));
  CU(cudaStreamSynchronize(c->stream));
  int rc = device_errors_read(c);
  if (rc || !n_changed) return rc;
  const uint32_t cnt = c->h_err[2];
  *n_changed = cnt;
  if (cnt > cap) return fail(DPCULL_ERR_CAPACITY, "changed list has %u entries, buffer %zu", cnt, cap);
  r->last_changed = cnt;
  if (cnt > spec) {
    if (!changed) return fail(DPCULL_ERR_INVALID_ARGUMENT, "null output");
    CU(cudaMemcpyAsync(changed + spec, r->changed + spec, (size_t)(cnt - spec) * 4, cudaMemcpyDeviceToHost,
                       c->stream));
    CU(cudaStreamSynchronize(c->stream));
  }
  return DPCULL_OK;
}

int dpcull_result_changed(dpcull_ctx c, dpcull_result rh, uint32_t* out, size_t cap, size_t* n)
{
  Result* r = get_result(c, rh);
  if (!r || !n) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad result %u", rh);
  return result_read(c, r, nullptr, out, cap, n);
}

int dpcull_result_bits(dpcull_ctx c, dpcull_result rh, uint32_t* out, size_t n_words, size_t* n_bits)
{
  Result* r = get_result(c, rh);
  if (!r) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad result %u", rh);
  const size_t words = (r->size_bits + 31) / 32;
  if (n_bits) *n_bits = r->size_bits;
  if (words > n_words) return fail(DPCULL_ERR_CAPACITY, "need %zu words", words);
  if (words && !out) return fail(DPCULL_ERR_INVALID_ARGUMENT, "null output");
  return result_read(c, r, out, nullptr, 0, nullptr);
}

int dpcull_result_read(dpcull_ctx c, dpcull_result rh, uint32_t* bits, size_t n_words, size_t* n_bits,
                       uint32_t* changed, size_t cap, size_t* n_changed)
{
  Result* r = get_result(c, rh);
  if (!r || !n_changed) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad result %u", rh);
  const size_t words = (r->size_bits + 31) / 32;
  if (n_bits) *n_bits = r->size_bits;
  if (bits && words > n_words) return fail(DPCULL_ERR_CAPACITY, "need %zu words", words);
  return result_read(c, r, bits, changed, cap, n_changed);
}

int dpcull_result_is_visible(dpcull_ctx c, dpcull_result rh, size_t index, int* visible)
{
  Result* r = get_result(c, rh);
  if (!r || !visible) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad result %u", rh);
  if (index >= r->size_bits) {  // ResultBitSet.h:75: unknown objects are visible
    *visible = 1;
    return DPCULL_OK;
  }
  uint32_t w = 0;
  CU(cudaMemcpyAsync(c->h_err + 2, r->bits + index / 32, 4, cudaMemcpyDeviceToHost, c->stream));
  CU(cudaStreamSynchronize(c->stream));
  w = c->h_err[2];
  *visible = (w >> (index % 32)) & 1u;
  return DPCULL_OK;
}

int dpcull_result_move(dpcull_ctx c, dpcull_result rh, size_t old_index, size_t new_index)
{
  Result* r = get_result(c, rh);
  if (!r) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad result %u", rh);
  if (!r->bits || new_index >= r->size_bits) return DPCULL_OK;
  const uint32_t old32 = old_index >= r->size_bits ? (uint32_t)r->size_bits : (uint32_t)old_index;
  if (launch_move_bit(r->bits, (uint32_t)r->size_bits, old32, (uint32_t)new_index, c->stream))
    return cuda_fail(cudaGetLastError(), "move bit");
  c->launches++;
  return DPCULL_OK;
}

int dpcull_result_device(dpcull_ctx c, dpcull_result rh, uint32_t** bits, uint32_t** changed,
                         uint32_t** n_changed)
{
  Result* r = get_result(c, rh);
  if (!r) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad result %u", rh);
  if (bits) *bits = r->bits;
  if (changed) *changed = r->changed;
  if (n_changed) *n_changed = r->n_changed;
  return DPCULL_OK;
}

// ---- batched -----------------------------------------------------------------------
int dpcull_cull_batched(dpcull_ctx c, const dpcull_job* jobs, size_t n_jobs, const dpcull_tuning* tuning)
{
  if (!c || (n_jobs && !jobs)) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad arguments");
  uint32_t maxv = 1;
  for (size_t j = 0; j < n_jobs; ++j) maxv = std::max(maxv, jobs[j].n_views);
  dpcull_tuning t = tuning ? *tuning : dpcull_tuning{(uint32_t)default_vpp(maxv), 1, 0, 0};
  if (!valid_vpp(t.views_per_pass)) return fail(DPCULL_ERR_INVALID_ARGUMENT, "views_per_pass must be 1, 2, 4 or 8");
  std::vector<CullScene> scenes;
  std::vector<CullView> views;
  uint32_t items = 0, item_tiles = kItemTiles;
  std::vector<uint32_t> groups;
  int rc = build_batch(c, jobs, n_jobs, t.views_per_pass, scenes, views, &items, &groups, nullptr, &item_tiles);
  if (rc) return rc;
  if (!items) return DPCULL_OK;
  CullScene* ds = nullptr;
  CullView* dv = nullptr;
  rc = dalloc(c, (void**)&ds, scenes.size() * sizeof(CullScene));
  if (rc) return rc;
  rc = dalloc(c, (void**)&dv, views.size() * sizeof(CullView));
  if (rc) {
    dfree(c, ds, scenes.size() * sizeof(CullScene));
    return rc;
  }
  cudaMemcpyAsync(ds, scenes.data(), scenes.size() * sizeof(CullScene), cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(dv, views.data(), views.size() * sizeof(CullView), cudaMemcpyHostToDevice, c->stream);
  const CacheMode mode = batch_mode(c, groups, scenes);
  rc = launch_batch(c, ds, dv, scenes, (uint32_t)views.size(), items, item_tiles, t, c->stream, nullptr, nullptr,
                    mode);
  if (!rc) note_launch(c, groups, scenes, mode);
  cudaStreamSynchronize(c->stream);
  dfree(c, ds, scenes.size() * sizeof(CullScene));
  dfree(c, dv, views.size() * sizeof(CullView));
  return rc;
}

static int plan_capture(dpcull_ctx c, Plan& p, int slot, CacheMode mode)
{
  cudaStream_t cs, side;
  cudaEvent_t fork, join;
  CU(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  CU(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
  CU(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
  CU(cudaEventCreateWithFlags(&join, cudaEventDisableTiming));
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess &&
      launch_copy_words(reinterpret_cast<uint32_t*>(p.d_views), reinterpret_cast<const uint32_t*>(p.h_views[slot]),
                        p.views.size() * sizeof(CullView) / 4, cs))
    e = cudaGetLastError() == cudaSuccess ? cudaErrorLaunchFailure : cudaGetLastError();
  int rc = DPCULL_OK;
  if (e == cudaSuccess) {
    const uint64_t before = c->launches;
    rc = launch_batch(c, p.d_scenes, p.d_views, p.scenes, (uint32_t)p.views.size(), p.n_items,
                      p.item_tiles, p.tuning, cs, p.kt[slot][0], p.kt[slot][1], mode, side, fork, p.d_emit_first,
                      p.emit_blocks);
    c->launches = before;  // counted when the graph is replayed
    if (rc == DPCULL_OK) {  // the side stream's timing nodes join the capture again
      e = cudaEventRecord(join, side);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(cs, join, 0);
    }
  }
  cudaError_t e2 = cudaStreamEndCapture(cs, &graph);
  if (e == cudaSuccess) e = e2;
  if (e == cudaSuccess && rc == DPCULL_OK) e = cudaGraphInstantiate(&p.exec[mode][slot], graph, 0);
  if (graph) cudaGraphDestroy(graph);
  cudaStreamDestroy(cs);
  cudaStreamDestroy(side);
  cudaEventDestroy(fork);
  cudaEventDestroy(join);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "plan graph capture");
  return DPCULL_OK;
}

static int time_batch(dpcull_ctx c, const CullScene* ds, const CullView* dv,
                      const std::vector<CullScene>& sc, const std::vector<CullView>& vw,
                      uint32_t items, uint32_t item_tiles, const dpcull_tuning& t, int reps, float* ms,
                      CacheMode mode)
{
  cudaEvent_t e0, e1;
  CU(cudaEventCreate(&e0));
  CU(cudaEventCreate(&e1));
  const uint32_t nvw = (uint32_t)vw.size();
  int rc = launch_batch(c, ds, dv, sc, nvw, items, item_tiles, t, c->stream, nullptr, nullptr, mode);  // warm-up
  if (!rc) cudaEventRecord(e0, c->stream);
  for (int i = 0; i < reps && !rc; ++i)
    rc = launch_batch(c, ds, dv, sc, nvw, items, item_tiles, t, c->stream, nullptr, nullptr, mode);
  if (!rc) {
    cudaEventRecord(e1, c->stream);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(ms, e0, e1);
    *ms /= (float)reps;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

int dpcull_autotune(dpcull_ctx c, const dpcull_job* jobs, size_t n_jobs, dpcull_tuning* out)
{
  if (!c || !out || (n_jobs && !jobs)) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad arguments");
  uint32_t maxv = 1;
  for (size_t j = 0; j < n_jobs; ++j) maxv = std::max(maxv, jobs[j].n_views);
  // Save every result's visibility words: tuning launches overwrite them.
  std::vector<std::pair<Result*, uint32_t*>> saved;
  std::vector<CullScene> scenes;
  std::vector<CullView> views;
  uint32_t items = 0;
  int rc = build_batch(c, jobs, n_jobs, 1, scenes, views, &items, nullptr, nullptr, nullptr);
  if (rc) return rc;
  const std::string key = tune_key(scenes, views);
  auto it = c->tune_cache.find(key);
  if (it != c->tune_cache.end()) {
    *out = it->second;
    return DPCULL_OK;
  }
  for (size_t j = 0; j < n_jobs; ++j)
    for (uint32_t v = 0; v < jobs[j].n_views; ++v) {
      Result* r = get_result(c, jobs[j].results[v]);
      uint32_t* copy = nullptr;
      rc = dalloc(c, (void**)&copy, r->words_cap * 4);
      if (rc) return rc;
      cudaMemcpyAsync(copy, r->bits, r->words_cap * 4, cudaMemcpyDeviceToDevice, c->stream);
      saved.push_back({r, copy});
    }
  dpcull_tuning best{(uint32_t)default_vpp(maxv), 1, 0, 0};
  float best_ms = 1e30f;
  // The kernel a plan of these jobs runs from its third launch on: the one that reads the
  // box caches when every scene keeps one (stored here first by one Fill launch, as a plan's
  // second launch would), the fused one otherwise.
  bool cached = c->box_cache && !c->exact_only && !scenes.empty();
  for (const CullScene& sc : scenes) cached = cached && sc.box;
  bool filled = false;
  const uint32_t vpps[4] = {1, 2, 4, 8};
  for (uint32_t vpp : vpps) {
    if (vpp > 1 && vpp / 2 >= maxv) continue;  // wider passes than any scene has views
    std::vector<CullScene> sc;
    std::vector<CullView> vw;
    std::vector<uint32_t> groups;
    uint32_t it_items = 0, it_tiles = kItemTiles;
    rc = build_batch(c, jobs, n_jobs, vpp, sc, vw, &it_items, &groups, nullptr, &it_tiles);
    if (rc || !it_items) break;
    CullScene* ds = nullptr;
    CullView* dv = nullptr;
    if (dalloc(c, (void**)&ds, sc.size() * sizeof(CullScene)) || dalloc(c, (void**)&dv, vw.size() * sizeof(CullView))) {
      rc = DPCULL_ERR_NO_MEMORY;
      break;
    }
    cudaMemcpyAsync(ds, sc.data(), sc.size() * sizeof(CullScene), cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(dv, vw.data(), vw.size() * sizeof(CullView), cudaMemcpyHostToDevice, c->stream);
    if (cached && !filled) {
      const dpcull_tuning ft{vpp, 1, 0, 0};
      rc = launch_batch(c, ds, dv, sc, (uint32_t)vw.size(), it_items, it_tiles, ft, c->stream, nullptr, nullptr,
                        kCacheFill);
      if (rc) break;
      note_launch(c, groups, sc, kCacheFill, false);
      filled = true;
    }
    const CacheMode mode = cached ? kCacheRead : kCacheNone;
    const int occ = cull_max_ctas_per_sm((int)vpp, mode);
    for (uint32_t tpt : {1u, 2u, 4u}) {
      for (int cps = 1; cps <= occ; ++cps) {
        dpcull_tuning t{vpp, tpt, (uint32_t)cps, 0};
        float ms = 0;
        rc = time_batch(c, ds, dv, sc, vw, it_items, it_tiles, t, 3, &ms, mode);
        if (rc) break;
        if (ms < best_ms) {
          best_ms = ms;
          best = t;
        }
      }
      if (rc) break;
    }
    cudaStreamSynchronize(c->stream);
    dfree(c, ds, sc.size() * sizeof(CullScene));
    dfree(c, dv, vw.size() * sizeof(CullView));
    if (rc) break;
  }
  for (auto& s : saved) {
    cudaMemcpyAsync(s.first->bits, s.second, s.first->words_cap * 4, cudaMemcpyDeviceToDevice, c->stream);
  }
  cudaStreamSynchronize(c->stream);
  for (auto& s : saved) dfree(c, s.second, s.first->words_cap * 4);
  if (rc) return rc;
  rc = check_device_errors(c);
  if (rc) return rc;
  c->tune_cache[key] = best;
  tune_cache_store(key, best);
  *out = best;
  return DPCULL_OK;
}

int dpcull_plan_create(dpcull_ctx c, const dpcull_job* jobs, size_t n_jobs,
                       const dpcull_tuning* tuning, dpcull_plan* out)
{
  if (!c || !out || (n_jobs && !jobs)) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad arguments");
  dpcull_tuning t{};
  if (tuning) {
    t = *tuning;
  } else {
    int rc = dpcull_autotune(c, jobs, n_jobs, &t);
    if (rc) return rc;
  }
  if (!valid_vpp(t.views_per_pass)) return fail(DPCULL_ERR_INVALID_ARGUMENT, "views_per_pass must be 1, 2, 4 or 8");
  Plan p;
  p.alive = true;
  p.tuning = t;
  int rc = build_batch(c, jobs, n_jobs, t.views_per_pass, p.scenes, p.views, &p.n_items, &p.groups, &p.results,
                       &p.item_tiles);
  if (rc) return rc;
  if (!p.n_items) return fail(DPCULL_ERR_STATE, "plan has no work (all groups empty)");
  for (uint32_t g : p.groups) p.incarnations.push_back(c->groups[g].incarnation);
  for (size_t j = 0; j < n_jobs; ++j) {
    p.all_groups.push_back(jobs[j].group);
    p.all_incarnations.push_back(c->groups[jobs[j].group].incarnation);
    for (uint32_t v = 0; v < jobs[j].n_views; ++v) p.all_results.push_back(jobs[j].results[v]);
  }
  CU(cudaMallocHost((void**)&p.h_counts, (p.all_results.size() + 2) * sizeof(uint32_t)));
  CU(cudaMallocHost((void**)&p.h_rcounts, (p.all_results.size() + 2) * sizeof(uint32_t)));
  rc = dalloc(c, (void**)&p.d_scenes, p.scenes.size() * sizeof(CullScene));
  if (!rc) rc = dalloc(c, (void**)&p.d_views, p.views.size() * sizeof(CullView));
  // The changed-list pass of the plan in one dimension: each view's own chunk count.
  std::vector<uint32_t> first(p.views.size() + 1, 0u);
  for (size_t v = 0; v < p.views.size(); ++v) first[v + 1] = first[v] + emit_blocks_of(p.views[v].n_words);
  p.emit_blocks = first.back();
  if (!rc) rc = dalloc(c, (void**)&p.d_emit_first, first.size() * sizeof(uint32_t));
  if (rc) return rc;
  CU(cudaMemcpyAsync(p.d_emit_first, first.data(), first.size() * sizeof(uint32_t), cudaMemcpyHostToDevice,
                     c->stream));
  CU(cudaMemcpyAsync(p.d_scenes, p.scenes.data(), p.scenes.size() * sizeof(CullScene), cudaMemcpyHostToDevice, c->stream));
  for (int s = 0; s < 2; ++s) {
    CU(cudaMallocHost((void**)&p.h_views[s], p.views.size() * sizeof(CullView)));
    memcpy(p.h_views[s], p.views.data(), p.views.size() * sizeof(CullView));
    CU(cudaEventCreateWithFlags(&p.done[s], cudaEventDisableTiming));
    CU(cudaEventCreate(&p.kt[s][0]));
    CU(cudaEventCreate(&p.kt[s][1]));
    rc = plan_capture(c, p, s, kCacheNone);  // the cache kernels' graphs on first use
    if (rc) return rc;
  }
  CU(cudaStreamSynchronize(c->stream));
  c->plans.push_back(p);
  *out = (dpcull_plan)(c->plans.size() - 1);
  return DPCULL_OK;
}

int dpcull_plan_set_views(dpcull_ctx c, dpcull_plan ph, const float* vps)
{
  Plan* p = get_plan(c, ph);
  if (!p || !vps) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad plan or matrices");
  const int s = p->next;
  if (p->pending[s]) {
    CU(cudaEventSynchronize(p->done[s]));
    p->pending[s] = false;
  }
  for (size_t v = 0; v < p->views.size(); ++v) {
    memcpy(p->h_views[s][v].vp, vps + 16 * v, 64);
    memcpy(p->views[v].vp, vps + 16 * v, 64);
  }
  p->fresh[s] = true;
  return DPCULL_OK;
}

static void plan_slot_copying(Plan* p, int s, bool on);

int dpcull_plan_launch(dpcull_ctx c, dpcull_plan ph)
{
  Plan* p = get_plan(c, ph);
  if (!p) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad plan %u", ph);
  for (size_t i = 0; i < p->all_groups.size(); ++i) {
    Group* g = get_group(c, p->all_groups[i]);
    if (!g || g->incarnation != p->all_incarnations[i])
      return fail(DPCULL_ERR_STATE, "plan is stale: group %u changed since the plan was built", p->all_groups[i]);
  }
  for (size_t i = 0; i < p->groups.size(); ++i) {
    Group* g = get_group(c, p->groups[i]);
    if (g->soa != p->scenes[i].soa || g->mats != p->scenes[i].mats || g->n_mats != p->scenes[i].n_mats)
      return fail(DPCULL_ERR_STATE, "plan is stale: group %u storage changed", p->groups[i]);
    int rc = check_cull_ready(*g);
    if (rc) return rc;
  }
  const int s = p->next;
  if (!p->fresh[s]) {
    if (p->pending[s]) {
      CU(cudaEventSynchronize(p->done[s]));
      p->pending[s] = false;
    }
    for (size_t v = 0; v < p->views.size(); ++v) memcpy(p->h_views[s][v].vp, p->views[v].vp, 64);
  }
  p->fresh[s] = false;
  if (p->copies) {
    // The launch writes its results into the slot's copy buffer too, unless a snapshot
    // still waits to be read from it; copies still reading the buffer finish first.
    const bool hold = p->snap_pending && p->snap_slot == s;
    plan_slot_copying(p, s, !hold);
    p->copied[s] = !hold;
    if (!hold && p->read_pending[s]) CU(cudaStreamWaitEvent(c->stream, p->copies_ev[s], 0));
  }
  const CacheMode mode = batch_mode(c, p->groups, p->scenes);
  if (!p->exec[mode][s]) {
    int rc = plan_capture(c, *p, s, mode);
    if (rc) return rc;
  }
  CU(cudaGraphLaunch(p->exec[mode][s], c->stream));
  CU(cudaEventRecord(p->done[s], c->stream));
  note_launch(c, p->groups, p->scenes, mode);
  p->pending[s] = true;
  p->next ^= 1;
  // the graph's kernels: the view copy, the cull, and the changed lists unless the cull
  // builds them
  c->launches += fused_emit_views((uint32_t)p->views.size(), max_words_of(p->scenes)) ? 2 : 3;
  return DPCULL_OK;
}

int dpcull_plan_kernel_ms(dpcull_ctx c, dpcull_plan ph, uint32_t back, float* ms)
{
  Plan* p = get_plan(c, ph);
  if (!p || !ms || back > 1) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad plan %u or argument", ph);
  const int s = back ? p->next : p->next ^ 1;  // the last launch used next ^ 1
  if (!p->pending[s]) return fail(DPCULL_ERR_STATE, "no such launch of plan %u", ph);
  CU(cudaEventSynchronize(p->kt[s][1]));
  CU(cudaEventElapsedTime(ms, p->kt[s][0], p->kt[s][1]));
  return DPCULL_OK;
}

int dpcull_plan_read(dpcull_ctx c, dpcull_plan ph, uint32_t* const* bits, uint32_t* const* changed,
                     const size_t* changed_cap, size_t* n_changed)
{
  Plan* p = get_plan(c, ph);
  if (!p) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad plan %u", ph);
  const size_t nr = p->all_results.size();
  std::vector<Result*> rs(nr);
  for (size_t i = 0; i < nr; ++i) {
    rs[i] = get_result(c, p->all_results[i]);
    if (!rs[i]) return fail(DPCULL_ERR_STATE, "plan %u: result %u was destroyed", ph, p->all_results[i]);
  }
  // 1. every changed count and the device error word, one wait (into a buffer of its own:
  //    a snapshot taken before this read keeps its counts for dpcull_plan_read_async)
  for (size_t i = 0; i < nr; ++i)
    CU(cudaMemcpyAsync(p->h_rcounts + i, rs[i]->n_changed, 4, cudaMemcpyDeviceToHost, c->stream));
  CU(cudaMemcpyAsync(p->h_rcounts + nr, &c->ctl->error, 2 * sizeof(unsigned int), cudaMemcpyDeviceToHost,
                     c->stream));
  CU(cudaStreamSynchronize(c->stream));
  if (p->h_rcounts[nr]) return check_device_errors(c);
  // 2. every requested array, one wait
  for (size_t i = 0; i < nr; ++i) {
    const uint32_t cnt = p->h_rcounts[i];
    if (n_changed) n_changed[i] = cnt;
    if (bits && bits[i] && rs[i]->size_bits)
      CU(cudaMemcpyAsync(bits[i], rs[i]->bits, (rs[i]->size_bits + 31) / 32 * 4, cudaMemcpyDeviceToHost,
                         c->stream));
    if (changed && changed[i] && cnt) {
      if (!changed_cap || cnt > changed_cap[i]) {
        CU(cudaStreamSynchronize(c->stream));
        return fail(DPCULL_ERR_CAPACITY, "plan %u: result %zu has %u changed objects", ph, i, cnt);
      }
      CU(cudaMemcpyAsync(changed[i], rs[i]->changed, (size_t)cnt * 4, cudaMemcpyDeviceToHost, c->stream));
    }
  }
  CU(cudaStreamSynchronize(c->stream));
  return DPCULL_OK;
}

// The copy buffers of a plan's results, one per slot (set up on the first asynchronous
// read, and again when a result's size changed), and the views' copy pointers.
static int plan_copies_setup(dpcull_ctx c, Plan* p, const std::vector<Result*>& rs)
{
  const size_t nr = rs.size();
  bool same = p->copies && p->snap_sizes.size() == nr;
  for (size_t i = 0; same && i < nr; ++i) same = p->snap_sizes[i] == rs[i]->size_bits;
  if (same) return DPCULL_OK;
  // Nothing may still read the old buffers or launch with views that point at them.
  for (int s = 0; s < 2; ++s)
    if (p->read_pending[s]) CU(cudaEventSynchronize(p->copies_ev[s]));
  CU(cudaStreamSynchronize(c->stream));
  for (int s = 0; s < 2; ++s) {
    p->read_pending[s] = p->copied[s] = p->copying[s] = false;
    dfree(c, p->cbuf[s], p->snap_words * 4);
    p->cbuf[s] = nullptr;
    for (size_t v = 0; v < p->views.size(); ++v) {
      p->h_views[s][v].copy_bits = p->h_views[s][v].copy_changed = p->h_views[s][v].copy_count = nullptr;
    }
  }
  dfree(c, p->d_copies, std::max<size_t>(2 * p->snap_sizes.size(), 1) * sizeof(ResultCopy));
  p->d_copies = nullptr;
  p->copies = false;
  p->snap_pending = false;
  p->snap_slot = -1;
  p->snap_sizes.assign(nr, 0);
  p->snap_bits.assign(nr, 0);
  p->snap_changed.assign(nr, 0);
  size_t total = (nr + 63) / 64 * 64;  // the counts
  uint32_t max_len = 1;
  for (size_t i = 0; i < nr; ++i) {
    const size_t n = rs[i]->size_bits, words = (n + 31) / 32;
    p->snap_sizes[i] = n;
    p->snap_bits[i] = total;
    total += (words + 63) / 64 * 64;
    p->snap_changed[i] = total;
    total += (n + 63) / 64 * 64;
    max_len = std::max<uint32_t>(max_len, (uint32_t)std::max(n, words));
  }
  p->snap_words = std::max<size_t>(total, 64);
  p->snap_max_len = max_len;
  int rc = dalloc(c, (void**)&p->cbuf[0], p->snap_words * 4);
  if (!rc) rc = dalloc(c, (void**)&p->cbuf[1], p->snap_words * 4);
  if (!rc) rc = dalloc(c, (void**)&p->d_copies, std::max<size_t>(2 * nr, 1) * sizeof(ResultCopy));
  if (rc) return rc;
  for (int s = 0; s < 2; ++s) CU(cudaMemsetAsync(p->cbuf[s], 0, (nr + 63) / 64 * 64 * 4, c->stream));
  std::vector<ResultCopy> h(2 * nr);
  for (int s = 0; s < 2; ++s)
    for (size_t i = 0; i < nr; ++i)
      h[s * nr + i] = ResultCopy{rs[i]->bits, rs[i]->changed, rs[i]->n_changed, p->cbuf[s] + p->snap_bits[i],
                                 p->cbuf[s] + p->snap_changed[i], p->cbuf[s] + i,
                                 (uint32_t)((rs[i]->size_bits + 31) / 32), 0};
  if (nr) CU(cudaMemcpyAsync(p->d_copies, h.data(), 2 * nr * sizeof(ResultCopy), cudaMemcpyHostToDevice, c->stream));
  // Launched view v culls result view_result[v] (the launched views are the jobs' views of
  // non-empty groups, in job and view order).
  p->view_result.assign(p->views.size(), -1);
  size_t i = 0;
  for (size_t v = 0; v < p->views.size(); ++v) {
    while (i < nr && p->all_results[i] != p->results[v]) ++i;
    if (i == nr) return fail(DPCULL_ERR_STATE, "plan views do not match its results");
    p->view_result[v] = (int)i++;
  }
  if (!p->copy_stream) CU(cudaStreamCreateWithFlags(&p->copy_stream, cudaStreamNonBlocking));
  if (!p->snap_ev) CU(cudaEventCreateWithFlags(&p->snap_ev, cudaEventDisableTiming));
  if (!p->counts_ev) CU(cudaEventCreateWithFlags(&p->counts_ev, cudaEventDisableTiming));
  for (int s = 0; s < 2; ++s)
    if (!p->copies_ev[s]) CU(cudaEventCreateWithFlags(&p->copies_ev[s], cudaEventDisableTiming));
  CU(cudaStreamSynchronize(c->stream));
  p->copies = true;
  return DPCULL_OK;
}

// Points the slot's views at its copy buffer (on) or at nothing (off).  The slot's last
// launch has finished (callers wait for it).
static void plan_slot_copying(Plan* p, int s, bool on)
{
  if (p->copying[s] == on) return;
  for (size_t v = 0; v < p->views.size(); ++v) {
    CullView& cv = p->h_views[s][v];
    const size_t i = (size_t)p->view_result[v];
    cv.copy_bits = on ? p->cbuf[s] + p->snap_bits[i] : nullptr;
    cv.copy_changed = on ? p->cbuf[s] + p->snap_changed[i] : nullptr;
    cv.copy_count = on ? p->cbuf[s] + i : nullptr;
  }
  p->copying[s] = on;
}

// The results of a plan's launches, in job and view order (every one still alive).
static int plan_results(dpcull_ctx c, dpcull_plan ph, Plan* p, std::vector<Result*>& rs)
{
  const size_t nr = p->all_results.size();
  rs.resize(nr);
  for (size_t i = 0; i < nr; ++i) {
    rs[i] = get_result(c, p->all_results[i]);
    if (!rs[i]) return fail(DPCULL_ERR_STATE, "plan %u: result %u was destroyed", ph, p->all_results[i]);
  }
  return DPCULL_OK;
}

int dpcull_plan_snapshot(dpcull_ctx c, dpcull_plan ph)
{
  Plan* p = get_plan(c, ph);
  if (!p) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad plan %u", ph);
  std::vector<Result*> rs;
  int rc = plan_results(c, ph, p, rs);
  if (!rc) rc = plan_copies_setup(c, p, rs);
  if (rc) return rc;
  const size_t nr = rs.size();
  const int L = p->next ^ 1;  // the slot of the last launch
  if (!p->copied[L]) {
    // That launch did not write its copies (it came before the first asynchronous read,
    // or ran while an earlier snapshot held the buffer): copy the live results, after the
    // copies still reading the buffer.
    if (p->read_pending[L]) CU(cudaStreamWaitEvent(c->stream, p->copies_ev[L], 0));
    if (launch_snapshot(p->d_copies + (size_t)L * nr, (uint32_t)nr, p->snap_max_len, c->stream))
      return cuda_fail(cudaGetLastError(), "snapshot launch");
    c->launches++;
    p->copied[L] = true;
  }
  CU(cudaEventRecord(p->snap_ev, c->stream));
  // The counts and the error word go to the host first: the list copies need the lengths.
  CU(cudaStreamWaitEvent(p->copy_stream, p->snap_ev, 0));
  if (nr) CU(cudaMemcpyAsync(p->h_counts, p->cbuf[L], nr * 4, cudaMemcpyDeviceToHost, p->copy_stream));
  CU(cudaMemcpyAsync(p->h_counts + nr, &c->ctl->error, 2 * sizeof(unsigned int), cudaMemcpyDeviceToHost,
                     p->copy_stream));
  CU(cudaEventRecord(p->counts_ev, p->copy_stream));
  p->snap_slot = L;
  p->snap_pending = true;
  return DPCULL_OK;
}

int dpcull_plan_read_async(dpcull_ctx c, dpcull_plan ph, uint32_t* const* bits, uint32_t* const* changed,
                           const size_t* changed_cap, size_t* n_changed)
{
  Plan* p = get_plan(c, ph);
  if (!p) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad plan %u", ph);
  std::vector<Result*> rs;
  int rc = plan_results(c, ph, p, rs);
  if (rc) return rc;
  // Without a pending snapshot, take one of the last launch now.
  if (!p->snap_pending) {
    rc = dpcull_plan_snapshot(c, ph);
    if (rc) return rc;
  }
  p->snap_pending = false;
  const int L = p->snap_slot;
  const size_t nr = rs.size();
  CU(cudaEventSynchronize(p->counts_ev));
  if (p->h_counts[nr]) return check_device_errors(c);
  for (size_t i = 0; i < nr; ++i) {
    const uint32_t cnt = p->h_counts[i];
    if (n_changed) n_changed[i] = cnt;
    if (changed && changed[i] && cnt && (!changed_cap || cnt > changed_cap[i]))
      return fail(DPCULL_ERR_CAPACITY, "plan %u: result %zu has %u changed objects", ph, i, cnt);
  }
  const uint32_t* buf = p->cbuf[L];
  for (size_t i = 0; i < nr; ++i) {
    const uint32_t cnt = p->h_counts[i];
    if (bits && bits[i] && p->snap_sizes[i])
      CU(cudaMemcpyAsync(bits[i], buf + p->snap_bits[i], (p->snap_sizes[i] + 31) / 32 * 4, cudaMemcpyDeviceToHost,
                         p->copy_stream));
    if (changed && changed[i] && cnt)
      CU(cudaMemcpyAsync(changed[i], buf + p->snap_changed[i], (size_t)cnt * 4, cudaMemcpyDeviceToHost,
                         p->copy_stream));
  }
  CU(cudaEventRecord(p->copies_ev[L], p->copy_stream));
  p->read_pending[L] = true;
  return DPCULL_OK;
}

int dpcull_plan_read_wait(dpcull_ctx c, dpcull_plan ph)
{
  Plan* p = get_plan(c, ph);
  if (!p) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad plan %u", ph);
  for (int s = 0; s < 2; ++s) {
    if (p->read_pending[s]) CU(cudaEventSynchronize(p->copies_ev[s]));
    p->read_pending[s] = false;
  }
  return DPCULL_OK;
}

int dpcull_plan_tuning(dpcull_ctx c, dpcull_plan ph, dpcull_tuning* out)
{
  Plan* p = get_plan(c, ph);
  if (!p || !out) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad plan %u", ph);
  *out = p->tuning;
  return DPCULL_OK;
}

int dpcull_plan_destroy(dpcull_ctx c, dpcull_plan ph)
{
  Plan* p = get_plan(c, ph);
  if (!p) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad plan %u", ph);
  cudaStreamSynchronize(c->stream);
  if (p->copy_stream) cudaStreamSynchronize(p->copy_stream);  // copies into h_counts / snap
  for (int s = 0; s < 2; ++s) {
    for (int m = 0; m < 3; ++m)
      if (p->exec[m][s]) cudaGraphExecDestroy(p->exec[m][s]);
    if (p->done[s]) cudaEventDestroy(p->done[s]);
    if (p->kt[s][0]) cudaEventDestroy(p->kt[s][0]);
    if (p->kt[s][1]) cudaEventDestroy(p->kt[s][1]);
    if (p->h_views[s]) cudaFreeHost(p->h_views[s]);
  }
  if (p->h_counts) cudaFreeHost(p->h_counts);
  if (p->h_rcounts) cudaFreeHost(p->h_rcounts);
  if (p->copy_stream) cudaStreamDestroy(p->copy_stream);
  if (p->snap_ev) cudaEventDestroy(p->snap_ev);
  if (p->counts_ev) cudaEventDestroy(p->counts_ev);
  for (int s = 0; s < 2; ++s) {
    if (p->copies_ev[s]) cudaEventDestroy(p->copies_ev[s]);
    dfree(c, p->cbuf[s], p->snap_words * 4);
  }
  dfree(c, p->d_copies, std::max<size_t>(2 * p->snap_sizes.size(), 1) * sizeof(ResultCopy));
  dfree(c, p->d_scenes, p->scenes.size() * sizeof(CullScene));
  dfree(c, p->d_views, p->views.size() * sizeof(CullView));
  dfree(c, p->d_emit_first, (p->views.size() + 1) * sizeof(uint32_t));
  *p = Plan();
  return DPCULL_OK;
}

// ---- transform tree ----------------------------------------------------------------
int dpcull_tree_create(dpcull_ctx c, size_t capacity, dpcull_tree* out)
{
  if (!c || !out || !capacity || capacity > 0xFFFFFFFFull) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad arguments");
  c->trees.emplace_back();
  Tree& t = c->trees.back();
  t.alive = true;
  t.cap = capacity;
  t.words = (capacity + 31) / 32;
  int rc = dalloc(c, (void**)&t.local, capacity * 64);
  if (!rc) rc = dalloc(c, (void**)&t.world, capacity * 64);
  if (!rc) rc = dalloc(c, (void**)&t.dirty_local, t.words * 4);
  if (!rc) rc = dalloc(c, (void**)&t.dirty_world, t.words * 4);
  if (rc) return rc;
  CU(cudaMemsetAsync(t.local, 0, capacity * 64, c->stream));
  CU(cudaMemsetAsync(t.world, 0, capacity * 64, c->stream));
  CU(cudaMemsetAsync(t.dirty_local, 0, t.words * 4, c->stream));
  CU(cudaMemsetAsync(t.dirty_world, 0, t.words * 4, c->stream));
  // Tree::Tree (Tree.cpp:38-47): the root (index 0) is the identity, local and world.
  static const float I[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  CU(cudaMemcpyAsync(t.local, I, 64, cudaMemcpyHostToDevice, c->stream));
  CU(cudaMemcpyAsync(t.world, I, 64, cudaMemcpyHostToDevice, c->stream));
  CU(cudaStreamSynchronize(c->stream));
  *out = (dpcull_tree)(c->trees.size() - 1);
  return DPCULL_OK;
}

// The groups that cull against a tree's world matrices: their cached boxes are stale
// once the tree has written new world matrices.
static int tree_groups_stale(dpcull_ctx c, dpcull_tree th)
{
  for (Group& g : c->groups)
    if (g.alive && g.tree == (int)th) {
      int rc = cache_stale(c, g);
      if (rc) return rc;
    }
  return DPCULL_OK;
}

// A tree's world array is about to go away (destroy, resize): the groups bound to it no
// longer follow the tree and are not cached until they get new matrices.
static void tree_unbind_groups(dpcull_ctx c, dpcull_tree th)
{
  for (Group& g : c->groups)
    if (g.alive && g.tree == (int)th) {
      g.tree = -1;
      g.cache_volatile = true;
    }
}

int dpcull_tree_destroy(dpcull_ctx c, dpcull_tree th)
{
  Tree* t = get_tree(c, th);
  if (!t) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad tree %u", th);
  tree_unbind_groups(c, th);
  cudaStreamSynchronize(c->stream);
  dfree(c, t->local, t->cap * 64);
  dfree(c, t->world, t->cap * 64);
  dfree(c, t->dirty_local, t->words * 4);
  dfree(c, t->dirty_world, t->words * 4);
  dfree(c, t->entries, t->entries_cap * 8);
  dfree(c, t->seg, t->seg_cap * 4);
  dfree(c, t->d_sched, t->sched_cap * sizeof(uint4));
  *t = Tree();
  return DPCULL_OK;
}

int dpcull_tree_resize(dpcull_ctx c, dpcull_tree th, size_t capacity)
{
  Tree* t = get_tree(c, th);
  if (!t) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad tree %u", th);
  if (capacity < t->cap || capacity > 0xFFFFFFFFull) return fail(DPCULL_ERR_INVALID_ARGUMENT, "capacity can only grow");
  if (capacity == t->cap) return DPCULL_OK;
  const size_t words = (capacity + 31) / 32;
  float *local = nullptr, *world = nullptr;
  uint32_t *dl = nullptr, *dw = nullptr;
  int rc = dalloc(c, (void**)&local, capacity * 64);
  if (!rc) rc = dalloc(c, (void**)&world, capacity * 64);
  if (!rc) rc = dalloc(c, (void**)&dl, words * 4);
  if (!rc) rc = dalloc(c, (void**)&dw, words * 4);
  if (rc) {
    dfree(c, local, capacity * 64);
    dfree(c, world, capacity * 64);
    dfree(c, dl, words * 4);
    return rc;
  }
  CU(cudaMemsetAsync(local, 0, capacity * 64, c->stream));
  CU(cudaMemsetAsync(world, 0, capacity * 64, c->stream));
  CU(cudaMemsetAsync(dl, 0, words * 4, c->stream));
  CU(cudaMemsetAsync(dw, 0, words * 4, c->stream));
  CU(cudaMemcpyAsync(local, t->local, t->cap * 64, cudaMemcpyDeviceToDevice, c->stream));
  CU(cudaMemcpyAsync(world, t->world, t->cap * 64, cudaMemcpyDeviceToDevice, c->stream));
  CU(cudaMemcpyAsync(dl, t->dirty_local, t->words * 4, cudaMemcpyDeviceToDevice, c->stream));
  CU(cudaMemcpyAsync(dw, t->dirty_world, t->words * 4, cudaMemcpyDeviceToDevice, c->stream));
  CU(cudaStreamSynchronize(c->stream));
  tree_unbind_groups(c, th);
  dfree(c, t->local, t->cap * 64);
  dfree(c, t->world, t->cap * 64);
  dfree(c, t->dirty_local, t->words * 4);
  dfree(c, t->dirty_world, t->words * 4);
  t->local = local;
  t->world = world;
  t->dirty_local = dl;
  t->dirty_world = dw;
  t->cap = capacity;
  t->words = words;
  return DPCULL_OK;
}

int dpcull_tree_set_structure(dpcull_ctx c, dpcull_tree th, size_t n_entries, const uint32_t* pairs,
                              size_t n_levels, const uint32_t* level_offsets)
{
  Tree* t = get_tree(c, th);
  if (!t) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad tree %u", th);
  if (n_entries && (!pairs || !level_offsets)) return fail(DPCULL_ERR_INVALID_ARGUMENT, "null arrays");
  if (n_levels && level_offsets[n_levels] != n_entries)
    return fail(DPCULL_ERR_INVALID_ARGUMENT, "level offsets do not cover the entries");
  for (size_t i = 0; i < 2 * n_entries; ++i)
    if (pairs[i] >= t->cap) return fail(DPCULL_ERR_OUT_OF_RANGE, "transform %u >= capacity %zu", pairs[i], t->cap);
  // Split each level into segments in which no entry reads a world matrix (or its dirty
  // bit) that another entry of the same segment writes.  The reference reads them in
  // list order, so a reader that follows its writer starts a new segment and a reader
  // that precedes it ends the segment before the writer.
  std::vector<uint32_t> seg;
  std::vector<uint8_t> written(t->cap, 0), read(t->cap, 0);
  std::vector<uint32_t> touched;
  for (size_t l = 0; l < n_levels; ++l) {
    const uint32_t b = level_offsets[l], e = level_offsets[l + 1];
    if (b > e || e > n_entries) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad level offsets");
    if (b == e) continue;
    seg.push_back(b);
    for (uint32_t i = b; i < e; ++i) {
      const uint32_t p = pairs[2 * i], x = pairs[2 * i + 1];
      if (written[p] || read[x] || written[x]) {
        seg.push_back(i);
        for (uint32_t k : touched) written[k] = read[k] = 0;
        touched.clear();
      }
      written[x] = 1;
      read[p] = 1;
      touched.push_back(x);
      touched.push_back(p);
    }
    for (uint32_t k : touched) written[k] = read[k] = 0;
    touched.clear();
  }
  seg.push_back((uint32_t)n_entries);
  // Launch schedule: runs of narrow segments share one single-CTA launch.
  const uint32_t kNarrow = 4096;
  t->schedule.clear();
  const size_t nseg = seg.size() - 1;
  size_t s = 0;
  while (s < nseg) {
    if (seg[s + 1] - seg[s] <= kNarrow) {
      size_t e = s;
      while (e < nseg && seg[e + 1] - seg[e] <= kNarrow) ++e;
      t->schedule.push_back({true, (uint32_t)s, (uint32_t)e});
      s = e;
    } else {
      t->schedule.push_back({false, seg[s], seg[s + 1]});
      ++s;
    }
  }
  if (n_entries > t->entries_cap) {
    dfree(c, t->entries, t->entries_cap * 8);
    t->entries = nullptr;
    int rc = dalloc(c, (void**)&t->entries, n_entries * 8);
    if (rc) return rc;
    t->entries_cap = n_entries;
  }
  if (seg.size() > t->seg_cap) {
    dfree(c, t->seg, t->seg_cap * 4);
    t->seg = nullptr;
    int rc = dalloc(c, (void**)&t->seg, seg.size() * 4);
    if (rc) return rc;
    t->seg_cap = seg.size();
  }
  // The cooperative kernel's schedule: block 0 takes runs of segments of at most 512
  // entries (two per thread), every wider segment is one grid step.
  const uint32_t kNarrowBlock = 512;
  std::vector<uint4> coop;
  t->max_wide = 0;
  for (size_t k = 0; k < nseg;) {
    if (seg[k + 1] - seg[k] <= kNarrowBlock) {
      size_t e = k;
      while (e < nseg && seg[e + 1] - seg[e] <= kNarrowBlock) ++e;
      coop.push_back(make_uint4(1u, (uint32_t)k, (uint32_t)e, 0u));
      k = e;
    } else {
      coop.push_back(make_uint4(0u, seg[k], seg[k + 1], 0u));
      t->max_wide = std::max(t->max_wide, seg[k + 1] - seg[k]);
      ++k;
    }
  }
  if (coop.size() > t->sched_cap) {
    dfree(c, t->d_sched, t->sched_cap * sizeof(uint4));
    t->d_sched = nullptr;
    int rc = dalloc(c, (void**)&t->d_sched, coop.size() * sizeof(uint4));
    if (rc) return rc;
    t->sched_cap = coop.size();
  }
  t->n_sched = (uint32_t)coop.size();
  if (n_entries) CU(cudaMemcpyAsync(t->entries, pairs, n_entries * 8, cudaMemcpyHostToDevice, c->stream));
  CU(cudaMemcpyAsync(t->seg, seg.data(), seg.size() * 4, cudaMemcpyHostToDevice, c->stream));
  if (!coop.empty())
    CU(cudaMemcpyAsync(t->d_sched, coop.data(), coop.size() * sizeof(uint4), cudaMemcpyHostToDevice, c->stream));
  CU(cudaStreamSynchronize(c->stream));
  return DPCULL_OK;
}

static int tree_scatter(dpcull_ctx c, Tree* t, float* dst, size_t k, const uint32_t* index,
                        const float* matrices, uint32_t* dirty)
{
  for (size_t i = 0; i < k; ++i)
    if (index[i] >= t->cap) return fail(DPCULL_ERR_OUT_OF_RANGE, "transform %u >= capacity %zu", index[i], t->cap);
  const void* src[2] = {matrices, index};
  const size_t bytes[2] = {64 * k, 4 * k};
  unsigned char* dev[2];
  int rc = stage_upload(c, 2, src, bytes, dev);
  if (rc) return rc;
  if (launch_scatter_matrices(dst, reinterpret_cast<float*>(dev[0]), reinterpret_cast<uint32_t*>(dev[1]),
                              (uint32_t)k, dirty, c->stream))
    return cuda_fail(cudaGetLastError(), "tree scatter");
  c->launches++;
  return DPCULL_OK;
}

int dpcull_tree_set_locals(dpcull_ctx c, dpcull_tree th, size_t k, const uint32_t* index, const float* m)
{
  Tree* t = get_tree(c, th);
  if (!t) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad tree %u", th);
  if (!k) return DPCULL_OK;
  if (!index || !m) return fail(DPCULL_ERR_INVALID_ARGUMENT, "null arrays");
  return tree_scatter(c, t, t->local, k, index, m, t->dirty_local);
}

int dpcull_tree_set_worlds(dpcull_ctx c, dpcull_tree th, size_t k, const uint32_t* index, const float* m)
{
  Tree* t = get_tree(c, th);
  if (!t) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad tree %u", th);
  if (!k) return DPCULL_OK;
  if (!index || !m) return fail(DPCULL_ERR_INVALID_ARGUMENT, "null arrays");
  int rc = tree_scatter(c, t, t->world, k, index, m, nullptr);
  return rc ? rc : tree_groups_stale(c, th);
}

int dpcull_tree_compute(dpcull_ctx c, dpcull_tree th)
{
  Tree* t = get_tree(c, th);
  if (!t) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad tree %u", th);
  XformLaunch a{t->entries, t->seg, t->local, t->world, t->dirty_local, t->dirty_world};
  // One cooperative launch for the whole tree (it clears both dirty bit arrays itself).
  if (t->words && launch_xform_tree(a, t->d_sched, t->n_sched, (uint32_t)t->words, t->max_wide, &c->ctl->bar_count,
                                    &c->ctl->error, c->sm_count, c->stream) == 0) {
    c->launches++;
    return tree_groups_stale(c, th);
  }
  cudaGetLastError();  // the device refused the cooperative launch: one launch per step
  CU(cudaMemsetAsync(t->dirty_world, 0, t->words * 4, c->stream));
  for (const TreeLaunch& L : t->schedule) {
    int rc = L.single_cta ? launch_xform_cta(a, L.a, L.b, c->stream)
                          : launch_xform_range(a, L.a, L.b, c->stream);
    if (rc) return cuda_fail(cudaGetLastError(), "tree launch");
    c->launches++;
  }
  CU(cudaMemsetAsync(t->dirty_local, 0, t->words * 4, c->stream));
  return tree_groups_stale(c, th);
}

int dpcull_tree_world_device(dpcull_ctx c, dpcull_tree th, const float** world, size_t* count)
{
  Tree* t = get_tree(c, th);
  if (!t || !world || !count) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad arguments");
  *world = t->world;
  *count = t->cap;
  return DPCULL_OK;
}

int dpcull_tree_world(dpcull_ctx c, dpcull_tree th, size_t first, size_t count, float* out)
{
  Tree* t = get_tree(c, th);
  if (!t || (count && !out)) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad arguments");
  if (first + count > t->cap) return fail(DPCULL_ERR_OUT_OF_RANGE, "range past capacity");
  if (count) CU(cudaMemcpyAsync(out, t->world + 16 * first, count * 64, cudaMemcpyDeviceToHost, c->stream));
  CU(cudaStreamSynchronize(c->stream));
  return DPCULL_OK;
}

int dpcull_tree_dirty_world(dpcull_ctx c, dpcull_tree th, uint32_t* words, size_t n_words)
{
  Tree* t = get_tree(c, th);
  if (!t || !words) return fail(DPCULL_ERR_INVALID_ARGUMENT, "bad arguments");
  const size_t k = std::min(n_words, t->words);
  CU(cudaMemcpyAsync(words, t->dirty_world, k * 4, cudaMemcpyDeviceToHost, c->stream));
  CU(cudaStreamSynchronize(c->stream));
  return DPCULL_OK;
}

}  // extern "C"
