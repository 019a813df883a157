// serve.cu -- culling service: device-resident scene pool with continuous batching.
//
// Threads: callers submit requests (any thread); one scheduler thread owns the scene
// pool and the streams.  Each scheduler turn
//   1. retires finished batches (event query): per-request visible counts (and kept
//      visibility words) come back in pinned memory, the scenes' in-flight counts drop;
//   2. if a stream is free, builds the next batch from the pending requests in arrival
//      order: a request whose scene is not on the device starts the scene's upload on
//      the upload stream (evicting least recently used scenes with no work in flight)
//      and stays pending until the upload's event has completed, so misses never delay
//      the hits batched with them; a request joins when its scene is on the device and
//      the batch's object-views stay under the cap; requests that cannot be admitted
//      yet stay pending and later ones go ahead;
//   3. launches the batch on that stream: descriptor upload, one persistent cull launch
//      over all (scene, view) pairs (the kernel of cull.cu with visibility words only),
//      and the copy back.
// Memory: scene buffers and per-batch outputs come from the device's stream-ordered
// pool (cudaMallocAsync / cudaFreeAsync), so eviction never synchronises the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <list>
#include <map>
#include <mutex>
#include <set>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/dpcull.h"
#include "dpcull_internal.h"

using namespace dpcull;

namespace {

constexpr uint32_t kMaxStreams = 8;
constexpr size_t kMaxBatchRequests = 4096;
// Descriptor buffer: the scenes of one batch, then (64-byte aligned) its views.
constexpr size_t kDescBytes = kMaxBatchRequests * sizeof(CullScene) + 64 +
                              kMaxBatchRequests * DPCULL_SERVER_MAX_VIEWS * sizeof(CullView);

double now_s()
{
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Scene {
  bool registered = false;
  size_t n = 0, cap = 0, n_mats = 0;
  const float* lower = nullptr;
  const float* extent = nullptr;
  const uint32_t* xform = nullptr;
  const float* mats = nullptr;
  float* dev = nullptr;          // 7 x cap rows, then n_mats x 16 floats
  const float* packed = nullptr; // the same layout in pinned host memory (shared)
  uint64_t bytes = 0;
  bool resident = false;
  bool uploading = false;        // upload issued, not yet seen complete: not evictable
  int pending = 0;               // batches in flight that use it
  uint64_t last_use = 0;
  cudaEvent_t ready = nullptr;   // recorded after the upload
  std::list<uint32_t>::iterator lru;  // position in the server's LRU list while resident
};

struct Request {
  uint64_t id;
  uint32_t scene, n_views, flags;
  float vps[DPCULL_SERVER_MAX_VIEWS * 16];
  double submit_s;
};

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  CullControl* ctl = nullptr;
  CullScene* d_scenes = nullptr;
  CullView* d_views = nullptr;
  CullScene* h_scenes = nullptr;  // pinned
  CullView* h_views = nullptr;    // pinned
  uint32_t* h_counts = nullptr;   // pinned, one per view
  bool busy = false;
  std::vector<Request> reqs;
  std::vector<Scene*> scn;        // the scene of each request, looked up under the scenes lock
  std::vector<size_t> bits_off;   // per request: word offset of its first view's bits
  uint32_t* d_out = nullptr;
  size_t out_bytes = 0;
  double start_s = 0;
  struct Kept {
    uint64_t id;
    std::vector<uint32_t> words;
  };
  std::vector<Kept> kept;         // pinned copies are staged through `kept_pinned`
  uint32_t* kept_pinned = nullptr;
  size_t kept_cap = 0;            // words
};

}  // namespace

struct dpcull_server_s {
  dpcull_ctx ctx = nullptr;
  int device = 0, sm_count = 0;
  uint64_t budget = 0, max_batch = 0;
  uint32_t n_streams = 0;
  Slot slots[kMaxStreams];

  std::mutex scenes_mu;      // residency state; the worker holds it across CUDA calls
  // Scenes by id.  dpcull_server_add_scene may grow the deque at any time (under
  // scenes_mu): references to its elements stay valid, but indexing it is only safe under
  // the lock, so the worker indexes it under the lock and keeps Scene pointers.
  std::deque<Scene> scenes;
  std::list<uint32_t> lru;   // resident scenes, least recently used first
  cudaStream_t up_stream = nullptr;  // scene uploads and evictions
  // What a submit checks (registered, size), under a lock the worker never takes, so a
  // submit never waits on the worker's uploads or evictions.
  struct SceneInfo {
    bool registered = false;
    uint64_t bytes = 0;
    size_t cap = 0;
  };
  std::mutex info_mu;
  std::vector<SceneInfo> info;
  std::map<std::pair<const void*, size_t>, uint32_t> max_index;
  // Pinned copies in the device layout, one per distinct set of host arrays.
  std::map<std::tuple<const void*, const void*, const void*, const void*, size_t>, float*> packed;

  std::mutex pending_mu;
  std::condition_variable pending_cv;
  std::deque<Request> pending;
  uint64_t next_id = 1;

  std::mutex done_mu;
  std::vector<dpcull_completion> done;
  std::unordered_map<uint64_t, std::vector<std::vector<uint32_t>>> results;

  uint64_t resident_bytes = 0, inflight_bytes = 0, uploading_bytes = 0, tick = 0;
  std::atomic<uint64_t> submitted{0}, completed{0};
  dpcull_server_stats stats{};
  std::atomic<bool> stop{false};
  std::thread worker;
  int error = DPCULL_OK;
};

namespace {

int vpp_for(uint32_t max_views)
{
  return max_views <= 1 ? 1 : max_views <= 2 ? 2 : max_views <= 4 ? 4 : 8;
}

uint64_t us_since(double t0) { return (uint64_t)((now_s() - t0) * 1e6); }

void evict(dpcull_server s, Scene& sc)
{
  const double t0 = now_s();
  // Every batch that read the scene has retired (pending == 0), so its memory is free to
  // go back to the pool in upload-stream order.
  cudaFreeAsync(sc.dev, s->up_stream);
  sc.dev = nullptr;
  sc.resident = false;
  s->lru.erase(sc.lru);
  s->resident_bytes -= sc.bytes;
  s->stats.scene_evictions++;
  s->stats.max_evict_call_us = std::max(s->stats.max_evict_call_us, us_since(t0));
}

// Makes room for `need` more bytes, evicting least recently used idle scenes.  With
// `take_uploaded`, a scene whose upload finished but whose requests are still queued may
// go too (they upload it again): admitting a ready request then never waits on uploads
// that wait on admissions.
bool make_room(dpcull_server s, uint64_t need, bool take_uploaded)
{
  while (s->resident_bytes + s->inflight_bytes + need > s->budget) {
    Scene* victim = nullptr;
    for (uint32_t id : s->lru) {
      Scene& sc = s->scenes[id];
      if (sc.pending != 0) continue;
      if (!sc.uploading || (take_uploaded && cudaEventQuery(sc.ready) == cudaSuccess)) {
        victim = &sc;
        break;
      }
    }
    if (!victim) return false;
    if (victim->uploading) {
      victim->uploading = false;
      s->uploading_bytes -= victim->bytes;
    }
    evict(s, *victim);
  }
  return true;
}

// Starts the upload of a scene on the upload stream (one copy from its pinned image).
void upload(dpcull_server s, Scene& sc, uint32_t id)
{
  const double t0 = now_s();
  cudaMallocAsync((void**)&sc.dev, sc.bytes, s->up_stream);
  cudaMemcpyAsync(sc.dev, sc.packed, sc.bytes, cudaMemcpyHostToDevice, s->up_stream);
  if (!sc.ready) cudaEventCreateWithFlags(&sc.ready, cudaEventDisableTiming);
  cudaEventRecord(sc.ready, s->up_stream);
  sc.resident = true;
  sc.uploading = true;
  s->uploading_bytes += sc.bytes;
  sc.lru = s->lru.insert(s->lru.end(), id);
  s->resident_bytes += sc.bytes;
  s->stats.scene_uploads++;
  s->stats.upload_bytes += sc.bytes;
  s->stats.max_upload_call_us = std::max(s->stats.max_upload_call_us, us_since(t0));
}

void retire(dpcull_server s, Slot& slot)
{
  const double t = now_s();
  std::vector<dpcull_completion> out;
  size_t v0 = 0;
  for (size_t i = 0; i < slot.reqs.size(); ++i) {
    const Request& q = slot.reqs[i];
    Scene& sc = *slot.scn[i];
    sc.pending--;
    dpcull_completion c{};
    c.request = q.id;
    c.scene = q.scene;
    c.n_views = q.n_views;
    for (uint32_t v = 0; v < q.n_views; ++v) c.visible[v] = slot.h_counts[v0 + v];
    c.objects = sc.n;
    c.submit_s = q.submit_s;
    c.start_s = slot.start_s;
    c.done_s = t;
    c.status = DPCULL_OK;
    out.push_back(c);
    v0 += q.n_views;
  }
  {
    std::lock_guard<std::mutex> lk(s->done_mu);
    for (auto& k : slot.kept) {
      auto it = std::find_if(slot.reqs.begin(), slot.reqs.end(), [&](const Request& r) { return r.id == k.id; });
      const Request& q = *it;
      const size_t words = slot.scn[it - slot.reqs.begin()]->cap / 32;
      std::vector<std::vector<uint32_t>> views(q.n_views);
      for (uint32_t v = 0; v < q.n_views; ++v)
        views[v].assign(k.words.begin() + v * words, k.words.begin() + (v + 1) * words);
      s->results[q.id] = std::move(views);
    }
    s->done.insert(s->done.end(), out.begin(), out.end());
  }
  s->inflight_bytes -= slot.out_bytes;
  s->completed += slot.reqs.size();
  slot.reqs.clear();
  slot.scn.clear();
  slot.kept.clear();
  slot.busy = false;
}

void copy_kept(Slot& slot)
{
  // After the event: the kept visibility words were staged in kept_pinned.
  size_t off = 0;
  for (auto& k : slot.kept) {
    std::memcpy(k.words.data(), slot.kept_pinned + off, k.words.size() * 4);
    off += k.words.size();
  }
}

// Starts the uploads of scenes that requests found missing (after the turn's batch went
// out, so no hit waits on these calls).  At most half the budget is in uploads that no
// batch has taken yet (any one scene may upload alone), and at most kUploadsPerTurn start
// per turn, so a burst of misses does not hold the scheduler from its next batch (the
// requests of the others stay pending and ask again next turn).
constexpr int kUploadsPerTurn = 8;
void start_uploads(dpcull_server s, const std::vector<uint32_t>& missing)
{
  if (missing.empty()) return;
  std::lock_guard<std::mutex> lk(s->scenes_mu);
  int started = 0;
  for (uint32_t id : missing) {
    if (started == kUploadsPerTurn) break;
    Scene& sc = s->scenes[id];
    if (sc.resident) continue;  // two requests of this turn wanted it
    if ((s->uploading_bytes == 0 || s->uploading_bytes + sc.bytes <= s->budget / 2) &&
        make_room(s, sc.bytes, false)) {
      upload(s, sc, id);
      ++started;
    }
  }
}

bool launch(dpcull_server s, Slot& slot)
{
  std::vector<Request> take;
  std::vector<Scene*> take_sc;  // Scene of each taken request (stable while the server lives)
  std::vector<uint32_t> missing;
  uint64_t work = 0, out_bytes = 0;
  uint32_t max_views = 1;
  // Take the pending requests out under the lock, decide outside it (submitters never
  // wait on CUDA calls), and put the ones not admitted back in front, in order.
  std::deque<Request> cand;
  {
    std::lock_guard<std::mutex> lk(s->pending_mu);
    cand.swap(s->pending);
  }
  std::deque<Request> left;
  {
    std::lock_guard<std::mutex> lk2(s->scenes_mu);
    bool full = false;
    for (auto& q : cand) {
      Scene& sc = s->scenes[q.scene];
      // A scene that is not on the device yet gets its upload started after this turn's
      // batch and its requests wait in the queue; the batch goes ahead with the scenes
      // that are ready, so a miss never holds up the hits of the same batch.
      if (!sc.resident) {
        missing.push_back(q.scene);
        left.push_back(q);
        continue;
      }
      if (sc.uploading && cudaEventQuery(sc.ready) != cudaSuccess) {
        left.push_back(q);
        continue;
      }
      const uint64_t w = (uint64_t)sc.n * q.n_views;
      if (full || take.size() >= kMaxBatchRequests || (!take.empty() && work + w > s->max_batch)) {
        full = true;
        left.push_back(q);
        continue;
      }
      const uint64_t ob = (uint64_t)q.n_views * (sc.cap / 8 + 4) + 256;  // >= its share of d_out
      sc.pending++;  // not a victim of its own admission
      const bool room = make_room(s, ob, true);
      sc.pending--;
      if (!room) {
        left.push_back(q);  // cannot be admitted yet: later requests may go ahead
        continue;
      }
      if (sc.uploading) {
        sc.uploading = false;
        s->uploading_bytes -= sc.bytes;
      }
      sc.pending++;
      sc.last_use = ++s->tick;
      s->lru.splice(s->lru.end(), s->lru, sc.lru);  // most recently used
      s->inflight_bytes += ob;
      out_bytes += ob;
      work += w;
      max_views = std::max(max_views, q.n_views);
      take.push_back(q);
      take_sc.push_back(&sc);
    }
  }
  if (!left.empty()) {
    std::lock_guard<std::mutex> lk(s->pending_mu);
    s->pending.insert(s->pending.begin(), left.begin(), left.end());
  }
  if (take.empty()) {
    start_uploads(s, missing);
    return false;
  }

  // Every scene of the batch was seen uploaded (its event complete) before admission.
  size_t n_views = 0;
  for (auto& q : take) n_views += q.n_views;
  cudaMallocAsync((void**)&slot.d_out, out_bytes, slot.stream);
  slot.out_bytes = out_bytes;
  uint32_t* counts = slot.d_out;  // one word per view, then the words of each view
  size_t words_off = (n_views + 63) / 64 * 64;
  cudaMemsetAsync(counts, 0, n_views * 4, slot.stream);

  const int vpp = vpp_for(max_views);
  uint64_t tile_groups = 0;
  for (size_t i = 0; i < take.size(); ++i)
    tile_groups += (take_sc[i]->cap / kTileObjects) * (uint64_t)((take[i].n_views + vpp - 1) / vpp);
  const uint32_t item_tiles = item_tiles_for(tile_groups, s->sm_count);
  uint32_t items = 0, max_tiles = 1, vi = 0;
  size_t kept_words = 0;
  slot.bits_off.clear();
  slot.kept.clear();
  // Scenes and views share one descriptor buffer (views right after this batch's
  // scenes), so they go up in one copy.
  const size_t voff = (take.size() * sizeof(CullScene) + 63) / 64 * 64;
  slot.h_views = reinterpret_cast<CullView*>(reinterpret_cast<char*>(slot.h_scenes) + voff);
  slot.d_views = reinterpret_cast<CullView*>(reinterpret_cast<char*>(slot.d_scenes) + voff);
  for (size_t i = 0; i < take.size(); ++i) {
    const Request& q = take[i];
    const Scene& sc = *take_sc[i];
    CullScene cs{};
    cs.soa = sc.dev;
    cs.mats = sc.dev + 7 * sc.cap;
    cs.cap = (uint32_t)sc.cap;
    cs.n_objects = (uint32_t)sc.n;
    cs.n_mats = (uint32_t)sc.n_mats;
    cs.view_begin = vi;
    cs.n_views = q.n_views;
    cs.n_vgroups = (q.n_views + vpp - 1) / vpp;
    cs.n_tiles = (uint32_t)(sc.cap / kTileObjects);
    cs.n_big = (cs.n_tiles + item_tiles - 1) / item_tiles;  // every item item_tiles long
    cs.item_begin = items;
    items += items_of(cs.n_tiles, cs.n_vgroups, item_tiles);
    max_tiles = std::max(max_tiles, cs.n_tiles);
    slot.h_scenes[i] = cs;
    slot.bits_off.push_back(words_off);
    for (uint32_t v = 0; v < q.n_views; ++v, ++vi) {
      CullView cv{};
      std::memcpy(cv.vp, q.vps + 16 * v, 64);
      cv.bits = slot.d_out + words_off + v * (sc.cap / 32);
      cv.flags = kViewNoChanged;
      cv.n_visible = counts + vi;
      cv.n_words = cs.n_tiles * kTileWords;
      slot.h_views[vi] = cv;
    }
    if (q.flags & DPCULL_REQUEST_KEEP_BITS) {
      slot.kept.push_back({q.id, std::vector<uint32_t>(q.n_views * (sc.cap / 32))});
      kept_words += q.n_views * (sc.cap / 32);
    }
    words_off += q.n_views * (sc.cap / 32);
  }
  cudaMemcpyAsync(slot.d_scenes, slot.h_scenes, voff + n_views * sizeof(CullView), cudaMemcpyHostToDevice,
                  slot.stream);
  CullLaunch a{};
  a.scenes = slot.d_scenes;
  a.views = slot.d_views;
  a.n_scenes = (uint32_t)take.size();
  a.n_items = items;
  a.item_tiles = item_tiles;
  a.items_per_ticket = 1;
  a.wide_mats = 1;  // 256-bit matrix loads only if every scene's array allows them
  for (size_t i = 0; i < take.size(); ++i)
    if ((uintptr_t)slot.h_scenes[i].mats & 31u) a.wide_mats = 0;
  a.ctl = slot.ctl;
  const int occ = cull_max_ctas_per_sm(vpp, kCacheNone);  // served scenes keep no box cache
  const long long want = ((long long)items + kWarpsPerCta - 1) / kWarpsPerCta;  // a warp per item
  const int grid = (int)std::max<long long>(1, std::min<long long>((long long)s->sm_count * occ, want));
  launch_cull(a, grid, vpp, slot.stream);
  cudaMemcpyAsync(slot.h_counts, counts, n_views * 4, cudaMemcpyDeviceToHost, slot.stream);
  if (kept_words) {
    if (kept_words > slot.kept_cap) {
      if (slot.kept_pinned) cudaFreeHost(slot.kept_pinned);
      cudaMallocHost((void**)&slot.kept_pinned, kept_words * 4);
      slot.kept_cap = kept_words;
    }
    size_t off = 0;
    for (size_t i = 0; i < take.size(); ++i)
      if (take[i].flags & DPCULL_REQUEST_KEEP_BITS) {
        const size_t w = take[i].n_views * (take_sc[i]->cap / 32);
        cudaMemcpyAsync(slot.kept_pinned + off, slot.d_out + slot.bits_off[i], w * 4, cudaMemcpyDeviceToHost, slot.stream);
        off += w;
      }
  }
  cudaFreeAsync(slot.d_out, slot.stream);
  slot.d_out = nullptr;
  cudaEventRecord(slot.done, slot.stream);
  slot.reqs = std::move(take);
  slot.scn = std::move(take_sc);
  slot.start_s = now_s();
  slot.busy = true;
  s->stats.batches++;
  s->stats.max_batch_requests = std::max<uint64_t>(s->stats.max_batch_requests, slot.reqs.size());
  if (cudaGetLastError() != cudaSuccess) s->error = DPCULL_ERR_CUDA;
  start_uploads(s, missing);
  return true;
}

void worker_main(dpcull_server s)
{
  cudaSetDevice(s->device);
  while (!s->stop.load()) {
    const double turn0 = now_s();
    bool progress = false;
    for (uint32_t i = 0; i < s->n_streams; ++i) {
      Slot& slot = s->slots[i];
      if (slot.busy && cudaEventQuery(slot.done) == cudaSuccess) {
        copy_kept(slot);
        retire(s, slot);
        progress = true;
      }
    }
    for (uint32_t i = 0; i < s->n_streams; ++i) {
      Slot& slot = s->slots[i];
      if (!slot.busy) {
        bool have;
        {
          std::lock_guard<std::mutex> lk(s->pending_mu);
          have = !s->pending.empty();
        }
        if (have && launch(s, slot)) progress = true;
        break;  // at most one new batch per turn, so that arrivals can join the next one
      }
    }
    const uint64_t turn_us = us_since(turn0);
    s->stats.max_turn_us = std::max(s->stats.max_turn_us, turn_us);
    if (turn_us > 1000) s->stats.slow_turns++;
    if (!progress) {
      bool busy = false;
      for (uint32_t i = 0; i < s->n_streams; ++i) busy |= s->slots[i].busy;
      std::unique_lock<std::mutex> lk(s->pending_mu);
      // Requests waiting for uploads are polled like batches in flight.
      if (busy || !s->pending.empty()) s->pending_cv.wait_for(lk, std::chrono::microseconds(5));
      else s->pending_cv.wait_for(lk, std::chrono::microseconds(200), [&] { return !s->pending.empty() || s->stop.load(); });
    }
  }
}

}  // namespace

extern "C" {

double dpcull_server_now(void) { return now_s(); }

int dpcull_server_create(dpcull_ctx ctx, uint64_t budget_bytes, uint32_t n_streams,
                         uint64_t max_batch_objects, dpcull_server* out)
{
  if (!ctx || !out || !n_streams || n_streams > kMaxStreams || !budget_bytes)
    return record_error(DPCULL_ERR_INVALID_ARGUMENT, "dpcull_server_create: bad arguments");
  dpcull_server s = new dpcull_server_s();
  s->ctx = ctx;
  ctx_info(ctx, &s->device, &s->sm_count);
  cudaSetDevice(s->device);
  s->budget = budget_bytes;
  s->max_batch = max_batch_objects ? max_batch_objects : (64ull << 20);
  s->n_streams = n_streams;
  s->stats.budget_bytes = budget_bytes;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, s->device) == cudaSuccess) {
    uint64_t keep = ~0ull;  // keep freed blocks for reuse instead of returning them
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    // Map the budget into the pool now (allocate and free it once), so that uploads
    // never wait for the pool to grow while requests are being served.  Best effort:
    // without the memory the pool grows on demand.
    void* reserve = nullptr;
    if (cudaMallocAsync(&reserve, budget_bytes, 0) == cudaSuccess) {
      cudaFreeAsync(reserve, 0);
      cudaStreamSynchronize(0);
      s->stats.reserved_bytes = budget_bytes;
    }
    cudaGetLastError();
  }
  if (cudaStreamCreateWithFlags(&s->up_stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    s->n_streams = 0;
    dpcull_server_destroy(s);
    return record_error(DPCULL_ERR_CUDA, "dpcull_server_create: stream set-up failed");
  }
  for (uint32_t i = 0; i < n_streams; ++i) {
    Slot& sl = s->slots[i];
    bool ok = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) == cudaSuccess &&
              cudaMalloc((void**)&sl.ctl, sizeof(CullControl)) == cudaSuccess &&
              cudaMemset(sl.ctl, 0, sizeof(CullControl)) == cudaSuccess &&
              cudaMalloc((void**)&sl.d_scenes, kDescBytes) == cudaSuccess &&
              cudaMallocHost((void**)&sl.h_scenes, kDescBytes) == cudaSuccess &&
              cudaMallocHost((void**)&sl.h_counts, kMaxBatchRequests * DPCULL_SERVER_MAX_VIEWS * 4) == cudaSuccess;
    if (!ok) {
      cudaGetLastError();
      s->n_streams = i + 1;
      dpcull_server_destroy(s);
      return record_error(DPCULL_ERR_NO_MEMORY, "dpcull_server_create: stream set-up failed");
    }
  }
  s->worker = std::thread(worker_main, s);
  *out = s;
  return DPCULL_OK;
}

int dpcull_server_destroy(dpcull_server s)
{
  if (!s) return record_error(DPCULL_ERR_INVALID_ARGUMENT, "null server");
  s->stop = true;
  s->pending_cv.notify_all();
  if (s->worker.joinable()) s->worker.join();
  cudaSetDevice(s->device);
  for (uint32_t i = 0; i < s->n_streams; ++i) {
    Slot& sl = s->slots[i];
    if (sl.stream) cudaStreamSynchronize(sl.stream);
  }
  if (s->up_stream) cudaStreamSynchronize(s->up_stream);
  for (auto& sc : s->scenes) {
    if (sc.dev) cudaFree(sc.dev);
    if (sc.ready) cudaEventDestroy(sc.ready);
  }
  if (s->up_stream) cudaStreamDestroy(s->up_stream);
  for (uint32_t i = 0; i < s->n_streams; ++i) {
    Slot& sl = s->slots[i];
    if (sl.stream) cudaStreamSynchronize(sl.stream);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.stream) cudaStreamDestroy(sl.stream);
    cudaFree(sl.ctl);
    cudaFree(sl.d_scenes);
    if (sl.h_scenes) cudaFreeHost(sl.h_scenes);
    if (sl.h_counts) cudaFreeHost(sl.h_counts);
    if (sl.kept_pinned) cudaFreeHost(sl.kept_pinned);
  }
  for (auto& kv : s->packed) cudaFreeHost(kv.second);
  delete s;
  return DPCULL_OK;
}

int dpcull_server_add_scene(dpcull_server s, uint32_t scene, size_t n, const float* lower,
                            const float* extent, const uint32_t* xform, const float* matrices,
                            size_t n_matrices)
{
  if (!s || !n || !lower || !extent || !xform || !matrices || !n_matrices || n > kMaxObjects)
    return record_error(DPCULL_ERR_INVALID_ARGUMENT, "dpcull_server_add_scene: bad arguments");
  std::lock_guard<std::mutex> lk(s->scenes_mu);
  // Index validation, once per (index array, length): catalogues share arrays.
  auto key = std::make_pair(static_cast<const void*>(xform), n);
  auto it = s->max_index.find(key);
  if (it == s->max_index.end()) {
    uint32_t m = 0;
    for (size_t i = 0; i < n; ++i) m = std::max(m, xform[i]);
    it = s->max_index.emplace(key, m).first;
  }
  if (it->second >= n_matrices)
    return record_error(DPCULL_ERR_OUT_OF_RANGE, "dpcull_server_add_scene: transform index past the matrices");
  if (scene >= s->scenes.size()) {
    if (scene > 16u * 1024u * 1024u) return record_error(DPCULL_ERR_INVALID_ARGUMENT, "scene id too large");
    // Growing the deque keeps every Scene where it is: the worker's Scene pointers stay
    // valid, and it only indexes the deque under this lock.
    s->scenes.resize(scene + 1);
  }
  Scene& sc = s->scenes[scene];
  if (sc.registered) return record_error(DPCULL_ERR_STATE, "dpcull_server_add_scene: scene already added");
  sc.registered = true;
  sc.n = n;
  sc.cap = (n + kTileObjects - 1) / kTileObjects * kTileObjects;
  sc.n_mats = n_matrices;
  sc.lower = lower;
  sc.extent = extent;
  sc.xform = xform;
  sc.mats = matrices;
  sc.bytes = ((7 * sc.cap * 4 + 16 * n_matrices * 4) + 255) & ~size_t(255);
  // One pinned copy in the device layout per distinct set of arrays: an upload is then a
  // single asynchronous copy.
  const auto pkey = std::make_tuple(static_cast<const void*>(lower), static_cast<const void*>(extent),
                                    static_cast<const void*>(xform), static_cast<const void*>(matrices), n);
  auto pk = s->packed.find(pkey);
  if (pk == s->packed.end()) {
    float* p = nullptr;
    if (cudaMallocHost((void**)&p, sc.bytes) != cudaSuccess) {
      cudaGetLastError();
      sc.registered = false;
      return record_error(DPCULL_ERR_NO_MEMORY, "dpcull_server_add_scene: pinned staging allocation failed");
    }
    std::memset(p, 0, sc.bytes);
    for (int r = 0; r < 3; ++r) {
      std::memcpy(p + r * sc.cap, lower + r * n, n * 4);
      std::memcpy(p + (3 + r) * sc.cap, extent + r * n, n * 4);
    }
    std::memcpy(p + 6 * sc.cap, xform, n * 4);
    std::memcpy(p + 7 * sc.cap, matrices, n_matrices * 64);
    pk = s->packed.emplace(pkey, p).first;
  }
  sc.packed = pk->second;
  {
    std::lock_guard<std::mutex> li(s->info_mu);
    if (scene >= s->info.size()) s->info.resize(scene + 1);
    s->info[scene] = dpcull_server_s::SceneInfo{true, sc.bytes, sc.cap};
  }
  return DPCULL_OK;
}

int dpcull_server_submit(dpcull_server s, uint32_t scene, uint32_t n_views, const float* vps,
                         uint32_t flags, uint64_t* request)
{
  if (!s || !vps || !n_views || n_views > DPCULL_SERVER_MAX_VIEWS)
    return record_error(DPCULL_ERR_INVALID_ARGUMENT, "dpcull_server_submit: 1..8 views");
  {
    std::lock_guard<std::mutex> lk(s->info_mu);
    if (scene >= s->info.size() || !s->info[scene].registered)
      return record_error(DPCULL_ERR_INVALID_ARGUMENT, "dpcull_server_submit: unknown scene");
    const auto& sc = s->info[scene];
    if (sc.bytes + n_views * (sc.cap / 8 + 4) > s->budget)
      return record_error(DPCULL_ERR_CAPACITY, "dpcull_server_submit: the scene does not fit the budget");
  }
  Request q{};
  q.scene = scene;
  q.n_views = n_views;
  q.flags = flags;
  std::memcpy(q.vps, vps, (size_t)n_views * 64);
  q.submit_s = now_s();
  {
    std::lock_guard<std::mutex> lk(s->pending_mu);
    q.id = s->next_id++;
    s->pending.push_back(q);
  }
  s->submitted++;
  s->pending_cv.notify_one();
  if (request) *request = q.id;
  return DPCULL_OK;
}

int dpcull_server_poll(dpcull_server s, dpcull_completion* out, size_t cap, size_t* n)
{
  if (!s || !n) return record_error(DPCULL_ERR_INVALID_ARGUMENT, "null argument");
  std::lock_guard<std::mutex> lk(s->done_mu);
  const size_t k = std::min(cap, s->done.size());
  if (k && out) std::memcpy(out, s->done.data(), k * sizeof(dpcull_completion));
  s->done.erase(s->done.begin(), s->done.begin() + k);
  *n = k;
  return s->error;
}

int dpcull_server_result(dpcull_server s, uint64_t request, uint32_t view, uint32_t* words,
                         size_t n_words)
{
  if (!s || !words) return record_error(DPCULL_ERR_INVALID_ARGUMENT, "null argument");
  std::lock_guard<std::mutex> lk(s->done_mu);
  auto it = s->results.find(request);
  if (it == s->results.end() || view >= it->second.size())
    return record_error(DPCULL_ERR_STATE, "no kept result for this request / view");
  const auto& w = it->second[view];
  if (n_words < w.size()) return record_error(DPCULL_ERR_CAPACITY, "buffer too small");
  std::memcpy(words, w.data(), w.size() * 4);
  return DPCULL_OK;
}

int dpcull_server_release(dpcull_server s, uint64_t request)
{
  if (!s) return record_error(DPCULL_ERR_INVALID_ARGUMENT, "null server");
  std::lock_guard<std::mutex> lk(s->done_mu);
  s->results.erase(request);
  return DPCULL_OK;
}

int dpcull_server_drain(dpcull_server s)
{
  if (!s) return record_error(DPCULL_ERR_INVALID_ARGUMENT, "null server");
  const auto t0 = std::chrono::steady_clock::now();
  while (s->completed.load() < s->submitted.load()) {
    std::this_thread::sleep_for(std::chrono::microseconds(20));
    if (std::chrono::steady_clock::now() - t0 > std::chrono::seconds(120))
      return record_error(DPCULL_ERR_TIMEOUT, "dpcull_server_drain: requests did not complete");
  }
  return s->error;
}

int dpcull_server_get_stats(dpcull_server s, dpcull_server_stats* out)
{
  if (!s || !out) return record_error(DPCULL_ERR_INVALID_ARGUMENT, "null argument");
  dpcull_server_stats st = s->stats;
  st.requests_submitted = s->submitted.load();
  st.requests_completed = s->completed.load();
  st.resident_bytes = s->resident_bytes;
  uint64_t rs = 0;
  {
    std::lock_guard<std::mutex> lk(s->scenes_mu);
    for (auto& sc : s->scenes) rs += sc.resident;
  }
  st.resident_scenes = rs;
  {
    std::lock_guard<std::mutex> lk(s->pending_mu);
    st.pending_requests = s->pending.size();
  }
  *out = st;
  return DPCULL_OK;
}

}  // extern "C"
