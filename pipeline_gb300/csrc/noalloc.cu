// noalloc.cu -- dpcull_cull_noalloc: the plain cull for callers that cannot allocate.
//
// Some callers of a culling backend may not allocate device memory at the point where
// they cull: a renderer's frame loop cannot afford cudaMalloc's implicit device-wide
// synchronisation in the middle of a frame, and a process whose device memory is
// entirely owned by another allocator (a framework's caching allocator, or a fixed
// budget reserved up front) has none to give.  The regular entry points allocate their
// result buffers and the cull's scratch lazily, so they are unusable there.  This entry
// point runs the same cull kernel and the same changed-list assembly on buffers the
// caller owns, and takes its scratch (the delta words of the changed list, the changed-list
// pass's per-chunk counts, ticket and block count, and the cull's control block) from one
// statically sized device array defined below.  It calls no cudaMalloc, cudaFree or other allocating routine.
//
// The array lives in every GPU that loads this library until the process exits
// (about 128 KB).  Its device address is looked up once per device, with that device
// current, on the first call made on the device, and kept for the life of the process.
// Every call blocks until its work is done (cudaStreamSynchronize, then a copy to host
// memory), so no call can be made inside a stream capture.  cudaDeviceReset destroys the array
// together with the device's context, so after a reset of a device this entry point
// must not be called on it again in the same process (the kept address would name
// memory of the old context).  All calls share the array and it keeps the last call's
// contents: each call clears the parts that must start at zero, and calls whose work
// overlaps on the GPU (on different streams, or on one stream from several host threads
// without ordering) race on it.  Each call waits for its own work on the stream
// (cudaStreamSynchronize) before it returns.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>

#include "../../include/dpcull.h"
#include "dpcull_internal.h"

namespace dpcull {
namespace {

constexpr size_t kNoallocWords = DPCULL_NOALLOC_MAX_OBJECTS / 32;
constexpr size_t kDeltaBytes = kNoallocWords * sizeof(uint32_t);
constexpr size_t kChunkOffset = kDeltaBytes;
constexpr size_t kCtlOffset = kChunkOffset + ((chunks_of(kNoallocWords) + 2) * sizeof(uint32_t) + 255) / 256 * 256;
constexpr size_t kScratchBytes = kCtlOffset + 256;
static_assert(DPCULL_NOALLOC_MAX_OBJECTS % kTileObjects == 0, "whole tiles");

// The scratch: delta words | chunk counts | control block.
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_lock;
unsigned char* g_scratch_dev[kMaxDevices] = {};

int noalloc_fail(int code, const char* msg) { return record_error(code, msg); }

// Device address of g_scratch on the current device (host code cannot use the symbol).
int scratch_address(int device, unsigned char** out)
{
  std::lock_guard<std::mutex> lock(g_lock);
  if (!g_scratch_dev[device]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) {
      cudaGetLastError();
      return DPCULL_ERR_CUDA;
    }
    g_scratch_dev[device] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_dev[device];
  return DPCULL_OK;
}

}  // namespace
}  // namespace dpcull

using namespace dpcull;

extern "C" int dpcull_cull_noalloc(const float* objects, size_t cap, size_t n, const float* matrices,
                                   size_t n_matrices, const float vp[16], uint32_t* bits,
                                   uint32_t* changed, uint32_t* n_changed, void* stream)
{
  if (n > DPCULL_NOALLOC_MAX_OBJECTS)
    return noalloc_fail(DPCULL_ERR_CAPACITY, "dpcull_cull_noalloc: more objects than DPCULL_NOALLOC_MAX_OBJECTS");
  if (!vp || !n_changed || (n && (!objects || !matrices || !bits || !changed)))
    return noalloc_fail(DPCULL_ERR_INVALID_ARGUMENT, "dpcull_cull_noalloc: null pointer");
  if (cap % kTileObjects || cap < n || n_matrices > 0xFFFFFFFFull)
    return noalloc_fail(DPCULL_ERR_INVALID_ARGUMENT,
                        "dpcull_cull_noalloc: cap must be a multiple of 128 and at least n");
  if (((uintptr_t)objects & 15) || ((uintptr_t)matrices & 15))
    return noalloc_fail(DPCULL_ERR_INVALID_ARGUMENT, "dpcull_cull_noalloc: objects and matrices must be 16-byte aligned");
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kMaxDevices) {
    cudaGetLastError();
    return noalloc_fail(DPCULL_ERR_CUDA, "dpcull_cull_noalloc: no current CUDA device");
  }
  unsigned char* s = nullptr;
  if (scratch_address(device, &s) != DPCULL_OK)
    return noalloc_fail(DPCULL_ERR_CUDA, "dpcull_cull_noalloc: cudaGetSymbolAddress failed");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CullControl* ctl = reinterpret_cast<CullControl*>(s + kCtlOffset);
  // The changed-list pass's counts, the ticket, CTA counter and error word must start at
  // zero (the counts end every call at zero; cleared here all the same).
  if (cudaMemsetAsync(s + kChunkOffset, 0, kCtlOffset - kChunkOffset + sizeof(CullControl), st) != cudaSuccess) {
    cudaGetLastError();
    return noalloc_fail(DPCULL_ERR_CUDA, "dpcull_cull_noalloc: cudaMemsetAsync failed");
  }
  if (n == 0) {
    if (cudaMemsetAsync(n_changed, 0, sizeof(uint32_t), st) != cudaSuccess) {
      cudaGetLastError();
      return noalloc_fail(DPCULL_ERR_CUDA, "dpcull_cull_noalloc: cudaMemsetAsync failed");
    }
    return cudaStreamSynchronize(st) == cudaSuccess ? DPCULL_OK : DPCULL_ERR_CUDA;
  }
  const uint32_t tiles = (uint32_t)((n + kTileObjects - 1) / kTileObjects);
  CullLaunch a{};
  a.n_scenes = 1;
  a.items_per_ticket = 1;
  a.ctl = ctl;
  a.one_scene.soa = objects;
  a.one_scene.mats = matrices;
  a.one_scene.cap = (uint32_t)cap;
  a.one_scene.n_objects = (uint32_t)n;
  a.one_scene.n_mats = (uint32_t)n_matrices;
  a.one_scene.n_views = 1;
  a.one_scene.n_vgroups = 1;
  a.one_scene.n_tiles = tiles;
  std::memcpy(a.one_view.vp, vp, sizeof a.one_view.vp);
  a.one_view.bits = bits;
  a.one_view.changed = changed;
  a.one_view.n_changed = n_changed;
  a.one_view.delta = reinterpret_cast<uint32_t*>(s);
  a.one_view.chunk_tot = reinterpret_cast<uint32_t*>(s + kChunkOffset);
  a.one_view.n_words = tiles * kTileWords;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  a.item_tiles = item_tiles_for(tiles, sms);
  a.n_items = lay_out_items(&a.one_scene, 1, a.item_tiles, tail_units(sms));
  const int grid = (int)((a.n_items + kWarpsPerCta - 1) / kWarpsPerCta);  // one item per warp
  a.emit_views = fused_emit_views(1, a.one_view.n_words);
  if (launch_cull(a, grid, 1, st) ||
      (!a.emit_views && launch_changed_lists(nullptr, a.one_view, 1, a.one_view.n_words, &ctl->error, st))) {
    cudaGetLastError();
    return noalloc_fail(DPCULL_ERR_CUDA, "dpcull_cull_noalloc: launch failed");
  }
  // Wait for the result, then report a transform index past the matrix array (the
  // kernel skips such objects and leaves their bits clear).
  unsigned int err[2] = {0, 0};
  if (cudaMemcpyAsync(err, &ctl->error, sizeof err, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    cudaGetLastError();
    return noalloc_fail(DPCULL_ERR_CUDA, "dpcull_cull_noalloc: the cull failed on the device");
  }
  if (err[0] & kErrWaitTimeout)
    return noalloc_fail(DPCULL_ERR_CUDA, "dpcull_cull_noalloc: changed-list assembly incomplete");
  if (err[0] & kErrBadTransform)
    return noalloc_fail(DPCULL_ERR_OUT_OF_RANGE, "dpcull_cull_noalloc: a transform index is past the matrix array");
  return DPCULL_OK;
}
