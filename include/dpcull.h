/*
 * dpcull.h -- C ABI of the GB300 culling backend for nvpro-pipeline.
 *
 * This is the boundary a dp::culling::cuda::Manager (the Mode::CUDA backend that the
 * reference declares in dp/culling/Manager.h:98 but never implements) and a
 * dp::transform tree binding reach the GPU through.  Plain C types only: pointers,
 * sizes and integer handles; no exceptions cross it.  Every function returns
 * DPCULL_OK (0) or a negative DPCULL_ERR_* code; dpcull_last_error() gives the
 * message of the calling thread's last failure.
 *
 * Conventions (the reference's, dp/math/Matmnt.h): a matrix is 16 floats, row-major,
 * row-vector convention (v' = v * M, world = local * parentWorld, clip = p * VP).
 * Visibility bit i of 32-bit word i/32 is object i of the group (ResultBitSet layout).
 * Object data is passed in planar form: lower[3][n] is the x row, then the y row, then
 * the z row of the boxes' lower corners; extent[3][n] likewise holds upper - lower,
 * exactly as ManagerBitSet::objectSetBoundingBox stores them
 * (dp/culling/src/ManagerBitSet.cpp:99-109).
 *
 * Results are bit-exact with the reference CPU manager (cpu::ManagerImpl::cull,
 * dp/culling/cpu/src/ManagerImpl.cpp:467-518) and transform tree
 * (dp/transform/src/Tree.cpp:133-166).
 *
 * Threading: a context owns one CUDA stream; calls on one context must not overlap.
 * Calls marked (async) only enqueue work; calls that return data to host memory
 * synchronize the context's stream first.
 */
#ifndef DPCULL_H
#define DPCULL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DPCULL_OK 0
#define DPCULL_ERR_INVALID_ARGUMENT (-1) /* bad handle, null pointer, bad size */
#define DPCULL_ERR_OUT_OF_RANGE (-2)     /* transform index >= matrix count, bad object index */
#define DPCULL_ERR_CUDA (-3)             /* a CUDA runtime call failed */
#define DPCULL_ERR_NO_MEMORY (-4)        /* device or pinned allocation failed */
#define DPCULL_ERR_STATE (-5)            /* call not valid in the current state */
#define DPCULL_ERR_TIMEOUT (-6)          /* a bounded device-side wait expired */
#define DPCULL_ERR_CAPACITY (-7)         /* caller's output buffer is too small */

typedef struct dpcull_ctx_s* dpcull_ctx;
typedef uint32_t dpcull_group;
typedef uint32_t dpcull_result;
typedef uint32_t dpcull_tree;
typedef uint32_t dpcull_plan;

/* Last error message of the calling thread ("" if none). */
const char* dpcull_last_error(void);
/* Library version, (major << 16) | minor. */
uint32_t dpcull_version(void);

/* ---- context ----------------------------------------------------------------------
 * Replaces the reference's Manager factory (cpu::Manager::create,
 * dp/culling/cpu/Manager.h:39-43).  device: CUDA ordinal; stream: a cudaStream_t to
 * work on, or NULL to let the context create its own. */
int dpcull_ctx_create(int device, void* stream, dpcull_ctx* out);
int dpcull_ctx_destroy(dpcull_ctx ctx);
/* Waits for all enqueued work; reports device-side errors (bad transform index,
 * expired wait) raised since the last check. */
int dpcull_ctx_synchronize(dpcull_ctx ctx);
/* The context's cudaStream_t. */
void* dpcull_ctx_stream(dpcull_ctx ctx);
/* Number of kernels this context has launched (graph launches count their kernels). */
uint64_t dpcull_ctx_kernel_launches(dpcull_ctx ctx);
/* Device bytes currently held by the context. */
uint64_t dpcull_ctx_device_bytes(dpcull_ctx ctx);
/* Cull-kernel launches of this context so far, by kind: out[0] the kernel that transforms
 * every box (no box cache), out[1] the one that also stores the box cache, out[2] the one
 * that reads it.  Every dpcull_cull, dpcull_cull_batched and dpcull_plan_launch counts one. */
int dpcull_ctx_cull_launches(dpcull_ctx ctx, uint64_t out[3]);
/* Enables (default) or disables the conservative prefilter for launches made after the
 * call (plans keep the setting they were created with).  Results are identical either
 * way: the prefilter only decides object-views whose outcome is certain under the
 * reference's rounding and sends all others through the exact test. */
int dpcull_ctx_set_prefilter(dpcull_ctx ctx, int enabled);
/* Whether groups keep their boxes between culls (default: on), as the reference keeps its
 * OBB cache between culls (GroupCPU::updateOBBs, dp/culling/cpu/src/ManagerImpl.cpp:
 * 114-162).  A group culled again with unchanged objects and matrices has its prefilter
 * boxes (20 bytes per object) and OBBs (64 bytes per object) stored by that cull, and every
 * later cull reads them instead of the objects and their world matrices; any change to the
 * group's objects or matrices (or a compute of the dpcull tree whose world matrices it is
 * bound to) makes them stale, and a group bound to other device matrices is never cached.
 * Results are identical either way.  Applies to every cull, batched cull and plan launch
 * issued after the call (plans created before it included). */
int dpcull_ctx_set_box_cache(dpcull_ctx ctx, int enabled);

/* ---- groups: a GroupBitSet's objects and matrices resident in HBM -------------------
 * Replaces Manager::groupCreate (dp/culling/Manager.h:119). */
int dpcull_group_create(dpcull_ctx ctx, dpcull_group* out);
int dpcull_group_destroy(dpcull_ctx ctx, dpcull_group g);
/* Replaces the group's objects with n new ones (groupAddObject x n after
 * objectSetBoundingBox / objectSetTransformIndex, Manager.h:113-120).  Host arrays. */
int dpcull_group_set_objects(dpcull_ctx ctx, dpcull_group g, size_t n, const float* lower,
                             const float* extent, const uint32_t* xform);
/* Appends k objects at indices n..n+k-1 (GroupBitSet::addObject,
 * dp/culling/src/GroupBitSet.cpp:76-91). */
int dpcull_group_append_objects(dpcull_ctx ctx, dpcull_group g, size_t k, const float* lower,
                                const float* extent, const uint32_t* xform);
/* Overwrites the listed objects in place (objectSetBoundingBox /
 * objectSetTransformIndex on grouped objects, ManagerBitSet.cpp:88-109). */
int dpcull_group_update_objects(dpcull_ctx ctx, dpcull_group g, size_t k, const uint32_t* index,
                                const float* lower, const float* extent, const uint32_t* xform);
/* Removes object `index` by moving the last object into its slot and remapping every
 * result's bit (GroupBitSet::removeObject + ResultBitSet::onNotify,
 * GroupBitSet.cpp:93-119, ResultBitSet.cpp:110-128). */
int dpcull_group_remove_object(dpcull_ctx ctx, dpcull_group g, size_t index);
int dpcull_group_count(dpcull_ctx ctx, dpcull_group g, size_t* n);
/* Copies `count` matrices from host memory at `matrices` with a byte stride into the
 * group's device matrix array (groupSetMatrices, Manager.h:124; the data is read now,
 * as the reference reads it when its cached boxes are rebuilt). */
int dpcull_group_set_matrices(dpcull_ctx ctx, dpcull_group g, const void* matrices, size_t count,
                              size_t stride);
/* Re-uploads only the listed matrices, read from matrices + index*stride
 * (groupMatrixChanged, Manager.h:125, as a dirty scatter). */
int dpcull_group_update_matrices(dpcull_ctx ctx, dpcull_group g, size_t k, const uint32_t* index,
                                 const void* matrices, size_t stride);
/* Uses a device matrix array in place (16-byte aligned, count x 16 floats), e.g. the
 * world matrices of a dpcull tree; no copy.  The caller keeps it alive. */
int dpcull_group_bind_device_matrices(dpcull_ctx ctx, dpcull_group g, const float* dev_matrices,
                                      size_t count);
/* Manager::getBoundingBox (Manager.h:142, ManagerBitSet.cpp:151-306), bit-exact. */
int dpcull_group_bounding_box(dpcull_ctx ctx, dpcull_group g, float lower[3], float upper[3]);

/* ---- results ------------------------------------------------------------------------
 * Replaces Manager::groupCreateResult (Manager.h:126).  A result starts with every
 * object visible, as ResultBitSet does on first use (ResultBitSet.cpp:65-79). */
int dpcull_result_create(dpcull_ctx ctx, dpcull_group g, dpcull_result* out);
int dpcull_result_destroy(dpcull_ctx ctx, dpcull_result r);
/* (async) Manager::cull (Manager.h:139): visibility of every object of g under vp
 * (16 floats, host memory), stored in r together with the ascending list of objects whose
 * visibility changed since r's previous cull. */
int dpcull_cull(dpcull_ctx ctx, dpcull_group g, dpcull_result r, const float vp[16]);
/* Manager::resultGetChanged (Manager.h:129): copies the changed list (group indices,
 * ascending) to host memory; *n receives its length.  DPCULL_ERR_CAPACITY if cap < *n.
 * Entries of `out` past *n may be overwritten. */
int dpcull_result_changed(dpcull_ctx ctx, dpcull_result r, uint32_t* out, size_t cap, size_t* n);
/* Visibility words of r (ceil(n/32) words); *n_bits receives the object count. */
int dpcull_result_bits(dpcull_ctx ctx, dpcull_result r, uint32_t* out, size_t n_words,
                       size_t* n_bits);
/* Both reads at once, in one host round trip in the common case: the visibility words
 * (bits may be NULL to skip; n_words its capacity; *n_bits receives the object count) and
 * the changed list (changed may be NULL to read the length only; cap its capacity;
 * *n_changed receives the length).  Entries of `changed` past *n_changed may be
 * overwritten.  The per-frame read of a reference caller: resultGetChanged plus the
 * visibility of every object. */
int dpcull_result_read(dpcull_ctx ctx, dpcull_result r, uint32_t* bits, size_t n_words, size_t* n_bits,
                       uint32_t* changed, size_t cap, size_t* n_changed);
/* Manager::resultObjectIsVisible (Manager.h:132) for group index `index`. */
int dpcull_result_is_visible(dpcull_ctx ctx, dpcull_result r, size_t index, int* visible);
/* ResultBitSet::onNotify (ResultBitSet.cpp:110-128) for one result: the object that
 * moved from old_index to new_index carries its visibility bit (an index past the
 * result's size counts as visible).  For hosts that keep the group's object order
 * themselves and re-upload objects with dpcull_group_set_objects. */
int dpcull_result_move(dpcull_ctx ctx, dpcull_result r, size_t old_index, size_t new_index);
/* Device pointers of r's visibility words, changed list and changed count. */
int dpcull_result_device(dpcull_ctx ctx, dpcull_result r, uint32_t** bits, uint32_t** changed,
                         uint32_t** n_changed);

/* ---- batched multi-scene, multi-view culling ----------------------------------------
 * One job culls one group under n_views view-projections into n_views results (one
 * result per view, each bound to that group).  All jobs run in one persistent launch. */
typedef struct dpcull_job {
  dpcull_group group;
  uint32_t n_views;
  const dpcull_result* results; /* n_views results of `group` */
  const float* vps;             /* n_views x 16 floats, host memory */
} dpcull_job;

typedef struct dpcull_tuning {
  uint32_t views_per_pass;   /* 1, 2, 4 or 8 views evaluated per object load ("views per warp") */
  uint32_t tiles_per_ticket; /* 512-object work items a warp claims at once ("tiles per CTA") */
  uint32_t ctas_per_sm;      /* persistent CTAs per SM (0 = occupancy limit) */
  uint32_t reserved;
} dpcull_tuning;

/* (async) One persistent launch over all jobs.  tuning may be NULL (defaults). */
int dpcull_cull_batched(dpcull_ctx ctx, const dpcull_job* jobs, size_t n_jobs,
                        const dpcull_tuning* tuning);
/* Builds a reusable plan for a fixed job list and captures its launch (view upload
 * included) in a CUDA graph.  tuning NULL = run the autotuner (cached per shape). */
int dpcull_plan_create(dpcull_ctx ctx, const dpcull_job* jobs, size_t n_jobs,
                       const dpcull_tuning* tuning, dpcull_plan* out);
/* Replaces the plan's view-projections (sum of n_views x 16 floats, job order). */
int dpcull_plan_set_views(dpcull_ctx ctx, dpcull_plan p, const float* vps);
/* (async) Replays the plan's graph. */
int dpcull_plan_launch(dpcull_ctx ctx, dpcull_plan p);
int dpcull_plan_tuning(dpcull_ctx ctx, dpcull_plan p, dpcull_tuning* out);
/* Duration in ms of the cull kernel alone in one of the plan's two most recent launches
 * (back = 0: the last one, 1: the one before), from CUDA events that the plan's graph
 * records on a side branch when the kernel can start and when it has finished; waits until
 * that kernel has finished.  No counterpart in the reference (measurement for the
 * kernel's roofline). */
int dpcull_plan_kernel_ms(dpcull_ctx ctx, dpcull_plan p, uint32_t back, float* ms);
/* Reads the results of the plan's last launch to the host in two waits: result i is the
 * i-th result of the plan's jobs in job and view order.  bits[i] (ceil(objects/32) words)
 * and changed[i] (changed_cap[i] entries) may be NULL to skip; n_changed[i] receives the
 * length of the changed list.  Pinned host buffers copy fastest.  Equivalent to
 * dpcull_result_bits + dpcull_result_changed on every result (ResultBitSet's
 * getChanged, dp/culling/src/ResultBitSet.cpp:61-108), with one wait per kind of data
 * instead of one or two per result.  DPCULL_ERR_CAPACITY when a list does not fit. */
int dpcull_plan_read(dpcull_ctx ctx, dpcull_plan p, uint32_t* const* bits, uint32_t* const* changed,
                     const size_t* changed_cap, size_t* n_changed);
/* The same read without waiting for the copies: the results of the plan's last launch are
 * snapshotted on the device, the call returns once their changed counts are known (after
 * that launch's kernels) with n_changed filled in, and the copies to bits / changed land
 * on a copy stream while the next dpcull_plan_launch runs.  The host buffers must stay
 * valid and untouched until dpcull_plan_read_wait returns (the next read_async waits for
 * the previous one's copies on the device).  When dpcull_plan_snapshot was called since the
 * last read, this reads that snapshot instead (results of the launch before the snapshot
 * call), so a frame loop can launch the next frame before it waits:
 *   set_views(i); snapshot (frame i-1); launch(i); read_wait; read_async (frame i-1).
 * No counterpart in the reference (it reads results synchronously). */
int dpcull_plan_read_async(dpcull_ctx ctx, dpcull_plan p, uint32_t* const* bits,
                           uint32_t* const* changed, const size_t* changed_cap, size_t* n_changed);
/* Snapshots the results of the plan's last launch on the device and starts copying their
 * changed counts to the host, without waiting; the next dpcull_plan_read_async reads this
 * snapshot.  A later dpcull_plan_launch may overwrite the results themselves.  From the
 * first snapshot or asynchronous read on, every launch of the plan also writes its results
 * into a second buffer of its own (one per graph slot), so the snapshot of a launch costs
 * no copy on the device; a launch made before that, or made while an unread snapshot holds
 * its buffer, is snapshotted by one copy of the results. */
int dpcull_plan_snapshot(dpcull_ctx ctx, dpcull_plan p);
int dpcull_plan_read_wait(dpcull_ctx ctx, dpcull_plan p);
int dpcull_plan_destroy(dpcull_ctx ctx, dpcull_plan p);
/* Autotunes views_per_pass / tiles_per_ticket / ctas_per_sm for the job list by timing
 * candidate launches (results of the jobs are overwritten). */
int dpcull_autotune(dpcull_ctx ctx, const dpcull_job* jobs, size_t n_jobs, dpcull_tuning* out);

/* ---- transform tree (dp::transform::Tree, dp/transform/Tree.h:42-129) ----------------
 * The host keeps the tree's structure (levels of (parent, transform) entries in the
 * reference's list order); the device keeps local and world matrices. */
int dpcull_tree_create(dpcull_ctx ctx, size_t capacity, dpcull_tree* out);
int dpcull_tree_destroy(dpcull_ctx ctx, dpcull_tree t);
/* Grows the capacity keeping every matrix and dirty bit (Tree::resizeDataStructures,
 * Tree.cpp:117-126; new entries are zero). */
int dpcull_tree_resize(dpcull_ctx ctx, dpcull_tree t, size_t capacity);
/* Level lists: pairs[2*i] = parent, pairs[2*i+1] = transform, level l spanning
 * [level_offsets[l], level_offsets[l+1]).  Replaces the structure set by addTransform /
 * removeTransform (Tree.cpp:54-98). */
int dpcull_tree_set_structure(dpcull_ctx ctx, dpcull_tree t, size_t n_entries,
                              const uint32_t* pairs, size_t n_levels,
                              const uint32_t* level_offsets);
/* Tree::updateLocalMatrix (Tree.h:87) for k transforms: writes the locals and marks
 * them dirty.  Matrices in host memory, 16 floats each. */
int dpcull_tree_set_locals(dpcull_ctx ctx, dpcull_tree t, size_t k, const uint32_t* index,
                           const float* matrices);
/* Sets world[index] without marking anything dirty (the fixed root, Tree.cpp:38-47). */
int dpcull_tree_set_worlds(dpcull_ctx ctx, dpcull_tree t, size_t k, const uint32_t* index,
                           const float* matrices);
/* (async) Tree::compute (Tree.cpp:133-166): propagates world matrices level by level
 * (one cooperative kernel launch); afterwards the dirty-world bits of this pass are
 * readable and the dirty-local bits are clear. */
int dpcull_tree_compute(dpcull_ctx ctx, dpcull_tree t);
/* Device pointer and capacity of the world matrix array (Tree::getWorldMatrices). */
int dpcull_tree_world_device(dpcull_ctx ctx, dpcull_tree t, const float** world, size_t* count);
/* Copies world matrices [first, first+count) to host memory. */
int dpcull_tree_world(dpcull_ctx ctx, dpcull_tree t, size_t first, size_t count, float* out);
/* Dirty-world bits of the last compute (the EventWorldMatricesChanged payload). */
int dpcull_tree_dirty_world(dpcull_ctx ctx, dpcull_tree t, uint32_t* words, size_t n_words);

/* ---- serving: device-resident scenes, continuous batching ---------------------------
 * A server keeps a pool of scenes resident in HBM under a byte budget (least recently
 * used scenes with no work in flight are evicted when a request needs room), admits cull
 * requests as they arrive, and packs every admissible pending request into the next
 * batch as soon as one of its streams is free: each batch is one persistent launch over
 * all (scene, view) pairs of its requests, batches on different streams overlap on the
 * device, and uploads of newly admitted scenes run on the batch's stream.  A request
 * culls one scene under 1..8 view-projections; its result is the visibility words of each
 * view (and the visible count), exactly those of dpcull_cull on the same data.  The
 * serving loop of the reference renderer has no counterpart: this is the GB300 service
 * around the cull of dp/culling/cpu/src/ManagerImpl.cpp:467-518. */
typedef struct dpcull_server_s* dpcull_server;

#define DPCULL_SERVER_MAX_VIEWS 8
#define DPCULL_REQUEST_KEEP_BITS 1u /* keep the visibility words for dpcull_server_result */

typedef struct dpcull_completion {
  uint64_t request;
  uint32_t scene;
  uint32_t n_views;
  uint32_t visible[DPCULL_SERVER_MAX_VIEWS]; /* visible objects per view */
  uint64_t objects;                          /* objects of the scene */
  double submit_s, start_s, done_s;          /* dpcull_server_now() clock */
  int32_t status;                            /* DPCULL_OK or an error code */
  uint32_t pad;
} dpcull_completion;

typedef struct dpcull_server_stats {
  uint64_t requests_submitted, requests_completed, batches;
  uint64_t scene_uploads, scene_evictions, upload_bytes;
  uint64_t resident_bytes, resident_scenes, budget_bytes;
  uint64_t max_batch_requests, pending_requests;
  /* scheduler timing: longest turn, turns over 1 ms, longest upload / eviction call (us) */
  uint64_t max_turn_us, slow_turns, max_upload_call_us, max_evict_call_us;
  uint64_t reserved_bytes;  /* budget mapped into the device pool at creation (0: grows on demand) */
} dpcull_server_stats;

/* Steady-clock seconds; the clock of dpcull_completion's timestamps. */
double dpcull_server_now(void);
/* n_streams batches may be in flight at once (1..8); max_batch_objects caps the
 * object-views of one batch (latency bound); the scheduler runs on its own thread. */
int dpcull_server_create(dpcull_ctx ctx, uint64_t budget_bytes, uint32_t n_streams,
                         uint64_t max_batch_objects, dpcull_server* out);
int dpcull_server_destroy(dpcull_server s);
/* Registers scene `scene` (ids are dense small integers).  The host arrays are copied
 * now into a pinned staging buffer in the device layout (scenes registered with the same
 * arrays share it), so every later upload is one asynchronous copy; the caller may free
 * them afterwards.  Planar lower[3][n] / extent[3][n], uint32 xform[n], n_matrices x 16
 * floats. */
int dpcull_server_add_scene(dpcull_server s, uint32_t scene, size_t n, const float* lower,
                            const float* extent, const uint32_t* xform, const float* matrices,
                            size_t n_matrices);
/* Thread-safe.  vps: n_views x 16 floats (copied). */
int dpcull_server_submit(dpcull_server s, uint32_t scene, uint32_t n_views, const float* vps,
                         uint32_t flags, uint64_t* request);
/* Completed requests since the last poll (up to cap); *n receives the count. */
int dpcull_server_poll(dpcull_server s, dpcull_completion* out, size_t cap, size_t* n);
/* Visibility words of view `view` of a completed DPCULL_REQUEST_KEEP_BITS request. */
int dpcull_server_result(dpcull_server s, uint64_t request, uint32_t view, uint32_t* words,
                         size_t n_words);
int dpcull_server_release(dpcull_server s, uint64_t request);
/* Waits until every submitted request has completed. */
int dpcull_server_drain(dpcull_server s);
int dpcull_server_get_stats(dpcull_server s, dpcull_server_stats* out);

/* ---- cull without allocation -------------------------------------------------------
 * No counterpart in the reference: an extra entry point of this library for callers
 * that cannot allocate device memory when they cull -- a frame loop that must not hit
 * cudaMalloc's implicit device synchronisation, or a process whose device memory is all
 * owned by another allocator (a framework's caching allocator, a budget reserved up
 * front).  It runs the plain cull of dpcull_cull on buffers the caller owns and takes its
 * scratch from one static device array of about 128 KB that every GPU loading this
 * library holds until the process exits; it calls no cudaMalloc, cudaFree or other
 * allocating routine.
 *   objects   device, 16-byte aligned: 7 rows of `cap` entries -- lower x, y, z,
 *             extent x, y, z (float) and the transform index (uint32);
 *             cap is a multiple of 128 and >= n; n <= DPCULL_NOALLOC_MAX_OBJECTS
 *             (larger n: DPCULL_ERR_CAPACITY)
 *   matrices  device, 16-byte aligned, n_matrices x 16 floats
 *   bits      device, cap/32 words: the previous visibility on entry (a result that was
 *             never culled is all ones for objects 0..n-1, zero past n), the new
 *             visibility on return
 *   changed   device, n entries: the ascending list of objects whose bit changed;
 *   n_changed device, one word: its length
 * The first call on a device looks up the scratch array's address with that device
 * current and keeps it until the process exits; do not call this entry point on a device
 * again after cudaDeviceReset of that device (the reset destroys the array).  Every call
 * shares the array (it keeps the last call's contents; each call clears what must start
 * at zero), so calls whose work overlaps on the GPU race.  Blocks: waits for its work on
 * `stream` (cudaStreamSynchronize) and returns after it has finished, so it cannot be
 * called inside a stream capture; DPCULL_ERR_OUT_OF_RANGE if a transform index is past
 * the matrix array (those objects are left invisible). */
#define DPCULL_NOALLOC_MAX_OBJECTS (1u << 20)
int dpcull_cull_noalloc(const float* objects, size_t cap, size_t n, const float* matrices,
                        size_t n_matrices, const float vp[16], uint32_t* bits, uint32_t* changed,
                        uint32_t* n_changed, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* DPCULL_H */
