/*
 * cull_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of nvpro-pipeline's culling path (dp::culling CPU manager,
 * ResultBitSet, GroupBitSet bookkeeping, bounding box) and of dp::transform::Tree.
 * It is the checker for the CUDA backend: only tests/, __graft_entry__.smoke()
 * and bench.py's cpu_baseline / reference leg may load it.  Nothing in the
 * product (pipeline_gb300/) links, imports or calls it.
 *
 * Parity is pinned against the reference itself: oracle/ref_harness.cpp exposes
 * the same handle API implemented by the real reference classes (built from the
 * reference sources by oracle/Makefile into oracle/_ref/), and the committed golden
 * fixtures under tests/golden/ were produced by that build.
 *
 * Conventions follow the reference: Mat44f is 16 floats, row-major, row-vector
 * convention (v' = v * M, world = local * parentWorld).  All arithmetic is FP32 in
 * the reference's exact operation order; this file must be compiled with
 * -ffp-contract=off (no fused multiply-add) so that it rounds like the reference.
 */
#ifndef DPCULL_ORACLE_H
#define DPCULL_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- math kernels (dp/math/Matmnt.h:1371-1415) ------------------------------ */
void orc_vec4_mul_mat44(const float v[4], const float m[16], float out[4]);
void orc_mat44_mul(const float a[16], const float b[16], float out[16]);

/* ---- stateless bulk paths (used for large parity cases and CPU timing) ------- */
/* OBB cache of dp/culling/cpu/src/ManagerImpl.cpp:114-162.  lower/extent are planar
 * [3][n] arrays (x row, y row, z row); idx[n] indexes mats[nmats][16].
 * obb_out is [n][16] = point, ex, ey, ez.  Returns 0, or -1 if an index is out of range. */
int orc_build_obbs(size_t n, const float* lower, const float* extent, const uint32_t* idx,
                   const float* mats, size_t nmats, float* obb_out);
/* isVisible loop of ManagerImpl.cpp:467-518 over a prebuilt OBB array.  bits_out has
 * ceil(n/32) words; bit i of word i/32 is object i; bits beyond n are zero. */
void orc_cull_obbs(size_t n, const float* obbs, const float vp[16], uint32_t* bits_out);
/* Same, rows [begin, end) only, with begin a multiple of 32 (thread partitions). */
void orc_cull_obbs_range(size_t begin, size_t end, const float* obbs, const float vp[16],
                         uint32_t* bits_out);
/* OBB build + cull without a cache (cold cull), one view. */
int orc_cull_soa(size_t n, const float* lower, const float* extent, const uint32_t* idx,
                 const float* mats, size_t nmats, const float vp[16], uint32_t* bits_out);
/* Multi-threaded warm cull over an OBB array (the all-cores CPU baseline). */
void orc_cull_obbs_mt(int nthreads, size_t n, const float* obbs, const float vp[16],
                      uint32_t* bits_out);
/* ResultBitSet::updateChanged on plain arrays (dp/culling/src/ResultBitSet.cpp:61-108)
 * for a result whose size already equals n: changed = vis ^ prev (ascending), then
 * prev = vis.  Returns the number of changed objects written to changed_out (which
 * must hold n entries). */
size_t orc_update_changed(size_t n, uint32_t* prev_bits, const uint32_t* vis_bits,
                          uint32_t* changed_out);
/* World-space bounding box of dp/culling/src/ManagerBitSet.cpp:268-306 (scalar path),
 * including the final Box3f(lower, upper) construction. */
void orc_bounding_box(size_t n, const float* lower, const float* extent, const uint32_t* idx,
                      const float* mats, float out_lower[3], float out_upper[3]);
/* Level-ordered world-matrix propagation of dp/transform/src/Tree.cpp:133-166 on plain
 * arrays.  entries is [n_entries][2] = (parent, transform), grouped by level in the
 * reference's list order; dirty_local / dirty_world are bit arrays over transforms
 * (dirty_world is updated in place and NOT cleared, so the caller can read the
 * EventWorldMatricesChanged payload). */
void orc_propagate(size_t n_entries, const uint32_t* entries, const float* local, float* world,
                   const uint32_t* dirty_local, uint32_t* dirty_world);

/* ---- stateful manager (mirrors dp::culling::Manager on the CPU backend) ------ */
typedef struct orc_mgr orc_mgr;
orc_mgr* orc_mgr_create(void);
void orc_mgr_destroy(orc_mgr* m);
int orc_object_create(orc_mgr* m);
void orc_object_set_bbox(orc_mgr* m, int obj, const float lower[3], const float upper[3]);
void orc_object_set_xform(orc_mgr* m, int obj, uint64_t index);
int orc_group_create(orc_mgr* m);
int orc_group_add(orc_mgr* m, int g, int obj);      /* 0, or -1 where the reference throws */
int orc_group_remove(orc_mgr* m, int g, int obj);   /* 0, or -1 where the reference throws */
size_t orc_group_count(orc_mgr* m, int g);
int orc_group_get_object(orc_mgr* m, int g, size_t index);
void orc_group_set_matrices(orc_mgr* m, int g, const void* mats, size_t count, size_t stride);
void orc_group_matrix_changed(orc_mgr* m, int g, size_t index);
int orc_result_create(orc_mgr* m, int g);
void orc_cull(orc_mgr* m, int g, int r, const float vp[16]);
size_t orc_result_changed(orc_mgr* m, int r, int* out_objs, size_t cap);
int orc_result_is_visible(orc_mgr* m, int r, int obj);
void orc_group_bbox(orc_mgr* m, int g, float lower[3], float upper[3]);
/* Bulk scene set-up in the order xbar::culling::CullingImpl::addObject uses
 * (CullingImpl.cpp:159-177): objectCreate, groupAddObject, objectSetTransformIndex,
 * objectSetBoundingBox(Box3f(lower, upper)).  lower/upper are planar [3][n]; returns the
 * first new object id (ids are consecutive). */
int orc_group_add_boxes(orc_mgr* m, int g, size_t n, const float* lower, const float* upper,
                        const uint32_t* xform);
/* The result's visibility bit array (m_results) as 32-bit words; returns its size in bits. */
size_t orc_result_bits(orc_mgr* m, int r, uint32_t* words, size_t nwords);

/* ---- stateful transform tree (mirrors dp::transform::Tree) ------------------- */
typedef struct orc_tree orc_tree;
orc_tree* orc_tree_create(void);
void orc_tree_destroy(orc_tree* t);
int64_t orc_tree_add(orc_tree* t, uint32_t parent, const float m[16]); /* -1 where it throws */
int orc_tree_remove(orc_tree* t, uint32_t index);                      /* -1 where it throws */
void orc_tree_update_local(orc_tree* t, uint32_t index, const float m[16]);
void orc_tree_compute(orc_tree* t);
/* median ms of Tree::compute after updating the n locals ids[] (CPU baseline timing) */
double orc_tree_time_compute(orc_tree* t, const uint32_t* ids, size_t n, const float* locals, int warm,
                             int reps);
size_t orc_tree_count(orc_tree* t);               /* getTransformCount(): the capacity */
const float* orc_tree_world(orc_tree* t);         /* getWorldMatrices() */
/* Dirty-world bits delivered by the last compute()'s EventWorldMatricesChanged. */
size_t orc_tree_last_dirty(orc_tree* t, uint32_t* words, size_t nwords);
/* Level entries in list order: writes (parent, transform) pairs, returns count, and
 * level_offsets[0..n_levels] (n_levels returned through *n_levels). */
size_t orc_tree_entries(orc_tree* t, uint32_t* pairs, size_t cap, uint32_t* level_offsets,
                        size_t level_cap, size_t* n_levels);

#ifdef __cplusplus
}
#endif
#endif
