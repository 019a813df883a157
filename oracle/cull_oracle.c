/*
 * cull_oracle.c -- TEST INFRASTRUCTURE ONLY (see cull_oracle.h).
 *
 * CPU restatement of the reference algorithm for the culling hot path.  Each
 * function names the reference file:line it follows (paths relative to the
 * nvpro-pipeline source tree).  Build with -O2 -ffp-contract=off.
 */
#define _POSIX_C_SOURCE 199309L /* clock_gettime */
#include "cull_oracle.h"

#include <float.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* ------------------------------------------------------------------------- */
/* math: dp/math/Matmnt.h:1371-1379 (Vec4 * Mat44) and :1381-1415 (Mat44 * Mat44).
 * Every element is the left-to-right sum ((a0*b0 + a1*b1) + a2*b2) + a3*b3. */
void orc_vec4_mul_mat44(const float v[4], const float m[16], float out[4])
{
  float r[4];
  for (int j = 0; j < 4; ++j) {
    float acc = v[0] * m[0 * 4 + j];
    acc = acc + v[1] * m[1 * 4 + j];
    acc = acc + v[2] * m[2 * 4 + j];
    acc = acc + v[3] * m[3 * 4 + j];
    r[j] = acc;
  }
  memcpy(out, r, sizeof r);
}

void orc_mat44_mul(const float a[16], const float b[16], float out[16])
{
  float r[16];
  for (int i = 0; i < 4; ++i) orc_vec4_mul_mat44(a + 4 * i, b, r + 4 * i);
  memcpy(out, r, sizeof r);
}

/* ------------------------------------------------------------------------- */
/* One object's OBB: dp/culling/cpu/src/ManagerImpl.cpp:129-155.
 * point = lowerLeft * M with lowerLeft = (lower, 1)  (ManagerBitSet.cpp:99-109);
 * ex/ey/ez = extent[k] * M row k (Vecnt.h:912-923 -> operator*= per component). */
static void obb_one(const float lower4[4], const float extent4[4], const float* M, float obb[16])
{
  orc_vec4_mul_mat44(lower4, M, obb);
  for (int k = 0; k < 3; ++k)
    for (int c = 0; c < 4; ++c) obb[4 + 4 * k + c] = M[4 * k + c] * extent4[k];
}

/* determineCullFlags: ManagerImpl.cpp:199-229 (note the else-if and the <=). */
static inline void cull_flags(const float p[4], unsigned* cfo, unsigned* cfa)
{
  unsigned cf = 0;
  if (p[0] <= -p[3]) cf |= 0x01; else if (p[3] <= p[0]) cf |= 0x02;
  if (p[1] <= -p[3]) cf |= 0x04; else if (p[3] <= p[1]) cf |= 0x08;
  if (p[2] <= -p[3]) cf |= 0x10; else if (p[3] <= p[2]) cf |= 0x20;
  *cfo |= cf;
  *cfa &= cf;
}

static inline void vadd(const float a[4], const float b[4], float o[4])
{
  for (int i = 0; i < 4; ++i) o[i] = a[i] + b[i];
}

/* isVisible(projection, OBB): ManagerImpl.cpp:263-289. */
static int is_visible(const float vp[16], const float obb[16])
{
  unsigned cfo = 0, cfa = ~0u;
  float v[8][4], x[4], y[4], z[4];
  orc_vec4_mul_mat44(obb + 0, vp, v[0]);
  orc_vec4_mul_mat44(obb + 4, vp, x);
  orc_vec4_mul_mat44(obb + 8, vp, y);
  orc_vec4_mul_mat44(obb + 12, vp, z);
  vadd(v[0], x, v[1]);
  vadd(v[0], y, v[2]);
  vadd(v[1], y, v[3]);
  vadd(v[0], z, v[4]);
  vadd(v[1], z, v[5]);
  vadd(v[2], z, v[6]);
  vadd(v[3], z, v[7]);
  for (int i = 0; i < 8; ++i) cull_flags(v[i], &cfo, &cfa);
  return !cfo || !cfa;
}

/* ------------------------------------------------------------------------- */
/* stateless bulk paths */

int orc_build_obbs(size_t n, const float* lower, const float* extent, const uint32_t* idx,
                   const float* mats, size_t nmats, float* obb_out)
{
  for (size_t i = 0; i < n; ++i) {
    if (idx[i] >= nmats) return -1;
    float l4[4] = {lower[i], lower[n + i], lower[2 * n + i], 1.0f};
    float e4[4] = {extent[i], extent[n + i], extent[2 * n + i], 0.0f};
    obb_one(l4, e4, mats + 16 * (size_t)idx[i], obb_out + 16 * i);
  }
  return 0;
}

void orc_cull_obbs_range(size_t begin, size_t end, const float* obbs, const float vp[16],
                         uint32_t* bits_out)
{
  /* BitArray visible(N) starts cleared and setBit(i, v) writes each bit
   * (ManagerImpl.cpp:477,511-514); bits past N stay zero. */
  for (size_t w = begin / 32; w < (end + 31) / 32; ++w) bits_out[w] = 0;
  for (size_t i = begin; i < end; ++i)
    if (is_visible(vp, obbs + 16 * i)) bits_out[i >> 5] |= 1u << (i & 31);
}

void orc_cull_obbs(size_t n, const float* obbs, const float vp[16], uint32_t* bits_out)
{
  orc_cull_obbs_range(0, n, obbs, vp, bits_out);
}

int orc_cull_soa(size_t n, const float* lower, const float* extent, const uint32_t* idx,
                 const float* mats, size_t nmats, const float vp[16], uint32_t* bits_out)
{
  for (size_t w = 0; w < (n + 31) / 32; ++w) bits_out[w] = 0;
  for (size_t i = 0; i < n; ++i) {
    if (idx[i] >= nmats) return -1;
    float l4[4] = {lower[i], lower[n + i], lower[2 * n + i], 1.0f};
    float e4[4] = {extent[i], extent[n + i], extent[2 * n + i], 0.0f};
    float obb[16];
    obb_one(l4, e4, mats + 16 * (size_t)idx[i], obb);
    if (is_visible(vp, obb)) bits_out[i >> 5] |= 1u << (i & 31);
  }
  return 0;
}

typedef struct {
  size_t begin, end;
  const float* obbs;
  const float* vp;
  uint32_t* bits;
} cull_job;

static void* cull_job_run(void* p)
{
  cull_job* j = (cull_job*)p;
  orc_cull_obbs_range(j->begin, j->end, j->obbs, j->vp, j->bits);
  return NULL;
}

void orc_cull_obbs_mt(int nthreads, size_t n, const float* obbs, const float vp[16],
                      uint32_t* bits_out)
{
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  cull_job jobs[256];
  size_t words = (n + 31) / 32;
  size_t per = (words + (size_t)nthreads - 1) / (size_t)nthreads;
  int launched = 0;
  for (int t = 0; t < nthreads; ++t) {
    size_t b = (size_t)t * per * 32, e = b + per * 32;
    if (b >= n) break;
    if (e > n) e = n;
    jobs[t] = (cull_job){b, e, obbs, vp, bits_out};
    if (pthread_create(&th[t], NULL, cull_job_run, &jobs[t]) != 0) {
      cull_job_run(&jobs[t]);
      th[t] = 0;
    }
    ++launched;
  }
  for (int t = 0; t < launched; ++t)
    if (th[t]) pthread_join(th[t], NULL);
}

size_t orc_update_changed(size_t n, uint32_t* prev_bits, const uint32_t* vis_bits,
                          uint32_t* changed_out)
{
  /* ResultBitSet.cpp:100-107: newVisible = first n bits of vis, changed = new ^ prev,
   * ascending traversal (BitArray.h:104-137), prev = new. */
  size_t words = (n + 31) / 32, cnt = 0;
  for (size_t w = 0; w < words; ++w) {
    uint32_t nv = vis_bits[w];
    if (w == words - 1 && (n & 31)) nv &= (1u << (n & 31)) - 1u;
    uint32_t ch = nv ^ prev_bits[w];
    while (ch) {
      unsigned b = (unsigned)__builtin_ctz(ch);
      changed_out[cnt++] = (uint32_t)(w * 32 + b);
      ch &= ch - 1u;
    }
    prev_bits[w] = nv;
  }
  return cnt;
}

/* Box update: dp/math/Boxnt.h:245-258 (NaN never replaces a bound). */
static inline void box_update(float lo[], float hi[], const float p[], int n)
{
  for (int i = 0; i < n; ++i) {
    if (lo[i] > p[i]) lo[i] = p[i];
    if (hi[i] < p[i]) hi[i] = p[i];
  }
}

/* Box3f(lower, upper): Boxnt.h:214-231 -- init() to (FLT_MAX, -FLT_MAX) then two updates. */
static void box3_construct(const float a[3], const float b[3], float lo[3], float hi[3])
{
  for (int i = 0; i < 3; ++i) { lo[i] = FLT_MAX; hi[i] = -FLT_MAX; }
  box_update(lo, hi, a, 3);
  box_update(lo, hi, b, 3);
}

static void bbox_accumulate(const float lower4[4], const float extent4[4], const float* M,
                            float lo4[4], float hi4[4])
{
  /* ManagerBitSet.cpp:268-306 (CPU fallback): corner 0 = lowerLeft * M, axes are
   * extent[k] times row k, corners built by the same add chain as isVisible. */
  float v[8][4], x[4], y[4], z[4];
  orc_vec4_mul_mat44(lower4, M, v[0]);
  for (int c = 0; c < 4; ++c) {
    x[c] = extent4[0] * M[0 + c];
    y[c] = extent4[1] * M[4 + c];
    z[c] = extent4[2] * M[8 + c];
  }
  vadd(v[0], x, v[1]);
  vadd(v[0], y, v[2]);
  vadd(v[1], y, v[3]);
  vadd(v[0], z, v[4]);
  vadd(v[1], z, v[5]);
  vadd(v[2], z, v[6]);
  vadd(v[3], z, v[7]);
  for (int i = 0; i < 8; ++i) box_update(lo4, hi4, v[i], 4);
}

void orc_bounding_box(size_t n, const float* lower, const float* extent, const uint32_t* idx,
                      const float* mats, float out_lower[3], float out_upper[3])
{
  float lo4[4], hi4[4];
  for (int i = 0; i < 4; ++i) { lo4[i] = FLT_MAX; hi4[i] = -FLT_MAX; }
  for (size_t i = 0; i < n; ++i) {
    float l4[4] = {lower[i], lower[n + i], lower[2 * n + i], 1.0f};
    float e4[4] = {extent[i], extent[n + i], extent[2 * n + i], 0.0f};
    bbox_accumulate(l4, e4, mats + 16 * (size_t)idx[i], lo4, hi4);
  }
  box3_construct(lo4, hi4, out_lower, out_upper);
}

void orc_propagate(size_t n_entries, const uint32_t* entries, const float* local, float* world,
                   const uint32_t* dirty_local, uint32_t* dirty_world)
{
  /* Tree.cpp:150-160: for each entry in level order, recompute when the parent's world
   * matrix or the local matrix is dirty: world[t] = local[t] * world[parent]. */
  for (size_t e = 0; e < n_entries; ++e) {
    uint32_t p = entries[2 * e], t = entries[2 * e + 1];
    int dw = (dirty_world[p >> 5] >> (p & 31)) & 1u;
    int dl = (dirty_local[t >> 5] >> (t & 31)) & 1u;
    if (dw || dl) {
      orc_mat44_mul(local + 16 * (size_t)t, world + 16 * (size_t)p, world + 16 * (size_t)t);
      dirty_world[t >> 5] |= 1u << (t & 31);
    }
  }
}

/* ------------------------------------------------------------------------- */
/* growable bit array with the reference BitArray semantics needed here */
typedef struct {
  size_t size;
  uint32_t* w;
  size_t cap_words;
} bits_t;

static void bits_reserve(bits_t* b, size_t nbits)
{
  size_t words = (nbits + 31) / 32;
  if (words > b->cap_words) {
    size_t nc = b->cap_words ? b->cap_words : 4;
    while (nc < words) nc *= 2;
    b->w = (uint32_t*)realloc(b->w, nc * sizeof(uint32_t));
    memset(b->w + b->cap_words, 0, (nc - b->cap_words) * sizeof(uint32_t));
    b->cap_words = nc;
  }
}
static inline int bits_get(const bits_t* b, size_t i) { return (b->w[i >> 5] >> (i & 31)) & 1u; }
static inline void bits_set(bits_t* b, size_t i, int v)
{
  if (v) b->w[i >> 5] |= 1u << (i & 31);
  else b->w[i >> 5] &= ~(1u << (i & 31));
}
/* BitArray::resize (BitArray.cpp:63-89): bits below min(old,new) kept, bits at or above
 * the new size cleared, newly added bits false. */
static void bits_resize(bits_t* b, size_t n)
{
  bits_reserve(b, n);
  for (size_t i = n; i < b->cap_words * 32; ++i) bits_set(b, i, 0);
  b->size = n;
}

/* ------------------------------------------------------------------------- */
/* stateful manager: ObjectBitSet / GroupBitSet / ResultBitSet / cpu::GroupCPU */
typedef struct {
  float lower4[4], extent4[4];
  uint64_t xform;     /* ObjectBitSet.cpp:39-44: default ~0 */
  size_t group_index; /* ~0 when not grouped */
} orc_object;

typedef struct {
  int* objs;
  size_t n, cap;
  size_t incarnation;     /* GroupBitSet.cpp:60: starts at 0 */
  int obb_dirty;          /* starts true */
  int bbox_dirty;         /* starts true */
  float bbox_lo[3], bbox_hi[3];
  const void* mats;
  size_t mats_count, mats_stride;
  float* obbs;
  size_t obbs_cap;
  size_t obb_incarnation; /* ManagerImpl.cpp:103-106: incarnation - 1 */
  int* results;
  size_t n_results, results_cap;
} orc_group;

typedef struct {
  int group;
  int* changed;
  size_t n_changed, changed_cap;
  size_t incarnation;     /* ResultBitSet.cpp:43: ~0 */
  bits_t bits;            /* m_results */
} orc_result;

struct orc_mgr {
  orc_object* objects;
  size_t n_objects, cap_objects;
  orc_group* groups;
  size_t n_groups, cap_groups;
  orc_result* results;
  size_t n_results, cap_results;
};

#define GROW(arr, n, cap)                                                  \
  do {                                                                     \
    if ((n) >= (cap)) {                                                    \
      size_t nc_ = (cap) ? 2 * (cap) : 16;                                 \
      void* p_ = realloc((arr), nc_ * sizeof(*(arr)));                     \
      memset((char*)p_ + (cap) * sizeof(*(arr)), 0, (nc_ - (cap)) * sizeof(*(arr))); \
      (arr) = p_;                                                          \
      (cap) = nc_;                                                         \
    }                                                                      \
  } while (0)

orc_mgr* orc_mgr_create(void) { return (orc_mgr*)calloc(1, sizeof(orc_mgr)); }

void orc_mgr_destroy(orc_mgr* m)
{
  if (!m) return;
  for (size_t g = 0; g < m->n_groups; ++g) {
    free(m->groups[g].objs);
    free(m->groups[g].obbs);
    free(m->groups[g].results);
  }
  for (size_t r = 0; r < m->n_results; ++r) {
    free(m->results[r].changed);
    free(m->results[r].bits.w);
  }
  free(m->objects);
  free(m->groups);
  free(m->results);
  free(m);
}

int orc_object_create(orc_mgr* m)
{
  GROW(m->objects, m->n_objects, m->cap_objects);
  orc_object* o = &m->objects[m->n_objects];
  memset(o, 0, sizeof *o);
  o->xform = ~(uint64_t)0;
  o->group_index = ~(size_t)0;
  return (int)m->n_objects++;
}

void orc_object_set_bbox(orc_mgr* m, int obj, const float lower[3], const float upper[3])
{
  /* ManagerBitSet.cpp:99-109: lowerLeft = (box.lower, 1), extent = (box.size, 0).
   * The group-dirty branch there never fires (ObjectBitSet::m_group is only ever
   * reset, GroupBitSet.cpp:76-91), so this does not dirty the owning group. */
  float lo[3], hi[3];
  box3_construct(lower, upper, lo, hi);
  orc_object* o = &m->objects[obj];
  for (int i = 0; i < 3; ++i) {
    o->lower4[i] = lo[i];
    o->extent4[i] = hi[i] - lo[i];
  }
  o->lower4[3] = 1.0f;
  o->extent4[3] = 0.0f;
}

void orc_object_set_xform(orc_mgr* m, int obj, uint64_t index)
{
  /* ManagerBitSet.cpp:88-97: same dead group-dirty branch as above. */
  m->objects[obj].xform = index;
}

int orc_group_create(orc_mgr* m)
{
  GROW(m->groups, m->n_groups, m->cap_groups);
  orc_group* g = &m->groups[m->n_groups];
  memset(g, 0, sizeof *g);
  g->obb_dirty = 1;
  g->bbox_dirty = 1;
  g->incarnation = 0;
  g->obb_incarnation = (size_t)0 - 1;
  return (int)m->n_groups++;
}

int orc_group_add(orc_mgr* m, int gi, int obj)
{
  /* GroupBitSet.cpp:76-91 */
  orc_group* g = &m->groups[gi];
  orc_object* o = &m->objects[obj];
  if (o->group_index != ~(size_t)0) return -1;
  o->group_index = g->n;
  GROW(g->objs, g->n, g->cap);
  g->objs[g->n++] = obj;
  ++g->incarnation;
  g->bbox_dirty = 1;
  g->obb_dirty = 1;
  return 0;
}

/* ResultBitSet::onNotify: ResultBitSet.cpp:110-128 */
static void result_on_move(orc_result* r, size_t old_index, size_t new_index)
{
  if (new_index < r->bits.size) {
    if (old_index < r->bits.size) bits_set(&r->bits, new_index, bits_get(&r->bits, old_index));
    else bits_set(&r->bits, new_index, 1);
  }
}

int orc_group_remove(orc_mgr* m, int gi, int obj)
{
  /* GroupBitSet.cpp:93-119: move the last object into the hole, notify
   * Event(old = new size, new = hole). */
  orc_group* g = &m->groups[gi];
  orc_object* o = &m->objects[obj];
  size_t hole = o->group_index;
  if (!(hole < g->n && g->objs[hole] == obj)) return -1;
  g->objs[hole] = g->objs[g->n - 1];
  m->objects[g->objs[hole]].group_index = hole;
  o->group_index = ~(size_t)0;
  g->n--;
  for (size_t k = 0; k < g->n_results; ++k) result_on_move(&m->results[g->results[k]], g->n, hole);
  g->bbox_dirty = 1;
  g->obb_dirty = 1;
  ++g->incarnation;
  return 0;
}

size_t orc_group_count(orc_mgr* m, int g) { return m->groups[g].n; }
int orc_group_get_object(orc_mgr* m, int g, size_t index) { return m->groups[g].objs[index]; }

void orc_group_set_matrices(orc_mgr* m, int gi, const void* mats, size_t count, size_t stride)
{
  /* GroupBitSet.cpp:121-135: only a changed pointer, count or stride dirties. */
  orc_group* g = &m->groups[gi];
  if (mats != g->mats || count != g->mats_count || stride != g->mats_stride) {
    g->mats = mats;
    g->mats_count = count;
    g->mats_stride = stride;
    g->bbox_dirty = 1;
    g->obb_dirty = 1;
  }
}

void orc_group_matrix_changed(orc_mgr* m, int gi, size_t index)
{
  /* GroupBitSet.h:140-150: indices past the matrix count are ignored. */
  orc_group* g = &m->groups[gi];
  if (index < g->mats_count) {
    g->bbox_dirty = 1;
    g->obb_dirty = 1;
  }
}

int orc_result_create(orc_mgr* m, int gi)
{
  GROW(m->results, m->n_results, m->cap_results);
  orc_result* r = &m->results[m->n_results];
  memset(r, 0, sizeof *r);
  r->group = gi;
  r->incarnation = ~(size_t)0;
  orc_group* g = &m->groups[gi];
  GROW(g->results, g->n_results, g->results_cap);
  g->results[g->n_results++] = (int)m->n_results;
  return (int)m->n_results++;
}

static const float* group_matrix(const orc_group* g, uint64_t index)
{
  return (const float*)((const char*)g->mats + index * g->mats_stride);
}

/* GroupCPU::updateOBBs: ManagerImpl.cpp:114-162 */
static void group_update_obbs(orc_mgr* m, orc_group* g)
{
  g->obb_dirty |= (g->obb_incarnation != g->incarnation);
  if (!g->obb_dirty) return;
  if (g->n > g->obbs_cap) {
    g->obbs = (float*)realloc(g->obbs, g->n * 16 * sizeof(float));
    g->obbs_cap = g->n;
  }
  for (size_t i = 0; i < g->n; ++i) {
    const orc_object* o = &m->objects[g->objs[i]];
    obb_one(o->lower4, o->extent4, group_matrix(g, o->xform), g->obbs + 16 * i);
  }
  g->obb_incarnation = g->incarnation;
  g->obb_dirty = 0;
}

/* ResultBitSet::updateChanged: ResultBitSet.cpp:61-108 */
static void result_update_changed(orc_mgr* m, orc_result* r, const uint32_t* vis)
{
  orc_group* g = &m->groups[r->group];
  size_t n = g->n;
  if (r->incarnation != g->incarnation) {
    r->incarnation = g->incarnation;
    size_t old = r->bits.size;
    bits_resize(&r->bits, n);
    for (size_t i = old; i < n; ++i) bits_set(&r->bits, i, 1); /* new objects start visible */
  }
  r->n_changed = 0;
  if (n > r->changed_cap) {
    r->changed = (int*)realloc(r->changed, n * sizeof(int));
    r->changed_cap = n;
  }
  for (size_t i = 0; i < n; ++i) {
    int nv = (vis[i >> 5] >> (i & 31)) & 1u;
    if (nv != bits_get(&r->bits, i)) r->changed[r->n_changed++] = g->objs[i];
    bits_set(&r->bits, i, nv);
  }
}

void orc_cull(orc_mgr* m, int gi, int ri, const float vp[16])
{
  /* cpu::ManagerImpl::cull: ManagerImpl.cpp:467-518 */
  orc_group* g = &m->groups[gi];
  group_update_obbs(m, g);
  size_t words = (g->n + 31) / 32;
  uint32_t* vis = (uint32_t*)calloc(words ? words : 1, sizeof(uint32_t));
  orc_cull_obbs(g->n, g->obbs, vp, vis);
  result_update_changed(m, &m->results[ri], vis);
  free(vis);
}

size_t orc_result_changed(orc_mgr* m, int ri, int* out, size_t cap)
{
  orc_result* r = &m->results[ri];
  size_t k = r->n_changed < cap ? r->n_changed : cap;
  if (k) memcpy(out, r->changed, k * sizeof(int));
  return r->n_changed;
}

int orc_result_is_visible(orc_mgr* m, int ri, int obj)
{
  /* ResultBitSet.h:69-76: never-culled objects count as visible. */
  orc_result* r = &m->results[ri];
  size_t gi = m->objects[obj].group_index;
  return gi < r->bits.size ? bits_get(&r->bits, gi) : 1;
}

void orc_group_bbox(orc_mgr* m, int gi, float lower[3], float upper[3])
{
  /* ManagerBitSet::getBoundingBox: ManagerBitSet.cpp:151-162 */
  orc_group* g = &m->groups[gi];
  if (g->bbox_dirty) {
    float lo4[4], hi4[4];
    for (int i = 0; i < 4; ++i) { lo4[i] = FLT_MAX; hi4[i] = -FLT_MAX; }
    for (size_t i = 0; i < g->n; ++i) {
      const orc_object* o = &m->objects[g->objs[i]];
      bbox_accumulate(o->lower4, o->extent4, group_matrix(g, o->xform), lo4, hi4);
    }
    box3_construct(lo4, hi4, g->bbox_lo, g->bbox_hi);
    g->bbox_dirty = 0;
  }
  memcpy(lower, g->bbox_lo, sizeof(float) * 3);
  memcpy(upper, g->bbox_hi, sizeof(float) * 3);
}

int orc_group_add_boxes(orc_mgr* m, int g, size_t n, const float* lower, const float* upper,
                        const uint32_t* xform)
{
  int first = -1;
  for (size_t i = 0; i < n; ++i) {
    int o = orc_object_create(m);
    if (first < 0) first = o;
    orc_group_add(m, g, o);
    orc_object_set_xform(m, o, xform[i]);
    float lo[3] = {lower[i], lower[n + i], lower[2 * n + i]};
    float hi[3] = {upper[i], upper[n + i], upper[2 * n + i]};
    orc_object_set_bbox(m, o, lo, hi);
  }
  return first;
}

size_t orc_result_bits(orc_mgr* m, int ri, uint32_t* words, size_t nwords)
{
  orc_result* r = &m->results[ri];
  size_t have = (r->bits.size + 31) / 32;
  size_t k = have < nwords ? have : nwords;
  if (k) memcpy(words, r->bits.w, k * sizeof(uint32_t));
  return r->bits.size;
}

/* ------------------------------------------------------------------------- */
/* transform tree: dp/transform/src/Tree.cpp */
typedef struct {
  uint32_t* pairs;
  size_t n, cap;
} level_list;

struct orc_tree {
  size_t capacity;       /* m_level.size() */
  float* local;
  float* world;
  uint32_t* level;
  bits_t free_bits;      /* true = free */
  bits_t dirty_local;    /* m_dirtyTransforms */
  bits_t dirty_world;    /* m_dirtyWorldMatrices */
  bits_t last_dirty;     /* copy of the payload of the last EventWorldMatricesChanged */
  level_list* levels;
  size_t n_levels;
};

static const size_t kVectorGrowth = 65536; /* Tree.cpp:35 */

static void tree_resize(orc_tree* t, size_t n)
{
  /* Tree::resizeDataStructures: Tree.cpp:117-126 (new free bits true, others false). */
  size_t old = t->capacity;
  t->local = (float*)realloc(t->local, n * 16 * sizeof(float));
  t->world = (float*)realloc(t->world, n * 16 * sizeof(float));
  t->level = (uint32_t*)realloc(t->level, n * sizeof(uint32_t));
  memset(t->local + 16 * old, 0, (n - old) * 16 * sizeof(float));
  memset(t->world + 16 * old, 0, (n - old) * 16 * sizeof(float));
  memset(t->level + old, 0, (n - old) * sizeof(uint32_t));
  bits_resize(&t->free_bits, n);
  for (size_t i = old; i < n; ++i) bits_set(&t->free_bits, i, 1);
  bits_resize(&t->dirty_local, n);
  bits_resize(&t->dirty_world, n);
  bits_resize(&t->last_dirty, n);
  t->capacity = n;
}

static const float kIdentity[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};

orc_tree* orc_tree_create(void)
{
  /* Tree::Tree: Tree.cpp:38-47 -- root 0 is identity, level -1, dirty local. */
  orc_tree* t = (orc_tree*)calloc(1, sizeof(orc_tree));
  tree_resize(t, kVectorGrowth);
  bits_set(&t->free_bits, 0, 0);
  bits_set(&t->dirty_local, 0, 1);
  memcpy(t->local, kIdentity, sizeof kIdentity);
  memcpy(t->world, kIdentity, sizeof kIdentity);
  t->level[0] = (uint32_t)-1;
  return t;
}

void orc_tree_destroy(orc_tree* t)
{
  if (!t) return;
  free(t->local);
  free(t->world);
  free(t->level);
  free(t->free_bits.w);
  free(t->dirty_local.w);
  free(t->dirty_world.w);
  free(t->last_dirty.w);
  for (size_t l = 0; l < t->n_levels; ++l) free(t->levels[l].pairs);
  free(t->levels);
  free(t);
}

static int tree_valid(orc_tree* t, uint32_t i)
{
  return i < t->free_bits.size && !bits_get(&t->free_bits, i);
}

int64_t orc_tree_add(orc_tree* t, uint32_t parent, const float m[16])
{
  /* Tree::addTransform: Tree.cpp:54-76; allocateIndex: :100-110 (first free bit). */
  if (!tree_valid(t, parent)) return -1;
  size_t idx = 0;
  while (idx < t->free_bits.size && !bits_get(&t->free_bits, idx)) ++idx;
  if (idx == t->free_bits.size) tree_resize(t, t->free_bits.size + kVectorGrowth);
  bits_set(&t->free_bits, idx, 0);
  uint32_t lvl = t->level[parent] + 1u;
  t->level[idx] = lvl;
  bits_set(&t->dirty_local, idx, 1);
  if (t->n_levels <= lvl) {
    t->levels = (level_list*)realloc(t->levels, (lvl + 1) * sizeof(level_list));
    memset(t->levels + t->n_levels, 0, (lvl + 1 - t->n_levels) * sizeof(level_list));
    t->n_levels = lvl + 1;
  }
  level_list* L = &t->levels[lvl];
  if (L->n == L->cap) {
    L->cap = L->cap ? 2 * L->cap : 64;
    L->pairs = (uint32_t*)realloc(L->pairs, L->cap * 2 * sizeof(uint32_t));
  }
  L->pairs[2 * L->n] = parent;
  L->pairs[2 * L->n + 1] = (uint32_t)idx;
  L->n++;
  memcpy(t->local + 16 * idx, m, 16 * sizeof(float));
  return (int64_t)idx;
}

int orc_tree_remove(orc_tree* t, uint32_t index)
{
  /* Tree::removeTransform: Tree.cpp:78-98 (swap-with-last inside its level list). */
  if (!tree_valid(t, index)) return -1;
  level_list* L = &t->levels[t->level[index]];
  for (size_t e = 0; e < L->n; ++e) {
    if (L->pairs[2 * e + 1] == index) {
      L->pairs[2 * e] = L->pairs[2 * (L->n - 1)];
      L->pairs[2 * e + 1] = L->pairs[2 * (L->n - 1) + 1];
      L->n--;
      break;
    }
  }
  bits_set(&t->free_bits, index, 1);
  return 0;
}

void orc_tree_update_local(orc_tree* t, uint32_t index, const float m[16])
{
  /* Tree.h:87 */
  memcpy(t->local + 16 * (size_t)index, m, 16 * sizeof(float));
  bits_set(&t->dirty_local, index, 1);
}

void orc_tree_compute(orc_tree* t)
{
  /* Tree::compute: Tree.cpp:133-166 */
  for (size_t l = 0; l < t->n_levels; ++l) {
    const level_list* L = &t->levels[l];
    orc_propagate(L->n, L->pairs, t->local, t->world, t->dirty_local.w, t->dirty_world.w);
  }
  memcpy(t->last_dirty.w, t->dirty_world.w, t->dirty_world.cap_words * sizeof(uint32_t));
  memset(t->dirty_local.w, 0, t->dirty_local.cap_words * sizeof(uint32_t));
  memset(t->dirty_world.w, 0, t->dirty_world.cap_words * sizeof(uint32_t));
}

/* CPU baseline of the transform propagation: `reps` timed runs (after `warm` untimed
 * ones) of Tree::compute, each after updateLocalMatrix on the n transforms ids[] (the
 * per-frame animated case); returns the median milliseconds of compute alone. */
double orc_tree_time_compute(orc_tree* t, const uint32_t* ids, size_t n, const float* locals, int warm,
                             int reps)
{
  double* ts = (double*)malloc(sizeof(double) * (size_t)(reps > 0 ? reps : 1));
  int k = 0;
  for (int i = 0; i < warm + reps; ++i) {
    for (size_t j = 0; j < n; ++j) orc_tree_update_local(t, ids[j], locals + 16 * j);
    struct timespec a, b;
    clock_gettime(CLOCK_MONOTONIC, &a);
    orc_tree_compute(t);
    clock_gettime(CLOCK_MONOTONIC, &b);
    if (i >= warm) ts[k++] = (double)(b.tv_sec - a.tv_sec) * 1e3 + (double)(b.tv_nsec - a.tv_nsec) * 1e-6;
  }
  for (int i = 1; i < k; ++i) /* insertion sort: a handful of values */
    for (int j = i; j > 0 && ts[j - 1] > ts[j]; --j) {
      double x = ts[j];
      ts[j] = ts[j - 1];
      ts[j - 1] = x;
    }
  const double med = k ? ts[k / 2] : 0.0;
  free(ts);
  return med;
}

size_t orc_tree_count(orc_tree* t) { return t->capacity; }
const float* orc_tree_world(orc_tree* t) { return t->world; }

size_t orc_tree_last_dirty(orc_tree* t, uint32_t* words, size_t nwords)
{
  size_t have = (t->capacity + 31) / 32;
  size_t k = have < nwords ? have : nwords;
  memcpy(words, t->last_dirty.w, k * sizeof(uint32_t));
  return have;
}

size_t orc_tree_entries(orc_tree* t, uint32_t* pairs, size_t cap, uint32_t* level_offsets,
                        size_t level_cap, size_t* n_levels)
{
  size_t total = 0;
  for (size_t l = 0; l < t->n_levels; ++l) {
    if (l < level_cap) level_offsets[l] = (uint32_t)total;
    for (size_t e = 0; e < t->levels[l].n; ++e, ++total)
      if (total < cap) {
        pairs[2 * total] = t->levels[l].pairs[2 * e];
        pairs[2 * total + 1] = t->levels[l].pairs[2 * e + 1];
      }
  }
  if (t->n_levels < level_cap) level_offsets[t->n_levels] = (uint32_t)total;
  *n_levels = t->n_levels;
  return total;
}
