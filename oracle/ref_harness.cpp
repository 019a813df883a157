// ref_harness.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Exposes the oracle's handle API (cull_oracle.h, prefix ref_ instead of orc_) on top of
// the REAL reference classes: dp::culling::cpu::Manager (ManagerBitSet / GroupBitSet /
// ResultBitSet / ObjectBitSet) and dp::transform::Tree, compiled from the reference
// sources by oracle/Makefile into oracle/_ref/libdpref.so.  Tests drive the same
// operation sequences through both libraries to pin the C restatement to the
// reference, and tests/golden/make_golden.py uses it to write the golden fixtures.
// This file contains no reference code; it only calls the reference's public API.
#include <dp/culling/Manager.h>
#include <dp/culling/cpu/Manager.h>
#include <dp/math/Boxnt.h>
#include <dp/math/Matmnt.h>
#include <dp/transform/Tree.h>
#include <dp/util/Observer.h>

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <vector>

// dp/culling/src/Manager.cpp also pulls in the OpenGL backend; only its destructor is needed.
namespace dp { namespace culling { Manager::~Manager() {} } }

namespace {

class IdPayload : public dp::culling::Payload
{
public:
  explicit IdPayload(int id) : m_id(id) {}
  int m_id;
};

struct RefMgr
{
  std::unique_ptr<dp::culling::Manager> mgr{dp::culling::cpu::Manager::create()};
  std::vector<dp::culling::ObjectSharedPtr> objects;
  std::vector<dp::culling::GroupSharedPtr> groups;
  std::vector<dp::culling::ResultSharedPtr> results;
  std::vector<int> result_group;
};

int object_id(RefMgr* m, dp::culling::ObjectSharedPtr const& o)
{
  auto p = std::static_pointer_cast<IdPayload>(m->mgr->objectGetUserData(o));
  return p->m_id;
}

class DirtyCapture : public dp::util::Observer
{
public:
  void onNotify(dp::util::Event const& event, dp::util::Payload*) override
  {
    auto const& e = static_cast<dp::transform::Tree::EventWorldMatricesChanged const&>(event);
    dp::util::BitArray const& b = e.getDirtyWorldMatrices();
    words.assign((b.getSize() + 31) / 32, 0u);
    for (size_t i = 0; i < b.getSize(); ++i)
      if (b.getBit(i)) words[i / 32] |= 1u << (i % 32);
  }
  void onDestroyed(dp::util::Subject const&, dp::util::Payload*) override {}
  std::vector<uint32_t> words;
};

struct RefTree
{
  dp::transform::Tree tree;
  DirtyCapture capture;
  RefTree() { tree.attach(&capture); }
  ~RefTree() { tree.detach(&capture); }
};

}  // namespace

extern "C" {

void* ref_mgr_create(void) { return new RefMgr(); }
void ref_mgr_destroy(void* h) { delete static_cast<RefMgr*>(h); }

int ref_object_create(void* h)
{
  RefMgr* m = static_cast<RefMgr*>(h);
  int id = (int)m->objects.size();
  m->objects.push_back(m->mgr->objectCreate(std::make_shared<IdPayload>(id)));
  return id;
}

void ref_object_set_bbox(void* h, int obj, const float lower[3], const float upper[3])
{
  RefMgr* m = static_cast<RefMgr*>(h);
  dp::math::Box3f box(dp::math::Vec3f(lower[0], lower[1], lower[2]),
                      dp::math::Vec3f(upper[0], upper[1], upper[2]));
  m->mgr->objectSetBoundingBox(m->objects[obj], box);
}

void ref_object_set_xform(void* h, int obj, uint64_t index)
{
  RefMgr* m = static_cast<RefMgr*>(h);
  m->mgr->objectSetTransformIndex(m->objects[obj], (size_t)index);
}

int ref_group_create(void* h)
{
  RefMgr* m = static_cast<RefMgr*>(h);
  m->groups.push_back(m->mgr->groupCreate());
  return (int)m->groups.size() - 1;
}

int ref_group_add(void* h, int g, int obj)
{
  RefMgr* m = static_cast<RefMgr*>(h);
  try { m->mgr->groupAddObject(m->groups[g], m->objects[obj]); } catch (std::exception const&) { return -1; }
  return 0;
}

int ref_group_remove(void* h, int g, int obj)
{
  RefMgr* m = static_cast<RefMgr*>(h);
  try { m->mgr->groupRemoveObject(m->groups[g], m->objects[obj]); } catch (std::exception const&) { return -1; }
  return 0;
}

size_t ref_group_count(void* h, int g)
{
  RefMgr* m = static_cast<RefMgr*>(h);
  return m->mgr->groupGetCount(m->groups[g]);
}

int ref_group_get_object(void* h, int g, size_t index)
{
  RefMgr* m = static_cast<RefMgr*>(h);
  return object_id(m, m->mgr->groupGetObject(m->groups[g], index));
}

void ref_group_set_matrices(void* h, int g, const void* mats, size_t count, size_t stride)
{
  RefMgr* m = static_cast<RefMgr*>(h);
  m->mgr->groupSetMatrices(m->groups[g], mats, count, stride);
}

void ref_group_matrix_changed(void* h, int g, size_t index)
{
  RefMgr* m = static_cast<RefMgr*>(h);
  m->mgr->groupMatrixChanged(m->groups[g], index);
}

int ref_result_create(void* h, int g)
{
  RefMgr* m = static_cast<RefMgr*>(h);
  m->results.push_back(m->mgr->groupCreateResult(m->groups[g]));
  m->result_group.push_back(g);
  return (int)m->results.size() - 1;
}

void ref_cull(void* h, int g, int r, const float vp[16])
{
  RefMgr* m = static_cast<RefMgr*>(h);
  dp::math::Mat44f VP;
  std::memcpy(&VP, vp, sizeof(float) * 16);
  m->mgr->cull(m->groups[g], m->results[r], VP);
}

size_t ref_result_changed(void* h, int r, int* out, size_t cap)
{
  RefMgr* m = static_cast<RefMgr*>(h);
  auto const& ch = m->mgr->resultGetChanged(m->results[r]);
  for (size_t i = 0; i < ch.size() && i < cap; ++i) out[i] = object_id(m, ch[i]);
  return ch.size();
}

int ref_result_is_visible(void* h, int r, int obj)
{
  RefMgr* m = static_cast<RefMgr*>(h);
  return m->mgr->resultObjectIsVisible(m->results[r], m->objects[obj]) ? 1 : 0;
}

void ref_group_bbox(void* h, int g, float lower[3], float upper[3])
{
  RefMgr* m = static_cast<RefMgr*>(h);
  dp::math::Box3f b = m->mgr->getBoundingBox(m->groups[g]);
  for (int i = 0; i < 3; ++i) {
    lower[i] = b.getLower()[i];
    upper[i] = b.getUpper()[i];
  }
}

int ref_group_add_boxes(void* h, int g, size_t n, const float* lower, const float* upper,
                        const uint32_t* xform)
{
  int first = -1;
  for (size_t i = 0; i < n; ++i) {
    int o = ref_object_create(h);
    if (first < 0) first = o;
    ref_group_add(h, g, o);
    ref_object_set_xform(h, o, xform[i]);
    float lo[3] = {lower[i], lower[n + i], lower[2 * n + i]};
    float hi[3] = {upper[i], upper[n + i], upper[2 * n + i]};
    ref_object_set_bbox(h, o, lo, hi);
  }
  return first;
}

// Visibility bits of a result, in group order, read through resultObjectIsVisible
// (ResultBitSet's bit array is private).  Returns the group's object count.
size_t ref_result_bits(void* h, int r, uint32_t* words, size_t nwords)
{
  RefMgr* m = static_cast<RefMgr*>(h);
  int g = m->result_group[r];
  size_t n = m->mgr->groupGetCount(m->groups[g]);
  for (size_t w = 0; w < nwords; ++w) words[w] = 0;
  for (size_t i = 0; i < n && i / 32 < nwords; ++i)
    if (m->mgr->resultObjectIsVisible(m->results[r], m->mgr->groupGetObject(m->groups[g], i)))
      words[i / 32] |= 1u << (i % 32);
  return n;
}

// Median time (ms) of `reps` culls of group g into result r after `warm` untimed ones.
// cold != 0 marks every matrix dirty before each cull (the per-frame animated case).
double ref_time_cull(void* h, int g, int r, const float vp[16], int warm, int reps, int cold,
                     size_t n_matrices)
{
  RefMgr* m = static_cast<RefMgr*>(h);
  dp::math::Mat44f VP;
  std::memcpy(&VP, vp, sizeof(float) * 16);
  std::vector<double> t;
  for (int i = 0; i < warm + reps; ++i) {
    if (cold)
      for (size_t k = 0; k < n_matrices; ++k) m->mgr->groupMatrixChanged(m->groups[g], k);
    auto t0 = std::chrono::steady_clock::now();
    m->mgr->cull(m->groups[g], m->results[r], VP);
    auto t1 = std::chrono::steady_clock::now();
    if (i >= warm) t.push_back(std::chrono::duration<double, std::milli>(t1 - t0).count());
  }
  std::sort(t.begin(), t.end());
  return t.empty() ? 0.0 : t[t.size() / 2];
}

// ---- transform tree ------------------------------------------------------------------
void* ref_tree_create(void) { return new RefTree(); }
void ref_tree_destroy(void* h) { delete static_cast<RefTree*>(h); }

int64_t ref_tree_add(void* h, uint32_t parent, const float mat[16])
{
  dp::math::Mat44f M;
  std::memcpy(&M, mat, sizeof(float) * 16);
  try { return (int64_t)static_cast<RefTree*>(h)->tree.addTransform(parent, M); }
  catch (std::exception const&) { return -1; }
}

int ref_tree_remove(void* h, uint32_t index)
{
  try { static_cast<RefTree*>(h)->tree.removeTransform(index); } catch (std::exception const&) { return -1; }
  return 0;
}

void ref_tree_update_local(void* h, uint32_t index, const float mat[16])
{
  dp::math::Mat44f M;
  std::memcpy(&M, mat, sizeof(float) * 16);
  static_cast<RefTree*>(h)->tree.updateLocalMatrix(index, M);
}

void ref_tree_compute(void* h) { static_cast<RefTree*>(h)->tree.compute(dp::math::cIdentity44f); }
size_t ref_tree_count(void* h) { return static_cast<RefTree*>(h)->tree.getTransformCount(); }
const float* ref_tree_world(void* h)
{
  return reinterpret_cast<const float*>(static_cast<RefTree*>(h)->tree.getWorldMatrices());
}

size_t ref_tree_last_dirty(void* h, uint32_t* words, size_t nwords)
{
  auto const& w = static_cast<RefTree*>(h)->capture.words;
  for (size_t i = 0; i < nwords && i < w.size(); ++i) words[i] = w[i];
  return w.size();
}

// Median time (ms) of Tree::compute after updateLocalMatrix on every listed transform.
double ref_time_tree_compute(void* h, const uint32_t* ids, size_t n, const float* locals,
                             int warm, int reps)
{
  RefTree* t = static_cast<RefTree*>(h);
  std::vector<double> ts;
  for (int i = 0; i < warm + reps; ++i) {
    for (size_t k = 0; k < n; ++k) {
      dp::math::Mat44f M;
      std::memcpy(&M, locals + 16 * k, sizeof(float) * 16);
      t->tree.updateLocalMatrix(ids[k], M);
    }
    auto t0 = std::chrono::steady_clock::now();
    t->tree.compute(dp::math::cIdentity44f);
    auto t1 = std::chrono::steady_clock::now();
    if (i >= warm) ts.push_back(std::chrono::duration<double, std::milli>(t1 - t0).count());
  }
  std::sort(ts.begin(), ts.end());
  return ts.empty() ? 0.0 : ts[ts.size() / 2];
}

}  // extern "C"
