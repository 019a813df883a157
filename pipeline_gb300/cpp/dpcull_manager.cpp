// dpcull_manager.cpp -- C++ host layer over the dpcull C ABI (see dpcull_manager.h).
#include "dpcull_manager.h"

#include <algorithm>
#include <cfloat>
#include <cstring>
#include <stdexcept>
#include <string>
#include <unordered_map>

namespace dpcull {

namespace {

void check(int rc, const char* what)
{
  if (rc != DPCULL_OK) throw std::runtime_error(std::string(what) + ": " + dpcull_last_error());
}

// Owns the dpcull context; groups and results keep it alive past the Manager, as the
// reference's shared objects may outlive their manager.
struct CtxHolder {
  dpcull_ctx ctx = nullptr;
  ~CtxHolder()
  {
    if (ctx) dpcull_ctx_destroy(ctx);
  }
};

}  // namespace

Box3f::Box3f()
{
  for (int i = 0; i < 3; ++i) {
    lower[i] = FLT_MAX;
    upper[i] = -FLT_MAX;
  }
}

Box3f::Box3f(const float lo[3], const float hi[3]) : Box3f()
{
  // dp/math/Boxnt.h:214-258: init, then update with each corner (NaN never replaces).
  for (const float* p : {lo, hi})
    for (int i = 0; i < 3; ++i) {
      if (lower[i] > p[i]) lower[i] = p[i];
      if (upper[i] < p[i]) upper[i] = p[i];
    }
}

Payload::~Payload() {}

class Object {
 public:
  float lowerLeft[4] = {0.f, 0.f, 0.f, 1.f};
  float extent[4] = {0.f, 0.f, 0.f, 0.f};
  size_t transformIndex = ~size_t(0);  // ObjectBitSet.cpp:39-44
  size_t groupIndex = ~size_t(0);
  PayloadSharedPtr userData;
};

class Result;

class Group {
 public:
  std::shared_ptr<CtxHolder> holder;
  std::vector<ObjectSharedPtr> objects;
  size_t incarnation = 0;                  // GroupBitSet.cpp:60
  size_t syncedIncarnation = ~size_t(0);   // cpu::GroupCPU: incarnation - 1
  bool obbDirty = true;
  bool bboxDirty = true;
  Box3f bbox;
  const void* matrices = nullptr;
  size_t matricesCount = 0, matricesStride = 0;
  dpcull_group dev = 0;
  bool haveBoxDev = false;
  dpcull_group boxDev = 0;
  std::vector<std::weak_ptr<Result>> results;

  ~Group()
  {
    for (auto& o : objects) o->groupIndex = ~size_t(0);  // GroupBitSet.cpp:67-74
    if (holder && holder->ctx) {
      dpcull_group_destroy(holder->ctx, dev);
      if (haveBoxDev) dpcull_group_destroy(holder->ctx, boxDev);
    }
  }
};

class Result {
 public:
  std::shared_ptr<CtxHolder> holder;
  GroupSharedPtr group;  // the result keeps its group alive (ResultBitSet.h:60)
  dpcull_result dev = 0;
  bool alive = false;
  std::vector<ObjectSharedPtr> changed;
  std::vector<uint32_t> bits;
  size_t sizeBits = 0;
  bool bitsValid = false;
  std::vector<uint32_t> scratch;

  ~Result()
  {
    if (alive && holder && holder->ctx) dpcull_result_destroy(holder->ctx, dev);
  }
};

// ---- Manager -----------------------------------------------------------------------------

Manager* Manager::create(int device) { return new Manager(device); }

Manager::Manager(int device)
{
  auto h = std::make_shared<CtxHolder>();
  check(dpcull_ctx_create(device, nullptr, &h->ctx), "dpcull_ctx_create");
  m_ctx = h->ctx;
  m_holder = h;
}

Manager::~Manager()
{
  if (m_ctx) dpcull_ctx_synchronize(m_ctx);
  // the context itself lives on while groups or results still hold it
}

ObjectSharedPtr Manager::objectCreate(PayloadSharedPtr const& userData)
{
  auto o = std::make_shared<Object>();
  o->userData = userData;
  return o;
}

void Manager::objectSetBoundingBox(ObjectSharedPtr const& object, Box3f const& box)
{
  // ManagerBitSet.cpp:99-109.  The reference's group-dirty branch never fires (the
  // object's group pointer is never set by GroupBitSet::addObject), so neither does it here.
  for (int i = 0; i < 3; ++i) {
    object->lowerLeft[i] = box.lower[i];
    object->extent[i] = box.upper[i] - box.lower[i];
  }
  object->lowerLeft[3] = 1.0f;
  object->extent[3] = 0.0f;
}

void Manager::objectSetTransformIndex(ObjectSharedPtr const& object, size_t index)
{
  object->transformIndex = index;  // ManagerBitSet.cpp:88-97 (same dead dirty branch)
}

void Manager::objectSetUserData(ObjectSharedPtr const& object, PayloadSharedPtr const& userData)
{
  object->userData = userData;
}

PayloadSharedPtr const& Manager::objectGetUserData(ObjectSharedPtr const& object)
{
  return object->userData;
}

GroupSharedPtr Manager::groupCreate()
{
  auto g = std::make_shared<Group>();
  g->holder = std::static_pointer_cast<CtxHolder>(m_holder);
  check(dpcull_group_create(m_ctx, &g->dev), "dpcull_group_create");
  return g;
}

void Manager::groupAddObject(GroupSharedPtr const& group, ObjectSharedPtr const& object)
{
  // GroupBitSet::addObject (GroupBitSet.cpp:76-91)
  if (object->groupIndex != ~size_t(0)) throw std::runtime_error("object already belongs to a different group");
  object->groupIndex = group->objects.size();
  group->objects.push_back(object);
  ++group->incarnation;
  group->bboxDirty = true;
  group->obbDirty = true;
}

ObjectSharedPtr Manager::groupGetObject(GroupSharedPtr const& group, size_t index)
{
  return group->objects.at(index);
}

void Manager::groupRemoveObject(GroupSharedPtr const& group, ObjectSharedPtr const& object)
{
  // GroupBitSet::removeObject (GroupBitSet.cpp:93-119) + ResultBitSet::onNotify.
  Group& g = *group;
  const size_t hole = object->groupIndex;
  if (!(hole < g.objects.size() && g.objects[hole] == object))
    throw std::runtime_error("object does not belong to this group");
  g.objects[hole] = g.objects.back();
  g.objects[hole]->groupIndex = hole;
  object->groupIndex = ~size_t(0);
  g.objects.pop_back();
  const size_t moved_from = g.objects.size();
  for (auto& w : g.results)
    if (auto r = w.lock()) {
      check(dpcull_result_move(m_ctx, r->dev, moved_from, hole), "dpcull_result_move");
      r->bitsValid = false;
    }
  g.bboxDirty = true;
  g.obbDirty = true;
  ++g.incarnation;
}

size_t Manager::groupGetCount(GroupSharedPtr const& group) { return group->objects.size(); }

void Manager::groupSetMatrices(GroupSharedPtr const& group, void const* matrices, size_t count,
                               size_t stride)
{
  // GroupBitSet::setMatrices (GroupBitSet.cpp:121-135): only a new pointer / count / stride.
  Group& g = *group;
  if (matrices != g.matrices || count != g.matricesCount || stride != g.matricesStride) {
    g.matrices = matrices;
    g.matricesCount = count;
    g.matricesStride = stride;
    g.bboxDirty = true;
    g.obbDirty = true;
  }
}

void Manager::groupMatrixChanged(GroupSharedPtr const& group, size_t index)
{
  // GroupBitSet::markMatrixDirty (GroupBitSet.h:140-150)
  if (index < group->matricesCount) {
    group->bboxDirty = true;
    group->obbDirty = true;
  }
}

ResultSharedPtr Manager::groupCreateResult(GroupSharedPtr const& group)
{
  auto r = std::make_shared<Result>();
  r->holder = std::static_pointer_cast<CtxHolder>(m_holder);
  r->group = group;
  check(dpcull_result_create(m_ctx, group->dev, &r->dev), "dpcull_result_create");
  r->alive = true;
  group->results.push_back(r);
  return r;
}

std::vector<ObjectSharedPtr> const& Manager::resultGetChanged(ResultSharedPtr const& result)
{
  return result->changed;
}

bool Manager::resultObjectIsVisible(ResultSharedPtr const& result, ObjectSharedPtr const& object)
{
  // ResultBitSet::isVisible (ResultBitSet.h:69-76): objects the result never saw are visible.
  Result& r = *result;
  if (!r.bitsValid) {
    size_t nbits = 0;
    int rc = dpcull_result_bits(m_ctx, r.dev, nullptr, 0, &nbits);
    if (rc != DPCULL_OK && rc != DPCULL_ERR_CAPACITY) check(rc, "dpcull_result_bits");
    r.bits.assign((nbits + 31) / 32 + 1, 0u);
    check(dpcull_result_bits(m_ctx, r.dev, r.bits.data(), r.bits.size(), &nbits), "dpcull_result_bits");
    r.sizeBits = nbits;
    r.bitsValid = true;
  }
  const size_t i = object->groupIndex;
  return i < r.sizeBits ? ((r.bits[i / 32] >> (i % 32)) & 1u) != 0 : true;
}

void Manager::uploadCurrent(Group& g, dpcull_group dg) const
{
  const size_t n = g.objects.size();
  std::vector<float> lower(3 * n), extent(3 * n);
  std::vector<uint32_t> xform(n);
  for (size_t i = 0; i < n; ++i) {
    const Object& o = *g.objects[i];
    for (int c = 0; c < 3; ++c) {
      lower[c * n + i] = o.lowerLeft[c];
      extent[c * n + i] = o.extent[c];
    }
    if (o.transformIndex > 0xFFFFFFFFull)
      throw std::runtime_error("transform index does not fit the device index type");
    xform[i] = (uint32_t)o.transformIndex;
  }
  check(dpcull_group_set_objects(m_ctx, dg, n, lower.data(), extent.data(), xform.data()),
        "dpcull_group_set_objects");
  check(dpcull_group_set_matrices(m_ctx, dg, g.matricesCount ? g.matrices : nullptr, g.matricesCount,
                                  g.matricesCount ? g.matricesStride : 64),
        "dpcull_group_set_matrices");
}

void Manager::sync(Group& g)
{
  // cpu::GroupCPU::updateOBBs (ManagerImpl.cpp:114-162): rebuild only when dirty.
  if (g.obbDirty || g.syncedIncarnation != g.incarnation) {
    uploadCurrent(g, g.dev);
    g.syncedIncarnation = g.incarnation;
    g.obbDirty = false;
  }
}

void Manager::finishCull(Result& r)
{
  Group& g = *r.group;
  size_t n = 0;
  r.scratch.resize(std::max<size_t>(g.objects.size(), 1));
  check(dpcull_result_changed(m_ctx, r.dev, r.scratch.data(), r.scratch.size(), &n), "dpcull_result_changed");
  r.changed.clear();
  r.changed.reserve(n);
  for (size_t k = 0; k < n; ++k) r.changed.push_back(g.objects[r.scratch[k]]);
  r.bitsValid = false;
}

void Manager::cull(GroupSharedPtr const& group, ResultSharedPtr const& result, Mat44f const& vp)
{
  if (result->group != group) throw std::runtime_error("result does not belong to this group");
  sync(*group);
  check(dpcull_cull(m_ctx, group->dev, result->dev, vp.m), "dpcull_cull");
  finishCull(*result);
}

void Manager::cullViews(GroupSharedPtr const& group, std::vector<ResultSharedPtr> const& results,
                        std::vector<Mat44f> const& vps)
{
  if (results.size() != vps.size() || results.empty())
    throw std::runtime_error("cullViews needs one result per view");
  for (auto& r : results)
    if (r->group != group) throw std::runtime_error("result does not belong to this group");
  sync(*group);
  std::vector<dpcull_result> rs;
  for (auto& r : results) rs.push_back(r->dev);
  dpcull_job job{group->dev, (uint32_t)vps.size(), rs.data(), vps.front().m};
  check(dpcull_cull_batched(m_ctx, &job, 1, nullptr), "dpcull_cull_batched");
  for (auto& r : results) finishCull(*r);
}

Box3f Manager::getBoundingBox(GroupSharedPtr const& group) const
{
  // ManagerBitSet::getBoundingBox (ManagerBitSet.cpp:151-162): recomputed from the current
  // objects and matrices when dirty.  A separate device copy is used so that the culling
  // copy keeps the contents of its last rebuild, as the reference's OBB cache does.
  Group& g = *group;
  if (g.bboxDirty) {
    if (!g.haveBoxDev) {
      check(dpcull_group_create(m_ctx, &g.boxDev), "dpcull_group_create");
      g.haveBoxDev = true;
    }
    uploadCurrent(g, g.boxDev);
    float lo[3], hi[3];
    check(dpcull_group_bounding_box(m_ctx, g.boxDev, lo, hi), "dpcull_group_bounding_box");
    for (int i = 0; i < 3; ++i) {
      g.bbox.lower[i] = lo[i];
      g.bbox.upper[i] = hi[i];
    }
    g.bboxDirty = false;
  }
  return g.bbox;
}

// ---- transform tree -------------------------------------------------------------------------
namespace transform {

static const size_t kVectorGrowth = 65536;  // Tree.cpp:35

Tree::Tree(dpcull_ctx ctx) : m_ctx(ctx)
{
  check(dpcull_tree_create(ctx, kVectorGrowth, &m_tree), "dpcull_tree_create");
  m_free.assign(kVectorGrowth, true);
  m_level.assign(kVectorGrowth, 0u);
  m_free[0] = false;          // Tree.cpp:38-47: root 0, identity, level -1
  m_level[0] = ~0u;
}

Tree::~Tree()
{
  if (m_ctx) dpcull_tree_destroy(m_ctx, m_tree);
}

void Tree::resize(size_t n)
{
  check(dpcull_tree_resize(m_ctx, m_tree, n), "dpcull_tree_resize");
  m_free.resize(n, true);
  m_level.resize(n, 0u);
}

Index Tree::addTransform(Index parent, Mat44f const& matrix)
{
  if (!isValidIndex(parent)) throw std::runtime_error("Tree::addTransform: Parent does not exist");
  size_t idx = std::find(m_free.begin(), m_free.end(), true) - m_free.begin();
  if (idx == m_free.size()) resize(m_free.size() + kVectorGrowth);
  m_free[idx] = false;
  const uint32_t lvl = m_level[parent] + 1u;
  m_level[idx] = lvl;
  if (m_levels.size() <= lvl) m_levels.resize(lvl + 1);
  m_levels[lvl].push_back({parent, (uint32_t)idx});
  m_pendingIndex.push_back((uint32_t)idx);
  m_pendingLocal.push_back(matrix);
  m_structureDirty = true;
  return (Index)idx;
}

void Tree::removeTransform(Index index)
{
  if (!isValidIndex(index)) throw std::runtime_error("Tree::removeTransform: Transform does not exist");
  auto& lst = m_levels[m_level[index]];
  for (size_t e = 0; e < lst.size(); ++e)
    if (lst[e].second == index) {
      lst[e] = lst.back();
      lst.pop_back();
      break;
    }
  m_free[index] = true;
  m_structureDirty = true;
}

void Tree::updateLocalMatrix(Index index, Mat44f const& matrix)
{
  m_pendingIndex.push_back(index);
  m_pendingLocal.push_back(matrix);
}

void Tree::compute(Mat44f const&)
{
  if (m_structureDirty) {
    std::vector<uint32_t> pairs, offsets{0u};
    for (auto& lvl : m_levels) {
      for (auto& e : lvl) {
        pairs.push_back(e.first);
        pairs.push_back(e.second);
      }
      offsets.push_back((uint32_t)(pairs.size() / 2));
    }
    check(dpcull_tree_set_structure(m_ctx, m_tree, pairs.size() / 2, pairs.data(), m_levels.size(),
                                    offsets.data()),
          "dpcull_tree_set_structure");
    m_structureDirty = false;
  }
  if (!m_pendingIndex.empty()) {
    // The last update of each transform wins (the scatter must not see duplicates).
    std::unordered_map<uint32_t, size_t> latest;
    for (size_t i = 0; i < m_pendingIndex.size(); ++i) latest[m_pendingIndex[i]] = i;
    std::vector<uint32_t> uidx;
    std::vector<Mat44f> umats;
    uidx.reserve(latest.size());
    umats.reserve(latest.size());
    for (size_t i = 0; i < m_pendingIndex.size(); ++i)
      if (latest[m_pendingIndex[i]] == i) {
        uidx.push_back(m_pendingIndex[i]);
        umats.push_back(m_pendingLocal[i]);
      }
    check(dpcull_tree_set_locals(m_ctx, m_tree, uidx.size(), uidx.data(), umats.front().m),
          "dpcull_tree_set_locals");
    m_pendingIndex.clear();
    m_pendingLocal.clear();
  }
  check(dpcull_tree_compute(m_ctx, m_tree), "dpcull_tree_compute");
}

Mat44f const* Tree::getWorldMatrices()
{
  m_worldHost.resize(m_level.size());
  check(dpcull_tree_world(m_ctx, m_tree, 0, m_worldHost.size(), m_worldHost.front().m), "dpcull_tree_world");
  return m_worldHost.data();
}

Mat44f const& Tree::getWorldMatrix(Index index) { return getWorldMatrices()[index]; }

std::vector<uint32_t> Tree::getDirtyWorldMatrices() const
{
  std::vector<uint32_t> w((m_level.size() + 31) / 32);
  check(dpcull_tree_dirty_world(m_ctx, m_tree, w.data(), w.size()), "dpcull_tree_dirty_world");
  return w;
}

const float* Tree::worldMatricesDevice() const
{
  const float* p = nullptr;
  size_t n = 0;
  check(dpcull_tree_world_device(m_ctx, m_tree, &p, &n), "dpcull_tree_world_device");
  return p;
}

}  // namespace transform
}  // namespace dpcull
