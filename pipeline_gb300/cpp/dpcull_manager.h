// dpcull_manager.h -- C++ host layer of the GB300 culling backend.
//
// dpcull::Manager has the surface and the semantics of dp::culling::Manager
// (dp/culling/Manager.h:108-143) as implemented by the reference's BitSet classes and CPU
// backend (GroupBitSet, ObjectBitSet, ResultBitSet, cpu::ManagerImpl), with the culling
// itself on the GPU through the C ABI of include/dpcull.h:
//   * objects, groups and results are shared_ptr handles; matrices are borrowed
//     (pointer + count + byte stride) and read when the group's cached boxes are rebuilt;
//   * the device copy of a group is rebuilt exactly when cpu::GroupCPU::updateOBBs would
//     rebuild its OBB cache (ManagerImpl.cpp:114-162): after groupSetMatrices with a new
//     pointer / count / stride, groupMatrixChanged, groupAddObject or groupRemoveObject.
//     As in the reference, objectSetBoundingBox / objectSetTransformIndex on an object
//     that is already in a group do not by themselves trigger that rebuild;
//   * results start all-visible, are resized on group changes and remapped on removals
//     like ResultBitSet (ResultBitSet.cpp:61-128); resultGetChanged lists the objects in
//     ascending group order;
//   * errors where the reference throws std::runtime_error throw std::runtime_error here;
//     device errors (for example a transform index past the matrix array) throw too.
// dpcull::transform::Tree mirrors dp::transform::Tree (dp/transform/Tree.h:42-129) with
// the propagation on the GPU.
#pragma once

#include <cstddef>
#include <cstdint>
#include <memory>
#include <vector>

#include "dpcull.h"

namespace dpcull {

struct Mat44f {
  float m[16];  // row-major, row-vector convention (the dp::math::Mat44f layout)
};

// dp::math::Box3f: constructed from two corners it keeps the component-wise extremes.
struct Box3f {
  float lower[3], upper[3];
  Box3f();
  Box3f(const float lo[3], const float hi[3]);
};

class Payload {
 public:
  virtual ~Payload();
};
using PayloadSharedPtr = std::shared_ptr<Payload>;

class Object;
class Group;
class Result;
using ObjectSharedPtr = std::shared_ptr<Object>;
using GroupSharedPtr = std::shared_ptr<Group>;
using ResultSharedPtr = std::shared_ptr<Result>;

class Manager {
 public:
  // The Mode::CUDA factory (device = CUDA ordinal).
  static Manager* create(int device = 0);
  explicit Manager(int device = 0);
  ~Manager();
  Manager(const Manager&) = delete;
  Manager& operator=(const Manager&) = delete;

  ObjectSharedPtr objectCreate(PayloadSharedPtr const& userData);
  void objectSetBoundingBox(ObjectSharedPtr const& object, Box3f const& boundingBox);
  void objectSetTransformIndex(ObjectSharedPtr const& object, size_t index);
  void objectSetUserData(ObjectSharedPtr const& object, PayloadSharedPtr const& userData);
  PayloadSharedPtr const& objectGetUserData(ObjectSharedPtr const& object);

  GroupSharedPtr groupCreate();
  void groupAddObject(GroupSharedPtr const& group, ObjectSharedPtr const& object);
  ObjectSharedPtr groupGetObject(GroupSharedPtr const& group, size_t index);
  void groupRemoveObject(GroupSharedPtr const& group, ObjectSharedPtr const& object);
  size_t groupGetCount(GroupSharedPtr const& group);
  void groupSetMatrices(GroupSharedPtr const& group, void const* matrices, size_t numberOfMatrices,
                        size_t stride);
  void groupMatrixChanged(GroupSharedPtr const& group, size_t index);
  ResultSharedPtr groupCreateResult(GroupSharedPtr const& group);

  std::vector<ObjectSharedPtr> const& resultGetChanged(ResultSharedPtr const& result);
  bool resultObjectIsVisible(ResultSharedPtr const& result, ObjectSharedPtr const& object);

  void cull(GroupSharedPtr const& group, ResultSharedPtr const& result, Mat44f const& viewProjection);
  Box3f getBoundingBox(GroupSharedPtr const& group) const;

  // GB300 extension: all views of one group in one persistent launch (one result per view).
  void cullViews(GroupSharedPtr const& group, std::vector<ResultSharedPtr> const& results,
                 std::vector<Mat44f> const& viewProjections);

  dpcull_ctx context() const { return m_ctx; }

 private:
  void sync(Group& g);
  void uploadCurrent(Group& g, dpcull_group dg) const;
  void finishCull(Result& r);
  dpcull_ctx m_ctx = nullptr;
  std::shared_ptr<void> m_holder;  // owns m_ctx; shared with groups and results
};

namespace transform {

using Index = uint32_t;

class Tree {
 public:
  explicit Tree(dpcull_ctx ctx);
  ~Tree();
  Tree(const Tree&) = delete;
  Tree& operator=(const Tree&) = delete;

  Index addTransform(Index parentIndex, Mat44f const& matrix);
  void removeTransform(Index transformIndex);
  void updateLocalMatrix(Index index, Mat44f const& matrix);
  // Propagation on the GPU; returns when the work is enqueued.
  void compute(Mat44f const& camera);
  // World matrices copied back to host memory (synchronizes).
  Mat44f const* getWorldMatrices();
  Mat44f const& getWorldMatrix(Index index);
  size_t getTransformCount() const { return m_level.size(); }
  // Dirty-world bits of the last compute, bit i of word i/32.
  std::vector<uint32_t> getDirtyWorldMatrices() const;
  // Device world matrix array (for dpcull_group_bind_device_matrices).
  const float* worldMatricesDevice() const;
  Index getRoot() const { return 0; }

 private:
  void resize(size_t n);
  bool isValidIndex(Index i) const { return i < m_free.size() && !m_free[i]; }
  dpcull_ctx m_ctx;
  dpcull_tree m_tree = 0;
  std::vector<bool> m_free;
  std::vector<uint32_t> m_level;
  std::vector<std::vector<std::pair<uint32_t, uint32_t>>> m_levels;
  std::vector<uint32_t> m_pendingIndex;
  std::vector<Mat44f> m_pendingLocal;
  std::vector<Mat44f> m_worldHost;
  bool m_structureDirty = true;
};

}  // namespace transform
}  // namespace dpcull
