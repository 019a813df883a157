// manager_parity.cpp -- drives dpcull::Manager (GPU) and the oracle's stateful manager
// (CPU restatement of the reference) through identical random operation sequences and
// compares every observable result: changed lists (object identities, in order),
// visibility queries, group order and bounding boxes.  Also dpcull::transform::Tree
// against the oracle tree.  Exit code 0 = all equal.
//
// Built and run by tests/test_gpu_cpp_manager.py.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <random>
#include <vector>

#include "cull_oracle.h"
#include "dpcull_manager.h"

namespace {

int g_fail = 0;
#define EXPECT(cond, ...)                    \
  do {                                       \
    if (!(cond)) {                           \
      std::fprintf(stderr, "FAIL %s:%d: ", __FILE__, __LINE__); \
      std::fprintf(stderr, __VA_ARGS__);     \
      std::fprintf(stderr, "\n");            \
      if (++g_fail > 20) std::exit(1);       \
    }                                        \
  } while (0)

class Id : public dpcull::Payload {
 public:
  explicit Id(int i) : id(i) {}
  int id;
};

int id_of(dpcull::Manager& m, dpcull::ObjectSharedPtr const& o)
{
  return std::static_pointer_cast<Id>(m.objectGetUserData(o))->id;
}

void random_matrix(std::mt19937& rng, float* M, float tscale)
{
  std::normal_distribution<float> n01;
  std::uniform_real_distribution<float> s(0.5f, 2.0f), t(-1000.f, 1000.f);
  float q[4] = {n01(rng), n01(rng), n01(rng), n01(rng)};
  float l = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  for (float& v : q) v /= l;
  const float x = q[0], y = q[1], z = q[2], w = q[3], sc = s(rng);
  const float R[9] = {1 - 2 * (y * y + z * z), 2 * (x * y + z * w), 2 * (x * z - y * w),
                      2 * (x * y - z * w), 1 - 2 * (x * x + z * z), 2 * (y * z + x * w),
                      2 * (x * z + y * w), 2 * (y * z - x * w), 1 - 2 * (x * x + y * y)};
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 3; ++c) M[4 * r + c] = sc * R[3 * r + c];
    M[4 * r + 3] = 0.f;
  }
  M[12] = t(rng) * tscale;
  M[13] = t(rng) * tscale;
  M[14] = t(rng) * tscale;
  M[15] = 1.f;
}

void perspective(float* P, float fovy, float aspect, float n, float f, float yaw)
{
  const float t = std::tan(fovy * 3.14159265f / 360.f) * n, r = t * aspect;
  float F[16] = {n / r, 0, 0, 0, 0, n / t, 0, 0, 0, 0, -(f + n) / (f - n), -1, 0, 0, -2 * f * n / (f - n), 0};
  const float c = std::cos(yaw), s = std::sin(yaw);
  float V[16] = {c, 0, -s, 0, 0, 1, 0, 0, s, 0, c, 0, 0, 0, 0, 1};
  orc_mat44_mul(V, F, P);
}

void run_manager_sequence(unsigned seed)
{
  std::mt19937 rng(seed);
  std::uniform_real_distribution<float> cen(-5.f, 5.f), ext(0.1f, 10.f), u01(0.f, 1.f);
  dpcull::Manager m(0);
  orc_mgr* o = orc_mgr_create();
  auto g = m.groupCreate();
  const int og = orc_group_create(o);
  std::vector<dpcull::ResultSharedPtr> rs = {m.groupCreateResult(g), m.groupCreateResult(g)};
  const int ors[2] = {orc_result_create(o, og), orc_result_create(o, og)};

  const int n_mats = 64 + (int)(seed % 50);
  std::vector<float> mats(16 * n_mats);
  const float tscale = 0.002f + 0.05f * (seed % 3);
  for (int i = 0; i < n_mats; ++i) random_matrix(rng, &mats[16 * i], tscale);
  m.groupSetMatrices(g, mats.data(), n_mats, 64);
  orc_group_set_matrices(o, og, mats.data(), n_mats, 64);

  std::vector<dpcull::ObjectSharedPtr> objs;  // index = oracle object id
  std::vector<int> alive;
  auto add_objects = [&](int k) {
    for (int i = 0; i < k; ++i) {
      const int oid = orc_object_create(o);
      auto obj = m.objectCreate(std::make_shared<Id>(oid));
      objs.push_back(obj);
      float c[3] = {cen(rng), cen(rng), cen(rng)}, lo[3], hi[3];
      for (int a = 0; a < 3; ++a) {
        const float e = ext(rng);
        lo[a] = c[a] - 0.5f * e;
        hi[a] = c[a] + 0.5f * e;
      }
      const size_t xf = rng() % n_mats;
      m.groupAddObject(g, obj);
      m.objectSetTransformIndex(obj, xf);
      m.objectSetBoundingBox(obj, dpcull::Box3f(lo, hi));
      EXPECT(orc_group_add(o, og, oid) == 0, "add");
      orc_object_set_xform(o, oid, xf);
      orc_object_set_bbox(o, oid, lo, hi);
      alive.push_back(oid);
    }
  };
  add_objects(500 + (int)(rng() % 3000));

  for (int step = 0; step < 14; ++step) {
    const unsigned op = rng() % 7;
    if (op == 0 && alive.size() > 1) {  // remove
      const size_t k = rng() % alive.size();
      const int oid = alive[k];
      alive.erase(alive.begin() + k);
      m.groupRemoveObject(g, objs[oid]);
      EXPECT(orc_group_remove(o, og, oid) == 0, "remove");
    } else if (op == 1) {
      add_objects(1 + (int)(rng() % 80));
    } else if (op == 2) {  // change matrices in place, sometimes marking them
      for (int k = 0; k < 6; ++k) random_matrix(rng, &mats[16 * (rng() % n_mats)], tscale);
      if (u01(rng) < 0.5f) {
        const size_t idx = rng() % (n_mats + 4);
        m.groupMatrixChanged(g, idx);
        orc_group_matrix_changed(o, og, idx);
      }
    } else if (op == 3) {  // change a grouped object's box without any dirty mark
      const int oid = alive[rng() % alive.size()];
      float lo[3] = {cen(rng), cen(rng), cen(rng)}, hi[3] = {lo[0] + 3, lo[1] + 3, lo[2] + 3};
      m.objectSetBoundingBox(objs[oid], dpcull::Box3f(lo, hi));
      orc_object_set_bbox(o, oid, lo, hi);
    } else if (op == 4) {  // bounding box
      dpcull::Box3f b = m.getBoundingBox(g);
      float lo[3], hi[3];
      orc_group_bbox(o, og, lo, hi);
      EXPECT(std::memcmp(lo, b.lower, 12) == 0 && std::memcmp(hi, b.upper, 12) == 0, "bbox step %d", step);
    }
    float vp[16];
    perspective(vp, 60.f + 30.f * u01(rng), 1.7f, 0.1f, 5000.f, 6.28f * u01(rng));
    const int which = u01(rng) < 0.7f ? 0 : 1;
    dpcull::Mat44f VP;
    std::memcpy(VP.m, vp, 64);
    m.cull(g, rs[which], VP);
    orc_cull(o, og, ors[which], vp);
    auto const& ch = m.resultGetChanged(rs[which]);
    std::vector<int> och(orc_result_changed(o, ors[which], nullptr, 0));
    orc_result_changed(o, ors[which], och.data(), och.size());
    EXPECT(ch.size() == och.size(), "seed %u step %d: %zu vs %zu changed", seed, step, ch.size(), och.size());
    for (size_t i = 0; i < ch.size() && i < och.size(); ++i)
      EXPECT(id_of(m, ch[i]) == och[i], "seed %u step %d: changed[%zu]", seed, step, i);
    EXPECT(m.groupGetCount(g) == orc_group_count(o, og), "count");
    for (size_t i = 0; i < alive.size(); i += 7) {
      const int oid = alive[i];
      for (int r = 0; r < 2; ++r)
        EXPECT(m.resultObjectIsVisible(rs[r], objs[oid]) == (orc_result_is_visible(o, ors[r], oid) != 0),
               "seed %u step %d visible obj %d result %d", seed, step, oid, r);
    }
    for (size_t i = 0; i < m.groupGetCount(g); i += 97)
      EXPECT(id_of(m, m.groupGetObject(g, i)) == orc_group_get_object(o, og, i), "order");
  }
  // batched views through the extension agree with per-view culls of the oracle
  std::vector<dpcull::Mat44f> vps(3);
  std::vector<dpcull::ResultSharedPtr> vr = {m.groupCreateResult(g), m.groupCreateResult(g), m.groupCreateResult(g)};
  int ovr[3];
  for (int v = 0; v < 3; ++v) {
    perspective(vps[v].m, 90.f, 1.f, 0.1f, 5000.f, 1.57f * v);
    ovr[v] = orc_result_create(o, og);
  }
  m.cullViews(g, vr, vps);
  for (int v = 0; v < 3; ++v) {
    orc_cull(o, og, ovr[v], vps[v].m);
    auto const& ch = m.resultGetChanged(vr[v]);
    std::vector<int> och(orc_result_changed(o, ovr[v], nullptr, 0));
    orc_result_changed(o, ovr[v], och.data(), och.size());
    EXPECT(ch.size() == och.size(), "views %d", v);
    for (size_t i = 0; i < ch.size() && i < och.size(); ++i) EXPECT(id_of(m, ch[i]) == och[i], "views changed");
  }
  orc_mgr_destroy(o);
}

void run_tree_sequence(unsigned seed)
{
  std::mt19937 rng(seed);
  dpcull::Manager m(0);
  dpcull::transform::Tree t(m.context());
  orc_tree* ot = orc_tree_create();
  std::vector<uint32_t> ids = {0};
  float M[16];
  for (int i = 0; i < 3000; ++i) {
    random_matrix(rng, M, 0.01f);
    const uint32_t parent = ids[rng() % ids.size()];
    dpcull::Mat44f mm;
    std::memcpy(mm.m, M, 64);
    const uint32_t a = t.addTransform(parent, mm);
    const int64_t b = orc_tree_add(ot, parent, M);
    EXPECT((int64_t)a == b, "tree add %u vs %lld", a, (long long)b);
    ids.push_back(a);
  }
  for (int step = 0; step < 5; ++step) {
    for (int k = 0; k < 50; ++k) {
      const uint32_t i = ids[1 + rng() % (ids.size() - 1)];
      random_matrix(rng, M, 0.01f);
      dpcull::Mat44f mm;
      std::memcpy(mm.m, M, 64);
      t.updateLocalMatrix(i, mm);
      orc_tree_update_local(ot, i, M);
    }
    if (step == 2) {  // orphan a subtree, then reuse its index
      const uint32_t v = ids[10];
      t.removeTransform(v);
      orc_tree_remove(ot, v);
      random_matrix(rng, M, 0.01f);
      dpcull::Mat44f mm;
      std::memcpy(mm.m, M, 64);
      EXPECT(t.addTransform(ids[3], mm) == v, "reuse");
      orc_tree_add(ot, ids[3], M);
    }
    dpcull::Mat44f I{};
    t.compute(I);
    orc_tree_compute(ot);
    const dpcull::Mat44f* w = t.getWorldMatrices();
    const float* ow = orc_tree_world(ot);
    EXPECT(std::memcmp(w, ow, 64 * 3001) == 0, "tree world step %d", step);
    std::vector<uint32_t> d = t.getDirtyWorldMatrices(), od(d.size());
    orc_tree_last_dirty(ot, od.data(), od.size());
    EXPECT(d == od, "tree dirty step %d", step);
  }
  orc_tree_destroy(ot);
}

}  // namespace

int main()
{
  for (unsigned seed = 1; seed <= 8; ++seed) run_manager_sequence(seed);
  for (unsigned seed = 1; seed <= 3; ++seed) run_tree_sequence(seed);
  if (g_fail) {
    std::fprintf(stderr, "%d failures\n", g_fail);
    return 1;
  }
  std::printf("manager_parity: all sequences equal\n");
  return 0;
}
