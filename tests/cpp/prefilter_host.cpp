// Host build of the cull's conservative prefilter (pipeline_gb300/csrc/dpcull_prefilter.h),
// the same source the CUDA kernels compile, exported for tests/test_prefilter_host.py.
#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <vector>

#include "dpcull_prefilter.h"

using dpcull::pf::F4;

// The prefilter box of one object as the kernels build it: built with
// -DPF_TIGHT, the radius the Fill launch stores in the box cache (pf::tight_radius),
// otherwise the one the fused kernel uses every launch.
static dpcull::pf::Box box_of(float lx, float ly, float lz, float ex, float ey, float ez, const F4& m0,
                              const F4& m1, const F4& m2, const F4& m3)
{
  dpcull::pf::Box b = dpcull::pf::make_box(lx, ly, lz, ex, ey, ez, m0, m1, m2, m3);
#ifdef PF_TIGHT
  b.r = dpcull::pf::tight_radius(ex, ey, ez, m0, m1, m2, b.r);
#endif
  return b;
}

// Classification of n objects (planar [3][n] lower / extent rows, transform indices into
// mats[][16]) in one view: 0 invisible, 1 visible, 2 undecided.
extern "C" void pf_classify_soa(size_t n, const float* lower, const float* extent,
                                const uint32_t* idx, const float* mats, const float* vp,
                                int8_t* out)
{
  dpcull::pf::Planes p;
  dpcull::pf::make_planes(vp, p);
  for (size_t i = 0; i < n; ++i) {
    const float* m = mats + 16 * (size_t)idx[i];
    const F4 m0{m[0], m[1], m[2], m[3]}, m1{m[4], m[5], m[6], m[7]};
    const F4 m2{m[8], m[9], m[10], m[11]}, m3{m[12], m[13], m[14], m[15]};
    const dpcull::pf::Box b = box_of(lower[i], lower[n + i], lower[2 * n + i],
                                                   extent[i], extent[n + i], extent[2 * n + i],
                                                   m0, m1, m2, m3);
    out[i] = (int8_t)dpcull::pf::classify(b, p);
  }
}

// Classification of n objects in each of n_views views decided as one group (the margin
// the kernels use for the views of one work item): out[v * n + i].
extern "C" void pf_classify_group_soa(size_t n, const float* lower, const float* extent,
                                      const uint32_t* idx, const float* mats, const float* vps,
                                      size_t n_views, int8_t* out)
{
  dpcull::pf::GroupMargin gm{0.f, 0.f};
  dpcull::pf::Planes planes[64];
  for (size_t v = 0; v < n_views && v < 64; ++v) {
    dpcull::pf::GroupMargin m;
    dpcull::pf::group_view(vps + 16 * v, planes[v], m);
    gm = dpcull::pf::merge(gm, m);
  }
  for (size_t i = 0; i < n; ++i) {
    const float* m = mats + 16 * (size_t)idx[i];
    const F4 m0{m[0], m[1], m[2], m[3]}, m1{m[4], m[5], m[6], m[7]};
    const F4 m2{m[8], m[9], m[10], m[11]}, m3{m[12], m[13], m[14], m[15]};
    const dpcull::pf::Box b = box_of(lower[i], lower[n + i], lower[2 * n + i],
                                                   extent[i], extent[n + i], extent[2 * n + i],
                                                   m0, m1, m2, m3);
    for (size_t v = 0; v < n_views && v < 64; ++v)
      out[v * n + i] = (int8_t)dpcull::pf::classify_group(b, planes[v], gm);
  }
}

// Leaving out the far plane (pf::far_plane_clear) for a whole scene: the boxes' bound as
// the cull's Fill launch gathers it (bound keys over the boxes whose margin is a number),
// the group margin of all n_views views, then per view whether its z-hi plane is cleared
// (clear[v]) and, for a cleared view, the boxes whose z-hi value is not above D or whose
// five-plane bits differ from the six-plane ones (bad[v], must stay 0).
extern "C" void pf_far_scene(size_t n, const float* lower, const float* extent, const uint32_t* idx,
                             const float* mats, const float* vps, size_t n_views, int32_t* clear,
                             int64_t* bad)
{
  using namespace dpcull::pf;
  std::vector<Box> boxes(n);
  uint32_t key[7] = {0, 0, 0, 0, 0, 0, 0};
  for (size_t i = 0; i < n; ++i) {
    const float* m = mats + 16 * (size_t)idx[i];
    const F4 m0{m[0], m[1], m[2], m[3]}, m1{m[4], m[5], m[6], m[7]};
    const F4 m2{m[8], m[9], m[10], m[11]}, m3{m[12], m[13], m[14], m[15]};
    const Box b = box_of(lower[i], lower[n + i], lower[2 * n + i], extent[i], extent[n + i],
                           extent[2 * n + i], m0, m1, m2, m3);
    boxes[i] = b;
    if (b.d0 == b.d0) {
      const uint32_t k3[3] = {bound_key(b.cx), bound_key(b.cy), bound_key(b.cz)};
      for (int a = 0; a < 3; ++a) {
        key[a] = std::max(key[a], k3[a]);
        key[3 + a] = std::max(key[3 + a], ~k3[a]);
      }
      key[6] = std::max(key[6], bound_key(b.d0));
    }
  }
  float lo[3], hi[3];
  for (int a = 0; a < 3; ++a) {
    hi[a] = bound_value(key[a]);
    lo[a] = bound_value(~key[3 + a]);
  }
  const float d0max = bound_value(key[6]);
  GroupMargin gm{0.f, 0.f};
  std::vector<Planes> planes(n_views);
  for (size_t v = 0; v < n_views; ++v) {
    GroupMargin m;
    group_view(vps + 16 * v, planes[v], m);
    gm = merge(gm, m);
  }
  for (size_t v = 0; v < n_views; ++v) {
    const Planes& p = planes[v];
    clear[v] = far_plane_clear(p.q[2][1], lo, hi, d0max, gm) ? 1 : 0;
    bad[v] = 0;
    if (!clear[v]) continue;
    for (size_t i = 0; i < n; ++i) {
      const Box& b = boxes[i];
      if (!(b.d0 == b.d0)) continue;
      float D, T;
      group_thresholds(b, gm, D, T);
      const float zh = plane(b, p.q[2][1]);
      uint32_t v6 = 0, u6 = 0, v5 = 0, u5 = 0;
      const float xl = plane(b, p.q[0][0]), xh = plane(b, p.q[0][1]);
      const float yl = plane(b, p.q[1][0]), yh = plane(b, p.q[1][1]), zl = plane(b, p.q[2][0]);
      decide_bits<1u>(xl, xh, yl, yh, zl, zh, D, -T, v6, u6);
      decide_bits5<1u>(xl, xh, yl, yh, zl, D, -T, v5, u5);
      if (!(zh > D) || v5 != v6 || u5 != u6) ++bad[v];
    }
  }
}

// Random bounds, planes and margins: where far_plane_clear holds, the plane value of the
// bound's corners and of random centres inside it, in the kernel's FMA order, must exceed
// D for every margin up to d0max.  Returns the clear cases; *violations counts failures.
extern "C" int64_t pf_far_fuzz(uint64_t seed, int64_t trials, int64_t* violations)
{
  using namespace dpcull::pf;
  uint64_t s = seed * 0x9E3779B97F4A7C15ull + 1;
  auto next = [&]() {
    s ^= s << 13;
    s ^= s >> 7;
    s ^= s << 17;
    return s;
  };
  auto unit = [&]() { return (double)(next() >> 11) * 0x1p-53; };       // [0, 1)
  auto sym = [&]() { return 2.0 * unit() - 1.0; };                       // [-1, 1)
  auto mag = [&]() { return std::ldexp(1.0, (int)(next() % 40) - 20); };  // 2^-20 .. 2^19
  int64_t cleared = 0;
  *violations = 0;
  for (int64_t t = 0; t < trials; ++t) {
    float lo[3], hi[3];
    const double scale = mag();
    for (int a = 0; a < 3; ++a) {
      const float c = (float)(sym() * scale), h = (float)(unit() * scale);
      lo[a] = c - h;
      hi[a] = c + h;
    }
    const double dir[3] = {sym(), sym(), sym()};
    const double len = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]) + 1e-30;
    const double qs = (next() & 1) ? 1.0 : unit();  // unit normal, or the far plane's shorter one
    F4 q{(float)(dir[0] / len * qs), (float)(dir[1] / len * qs), (float)(dir[2] / len * qs), 0.f};
    // offset: from well inside to just past the bound, scaled like the bound
    q.w = (float)((next() % 4 == 0 ? sym() : unit()) * scale * 4.0 + scale * 1.7 * qs);
    const GroupMargin m{(float)(unit() * 0x1p-18), (float)(unit() * scale * 0x1p-20)};
    const float d0max = (float)(unit() * scale * 0x1p-18);
    if (!far_plane_clear(q, lo, hi, d0max, m)) continue;
    ++cleared;
    for (int k = 0; k < 24; ++k) {
      Box b{};
      float c[3];  // the 8 corners of the bound, then random points inside it
      for (int a = 0; a < 3; ++a) {
        c[a] = k < 8 ? (((k >> a) & 1) ? hi[a] : lo[a]) : lo[a] + (float)unit() * (hi[a] - lo[a]);
        c[a] = std::fmin(std::fmax(c[a], lo[a]), hi[a]);
      }
      b.cx = c[0];
      b.cy = c[1];
      b.cz = c[2];
      b.d0 = (float)(unit() * d0max);
      if (k == 8) b.d0 = d0max;
      float D, T;
      b.r = 0.f;
      group_thresholds(b, m, D, T);
      if (!(plane(b, q) > D)) ++*violations;
    }
  }
  return cleared;
}
