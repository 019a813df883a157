// Host build of the cull's conservative prefilter (pipeline_gb300/csrc/dpcull_prefilter.h),
// the same source the CUDA kernels compile, exported for tests/test_prefilter_host.py.
#include <cstddef>
#include <cstdint>

#include "dpcull_prefilter.h"

using dpcull::pf::F4;

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
    const dpcull::pf::Box b = dpcull::pf::make_box(lower[i], lower[n + i], lower[2 * n + i],
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
    const dpcull::pf::Box b = dpcull::pf::make_box(lower[i], lower[n + i], lower[2 * n + i],
                                                   extent[i], extent[n + i], extent[2 * n + i],
                                                   m0, m1, m2, m3);
    for (size_t v = 0; v < n_views && v < 64; ++v)
      out[v * n + i] = (int8_t)dpcull::pf::classify_group(b, planes[v], gm);
  }
}
