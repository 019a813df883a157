// dpcull_prefilter.h -- conservative frustum classification that never contradicts the
// reference's rounded box test (dp/culling/cpu/src/ManagerImpl.cpp:199-229,263-289).
//
// The cull decides most (object, view) pairs here, with a few FMA-pipe operations and
// min/max, and sends only the pairs this test cannot decide through the exact test in the
// reference's operation order (dpcull_exact.cuh).  Plain C++ on float: the same source is
// compiled into the CUDA kernels and into a host test that checks it against the oracle.
//
// Notation.  The reference's cached box is the float 4-vectors p = (lower,1)*M and
// X = ex*M_0, Y = ey*M_1, Z = ez*M_2 (M_i = row i of the world matrix).  Its 8 real
// corners are C_s = p + s1 X + s2 Y + s3 Z; the reference evaluates rounded corners c_s =
// fl(p*VP) + fl(X*VP) + ... (its add chain).  For an axis a in {x, y, z} with VP column
// col_a and col_w, the reference's "lo" test on a corner is c_a <= -c_w, i.e.
// c_a + c_w <= 0, and its "hi" test is !(c_a + c_w <= 0) && c_w - c_a <= 0.  A cfa bit
// (ManagerImpl.cpp:224-227) is set when every corner has it; visible <=> no cfa bit.
// u = 2^-24.
//
// Planes (per view).  Pi_lo = col_a + col_w, Pi_hi = col_w - col_a, B_a[i] = |col_a[i]| +
// |col_w[i]| (so |Pi_i| <= B_a[i]), Nx_a = ||B_a,xyz||, Bw_a = B_a[w].  The stored plane
// is Q = fl(fl(Pi) * r), r = fl(1 / Nx'_a) with Nx'_a >= Nx_a; hence Q = r Pi + eps,
// |eps_i| <= 2.01u r |Pi_i|, r Nx_a <= 1 + u and ||Q_xyz|| <= 1 + 3.1u.  Stored with it:
// q >= ||Q_xyz|| and, per view, g = delta rho with rho >= max_a Bw_a / Nx'_a.
//
// Box (per object).  Only affine world matrices (column w = (0, 0, 0, 1), every matrix
// of the reference's scene graph) are bounded; a box with a projective matrix gets a NaN
// margin and all its pairs take the exact test.  Then X_w = Y_w = Z_w = 0 and p_w = 1.
// b_j = sum_i (|l_i| + |e_i|) |M_ij| + |M_3j| bounds every magnitude involved
// (|p_j| + |X_j| + |Y_j| + |Z_j| <= (1 + 5.01u) b_j); Bxyz >= ||b_xyz|| and b_w = 1.  For
// every axis, with S_a = sum_j b_j B_a[j]: r S_a <= r (Bxyz Nx_a + Bw_a) <= (1 + u) Bxyz +
// rho (Cauchy-Schwarz on xyz only: the view's translation row lives in w, apart from the
// objects' xyz magnitudes).  The centre K = p + (X + Y + Z) / 2 is the mean of the 8
// corners.  We compute c~ = (l + e/2) * M with FMAs (c~_w = 1 exactly): |c~_j - K_j| <=
// 9.7u b_j.  R >= (||X_xyz|| + ||Y_xyz|| + ||Z_xyz||) / 2, so for every corner C_s.Q lies
// in K.Q +- E with E = R q (|X.Q| <= ||X_xyz|| ||Q_xyz|| as X_w = 0).
//
// Errors, in the plane's units (all of the form u r S_a):
//   |r (c_a + c_w)_s - r C_s.Pi| <= 7.04u r S_a   (the reference's dot products and add
//                                                  chain, 7u sum_j a_j B_a[j]),
//   |C_s.eps| <= 2.02u r S_a,
//   |L - K.Q| <= 13.75u r S_a   (L = fl(c~.Q), an FMA chain: 9.72u + 4.02u),
// so every r (c_a + c_w)_s (and the hi analogue c_w - c_a) is within 22.9u (Bxyz + rho) of
// the real value that L and E describe.  The margin is D = d0 + g with d0 = delta Bxyz +
// eta per box and g = delta rho per view, delta = 2^-19 = 32u, which also absorbs the
// roundings of D and of t = fl(L + E), s = fl(L - E) (each a relative u of the tested
// quantity); eta = 2^-120 absorbs subnormal rounding.
//
// Decisions (for one view):
//   * visible   if L > D for all six planes: the corner mean K is inside every plane, so
//     for each plane some corner has a strictly positive rounded value and no cfa bit can
//     be set;
//   * invisible if for some axis t_lo = fl(L_lo + E_lo) <= -D (every corner passes the lo
//     test), or t_hi <= -D and s_lo = fl(L_lo - E_lo) >= D (every corner fails the lo
//     test and passes the hi test);
//   * otherwise undecided.
// The bounds need finite values without overflow: a box whose Bxyz is not below 2^50 (or
// is NaN) gets d0 = NaN, and a view whose entries are not finite, whose Nx'_a is not in
// [2^-60, 2^50) or whose rho is not below 2^50 gets g = NaN; every pair of either is
// undecided (no comparison with a NaN margin holds).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define DPCULL_HD __host__ __device__ __forceinline__
#else
#define DPCULL_HD inline
#endif

namespace dpcull {
namespace pf {

#ifdef DPCULL_PF_TEST_DELTA
// Host tests only: a deliberately weakened margin, to show that the tests can see one.
constexpr float kDelta = DPCULL_PF_TEST_DELTA;
#else
constexpr float kDelta = 0x1p-19f;
#endif
constexpr float kInflate = 1.0f + 0x1p-18f;
#ifdef DPCULL_PF_TEST_DELTA
constexpr float kEta = 0.f;
#else
constexpr float kEta = 0x1p-120f;
#endif
constexpr float kLimit = 0x1p50f;
constexpr float kTiny = 0x1p-60f;

struct alignas(16) F4 {
  float x, y, z, w;
};

DPCULL_HD float nan_value()
{
  const uint32_t bits = 0x7fc00000u;
  float f;
  memcpy(&f, &bits, sizeof f);
  return f;
}

// Upper bound of the Euclidean norm of (x, y, z, w): the inflated square root of the FMA
// sum of squares, or the inflated L1 norm when the squares could underflow.
DPCULL_HD float bound_norm(float x, float y, float z, float w = 0.f)
{
  const float l1 = (std::fabs(x) + std::fabs(y) + std::fabs(z) + std::fabs(w)) * kInflate;
  if (l1 < kTiny) return l1 * kInflate;
  return std::sqrt(std::fma(x, x, std::fma(y, y, std::fma(z, z, w * w)))) * kInflate;
}

// Prefilter planes of one view (128 bytes, staged in shared memory by the cull).
struct Planes {
  F4 q[3][2];  // axis a: lo plane Q_lo, hi plane Q_hi
  F4 n01;      // (q_lo, q_hi) of axes x and y
  F4 n2g;      // (q_lo, q_hi) of axis z, then g (NaN when the view cannot be bounded), 0
  DPCULL_HD float qlo(int a) const { return a == 0 ? n01.x : a == 1 ? n01.z : n2g.x; }
  DPCULL_HD float qhi(int a) const { return a == 0 ? n01.y : a == 1 ? n01.w : n2g.y; }
};

// Builds the planes of a row-major Mat44f view-projection; false when the view cannot be
// bounded (its pairs then all take the exact test).
DPCULL_HD bool make_planes(const float* vp, Planes& out)
{
  bool ok = true;
  for (int i = 0; i < 16; ++i) ok = ok && std::isfinite(vp[i]);
  float rho = 0.f, qn[3][2];
  for (int a = 0; a < 3; ++a) {
    float B[4], lo[4], hi[4];
    for (int i = 0; i < 4; ++i) {
      const float ca = vp[4 * i + a], cw = vp[4 * i + 3];
      B[i] = std::fabs(ca) + std::fabs(cw);
      lo[i] = ca + cw;
      hi[i] = cw - ca;
    }
    const float nx = bound_norm(B[0], B[1], B[2]) * kInflate;
    ok = ok && nx < kLimit && nx >= kTiny;
    const float r = ok ? 1.0f / nx : 0.f;
    rho = std::fmax(rho, B[3] * r * kInflate);
    const F4 ql = {lo[0] * r, lo[1] * r, lo[2] * r, lo[3] * r};
    const F4 qh = {hi[0] * r, hi[1] * r, hi[2] * r, hi[3] * r};
    out.q[a][0] = ql;
    out.q[a][1] = qh;
    qn[a][0] = bound_norm(ql.x, ql.y, ql.z) * kInflate;
    qn[a][1] = bound_norm(qh.x, qh.y, qh.z) * kInflate;
  }
  ok = ok && rho < kLimit;
  // A NaN g makes every margin of the view NaN: no comparison holds, nothing is decided.
  const float g = ok ? kDelta * rho * kInflate : nan_value();
  out.n01 = F4{qn[0][0], qn[0][1], qn[1][0], qn[1][1]};
  out.n2g = F4{qn[2][0], qn[2][1], g, 0.f};
  return ok;
}

// Prefilter box of one object: centre c (c.w == 1), extent bound R and margin d0 (NaN
// when the bounds do not apply, including every box with a projective world matrix).
struct Box {
  float cx, cy, cz;
  float r, d0;
};

// Square root for the upper bounds below: on the GPU the hardware approximation
// (sqrt.approx.f32; tests/test_gpu_prefilter_sqrt.py checks every input in [2^-120, 2^127]
// against the correctly rounded root: relative error below 2^-21, so the 2^-18 inflation
// that follows every use keeps the bound), on the host the correctly rounded one.
DPCULL_HD float sqrt_bound(float x)
{
#if defined(__CUDA_ARCH__)
  float r;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  return std::sqrt(x);
#endif
}

// Upper bound of ||(r.x, r.y, r.z)||: the 2^-120 addend keeps every partial sum normal.
DPCULL_HD float row_norm(const F4& m)
{
  return sqrt_bound(std::fma(m.x, m.x, std::fma(m.y, m.y, std::fma(m.z, m.z, 0x1p-120f)))) * kInflate;
}

// True when the matrix maps w = 1 to w = 1 and directions to w = 0 (no projective part).
DPCULL_HD bool is_affine(const F4& m0, const F4& m1, const F4& m2, const F4& m3)
{
  return m0.w == 0.f && m1.w == 0.f && m2.w == 0.f && m3.w == 1.f;
}

DPCULL_HD Box make_box(float lx, float ly, float lz, float ex, float ey, float ez, const F4& m0,
                       const F4& m1, const F4& m2, const F4& m3)
{
  const float cx0 = std::fma(0.5f, ex, lx), cy0 = std::fma(0.5f, ey, ly), cz0 = std::fma(0.5f, ez, lz);
  Box b;
  b.cx = std::fma(cz0, m2.x, std::fma(cy0, m1.x, std::fma(cx0, m0.x, m3.x)));
  b.cy = std::fma(cz0, m2.y, std::fma(cy0, m1.y, std::fma(cx0, m0.y, m3.y)));
  b.cz = std::fma(cz0, m2.z, std::fma(cy0, m1.z, std::fma(cx0, m0.z, m3.z)));
  const float n0 = row_norm(m0), n1 = row_norm(m1), n2 = row_norm(m2);
  const float aex = std::fabs(ex), aey = std::fabs(ey), aez = std::fabs(ez);
  b.r = 0.5f * kInflate * (aex * n0 + aey * n1 + aez * n2);
  const float sx = std::fabs(lx) + aex, sy = std::fabs(ly) + aey, sz = std::fabs(lz) + aez;
  const float bxyz = kInflate * (sx * n0 + sy * n1 + sz * n2 +
                                 (std::fabs(m3.x) + std::fabs(m3.y) + std::fabs(m3.z)));
  b.d0 = (bxyz < kLimit && is_affine(m0, m1, m2, m3)) ? std::fma(kDelta, bxyz, kEta) : nan_value();
  return b;
}

// One axis of one view for one box: folds the axis's planes into the running minima
//   mi = min over planes of L (the visible test), mo = min over axes of the invisible
//   candidate min(t_lo, max(t_hi, -s_lo)).
// c.w == 1: Q_w is the addend of L; E = R q, and t = fl(L + R q), s = fl(L - R q) are one
// rounding each.
template <bool kFirst = false>
DPCULL_HD void axis(const Box& b, const F4& ql, const F4& qh, float nl, float nh, float& mi,
                    float& mo)
{
  const float Ll = std::fma(b.cz, ql.z, std::fma(b.cy, ql.y, std::fma(b.cx, ql.x, ql.w)));
  const float Lh = std::fma(b.cz, qh.z, std::fma(b.cy, qh.y, std::fma(b.cx, qh.x, qh.w)));
  const float tl = std::fma(b.r, nl, Ll), sl = std::fma(-b.r, nl, Ll);
  const float th = std::fma(b.r, nh, Lh);
  if (kFirst) {  // the first axis starts the minima
    mo = std::fmin(tl, std::fmax(th, -sl));
    mi = std::fmin(Ll, Lh);
  } else {
    mo = std::fmin(mo, std::fmin(tl, std::fmax(th, -sl)));
    mi = std::fmin(mi, std::fmin(Ll, Lh));
  }
}

enum : int { kInvisible = 0, kVisible = 1, kUndecided = 2 };

// Whole classification of one box in one view (the kernels inline the same steps, with
// the view's planes shared by several boxes).
DPCULL_HD int classify(const Box& b, const Planes& p)
{
  const float d = b.d0 + p.n2g.z;
  float mi, mo;
  axis<true>(b, p.q[0][0], p.q[0][1], p.qlo(0), p.qhi(0), mi, mo);
  for (int a = 1; a < 3; ++a) axis(b, p.q[a][0], p.q[a][1], p.qlo(a), p.qhi(a), mi, mo);
  if (mi > d) return kVisible;
  if (mo <= -d) return kInvisible;
  return kUndecided;
}

}  // namespace pf
}  // namespace dpcull
