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
// Planes (per view).  For plane k (axis a, side lo/hi): Pi_k = col_a + col_w (lo) or
// col_w - col_a (hi), B_a[i] = |col_a[i]| + |col_w[i]| (so |Pi_i| <= B_a[i]),
// Nx_a = ||B_a,xyz||, Bw_a = B_a[w].  The stored plane is Q = fl(fl(Pi) * r_k) with
// r_k = fl(1 / n_k); hence Q = r_k Pi + eps, |eps_i| <= 2.01u r_k |Pi_i|.  The five planes
// other than z-hi (class A) use n_k >= ||Pi_k,xyz||, so ||Q_xyz|| <= 1 + 3.1u; the z-hi
// plane (class B: the far plane of a perspective view, often nearly pure w) uses
// n_k >= Nx_z and keeps q >= ||Q_xyz|| (<= 1 + 3.1u).  Per class, kappa >= r_k Nx_a and
// rho >= r_k Bw_a (the largest over the class's planes) give the margin terms below.
//
// Box (per object).  Only affine world matrices (column w = (0, 0, 0, 1), every matrix
// of the reference's scene graph) are bounded; a box with a projective matrix gets a NaN
// margin and all its pairs take the exact test.  Then X_w = Y_w = Z_w = 0 and p_w = 1.
// b_j = sum_i (|l_i| + |e_i|) |M_ij| + |M_3j| bounds every magnitude involved
// (|p_j| + |X_j| + |Y_j| + |Z_j| <= (1 + 5.01u) b_j); Bxyz >= ||b_xyz|| and b_w = 1.  For
// plane k, with S_a = sum_j b_j B_a[j]: r_k S_a <= r_k (Bxyz Nx_a + Bw_a) <= Bxyz kappa +
// rho (Cauchy-Schwarz on xyz only: the view's translation row lives in w, apart from the
// objects' xyz magnitudes).  The centre K = p + (X + Y + Z) / 2 is the mean of the 8
// corners.  We compute c~ = (l + e/2) * M with FMAs (c~_w = 1 exactly): |c~_j - K_j| <=
// 9.7u b_j.  R >= (||X_xyz|| + ||Y_xyz|| + ||Z_xyz||) / 2, so for every corner C_s.Q lies
// in K.Q +- E with E = R q (|X.Q| <= ||X_xyz|| ||Q_xyz|| as X_w = 0); the stored radius
// r' = R (1 + 2^-18) >= E / (1 - u) for every class-A plane (q <= 1 + 3.1u).
//
// Errors, in the plane's units (all of the form u r_k S_a):
//   |r (c_a + c_w)_s - r C_s.Pi| <= 7.04u r S_a   (the reference's dot products and add
//                                                  chain, 7u sum_j a_j B_a[j]),
//   |C_s.eps| <= 2.02u r S_a,
//   |L - K.Q| <= 13.75u r S_a   (L = fl(c~.Q), an FMA chain: 9.72u + 4.02u),
// so every r (c_a + c_w)_s (and the hi analogue c_w - c_a) is within
// 22.9u (Bxyz kappa + rho) of the real value that L and E describe.  The margins are
// D = d0 kappa + g per class with d0 = delta Bxyz + eta per box and g = delta rho per view,
// delta = 2^-19 = 32u, which also absorbs the roundings of D and of the thresholds below
// (each a relative u of the tested quantity); eta = 2^-120 absorbs subnormal rounding.
//
// Decisions (for one view; T_A = fl(D_A + r'), u = fl(L_zhi + R q)):
//   * visible   if L > D_A for the class-A planes and L_zhi > D_B: the corner mean K is
//     inside every plane, so for each plane some corner has a strictly positive rounded
//     value and no cfa bit can be set;
//   * invisible if some lo plane has L <= -T_A (every corner passes the lo test), or the
//     x-hi / y-hi plane has L <= -T_A while its lo plane has L >= T_A (every corner fails
//     the lo test and passes the hi test), or u <= -D_B while the z-lo plane has
//     L >= T_A;
//   * otherwise undecided.
// The bounds need finite values without overflow: a box whose Bxyz is not below 2^50 (or
// is NaN) gets d0 = NaN, and a view whose entries are not finite, whose plane or axis
// norms are not in [2^-60, 2^50) or whose kappa or rho is not below 2^50 gets NaN
// margins; every pair of either is undecided (no comparison with a NaN margin holds).
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

// Prefilter planes of one view (112 bytes, staged in shared memory by the cull).
struct Planes {
  F4 q[3][2];  // axis a: lo plane, hi plane
  F4 m;        // (kappa_A, g_A, kappa_B, g_B); the g are NaN when the view cannot be bounded
  F4 qf;       // (q of the z-hi plane, 0, 0, 0)
};

// Builds the planes of a row-major Mat44f view-projection; false when the view cannot be
// bounded (its pairs then all take the exact test).
DPCULL_HD bool make_planes(const float* vp, Planes& out)
{
  bool ok = true;
  for (int i = 0; i < 16; ++i) ok = ok && std::isfinite(vp[i]);
  float kA = 0.f, rA = 0.f, kB = 0.f, rB = 0.f, qf = 0.f;
  for (int a = 0; a < 3; ++a) {
    float B[4], pl[2][4];
    for (int i = 0; i < 4; ++i) {
      const float ca = vp[4 * i + a], cw = vp[4 * i + 3];
      B[i] = std::fabs(ca) + std::fabs(cw);
      pl[0][i] = ca + cw;
      pl[1][i] = cw - ca;
    }
    const float nx = bound_norm(B[0], B[1], B[2]) * kInflate;
    ok = ok && nx < kLimit && nx >= kTiny;
    for (int h = 0; h < 2; ++h) {
      const bool far = a == 2 && h == 1;
      const float n = far ? nx : bound_norm(pl[h][0], pl[h][1], pl[h][2]) * kInflate;
      ok = ok && n < kLimit && n >= kTiny;
      const float r = ok ? 1.0f / n : 0.f;
      const F4 q = {pl[h][0] * r, pl[h][1] * r, pl[h][2] * r, pl[h][3] * r};
      out.q[a][h] = q;
      const float kap = nx * r * kInflate, rho = B[3] * r * kInflate;
      if (far) {
        kB = kap;
        rB = rho;
        qf = bound_norm(q.x, q.y, q.z) * kInflate;
      } else {
        kA = std::fmax(kA, kap);
        rA = std::fmax(rA, rho);
      }
    }
  }
  ok = ok && kA < kLimit && rA < kLimit && kB < kLimit && rB < kLimit;
  // A NaN g makes every margin of the view NaN: no comparison holds, nothing is decided.
  const float nan = nan_value();
  out.m = F4{kA, ok ? kDelta * rA * kInflate : nan, kB, ok ? kDelta * rB * kInflate : nan};
  out.qf = F4{qf, 0.f, 0.f, 0.f};
  return ok;
}

// Prefilter box of one object: centre c (c.w == 1), radius r' = R (1 + 2^-18) and margin
// d0 (NaN when the bounds do not apply, including every box with a projective world
// matrix).
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
  return (m0.w == 0.f) & (m1.w == 0.f) & (m2.w == 0.f) & (m3.w == 1.f);  // no branches
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
  b.r = 0.5f * kInflate * (aex * n0 + aey * n1 + aez * n2) * kInflate;
  const float sx = std::fabs(lx) + aex, sy = std::fabs(ly) + aey, sz = std::fabs(lz) + aez;
  const float bxyz = kInflate * (sx * n0 + sy * n1 + sz * n2 +
                                 (std::fabs(m3.x) + std::fabs(m3.y) + std::fabs(m3.z)));
  b.d0 = ((bxyz < kLimit) & is_affine(m0, m1, m2, m3)) ? std::fma(kDelta, bxyz, kEta) : nan_value();
  return b;
}

// A tighter radius for boxes that are built once and kept (the group's box cache): every
// corner offset from the centre is (s1 X + s2 Y + s3 Z) / 2, so R may be half the largest
// of the four norms ||s1 X + s2 Y + Z|| (the 8 sign patterns in +- pairs) instead of
// (||X|| + ||Y|| + ||Z||) / 2 -- up to sqrt(3) smaller for the rotations and scales of a
// scene graph.  Each component of s1 X + s2 Y + Z is computed from the reference's rounded
// X_j = fl(ex M_0j) (exact up to the sign) and two FMAs with the exact products e M, so it
// is within 3u (|X_j| + |Y_j| + |Z_j|) of the real value, and the error vector's norm is
// at most 3u (||X|| + ||Y|| + ||Z||) <= 6u R_loose; the added 2^-20 r_loose covers it.
// Each norm is bounded like row_norm (sqrt_bound, then 2^-18), and the result is inflated
// by (1 + 2^-18) twice like the loose radius.  Never above r_loose (a NaN gives r_loose).
DPCULL_HD float tight_radius(float ex, float ey, float ez, const F4& m0, const F4& m1, const F4& m2, float r_loose)
{
  const float X[3] = {ex * m0.x, ex * m0.y, ex * m0.z};
  float nmax = 0.f;
  for (int s = 0; s < 4; ++s) {
    const float sx = (s & 1) ? -1.f : 1.f, sy = (s & 2) ? -ey : ey;
    const float vx = std::fma(ez, m2.x, std::fma(sy, m1.x, sx * X[0]));
    const float vy = std::fma(ez, m2.y, std::fma(sy, m1.y, sx * X[1]));
    const float vz = std::fma(ez, m2.z, std::fma(sy, m1.z, sx * X[2]));
    nmax = std::fmax(nmax, sqrt_bound(std::fma(vx, vx, std::fma(vy, vy, std::fma(vz, vz, 0x1p-120f)))) * kInflate);
  }
  const float r = (0.5f * nmax + r_loose * 0x1p-20f) * kInflate * kInflate;
  return std::fmin(r, r_loose);
}

// Plane value L = c.Q (c.w == 1: Q_w is the addend).
DPCULL_HD float plane(const Box& b, const F4& q)
{
  return std::fma(b.cz, q.z, std::fma(b.cy, q.y, std::fma(b.cx, q.x, q.w)));
}

// A view's planes in registers, read once for several boxes.
struct PlaneRegs {
  F4 xl, xh, yl, yh, zl, zh, m;
  float qf;
};

DPCULL_HD PlaneRegs load_planes(const Planes& p)
{
  return PlaneRegs{p.q[0][0], p.q[0][1], p.q[1][0], p.q[1][1], p.q[2][0], p.q[2][1], p.m, p.qf.x};
}

// All ones when the comparison holds, zero otherwise (false with a NaN operand, like the
// C++ comparison); on the GPU one set.*.u32.f32 instruction.
DPCULL_HD uint32_t mask_gt(float a, float b)
{
#if defined(__CUDA_ARCH__)
  uint32_t r;
  asm("set.gt.u32.f32 %0, %1, %2;" : "=r"(r) : "f"(a), "f"(b));
  return r;
#else
  return a > b ? ~0u : 0u;
#endif
}

DPCULL_HD uint32_t mask_le(float a, float b)
{
#if defined(__CUDA_ARCH__)
  uint32_t r;
  asm("set.le.u32.f32 %0, %1, %2;" : "=r"(r) : "f"(a), "f"(b));
  return r;
#else
  return a <= b ? ~0u : 0u;
#endif
}

DPCULL_HD uint32_t mask_ge(float a, float b)
{
#if defined(__CUDA_ARCH__)
  uint32_t r;
  asm("set.ge.u32.f32 %0, %1, %2;" : "=r"(r) : "f"(a), "f"(b));
  return r;
#else
  return a >= b ? ~0u : 0u;
#endif
}

// The decisions of the comment at the top for one box in one view, from its six plane
// values (lo / hi of x, y, z), as all-ones / zero masks.
DPCULL_HD void decide_masks(const Box& b, float xl, float xh, float yl, float yh, float zl, float zh,
                            const F4& m, float qf, uint32_t& visible, uint32_t& invisible)
{
  const float da = std::fma(b.d0, m.x, m.y), db = std::fma(b.d0, m.z, m.w);
  const float ta = da + b.r;
  const float uf = std::fma(b.r, qf, zh);
  const float mlo = std::fmin(std::fmin(xl, yl), zl);
  const float min_in = std::fmin(std::fmin(mlo, xh), yh);
  const float o = std::fmin(mlo, std::fmin(std::fmax(xh, -xl), std::fmax(yh, -yl)));
  visible = mask_gt(min_in, da) & mask_gt(zh, db);
  invisible = mask_le(o, -ta) | (mask_le(uf, -db) & mask_ge(zl, ta));
}

DPCULL_HD void decide_values(const Box& b, float xl, float xh, float yl, float yh, float zl, float zh,
                             const F4& m, float qf, bool& visible, bool& invisible)
{
  uint32_t vis, inv;
  decide_masks(b, xl, xh, yl, yh, zl, zh, m, qf, vis, inv);
  visible = vis != 0;
  invisible = inv != 0;
}

DPCULL_HD void decide(const Box& b, const PlaneRegs& p, bool& visible, bool& invisible)
{
  decide_values(b, plane(b, p.xl), plane(b, p.xh), plane(b, p.yl), plane(b, p.yh), plane(b, p.zl),
                plane(b, p.zh), p.m, p.qf, visible, invisible);
}

enum : int { kInvisible = 0, kVisible = 1, kUndecided = 2 };

// ---- decisions against the margin of a group of views -----------------------------------
// The kernels evaluate up to 8 views per object load.  Instead of each view's own margin
// classes they use the largest kappa and g over all six planes of every view of the group
// (K, G): every margin grows, so every decision stays one of the decisions above.  The
// far plane keeps its normalisation (class B); its radius term R q (q <= 1 + 3.1u) is
// covered by the class-A inflated radius r'.  Then one pair of thresholds per box serves
// every plane of every view of the group: D = fl(d0 K + G), T = fl(D + r').
//   visible   if all six plane values exceed D;
//   invisible if some lo plane value is <= -T, or for some axis the hi value is <= -T
//             while the lo value is >= T (max(hi, -lo) <= -T).
// A view that cannot be bounded gets NaN planes: NaN plane values fail both tests (the
// minima and maxima of NaNs are NaN), so each of its pairs is undecided whatever the
// group's margin.
struct GroupMargin {
  float k, g;
};

// The planes of one view for a group decision and the view's contribution to the group
// margin (0 for a view that cannot be bounded).
DPCULL_HD bool group_view(const float* vp, Planes& p, GroupMargin& m)
{
  const bool ok = make_planes(vp, p);
  if (ok) {
    m.k = std::fmax(p.m.x, p.m.z);
    m.g = std::fmax(p.m.y, p.m.w);
  } else {
    const float nan = nan_value();
    for (int a = 0; a < 3; ++a)
      for (int h = 0; h < 2; ++h) p.q[a][h] = F4{nan, nan, nan, nan};
    m.k = 0.f;
    m.g = 0.f;
  }
  return ok;
}

DPCULL_HD GroupMargin merge(const GroupMargin& a, const GroupMargin& b)
{
  return GroupMargin{std::fmax(a.k, b.k), std::fmax(a.g, b.g)};
}

// Thresholds of one box against a group margin (NaN when the box cannot be bounded).
// D >= +0 otherwise: d0, the group's kappa and g are never negative (unbounded views
// contribute zeros to the margin), so D is an FMA of non-negative terms.
DPCULL_HD void group_thresholds(const Box& b, const GroupMargin& m, float& D, float& T)
{
  D = std::fma(b.d0, m.k, m.g);
  T = D + b.r;
}

// The group decision from the six plane values, as bits: ORs BIT into `visible` when the
// pair is decided visible and into `undecided` when it is decided neither visible nor
// invisible.  Visible if all six plane values are above D; invisible if the box is outside
// a lo plane, or outside a hi plane with every corner inside its lo plane (the reference's
// `else if`), by T: o <= -T with o = min(xl, yl, zl, max(xh, -xl), max(yh, -yl),
// max(zh, -zl)); a NaN comparison decides nothing.  One value serves both tests: D >= 0
// (or NaN), and then "all six > D" <=> o > D (if every value is above D >= 0, each -lo is
// negative and each max(hi, -lo) is hi; if o > D, every lo value is above 0, so each
// max(hi, -lo) above D is hi).  negT = -T.  On the GPU each bit costs one comparison and
// one predicated OR (the undecided comparison is "greater than or unordered", i.e.
// !(o <= -T), combined with !vis in the same setp).
template <uint32_t BIT>
DPCULL_HD void decide_bits(float xl, float xh, float yl, float yh, float zl, float zh, float D, float negT,
                           uint32_t& visible, uint32_t& undecided)
{
  const float o = std::fmin(std::fmin(std::fmin(xl, yl), std::fmin(zl, std::fmax(xh, -xl))),
                            std::fmin(std::fmax(yh, -yl), std::fmax(zh, -zl)));
#if defined(__CUDA_ARCH__)
  asm("{\n\t.reg .pred pv, pu;\n\t"
      "setp.gt.f32 pv, %2, %3;\n\t"
      "setp.gtu.and.f32 pu, %2, %4, !pv;\n\t"
      "@pv or.b32 %0, %0, %5;\n\t"
      "@pu or.b32 %1, %1, %5;\n\t}"
      : "+r"(visible), "+r"(undecided)
      : "f"(o), "f"(D), "f"(negT), "n"(BIT));
#else
  const bool vis = o > D;
  if (vis) visible |= BIT;
  else if (!(o <= negT)) undecided |= BIT;
#endif
}

// ---- leaving out the far plane --------------------------------------------------------
// A group whose box cache is valid also keeps a bound of its scene (the box [lo, hi] of the
// prefilter-box centres and the largest margin d0, over every box whose d0 is a number:
// the pairs of the others are undecided whatever their plane values).  When the z-hi
// plane value of every box in that bound is above its threshold D, that plane changes no
// decision: max(zh, -zl) >= zh > D >= 0 >= -T, so with it o > D holds exactly when it
// holds without it, and o <= -T likewise.  The cached kernel then evaluates five planes:
// decide_bits5 gives the same bits as decide_bits for every box of the scene.
//
// far_plane_clear shows zh > D for every centre c in [lo, hi] and every d0 <= d0max
// (D = fl(d0 K + G) grows with d0 as K >= 0).  The exact minimum of c.Q over the box is
// Q_w + sum_k min(Q_k lo_k, Q_k hi_k); the kernel's FMA chain for zh and the sum below each
// round by less than 4u M, M = |Q_w| + sum_k |Q_k| max(|lo_k|, |hi_k|), and the test keeps
// 2^-16 M = 256u M in hand.  Any NaN (an empty bound, a view that cannot be bounded) makes
// it false.
DPCULL_HD bool far_plane_clear(const F4& q, const float (&lo)[3], const float (&hi)[3], float d0max,
                               const GroupMargin& m)
{
  const float qa[3] = {q.x, q.y, q.z};
  float lb = q.w, mag = std::fabs(q.w);
  for (int k = 0; k < 3; ++k) {
    const float a = qa[k] * lo[k], b = qa[k] * hi[k];
    lb += a < b ? a : b;  // a NaN product makes lb NaN (no fmin: it would drop the NaN)
    mag += std::fabs(qa[k]) * std::fmax(std::fabs(lo[k]), std::fabs(hi[k]));
  }
  return lb - mag * 0x1p-16f > std::fma(d0max, m.k, m.g);
}

// decide_bits without the z-hi plane, for boxes whose scene bound passed far_plane_clear.
template <uint32_t BIT>
DPCULL_HD void decide_bits5(float xl, float xh, float yl, float yh, float zl, float D, float negT,
                            uint32_t& visible, uint32_t& undecided)
{
  const float o = std::fmin(std::fmin(std::fmin(xl, yl), zl), std::fmin(std::fmax(xh, -xl), std::fmax(yh, -yl)));
#if defined(__CUDA_ARCH__)
  asm("{\n\t.reg .pred pv, pu;\n\t"
      "setp.gt.f32 pv, %2, %3;\n\t"
      "setp.gtu.and.f32 pu, %2, %4, !pv;\n\t"
      "@pv or.b32 %0, %0, %5;\n\t"
      "@pu or.b32 %1, %1, %5;\n\t}"
      : "+r"(visible), "+r"(undecided)
      : "f"(o), "f"(D), "f"(negT), "n"(BIT));
#else
  const bool vis = o > D;
  if (vis) visible |= BIT;
  else if (!(o <= negT)) undecided |= BIT;
#endif
}

// Order-preserving keys of the scene bound (the cache's bound words; all zero = empty):
// key(f) grows with f, so atomicMax of key(c) keeps the largest centre and atomicMax of
// ~key(c) the smallest.  NaN keys decode to NaN.
DPCULL_HD uint32_t bound_key(float f)
{
  uint32_t b;
  memcpy(&b, &f, sizeof b);
  return (b & 0x80000000u) ? ~b : b | 0x80000000u;
}

DPCULL_HD float bound_value(uint32_t key)
{
  const uint32_t b = (key & 0x80000000u) ? key & 0x7FFFFFFFu : ~key;
  float f;
  memcpy(&f, &b, sizeof f);
  return f;
}

// Whole classification of one box in one view of a group with margin m.
DPCULL_HD int classify_group(const Box& b, const Planes& p, const GroupMargin& m)
{
  float D, T;
  group_thresholds(b, m, D, T);
  uint32_t vis = 0, und = 0;
  decide_bits<1u>(plane(b, p.q[0][0]), plane(b, p.q[0][1]), plane(b, p.q[1][0]), plane(b, p.q[1][1]),
                  plane(b, p.q[2][0]), plane(b, p.q[2][1]), D, -T, vis, und);
  return vis ? kVisible : und ? kUndecided : kInvisible;
}



// Whole classification of one box in one view (the kernels run decide() with the view's
// planes loaded once for several boxes).
DPCULL_HD int classify(const Box& b, const Planes& p)
{
  bool vis, inv;
  decide(b, load_planes(p), vis, inv);
  return vis ? kVisible : inv ? kInvisible : kUndecided;
}

}  // namespace pf
}  // namespace dpcull
