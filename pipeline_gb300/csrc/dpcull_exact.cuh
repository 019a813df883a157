// dpcull_exact.cuh -- FP32 arithmetic in the reference's exact operation order.
//
// Every multiply and add is an explicit round-to-nearest intrinsic (__fmul_rn /
// __fadd_rn), which the compiler never contracts into an FMA, so results are
// bit-identical to the reference CPU manager compiled without FMA contraction
// whatever the build flags.  Matrices are Mat44f in the reference layout: four float4
// rows, row-major, row-vector convention (v' = v * M).
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

namespace dpcull {

__device__ __forceinline__ float xmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float xadd(float a, float b) { return __fadd_rn(a, b); }

// One output column of Vec4 * Mat44 (dp/math/Matmnt.h:1371-1379):
// ((v0*m0j + v1*m1j) + v2*m2j) + v3*m3j.
__device__ __forceinline__ float dot_col(float v0, float v1, float v2, float v3, float m0,
                                         float m1, float m2, float m3)
{
  return xadd(xadd(xadd(xmul(v0, m0), xmul(v1, m1)), xmul(v2, m2)), xmul(v3, m3));
}

__device__ __forceinline__ float4 vec4_mul_mat44(float4 v, float4 r0, float4 r1, float4 r2,
                                                 float4 r3)
{
  return make_float4(dot_col(v.x, v.y, v.z, v.w, r0.x, r1.x, r2.x, r3.x),
                     dot_col(v.x, v.y, v.z, v.w, r0.y, r1.y, r2.y, r3.y),
                     dot_col(v.x, v.y, v.z, v.w, r0.z, r1.z, r2.z, r3.z),
                     dot_col(v.x, v.y, v.z, v.w, r0.w, r1.w, r2.w, r3.w));
}

// Same product with a matrix held in shared memory as 16 floats.
__device__ __forceinline__ float4 vec4_mul_mat44_s(float4 v, const float* m)
{
  const float4 r0 = *reinterpret_cast<const float4*>(m + 0);
  const float4 r1 = *reinterpret_cast<const float4*>(m + 4);
  const float4 r2 = *reinterpret_cast<const float4*>(m + 8);
  const float4 r3 = *reinterpret_cast<const float4*>(m + 12);
  return vec4_mul_mat44(v, r0, r1, r2, r3);
}

__device__ __forceinline__ float4 vadd4(float4 a, float4 b)
{
  return make_float4(xadd(a.x, b.x), xadd(a.y, b.y), xadd(a.z, b.z), xadd(a.w, b.w));
}

// Row times scalar: Vecnt.h:912-923 (operator*(s, v) -> v *= s per component).
__device__ __forceinline__ float4 vscale4(float4 r, float s)
{
  return make_float4(xmul(r.x, s), xmul(r.y, s), xmul(r.z, s), xmul(r.w, s));
}

// The cached world-space box of dp/culling/cpu/src/ManagerImpl.cpp:114-162:
// point = (lower, 1) * M, axis k = extent[k] * M row k.
struct Obb {
  float4 p, ex, ey, ez;
};

__device__ __forceinline__ Obb make_obb(float lx, float ly, float lz, float ex, float ey, float ez,
                                        float4 r0, float4 r1, float4 r2, float4 r3)
{
  Obb o;
  // The fourth term is 1.0f * M[3][j]; a product with 1.0f is exact, so it is M[3][j].
  o.p = make_float4(xadd(xadd(xadd(xmul(lx, r0.x), xmul(ly, r1.x)), xmul(lz, r2.x)), r3.x),
                    xadd(xadd(xadd(xmul(lx, r0.y), xmul(ly, r1.y)), xmul(lz, r2.y)), r3.y),
                    xadd(xadd(xadd(xmul(lx, r0.z), xmul(ly, r1.z)), xmul(lz, r2.z)), r3.z),
                    xadd(xadd(xadd(xmul(lx, r0.w), xmul(ly, r1.w)), xmul(lz, r2.w)), r3.w));
  o.ex = vscale4(r0, ex);
  o.ey = vscale4(r1, ey);
  o.ez = vscale4(r2, ez);
  return o;
}

// Clip-volume accumulator of determineCullFlags (ManagerImpl.cpp:199-229): a bit stays
// set only while every corner so far is outside that plane.  The "hi" test is the
// else-branch, so it only counts where the "lo" test failed.
struct ClipAcc {
  bool lx = true, hx = true, ly = true, hy = true, lz = true, hz = true;
  __device__ __forceinline__ void add(float4 c)
  {
    const bool ax = c.x <= -c.w, ay = c.y <= -c.w, az = c.z <= -c.w;
    lx &= ax;
    hx &= (!ax) & (c.w <= c.x);
    ly &= ay;
    hy &= (!ay) & (c.w <= c.y);
    lz &= az;
    hz &= (!az) & (c.w <= c.z);
  }
  // isVisible returns !cfo || !cfa; cfo == 0 forces cfa == 0, so this is cfa == 0.
  __device__ __forceinline__ bool visible() const { return !(lx | hx | ly | hy | lz | hz); }
};

// isVisible(projection, OBB): ManagerImpl.cpp:263-289, corner order and add chain kept.
__device__ __forceinline__ bool obb_visible(const Obb& o, const float* vp)
{
  const float4 v0 = vec4_mul_mat44_s(o.p, vp);
  const float4 x = vec4_mul_mat44_s(o.ex, vp);
  const float4 y = vec4_mul_mat44_s(o.ey, vp);
  const float4 z = vec4_mul_mat44_s(o.ez, vp);
  const float4 v1 = vadd4(v0, x);
  const float4 v2 = vadd4(v0, y);
  const float4 v3 = vadd4(v1, y);
  ClipAcc acc;
  acc.add(v0);
  acc.add(v1);
  acc.add(v2);
  acc.add(v3);
  acc.add(vadd4(v0, z));
  acc.add(vadd4(v1, z));
  acc.add(vadd4(v2, z));
  acc.add(vadd4(v3, z));
  return acc.visible();
}

// ---------------------------------------------------------------------------------------
// Conservative classification that never contradicts obb_visible().
//
// Let p, ex, ey, ez be the (float) box of make_obb and C_k = p + s ex + t ey + u ez the
// 8 exact real corners; obb_visible() evaluates rounded corners c_k.  With col_j column j
// of VP, the reference tests "lo a" (a = x, y, z) as c_a <= -c_w, i.e. c_a + c_w <= 0,
// and "hi a" as !(c_a <= -c_w) && c_w <= c_a.  Let Pi = col_a + col_w (lo) or
// col_w - col_a (hi) and B_a[i] = |col_a[i]| + |col_w[i]|.
//   * rounding: |(c_a + c_w) - (C_a + C_w)| <= 7u * sum_i a_i B_a[i] <= 7u * A * N_a,
//     u = 2^-24, a_i = |p_i|+|ex_i|+|ey_i|+|ez_i|, A = ||a||, N_a = ||B_a|| (the 4-term
//     dot products and the 3-add corner chain, then Cauchy-Schwarz); the same bound holds
//     for the hi test's c_w - c_a;
//   * extent: over the 8 corners, C.Pi lies within centre.Pi +- (Rxyz n + Rw m), centre =
//     p + (ex+ey+ez)/2, Rxyz = (||ex_xyz||+||ey_xyz||+||ez_xyz||)/2,
//     Rw = (|ex_w|+|ey_w|+|ez_w|)/2, n = ||Pi_xyz||, m = |Pi_w|, since
//     |e.Pi| <= ||e_xyz|| ||Pi_xyz|| + |e_w| |Pi_w| (Rw = 0 for affine world matrices);
//   * this test: L = fl(cc_a +- cc_w) with cc = fl(centre' . VP) (FMA chains, centre'
//     rounded) is within 9u * A * N_a of centre.Pi.
// So with T >= Rxyz n + Rw m + 16u A N_a: L <= -T proves every rounded corner outside
// that plane; "lo" outside sets the cfa bit (invisible); "hi" outside together with
// L_lo > T_lo (no corner satisfies the lo test) sets the hi bit (invisible); L > T for all
// six planes proves every corner strictly inside (cf = 0: visible).  Anything else is
// undecided and goes through obb_visible().
// Slack: the margin uses delta = 2^-19 = 32u for 16u; n and m come from Pi rounded in
// float (|fl(x+y)| >= |x+y| (1-u)) and, like every norm here, are inflated by 2^-18 and
// taken as the (inflated) L1 norm when tiny, so squares never underflow; eta = 2^-120
// absorbs subnormal rounding.  The bounds need finite values without overflow: a box with
// A >= 2^50 or a view with a non-finite entry or a norm >= 2^50 gets NaN bounds, every
// comparison fails and the pair is undecided (then |terms| <= A N_a < 2^100).
constexpr float kPfDelta = 0x1p-19f;
constexpr float kPfInflate = 1.0f + 0x1p-18f;
constexpr float kPfEta = 0x1p-120f;
constexpr float kPfLimit = 0x1p50f;
constexpr float kPfTiny = 0x1p-60f;

__device__ __forceinline__ float pf_nan() { return __int_as_float(0x7fffffff); }

// Upper bound of the Euclidean norm of (x, y, z[, w]).
__device__ __forceinline__ float bound_norm(float x, float y, float z, float w = 0.f)
{
  const float l1 = (fabsf(x) + fabsf(y) + fabsf(z) + fabsf(w)) * kPfInflate;
  if (l1 < kPfTiny) return l1 * kPfInflate;
  return sqrtf(fmaf(x, x, fmaf(y, y, fmaf(z, z, w * w)))) * kPfInflate;
}

struct PfObject {
  float4 c;    // box centre
  float rxyz;  // Rxyz (inflated)
  float rw;    // Rw (inflated)
  float da;    // delta * A (inflated), NaN when the bounds do not apply
};

__device__ __forceinline__ PfObject pf_object(const Obb& o)
{
  PfObject b;
  b.c = make_float4(fmaf(0.5f, o.ez.x, fmaf(0.5f, o.ey.x, fmaf(0.5f, o.ex.x, o.p.x))),
                    fmaf(0.5f, o.ez.y, fmaf(0.5f, o.ey.y, fmaf(0.5f, o.ex.y, o.p.y))),
                    fmaf(0.5f, o.ez.z, fmaf(0.5f, o.ey.z, fmaf(0.5f, o.ex.z, o.p.z))),
                    fmaf(0.5f, o.ez.w, fmaf(0.5f, o.ey.w, fmaf(0.5f, o.ex.w, o.p.w))));
  const float A = bound_norm(fabsf(o.p.x) + fabsf(o.ex.x) + fabsf(o.ey.x) + fabsf(o.ez.x),
                             fabsf(o.p.y) + fabsf(o.ex.y) + fabsf(o.ey.y) + fabsf(o.ez.y),
                             fabsf(o.p.z) + fabsf(o.ex.z) + fabsf(o.ey.z) + fabsf(o.ez.z),
                             fabsf(o.p.w) + fabsf(o.ex.w) + fabsf(o.ey.w) + fabsf(o.ez.w)) *
                  kPfInflate;
  b.rxyz = 0.5f * (bound_norm(o.ex.x, o.ex.y, o.ex.z) + bound_norm(o.ey.x, o.ey.y, o.ey.z) +
                   bound_norm(o.ez.x, o.ez.y, o.ez.z)) * kPfInflate;
  b.rw = 0.5f * (fabsf(o.ex.w) + fabsf(o.ey.w) + fabsf(o.ez.w)) * kPfInflate * kPfInflate;
  b.da = A < kPfLimit ? kPfDelta * A : pf_nan();
  return b;
}

// Per-view bounds: N[a] for the rounding margin, and per plane (lo x, hi x, lo y, hi y,
// lo z, hi z) the pair (n, m) of the extent term.  NaN when the view cannot be bounded.
struct PfView {
  float4 N;       // N_x, N_y, N_z, unused
  float4 nm[3];   // axis a: (n_lo, m_lo, n_hi, m_hi)
};

__device__ __forceinline__ PfView pf_view(const float* vp)
{
  PfView r;
  bool ok = true;
  float N[3];
  float nm[3][4];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float B[4], lo[4], hi[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float ca = vp[4 * i + a], cw = vp[4 * i + 3];
      ok &= isfinite(ca) && isfinite(cw);
      B[i] = fabsf(ca) + fabsf(cw);
      lo[i] = ca + cw;
      hi[i] = cw - ca;
    }
    N[a] = bound_norm(B[0], B[1], B[2], B[3]) * kPfInflate;
    nm[a][0] = bound_norm(lo[0], lo[1], lo[2]) * kPfInflate;
    nm[a][1] = fabsf(lo[3]) * kPfInflate * kPfInflate;
    nm[a][2] = bound_norm(hi[0], hi[1], hi[2]) * kPfInflate;
    nm[a][3] = fabsf(hi[3]) * kPfInflate * kPfInflate;
    ok &= N[a] < kPfLimit;
  }
  const float q = ok ? 0.f : pf_nan();  // NaN poisons every threshold of this view
  r.N = make_float4(N[0] + q, N[1] + q, N[2] + q, 0.f);
#pragma unroll
  for (int a = 0; a < 3; ++a)
    r.nm[a] = make_float4(nm[a][0] + q, nm[a][1] + q, nm[a][2] + q, nm[a][3] + q);
  return r;
}

enum : int { kPfInvisible = 0, kPfVisible = 1, kPfAmbiguous = 2 };

// View data read from shared memory once per (view, 4 objects).
struct PfViewRegs {
  float4 r0, r1, r2, r3;
  PfView b;
};

__device__ __forceinline__ PfViewRegs pf_load_view(const float* vp, const PfView& pv)
{
  PfViewRegs v;
  v.r0 = *reinterpret_cast<const float4*>(vp + 0);
  v.r1 = *reinterpret_cast<const float4*>(vp + 4);
  v.r2 = *reinterpret_cast<const float4*>(vp + 8);
  v.r3 = *reinterpret_cast<const float4*>(vp + 12);
  v.b = pv;
  return v;
}

__device__ __forceinline__ int pf_classify(const PfObject& b, const PfViewRegs& v)
{
  const float cx = fmaf(b.c.w, v.r3.x, fmaf(b.c.z, v.r2.x, fmaf(b.c.y, v.r1.x, b.c.x * v.r0.x)));
  const float cy = fmaf(b.c.w, v.r3.y, fmaf(b.c.z, v.r2.y, fmaf(b.c.y, v.r1.y, b.c.x * v.r0.y)));
  const float cz = fmaf(b.c.w, v.r3.z, fmaf(b.c.z, v.r2.z, fmaf(b.c.y, v.r1.z, b.c.x * v.r0.z)));
  const float cw = fmaf(b.c.w, v.r3.w, fmaf(b.c.z, v.r2.w, fmaf(b.c.y, v.r1.w, b.c.x * v.r0.w)));
  const float ex = fmaf(b.da, v.b.N.x, kPfEta), ey = fmaf(b.da, v.b.N.y, kPfEta),
              ez = fmaf(b.da, v.b.N.z, kPfEta);
  const float txl = fmaf(b.rxyz, v.b.nm[0].x, fmaf(b.rw, v.b.nm[0].y, ex));
  const float txh = fmaf(b.rxyz, v.b.nm[0].z, fmaf(b.rw, v.b.nm[0].w, ex));
  const float tyl = fmaf(b.rxyz, v.b.nm[1].x, fmaf(b.rw, v.b.nm[1].y, ey));
  const float tyh = fmaf(b.rxyz, v.b.nm[1].z, fmaf(b.rw, v.b.nm[1].w, ey));
  const float tzl = fmaf(b.rxyz, v.b.nm[2].x, fmaf(b.rw, v.b.nm[2].y, ez));
  const float tzh = fmaf(b.rxyz, v.b.nm[2].z, fmaf(b.rw, v.b.nm[2].w, ez));
  const float lox = cx + cw, hix = cw - cx;
  const float loy = cy + cw, hiy = cw - cy;
  const float loz = cz + cw, hiz = cw - cz;
  const bool out = (lox <= -txl) | ((hix <= -txh) & (lox > txl)) | (loy <= -tyl) |
                   ((hiy <= -tyh) & (loy > tyl)) | (loz <= -tzl) | ((hiz <= -tzh) & (loz > tzl));
  const bool in = (lox > txl) & (hix > txh) & (loy > tyl) & (hiy > tyh) & (loz > tzl) & (hiz > tzh);
  return out ? kPfInvisible : (in ? kPfVisible : kPfAmbiguous);
}

}  // namespace dpcull
