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

}  // namespace dpcull
