// stencil.cuh -- the fp32 7-point stencil point arithmetic shared by every
// fp32 stencil kernel (matrix.cu and the fused last step of a polynomial
// chain, stencil_dot.cuh), so that all of them round identically.
#pragma once

#include <cuda_runtime.h>

namespace idrs {

// stencil coefficients (centre, x-1, x+1, y-1, y+1, z-1, z+1), the scale of
// the epilogue and the diagonal scaling folded in
struct St7 {
  float c0, cw, ce, cs, cn, cf, cb;
};
// one point: centre product, then the six neighbours fused in a fixed order
// (explicit FMAs, so every fp32 stencil kernel rounds identically whatever
// contraction the compiler would pick)
__device__ __forceinline__ float st7_point(const St7& c, float xc, float w, float e, float s, float n, float f,
                                           float b) {
  float r = c.c0 * xc;
  r = fmaf(c.cw, w, r);
  r = fmaf(c.ce, e, r);
  r = fmaf(c.cs, s, r);
  r = fmaf(c.cn, n, r);
  r = fmaf(c.cf, f, r);
  return fmaf(c.cb, b, r);
}
// Four consecutive points as two pairs, (x, y) and (z, w), each step of
// st7_point done for both points of a pair by one paired instruction
// (__fmul2_rn / __ffma2_rn: two fp32 lanes, each rounded exactly as fmulf /
// fmaf), so the results are bitwise those of st7_point and the FMA issue
// slots are halved.  The x-neighbour pairs (left, x), (y, z), (w, right)
// are shared by the west term of one pair and the east term of the other.
__device__ __forceinline__ float4 st7_apply(const St7& c, float4 xm, float4 xc, float4 xp, float4 xs,
                                            float4 xn, float left, float right) {
  const float2 c0 = make_float2(c.c0, c.c0), cw = make_float2(c.cw, c.cw), ce = make_float2(c.ce, c.ce);
  const float2 cs = make_float2(c.cs, c.cs), cn = make_float2(c.cn, c.cn);
  const float2 cf = make_float2(c.cf, c.cf), cb = make_float2(c.cb, c.cb);
  const float2 sh0 = make_float2(left, xc.x), sh1 = make_float2(xc.y, xc.z), sh2 = make_float2(xc.w, right);
  float2 p = __fmul2_rn(c0, make_float2(xc.x, xc.y));
  float2 q = __fmul2_rn(c0, make_float2(xc.z, xc.w));
  p = __ffma2_rn(cw, sh0, p);
  q = __ffma2_rn(cw, sh1, q);
  p = __ffma2_rn(ce, sh1, p);
  q = __ffma2_rn(ce, sh2, q);
  p = __ffma2_rn(cs, make_float2(xs.x, xs.y), p);
  q = __ffma2_rn(cs, make_float2(xs.z, xs.w), q);
  p = __ffma2_rn(cn, make_float2(xn.x, xn.y), p);
  q = __ffma2_rn(cn, make_float2(xn.z, xn.w), q);
  p = __ffma2_rn(cf, make_float2(xm.x, xm.y), p);
  q = __ffma2_rn(cf, make_float2(xm.z, xm.w), q);
  p = __ffma2_rn(cb, make_float2(xp.x, xp.y), p);
  q = __ffma2_rn(cb, make_float2(xp.z, xp.w), q);
  return make_float4(p.x, p.y, q.x, q.y);
}
__device__ __forceinline__ void axpy4(float4& r, float a, float4 x) {
  const float2 aa = make_float2(a, a);
  const float2 p = __ffma2_rn(aa, make_float2(x.x, x.y), make_float2(r.x, r.y));
  const float2 q = __ffma2_rn(aa, make_float2(x.z, x.w), make_float2(r.z, r.w));
  r = make_float4(p.x, p.y, q.x, q.y);
}

constexpr int kF4Rows = 8;

__device__ __forceinline__ float4 ld4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }

}  // namespace idrs
