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
__device__ __forceinline__ float4 st7_apply(const St7& c, float4 xm, float4 xc, float4 xp, float4 xs,
                                            float4 xn, float left, float right) {
  float4 r;
  r.x = st7_point(c, xc.x, left, xc.y, xs.x, xn.x, xm.x, xp.x);
  r.y = st7_point(c, xc.y, xc.x, xc.z, xs.y, xn.y, xm.y, xp.y);
  r.z = st7_point(c, xc.z, xc.y, xc.w, xs.z, xn.z, xm.z, xp.z);
  r.w = st7_point(c, xc.w, xc.z, right, xs.w, xn.w, xm.w, xp.w);
  return r;
}
__device__ __forceinline__ void axpy4(float4& r, float a, float4 x) {
  r.x = fmaf(a, x.x, r.x); r.y = fmaf(a, x.y, r.y); r.z = fmaf(a, x.z, r.z); r.w = fmaf(a, x.w, r.w);
}

constexpr int kF4Rows = 8;

__device__ __forceinline__ float4 ld4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }

}  // namespace idrs
