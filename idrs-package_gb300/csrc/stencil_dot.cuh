// stencil_dot.cuh -- the last product of an fp32 polynomial chain on the
// matrix-free stencil, w = Ks y, with the projection P^T w of IDR(s)
// (idrs.inc:189-204, P_DOT of the new G column) accumulated in the same
// pass: w is written once and never read back for the s inner products.
// The partial sums (Neumaier-compensated fp32, as the fused vector passes)
// go through the grid reduction of common.cuh, whose last block runs the
// solver's tail.  Templated on that tail, so it lives in a header included
// by the solver translation units.
#pragma once

#include <cstdlib>

#include "fused.cuh"
#include "matrix.cuh"
#include "stencil.cuh"

namespace idrs {

// One thread owns four consecutive x-points of a row and marches in z like
// k_stencil7_f4 (same point arithmetic, so w is bitwise the same); acc_d +=
// PT_d . w over the thread's points for d < nd.  OM: the omega step's three
// inner products instead (idrs.inc:254-270, the separate pass BOmDots):
// acc_0 += w . r, acc_1 += w . w, acc_2 += r . r with r = PT's row 0 (ND 3,
// nd 1), so the new t = w is not read back for them.
template <int ND, class Tail, bool OM = false>
__global__ void __launch_bounds__(32 * kF4Rows) k_stencil7_f4_dot(int nx, int ny, int nz, int zc, St7 c,
                                                                  const float* __restrict__ x, float* __restrict__ y,
                                                                  const float* __restrict__ PT, long ld, int nd,
                                                                  RedBuf rb, Tail tail, const int* __restrict__ skip) {
  pdl_wait();
  pdl_trigger();
  if (skip && *(volatile const int*)skip) return;
  const int lane = threadIdx.x;
  const int i0 = (blockIdx.x * 32 + lane) * 4;
  const int j = blockIdx.y * kF4Rows + threadIdx.y;
  const int z0 = blockIdx.z * zc;
  const int z1 = min(nz, z0 + zc);
  const bool in = (i0 < nx) && (j < ny);
  const long plane = (long)nx * ny;
  long p = (long)j * nx + i0 + plane * z0;
  const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
  kfloat acc[ND];
#pragma unroll
  for (int d = 0; d < ND; ++d) acc_zero(acc[d]);
  kfloat2 a01 = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};  // accumulators 0 and 1 (OM, ND 2)
  float4 xm = (in && z0 > 0) ? ld4(x + p - plane) : zero;
  float4 xc = in ? ld4(x + p) : zero;
  float4 xp = (in && z0 + 1 < nz) ? ld4(x + p + plane) : zero;
  // plane z+2 of x and the shadow rows of plane z+1 are already in registers
  // when iteration z starts: the HBM streams are requested two iterations
  // ahead of their use (0.662 against 0.6635 s for the 256^3 mixed solve)
  float4 xq = (in && z0 + 2 < nz) ? ld4(x + p + 2 * plane) : zero;
  float4 qn[ND];
#pragma unroll
  for (int d = 0; d < ND; ++d) qn[d] = (in && d < nd) ? ld4(PT + d * ld + p) : zero;
  for (int z = z0; z < z1; ++z, p += plane) {
    const float4 xpp = xq;
    xq = (in && z + 3 < nz) ? ld4(x + p + 3 * plane) : zero;
    float4 q[ND];
#pragma unroll
    for (int d = 0; d < ND; ++d) {
      q[d] = qn[d];
      qn[d] = (in && d < nd && z + 1 < z1) ? ld4(PT + d * ld + p + plane) : zero;
    }
    const float4 xs = (in && j > 0) ? ld4(x + p - nx) : zero;
    const float4 xn = (in && j + 1 < ny) ? ld4(x + p + nx) : zero;
    float left = __shfl_up_sync(0xffffffffu, xc.w, 1);
    float right = __shfl_down_sync(0xffffffffu, xc.x, 1);
    if (lane == 0) left = (in && i0 > 0) ? __ldg(x + p - 1) : 0.f;
    if (lane == 31) right = (in && i0 + 4 < nx) ? __ldg(x + p + 4) : 0.f;
    if (in) {
      const float4 r = st7_apply(c, xm, xc, xp, xs, xn, left, right);
      *reinterpret_cast<float4*>(y + p) = r;
      // every product added to the compensated accumulator, as in the
      // separate pass (the projection's accuracy steers the fp32 IDR(s));
      // accumulators 0 and 1 advance together by paired instructions (the
      // rounded product, then TwoSum)
      if constexpr (OM) {
        two_sum_add2(a01, __fmul2_rn(make_float2(q[0].x, r.x), make_float2(r.x, r.x)));
        two_sum_add2(a01, __fmul2_rn(make_float2(q[0].y, r.y), make_float2(r.y, r.y)));
        two_sum_add2(a01, __fmul2_rn(make_float2(q[0].z, r.z), make_float2(r.z, r.z)));
        two_sum_add2(a01, __fmul2_rn(make_float2(q[0].w, r.w), make_float2(r.w, r.w)));
        acc_add(acc[2], q[0].x * q[0].x);
        acc_add(acc[2], q[0].y * q[0].y);
        acc_add(acc[2], q[0].z * q[0].z);
        acc_add(acc[2], q[0].w * q[0].w);
      } else if constexpr (ND == 2) {  // row 1 of q is zero when nd = 1; its sum is then unused
        two_sum_add2(a01, __fmul2_rn(make_float2(q[0].x, q[1].x), make_float2(r.x, r.x)));
        two_sum_add2(a01, __fmul2_rn(make_float2(q[0].y, q[1].y), make_float2(r.y, r.y)));
        two_sum_add2(a01, __fmul2_rn(make_float2(q[0].z, q[1].z), make_float2(r.z, r.z)));
        two_sum_add2(a01, __fmul2_rn(make_float2(q[0].w, q[1].w), make_float2(r.w, r.w)));
      } else {
#pragma unroll
        for (int d = 0; d < ND; ++d)
          if (d < nd) {
            acc_add(acc[d], q[d].x * r.x);
            acc_add(acc[d], q[d].y * r.y);
            acc_add(acc[d], q[d].z * r.z);
            acc_add(acc[d], q[d].w * r.w);
          }
      }
    }
    xm = xc;
    xc = xp;
    xp = xpp;
  }
  if constexpr (OM || ND == 2) {
    acc[0].s = a01.s.x;
    acc[0].c = a01.c.x;
    acc[1].s = a01.s.y;
    acc[1].c = a01.c.y;
  }
  const int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
  grid_reduce_tail_at<ND>(acc, rb, tail, lane + 32 * threadIdx.y, bid, gridDim.x * gridDim.y * gridDim.z);
}

// IDRS_FUSED_PDOT=0 in the environment keeps the projection a separate pass
// (read once per process; for comparisons)
inline bool fused_pdot_enabled() {
  static const bool on = [] {
    const char* e = getenv("IDRS_FUSED_PDOT");
    return !(e && e[0] == '0');
  }();
  return on;
}

// w = Ks p(Ks) v and the tail of P^T w in the last pass when the operator is
// the fp32 matrix-free stencil with its polynomial by the recurrence (or no
// polynomial), the vectors are 16-byte aligned and nd <= 8; false (nothing
// launched) otherwise.  OM: the omega step's w . r, w . w, r . r with r = PT
// (nd 1) instead.
template <class Tail, bool OM = false>
bool chain_with_pdot(Operator& A, const float* v, float* w, float* t1, float* t2, float* t3, float* t4,
                     const float* PT, long ld, int nd, RedBuf rb, Tail tail, const int* skip, cudaStream_t st) {
  if (nd < 1 || nd > 8 || (OM && nd != 1) || !fused_pdot_enabled()) return false;
  if (A.degree > 0 && !use_recurrence(A, 32)) return false;
  const MatView& M = A.view(32);
  if (M.format != FMT_STENCIL7 || M.nx % 4 != 0) return false;
  for (const void* q : {(const void*)v, (const void*)w, (const void*)t1, (const void*)t2, (const void*)t3,
                        (const void*)t4, (const void*)PT})
    if (q && !aligned_f4(q)) return false;
  if (ld % 4 != 0) return false;
  const int gx = (M.nx + 127) / 128, gy = (M.ny + kF4Rows - 1) / kF4Rows;
  const long xy = (long)gx * gy;
  if (xy > kMaxRedBlocks) return false;  // one partial slot per block
  const long target = (long)num_sms() * 8;
  int zc = (int)std::max(1L, std::min((long)M.nz, (M.nz * xy + target - 1) / target));
  if (zc < 4 && M.nz >= 4) zc = 4;
  while (xy * ((M.nz + zc - 1) / zc) > kMaxRedBlocks) ++zc;
  const float* y = A.degree > 0 ? op_chain_recur_head<float>(M, A.jac, A.degree, v, t1, t2, t3, t4, skip, st) : v;
  const St7 c{float(M.st[0]), float(M.st[1]), float(M.st[2]), float(M.st[3]), float(M.st[4]), float(M.st[5]),
              float(M.st[6])};
  dim3 blk(32, kF4Rows, 1), grid(gx, gy, (M.nz + zc - 1) / zc);
  auto kern = OM ? k_stencil7_f4_dot<3, Tail, true>
             : nd <= 2 ? k_stencil7_f4_dot<2, Tail> : nd <= 4 ? k_stencil7_f4_dot<4, Tail> : k_stencil7_f4_dot<8, Tail>;
  launch_pdl(kern, grid, blk, 0, st, M.nx, M.ny, M.nz, zc, c, y, w, PT, ld, nd, rb, tail, skip);
  IDRS_LAUNCH_CHECK();
  return true;
}

}  // namespace idrs
