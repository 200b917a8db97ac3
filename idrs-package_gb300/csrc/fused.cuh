// fused.cuh -- the generic fused vector kernel and the ND-bucket dispatch.
//
// A Body describes one pass over the vectors: `prepare(sh)` loads the pass's
// scalar coefficients (written by an earlier tail) into shared memory, and
// `operator()(i, sh, acc)` updates element i and accumulates the pass's
// reductions.  The kernel then reduces over the grid and the last block runs
// the Tail.  Every pass returns at once when the solver has stopped.
#pragma once

#include <type_traits>

#include "common.cuh"

namespace idrs {

// ---------------------------------------------------------------------------
// packs: W consecutive elements of a vector moved as one access (one 16-byte
// load / store for four floats).  A Body that declares `kPack = true` writes
// its update once, as `template <int W, int ND, class A> run(i, sh, acc)` on
// pack index i (elements W i .. W i + W - 1), and says through `pack_ok()`
// whether its vectors allow W = 4 (16-byte aligned, column strides a
// multiple of four).  Every element gets the same operations as with W = 1;
// only the order of the reduction sums changes.
// ---------------------------------------------------------------------------
template <class T, int W>
struct Pk {
  T v[W];
};
template <int W, class T>
__device__ __forceinline__ Pk<T, W> pk_ld(const T* p, long i) {
  Pk<T, W> r;
  if constexpr (W == 4 && std::is_same<T, float>::value) {
    const float4 q = *reinterpret_cast<const float4*>(p + 4 * i);
    r.v[0] = q.x; r.v[1] = q.y; r.v[2] = q.z; r.v[3] = q.w;
  } else {
#pragma unroll
    for (int k = 0; k < W; ++k) r.v[k] = p[(long)W * i + k];
  }
  return r;
}
template <int W, class T>
__device__ __forceinline__ void pk_st(T* p, long i, const Pk<T, W>& r) {
  if constexpr (W == 4 && std::is_same<T, float>::value) {
    *reinterpret_cast<float4*>(p + 4 * i) = make_float4(r.v[0], r.v[1], r.v[2], r.v[3]);
  } else {
#pragma unroll
    for (int k = 0; k < W; ++k) p[(long)W * i + k] = r.v[k];
  }
}
// a - c b, a + c b, c b (c a scalar)
template <class T, int W>
__device__ __forceinline__ Pk<T, W> pk_msub(const Pk<T, W>& a, T c, const Pk<T, W>& b) {
  Pk<T, W> r;
#pragma unroll
  for (int k = 0; k < W; ++k) r.v[k] = a.v[k] - c * b.v[k];
  return r;
}
template <class T, int W>
__device__ __forceinline__ Pk<T, W> pk_madd(const Pk<T, W>& a, T c, const Pk<T, W>& b) {
  Pk<T, W> r;
#pragma unroll
  for (int k = 0; k < W; ++k) r.v[k] = a.v[k] + c * b.v[k];
  return r;
}
template <class T, int W>
__device__ __forceinline__ Pk<T, W> pk_scale(T c, const Pk<T, W>& b) {
  Pk<T, W> r;
#pragma unroll
  for (int k = 0; k < W; ++k) r.v[k] = c * b.v[k];
  return r;
}
// acc += conj(a_k) b_k, a_k b_k or |a_k|^2 for k = 0 .. W-1, in that order
template <class A, class T, int W>
__device__ __forceinline__ void pk_acc_dot(A& acc, const Pk<T, W>& a, const Pk<T, W>& b) {
#pragma unroll
  for (int k = 0; k < W; ++k) acc_add(acc, conj_(a.v[k]) * b.v[k]);
}
template <class A, class T, int W>
__device__ __forceinline__ void pk_acc_mul(A& acc, const Pk<T, W>& a, const Pk<T, W>& b) {
#pragma unroll
  for (int k = 0; k < W; ++k) acc_add(acc, a.v[k] * b.v[k]);
}
template <class A, class T, int W>
__device__ __forceinline__ void pk_acc_abs2(A& acc, const Pk<T, W>& a) {
#pragma unroll
  for (int k = 0; k < W; ++k) acc_add(acc, abs2_(a.v[k]));
}
inline bool aligned_f4(const void* p) { return ((uintptr_t)p & 15u) == 0; }

template <class B, class = void>
struct has_pack : std::false_type {};
template <class B>
struct has_pack<B, std::void_t<decltype(B::kPack)>> : std::bool_constant<B::kPack> {};

template <int ND, class T, class Body, class Tail, int W = 1>
__global__ void __launch_bounds__(kThreads) k_fused(long n, Body body, Tail tail, RedBuf rb,
                                                    const int* __restrict__ skip) {
  pdl_wait();
  pdl_trigger();
  if (skip && *(volatile const int*)skip) return;
  using A = typename acc_of<T>::type;
  __shared__ typename Body::Shared sh;
  body.prepare(sh);
  __syncthreads();
  A acc[ND > 0 ? ND : 1];
#pragma unroll
  for (int d = 0; d < (ND > 0 ? ND : 1); ++d) acc_zero(acc[d]);
  const long stride = (long)gridDim.x * blockDim.x;
  const long t0 = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if constexpr (W > 1) {
    const long np = n / W;
    for (long i = t0; i < np; i += stride) body.template run<W>(i, sh, acc);
    for (long e = np * W + t0; e < n; e += stride) body.template run<1>(e, sh, acc);
  } else if constexpr (has_pack<Body>::value) {
    for (long i = t0; i < n; i += stride) body.template run<1>(i, sh, acc);
  } else {
    for (long i = t0; i < n; i += stride) body(i, sh, acc);
  }
  if constexpr (ND > 0) grid_reduce_tail<ND>(acc, rb, tail);
}

// Launch with a compile-time reduction count ND (0: no reduction, no tail).
// Reductions launch as many blocks as fit on the SMs at once (found once per
// kernel from its register and shared-memory use), up to the partial slots.
template <int ND, class T, class Body, class Tail, int W = 1>
inline int resident_blocks() {
  static const int per_sm = [] {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_fused<ND, T, Body, Tail, W>, kThreads, 0) !=
        cudaSuccess)
      b = 0;
    return b > 0 ? b : 4;
  }();
  return per_sm;
}

// fp32 bodies with packs run four elements per thread and access when their
// vectors allow it
template <int ND, class T, class Body, class Tail>
inline void launch_fused(long n, const Body& body, const Tail& tail, RedBuf rb, const int* skip,
                         cudaStream_t st) {
  if constexpr (has_pack<Body>::value && std::is_same<T, float>::value) {
    if (body.pack_ok()) {
      const long np = (n + 3) / 4;
      int grid = (ND > 0) ? red_grid(np, resident_blocks<ND, T, Body, Tail, 4>()) : stream_grid(np);
      launch_pdl(k_fused<ND, T, Body, Tail, 4>, dim3(grid), dim3(kThreads), 0, st, n, body, tail, rb, skip);
      IDRS_LAUNCH_CHECK();
      return;
    }
  }
  int grid = (ND > 0) ? red_grid(n, resident_blocks<ND, T, Body, Tail>()) : stream_grid(n);
  launch_pdl(k_fused<ND, T, Body, Tail>, dim3(grid), dim3(kThreads), 0, st, n, body, tail, rb, skip);
  IDRS_LAUNCH_CHECK();
}

// Launch with a runtime reduction count nd <= 24, rounded up to a bucket.
// Bodies must guard their accumulation with `d < nd`.
template <class T, class Body, class Tail>
inline void launch_fused_nd(int nd, long n, const Body& body, const Tail& tail, RedBuf rb,
                            const int* skip, cudaStream_t st) {
  if (nd <= 1) launch_fused<1, T>(n, body, tail, rb, skip, st);
  else if (nd <= 2) launch_fused<2, T>(n, body, tail, rb, skip, st);
  else if (nd <= 3) launch_fused<3, T>(n, body, tail, rb, skip, st);
  else if (nd <= 4) launch_fused<4, T>(n, body, tail, rb, skip, st);
  else if (nd <= 5) launch_fused<5, T>(n, body, tail, rb, skip, st);
  else if (nd <= 8) launch_fused<8, T>(n, body, tail, rb, skip, st);
  else if (nd <= 9) launch_fused<9, T>(n, body, tail, rb, skip, st);
  else if (nd <= 16) launch_fused<16, T>(n, body, tail, rb, skip, st);
  else if (nd <= 17) launch_fused<17, T>(n, body, tail, rb, skip, st);
  else launch_fused<24, T>(n, body, tail, rb, skip, st);
}

struct NoShared {};

}  // namespace idrs
