// fused.cuh -- the generic fused vector kernel and the ND-bucket dispatch.
//
// A Body describes one pass over the vectors: `prepare(sh)` loads the pass's
// scalar coefficients (written by an earlier tail) into shared memory, and
// `operator()(i, sh, acc)` updates element i and accumulates the pass's
// reductions.  The kernel then reduces over the grid and the last block runs
// the Tail.  Every pass returns at once when the solver has stopped.
#pragma once

#include "common.cuh"

namespace idrs {

template <int ND, class T, class Body, class Tail>
__global__ void __launch_bounds__(kThreads) k_fused(long n, Body body, Tail tail, RedBuf rb,
                                                    const int* __restrict__ skip) {
  if (skip && *(volatile const int*)skip) return;
  using A = typename acc_of<T>::type;
  __shared__ typename Body::Shared sh;
  body.prepare(sh);
  __syncthreads();
  A acc[ND > 0 ? ND : 1];
#pragma unroll
  for (int d = 0; d < (ND > 0 ? ND : 1); ++d) acc_zero(acc[d]);
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += stride) body(i, sh, acc);
  if constexpr (ND > 0) grid_reduce_tail<ND>(acc, rb, tail);
}

// Launch with a compile-time reduction count ND (0: no reduction, no tail).
// Reductions launch as many blocks as fit on the SMs at once (found once per
// kernel from its register and shared-memory use), up to the partial slots.
template <int ND, class T, class Body, class Tail>
inline int resident_blocks() {
  static const int per_sm = [] {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_fused<ND, T, Body, Tail>, kThreads, 0) != cudaSuccess)
      b = 0;
    return b > 0 ? b : 4;
  }();
  return per_sm;
}

template <int ND, class T, class Body, class Tail>
inline void launch_fused(long n, const Body& body, const Tail& tail, RedBuf rb, const int* skip,
                         cudaStream_t st) {
  int grid = (ND > 0) ? red_grid(n, resident_blocks<ND, T, Body, Tail>()) : stream_grid(n);
  k_fused<ND, T, Body, Tail><<<grid, kThreads, 0, st>>>(n, body, tail, rb, skip);
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
