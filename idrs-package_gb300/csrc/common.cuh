// common.cuh -- scalar types, error handling, launch geometry and the grid
// reduction used by every fused kernel of the IDRS GB300 library.
//
// Design notes
// * Vectors live in HBM as plain arrays of T, T in {double, float,
//   cplx<double>, cplx<float>} (complex interleaved, layout-compatible with
//   Fortran complex and C99 _Complex).
// * Every reduction kernel writes one partial per block into a scratch array
//   and the last block to finish (atomic ticket) sums the partials in a fixed
//   order and runs a "tail" functor on one thread.  The tail carries the
//   solver's small s x s scalar work (triangular solves, Givens rotations,
//   convergence tests), so no scalar ever travels to the host inside an
//   iteration.  The fixed summation order makes results reproducible.
// * fp32 kernels accumulate dot products in fp32 with Neumaier compensation
//   (TwoSum); tails see the compensated sum promoted to double.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <string>
#include <stdexcept>
#include <type_traits>
#include <utility>

namespace idrs {

// ---------------------------------------------------------------------------
// complex numbers
// ---------------------------------------------------------------------------
template <class R>
struct alignas(2 * sizeof(R)) cplx {
  R x, y;
  __host__ __device__ constexpr cplx() : x(0), y(0) {}
  __host__ __device__ constexpr cplx(R re) : x(re), y(0) {}
  __host__ __device__ constexpr cplx(R re, R im) : x(re), y(im) {}
  template <class Q>
  __host__ __device__ explicit cplx(cplx<Q> o) : x(R(o.x)), y(R(o.y)) {}
};
template <class R> __host__ __device__ inline cplx<R> operator+(cplx<R> a, cplx<R> b) { return {a.x + b.x, a.y + b.y}; }
template <class R> __host__ __device__ inline cplx<R> operator-(cplx<R> a, cplx<R> b) { return {a.x - b.x, a.y - b.y}; }
template <class R> __host__ __device__ inline cplx<R> operator-(cplx<R> a) { return {-a.x, -a.y}; }
template <class R> __host__ __device__ inline cplx<R> operator*(cplx<R> a, cplx<R> b) {
  return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <class R> __host__ __device__ inline cplx<R> operator*(R a, cplx<R> b) { return {a * b.x, a * b.y}; }
template <class R> __host__ __device__ inline cplx<R> operator*(cplx<R> a, R b) { return {a.x * b, a.y * b}; }
template <class R> __host__ __device__ inline cplx<R> operator/(cplx<R> a, R b) { return {a.x / b, a.y / b}; }
// Smith's algorithm for complex division.
template <class R> __host__ __device__ inline cplx<R> operator/(cplx<R> a, cplx<R> b) {
  if (fabs(b.x) >= fabs(b.y)) {
    R r = b.y / b.x, d = b.x + b.y * r;
    return {(a.x + a.y * r) / d, (a.y - a.x * r) / d};
  } else {
    R r = b.x / b.y, d = b.x * r + b.y;
    return {(a.x * r + a.y) / d, (a.y * r - a.x) / d};
  }
}
template <class R> __host__ __device__ inline bool operator==(cplx<R> a, cplx<R> b) { return a.x == b.x && a.y == b.y; }
template <class R> __host__ __device__ inline bool operator!=(cplx<R> a, cplx<R> b) { return !(a == b); }
template <class R> __host__ __device__ inline cplx<R>& operator+=(cplx<R>& a, cplx<R> b) { a = a + b; return a; }
template <class R> __host__ __device__ inline cplx<R>& operator-=(cplx<R>& a, cplx<R> b) { a = a - b; return a; }

template <class R> __host__ __device__ inline cplx<R> conj_(cplx<R> a) { return {a.x, -a.y}; }
__host__ __device__ inline double conj_(double a) { return a; }
__host__ __device__ inline float conj_(float a) { return a; }
template <class R> __host__ __device__ inline R abs_(cplx<R> a) { return hypot(a.x, a.y); }
__host__ __device__ inline double abs_(double a) { return fabs(a); }
__host__ __device__ inline float abs_(float a) { return fabsf(a); }
template <class R> __host__ __device__ inline R abs2_(cplx<R> a) { return a.x * a.x + a.y * a.y; }
__host__ __device__ inline double abs2_(double a) { return a * a; }
__host__ __device__ inline float abs2_(float a) { return a * a; }
template <class R> __host__ __device__ inline R real_(cplx<R> a) { return a.x; }
__host__ __device__ inline double real_(double a) { return a; }
__host__ __device__ inline float real_(float a) { return a; }
template <class R> __host__ __device__ inline R imag_(cplx<R> a) { return a.y; }
__host__ __device__ inline double imag_(double) { return 0.0; }
__host__ __device__ inline float imag_(float) { return 0.0f; }

using c64 = cplx<float>;
using c128 = cplx<double>;

// ---------------------------------------------------------------------------
// traits
// ---------------------------------------------------------------------------
template <class T> struct traits;
template <> struct traits<double> { using real = double; using wide = double; static constexpr bool is_cplx = false; };
template <> struct traits<float> { using real = float; using wide = double; static constexpr bool is_cplx = false; };
template <> struct traits<c128> { using real = double; using wide = c128; static constexpr bool is_cplx = true; };
template <> struct traits<c64> { using real = float; using wide = c128; static constexpr bool is_cplx = true; };

// Conversion of wide (double / c128) scalars to the vector type T.
template <class T> __host__ __device__ inline T narrow(double v) { return T(v); }
template <> __host__ __device__ inline c128 narrow<c128>(double v) { return c128(v, 0.0); }
template <> __host__ __device__ inline c64 narrow<c64>(double v) { return c64(float(v), 0.f); }
template <class T> __host__ __device__ inline T narrow(c128 v);
template <> __host__ __device__ inline c128 narrow<c128>(c128 v) { return v; }
template <> __host__ __device__ inline c64 narrow<c64>(c128 v) { return c64(float(v.x), float(v.y)); }
template <> __host__ __device__ inline double narrow<double>(c128 v) { return v.x; }
template <> __host__ __device__ inline float narrow<float>(c128 v) { return float(v.x); }
__host__ __device__ inline double widen(double v) { return v; }
__host__ __device__ inline double widen(float v) { return double(v); }
__host__ __device__ inline c128 widen(c128 v) { return v; }
__host__ __device__ inline c128 widen(c64 v) { return c128(double(v.x), double(v.y)); }

// ---------------------------------------------------------------------------
// accumulators: plain for fp64, Neumaier-compensated for fp32
// ---------------------------------------------------------------------------
struct kfloat {
  float s, c;
};
__device__ __forceinline__ void two_sum_add(float& s, float& c, float v) {
  float t = s + v;
  float bp = t - s;
  float err = (s - (t - bp)) + (v - bp);
  s = t;
  c += err;
}

// two compensated accumulators advanced together: every step of two_sum_add
// for both by one paired instruction (__fadd2_rn: each lane rounded as the
// scalar addition; x - y is x + (-y) exactly)
struct kfloat2 {
  float2 s, c;
};
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ void two_sum_add2(kfloat2& a, float2 v) {
  const float2 t = __fadd2_rn(a.s, v);
  const float2 bp = __fadd2_rn(t, neg2(a.s));
  const float2 err = __fadd2_rn(__fadd2_rn(a.s, neg2(__fadd2_rn(t, neg2(bp)))), __fadd2_rn(v, neg2(bp)));
  a.s = t;
  a.c = __fadd2_rn(a.c, err);
}

template <class T> struct acc_of;
template <> struct acc_of<double> { using type = double; };
template <> struct acc_of<c128> { using type = c128; };
template <> struct acc_of<float> { using type = kfloat; };
struct kc64 { kfloat re, im; };
template <> struct acc_of<c64> { using type = kc64; };

__device__ __forceinline__ void acc_zero(double& a) { a = 0.0; }
__device__ __forceinline__ void acc_zero(c128& a) { a = c128(0.0, 0.0); }
__device__ __forceinline__ void acc_zero(kfloat& a) { a.s = 0.f; a.c = 0.f; }
__device__ __forceinline__ void acc_zero(kc64& a) { acc_zero(a.re); acc_zero(a.im); }
__device__ __forceinline__ void acc_add(double& a, double v) { a += v; }
__device__ __forceinline__ void acc_add(c128& a, c128 v) { a = a + v; }
__device__ __forceinline__ void acc_add(kfloat& a, float v) { two_sum_add(a.s, a.c, v); }
__device__ __forceinline__ void acc_add(kc64& a, c64 v) { two_sum_add(a.re.s, a.re.c, v.x); two_sum_add(a.im.s, a.im.c, v.y); }
// real-valued contributions (norms) into complex accumulators
__device__ __forceinline__ void acc_add(c128& a, double v) { a.x += v; }
__device__ __forceinline__ void acc_add(kc64& a, float v) { two_sum_add(a.re.s, a.re.c, v); }
__device__ __forceinline__ void acc_merge(double& a, double b) { a += b; }
__device__ __forceinline__ void acc_merge(c128& a, c128 b) { a = a + b; }
__device__ __forceinline__ void acc_merge(kfloat& a, kfloat b) { two_sum_add(a.s, a.c, b.s); a.c += b.c; }
__device__ __forceinline__ void acc_merge(kc64& a, kc64 b) { acc_merge(a.re, b.re); acc_merge(a.im, b.im); }
__device__ __forceinline__ double acc_value(double a) { return a; }
__device__ __forceinline__ c128 acc_value(c128 a) { return a; }
__device__ __forceinline__ double acc_value(kfloat a) { return double(a.s) + double(a.c); }
__device__ __forceinline__ c128 acc_value(kc64 a) { return c128(acc_value(a.re), acc_value(a.im)); }
__device__ __forceinline__ double shfl_xor(double v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ __forceinline__ c128 shfl_xor(c128 v, int m) { return c128(shfl_xor(v.x, m), shfl_xor(v.y, m)); }
__device__ __forceinline__ kfloat shfl_xor(kfloat v, int m) {
  return kfloat{__shfl_xor_sync(0xffffffffu, v.s, m), __shfl_xor_sync(0xffffffffu, v.c, m)};
}
__device__ __forceinline__ kc64 shfl_xor(kc64 v, int m) { return kc64{shfl_xor(v.re, m), shfl_xor(v.im, m)}; }

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
void set_error(const std::string& msg);
const char* last_error();

struct cuda_error {
  cudaError_t code;
  std::string where;
};
#define IDRS_CUDA(call)                                                              \
  do {                                                                               \
    cudaError_t e__ = (call);                                                        \
    if (e__ != cudaSuccess) throw ::idrs::cuda_error{e__, std::string(#call) + " @ " \
                                                     __FILE__ ":" + std::to_string(__LINE__)}; \
  } while (0)
void count_launch();
void uncount_launches(long k);  // launches that were captured into a graph, not run
long launch_count();
#define IDRS_LAUNCH_CHECK()   \
  do {                        \
    ::idrs::count_launch();   \
    IDRS_CUDA(cudaPeekAtLastError()); \
  } while (0)

// ---------------------------------------------------------------------------
// Programmatic dependent launch.  The kernels of the solver passes and of the
// fp32 stencil chain start with pdl_wait() (griddepcontrol.wait: every
// earlier kernel of the stream has completed and its writes are visible),
// before they read anything, the skip flag included, and then pdl_trigger()
// (griddepcontrol.launch_dependents).  Launched by launch_pdl, such a kernel
// may be put on the SMs while the kernel before it drains its last blocks, so
// its launch and block start-up overlap that tail; without the attribute
// (IDRS_PDL=0, read once per process) both instructions are no-ops.  Only
// kernels that wait first may go through launch_pdl.  Launches into a stream
// capture go without the attribute: replayed graphs already start kernels
// back to back, and there the attribute measured slower (fp32 Chebyshev(8)
// product at 256^3: 0.2495 ms without, 0.2528 ms with it; launched directly
// 0.2587 ms without, 0.2521 ms with it).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
bool pdl_enabled();
template <class... KArgs, class... Args>
inline void launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                       Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) {
    cudaGetLastError();
    cs = cudaStreamCaptureStatusActive;
  }
  at[0].val.programmaticStreamSerializationAllowed = (pdl_enabled() && cs == cudaStreamCaptureStatusNone) ? 1 : 0;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  IDRS_CUDA(cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...));
}

// ---------------------------------------------------------------------------
// launch geometry: 152 SMs on GB300; grids are multiples of the SM count.
// ---------------------------------------------------------------------------
int num_sms();
constexpr int kThreads = 256;
constexpr int kMaxRedBlocks = 2048;  // partial slots per reduction value
constexpr int kMaxND = 24;           // maximum fused reductions in one kernel

inline int stream_grid(long n, int per_thread = 1) {
  long need = (n + (long)kThreads * per_thread - 1) / ((long)kThreads * per_thread);
  long cap = (long)num_sms() * 8;
  long g = need < cap ? need : cap;
  return g < 1 ? 1 : (int)g;
}
inline int red_grid(long n, int blocks_per_sm = 4) {
  long need = (n + kThreads - 1) / kThreads;
  long cap = (long)num_sms() * blocks_per_sm;
  long g = need < cap ? need : cap;
  if (g > kMaxRedBlocks) g = kMaxRedBlocks;
  return g < 1 ? 1 : (int)g;
}

// Scratch of the grid reductions: one ticket counter and kMaxRedBlocks x
// kMaxND partials of the widest accumulator type.
struct RedBuf {
  unsigned int* ticket;
  void* partials;
};

// ---------------------------------------------------------------------------
// block + grid reduction with a last-block tail
// ---------------------------------------------------------------------------
template <class A>
__device__ __forceinline__ void warp_reduce(A& a) {
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) acc_merge(a, shfl_xor(a, m));
}

__device__ __forceinline__ double load_cg(const double* p) { return __ldcg(p); }
__device__ __forceinline__ c128 load_cg(const c128* p) { return c128(__ldcg(&p->x), __ldcg(&p->y)); }
__device__ __forceinline__ kfloat load_cg(const kfloat* p) { return kfloat{__ldcg(&p->s), __ldcg(&p->c)}; }
__device__ __forceinline__ kc64 load_cg(const kc64* p) { return kc64{load_cg(&p->re), load_cg(&p->im)}; }

// Reduces ND accumulators over the grid; the last block to finish calls
// tail(vals) on thread 0 with the totals widened to double / c128.  Partials
// are combined in a fixed order, so the result does not depend on block
// scheduling.  Must be reached by every thread of every block.
// The same for blocks of any shape with kThreads threads: tid is the
// thread's linear index in its block, bid the block's linear index and
// nblocks the number of blocks (<= kMaxRedBlocks).
template <int ND, class A, class Tail>
__device__ __forceinline__ void grid_reduce_tail_at(A (&acc)[ND], RedBuf rb, const Tail& tail, int tid, int bid,
                                                    int nblocks) {
  using W = decltype(acc_value(acc[0]));
  __shared__ A sh[kThreads / 32][ND];
  __shared__ bool is_last;
  const int lane = tid & 31, wid = tid >> 5;
#pragma unroll
  for (int d = 0; d < ND; ++d) warp_reduce(acc[d]);
  if (lane == 0) {
#pragma unroll
    for (int d = 0; d < ND; ++d) sh[wid][d] = acc[d];
  }
  __syncthreads();
  A* part = reinterpret_cast<A*>(rb.partials);
  if (tid < ND) {
    A t = sh[0][tid];
    for (int w = 1; w < kThreads / 32; ++w) acc_merge(t, sh[w][tid]);
    part[(size_t)bid * ND + tid] = t;
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) {
    unsigned int prev = atomicAdd(rb.ticket, 1u);
    is_last = (prev == (unsigned)nblocks - 1);
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  A t[ND];
#pragma unroll
  for (int d = 0; d < ND; ++d) acc_zero(t[d]);
  for (int b = tid; b < nblocks; b += kThreads) {
#pragma unroll
    for (int d = 0; d < ND; ++d) acc_merge(t[d], load_cg(part + (size_t)b * ND + d));
  }
#pragma unroll
  for (int d = 0; d < ND; ++d) warp_reduce(t[d]);
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int d = 0; d < ND; ++d) sh[wid][d] = t[d];
  }
  __syncthreads();
  if (tid == 0) {
    W vals[ND];
#pragma unroll
    for (int d = 0; d < ND; ++d) {
      A u = sh[0][d];
      for (int w = 1; w < kThreads / 32; ++w) acc_merge(u, sh[w][d]);
      vals[d] = acc_value(u);
    }
    *rb.ticket = 0u;
    tail(vals);
  }
}

template <int ND, class A, class Tail>
__device__ __forceinline__ void grid_reduce_tail(A (&acc)[ND], RedBuf rb, const Tail& tail) {
  grid_reduce_tail_at<ND>(acc, rb, tail, (int)threadIdx.x, (int)blockIdx.x, (int)gridDim.x);
}

// Tail that does nothing (plain reductions whose result is not needed).
struct NoTail {
  template <class W> __device__ void operator()(const W*) const {}
};

}  // namespace idrs
