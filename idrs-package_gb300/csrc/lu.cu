// lu.cu -- shift-and-invert preconditioners: the dense (which_precon 2) and
// band (which_precon 3) LU factors of K + shift C + shift^2 M
// (user_module.f90:1383-1463 and :1520-1602), built and factored on the
// device, and their triangular solves (LU_solve :1703-1831, band_LU_solve
// :2181-2336).
//
// Both factorisations are the reference's: no pivoting, the unit lower
// factor below the diagonal, a zero pivot is an error.  The elimination is
// sequential in the pivot index and runs as ONE block of 1024 threads that
// walks the pivots with a barrier per step.
//
// Band factor layout (n_pad = n rounded up to 32 columns, all zero-padded):
//   L part  [0, n_pad hb)          L(k+d, k)          at (d-1) + hb k
//   W part  [n_pad hb, 2 n_pad hb) W(k-d, k)          at n_pad hb + (d-1) + hb k
//   D part  [2 n_pad hb, +n_pad)   1 / U(k,k)         at 2 n_pad hb + k
// for d = 1..hb.  During the elimination the W part holds U itself and the D
// part the diagonal; k_band_finish then stores W(i,k) = U(i,k) / U(k,k) and
// 1 / U(k,k).  Every column a solve step reads is contiguous, and the
// backward substitution becomes a unit upper solve plus one diagonal scaling,
// so each step has a single FP64 FMA on its critical path (GB300 issues one
// FP64 warp instruction per 64 cycles on an SM sub-partition; the latency is
// the same).  The dense factor stays column-major n x n with U in place.
//
// The band solve (k_band_trsv) is one CTA: TMA bulk copies stage 32-column
// chunks of the factor in shared memory (double buffered, mbarrier
// completion), the solution window of hb + 2 chunk rows lives in shared
// memory as separate real / imaginary planes, and for complex vectors the
// real and imaginary halves of each row update run on different warps (two
// FMAs each instead of four).
#include <atomic>
#include <mutex>
#include <stdexcept>

#include "matrix.cuh"
#include "tma.cuh"

namespace idrs {

namespace {

constexpr int kLUThreads = 1024;
constexpr size_t kTrsvSmemBudget = 200 * 1024;

__host__ __device__ inline long pad32(long n) { return (n + 31) / 32 * 32; }

// The factorisation and the dense solve spell out every multiply-subtract
// as FMAs and every complex division as Smith's algorithm with FMAs, in one
// fixed order.  The oracle restates exactly these operations, so both give
// the same factor bit for bit: without pivoting the elimination's growth
// (about 1.8e4 on a uniform random 120 x 120 matrix) turns the difference
// between one rounding (FMA) and two (product, then difference) into
// relative differences of 5e-9 in the solution.
// a - l b, l the factor's entry (the band solve's band_upd forms the same
// FMAs in the same order)
__device__ __forceinline__ double lu_msub(double a, double l, double b) { return fma(-l, b, a); }
__device__ __forceinline__ c128 lu_msub(c128 a, c128 l, c128 b) {
  return c128(fma(l.y, b.y, fma(-l.x, b.x, a.x)), fma(-l.y, b.x, fma(-l.x, b.y, a.y)));
}
__device__ __forceinline__ c128 lu_msub(c128 a, double l, c128 b) { return c128(fma(-l, b.x, a.x), fma(-l, b.y, a.y)); }
// a / b
__device__ __forceinline__ double lu_div(double a, double b) { return a / b; }
__device__ __forceinline__ c128 lu_div(c128 a, double b) { return c128(a.x / b, a.y / b); }
__device__ __forceinline__ c128 lu_div(c128 a, c128 b) {
  if (fabs(b.x) >= fabs(b.y)) {
    const double r = b.y / b.x, d = fma(b.y, r, b.x);
    return c128(fma(a.y, r, a.x) / d, fma(-a.x, r, a.y) / d);
  }
  const double r = b.x / b.y, d = fma(b.x, r, b.y);
  return c128(fma(a.x, r, a.y) / d, fma(a.y, r, -a.x) / d);
}

template <class V> __device__ __forceinline__ bool is_zero(V v);
// +0 or -0, tested on the bits (the same answer as v == 0.0): an FP64 compare
// would take a slot of GB300's FP64 pipe beside every multiply-subtract
template <> __device__ __forceinline__ bool is_zero<double>(double v) {
  return ((unsigned long long)__double_as_longlong(v) << 1) == 0ull;
}
template <> __device__ __forceinline__ bool is_zero<c128>(c128 v) {
  return (((unsigned long long)__double_as_longlong(v.x) | (unsigned long long)__double_as_longlong(v.y)) << 1) ==
         0ull;
}

// index of entry (i, j), |i - j| <= hb, in the band factor layout above
__host__ __device__ __forceinline__ long band_idx(long n_pad, int hb, long i, long j) {
  if (i == j) return 2 * n_pad * hb + i;
  if (i > j) return (i - j - 1) + (long)hb * j;
  return n_pad * hb + (j - i - 1) + (long)hb * j;
}

// value k of a CRS/COO user matrix as V
template <class V>
__device__ __forceinline__ V entry(const void* val, int vals, long k) {
  if (vals == 2) return narrow<V>(((const c128*)val)[k]);
  if (vals == 1) return narrow<V>(c128(((const double*)val)[k], 0.0));
  return narrow<V>(c128(1.0, 0.0));
}

// S += coef * X in dense (hb < 0) or band (hb >= 0) storage, one thread per
// row of X (rows are disjoint, so no atomics).  CRS/COO (row-sorted) only.
template <class V>
__global__ void k_scatter(int n, const int* __restrict__ rp, const int* __restrict__ ci,
                          const void* __restrict__ val, int vals, V coef, int hb, V* S) {
  const long n_pad = pad32(n);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    for (int k = rp[i]; k < rp[i + 1]; ++k) {
      const long c = ci[k];
      const long idx = hb < 0 ? i + (long)n * c : band_idx(n_pad, hb, i, c);
      S[idx] = S[idx] + coef * entry<V>(val, vals, k);
    }
}

// the diagonal of S += d
template <class V>
__global__ void k_add_diag(int n, int hb, V d, V* S) {
  const long n_pad = pad32(n);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const long idx = hb < 0 ? i + (long)n * i : band_idx(n_pad, hb, i, i);
    S[idx] = S[idx] + d;
  }
}

// S = S + a * X (+ b * Y) elementwise
template <class V>
__global__ void k_axpby(long cnt, V* S, const V* X, V a, const V* Y, V b) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * (long)blockDim.x) {
    V s = S[i] + a * X[i];
    if (Y) s = s + b * Y[i];
    S[i] = s;
  }
}

// In-place LU without pivoting.  Dense: hb = n.  For pivot k the rows
// i in (k, min(k+hb, n-1)] get l = S(i,k)/S(k,k) (rows with S(i,k) = 0 are
// skipped, as in the reference), then S(i, j) -= l S(k, j) for the columns
// j in (k, k+hb].  *bad = 1-based index of a zero pivot.  Consecutive
// threads take consecutive rows of one column (contiguous in both layouts).
template <class V>
__global__ void __launch_bounds__(kLUThreads) k_lu_factor(long n, int hb, bool band, V* S, int* bad) {
  const long n_pad = pad32(n);
  auto at = [&](long i, long j) -> V& { return band ? S[band_idx(n_pad, hb, i, j)] : S[i + n * j]; };
  const long last_k = band ? n - 1 : n;  // the band form never tests the last pivot
  for (long k = 0; k < last_k; ++k) {
    const V p = at(k, k);
    if (is_zero(p)) {
      if (threadIdx.x == 0) *bad = (int)(k + 1);
      return;
    }
    const long last = k + hb < n - 1 ? k + hb : n - 1;
    for (long i = k + 1 + threadIdx.x; i <= last; i += blockDim.x) {
      V& l = at(i, k);
      if (!is_zero(l)) l = lu_div(l, p);
    }
    __syncthreads();
    const long rows = last - k, cols = last - k;
    for (long q = threadIdx.x; q < rows * cols; q += blockDim.x) {
      const long i = k + 1 + q % rows, j = k + 1 + q / rows;
      const V l = at(i, k);
      if (!is_zero(l)) at(i, j) = lu_msub(at(i, j), l, at(k, j));
    }
    __syncthreads();
  }
}

// LU on all SMs for large matrices (dense n >= kLUBlockedMin, band hb >=
// kLUBlk as well): blocks of kLUBlk pivots, every entry given the same
// operations in the same order as in k_lu_factor, so the factor is the same
// bit for bit.  Pivot k updates the entries (i, j) with k < i, j <= min(k +
// hb, n - 1) (hb = n dense).  For the block of pivots k0 .. k0+nb-1: (1) the
// panel -- the block's columns below their pivots -- one thread per row, after
// each CTA has factored the block's diagonal part; (2) the block row -- the block's rows right of the panel -- by
// forward substitution in pivot order, one thread per column; (3) the
// trailing entries, up to nb multiply-subtracts each in pivot order, in 16 x
// 16 tiles of all SMs.  Every kernel returns at once after a zero pivot.
constexpr int kLUBlk = 16;
constexpr long kLUBlockedMin = 256;

// The panel on as many CTAs as its rows need (kLUPanelRows rows each).  Every
// CTA factors the block's nb x nb diagonal part in shared memory (the steps of
// k_lu_factor) and each thread owns one row below the block: pivot q needs
// only row q of the diagonal part, final after step q - 1, so the rows take
// pivot q while the diagonal part divides its column q (GB300's FP64 pipe is
// slow enough that the two chains would otherwise add up).  Once the pivot
// rows are final the rows are independent, and every entry gets the same
// operations in the same order as in k_lu_factor.  The diagonal part is
// written back by the CTA that read it last (ctl[1] counts the CTAs that hold
// their copy; ctl[0] is the zero-pivot flag), so no CTA reads a factored entry.
constexpr int kLUPanelRows = 64;

template <class V>
__global__ void __launch_bounds__(kLUPanelRows) k_lu_panel(long n, int hb, bool band, long k0, int nb, V* S,
                                                           int* ctl) {
  if (*(volatile int*)ctl) return;
  const long n_pad = pad32(n);
  auto at = [&](long i, long j) -> V& { return band ? S[band_idx(n_pad, hb, i, j)] : S[i + n * j]; };
  __shared__ V D[kLUBlk][kLUBlk + 1];  // D[r][c] = S(k0 + r, k0 + c), in the band (hb >= kLUBlk)
  __shared__ bool writer;
  for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) D[t % nb][t / nb] = at(k0 + t % nb, k0 + t / nb);
  // this thread's row (the grid covers every row a pivot of the block reaches)
  const long rend = (k0 + nb - 1 + hb < n - 1) ? k0 + nb - 1 + hb : n - 1;
  const long i = k0 + nb + blockIdx.x * (long)blockDim.x + threadIdx.x;
  const bool row = i <= rend;
  const V zero = narrow<V>(c128(0.0, 0.0));
  V c[kLUBlk];  // c[q] = S(i, k0 + q), zero where pivot k0 + q does not reach row i
#pragma unroll
  for (int q = 0; q < kLUBlk; ++q) c[q] = (row && q < nb && i - (k0 + q) <= hb) ? at(i, k0 + q) : zero;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    writer = atomicAdd(ctl + 1, 1) == (int)gridDim.x - 1;
    if (writer) {
      __threadfence();
      ctl[1] = 0;
    }
  }
#pragma unroll
  for (int q = 0; q < kLUBlk; ++q) {
    if (q >= nb) break;  // k0 + q < last_k: nb <= last_k - k0
    __syncthreads();
    const V p = D[q][q];
    if (is_zero(p)) {  // the same in every CTA; the factor is discarded
      if (blockIdx.x == 0 && threadIdx.x == 0) *ctl = (int)(k0 + q + 1);
      return;
    }
    if (row && i - (k0 + q) <= hb) {  // pivot k0 + q on this thread's row
      V l = c[q];
      if (!is_zero(l)) l = lu_div(l, p);
      c[q] = l;
      if (!is_zero(l)) {
#pragma unroll
        for (int j = q + 1; j < kLUBlk; ++j)
          if (j < nb) c[j] = lu_msub(c[j], l, D[q][j]);
      }
    }
    for (int r = q + 1 + threadIdx.x; r < nb; r += blockDim.x) {
      const V l = D[r][q];
      if (!is_zero(l)) D[r][q] = lu_div(l, p);
    }
    __syncthreads();
    const int m = nb - 1 - q;
    for (int t = threadIdx.x; t < m * m; t += blockDim.x) {
      const int r = q + 1 + t % m, j = q + 1 + t / m;
      const V l = D[r][q];
      if (!is_zero(l)) D[r][j] = lu_msub(D[r][j], l, D[q][j]);
    }
  }
  __syncthreads();
  if (writer)
    for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) at(k0 + t % nb, k0 + t / nb) = D[t % nb][t / nb];
  if (row) {
#pragma unroll
    for (int q = 0; q < kLUBlk; ++q)
      if (q < nb && i - (k0 + q) <= hb) at(i, k0 + q) = c[q];
  }
}

// block row: the block's strictly lower 16 x 16 part of L in shared memory,
// each thread's column of the block rows in registers (the loads of both are
// independent), then the forward substitution in pivot order
template <class V>
__global__ void __launch_bounds__(256) k_lu_blockrow(long n, int hb, bool band, long last_k, long k0, int nb, V* S,
                                                     const int* bad) {
  if (*(volatile const int*)bad) return;
  const long n_pad = pad32(n);
  auto at = [&](long i, long j) -> V& { return band ? S[band_idx(n_pad, hb, i, j)] : S[i + n * j]; };
  __shared__ V sL[kLUBlk][kLUBlk];  // sL[q][r] = l(k0+q, k0+r), r < q (0 where the pivot does not reach)
  const V zero = narrow<V>(c128(0.0, 0.0));
  for (int t = threadIdx.x; t < kLUBlk * kLUBlk; t += blockDim.x) {
    const int q = t / kLUBlk, r = t % kLUBlk;
    sL[q][r] = (r < q && q < nb && k0 + r < last_k && q - r <= hb) ? at(k0 + q, k0 + r) : zero;
  }
  __syncthreads();
  const long jend = (k0 + nb - 1 + hb < n - 1) ? k0 + nb - 1 + hb : n - 1;  // the last column any pivot reaches
  for (long j = k0 + nb + blockIdx.x * (long)blockDim.x + threadIdx.x; j <= jend; j += gridDim.x * (long)blockDim.x) {
    V c[kLUBlk];  // c[q] = S(k0+q, j), zero outside the band (never read there)
#pragma unroll
    for (int q = 0; q < kLUBlk; ++q) c[q] = (q < nb && j - (k0 + q) <= hb) ? at(k0 + q, j) : zero;
#pragma unroll
    for (int q = 1; q < kLUBlk; ++q) {
      if (q >= nb || j - (k0 + q) > hb) continue;  // outside the band: never updated
      V a = c[q];
#pragma unroll
      for (int r = 0; r < q; ++r) {
        if (j - (k0 + r) > hb) continue;  // pivot k0+r does not reach column j
        const V l = sL[q][r];
        if (!is_zero(l)) a = lu_msub(a, l, c[r]);
      }
      c[q] = a;
      at(k0 + q, j) = a;
    }
  }
}

template <class V>
__global__ void __launch_bounds__(256) k_lu_trail(long n, int hb, bool band, long last_k, long k0, int nb, V* S,
                                                  const int* bad) {
  if (*(volatile const int*)bad) return;
  __shared__ V sl[16][kLUBlk + 1];  // l(i, k0 + q) of the tile's rows (0 outside the band)
  __shared__ V su[kLUBlk][16 + 1];  // u(k0 + q, j) of the tile's columns (0 outside the band)
  const long n_pad = pad32(n);
  auto at = [&](long i, long j) -> V& { return band ? S[band_idx(n_pad, hb, i, j)] : S[i + n * j]; };
  const long base = k0 + nb;
  const long end = (k0 + nb - 1 + hb < n - 1) ? k0 + nb - 1 + hb : n - 1;  // rows / columns up to end
  const int tx = threadIdx.x, ty = threadIdx.y;
  const long i0 = base + blockIdx.x * 16L, j0 = base + blockIdx.y * 16L;
  const V zero = narrow<V>(c128(0.0, 0.0));
  if (ty < nb) {
    const long i = i0 + tx, k = k0 + ty;
    sl[tx][ty] = (i <= end && k < last_k && i - k <= hb) ? at(i, k) : zero;
  }
  if (tx < nb) {
    const long j = j0 + ty, k = k0 + tx;
    su[tx][ty] = (j <= end && k < last_k && j - k <= hb) ? at(k, j) : zero;
  }
  __syncthreads();
  const long i = i0 + tx, j = j0 + ty;
  if (i > end || j > end || (band && (i - j > hb || j - i > hb))) return;
  V a = at(i, j);
  for (int q = 0; q < nb; ++q) {
    const V l = sl[tx][q];
    if (!is_zero(l) && j - (k0 + q) <= hb) a = lu_msub(a, l, su[q][ty]);
  }
  at(i, j) = a;
}

// the dense trailing update in 64 x 64 tiles: each thread of 16 x 16 owns the
// entries (i0 + tx + 16a, j0 + ty + 16b), a, b < 4, so a pivot costs 8 shared
// loads for 16 multiply-subtracts (k_lu_trail: 2 per one); every entry gets
// k_lu_trail's operations in the same order
template <class V>
__global__ void __launch_bounds__(256) k_lu_trail_dense4(long n, long k0, int nb, V* S, const int* bad) {
  if (*(volatile const int*)bad) return;
  __shared__ V sl[kLUBlk][64 + 1];  // sl[q][r] = l(i0 + r, k0 + q)
  __shared__ V su[kLUBlk][64 + 1];  // su[q][c] = u(k0 + q, j0 + c)
  const long base = k0 + nb, end = n - 1;
  const int tx = threadIdx.x, ty = threadIdx.y, t = tx + 16 * ty;
  const long i0 = base + blockIdx.x * 64L, j0 = base + blockIdx.y * 64L;
  const V zero = narrow<V>(c128(0.0, 0.0));
  for (int e = t; e < kLUBlk * 64; e += 256) {
    const int r = e % 64, q = e / 64;  // column k0 + q of L, down the rows
    sl[q][r] = (q < nb && i0 + r <= end) ? S[(i0 + r) + n * (k0 + q)] : zero;
    const int qu = e % kLUBlk, c = e / kLUBlk;  // row k0 + qu of U, one column at a time
    su[qu][c] = (qu < nb && j0 + c <= end) ? S[(k0 + qu) + n * (j0 + c)] : zero;
  }
  __syncthreads();
  V acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const long i = i0 + tx + 16 * a, j = j0 + ty + 16 * b;
      acc[a][b] = (i <= end && j <= end) ? S[i + n * j] : zero;
    }
  for (int q = 0; q < nb; ++q) {
    V l[4], u[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) l[a] = sl[q][tx + 16 * a];
#pragma unroll
    for (int b = 0; b < 4; ++b) u[b] = su[q][ty + 16 * b];
#pragma unroll
    for (int a = 0; a < 4; ++a)
      if (!is_zero(l[a]))
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = lu_msub(acc[a][b], l[a], u[b]);
  }
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const long i = i0 + tx + 16 * a, j = j0 + ty + 16 * b;
      if (i <= end && j <= end) S[i + n * j] = acc[a][b];
    }
}

// W(i,k) = U(i,k) / U(k,k) and D(k) = 1 / U(k,k), one thread per column
template <class V>
__global__ void k_band_finish(long n, int hb, V* S) {
  const long n_pad = pad32(n);
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += gridDim.x * (long)blockDim.x) {
    V* d = S + band_idx(n_pad, hb, k, k);
    const V u = *d;
    V* w = S + n_pad * hb + (long)hb * k;
    for (int q = 0; q < hb && q < k; ++q) w[q] = w[q] / u;
    *d = narrow<V>(c128(1.0, 0.0)) / u;
  }
}

// x = U^-1 L^-1 b (unit lower L) for the DENSE factor, column-oriented like
// the reference (U on the diagonal, divisions as in LU_solve); T = V, or a
// complex vector with a real factor
template <class V, class T>
__global__ void __launch_bounds__(kLUThreads) k_lu_solve(long n, const V* __restrict__ S, const T* b, T* x,
                                                         const int* __restrict__ skip) {
  if (skip && *(volatile const int*)skip) return;
  auto at = [&](long i, long j) -> V { return S[i + n * j]; };
  if (x != b)
    for (long i = threadIdx.x; i < n; i += blockDim.x) x[i] = b[i];
  __syncthreads();
  for (long k = 0; k < n; ++k) {
    const T xp = x[k];
    for (long i = k + 1 + threadIdx.x; i < n; i += blockDim.x) x[i] = lu_msub(x[i], at(i, k), xp);
    __syncthreads();
  }
  for (long k = n - 1; k >= 0; --k) {
    __shared__ T xk;
    if (threadIdx.x == 0) {
      xk = lu_div(x[k], at(k, k));
      x[k] = xk;
    }
    __syncthreads();
    const T xp = xk;
    for (long i = k - 1 - threadIdx.x; i >= 0; i -= blockDim.x) x[i] = lu_msub(x[i], at(i, k), xp);
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// band solves
// ---------------------------------------------------------------------------
// y -= f p as FMAs on the real (part 0) or imaginary (part 1) plane; both
// band kernels use exactly these operations, so their results are identical
// (the operands are selected, not the results: one FMA chain per plane)
__device__ __forceinline__ double band_upd(int part, double f, double y, double pr, double pi) {
  return fma(-f, part ? pi : pr, y);
}
__device__ __forceinline__ double band_upd(int part, c128 f, double y, double pr, double pi) {
  const double a = part ? pi : pr, c = part ? pr : pi, g = part ? -f.y : f.y;
  return fma(g, c, fma(-f.x, a, y));
}
// (re, im) * d
__device__ __forceinline__ void band_scale(double& re, double& im, double d) { re *= d; im *= d; }
__device__ __forceinline__ void band_scale(double& re, double& im, c128 d) {
  const double r = re * d.x - im * d.y;
  im = re * d.y + im * d.x;
  re = r;
}
template <class T> __device__ __forceinline__ void split(T v, double& re, double& im) {
  const c128 w = c128(widen(v));
  re = w.x;
  im = w.y;
}
template <class T> __device__ __forceinline__ T join(double re, double im) {
  if constexpr (traits<T>::is_cplx) return T(re, im);
  else return T(re);
}

// Band solve x = D (W^-1 (L^-1 b)), one CTA of parts x rw threads (parts = 2
// for complex vectors, rw = hb rounded up to a warp).  Thread (part, r)
// updates row k+1+r (forward) or k-1-r (backward) of step k.  The 2 nc
// chunks of cc factor columns (forward L chunks 0..nc-1, then backward W
// chunks nc-1..0) stream through two shared buffers; chunk g uses buffer and
// mbarrier g & 1 with phase parity (g >> 1) & 1.  Rows enter the ws-slot
// window (slot = row & (ws-1), ws >= hb + 2 cc) a chunk ahead of their first
// update and leave it a chunk after they are final, written to x (forward: y;
// backward: D y).  A chunk whose copy has not landed after kTmaWaitCycles
// sets *fault and the solve returns NaN.
template <class V, class T>
__global__ void __launch_bounds__(kLUThreads) k_band_trsv(long n, int hb, int cc, int ws, const V* __restrict__ F,
                                                          const T* b, T* x, const int* __restrict__ skip,
                                                          int* fault) {
  if (skip && *(volatile const int*)skip) return;
  constexpr bool TC = traits<T>::is_cplx;
  extern __shared__ __align__(128) unsigned char sm[];
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sm);
  volatile int* sflag = reinterpret_cast<volatile int*>(sm + 16);
  const long chunk = (long)cc * hb;
  V* Fs = reinterpret_cast<V*>(sm + 32);
  double* yr = reinterpret_cast<double*>(sm + 32 + 2 * chunk * sizeof(V));
  double* yi = yr + ws;
  const long m = ws - 1;
  const int nt = blockDim.x, tid = threadIdx.x;
  const int rw = TC ? nt / 2 : nt;
  const int part = tid / rw, r = tid - part * rw;
  const long n_pad = pad32(n);
  const long nc = (n + cc - 1) / cc;
  const V* Wg = F + n_pad * hb;
  const V* dinv = F + 2 * n_pad * hb;
  const unsigned bytes = (unsigned)(chunk * sizeof(V));
  auto src = [&](long g) { return g < nc ? F + g * chunk : Wg + (2 * nc - 1 - g) * chunk; };
  if (tid == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    *sflag = 0;
    mbar_init_fence();
    mbar_expect_tx(&mbar[0], bytes);
    bulk_g2s(Fs, src(0), bytes, &mbar[0]);
  }
  __syncthreads();
  // thread 0: wait for chunk g, then start chunk g + 1 in the other buffer
  // (free: its last reader finished before the barrier that ended chunk g - 1)
  auto stage = [&](long g) {
    if (tid == 0) {
      if (!mbar_wait(&mbar[g & 1], (g >> 1) & 1)) {
        *sflag = 1;
      } else if (g + 1 < 2 * nc) {
        proxy_async_fence();
        mbar_expect_tx(&mbar[(g + 1) & 1], bytes);
        bulk_g2s(Fs + ((g + 1) & 1) * chunk, src(g + 1), bytes, &mbar[(g + 1) & 1]);
      }
    }
  };
  auto load = [&](const T* v, long i) {
    double re, im;
    split(v[i], re, im);
    yr[i & m] = re;
    if (TC) yi[i & m] = im;
  };
  long g = 0;
  // forward: y = L^-1 b
  long hi = 0, wr = 0;
  for (long c = 0; c < nc; ++c, ++g) {
    const long k0 = c * cc;
    stage(g);
    for (long i = wr + tid; i < k0; i += nt) x[i] = join<T>(yr[i & m], TC ? yi[i & m] : 0.0);
    wr = k0;
    const long nh = min(n, k0 + cc + hb);
    for (long i = hi + tid; i < nh; i += nt) load(b, i);
    hi = nh;
    __syncthreads();
    if (*sflag) break;
    if (tid) mbar_wait(&mbar[g & 1], (g >> 1) & 1);  // completed: acquires the chunk
    const V* Fc = Fs + (g & 1) * chunk;
    const long kend = min(k0 + cc, n - 1);
    V fn = r < hb ? Fc[r] : V(0.0);
    for (long k = k0; k < kend; ++k) {
      const V f = fn;
      if (r < hb && k + 1 < k0 + cc) fn = Fc[(k + 1 - k0) * hb + r];
      const long i = k + 1 + r;
      if (r < hb && i < n) {
        double* y = part ? yi : yr;
        y[i & m] = band_upd(part, f, y[i & m], yr[k & m], TC ? yi[k & m] : 0.0);
      }
      __syncthreads();
    }
  }
  if (!*sflag) {
    for (long i = wr + tid; i < n; i += nt) x[i] = join<T>(yr[i & m], TC ? yi[i & m] : 0.0);
    __syncthreads();
    // backward: x = D W^-1 y
    long lo = n, wl = n;
    for (long c = nc - 1; c >= 0; --c, ++g) {
      const long k0 = c * cc, top = min(n, k0 + cc) - 1;
      stage(g);
      for (long i = top + 1 + tid; i < wl; i += nt) {
        double re = yr[i & m], im = TC ? yi[i & m] : 0.0;
        band_scale(re, im, dinv[i]);
        x[i] = join<T>(re, im);
      }
      wl = top + 1;
      const long nl = max(0L, k0 - hb);
      for (long i = nl + tid; i < lo; i += nt) load(x, i);
      lo = nl;
      __syncthreads();
      if (*sflag) break;
      if (tid) mbar_wait(&mbar[g & 1], (g >> 1) & 1);
      const V* Fc = Fs + (g & 1) * chunk;
      const long kend = max(k0, 1L);
      V fn = r < hb ? Fc[(top - k0) * hb + r] : V(0.0);
      for (long k = top; k >= kend; --k) {
        const V f = fn;
        if (r < hb && k - 1 >= k0) fn = Fc[(k - 1 - k0) * hb + r];
        const long i = k - 1 - r;
        if (r < hb && i >= 0) {
          double* y = part ? yi : yr;
          y[i & m] = band_upd(part, f, y[i & m], yr[k & m], TC ? yi[k & m] : 0.0);
        }
        __syncthreads();
      }
    }
    if (!*sflag)
      for (long i = tid; i < wl; i += nt) {
        double re = yr[i & m], im = TC ? yi[i & m] : 0.0;
        band_scale(re, im, dinv[i]);
        x[i] = join<T>(re, im);
      }
  }
  if (*sflag) {
    // the lost copy may still land: wait once more (bounded), then report
    if (tid == 0) {
      mbar_wait(&mbar[g & 1], (g >> 1) & 1);
      *(volatile int*)fault = 1;
    }
    for (long i = tid; i < n; i += nt) x[i] = join<T>(nan(""), TC ? nan("") : 0.0);
  }
}

// The same solve for bands too wide to stage: the solution in HBM, every
// step's column read directly, the identical FMAs per element.
template <class V, class T>
__global__ void __launch_bounds__(kLUThreads) k_band_trsv_g(long n, int hb, const V* __restrict__ F, const T* b,
                                                            T* x, const int* __restrict__ skip) {
  if (skip && *(volatile const int*)skip) return;
  constexpr bool TC = traits<T>::is_cplx;
  const long n_pad = pad32(n);
  const V* Wg = F + n_pad * hb;
  const V* dinv = F + 2 * n_pad * hb;
  if (x != b)
    for (long i = threadIdx.x; i < n; i += blockDim.x) x[i] = b[i];
  __syncthreads();
  auto step = [&](long k, long i, const V f) {
    double pr, pi, yr, yi;
    split(x[k], pr, pi);
    split(x[i], yr, yi);
    yr = band_upd(0, f, yr, pr, pi);
    if (TC) yi = band_upd(1, f, yi, pr, pi);
    x[i] = join<T>(yr, yi);
  };
  for (long k = 0; k + 1 < n; ++k) {
    for (long r = threadIdx.x; r < hb && k + 1 + r < n; r += blockDim.x) step(k, k + 1 + r, F[(long)hb * k + r]);
    __syncthreads();
  }
  for (long k = n - 1; k >= 1; --k) {
    for (long r = threadIdx.x; r < hb && k - 1 - r >= 0; r += blockDim.x) step(k, k - 1 - r, Wg[(long)hb * k + r]);
    __syncthreads();
  }
  for (long i = threadIdx.x; i < n; i += blockDim.x) {
    double re, im;
    split(x[i], re, im);
    band_scale(re, im, dinv[i]);
    x[i] = join<T>(re, im);
  }
}

// x = D b (half band 0)
template <class V, class T>
__global__ void k_band_diag(long n, const V* __restrict__ dinv, const T* b, T* x, const int* __restrict__ skip) {
  if (skip && *(volatile const int*)skip) return;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (long)blockDim.x) {
    double re, im;
    split(b[i], re, im);
    band_scale(re, im, dinv[i]);
    x[i] = join<T>(re, im);
  }
}

struct TrsvShape {
  int threads = 0, cc = 0, ws = 0;
  size_t smem = 0;
};

// the staged kernel's launch shape, or threads = 0 when the band is too wide
template <class V, class T>
TrsvShape trsv_shape(int hb) {
  TrsvShape s;
  const int parts = traits<T>::is_cplx ? 2 : 1;
  const int rw = (hb + 31) / 32 * 32;
  if (hb <= 0 || rw * parts > kLUThreads) return s;
  for (int cc : {32, 16, 8}) {
    int ws = 1;
    while (ws < hb + 2 * cc + 1) ws *= 2;
    const size_t smem = 32 + 2 * (size_t)cc * hb * sizeof(V) + (size_t)parts * ws * sizeof(double);
    if (smem <= kTrsvSmemBudget) {
      s.threads = rw * parts;
      s.cc = cc;
      s.ws = ws;
      s.smem = smem;
      return s;
    }
  }
  return s;
}

template <class V, class T>
void band_solve(const UserMatrix& P, const T* b, T* x, const int* skip, cudaStream_t st) {
  const long n = P.nrows;
  const int hb = P.half_band;
  const V* F = (const V*)P.band;
  if (n == 0) return;
  if (hb == 0) {
    k_band_diag<V, T><<<stream_grid(n), kThreads, 0, st>>>(n, F, b, x, skip);
    IDRS_LAUNCH_CHECK();
    return;
  }
  const TrsvShape s = trsv_shape<V, T>(hb);
  if (s.threads) {
    // the attribute belongs to the current device: one bit per device
    static std::atomic<uint64_t> attr_set{0};
    int dev = 0;
    IDRS_CUDA(cudaGetDevice(&dev));
    const uint64_t bit = dev < 64 ? uint64_t(1) << dev : 0;
    if (!bit || !(attr_set.load() & bit)) {
      IDRS_CUDA(cudaFuncSetAttribute(k_band_trsv<V, T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kTrsvSmemBudget));
      attr_set.fetch_or(bit);
    }
    k_band_trsv<V, T><<<1, s.threads, s.smem, st>>>(n, hb, s.cc, s.ws, F, b, x, skip, device_fault_word());
  } else {
    k_band_trsv_g<V, T><<<1, kLUThreads, 0, st>>>(n, hb, F, b, x, skip);
  }
  IDRS_LAUNCH_CHECK();
}

// dst = X's first cnt values (a dense X, column-major like the dense factor)
template <class V>
__global__ void k_form_dense(long cnt, const void* __restrict__ src, int vals, V* dst) {
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < cnt; k += gridDim.x * (long)blockDim.x)
    dst[k] = entry<V>(src, vals, k);
}

// a CDS X (diagonal d of row i at band[i + n (d + hx)]) into the band factor
// layout, entries whose column lies outside the matrix left out
template <class V>
__global__ void k_form_cds(long n, long n_pad, int hx, int hb, const void* __restrict__ src, int vals, V* dst) {
  const long cnt = n * (2L * hx + 1);
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < cnt; t += gridDim.x * (long)blockDim.x) {
    const long i = t % n, j = i + (t / n - hx);
    if (j >= 0 && j < n) dst[band_idx(n_pad, hb, i, j)] = entry<V>(src, vals, t);
  }
}

// X's terms for the formats the scatter kernel does not read: a CDS matrix
// into the band factor, a dense matrix into the dense factor, written on the
// device into the ZEROED buffer dst (every caller adds its terms with
// coefficient one into a fresh buffer; hb >= X's half band).  Band entries
// whose column lies outside the matrix are left out (the elimination never
// reads them).  The reference has no band form of a dense matrix and no dense
// form of a CDS one (real_band / real_dense leave the result zero,
// user_module.f90:1163-1235, :1981-2066), so those combinations add nothing
// here either.
template <class V>
void device_form(const UserMatrix& X, V* dst, bool dense, int hb) {
  const long n = X.nrows;
  const int vals = X.vals == 2 ? 2 : 1;  // dense and CDS values are real or complex
  if (dense && X.format == FMT_DENSE) {
    const long cnt = n * std::min<long>(n, X.ncols);
    k_form_dense<V><<<stream_grid(cnt), kThreads>>>(cnt, X.mat, vals, dst);
    IDRS_LAUNCH_CHECK();
  } else if (!dense && X.format == FMT_CDS) {
    const int hx = X.half_band;
    k_form_cds<V><<<stream_grid(n * (2L * hx + 1)), kThreads>>>(n, pad32(n), hx, hb, X.band, vals, dst);
    IDRS_LAUNCH_CHECK();
  }
}

template <class V>
void build_typed(const UserMatrix& K, const UserMatrix* M, const UserMatrix* C, bool has_shift,
                 c128 shift, bool dense, int hb, UserMatrix& P) {
  const int n = K.nrows;
  const long cnt = dense ? (long)n * n : (2L * hb + 1) * pad32(n);
  const int hbs = dense ? -1 : hb;
  V* S = nullptr;
  IDRS_CUDA(cudaMalloc((void**)&S, sizeof(V) * std::max<long>(cnt, 1)));
  IDRS_CUDA(cudaMemset(S, 0, sizeof(V) * std::max<long>(cnt, 1)));
  auto scatter = [&](const UserMatrix& X, V* dst, V coef) {
    if (X.format == FMT_CRS || X.format == FMT_COO) {
      k_scatter<V><<<stream_grid(n), kThreads>>>(n, X.row_ptr, X.col_ind, X.val, X.vals, coef, hbs, dst);
      IDRS_LAUNCH_CHECK();
    } else {
      device_form<V>(X, dst, dense, hb);  // coef is one at every call
    }
  };
  const V one = narrow<V>(c128(1.0, 0.0));
  const V sh = narrow<V>(shift);
  scatter(K, S, one);
  if (has_shift) {
    // each matrix converted on its own, then combined like the reference
    V *Cd = nullptr, *Md = nullptr;
    if (C) {
      IDRS_CUDA(cudaMalloc((void**)&Cd, sizeof(V) * std::max<long>(cnt, 1)));
      IDRS_CUDA(cudaMemset(Cd, 0, sizeof(V) * std::max<long>(cnt, 1)));
      scatter(*C, Cd, one);
    }
    if (M) {
      IDRS_CUDA(cudaMalloc((void**)&Md, sizeof(V) * std::max<long>(cnt, 1)));
      IDRS_CUDA(cudaMemset(Md, 0, sizeof(V) * std::max<long>(cnt, 1)));
      scatter(*M, Md, one);
    }
    const V zero = narrow<V>(c128(0.0, 0.0));
    if (M && C) k_axpby<V><<<stream_grid(cnt), kThreads>>>(cnt, S, Cd, sh, Md, sh * sh);
    else if (C) k_axpby<V><<<stream_grid(cnt), kThreads>>>(cnt, S, Cd, sh, nullptr, zero);
    else if (M) k_axpby<V><<<stream_grid(cnt), kThreads>>>(cnt, S, Md, zero - sh, nullptr, zero);
    if (M || C) IDRS_LAUNCH_CHECK();
    if (C && !M) { k_add_diag<V><<<stream_grid(n), kThreads>>>(n, hbs, sh * sh, S); IDRS_LAUNCH_CHECK(); }
    if (!C && !M) { k_add_diag<V><<<stream_grid(n), kThreads>>>(n, hbs, zero - sh, S); IDRS_LAUNCH_CHECK(); }
    IDRS_CUDA(cudaDeviceSynchronize());
    if (Cd) cudaFree(Cd);
    if (Md) cudaFree(Md);
  }
  int* bad = nullptr;
  IDRS_CUDA(cudaMalloc((void**)&bad, 2 * sizeof(int)));  // the zero-pivot flag, the panel's CTA count
  IDRS_CUDA(cudaMemset(bad, 0, 2 * sizeof(int)));
  const int hbf = dense ? (int)n : hb;
  if (n >= kLUBlockedMin && (dense || hb >= kLUBlk)) {
    const long last_k = dense ? n : n - 1;  // the band form never tests the last pivot
    for (long k0 = 0; k0 < last_k; k0 += kLUBlk) {
      const int nb = (int)std::min<long>(kLUBlk, last_k - k0);
      {
        const long below = std::min<long>(k0 + nb - 1 + hbf, n - 1) - (k0 + nb) + 1;  // rows under the block
        const long g = std::max<long>(1, (below + kLUPanelRows - 1) / kLUPanelRows);
        k_lu_panel<V><<<(unsigned)g, kLUPanelRows>>>(n, hbf, !dense, k0, nb, S, bad);
      }
      const long end = std::min<long>(k0 + nb - 1 + hbf, n - 1);
      const long rest = end - (k0 + nb) + 1;
      if (rest > 0) {
        // one warp per CTA: each column is a chain of FP64 multiply-subtracts, so
        // the columns go to as many SMs as they fill
        k_lu_blockrow<V><<<(unsigned)((rest + 31) / 32), 32>>>(n, hbf, !dense, last_k, k0, nb, S, bad);
        IDRS_LAUNCH_CHECK();
        const long g4 = (rest + 63) / 64;
        if (dense && g4 * g4 >= 2L * num_sms()) {  // 64 x 64 tiles while they fill the SMs twice
          k_lu_trail_dense4<V><<<dim3((unsigned)g4, (unsigned)g4), dim3(16, 16)>>>(n, k0, nb, S, bad);
        } else {
          const dim3 g((unsigned)((rest + 15) / 16), (unsigned)((rest + 15) / 16));
          k_lu_trail<V><<<g, dim3(16, 16)>>>(n, hbf, !dense, last_k, k0, nb, S, bad);
        }
        IDRS_LAUNCH_CHECK();
      }
    }
  } else {
    k_lu_factor<V><<<1, kLUThreads>>>(n, hbf, !dense, S, bad);
    IDRS_LAUNCH_CHECK();
  }
  if (!dense) {
    k_band_finish<V><<<stream_grid(n), kThreads>>>(n, hb, S);
    IDRS_LAUNCH_CHECK();
  }
  int h = 0;
  IDRS_CUDA(cudaMemcpy(&h, bad, sizeof(int), cudaMemcpyDeviceToHost));
  cudaFree(bad);
  if (h) {
    cudaFree(S);
    throw std::runtime_error("Pivot equal to zero in LU decomposition");
  }
  if (dense) {
    P.format = FMT_DENSE;
    P.mat = S;
  } else {
    P.format = FMT_CDS;
    P.band = S;
    P.half_band = hb;
  }
}

int band_of(const UserMatrix& X) {
  if (X.format == FMT_DENSE) return X.ncols;
  if (X.format == FMT_CDS) return X.half_band;
  if (X.format != FMT_CRS && X.format != FMT_COO) return 0;
  std::vector<int> rp(X.nrows + 1), ci(std::max<long>(X.nnz, 1));
  IDRS_CUDA(cudaMemcpy(rp.data(), X.row_ptr, sizeof(int) * (X.nrows + 1), cudaMemcpyDeviceToHost));
  if (X.nnz) IDRS_CUDA(cudaMemcpy(ci.data(), X.col_ind, sizeof(int) * X.nnz, cudaMemcpyDeviceToHost));
  int hb = 0;
  for (int i = 0; i < X.nrows; ++i)
    for (int k = rp[i]; k < rp[i + 1]; ++k) hb = std::max(hb, std::abs(ci[k] - i));
  return hb;
}

}  // namespace

void lu_build(const UserMatrix& K, const UserMatrix* M, const UserMatrix* C, bool has_shift,
              c128 shift, int which, bool cplx, UserMatrix& P) {
  for (const UserMatrix* X : {&K, M, C})
    if (X && X->format != FMT_CRS && X->format != FMT_COO && X->format != FMT_CDS && X->format != FMT_DENSE)
      throw std::runtime_error("shift-and-invert: K, M and C must be CRS, COO, CDS or dense");
  const bool dense = which == 2;
  int hb = 0;
  if (!dense) {
    hb = band_of(K);
    if (has_shift && C) hb = std::max(hb, band_of(*C));
    if (has_shift && M) hb = std::max(hb, band_of(*M));
  }
  P.which_precon = which;
  P.vals = cplx ? 2 : 1;
  if (cplx) build_typed<c128>(K, M, C, has_shift, shift, dense, hb, P);
  else build_typed<double>(K, M, C, has_shift, shift, dense, hb, P);
}

template <class T>
void lu_solve(const UserMatrix& P, const T* b, T* x, const int* skip, cudaStream_t st) {
  const bool dense = P.format == FMT_DENSE;
  const long n = P.nrows;
  if (P.vals == 2 && !traits<T>::is_cplx) throw std::runtime_error("shift-and-invert: complex factor in a real problem");
  if (dense) {
    if (P.vals == 2) {
      if constexpr (traits<T>::is_cplx) k_lu_solve<c128, T><<<1, kLUThreads, 0, st>>>(n, (const c128*)P.mat, b, x, skip);
    } else {
      k_lu_solve<double, T><<<1, kLUThreads, 0, st>>>(n, (const double*)P.mat, b, x, skip);
    }
    IDRS_LAUNCH_CHECK();
    return;
  }
  if (P.vals == 2) {
    if constexpr (traits<T>::is_cplx) band_solve<c128, T>(P, b, x, skip, st);
  } else {
    band_solve<double, T>(P, b, x, skip, st);
  }
}

// One mapped, portable host word for the whole process (every device can
// write it; with unified addressing its device address is the host address).
static std::atomic<int*> g_fault_host{nullptr};
static std::once_flag g_fault_once;

int* device_fault_word() {
  std::call_once(g_fault_once, [] {
    int* h = nullptr;
    IDRS_CUDA(cudaHostAlloc((void**)&h, sizeof(int), cudaHostAllocMapped | cudaHostAllocPortable));
    *h = 0;
    g_fault_host.store(h);
  });
  int* h = g_fault_host.load();
  if (!h) throw std::runtime_error("mapped fault word unavailable");
  int* d = nullptr;
  IDRS_CUDA(cudaHostGetDevicePointer((void**)&d, h, 0));
  return d;
}

int take_device_fault() {
  int* h = g_fault_host.load();
  if (!h) return 0;
  return __atomic_exchange_n(h, 0, __ATOMIC_ACQ_REL);
}

namespace {
// y = y + a x
template <class T>
__global__ void k_si_axpy(long n, T a, const T* __restrict__ x, T* y) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (long)blockDim.x)
    y[i] = y[i] + a * x[i];
}
// w1 = v2 - s t2, w2 = -t2
template <class T>
__global__ void k_si_finish(long nn, T s, const T* __restrict__ v, const T* __restrict__ t2, T* w,
                            const int* __restrict__ skip) {
  if (skip && *(volatile const int*)skip) return;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < nn; i += gridDim.x * (long)blockDim.x) {
    const T t = t2[i];
    w[i] = v[nn + i] - s * t;
    w[nn + i] = T(0.0) - t;
  }
}
}  // namespace

template <class T>
void block_si_precon(const MatView& V, long nn, const T* v, T* w, const int* skip, cudaStream_t st) {
  T* a = (T*)V.si_tmp;
  T* b = a + nn;
  const T sh = narrow<T>(V.si_shift);
  spmv<T>(V.si_C->view64(), v + nn, a, T(1.0), T(1.0), v, skip, st);  // a = v1 + C v2
  if (V.si_M) {
    spmv<T>(V.si_M->view64(), v + nn, b, T(1.0), T(0.0), nullptr, skip, st);
    k_si_axpy<T><<<stream_grid(nn), kThreads, 0, st>>>(nn, sh, b, a);
  } else {
    k_si_axpy<T><<<stream_grid(nn), kThreads, 0, st>>>(nn, sh, v + nn, a);
  }
  IDRS_LAUNCH_CHECK();
  lu_solve<T>(*V.lu, a, b, skip, st);
  k_si_finish<T><<<stream_grid(nn), kThreads, 0, st>>>(nn, sh, v, b, w, skip);
  IDRS_LAUNCH_CHECK();
}

template void block_si_precon<double>(const MatView&, long, const double*, double*, const int*, cudaStream_t);
template void block_si_precon<c128>(const MatView&, long, const c128*, c128*, const int*, cudaStream_t);
template void lu_solve<double>(const UserMatrix&, const double*, double*, const int*, cudaStream_t);
template void lu_solve<c128>(const UserMatrix&, const c128*, c128*, const int*, cudaStream_t);

}  // namespace idrs
