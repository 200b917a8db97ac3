// lu.cu -- shift-and-invert preconditioners: the dense (which_precon 2) and
// band (which_precon 3) LU factors of K + shift C + shift^2 M
// (user_module.f90:1383-1463 and :1520-1602), built and factored on the
// device, and their triangular solves (LU_solve :1703-1831, band_LU_solve
// :2181-2336).
//
// Both factorisations are the reference's: no pivoting, the unit lower
// factor below the diagonal, a zero pivot is an error.  The elimination and
// the solves are sequential in the pivot index, so each runs as ONE block of
// 1024 threads that walks the pivots with a barrier per step; the threads
// share the rows (and for the factorisation the columns) of each step.  The
// factor stays in HBM (band: n x (2 hb + 1), dense: n x n, column-major), the
// band rows a step touches stay in L1/L2.
#include <stdexcept>

#include "matrix.cuh"

namespace idrs {

namespace {

constexpr int kLUThreads = 1024;

template <class V> __device__ __forceinline__ bool is_zero(V v);
template <> __device__ __forceinline__ bool is_zero<double>(double v) { return v == 0.0; }
template <> __device__ __forceinline__ bool is_zero<c128>(c128 v) { return v.x == 0.0 && v.y == 0.0; }

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
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    for (int k = rp[i]; k < rp[i + 1]; ++k) {
      const long c = ci[k];
      const long idx = hb < 0 ? i + (long)n * c : i + (long)n * (c - i + hb);
      S[idx] = S[idx] + coef * entry<V>(val, vals, k);
    }
}

// the diagonal of S += d
template <class V>
__global__ void k_add_diag(int n, int hb, V d, V* S) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const long idx = hb < 0 ? i + (long)n * i : i + (long)n * hb;
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
// j in (k, k+hb].  *bad = 1-based index of a zero pivot.
template <class V>
__global__ void __launch_bounds__(kLUThreads) k_lu_factor(long n, int hb, bool band, V* S, int* bad) {
  auto at = [&](long i, long j) -> V& { return band ? S[i + n * (j - i + hb)] : S[i + n * j]; };
  __shared__ int zero;
  if (threadIdx.x == 0) zero = 0;
  __syncthreads();
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
      if (!is_zero(l)) l = l / p;
    }
    __syncthreads();
    const long rows = last - k, cols = last - k;
    for (long q = threadIdx.x; q < rows * cols; q += blockDim.x) {
      const long i = k + 1 + q / cols, j = k + 1 + q % cols;
      const V l = at(i, k);
      if (!is_zero(l)) at(i, j) = at(i, j) - l * at(k, j);
    }
    __syncthreads();
  }
  (void)zero;
}

// x = U^-1 L^-1 b (unit lower L), column-oriented like the reference
template <class V, class T>
__global__ void __launch_bounds__(kLUThreads) k_lu_solve(long n, int hb, bool band, const V* __restrict__ S,
                                                         const T* b, T* x, const int* __restrict__ skip) {
  if (skip && *(volatile const int*)skip) return;
  auto at = [&](long i, long j) -> V { return band ? S[i + n * (j - i + hb)] : S[i + n * j]; };
  if (x != b)
    for (long i = threadIdx.x; i < n; i += blockDim.x) x[i] = b[i];
  __syncthreads();
  for (long k = 0; k < n; ++k) {
    const T xp = x[k];
    const long up = k + hb < n - 1 ? k + hb : n - 1;
    for (long i = k + 1 + threadIdx.x; i <= up; i += blockDim.x) x[i] = x[i] - xp * narrow<T>(widen(at(i, k)));
    __syncthreads();
  }
  for (long k = n - 1; k >= 0; --k) {
    __shared__ T xk;
    if (threadIdx.x == 0) {
      xk = x[k] / narrow<T>(widen(at(k, k)));
      x[k] = xk;
    }
    __syncthreads();
    const T xp = xk;
    const long low = k - hb > 0 ? k - hb : 0;
    for (long i = k - 1 - threadIdx.x; i >= low; i -= blockDim.x) x[i] = x[i] - xp * narrow<T>(widen(at(i, k)));
    __syncthreads();
  }
}

template <class V>
void build_typed(const UserMatrix& K, const UserMatrix* M, const UserMatrix* C, bool has_shift,
                 c128 shift, bool dense, int hb, UserMatrix& P) {
  const int n = K.nrows;
  const long w = dense ? n : 2L * hb + 1;
  const long cnt = (long)n * w;
  const int hbs = dense ? -1 : hb;
  V* S = nullptr;
  IDRS_CUDA(cudaMalloc((void**)&S, sizeof(V) * std::max<long>(cnt, 1)));
  IDRS_CUDA(cudaMemset(S, 0, sizeof(V) * std::max<long>(cnt, 1)));
  auto scatter = [&](const UserMatrix& X, V* dst, V coef) {
    k_scatter<V><<<stream_grid(n), kThreads>>>(n, X.row_ptr, X.col_ind, X.val, X.vals, coef, hbs, dst);
    IDRS_LAUNCH_CHECK();
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
  IDRS_CUDA(cudaMalloc((void**)&bad, sizeof(int)));
  IDRS_CUDA(cudaMemset(bad, 0, sizeof(int)));
  k_lu_factor<V><<<1, kLUThreads>>>(n, dense ? n : hb, !dense, S, bad);
  IDRS_LAUNCH_CHECK();
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
    if (X && X->format != FMT_CRS && X->format != FMT_COO)
      throw std::runtime_error("shift-and-invert: K, M and C must be CRS or COO");
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
  const int hb = dense ? (int)n : P.half_band;
  const void* S = dense ? P.mat : P.band;
  if (P.vals == 2) {
    if constexpr (traits<T>::is_cplx)
      k_lu_solve<c128, T><<<1, kLUThreads, 0, st>>>(n, hb, !dense, (const c128*)S, b, x, skip);
    else
      throw std::runtime_error("shift-and-invert: complex factor in a real problem");
  } else {
    k_lu_solve<double, T><<<1, kLUThreads, 0, st>>>(n, hb, !dense, (const double*)S, b, x, skip);
  }
  IDRS_LAUNCH_CHECK();
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
