// deflation.cu -- the deflation preconditioner of type(matrix)
// (matrix_module.f90:1284-1623): make_deflation, Pmul and add_deflation /
// ms_add_deflation, for the fp64 real and complex operators.
//
// Every projection is two fused passes: the k inner products V^H w in one
// reduction whose last block solves the k x k system on the device (Gaussian
// elimination with partial pivoting, the solver of the IDR(s) tails), and one
// element pass that subtracts the combination.  Nothing goes back to the host,
// so a deflated operator keeps the solvers' launch-ahead pipeline.
#include <stdexcept>

#include "idrs_gpu.cuh"

namespace idrs {

namespace {

constexpr int kDefMax = MAXS;  // deflation vectors (the device solver's size)

// acc_j = sum_i conj(V_j[i]) w[i], j < k   (dot_product(V(:,j), w))
template <class T>
struct BDefDots {
  const T* V; long n; const T* w; int k;
  using Shared = NoShared;
  __device__ void prepare(Shared&) const {}
  template <int ND, class A>
  __device__ void operator()(long i, Shared&, A (&acc)[ND]) const {
    const T wi = w[i];
#pragma unroll
    for (int d = 0; d < ND; ++d)
      if (d < k) acc_add(acc[d], conj_(V[d * n + i]) * wi);
  }
};

// coefficients t of the projection: t = s (solve = false, I - V V^H), or
// t = (E - sigma_s I)^-1 s
template <class W>
struct TDefSolve {
  const W* E; W* t; int k; bool solve; W sigma_s;
  __device__ void operator()(const W* s) const {
    if (!solve) {
      for (int j = 0; j < k; ++j) t[j] = s[j];
      return;
    }
    W H[MAXS * MAXS];
    for (int j = 0; j < k; ++j)
      for (int i = 0; i < k; ++i) H[i + MAXS * j] = E[i + MAXS * j] - (i == j ? sigma_s : W(0.0));
    solve_small<W>(k, H, s, t);
  }
};

// E(:, j) = V^H AV_j
template <class W>
struct TDefColumn {
  W* col; int k;
  __device__ void operator()(const W* s) const {
    for (int i = 0; i < k; ++i) col[i] = s[i];
  }
};

// out = fa * (w - sum_j W_j t_j) + fcv * fv
template <class T>
__global__ void __launch_bounds__(kThreads) k_defl_pmul(long n, const T* __restrict__ w, T* out,
                                                        const T* __restrict__ Wm, int k,
                                                        const T* __restrict__ t, T fa, T fcv,
                                                        const T* __restrict__ fv,
                                                        const int* __restrict__ skip) {
  if (skip && *(volatile const int*)skip) return;
  __shared__ T ts[kDefMax];
  if (threadIdx.x < k) ts[threadIdx.x] = t[threadIdx.x];
  __syncthreads();
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += stride) {
    T acc = T(0.0);
    for (int j = 0; j < k; ++j) acc = acc + Wm[j * n + i] * ts[j];
    T r = fa * (w[i] - acc);
    if (fv) r = r + fcv * fv[i];
    out[i] = r;
  }
}

// x = sum_j V_j t1_j + (y - sum_j V_j t2_j)
template <class T>
__global__ void __launch_bounds__(kThreads) k_defl_add(long n, const T* __restrict__ V, int k,
                                                       const T* __restrict__ t1,
                                                       const T* __restrict__ t2,
                                                       const T* __restrict__ y, T* x,
                                                       const int* __restrict__ skip) {
  if (skip && *(volatile const int*)skip) return;
  __shared__ T a[kDefMax], c[kDefMax];
  if (threadIdx.x < k) { a[threadIdx.x] = t1[threadIdx.x]; c[threadIdx.x] = t2[threadIdx.x]; }
  __syncthreads();
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += stride) {
    T x1 = T(0.0), v2 = T(0.0);
    for (int j = 0; j < k; ++j) x1 = x1 + V[j * n + i] * a[j];
    for (int j = 0; j < k; ++j) v2 = v2 + V[j * n + i] * c[j];
    x[i] = x1 + (y[i] - v2);
  }
}

template <class T>
void dots_then(const Deflation& D, const T* w, const TDefSolve<T>& tail, const int* skip,
               cudaStream_t st) {
  launch_fused_nd<T>(D.k, D.n, BDefDots<T>{(const T*)D.V, D.n, w, D.k}, tail, D.rb, skip, st);
}

template <class T>
void make_typed(Operator& A, Deflation& D, const T* V) {
  const long n = D.n;
  const int k = D.k;
  cudaStream_t st = D.st;
  IDRS_CUDA(cudaMemcpyAsync(D.V, V, sizeof(T) * n * k, cudaMemcpyDeviceToDevice, st));
  // AV_j = real_mv(A, V_j): the scaled system matrix without polynomial or projector
  MatView Ks = A.view(64);
  Ks.defl = nullptr;
  for (int j = 0; j < k; ++j)
    ks_mv<T>(Ks, (const T*)D.V + (size_t)n * j, (T*)D.AV + (size_t)n * j, T(1), T(0), nullptr, nullptr, st);
  IDRS_CUDA(cudaMemsetAsync(D.E, 0, sizeof(T) * MAXS * MAXS, st));
  for (int j = 0; j < k; ++j)
    launch_fused_nd<T>(k, n, BDefDots<T>{(const T*)D.V, n, (const T*)D.AV + (size_t)n * j, k},
                       TDefColumn<T>{(T*)D.E + (size_t)MAXS * j, k}, D.rb, nullptr, st);
}

}  // namespace

void deflation_free(Deflation* D) {
  if (!D) return;
  for (void* p : {D->V, D->AV, D->E, D->coef, D->tmp, D->tmp2})
    if (p) cudaFreeAsync(p, D->st);
  free_redbuf(D->rb, D->st);
  delete D;
}

void deflation_make(Operator& A, const void* V, int k) {
  if (A.defl) { deflation_free(A.defl); A.defl = nullptr; }
  if (k <= 0) return;
  if (k > kDefMax) throw std::runtime_error("make_deflation: at most 16 deflation vectors");
  auto* D = new Deflation();
  D->k = k;
  D->multishift = A.multishift;
  D->cplx = A.cplx;
  D->n = A.n();
  D->st = A.stream;
  const size_t es = A.cplx ? 16 : 8;
  try {
    IDRS_CUDA(cudaMallocAsync(&D->V, es * D->n * k, D->st));
    IDRS_CUDA(cudaMallocAsync(&D->AV, es * D->n * k, D->st));
    IDRS_CUDA(cudaMallocAsync(&D->E, es * MAXS * MAXS, D->st));
    IDRS_CUDA(cudaMallocAsync(&D->coef, es * 2 * MAXS, D->st));
    IDRS_CUDA(cudaMallocAsync(&D->tmp, es * std::max<long>(D->n, 1), D->st));
    IDRS_CUDA(cudaMallocAsync(&D->tmp2, es * std::max<long>(D->n, 1), D->st));
    D->rb = alloc_redbuf(D->st);
    if (A.cplx) make_typed<c128>(A, *D, (const c128*)V);
    else make_typed<double>(A, *D, (const double*)V);
    IDRS_CUDA(cudaStreamSynchronize(D->st));
  } catch (...) {
    deflation_free(D);
    throw;
  }
  A.defl = D;
}

template <class T>
void deflation_pmul(const Deflation& D, const T* w, T* out, T fa, T fcv, const T* fv,
                    const int* skip, cudaStream_t st) {
  T* t = (T*)D.coef;
  dots_then<T>(D, w, TDefSolve<T>{(const T*)D.E, t, D.k, !D.multishift, T(0.0)}, skip, st);
  const T* Wm = (const T*)(D.multishift ? D.V : D.AV);
  k_defl_pmul<T><<<stream_grid(D.n), kThreads, 0, st>>>(D.n, w, out, Wm, D.k, t, fa, fcv, fv, skip);
  IDRS_LAUNCH_CHECK();
}

template <class T>
void deflation_add(Operator& A, c128 sigma_s, const T* b, const T* y, T* x, const int* skip,
                   cudaStream_t st) {
  const Deflation& D = *A.defl;
  T* t1 = (T*)D.coef;
  T* t2 = t1 + MAXS;
  const T ss = narrow<T>(sigma_s);
  dots_then<T>(D, b, TDefSolve<T>{(const T*)D.E, t1, D.k, true, ss}, skip, st);
  // Ay - sigma_s y with Ay = real_mv(A, y)
  MatView Ks = A.view(64);
  Ks.defl = nullptr;
  T* ay = (T*)D.tmp2;
  ks_mv<T>(Ks, y, ay, T(1), T(0) - ss, y, skip, st);
  dots_then<T>(D, ay, TDefSolve<T>{(const T*)D.E, t2, D.k, true, ss}, skip, st);
  k_defl_add<T><<<stream_grid(D.n), kThreads, 0, st>>>(D.n, (const T*)D.V, D.k, t1, t2, y, x, skip);
  IDRS_LAUNCH_CHECK();
}

template void deflation_pmul<double>(const Deflation&, const double*, double*, double, double,
                                     const double*, const int*, cudaStream_t);
template void deflation_pmul<c128>(const Deflation&, const c128*, c128*, c128, c128, const c128*,
                                   const int*, cudaStream_t);
template void deflation_add<double>(Operator&, c128, const double*, const double*, double*,
                                    const int*, cudaStream_t);
template void deflation_add<c128>(Operator&, c128, const c128*, const c128*, c128*, const int*,
                                  cudaStream_t);

}  // namespace idrs
