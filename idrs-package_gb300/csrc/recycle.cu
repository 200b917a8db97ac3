// recycle.cu -- recycling outputs of IDRS_RITZ (ritz_module.f90:389-556).
//
// Host part: the dense work on the (nritz x nritz) Hessenberg matrix, i.e.
// RSI_power (dense_la_module.f90:531-603, with RQR_factorization :84-124 and
// RQR_solve :159-190) and the omega ordering (ritz_module.f90:497-520).
// Device part: rcompute_U0 (ritz_module.f90:100-160), one operator product
// and one fused element pass per Ritz step, and global_RQR_factorization
// (ritz_module.f90:66-96) as fused modified Gram-Schmidt passes whose
// coefficients stay on the device.
#include <cfloat>
#include <cmath>
#include <complex>
#include <memory>
#include <stdexcept>
#include <vector>

#include "idrs_gpu.cuh"
#include "recycle.h"
#include "setup.h"

namespace idrs {

// ------------------------------------------------------------------- host
namespace {

// RQR_factorization with two refinement sweeps.  Q (m x n), R (n x n),
// column-major.  Returns 0 or the 1-based dependent column (Q, R partial).
int rqr_factorization(int m, int n, const double* V, int ldv, double* Q, double* R) {
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) Q[i + (size_t)m * j] = V[i + (size_t)ldv * j];
  std::fill(R, R + (size_t)n * n, 0.0);
  for (int j = 0; j < n; ++j) {
    double* qj = Q + (size_t)m * j;
    for (int sweep = 0; sweep < 2; ++sweep)
      for (int i = 0; i < j; ++i) {
        const double* qi = Q + (size_t)m * i;
        double t = 0;
        for (int q = 0; q < m; ++q) t += qi[q] * qj[q];
        for (int q = 0; q < m; ++q) qj[q] = qj[q] - t * qi[q];
        R[i + (size_t)n * j] += t;
      }
    double nr = 0;
    for (int q = 0; q < m; ++q) nr += qj[q] * qj[q];
    const double rjj = std::sqrt(nr);
    R[j + (size_t)n * j] = rjj;
    if (!(rjj > DBL_MIN)) return j + 1;
    for (int q = 0; q < m; ++q) qj[q] = qj[q] / rjj;
  }
  return 0;
}

// X (n x s) = R^-1 (Q^T B), Q (m x n), B (m x s)
void rqr_solve(int m, int n, int s, const double* Q, const double* R, const double* B, double* X) {
  for (int c = 0; c < s; ++c)
    for (int i = 0; i < n; ++i) {
      double t = 0;
      const double* qi = Q + (size_t)m * i;
      const double* bc = B + (size_t)m * c;
      for (int q = 0; q < m; ++q) t += qi[q] * bc[q];
      X[i + (size_t)n * c] = t;
    }
  for (int j = n - 1; j >= 0; --j)
    for (int c = 0; c < s; ++c) {
      double* xc = X + (size_t)n * c;
      xc[j] = xc[j] / R[j + (size_t)n * j];
      for (int i = 0; i < j; ++i) xc[i] = xc[i] - R[i + (size_t)n * j] * xc[j];
    }
}

}  // namespace

int si_power(const double* H, int ldh, int n, int s, double shift, uint64_t seed, double* vec) {
  if (s < 1 || n < s) return 1;
  const size_t nn = (size_t)n * n, ns = (size_t)n * s;
  std::vector<double> A(nn), Q(nn), R(nn), sv(ns), Qs(ns), Rs((size_t)s * s);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) A[i + (size_t)n * j] = H[i + (size_t)ldh * j];
  for (int i = 0; i < n; ++i) A[i + (size_t)n * i] -= shift;
  rqr_factorization(n, n, A.data(), n, Q.data(), R.data());
  for (size_t k = 0; k < ns; ++k) sv[k] = uniform01(seed, (uint64_t)k);
  rqr_factorization(n, s, sv.data(), n, Qs.data(), Rs.data());
  // the change of the summed column lengths, relative to the start block's,
  // ends the iteration (tolerance 1e-3, at most 1000 sweeps)
  double trace0 = 0;
  for (int i = 0; i < s; ++i) trace0 += Rs[i + (size_t)s * i];
  double trace_old = trace0, err = 1;
  for (int iter = 0; err > 1e-3 && iter < 1000; ++iter) {
    rqr_solve(n, n, s, Q.data(), R.data(), Qs.data(), sv.data());
    rqr_factorization(n, s, sv.data(), n, Qs.data(), Rs.data());
    double trace = 0;
    for (int i = 0; i < s; ++i) trace += Rs[i + (size_t)s * i];
    err = std::fabs(trace - trace_old) / trace0;
    trace_old = trace;
  }
  std::copy(Qs.begin(), Qs.end(), vec);
  return 0;
}

void ritz_omega(const double* Hf, int ldh, int n_omega, double* omega) {
  std::vector<std::complex<double>> rv(n_omega);
  std::vector<double> p(n_omega, 1.0);
  int converged = 0;
  qr_eig(Hf, ldh, n_omega, rv.data(), &converged);
  for (int i = 0; i < n_omega; ++i) {
    double w = rv[i].real();
    if (std::fabs(w) < DBL_EPSILON) w = 1.0;
    omega[i] = 1.0 / w;
  }
  for (int i = 0; i < n_omega; ++i) {
    int mp = i;  // first position of max |p| over i..n_omega-1
    for (int k = i + 1; k < n_omega; ++k)
      if (std::fabs(p[k]) > std::fabs(p[mp])) mp = k;
    std::swap(omega[mp], omega[i]);
    for (int k = 0; k < n_omega; ++k) p[k] = p[k] * (1.0 - rv[k].real() * omega[i]);
  }
}

void ritz_omega(const std::complex<double>* Hf, int ldh, int n_omega, std::complex<double>* omega) {
  using cd = std::complex<double>;
  std::vector<cd> rv(n_omega), p(n_omega, cd(1.0, 0.0));
  int converged = 0;
  qr_eig(Hf, ldh, n_omega, rv.data(), &converged);
  for (int i = 0; i < n_omega; ++i) {
    cd w = rv[i];
    if (std::abs(w) < DBL_EPSILON) w = cd(1.0, 0.0);
    omega[i] = cd(1.0, 0.0) / w;
  }
  for (int i = 0; i < n_omega; ++i) {
    int mp = i;
    for (int k = i + 1; k < n_omega; ++k)
      if (std::abs(p[k]) > std::abs(p[mp])) mp = k;
    std::swap(omega[mp], omega[i]);
    for (int k = 0; k < n_omega; ++k) p[k] = p[k] * (cd(1.0, 0.0) - rv[k] * omega[i]);
  }
}

// ----------------------------------------------------------------- device
namespace {

struct DevVec {
  void* p = nullptr;
  cudaStream_t st;
  DevVec(size_t bytes, cudaStream_t s) : st(s) {
    IDRS_CUDA(cudaMallocAsync(&p, std::max<size_t>(bytes, 16), s));
  }
  DevVec(const DevVec&) = delete;
  DevVec& operator=(const DevVec&) = delete;
  ~DevVec() { if (p) cudaFreeAsync(p, st); }
  template <class T> T* as() const { return (T*)p; }
};

// Coefficients of one Ritz step of compute_U0.
template <class T>
struct U0Step {
  T e[MAXS];             // eigvec(i, 1:ns)
  T h[MAXS + 1];         // H(low:i, i)
  int col[MAXS + 1];     // ring columns of v_low .. v_i
  int nl, ns;            // window length, number of U columns
  int cur, next;         // ring columns of v_i and v_{i+1}
  T hden;                // H(i+1, i)
};

// U(:,j) += e_j v_i;  v_{i+1} = (t - sum_l h_l v_l) / hden.  v_{i+1}
// overwrites the ring column of v_{i-ns}, which this thread reads first.
template <class T>
__global__ void __launch_bounds__(kThreads) k_u0_step(long n, const T* __restrict__ t, T* W, T* U,
                                                      U0Step<T> c) {
  const long stride = (long)gridDim.x * blockDim.x;
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += stride) {
    const T v = W[c.cur * n + q];
    for (int j = 0; j < c.ns; ++j) U[j * n + q] = U[j * n + q] + c.e[j] * v;
    T acc = T(0.0);
    for (int l = 0; l < c.nl; ++l) acc = acc + W[c.col[l] * n + q] * c.h[l];
    W[c.next * n + q] = (t[q] - acc) / c.hden;
  }
}

// x(:,j) = x(:,j) / d[j]   (d: real values on the device)
template <class T>
__global__ void k_div_cols(long n, int cols, T* x, const double* d) {
  const long stride = (long)gridDim.x * blockDim.x;
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n * cols; q += stride) {
    const long j = q / n;
    x[q] = x[q] / T(d[j]);
  }
}

inline double mag(double v) { return std::fabs(v); }
inline double mag(c128 v) { return std::hypot(v.x, v.y); }

__device__ inline double re_part(double v) { return v; }
__device__ inline double re_part(c128 v) { return v.x; }

// stores sqrt(Re v) (a norm) as a real value
template <class W> struct TNormAt {
  double* out;
  __device__ void operator()(const W* v) const { *out = sqrt(re_part(v[0])); }
};

// R(i, j) = v (an inner product) or sqrt(Re v) (the norm, i = j)
template <class W> struct TRAt {
  W* out; bool root;
  __device__ void operator()(const W* v) const {
    if (root) *out = W(sqrt(re_part(v[0])));
    else *out = v[0];
  }
};

// One modified Gram-Schmidt pass on column j: with i > 0 first
// Q_j -= R(i-1,j) Q_{i-1}; then acc0 = Q_i^H Q_j (i < j) or |Q_j|^2 (i = j).
template <class T>
struct BMgsPass {
  T* Q; long ld; int i, j; const T* Rj;
  struct Shared { T c; };
  __device__ void prepare(Shared& sh) const {
    if (threadIdx.x == 0) sh.c = i > 0 ? Rj[i - 1] : T(0.0);
  }
  template <int ND, class A>
  __device__ void operator()(long q, Shared& sh, A (&acc)[ND]) const {
    T qj = Q[j * ld + q];
    if (i > 0) {
      qj = qj - sh.c * Q[(i - 1) * ld + q];
      Q[j * ld + q] = qj;
    }
    if (i < j) acc_add(acc[0], conj_(Q[i * ld + q]) * qj);
    else acc_add(acc[0], abs2_(qj));
  }
};

// Q_j = Q_j / R(j,j) when |R(j,j)| > DBL_MIN (else left for the host check)
template <class T>
__global__ void k_mgs_scale(long n, T* qj, const T* rjj) {
  const T r = *rjj;
  if (!(abs_(r) > DBL_MIN)) return;
  const long stride = (long)gridDim.x * blockDim.x;
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += stride) qj[q] = qj[q] / r;
}

}  // namespace

template <class T>
void compute_u0(Operator& A, Operator* M, const T* H, int ldh, int nritz, const T* eigvec, int ns,
                const T* b, T* U, double* resnrm, cudaStream_t st) {
  if (ns < 1 || ns > MAXS) throw std::runtime_error("compute_U0: dimension of U0 out of range");
  if (nritz < 1 || ldh < nritz + 1) throw std::runtime_error("compute_U0: bad Hessenberg size");
  const long n = A.n();
  const int ring = ns + 1;
  DevVec W(sizeof(T) * n * ring, st), t(sizeof(T) * n, st), t1(sizeof(T) * n, st), t2(sizeof(T) * n, st);
  std::unique_ptr<DevVec> u;
  if (M) u.reset(new DevVec(sizeof(T) * n, st));
  IDRS_CUDA(cudaMemsetAsync(U, 0, sizeof(T) * n * ns, st));
  IDRS_CUDA(cudaMemcpyAsync(W.p, b, sizeof(T) * n, cudaMemcpyDeviceToDevice, st));
  std::vector<int> ind(nritz + 1, 0);
  int k = 0;
  for (int i = 1; i <= nritz; ++i) {
    k = k + 1;
    if (k > ring) k = 1;
    ind[i] = k;
    const T* v = W.as<T>() + (size_t)(k - 1) * n;
    if (M) {
      op_precon<T>(*M, 64, v, u->as<T>(), nullptr, st);
      op_chain<T>(A.view(64), A.alpha_p, A.degree, u->as<T>(), t.as<T>(), t1.as<T>(), t2.as<T>(), nullptr, st);
    } else {
      op_chain<T>(A.view(64), A.alpha_p, A.degree, v, t.as<T>(), t1.as<T>(), t2.as<T>(), nullptr, st);
    }
    U0Step<T> c{};
    for (int j = 0; j < ns; ++j) c.e[j] = eigvec[(i - 1) + (size_t)nritz * j];
    const int low = std::max(1, i - ns);
    c.nl = i - low + 1;
    for (int l = low; l <= i; ++l) {
      c.col[l - low] = ind[l] - 1;
      c.h[l - low] = H[(l - 1) + (size_t)ldh * (i - 1)];
    }
    c.ns = ns;
    c.cur = k - 1;
    c.next = k % ring;
    c.hden = H[i + (size_t)ldh * (i - 1)];
    k_u0_step<T><<<stream_grid(n), kThreads, 0, st>>>(n, t.as<T>(), W.as<T>(), U, c);
    IDRS_LAUNCH_CHECK();
  }
  if (resnrm) {
    // norms of U(:,j) and of v_{nritz+1}, then U(:,j) /= |U(:,j)|
    using Wt = typename traits<T>::wide;
    DevVec nr(sizeof(double) * (ns + 1), st);
    for (int j = 0; j < ns; ++j)
      launch_fused<1, T>(n, BNorm<T>{U + (size_t)n * j}, TNormAt<Wt>{nr.as<double>() + j}, A.red, nullptr, st);
    const T* vlast = W.as<T>() + (size_t)(k % ring) * n;
    launch_fused<1, T>(n, BNorm<T>{vlast}, TNormAt<Wt>{nr.as<double>() + ns}, A.red, nullptr, st);
    k_div_cols<T><<<stream_grid(n * ns), kThreads, 0, st>>>(n, ns, U, nr.as<double>());
    IDRS_LAUNCH_CHECK();
    std::vector<double> h(ns + 1);
    IDRS_CUDA(cudaMemcpyAsync(h.data(), nr.p, sizeof(double) * (ns + 1), cudaMemcpyDeviceToHost, st));
    IDRS_CUDA(cudaStreamSynchronize(st));
    const double hl = mag(H[nritz + (size_t)ldh * (nritz - 1)]);
    for (int j = 0; j < ns; ++j)
      resnrm[j] = h[ns] * hl * mag(eigvec[(nritz - 1) + (size_t)nritz * j]) / h[j];
  }
}

template <class T>
int global_qr(long n, int s, T* Q, T* R, RedBuf rb, cudaStream_t st) {
  using Wt = typename traits<T>::wide;
  DevVec dR(sizeof(T) * s * s, st);
  IDRS_CUDA(cudaMemsetAsync(dR.p, 0, sizeof(T) * s * s, st));
  for (int j = 0; j < s; ++j) {
    T* Rj = dR.as<T>() + (size_t)s * j;
    for (int i = 0; i <= j; ++i)
      launch_fused<1, T>(n, BMgsPass<T>{Q, n, i, j, Rj}, TRAt<Wt>{(Wt*)(Rj + i), i == j}, rb, nullptr, st);
    k_mgs_scale<T><<<stream_grid(n), kThreads, 0, st>>>(n, Q + (size_t)n * j, Rj + j);
    IDRS_LAUNCH_CHECK();
  }
  std::vector<T> h((size_t)s * s);
  IDRS_CUDA(cudaMemcpyAsync(h.data(), dR.p, sizeof(T) * s * s, cudaMemcpyDeviceToHost, st));
  IDRS_CUDA(cudaStreamSynchronize(st));
  if (R) std::copy(h.begin(), h.end(), R);
  for (int j = 0; j < s; ++j)
    if (!(mag(h[j + (size_t)s * j]) > DBL_MIN)) return j + 1;
  return 0;
}

template void compute_u0<double>(Operator&, Operator*, const double*, int, int, const double*, int,
                                 const double*, double*, double*, cudaStream_t);
template void compute_u0<c128>(Operator&, Operator*, const c128*, int, int, const c128*, int,
                               const c128*, c128*, double*, cudaStream_t);
template int global_qr<double>(long, int, double*, double*, RedBuf, cudaStream_t);
template int global_qr<c128>(long, int, c128*, c128*, RedBuf, cudaStream_t);

}  // namespace idrs
