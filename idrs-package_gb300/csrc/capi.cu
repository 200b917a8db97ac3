// capi.cu -- the extern "C" boundary (include/idrs_gb300.h).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <mutex>
#include <complex>
#include <cstring>
#include <memory>
#include <new>
#include <stdexcept>
#include <vector>

#include "../../include/idrs_gb300.h"
#include "adjoint.h"
#include "recycle.h"
#include "idrs_gpu.cuh"
#include "ms_gpu.cuh"
#include "setup.h"
#include "tma.cuh"

using namespace idrs;

struct idrs_user_matrix_s : UserMatrix {};
struct idrs_matrix_s : Operator {};

namespace {

using cd = std::complex<double>;

struct arg_error : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct unsupported_error : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// A lost staged copy (k_band_trsv) sets the process's fault word.  The word
// is cleared when a call starts, so a fault is charged only to the call that
// saw it.  A call in host-pointer mode has synchronised its stream (its
// results are copied back) before the word is read; a call in device-pointer
// mode may return while its kernels still run, and then reports a lost copy
// only through the NaN values the solve writes.
template <class F>
int guard(F&& f) {
  try {
    take_device_fault();
    const int rc = f();
    if (take_device_fault()) {
      set_error("a staged (TMA) copy never arrived; the result is invalid");
      return IDRS_ERR_CUDA;
    }
    return rc;
  } catch (const cuda_error& e) {
    set_error(std::string(cudaGetErrorString(e.code)) + " (" + e.where + ")");
    return e.code == cudaErrorMemoryAllocation ? IDRS_ERR_ALLOC : IDRS_ERR_CUDA;
  } catch (const arg_error& e) {
    set_error(e.what());
    return IDRS_ERR_ARG;
  } catch (const unsupported_error& e) {
    set_error(e.what());
    return IDRS_ERR_UNSUPPORTED;
  } catch (const std::bad_alloc&) {
    set_error("host allocation failed");
    return IDRS_ERR_ALLOC;
  } catch (const std::exception& e) {
    set_error(e.what());
    return IDRS_ERR_ARG;
  }
}

#define REQUIRE(cond, msg) \
  do {                     \
    if (!(cond)) throw arg_error(msg); \
  } while (0)

// The stream-ordered pool of each device keeps the memory of finished calls
// (release threshold: never), so the per-call work vectors of a solve are
// reused instead of mapped again; set once per device, from any thread.
void init_runtime() {
  static std::atomic<uint64_t> done{0};
  static std::mutex mu;
  int dev = 0;
  IDRS_CUDA(cudaGetDevice(&dev));
  const uint64_t bit = dev < 64 ? uint64_t(1) << dev : 0;
  if (bit && (done.load(std::memory_order_acquire) & bit)) return;
  std::lock_guard<std::mutex> lock(mu);
  if (bit && (done.load() & bit)) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  cudaGetLastError();
  done.fetch_or(bit, std::memory_order_release);
}

// device buffer owned for the duration of one call
struct DBuf {
  void* p = nullptr;
  cudaStream_t st = nullptr;
  DBuf() = default;
  DBuf(size_t bytes, cudaStream_t s) : st(s) {
    IDRS_CUDA(cudaMallocAsync(&p, std::max<size_t>(bytes, 16), s));
  }
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept : p(o.p), st(o.st) { o.p = nullptr; }
  DBuf& operator=(DBuf&& o) noexcept {
    if (this != &o) {
      if (p) cudaFreeAsync(p, st);
      p = o.p; st = o.st; o.p = nullptr;
    }
    return *this;
  }
  ~DBuf() { if (p) cudaFreeAsync(p, st); }
  template <class T> T* as() const { return (T*)p; }
};

void* upload(const void* h, size_t bytes) {
  void* d = nullptr;
  IDRS_CUDA(cudaMalloc(&d, std::max<size_t>(bytes, 16)));
  if (h && bytes) IDRS_CUDA(cudaMemcpy(d, h, bytes, cudaMemcpyHostToDevice));
  return d;
}

// Lanes per row of the CRS kernel: one thread per row for short rows (no
// FP64 shuffle additions), otherwise a power-of-two sub-warp.
int crs_group(long nnz, long nrows) {
  double mean = nrows > 0 ? (double)nnz / nrows : 1.0;
  if (mean <= 16.0) return 1;
  int g = 2;
  while (g < 32 && g < mean) g *= 2;
  return g;
}

// Vector staging for host-pointer mode: uploads `in`, gives a device pointer,
// and downloads to `out` on finish().
struct Staged {
  Operator* A;
  size_t bytes;
  std::vector<DBuf> bufs;
  Staged(Operator* a, size_t b) : A(a), bytes(b) {}
  const void* in(const void* h) {
    if (!h) return nullptr;
    if (A->device_pointers) return h;
    bufs.emplace_back(bytes, A->stream);
    IDRS_CUDA(cudaMemcpyAsync(bufs.back().p, h, bytes, cudaMemcpyHostToDevice, A->stream));
    return bufs.back().p;
  }
  void* out(void* h) {
    if (A->device_pointers) return h;
    bufs.emplace_back(bytes, A->stream);
    return bufs.back().p;
  }
  void finish(void* h, const void* d) {
    if (A->device_pointers || !h) return;
    IDRS_CUDA(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, A->stream));
  }
};

const void* find_shadow(Operator* A, int s) {
  for (auto& p : A->shadows)
    if (p.first == s) return p.second;
  return nullptr;
}

// ----------------------------------------------------------------- diagonal
template <class V>
__global__ void k_diag_crs(int n, const int* rp, const int* ci, const V* val, V* D) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (long)blockDim.x) {
    V d = V(0.0);
    for (int k = rp[i]; k < rp[i + 1]; ++k)
      if (ci[k] == i) d = d + val[k];
    D[i] = d;
  }
}
template <class V>
__global__ void k_diag_cds(int n, int hb, const V* band, V* D) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (long)blockDim.x)
    D[i] = band[i + (long)n * hb];
}
template <class V>
__global__ void k_diag_dense(int n, const V* mat, V* D) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (long)blockDim.x)
    D[i] = mat[i + (long)n * i];
}
template <class V>
__global__ void k_diag_fix(int n, V* D, V shift) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (long)blockDim.x) {
    V d = D[i];
    if (d == V(0.0)) d = V(1.0);  // where (D == 0) D = 1 (user_module.f90:1043-1045)
    D[i] = d - shift;
  }
}

template <class V>
void diagonal_into(const UserMatrix& K, V* D, cudaStream_t st) {
  int n = K.nrows;
  switch (K.format) {
    case FMT_CRS:
    case FMT_COO: k_diag_crs<V><<<stream_grid(n), kThreads, 0, st>>>(n, K.row_ptr, K.col_ind, (const V*)K.val, D); break;
    case FMT_CDS: k_diag_cds<V><<<stream_grid(n), kThreads, 0, st>>>(n, K.half_band, (const V*)K.band, D); break;
    case FMT_DENSE: k_diag_dense<V><<<stream_grid(n), kThreads, 0, st>>>(n, (const V*)K.mat, D); break;
    default: throw unsupported_error("diagonal: unsupported format");
  }
  IDRS_LAUNCH_CHECK();
}
__global__ void k_promote(long n, const double* a, c128* b) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (long)blockDim.x) b[i] = c128(a[i], 0.0);
}

// Diagonal of K (complex if K is complex or `want_cplx`), D==0 -> 1, minus shift.
void* make_diagonal(const UserMatrix& K, bool want_cplx, c128 shift, bool* is_cplx) {
  int n = K.nrows;
  bool cplx = want_cplx || K.vals == 2;
  *is_cplx = cplx;
  void* D = nullptr;
  IDRS_CUDA(cudaMalloc(&D, (cplx ? 16 : 8) * (size_t)std::max(n, 1)));
  cudaStream_t st = nullptr;
  if (cplx) {
    if (K.vals == 2) {
      diagonal_into<c128>(K, (c128*)D, st);
    } else {
      double* tmp = nullptr;
      IDRS_CUDA(cudaMalloc(&tmp, 8 * (size_t)std::max(n, 1)));
      diagonal_into<double>(K, tmp, st);
      k_promote<<<stream_grid(n), kThreads, 0, st>>>(n, tmp, (c128*)D);
      IDRS_LAUNCH_CHECK();
      IDRS_CUDA(cudaDeviceSynchronize());
      cudaFree(tmp);
    }
    k_diag_fix<c128><<<stream_grid(n), kThreads, 0, st>>>(n, (c128*)D, shift);
  } else {
    diagonal_into<double>(K, (double*)D, st);
    k_diag_fix<double><<<stream_grid(n), kThreads, 0, st>>>(n, (double*)D, shift.x);
  }
  IDRS_LAUNCH_CHECK();
  IDRS_CUDA(cudaDeviceSynchronize());
  return D;
}


// -------------------------------------------------- polynomial set-up
int set_preconditioner(Operator* A, int preconditioner, int degree, const double* foci,
                       const double* center, const double* H, int ldh, int nh) {
  REQUIRE(preconditioner >= 0 && preconditioner <= 3, "illegal value for preconditioner");
  REQUIRE(degree >= 0 && degree <= 62, "illegal polynomial degree");
  A->preconditioner = preconditioner;
  A->degree = (preconditioner == 0) ? 0 : degree;
  A->alpha_p.assign(A->degree + 1, c128(1.0, 0.0));
  A->jac = JacobiCols();
  if (A->degree == 0) return IDRS_OK;
  // keeps the tridiagonal Jacobi matrix for the stable fp32 evaluation
  auto keep_jacobi = [&](const std::vector<cd>& J) {
    const int d = A->degree, ld = d + 2;
    A->jac.a.assign(d + 1, c128(0.0));
    A->jac.b.assign(d + 1, c128(0.0));
    A->jac.c.assign(d + 1, c128(0.0));
    for (int i = 1; i <= d + 1; ++i) {
      if (i >= 2) A->jac.a[i - 1] = c128(J[(i - 2) + (size_t)ld * (i - 1)].real(), J[(i - 2) + (size_t)ld * (i - 1)].imag());
      A->jac.b[i - 1] = c128(J[(i - 1) + (size_t)ld * (i - 1)].real(), J[(i - 1) + (size_t)ld * (i - 1)].imag());
      A->jac.c[i - 1] = c128(J[i + (size_t)ld * (i - 1)].real(), J[i + (size_t)ld * (i - 1)].imag());
    }
  };
  if (!A->cplx) {
    std::vector<double> al(A->degree + 1);
    int st = 0;
    if (preconditioner == 1) {
      double c;
      if (center) c = *center - A->seed.x;
      else if (H) analyse_spectrum(H, ldh, nh, nullptr, &c, nullptr);
      else c = 1.0;
      st = neumann(A->degree, c, al.data());
      keep_jacobi(neumann_jacobi(A->degree, cd(c, 0.0)));
    } else if (preconditioner == 2) {
      double f[2];
      if (foci) { f[0] = foci[0] - A->seed.x; f[1] = foci[1] - A->seed.x; }
      else if (H) analyse_spectrum(H, ldh, nh, f, nullptr, nullptr);
      else { f[0] = 0.25; f[1] = 1.75; }
      st = chebyshev(A->degree, f, al.data());
      cd fc[2] = {cd(f[0], 0.0), cd(f[1], 0.0)};
      keep_jacobi(chebyshev_jacobi(A->degree, fc));
    } else {
      REQUIRE(H, "the Hessenberg preconditioner needs H");
      st = compute_alpha(A->degree, H, ldh, nh, al.data());
    }
    REQUIRE(st == 0, "Hessenberg matrix too small for polynomial degree");
    for (int i = 0; i <= A->degree; ++i) A->alpha_p[i] = c128(al[i], 0.0);
  } else {
    std::vector<cd> al(A->degree + 1);
    cd seed(A->seed.x, A->seed.y);
    int st = 0;
    std::vector<cd> Hc;
    if (H) {
      Hc.resize((size_t)ldh * nh);
      for (size_t i = 0; i < Hc.size(); ++i) Hc[i] = cd(H[2 * i], H[2 * i + 1]);
    }
    if (preconditioner == 1) {
      cd c;
      if (center) c = cd(center[0], center[1]) - seed;
      else if (H) analyse_spectrum(Hc.data(), ldh, nh, nullptr, &c, nullptr);
      else c = 1.0;
      st = neumann(A->degree, c, al.data());
      keep_jacobi(neumann_jacobi(A->degree, c));
    } else if (preconditioner == 2) {
      cd f[2];
      if (foci) { f[0] = cd(foci[0], foci[1]) - seed; f[1] = cd(foci[2], foci[3]) - seed; }
      else if (H) analyse_spectrum(Hc.data(), ldh, nh, f, nullptr, nullptr);
      else { f[0] = 0.25; f[1] = 1.75; }
      st = chebyshev(A->degree, f, al.data());
      keep_jacobi(chebyshev_jacobi(A->degree, f));
    } else {
      REQUIRE(H, "the Hessenberg preconditioner needs H");
      st = compute_alpha(A->degree, Hc.data(), ldh, nh, al.data());
    }
    REQUIRE(st == 0, "Hessenberg matrix too small for polynomial degree");
    for (int i = 0; i <= A->degree; ++i) A->alpha_p[i] = c128(al[i].real(), al[i].imag());
  }
  return IDRS_OK;
}

// ---------------------------------------------------------------- solvers
template <class T>
int run_idrs(Operator* A, const double* b, int s, Operator* M1, const double* tolerance,
             const int* maximum_iterations, const int* variant, int* flag, double* relres,
             int* iterations, const double* x0, const double* U0, const double* omega, int n_omega,
             double* resvec, int resvec_len, double* H, int ldh, int nritz, double* x) {
  using W = typename traits<T>::wide;
  REQUIRE(A && b && x, "idrs: A, b and x are required");
  REQUIRE(s >= 1, "idrs: s must be positive");
  if (s > MAXS) throw unsupported_error("idrs: s > 16 is not supported by the GPU path");
  SolveOpts o;
  if (tolerance) {
    REQUIRE(*tolerance >= 0, "Illegal value for parameter tolerance");
    o.tol = *tolerance;
  }
  const long n = A->n();
  o.maxit = maximum_iterations ? *maximum_iterations : (int)std::min<long>(2 * n, 1000);
  o.method = variant ? *variant : 1;
  REQUIRE(o.method >= 1 && o.method <= 4, "idrs: variant must be 1..4");
  REQUIRE(o.method == 1 || s == 1, "idrs: variants 2-4 use s = 1");
  if (flag) *flag = -1;
  if (relres) *relres = 1.0;
  if (iterations) *iterations = 0;
  if (resvec) REQUIRE(o.maxit + 1 <= resvec_len, "Length of vector with residual norms too small, should be maxit+1");
  bool out_H = (H != nullptr) && nritz > 0;
  if (H && nritz > 0) REQUIRE(ldh == nritz + 1, "Second dimension of H incompatible, with first");
  cudaStream_t st = A->stream;
  Staged sv(A, sizeof(T) * n);
  const T* d_b = (const T*)sv.in(b);
  const T* d_x0 = (const T*)sv.in(x0);
  T* d_x = (T*)sv.out(x);
  Staged su(A, sizeof(T) * n * s);
  const T* d_U0 = (const T*)su.in(U0);
  DBuf d_res, d_H, d_om;
  if (resvec) { d_res = DBuf(sizeof(double) * resvec_len, st); IDRS_CUDA(cudaMemsetAsync(d_res.p, 0, sizeof(double) * resvec_len, st)); }
  if (out_H) { d_H = DBuf(sizeof(W) * ldh * nritz, st); IDRS_CUDA(cudaMemsetAsync(d_H.p, 0, sizeof(W) * ldh * nritz, st)); }
  if (omega && n_omega > 0) {
    d_om = DBuf(sizeof(W) * n_omega, st);
    IDRS_CUDA(cudaMemcpyAsync(d_om.p, omega, sizeof(W) * n_omega, cudaMemcpyHostToDevice, st));
  }
  o.M1 = M1;
  o.x0 = d_x0;
  o.U0 = d_U0;
  o.omega = d_om.p;
  o.n_omega = n_omega;
  o.resvec = d_res.as<double>();
  o.resvec_len = resvec_len;
  o.H = out_H ? d_H.p : nullptr;
  o.ldH = ldh;
  o.nritz = out_H ? nritz : 0;
  o.PT = find_shadow(A, s);
  IdrsGpu<T> solver(*A, 64, s, o.method);
  solver.solve(d_b, d_x, o);
  auto h = solver.state();
  sv.finish(x, d_x);
  if (resvec) IDRS_CUDA(cudaMemcpyAsync(resvec, d_res.p, sizeof(double) * resvec_len, cudaMemcpyDeviceToHost, st));
  if (out_H) IDRS_CUDA(cudaMemcpyAsync(H, d_H.p, sizeof(W) * ldh * nritz, cudaMemcpyDeviceToHost, st));
  IDRS_CUDA(cudaStreamSynchronize(st));
  if (flag) *flag = h.info;
  if (relres) *relres = h.relres;
  if (iterations) *iterations = h.iter;
  return IDRS_OK;
}

template <class T, class Tin>
void run_qmr_typed(Operator* A, int s, const T* d_b, T* d_x, SolveOpts& o, int* flag,
                   double* relres, int* iterations) {
  QmrGpu<T, Tin> solver(*A, s, o);
  solver.solve(d_b, d_x, o);
  auto h = solver.state();
  A->last_inner_calls = h.inner_calls;
  A->last_inner_total = h.inner_total;
  A->last_inner_max = h.inner_max;
  if (flag) *flag = h.info;
  if (relres) *relres = h.relres;
  if (iterations) *iterations = h.iter;
}

template <class T, class Tlow>
int run_qmridr(Operator* A, const double* b, int s, Operator* M1, const double* tolerance,
               const int* maximum_iterations, int* flag, double* relres, int* iterations,
               const int* inner_s, const double* inner_tolerance, const int* inner_iterations,
               const double* x0, const double* omega, int n_omega, double* resvec,
               int resvec_len, const int* inner_precision, double* x) {
  using W = typename traits<T>::wide;
  REQUIRE(A && b && x, "qmridr: A, b and x are required");
  REQUIRE(s >= 1, "qmridr: s must be positive");
  if (s > MAXS) throw unsupported_error("qmridr: s > 16 is not supported by the GPU path");
  SolveOpts o;
  if (tolerance) {
    REQUIRE(*tolerance >= 0, "Illegal value for parameter tolerance");
    o.tol = *tolerance;
  }
  const long n = A->n();
  o.maxit = maximum_iterations ? *maximum_iterations : (int)std::min<long>(2 * n, 1000);
  o.in_s = inner_s ? *inner_s : 4;
  REQUIRE(o.in_s >= 1, "Illegal value for parameter inner_s");
  if (o.in_s > MAXS) throw unsupported_error("qmridr: inner_s > 16 is not supported by the GPU path");
  o.in_tol = inner_tolerance ? *inner_tolerance : kInnerTolDefault;
  REQUIRE(o.in_tol >= 0, "Illegal value for parameter inner_tolerance");
  o.in_it = inner_iterations ? *inner_iterations : 0;
  o.in_prec = inner_precision ? *inner_precision : 64;
  REQUIRE(o.in_prec == 64 || o.in_prec == 32, "inner_precision must be 64 or 32");
  if (flag) *flag = -1;
  if (relres) *relres = 1.0;
  if (iterations) *iterations = 0;
  if (resvec) REQUIRE(o.maxit + 1 <= resvec_len, "Length of vector with residual norms too small, should be maxit+1");
  cudaStream_t st = A->stream;
  Staged sv(A, sizeof(T) * n);
  const T* d_b = (const T*)sv.in(b);
  const T* d_x0 = (const T*)sv.in(x0);
  T* d_x = (T*)sv.out(x);
  DBuf d_res, d_om;
  if (resvec) { d_res = DBuf(sizeof(double) * resvec_len, st); IDRS_CUDA(cudaMemsetAsync(d_res.p, 0, sizeof(double) * resvec_len, st)); }
  if (omega && n_omega > 0) {
    d_om = DBuf(sizeof(W) * n_omega, st);
    IDRS_CUDA(cudaMemcpyAsync(d_om.p, omega, sizeof(W) * n_omega, cudaMemcpyHostToDevice, st));
  }
  o.M1 = M1;
  o.x0 = d_x0;
  o.omega = d_om.p;
  o.n_omega = n_omega;
  o.resvec = d_res.as<double>();
  o.resvec_len = resvec_len;
  o.PT = find_shadow(A, s);
  if (o.in_it > 0 && o.in_prec == 32) run_qmr_typed<T, Tlow>(A, s, d_b, d_x, o, flag, relres, iterations);
  else run_qmr_typed<T, T>(A, s, d_b, d_x, o, flag, relres, iterations);
  sv.finish(x, d_x);
  if (resvec) IDRS_CUDA(cudaMemcpyAsync(resvec, d_res.p, sizeof(double) * resvec_len, cudaMemcpyDeviceToHost, st));
  IDRS_CUDA(cudaStreamSynchronize(st));
  return IDRS_OK;
}

// ------------------------------------------------------------- multishift
// Shifts and user omegas arrive as host arrays of the vector kind; x is
// n x n_sigma column-major; resvec(resvec_len, n_sigma) column-major.
template <class T>
struct MsCommon {
  using W = typename traits<T>::wide;
  DBuf d_sigma, d_res, d_om;
  void setup(Operator* A, int n_sigma, const double* sigma, const double* omega, int n_omega,
             double* resvec, int resvec_len, int maxit, SolveOpts& o) {
    cudaStream_t st = A->stream;
    d_sigma = DBuf(sizeof(W) * n_sigma, st);
    IDRS_CUDA(cudaMemcpyAsync(d_sigma.p, sigma, sizeof(W) * n_sigma, cudaMemcpyHostToDevice, st));
    if (resvec) {
      REQUIRE(maxit + 1 <= resvec_len, "Length of vector with residual norms too small, should be maxit+1");
      size_t bytes = sizeof(double) * (size_t)resvec_len * n_sigma;
      d_res = DBuf(bytes, st);
      IDRS_CUDA(cudaMemsetAsync(d_res.p, 0, bytes, st));
    }
    if (omega && n_omega > 0) {
      d_om = DBuf(sizeof(W) * n_omega, st);
      IDRS_CUDA(cudaMemcpyAsync(d_om.p, omega, sizeof(W) * n_omega, cudaMemcpyHostToDevice, st));
    }
    o.omega = d_om.p;
    o.n_omega = (omega && n_omega > 0) ? n_omega : 0;
    o.resvec = d_res.as<double>();
    o.resvec_len = resvec_len;
  }
  void finish(Operator* A, int n_sigma, double* resvec, int resvec_len) {
    if (resvec)
      IDRS_CUDA(cudaMemcpyAsync(resvec, d_res.p, sizeof(double) * (size_t)resvec_len * n_sigma,
                                cudaMemcpyDeviceToHost, A->stream));
  }
};

template <class T>
int run_msidrs(Operator* A, const double* b, int n_sigma, const double* sigma, int s, Operator* M1,
               const double* tolerance, const int* maximum_iterations, const int* variant,
               int* flag, double* relres, int* iterations, const double* omega, int n_omega,
               double* resvec, int resvec_len, double* colfac, double* x) {
  using W = typename traits<T>::wide;
  REQUIRE(A && b && sigma && x, "msidrs: A, b, sigma and x are required");
  REQUIRE(s >= 1, "msidrs: s must be positive");
  REQUIRE(n_sigma >= 1, "msidrs: at least one shift is required");
  if (s > MAXS) throw unsupported_error("msidrs: s > 16 is not supported by the GPU path");
  if (n_sigma > MAXSIG) throw unsupported_error("msidrs: more than 64 shifts are not supported by the GPU path");
  SolveOpts o;
  if (tolerance) {
    REQUIRE(*tolerance >= 0, "Illegal value for parameter tolerance");
    o.tol = *tolerance;
  }
  const long n = A->n();
  o.maxit = maximum_iterations ? *maximum_iterations : (int)std::min<long>(2 * n, 1000);
  o.method = variant ? *variant : 1;
  REQUIRE(o.method == 1 || o.method == 2, "msidrs: variant must be 1 (msidrs) or 2 (msbicgstab)");
  REQUIRE(o.method == 1 || s == 1, "msidrs: variant 2 uses one shadow vector (s = 1)");
  if (flag) *flag = -1;
  if (relres) for (int k = 0; k < n_sigma; ++k) relres[k] = 1.0;
  if (iterations) *iterations = 0;
  MsCommon<T> mc;
  mc.setup(A, n_sigma, sigma, omega, n_omega, resvec, resvec_len, o.maxit, o);
  Staged sv(A, sizeof(T) * n), sx(A, sizeof(T) * n * n_sigma);
  const T* d_b = (const T*)sv.in(b);
  T* d_x = (T*)sx.out(x);
  o.M1 = M1;
  o.PT = find_shadow(A, s);
  o.inner = false;
  MsIdrsGpu<T> solver(*A, 64, s, n_sigma, o.method);
  solver.solve(d_b, mc.d_sigma.template as<W>(), d_x, o);
  auto h = solver.state();
  if (flag) *flag = h.info;
  if (iterations) *iterations = h.iter;
  if (relres) for (int k = 0; k < n_sigma; ++k) relres[k] = h.normr[k] / h.normb;
  if (colfac) std::memcpy(colfac, h.phi, sizeof(W) * n_sigma);
  sx.finish(x, d_x);
  mc.finish(A, n_sigma, resvec, resvec_len);
  IDRS_CUDA(cudaStreamSynchronize(A->stream));
  return IDRS_OK;
}

template <class T, class Tin>
void run_msqmr_typed(Operator* A, int s, int n_sigma, const T* d_b, const typename traits<T>::wide* d_sigma,
                     T* d_x, SolveOpts& o, int* flag, double* relres, int* iterations) {
  MsQmrGpu<T, Tin> solver(*A, s, n_sigma, o);
  solver.solve(d_b, d_sigma, d_x, o);
  auto h = solver.state();
  if (flag) *flag = h.info;
  if (iterations) *iterations = h.iter;
  if (relres) for (int k = 0; k < n_sigma; ++k) relres[k] = h.normr[k] / h.normb;
}

template <class T, class Tlow>
int run_msqmridr(Operator* A, const double* b, int n_sigma, const double* sigma, int s, Operator* M1,
                 const double* tolerance, const int* maximum_iterations, int* flag, double* relres,
                 int* iterations, const int* inner_s, const double* inner_tolerance,
                 const int* inner_iterations, const double* omega, int n_omega, double* resvec,
                 int resvec_len, const int* inner_precision, double* x) {
  using W = typename traits<T>::wide;
  REQUIRE(A && b && sigma && x, "msqmridr: A, b, sigma and x are required");
  REQUIRE(s >= 1, "msqmridr: s must be positive");
  REQUIRE(n_sigma >= 1, "msqmridr: at least one shift is required");
  if (s > MAXS) throw unsupported_error("msqmridr: s > 16 is not supported by the GPU path");
  if (n_sigma + 1 > MAXSIG) throw unsupported_error("msqmridr: more than 63 shifts are not supported by the GPU path");
  SolveOpts o;
  if (tolerance) {
    REQUIRE(*tolerance >= 0, "Illegal value for parameter tolerance");
    o.tol = *tolerance;
  }
  const long n = A->n();
  o.maxit = maximum_iterations ? *maximum_iterations : (int)std::min<long>(2 * n, 1000);
  o.in_s = inner_s ? *inner_s : 4;
  REQUIRE(o.in_s >= 1, "Illegal value for parameter inner_s");
  if (o.in_s > MAXS) throw unsupported_error("msqmridr: inner_s > 16 is not supported by the GPU path");
  o.in_tol = inner_tolerance ? *inner_tolerance : kInnerTolDefault;
  REQUIRE(o.in_tol >= 0, "Illegal value for parameter inner_tolerance");
  o.in_it = inner_iterations ? *inner_iterations : 0;
  o.in_prec = inner_precision ? *inner_precision : 64;
  REQUIRE(o.in_prec == 64 || o.in_prec == 32, "inner_precision must be 64 or 32");
  if (flag) *flag = -1;
  if (relres) for (int k = 0; k < n_sigma; ++k) relres[k] = 1.0;
  if (iterations) *iterations = 0;
  MsCommon<T> mc;
  mc.setup(A, n_sigma, sigma, omega, n_omega, resvec, resvec_len, o.maxit, o);
  Staged sv(A, sizeof(T) * n), sx(A, sizeof(T) * n * n_sigma);
  const T* d_b = (const T*)sv.in(b);
  T* d_x = (T*)sx.out(x);
  o.M1 = M1;
  o.PT = find_shadow(A, s);
  const W* d_sigma = mc.d_sigma.template as<W>();
  if (o.in_it > 0 && o.in_prec == 32)
    run_msqmr_typed<T, Tlow>(A, s, n_sigma, d_b, d_sigma, d_x, o, flag, relres, iterations);
  else
    run_msqmr_typed<T, T>(A, s, n_sigma, d_b, d_sigma, d_x, o, flag, relres, iterations);
  sx.finish(x, d_x);
  mc.finish(A, n_sigma, resvec, resvec_len);
  IDRS_CUDA(cudaStreamSynchronize(A->stream));
  return IDRS_OK;
}

template <class W> struct TStoreVals {
  W* out; int cnt;
  __device__ void operator()(const W* v) const { for (int q = 0; q < cnt; ++q) out[q] = v[q]; }
};
template <class T>
struct BDotc {
  const T* u; const T* v;
  using Shared = NoShared;
  __device__ void prepare(Shared&) const {}
  template <int ND, class A>
  __device__ void operator()(long i, Shared&, A (&acc)[ND]) const { acc_add(acc[0], conj_(u[i]) * v[i]); }
};

// D = dK + a dC + b dM + c   (each diagonal with zeros replaced by 1)
template <class V>
__global__ void k_diag_combine(int n, V* D, const V* dC, const V* dM, V a, V b, V c) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (long)blockDim.x) {
    V d = D[i];
    if (dC) d = d + a * dC[i];
    if (dM) d = d + b * dM[i];
    D[i] = d + c;
  }
}
template <class V>
__global__ void k_fill(long n, V* D, V v) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (long)blockDim.x) D[i] = v;
}

// REAL_PRECON / COMPLEX_PRECON diagonal with mass and damping matrices
// (user_module.f90:1352-1381): diag(K) + shift diag(C) + shift^2 diag(M);
// C only: diag(K) + shift diag(C) + shift^2; M only: diag(K) - shift diag(M).
static void* diagonal_with_mc(const UserMatrix& K, const UserMatrix* Mm, const UserMatrix* Cm,
                              bool want_cplx, c128 shift, bool* is_cplx) {
  const int n = K.nrows;
  bool cplx = want_cplx || shift.y != 0.0 || K.vals == 2 || (Mm && Mm->vals == 2) || (Cm && Cm->vals == 2);
  *is_cplx = cplx;
  auto diag_of = [&](const UserMatrix& X) -> void* {
    bool c = false;
    if (X.format == FMT_STENCIL7) {
      void* d = nullptr;
      IDRS_CUDA(cudaMalloc(&d, (cplx ? 16 : 8) * (size_t)std::max(n, 1)));
      double v = X.st[0] == 0.0 ? 1.0 : X.st[0];
      if (cplx) k_fill<c128><<<stream_grid(n), kThreads>>>(n, (c128*)d, c128(v, 0.0));
      else k_fill<double><<<stream_grid(n), kThreads>>>(n, (double*)d, v);
      IDRS_LAUNCH_CHECK();
      return d;
    }
    return make_diagonal(X, cplx, c128(0.0), &c);
  };
  void* D = diag_of(K);
  void* dC = Cm ? diag_of(*Cm) : nullptr;
  void* dM = Mm ? diag_of(*Mm) : nullptr;
  c128 a(0.0), b(0.0), c(0.0);
  if (Mm && Cm) { a = shift; b = shift * shift; }
  else if (Cm) { a = shift; c = shift * shift; }
  else if (Mm) { b = c128(-shift.x, -shift.y); }
  else { c = c128(-shift.x, -shift.y); }
  if (cplx)
    k_diag_combine<c128><<<stream_grid(n), kThreads>>>(n, (c128*)D, (const c128*)dC, (const c128*)dM, a, b, c);
  else
    k_diag_combine<double><<<stream_grid(n), kThreads>>>(n, (double*)D, (const double*)dC, (const double*)dM,
                                                         a.x, b.x, c.x);
  IDRS_LAUNCH_CHECK();
  IDRS_CUDA(cudaDeviceSynchronize());
  if (dC) cudaFree(dC);
  if (dM) cudaFree(dM);
  return D;
}

static int precon_common(int which, idrs_user_matrix K, c128 shift, bool want_cplx, idrs_user_matrix* P,
                         idrs_user_matrix Mm = nullptr, idrs_user_matrix Cm = nullptr,
                         bool has_shift = false) {
  REQUIRE(K && P, "real_precon: bad arguments");
  if (which < 0 || which > 3) throw unsupported_error("precon: which_precon must be 0..3");
  for (const UserMatrix* X : {(const UserMatrix*)Mm, (const UserMatrix*)Cm})
    REQUIRE(!X || (X->nrows == K->nrows && X->ncols == K->ncols), "precon: M and C must match K");
  auto* M = new idrs_user_matrix_s();
  M->format = FMT_CDS;
  M->which_precon = which;
  M->nrows = K->nrows;
  M->ncols = K->ncols;
  if (which == 2 || which == 3) {
    // shift-and-invert: dense (2) or band (3) LU of the shifted matrix
    bool cplx = want_cplx || shift.y != 0.0 || K->vals == 2 || (Mm && Mm->vals == 2) || (Cm && Cm->vals == 2);
    try {
      lu_build(*K, has_shift ? Mm : nullptr, has_shift ? Cm : nullptr, has_shift, shift, which, cplx, *M);
    } catch (const cuda_error&) {
      delete M;
      throw;
    } catch (const std::exception& e) {
      delete M;
      throw arg_error(e.what());
    }
    *P = M;
    return IDRS_OK;
  }
  if (which == 1 && (Mm || Cm)) {
    for (const UserMatrix* X : {(const UserMatrix*)Mm, (const UserMatrix*)Cm})
      REQUIRE(!X || (X->nrows == K->nrows && X->ncols == K->ncols), "precon: M and C must match K");
    bool cplx = false;
    M->diag = diagonal_with_mc(*K, Mm, Cm, want_cplx, shift, &cplx);
    M->diag_cplx = cplx;
  } else if (which == 1) {
    if (K->format == FMT_STENCIL7) {
      M->diag_uniform = true;
      c128 d(K->st[0], 0.0);
      if (d == c128(0.0)) d = c128(1.0);
      M->diag_u = d - shift;
      M->diag_cplx = (M->diag_u.y != 0.0);
    } else {
      bool cplx = false;
      M->diag = make_diagonal(*K, want_cplx || shift.y != 0.0, shift, &cplx);
      M->diag_cplx = cplx;
    }
  }
  *P = M;
  return IDRS_OK;
}

static int diag_out(idrs_user_matrix K, double* D, bool cplx) {
  REQUIRE(K && D, "diagonal: bad arguments");
  int n = K->nrows;
  if (K->format == FMT_STENCIL7) {
    for (int i = 0; i < n; ++i) {
      double d = K->st[0] == 0.0 ? 1.0 : K->st[0];
      if (cplx) { D[2 * i] = d; D[2 * i + 1] = 0.0; } else D[i] = d;
    }
    return IDRS_OK;
  }
  bool is_c = false;
  void* d = make_diagonal(*K, cplx, c128(0.0), &is_c);
  if (!cplx && is_c) { cudaFree(d); throw arg_error("real_diagonal of a complex matrix"); }
  IDRS_CUDA(cudaMemcpy(D, d, (cplx ? 16 : 8) * (size_t)n, cudaMemcpyDeviceToHost));
  cudaFree(d);
  return IDRS_OK;
}

static int user_mv(idrs_user_matrix K, const double* v, double* w, bool cplx) {
  REQUIRE(K && v && w, "user_mv: bad arguments");
  MatView M = K->view64();
  size_t vb = (cplx ? 16 : 8) * (size_t)K->ncols, wb = (cplx ? 16 : 8) * (size_t)K->nrows;
  void *dv = upload(v, vb), *dw = nullptr;
  IDRS_CUDA(cudaMalloc(&dw, std::max<size_t>(wb, 16)));
  if (cplx) spmv<c128>(M, (const c128*)dv, (c128*)dw, c128(1.0), c128(0.0), nullptr, nullptr, nullptr);
  else spmv<double>(M, (const double*)dv, (double*)dw, 1.0, 0.0, nullptr, nullptr, nullptr);
  IDRS_CUDA(cudaMemcpy(w, dw, wb, cudaMemcpyDeviceToHost));
  cudaFree(dv);
  cudaFree(dw);
  return IDRS_OK;
}

static int ms_parameters(idrs_matrix A, int n_sigma, const double* sigma, double* sigma_p, bool cplx) {
  REQUIRE(A && sigma && sigma_p && n_sigma >= 1, "ms_parameters: bad arguments");
  REQUIRE(A->cplx == cplx, "ms_parameters: real/complex mismatch");
  int d = A->degree;
  A->n_sigma = n_sigma;
  A->alpha_s.assign((size_t)(d + 1) * n_sigma, c128(0.0));
  A->sigma_s.assign(n_sigma, c128(0.0));
  const cd seed(A->seed.x, A->seed.y), shift(A->shift.x, A->shift.y);
  auto sig = [&](int i) { return cplx ? cd(sigma[2 * i], sigma[2 * i + 1]) : cd(sigma[i], 0.0); };
  if (A->shift_invert) {
    REQUIRE(shift != seed, "Preconditioner shift should not be equal to seed, choose preconditioner shift and seed differently");
    for (int i = 0; i < n_sigma; ++i)
      REQUIRE(shift != sig(i), "Preconditioner shift should not be equal to one of the shifts, choose different preconditioner shift");
  }
  for (int i = 0; i < n_sigma; ++i) {
    // shift-and-invert: (sigma - seed)/(sigma - shift) (matrix_module.f90:445-455)
    cd ss = A->shift_invert ? (sig(i) - seed) / (sig(i) - shift) : sig(i) - seed;
    A->sigma_s[i] = c128(ss.real(), ss.imag());
    cd sp;
    if (d > 0) {
      std::vector<cd> as(d + 1);
      as[d] = cd(A->alpha_p[d].x, A->alpha_p[d].y);
      for (int k = d - 1; k >= 0; --k) as[k] = cd(A->alpha_p[k].x, A->alpha_p[k].y) + ss * as[k + 1];
      for (int k = 0; k <= d; ++k) A->alpha_s[k + (size_t)(d + 1) * i] = c128(as[k].real(), as[k].imag());
      sp = ss * as[0];
    } else {
      sp = ss;
    }
    if (cplx) { sigma_p[2 * i] = sp.real(); sigma_p[2 * i + 1] = sp.imag(); }
    else sigma_p[i] = sp.real();
  }
  return IDRS_OK;
}

template <class T>
static int matvec_t(idrs_matrix A, const double* v, double* w) {
  REQUIRE(A && v && w, "matvec: bad arguments");
  long n = A->n();
  Staged sv(A, sizeof(T) * n);
  const T* dv = (const T*)sv.in(v);
  T* dw = (T*)sv.out(w);
  DBuf t1(sizeof(T) * n, A->stream), t2(sizeof(T) * n, A->stream);
  DBuf t3(use_recurrence(*A, 64) ? sizeof(T) * n : 0, A->stream);
  op_apply<T>(*A, 64, dv, dw, t1.as<T>(), t2.as<T>(), use_recurrence(*A, 64) ? t3.as<T>() : nullptr, nullptr,
              nullptr, A->stream);
  sv.finish(w, dw);
  IDRS_CUDA(cudaStreamSynchronize(A->stream));
  return IDRS_OK;
}

template <class T>
static int precon_t(idrs_matrix A, const double* v, double* w) {
  REQUIRE(A && v && w, "precon: bad arguments");
  long n = A->n();
  Staged sv(A, sizeof(T) * n);
  const T* dv = (const T*)sv.in(v);
  T* dw = (T*)sv.out(w);
  op_precon<T>(*A, 64, dv, dw, nullptr, A->stream);
  sv.finish(w, dw);
  IDRS_CUDA(cudaStreamSynchronize(A->stream));
  return IDRS_OK;
}

template <class T>
static int scaleback_t(idrs_matrix A, const double* b, const double* y, double* x) {
  REQUIRE(A && y && x, "scaleback: bad arguments");
  REQUIRE(b || !A->defl, "scaleback: a deflated operator needs b");
  long n = A->n();
  Staged sv(A, sizeof(T) * n);
  const T* dy = (const T*)sv.in(y);
  const T* db = (const T*)sv.in(b);
  T* dx = (T*)sv.out(x);
  DBuf t1(sizeof(T) * n, A->stream), t2(sizeof(T) * n, A->stream);
  op_scaleback<T>(*A, 64, A->alpha_p, A->degree, dy, dx, t1.as<T>(), t2.as<T>(), nullptr, A->stream, db);
  sv.finish(x, dx);
  IDRS_CUDA(cudaStreamSynchronize(A->stream));
  return IDRS_OK;
}

template <class T>
static int ms_scaleback_t(idrs_matrix A, int n_sigma, const double* sigma, const double* b,
                          const double* y, double* x) {
  REQUIRE(A && y && x && n_sigma >= 1, "ms_scaleback: bad arguments");
  REQUIRE(A->degree == 0 || A->n_sigma == n_sigma, "ms_scaleback: call ms_parameters with these shifts first");
  REQUIRE(!A->defl || (b && (int)A->sigma_s.size() == n_sigma),
          "ms_scaleback: a deflated operator needs b and ms_parameters with these shifts");
  long n = A->n();
  Staged sv(A, sizeof(T) * n * n_sigma), sb(A, sizeof(T) * n);
  const T* dy = (const T*)sv.in(y);
  const T* db = (const T*)sb.in(b);
  T* dx = (T*)sv.out(x);
  DBuf t1(sizeof(T) * n, A->stream), t2(sizeof(T) * n, A->stream);
  int d = A->degree;
  for (int i = 0; i < n_sigma; ++i) {
    std::vector<c128> al(A->alpha_s.begin() + (size_t)(d + 1) * i, A->alpha_s.begin() + (size_t)(d + 1) * (i + 1));
    if (d == 0) al.assign(1, c128(1.0));
    const c128 ss = A->defl ? A->sigma_s[i] : c128(0.0);
    c128 factor(1.0, 0.0);
    if (A->shift_invert) {  // (seed - shift)/(sigma - shift), matrix_module.f90:755-761
      REQUIRE(sigma, "ms_scaleback: shift-and-invert needs the shifts");
      const cd sg = traits<T>::is_cplx ? cd(sigma[2 * i], sigma[2 * i + 1]) : cd(sigma[i], 0.0);
      const cd f = (cd(A->seed.x, A->seed.y) - cd(A->shift.x, A->shift.y)) / (sg - cd(A->shift.x, A->shift.y));
      factor = c128(f.real(), f.imag());
    }
    op_scaleback<T>(*A, 64, al, d, dy + n * i, dx + n * i, t1.as<T>(), t2.as<T>(), nullptr, A->stream,
                    db, ss, factor);
  }
  sv.finish(x, dx);
  IDRS_CUDA(cudaStreamSynchronize(A->stream));
  return IDRS_OK;
}

template <class T>
static int norm_t(idrs_matrix A, const double* u, const double* v, double* out, bool dot) {
  using W = typename traits<T>::wide;
  REQUIRE(A && u && out && (!dot || v), "norm/inprod: bad arguments");
  long n = A->n();
  Staged sv(A, sizeof(T) * n);
  const T* du = (const T*)sv.in(u);
  const T* dv = dot ? (const T*)sv.in(v) : nullptr;
  DBuf res(sizeof(W), A->stream);
  if (dot) launch_fused<1, T>(n, BDotc<T>{du, dv}, TStoreVals<W>{res.as<W>(), 1}, A->red, nullptr, A->stream);
  else launch_fused<1, T>(n, BNorm<T>{du}, TStoreVals<W>{res.as<W>(), 1}, A->red, nullptr, A->stream);
  W h;
  IDRS_CUDA(cudaMemcpyAsync(&h, res.p, sizeof(W), cudaMemcpyDeviceToHost, A->stream));
  IDRS_CUDA(cudaStreamSynchronize(A->stream));
  if (dot) {
    out[0] = real_(h);
    if (traits<T>::is_cplx) out[1] = imag_(h);
  } else {
    out[0] = std::sqrt(real_(h));
  }
  return IDRS_OK;
}
}  // namespace

// ===========================================================================
extern "C" {

int idrs_real_diagonal(idrs_user_matrix K, double* D) { return guard([&] { return diag_out(K, D, false); }); }

int idrs_complex_diagonal(idrs_user_matrix K, double* D) { return guard([&] { return diag_out(K, D, true); }); }

int idrs_ruser_mv(idrs_user_matrix K, const double* v, double* w) { return guard([&] { return user_mv(K, v, w, false); }); }

int idrs_cuser_mv(idrs_user_matrix K, const double* v, double* w) { return guard([&] { return user_mv(K, v, w, true); }); }

int idrs_real_ms_parameters(idrs_matrix A, int n_sigma, const double* sigma, double* sigma_p) {
  return guard([&] { return ms_parameters(A, n_sigma, sigma, sigma_p, false); });
}

int idrs_complex_ms_parameters(idrs_matrix A, int n_sigma, const double* sigma, double* sigma_p) {
  return guard([&] { return ms_parameters(A, n_sigma, sigma, sigma_p, true); });
}

int idrs_rmatvec(idrs_matrix A, const double* v, double* w) {
  return guard([&] { REQUIRE(A && !A->cplx, "rmatvec: real handle required"); return matvec_t<double>(A, v, w); });
}

int idrs_rmatvec32(idrs_matrix A, const double* v, double* w) {
  return guard([&] {
    REQUIRE(A && !A->cplx && v && w, "rmatvec32: real handle, v and w required");
    const long n = A->n();
    cudaStream_t st = A->stream;
    Staged sv(A, sizeof(double) * n);
    const double* dv = (const double*)sv.in(v);
    double* dw = (double*)sv.out(w);
    DBuf v32(4 * n, st), w32(4 * n, st), t1(4 * n, st), t2(4 * n, st), t3(4 * n, st), t4(4 * n, st);
    vec_convert<double, float>(n, dv, v32.as<float>(), nullptr, st);
    const MatView& M = A->view(32);
    if (A->jac.valid())
      op_chain_recur<float>(M, A->jac, A->degree, v32.as<float>(), w32.as<float>(), t1.as<float>(),
                            t2.as<float>(), t3.as<float>(), t4.as<float>(), nullptr, st, 1.0f, 0.0f, nullptr);
    else
      op_chain<float>(M, A->alpha_p, A->degree, v32.as<float>(), w32.as<float>(), t1.as<float>(),
                      t2.as<float>(), nullptr, st, 1.0f, 0.0f, nullptr);
    vec_convert<float, double>(n, w32.as<float>(), dw, nullptr, st);
    sv.finish(w, dw);
    IDRS_CUDA(cudaStreamSynchronize(st));
    return IDRS_OK;
  });
}

int idrs_cmatvec(idrs_matrix A, const double* v, double* w) {
  return guard([&] { REQUIRE(A && A->cplx, "cmatvec: complex handle required"); return matvec_t<c128>(A, v, w); });
}

int idrs_rprecon(idrs_matrix A, const double* v, double* w) {
  return guard([&] { REQUIRE(A && !A->cplx, "rprecon: real handle required"); return precon_t<double>(A, v, w); });
}

int idrs_cprecon(idrs_matrix A, const double* v, double* w) {
  return guard([&] { REQUIRE(A && A->cplx, "cprecon: complex handle required"); return precon_t<c128>(A, v, w); });
}

int idrs_rscaleback(idrs_matrix A, const double* b, const double* y, double* x) {
  return guard([&] { REQUIRE(A && !A->cplx, "rscaleback: real handle required"); return scaleback_t<double>(A, b, y, x); });
}

int idrs_cscaleback(idrs_matrix A, const double* b, const double* y, double* x) {
  return guard([&] { REQUIRE(A && A->cplx, "cscaleback: complex handle required"); return scaleback_t<c128>(A, b, y, x); });
}

int idrs_ms_rscaleback(idrs_matrix A, int n_sigma, const double* sigma, const double* b,
                       const double* y, double* x) {
  return guard([&] { REQUIRE(A && !A->cplx, "ms_rscaleback: real handle required"); return ms_scaleback_t<double>(A, n_sigma, sigma, b, y, x); });
}

int idrs_ms_cscaleback(idrs_matrix A, int n_sigma, const double* sigma, const double* b,
                       const double* y, double* x) {
  return guard([&] { REQUIRE(A && A->cplx, "ms_cscaleback: complex handle required"); return ms_scaleback_t<c128>(A, n_sigma, sigma, b, y, x); });
}

int idrs_rnorm(idrs_matrix A, const double* w, double* norm) { return guard([&] { return norm_t<double>(A, w, nullptr, norm, false); }); }

int idrs_cnorm(idrs_matrix A, const double* w, double* norm) { return guard([&] { return norm_t<c128>(A, w, nullptr, norm, false); }); }

int idrs_rinprod(idrs_matrix A, const double* u, const double* v, double* uv) { return guard([&] { return norm_t<double>(A, u, v, uv, true); }); }

int idrs_cinprod(idrs_matrix A, const double* u, const double* v, double* uv) { return guard([&] { return norm_t<c128>(A, u, v, uv, true); }); }

const char* idrs_last_error(void) { return idrs::last_error(); }
long idrs_launch_count(void) { return idrs::launch_count(); }
long idrs_pp_struct_size(int which) {
  switch (which) {
    case 0: return (long)sizeof(idrs_pp_options);
    case 1: return (long)sizeof(idrs_pp_report);
    case 2: return (long)sizeof(idrs_pp_inputs);
    default: return 0;
  }
}
int idrs_version(void) { return 10000; }

int idrs_crs_format(int nrows, int ncols, const int* row_ptr, const int* col_ind,
                    const double* rval, const double* cval, idrs_user_matrix* K) {
  return guard([&] {
    REQUIRE(K && row_ptr && nrows >= 0 && ncols >= 0, "crs_format: bad arguments");
    init_runtime();
    long base = row_ptr[0];
    long nnz = (long)row_ptr[nrows] - base;
    REQUIRE(nnz >= 0 && (nnz == 0 || col_ind), "crs_format: bad row pointers");
    std::vector<int> rp(nrows + 1), ci(std::max<long>(nnz, 1));
    for (int i = 0; i <= nrows; ++i) {
      rp[i] = (int)(row_ptr[i] - base);
      if (i > 0) REQUIRE(rp[i] >= rp[i - 1], "crs_format: row pointers must not decrease");
    }
    for (long k = 0; k < nnz; ++k) {
      int c = col_ind[k] - 1;
      REQUIRE(c >= 0 && c < ncols, "crs_format: column index out of range");
      ci[k] = c;
    }
    auto* M = new idrs_user_matrix_s();
    M->format = FMT_CRS;
    M->nrows = nrows;
    M->ncols = ncols;
    M->nnz = nnz;
    M->row_ptr = (int*)upload(rp.data(), sizeof(int) * (nrows + 1));
    M->col_ind = (int*)upload(ci.data(), sizeof(int) * nnz);
    if (cval) {
      M->vals = 2;
      M->val = upload(cval, 16 * (size_t)nnz);
    } else {
      M->vals = 1;
      if (rval) M->val = upload(rval, 8 * (size_t)nnz);
      else {
        std::vector<double> ones(std::max<long>(nnz, 1), 1.0);
        M->val = upload(ones.data(), 8 * (size_t)nnz);
      }
    }
    M->group = crs_group(nnz, nrows);
    build_row_plan(*M, rp.data());
    *K = M;
    return IDRS_OK;
  });
}

int idrs_coo_format(int nrows, int ncols, int nnz, const int* indx, const int* jndx,
                    const double* rval, const double* cval, idrs_user_matrix* K) {
  return guard([&] {
    REQUIRE(K && nrows >= 0 && ncols >= 0 && nnz >= 0 && (nnz == 0 || (indx && jndx)),
            "coo_format: bad arguments");
    init_runtime();
    // stable counting sort by row: rows keep the caller's order of entries
    std::vector<int> cnt(nrows + 1, 0);
    for (int k = 0; k < nnz; ++k) {
      REQUIRE(indx[k] >= 1 && indx[k] <= nrows && jndx[k] >= 1 && jndx[k] <= ncols,
              "coo_format: index out of range");
      cnt[indx[k]]++;
    }
    for (int i = 0; i < nrows; ++i) cnt[i + 1] += cnt[i];
    std::vector<int> pos(cnt.begin(), cnt.end() - 1), ci(std::max(nnz, 1));
    size_t vs = cval ? 2 : 1;
    std::vector<double> val(std::max<size_t>((size_t)nnz * vs, 1), 1.0);
    for (int k = 0; k < nnz; ++k) {
      int p = pos[indx[k] - 1]++;
      ci[p] = jndx[k] - 1;
      if (cval) { val[2 * p] = cval[2 * k]; val[2 * p + 1] = cval[2 * k + 1]; }
      else if (rval) val[p] = rval[k];
    }
    auto* M = new idrs_user_matrix_s();
    M->format = FMT_COO;
    M->nrows = nrows;
    M->ncols = ncols;
    M->nnz = nnz;
    M->row_ptr = (int*)upload(cnt.data(), sizeof(int) * (nrows + 1));
    M->col_ind = (int*)upload(ci.data(), sizeof(int) * nnz);
    M->vals = cval ? 2 : 1;
    M->val = upload(val.data(), 8 * vs * (size_t)nnz);
    M->group = crs_group(nnz, nrows);
    build_coo_rows(*M, cnt.data());
    *K = M;
    return IDRS_OK;
  });
}

int idrs_cds_format(int nrows, int ncols, int half_band, const double* rband, const double* cband,
                    idrs_user_matrix* K) {
  return guard([&] {
    REQUIRE(K && nrows >= 0 && half_band >= 0 && half_band < std::max(nrows, 1),
            "cds_format: bad arguments");
    init_runtime();
    size_t cnt = (size_t)nrows * (2 * half_band + 1);
    auto* M = new idrs_user_matrix_s();
    M->format = FMT_CDS;
    M->nrows = nrows;
    M->ncols = ncols;
    M->half_band = half_band;
    if (cband) { M->vals = 2; M->band = upload(cband, 16 * cnt); }
    else {
      M->vals = 1;
      if (rband) M->band = upload(rband, 8 * cnt);
      else { std::vector<double> ones(std::max<size_t>(cnt, 1), 1.0); M->band = upload(ones.data(), 8 * cnt); }
    }
    *K = M;
    return IDRS_OK;
  });
}

int idrs_dense_format(int nrows, int ncols, const double* rmat, const double* cmat,
                      idrs_user_matrix* K) {
  return guard([&] {
    REQUIRE(K && nrows >= 0 && ncols >= 0 && (rmat || cmat), "dense_format: bad arguments");
    init_runtime();
    size_t cnt = (size_t)nrows * ncols;
    auto* M = new idrs_user_matrix_s();
    M->format = FMT_DENSE;
    M->nrows = nrows;
    M->ncols = ncols;
    if (cmat) { M->vals = 2; M->mat = upload(cmat, 16 * cnt); }
    else { M->vals = 1; M->mat = upload(rmat, 8 * cnt); }
    *K = M;
    return IDRS_OK;
  });
}

int idrs_stencil7_format(int nx, int ny, int nz, const double* coef, idrs_user_matrix* K) {
  return guard([&] {
    REQUIRE(K && coef && nx >= 1 && ny >= 1 && nz >= 1, "stencil7_format: bad arguments");
    REQUIRE((long)nx * ny * nz < (1L << 31), "stencil7_format: grid too large");
    init_runtime();
    auto* M = new idrs_user_matrix_s();
    M->format = FMT_STENCIL7;
    M->nrows = M->ncols = nx * ny * nz;
    M->nx = nx; M->ny = ny; M->nz = nz;
    for (int i = 0; i < 7; ++i) M->st[i] = coef[i];
    *K = M;
    return IDRS_OK;
  });
}

int idrs_real_precon(int which_precon, idrs_user_matrix K, const double* shift, idrs_user_matrix* P) {
  return guard([&] {
    return precon_common(which_precon, K, c128(shift ? *shift : 0.0, 0.0), false, P, nullptr, nullptr,
                         shift != nullptr);
  });
}
int idrs_complex_precon(int which_precon, idrs_user_matrix K, const double* shift, idrs_user_matrix* P) {
  return guard([&] {
    c128 sh = shift ? c128(shift[0], shift[1]) : c128(0.0);
    return precon_common(which_precon, K, sh, true, P, nullptr, nullptr, shift != nullptr);
  });
}
int idrs_real_precon_ext(int which_precon, idrs_user_matrix K, idrs_user_matrix M,
                         idrs_user_matrix C, const double* shift, idrs_user_matrix* P) {
  return guard([&] {
    // without a shift the reference takes K alone
    if (!shift) return precon_common(which_precon, K, c128(0.0), false, P);
    return precon_common(which_precon, K, c128(*shift, 0.0), false, P, M, C, true);
  });
}
int idrs_complex_precon_ext(int which_precon, idrs_user_matrix K, idrs_user_matrix M,
                            idrs_user_matrix C, const double* shift, idrs_user_matrix* P) {
  return guard([&] {
    if (!shift) return precon_common(which_precon, K, c128(0.0), true, P);
    return precon_common(which_precon, K, c128(shift[0], shift[1]), true, P, M, C, true);
  });
}

int idrs_user_matrix_free(idrs_user_matrix K) {
  return guard([&] {
    if (K) user_matrix_release(K);
    return IDRS_OK;
  });
}

int idrs_matrix_create(idrs_user_matrix K, idrs_user_matrix P, int is_complex, const double* seed,
                       idrs_matrix* A) {
  return guard([&] {
    REQUIRE(K && A, "matrix_create: bad arguments");
    REQUIRE(K->nrows == K->ncols, "matrix_create: K must be square");
    REQUIRE(!P || P->nrows == K->nrows, "matrix_create: P size mismatch");
    init_runtime();
    auto* M = new idrs_matrix_s();
    M->K = K;
    K->refcount++;
    if (P) { M->P = P; P->refcount++; }
    M->cplx = is_complex != 0;
    if (seed) M->seed = M->cplx ? c128(seed[0], seed[1]) : c128(seed[0], 0.0);
    REQUIRE(M->cplx || K->vals != 2, "matrix_create: complex matrix in a real problem");
    IDRS_CUDA(cudaStreamCreateWithFlags(&M->stream, cudaStreamNonBlocking));
    M->own_stream = true;
    M->alpha_p.assign(1, c128(1.0));
    M->red = alloc_redbuf(M->stream);
    int st = build_operator(M);
    if (st != 0) {
      std::string msg = idrs::last_error();
      operator_free(M);
      delete M;
      set_error(msg);
      return st == 5 ? IDRS_ERR_UNSUPPORTED : IDRS_ERR_ARG;
    }
    IDRS_CUDA(cudaStreamSynchronize(M->stream));
    *A = M;
    return IDRS_OK;
  });
}

}  // extern "C"

// ------------------------------------------------- mass / damping systems
namespace {

// One CRS term of an assembled system row: coef * M(row, :) at column offset.
struct SysTerm {
  const int* rp = nullptr; const int* ci = nullptr; const void* val = nullptr;
  bool vcplx = false; c128 coef; int col_off = 0;
};

// Output row r of the assembled matrix.  Rows r < nn concatenate the terms'
// rows r (and an optional diagonal entry diag_top at (r, r)); rows nn + i of
// the block system hold 1 at (nn+i, i) and, with a seed, -seed at (nn+i, nn+i).
template <class V>
__global__ void k_sys_fill(int nn, int nrows, const int* __restrict__ rp_out, int* ci_out,
                           V* val_out, SysTerm t0, SysTerm t1, SysTerm t2, int nterms,
                           bool has_diag_top, c128 diag_top, bool block, c128 low_diag) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += gridDim.x * blockDim.x) {
    int o = rp_out[r];
    if (r < nn) {
      const SysTerm ts[3] = {t0, t1, t2};
      for (int q = 0; q < nterms; ++q) {
        const SysTerm& t = ts[q];
        for (int k = t.rp[r]; k < t.rp[r + 1]; ++k, ++o) {
          ci_out[o] = t.ci[k] + t.col_off;
          c128 v = t.vcplx ? ((const c128*)t.val)[k] : c128(((const double*)t.val)[k], 0.0);
          val_out[o] = narrow<V>(t.coef * v);
        }
      }
      if (has_diag_top) { ci_out[o] = r; val_out[o] = narrow<V>(diag_top); }
    } else if (block) {
      const int i = r - nn;
      ci_out[o] = i;
      val_out[o] = narrow<V>(c128(1.0, 0.0));
      if (low_diag.x != 0.0 || low_diag.y != 0.0) { ci_out[o + 1] = r; val_out[o + 1] = narrow<V>(low_diag); }
    }
  }
}

// D = [P; 1] for the block system (rprecon scales the first half only)
__global__ void k_block_diag(long nn, const void* pd, bool pcplx, bool uniform, c128 pu, bool ocplx,
                             void* out) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < 2 * nn; i += gridDim.x * (long)blockDim.x) {
    c128 v(1.0, 0.0);
    if (i < nn) v = uniform ? pu : (pcplx ? ((const c128*)pd)[i] : c128(((const double*)pd)[i], 0.0));
    if (ocplx) ((c128*)out)[i] = v;
    else ((double*)out)[i] = v.x;
  }
}

std::vector<int> host_row_ptr(const UserMatrix& M) {
  std::vector<int> rp(M.nrows + 1);
  IDRS_CUDA(cudaMemcpy(rp.data(), M.row_ptr, sizeof(int) * (M.nrows + 1), cudaMemcpyDeviceToHost));
  return rp;
}

// The system matrix of real_mv / complex_mv (matrix_module.f90:170-264)
// assembled once as one CRS matrix, so that each product is a single SpMV:
//   standard: K + seed C + seed^2 M | K + seed C + seed^2 I | K - seed M
//   block (multishift with C), 2nn x 2nn:
//     [ -C - seed M   -K      ]   (without M: -seed I in the (1,1) block)
//     [  I            -seed I ]
// K, M, C: CRS or COO (COO is stored row-sorted with row pointers, so both
// are read the same way); the result is CRS.
idrs_user_matrix assemble_system(const UserMatrix& K, const UserMatrix* Mm, const UserMatrix* Cm,
                                 c128 seed, bool block) {
  const int nn = K.nrows;
  const bool seeded = seed.x != 0.0 || seed.y != 0.0;
  std::vector<const UserMatrix*> srcs;  // the matrix of each term
  auto term = [&](const UserMatrix& M, c128 coef, int off) {
    SysTerm t;
    t.rp = M.row_ptr; t.ci = M.col_ind; t.val = M.val; t.vcplx = M.vals == 2; t.coef = coef; t.col_off = off;
    srcs.push_back(&M);
    return t;
  };
  std::vector<SysTerm> terms;
  bool has_diag_top = false;
  c128 diag_top(0.0, 0.0), low_diag(0.0, 0.0);
  const c128 one(1.0, 0.0), mone(-1.0, 0.0);
  if (block) {
    terms.push_back(term(*Cm, mone, 0));
    terms.push_back(term(K, mone, nn));
    if (seeded) {
      if (Mm) terms.push_back(term(*Mm, c128(-seed.x, -seed.y), 0));
      else { has_diag_top = true; diag_top = c128(-seed.x, -seed.y); }
      low_diag = c128(-seed.x, -seed.y);
    }
  } else {
    terms.push_back(term(K, one, 0));
    if (Cm) {
      terms.push_back(term(*Cm, seed, 0));
      if (Mm) terms.push_back(term(*Mm, seed * seed, 0));
      else { has_diag_top = true; diag_top = seed * seed; }
    } else if (Mm) {
      terms.push_back(term(*Mm, c128(-seed.x, -seed.y), 0));
    }
  }
  std::vector<std::vector<int>> rps;
  for (const UserMatrix* src : srcs) rps.push_back(host_row_ptr(*src));
  const int nrows = block ? 2 * nn : nn;
  std::vector<int> rp(nrows + 1, 0);
  for (int r = 0; r < nrows; ++r) {
    long len = 0;
    if (r < nn) {
      for (auto& h : rps) len += h[r + 1] - h[r];
      if (has_diag_top) len += 1;
    } else {
      len = 1 + ((low_diag.x != 0.0 || low_diag.y != 0.0) ? 1 : 0);
    }
    REQUIRE((long)rp[r] + len <= INT32_MAX, "system matrix: more than 2^31 nonzeros");
    rp[r + 1] = rp[r] + (int)len;
  }
  const long nnz = rp[nrows];
  bool cplx = seed.y != 0.0 || K.vals == 2 || (Mm && Mm->vals == 2) || (Cm && Cm->vals == 2);
  auto* S = new idrs_user_matrix_s();
  S->format = FMT_CRS;
  S->nrows = S->ncols = nrows;
  S->nnz = nnz;
  S->vals = cplx ? 2 : 1;
  S->row_ptr = (int*)upload(rp.data(), sizeof(int) * (nrows + 1));
  IDRS_CUDA(cudaMalloc((void**)&S->col_ind, sizeof(int) * std::max<long>(nnz, 1)));
  IDRS_CUDA(cudaMalloc(&S->val, (cplx ? 16 : 8) * std::max<long>(nnz, 1)));
  SysTerm t[3];
  for (size_t q = 0; q < terms.size(); ++q) t[q] = terms[q];
  const int grid = std::max(1, std::min((nrows + 255) / 256, num_sms() * 8));
  if (cplx)
    k_sys_fill<c128><<<grid, 256>>>(nn, nrows, S->row_ptr, S->col_ind, (c128*)S->val, t[0], t[1], t[2],
                                    (int)terms.size(), has_diag_top, diag_top, block, low_diag);
  else
    k_sys_fill<double><<<grid, 256>>>(nn, nrows, S->row_ptr, S->col_ind, (double*)S->val, t[0], t[1], t[2],
                                      (int)terms.size(), has_diag_top, diag_top, block, low_diag);
  IDRS_LAUNCH_CHECK();
  IDRS_CUDA(cudaDeviceSynchronize());
  S->group = crs_group(nnz, nrows);
  build_row_plan(*S, rp.data());
  return S;
}

idrs_user_matrix block_diagonal(const UserMatrix& P, long nn) {
  auto* D = new idrs_user_matrix_s();
  D->format = P.format;
  D->which_precon = 1;
  D->nrows = D->ncols = (int)(2 * nn);
  const bool ocplx = P.diag_cplx || (P.diag_uniform && P.diag_u.y != 0.0);
  D->diag_cplx = ocplx;
  IDRS_CUDA(cudaMalloc(&D->diag, (ocplx ? 16 : 8) * (size_t)(2 * nn)));
  k_block_diag<<<stream_grid(2 * nn), kThreads>>>(nn, P.diag, P.diag_cplx, P.diag_uniform, P.diag_u, ocplx, D->diag);
  IDRS_LAUNCH_CHECK();
  IDRS_CUDA(cudaDeviceSynchronize());
  return D;
}

}  // namespace

inline bool block_of(int multishift, const UserMatrix* Cm) { return multishift && Cm; }

extern "C" {

int idrs_matrix_create_ext(idrs_user_matrix K, idrs_user_matrix Mm, idrs_user_matrix Cm,
                           idrs_user_matrix P, int is_complex, const double* seed,
                           const double* shift, int multishift, idrs_matrix* A) {
  return guard([&] {
    REQUIRE(K && A, "matrix_create: bad arguments");
    const bool si = P && shift;
    auto finish = [&](int st) {
      if (st) return st;
      (*A)->multishift = multishift != 0;
      if (si) {
        (*A)->shift_invert = true;
        (*A)->shift = is_complex ? c128(shift[0], shift[1]) : c128(shift[0], 0.0);
      }
      return IDRS_OK;
    };
    if (!Mm && !Cm) return finish(idrs_matrix_create(K, P, is_complex, seed, A));
    REQUIRE(K->nrows == K->ncols, "matrix_create: K must be square");
    for (const UserMatrix* X : {(const UserMatrix*)Mm, (const UserMatrix*)Cm}) {
      if (!X) continue;
      REQUIRE(X->nrows == K->nrows && X->ncols == K->ncols, "matrix_create: M and C must match K");
      if (X->format != FMT_CRS && X->format != FMT_COO)
        throw unsupported_error("matrix_create: mass and damping matrices must be CRS or COO");
    }
    if (K->format != FMT_CRS && K->format != FMT_COO)
      throw unsupported_error("matrix_create: with mass or damping matrices K must be CRS or COO");
    REQUIRE(!P || P->nrows == K->nrows, "matrix_create: P size mismatch");
    const bool block_si = block_of(multishift, Cm) && P && (P->which_precon == 2 || P->which_precon == 3);
    REQUIRE(!P || P->which_precon <= 1 || !block_of(multishift, Cm) || shift,
            "matrix_create: an LU preconditioner of the block system needs the shift");
    init_runtime();
    const bool cplx = is_complex != 0;
    c128 sd(0.0, 0.0);
    if (seed) sd = cplx ? c128(seed[0], seed[1]) : c128(seed[0], 0.0);
    const bool block = multishift && Cm;
    const bool seeded = sd.x != 0.0 || sd.y != 0.0;
    idrs_user_matrix S = nullptr, D = nullptr;
    if (block || seeded) S = assemble_system(*K, Mm, Cm, sd, block);
    if (block && P && !block_si) D = block_diagonal(*P, K->nrows);
    // an assembled matrix already holds the seed: build without it, then
    // record it for the parameters derived from it (foci, centre, shifts)
    int st = idrs_matrix_create(S ? S : K, block_si ? nullptr : (D ? D : P), is_complex,
                                S ? nullptr : seed, A);
    // the operator holds its own references
    if (S) user_matrix_release(S);
    if (D) user_matrix_release(D);
    if (st) return st;
    if (block_si) {
      // rprecon's block form (matrix_module.f90:318-345): P (n x n), C, M and
      // the shift; the products apply it before the assembled block matrix
      REQUIRE(P->nrows == K->nrows, "matrix_create: P must have the size of K");
      Operator* op = *A;
      op->P = P; P->refcount++;
      op->si_C = Cm; Cm->refcount++;
      if (Mm) { op->si_M = Mm; Mm->refcount++; }
      const size_t es = op->cplx ? 16 : 8;
      IDRS_CUDA(cudaMallocAsync(&op->lu_tmp, es * 2 * K->nrows, op->stream));
      IDRS_CUDA(cudaMallocAsync(&op->si_tmp, es * 2 * K->nrows, op->stream));
      IDRS_CUDA(cudaStreamSynchronize(op->stream));
    }
    if (S) {
      (*A)->seed = sd;
      (*A)->seed_folded = true;
    }
    return finish(IDRS_OK);
  });
}

int idrs_make_deflation(idrs_matrix A, const double* V, int k) {
  return guard([&] {
    REQUIRE(A && k >= 0 && (k == 0 || V), "make_deflation: bad arguments");
    REQUIRE(k <= MAXS, "make_deflation: at most 16 deflation vectors");
    const long n = A->n();
    Staged sv(A, (A->cplx ? 16 : 8) * (size_t)n * std::max(k, 1));
    const void* dV = k ? sv.in(V) : nullptr;
    deflation_make(*A, dV, k);
    return IDRS_OK;
  });
}

}  // extern "C"

template <class T>
static int pmul_t(idrs_matrix A, const double* v, double* w) {
  REQUIRE(A && v && w, "pmul: bad arguments");
  const long n = A->n();
  Staged sv(A, sizeof(T) * n);
  const T* dv = (const T*)sv.in(v);
  T* dw = (T*)sv.out(w);
  if (A->defl && A->defl->k > 0)
    deflation_pmul<T>(*A->defl, dv, dw, T(1.0), T(0.0), nullptr, nullptr, A->stream);
  else
    vec_copy<T>(n, dv, dw, nullptr, A->stream);
  sv.finish(w, dw);
  IDRS_CUDA(cudaStreamSynchronize(A->stream));
  return IDRS_OK;
}

extern "C" {

int idrs_rpmul(idrs_matrix A, const double* v, double* w) {
  return guard([&] { REQUIRE(A && !A->cplx, "rpmul: real handle required"); return pmul_t<double>(A, v, w); });
}
int idrs_cpmul(idrs_matrix A, const double* v, double* w) {
  return guard([&] { REQUIRE(A && A->cplx, "cpmul: complex handle required"); return pmul_t<c128>(A, v, w); });
}

int idrs_matrix_free(idrs_matrix A) {
  return guard([&] {
    if (A) {
      operator_free(A);
      delete A;
    }
    return IDRS_OK;
  });
}

int idrs_matrix_set_stream(idrs_matrix A, void* cuda_stream) {
  return guard([&] {
    REQUIRE(A, "set_stream: bad handle");
    IDRS_CUDA(cudaStreamSynchronize(A->stream));
    if (A->own_stream) cudaStreamDestroy(A->stream);
    A->stream = (cudaStream_t)cuda_stream;
    A->own_stream = false;
    return IDRS_OK;
  });
}

int idrs_matrix_set_pointer_mode(idrs_matrix A, int mode) {
  return guard([&] {
    REQUIRE(A && (mode == IDRS_POINTER_HOST || mode == IDRS_POINTER_DEVICE), "set_pointer_mode: bad arguments");
    A->device_pointers = (mode == IDRS_POINTER_DEVICE);
    return IDRS_OK;
  });
}

int idrs_matrix_set_poly_eval(idrs_matrix A, int mode) {
  return guard([&] {
    REQUIRE(A && (mode == IDRS_POLY_HORNER || mode == IDRS_POLY_RECURRENCE), "set_poly_eval: bad arguments");
    A->poly_eval = mode;
    return IDRS_OK;
  });
}

int idrs_matrix_set_shadow(idrs_matrix A, int s, const double* PT) {
  return guard([&] {
    REQUIRE(A && s >= 1, "set_shadow: bad arguments");
    for (auto it = A->shadows.begin(); it != A->shadows.end(); ++it)
      if (it->first == s) { cudaFree(it->second); A->shadows.erase(it); break; }
    if (PT) {
      size_t bytes = (A->cplx ? 16 : 8) * (size_t)s * A->n();
      A->shadows.emplace_back(s, upload(PT, bytes));
    }
    return IDRS_OK;
  });
}

int idrs_real_preconditioner(idrs_matrix A, int preconditioner, int degree, const double* foci,
                             const double* center, const double* H, int ldh, int nh) {
  return guard([&] {
    REQUIRE(A && !A->cplx, "real_preconditioner: real matrix handle required");
    return set_preconditioner(A, preconditioner, degree, foci, center, H, ldh, nh);
  });
}
int idrs_complex_preconditioner(idrs_matrix A, int preconditioner, int degree, const double* foci,
                                const double* center, const double* H, int ldh, int nh) {
  return guard([&] {
    REQUIRE(A && A->cplx, "complex_preconditioner: complex matrix handle required");
    return set_preconditioner(A, preconditioner, degree, foci, center, H, ldh, nh);
  });
}

int idrs_matrix_get_alpha(idrs_matrix A, double* alpha, int* degree) {
  return guard([&] {
    REQUIRE(A, "get_alpha: bad handle");
    if (degree) *degree = A->degree;
    if (alpha)
      for (int i = 0; i <= A->degree; ++i) {
        if (A->cplx) { alpha[2 * i] = A->alpha_p[i].x; alpha[2 * i + 1] = A->alpha_p[i].y; }
        else alpha[i] = A->alpha_p[i].x;
      }
    return IDRS_OK;
  });
}

int idrs_time_matvec(idrs_matrix A, int prec, int warmup, int reps, double* ms_per_product,
                     double* ms_per_launch) {
  return guard([&] {
    REQUIRE(A && (prec == 64 || prec == 32) && reps >= 1 && warmup >= 0, "time_matvec: bad arguments");
    long n = A->n();
    cudaStream_t st = A->stream;
    size_t es = (A->cplx ? 2 : 1) * (prec == 64 ? 8 : 4);
    DBuf v(es * n, st), w(es * n, st), t1(es * n, st), t2(es * n, st), t3(es * n, st), t4(es * n, st);
    IDRS_CUDA(cudaMemsetAsync(v.p, 0, es * n, st));
    auto once = [&] {
      auto run = [&](auto z) {
        using T = decltype(z);
        op_apply<T>(*A, prec, v.as<T>(), w.as<T>(), t1.as<T>(), t2.as<T>(), t3.as<T>(), t4.as<T>(), nullptr, st);
      };
      if (prec == 64 && !A->cplx) run(0.0);
      else if (prec == 32 && !A->cplx) run(0.0f);
      else if (prec == 64) run(c128(0.0));
      else run(c64(0.0f));
    };
    for (int i = 0; i < warmup; ++i) once();
    cudaEvent_t e0, e1;
    IDRS_CUDA(cudaEventCreate(&e0));
    IDRS_CUDA(cudaEventCreate(&e1));
    IDRS_CUDA(cudaEventRecord(e0, st));
    for (int i = 0; i < reps; ++i) once();
    IDRS_CUDA(cudaEventRecord(e1, st));
    IDRS_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    IDRS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (ms_per_product) *ms_per_product = ms / reps;
    if (ms_per_launch) *ms_per_launch = ms / reps / (A->degree + 1);
    return IDRS_OK;
  });
}

int idrs_time_matvec_graph(idrs_matrix A, int prec, int warmup, int reps, double* ms_per_product) {
  return guard([&] {
    // warmup >= 1: the direct products before the capture make every lazily
    // allocated work array of the operator exist outside the graph
    REQUIRE(A && (prec == 64 || prec == 32) && reps >= 1 && warmup >= 1 && ms_per_product,
            "time_matvec_graph: bad arguments");
    long n = A->n();
    cudaStream_t st = A->stream;
    size_t es = (A->cplx ? 2 : 1) * (prec == 64 ? 8 : 4);
    DBuf v(es * n, st), w(es * n, st), t1(es * n, st), t2(es * n, st), t3(es * n, st), t4(es * n, st);
    IDRS_CUDA(cudaMemsetAsync(v.p, 0, es * n, st));
    auto once = [&] {
      auto run = [&](auto z) {
        using T = decltype(z);
        op_apply<T>(*A, prec, v.as<T>(), w.as<T>(), t1.as<T>(), t2.as<T>(), t3.as<T>(), t4.as<T>(), nullptr, st);
      };
      if (prec == 64 && !A->cplx) run(0.0);
      else if (prec == 32 && !A->cplx) run(0.0f);
      else if (prec == 64) run(c128(0.0));
      else run(c64(0.0f));
    };
    for (int i = 0; i < warmup; ++i) once();
    IDRS_CUDA(cudaStreamSynchronize(st));
    // one product captured as a graph (as the IDR(s) cycles run it), then replayed
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    IDRS_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    const long l0 = launch_count();
    bool ok = true;
    try {
      once();
    } catch (const cuda_error&) {
      ok = false;
    }
    const cudaError_t ce = cudaStreamEndCapture(st, &g);
    const long captured = launch_count() - l0;
    uncount_launches(captured);  // captured, not run: the replays count them
    if (!ok || ce != cudaSuccess || !g || cudaGraphInstantiate(&ge, g, 0) != cudaSuccess) {
      cudaGetLastError();
      if (g) cudaGraphDestroy(g);
      REQUIRE(false, "time_matvec_graph: the product cannot be captured as a CUDA graph");
    }
    cudaGraphDestroy(g);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float ms = 0;
    cudaError_t re = cudaGraphLaunch(ge, st);
    if (re == cudaSuccess) re = cudaEventCreate(&e0);
    if (re == cudaSuccess) re = cudaEventCreate(&e1);
    if (re == cudaSuccess) re = cudaEventRecord(e0, st);
    for (int i = 0; i < reps && re == cudaSuccess; ++i) re = cudaGraphLaunch(ge, st);
    if (re == cudaSuccess) re = cudaEventRecord(e1, st);
    if (re == cudaSuccess) re = cudaEventSynchronize(e1);
    if (re == cudaSuccess) re = cudaEventElapsedTime(&ms, e0, e1);
    for (long q = 0; q < captured * (reps + 1); ++q) count_launch();
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaGraphExecDestroy(ge);
    IDRS_CUDA(re);
    *ms_per_product = ms / reps;
    return IDRS_OK;
  });
}

int idrs_time_sparse_outer_grad(idrs_matrix A, int warmup, int reps, double* ms_per_call) {
  return guard([&] {
    REQUIRE(A && reps >= 1 && warmup >= 0 && ms_per_call, "time_sparse_outer_grad: bad arguments");
    REQUIRE(A->K->format == FMT_CRS && A->K->vals != 2, "time_sparse_outer_grad: real CRS matrix required");
    const long n = A->n(), nnz = A->K->nnz;
    cudaStream_t st = A->stream;
    DBuf lam(sizeof(double) * n, st), x(sizeof(double) * n, st), g(sizeof(double) * std::max(nnz, 1L), st);
    IDRS_CUDA(cudaMemsetAsync(lam.p, 0, sizeof(double) * n, st));
    IDRS_CUDA(cudaMemsetAsync(x.p, 0, sizeof(double) * n, st));
    auto once = [&] { sparse_outer_grad(*A->K, lam.as<double>(), x.as<double>(), g.as<double>(), st); };
    for (int i = 0; i < warmup; ++i) once();
    cudaEvent_t e0, e1;
    IDRS_CUDA(cudaEventCreate(&e0));
    IDRS_CUDA(cudaEventCreate(&e1));
    IDRS_CUDA(cudaEventRecord(e0, st));
    for (int i = 0; i < reps; ++i) once();
    IDRS_CUDA(cudaEventRecord(e1, st));
    IDRS_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    IDRS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms_per_call = ms / reps;
    return IDRS_OK;
  });
}

int idrs_ridrs(idrs_matrix A, const double* b, int s, idrs_matrix M1, const double* tolerance,
               const int* maximum_iterations, const int* variant, int* flag, double* relres,
               int* iterations, const double* x0, const double* U0, const double* omega,
               int n_omega, double* resvec, int resvec_len, double* H, int ldh, int nritz,
               double* x) {
  return guard([&] {
    REQUIRE(A && !A->cplx, "ridrs: real matrix handle required");
    return run_idrs<double>(A, b, s, M1, tolerance, maximum_iterations, variant, flag, relres,
                            iterations, x0, U0, omega, n_omega, resvec, resvec_len, H, ldh, nritz, x);
  });
}
int idrs_cidrs(idrs_matrix A, const double* b, int s, idrs_matrix M1, const double* tolerance,
               const int* maximum_iterations, const int* variant, int* flag, double* relres,
               int* iterations, const double* x0, const double* U0, const double* omega,
               int n_omega, double* resvec, int resvec_len, double* H, int ldh, int nritz,
               double* x) {
  return guard([&] {
    REQUIRE(A && A->cplx, "cidrs: complex matrix handle required");
    return run_idrs<c128>(A, b, s, M1, tolerance, maximum_iterations, variant, flag, relres,
                          iterations, x0, U0, omega, n_omega, resvec, resvec_len, H, ldh, nritz, x);
  });
}

int idrs_rqmridr(idrs_matrix A, const double* b, int s, idrs_matrix M1, const double* tolerance,
                 const int* maximum_iterations, int* flag, double* relres, int* iterations,
                 const int* inner_s, const double* inner_tolerance, const int* inner_iterations,
                 const double* x0, const double* omega, int n_omega, double* resvec,
                 int resvec_len, const int* inner_precision, double* x) {
  return guard([&] {
    REQUIRE(A && !A->cplx, "rqmridr: real matrix handle required");
    return run_qmridr<double, float>(A, b, s, M1, tolerance, maximum_iterations, flag, relres,
                                     iterations, inner_s, inner_tolerance, inner_iterations, x0,
                                     omega, n_omega, resvec, resvec_len, inner_precision, x);
  });
}
int idrs_cqmridr(idrs_matrix A, const double* b, int s, idrs_matrix M1, const double* tolerance,
                 const int* maximum_iterations, int* flag, double* relres, int* iterations,
                 const int* inner_s, const double* inner_tolerance, const int* inner_iterations,
                 const double* x0, const double* omega, int n_omega, double* resvec,
                 int resvec_len, const int* inner_precision, double* x) {
  return guard([&] {
    REQUIRE(A && A->cplx, "cqmridr: complex matrix handle required");
    return run_qmridr<c128, c64>(A, b, s, M1, tolerance, maximum_iterations, flag, relres,
                                 iterations, inner_s, inner_tolerance, inner_iterations, x0,
                                 omega, n_omega, resvec, resvec_len, inner_precision, x);
  });
}

int idrs_rmsidrs(idrs_matrix A, const double* b, int n_sigma, const double* sigma, int s,
                 idrs_matrix M1, const double* tolerance, const int* maximum_iterations,
                 const int* variant, int* flag, double* relres, int* iterations,
                 const double* omega, int n_omega, double* resvec, int resvec_len, double* colfac,
                 double* x) {
  return guard([&] {
    REQUIRE(A && !A->cplx, "rmsidrs: real matrix handle required");
    return run_msidrs<double>(A, b, n_sigma, sigma, s, M1, tolerance, maximum_iterations, variant,
                              flag, relres, iterations, omega, n_omega, resvec, resvec_len, colfac, x);
  });
}
int idrs_cmsidrs(idrs_matrix A, const double* b, int n_sigma, const double* sigma, int s,
                 idrs_matrix M1, const double* tolerance, const int* maximum_iterations,
                 const int* variant, int* flag, double* relres, int* iterations,
                 const double* omega, int n_omega, double* resvec, int resvec_len, double* colfac,
                 double* x) {
  return guard([&] {
    REQUIRE(A && A->cplx, "cmsidrs: complex matrix handle required");
    return run_msidrs<c128>(A, b, n_sigma, sigma, s, M1, tolerance, maximum_iterations, variant,
                            flag, relres, iterations, omega, n_omega, resvec, resvec_len, colfac, x);
  });
}
int idrs_rmsqmridr(idrs_matrix A, const double* b, int n_sigma, const double* sigma, int s,
                   idrs_matrix M1, const double* tolerance, const int* maximum_iterations,
                   int* flag, double* relres, int* iterations, const int* inner_s,
                   const double* inner_tolerance, const int* inner_iterations,
                   const double* omega, int n_omega, double* resvec, int resvec_len,
                   const int* inner_precision, double* x) {
  return guard([&] {
    REQUIRE(A && !A->cplx, "rmsqmridr: real matrix handle required");
    return run_msqmridr<double, float>(A, b, n_sigma, sigma, s, M1, tolerance, maximum_iterations,
                                       flag, relres, iterations, inner_s, inner_tolerance,
                                       inner_iterations, omega, n_omega, resvec, resvec_len,
                                       inner_precision, x);
  });
}
int idrs_cmsqmridr(idrs_matrix A, const double* b, int n_sigma, const double* sigma, int s,
                   idrs_matrix M1, const double* tolerance, const int* maximum_iterations,
                   int* flag, double* relres, int* iterations, const int* inner_s,
                   const double* inner_tolerance, const int* inner_iterations,
                   const double* omega, int n_omega, double* resvec, int resvec_len,
                   const int* inner_precision, double* x) {
  return guard([&] {
    REQUIRE(A && A->cplx, "cmsqmridr: complex matrix handle required");
    return run_msqmridr<c128, c64>(A, b, n_sigma, sigma, s, M1, tolerance, maximum_iterations,
                                   flag, relres, iterations, inner_s, inner_tolerance,
                                   inner_iterations, omega, n_omega, resvec, resvec_len,
                                   inner_precision, x);
  });
}

int idrs_solve_stats(idrs_matrix A, int* inner_solves, int* inner_iterations, int* inner_max) {
  return guard([&] {
    REQUIRE(A, "solve_stats: matrix handle required");
    if (inner_solves) *inner_solves = A->last_inner_calls;
    if (inner_iterations) *inner_iterations = A->last_inner_total;
    if (inner_max) *inner_max = A->last_inner_max;
    return IDRS_OK;
  });
}

// ------------------------------------------------------------------ adjoint
int idrs_crs_transpose(idrs_user_matrix K, idrs_user_matrix* KT) {
  return guard([&] {
    REQUIRE(K && KT, "crs_transpose: K and KT are required");
    REQUIRE(K->format == FMT_CRS, "crs_transpose: CRS matrix required");
    init_runtime();
    auto* M = new idrs_user_matrix_s();
    try {
      crs_transpose(*K, *M, nullptr);
    } catch (...) {
      delete M;
      throw;
    }
    *KT = M;
    return IDRS_OK;
  });
}

int idrs_rsparse_outer_grad(idrs_matrix A, const double* lambda, const double* x, double* grad) {
  return guard([&] {
    REQUIRE(A && lambda && x && grad, "sparse_outer_grad: bad arguments");
    REQUIRE(A->K->format == FMT_CRS && A->K->vals != 2, "sparse_outer_grad: real CRS matrix required");
    const long n = A->n();
    Staged sv(A, sizeof(double) * n), sg(A, sizeof(double) * A->K->nnz);
    const double* d_l = (const double*)sv.in(lambda);
    const double* d_x = (const double*)sv.in(x);
    double* d_g = (double*)sg.out(grad);
    sparse_outer_grad(*A->K, d_l, d_x, d_g, A->stream);
    sg.finish(grad, d_g);
    IDRS_CUDA(cudaStreamSynchronize(A->stream));
    return IDRS_OK;
  });
}

int idrs_radjoint(idrs_matrix AT, idrs_user_matrix K, const double* x, const double* g, int s,
                  const double* tolerance, const int* maximum_iterations, int* flag,
                  double* relres, int* iterations, double* lambda, double* grad) {
  return guard([&] {
    REQUIRE(AT && !AT->cplx && K && x && g && lambda, "radjoint: AT, K, x, g and lambda are required");
    REQUIRE(K->format == FMT_CRS && K->vals != 2, "radjoint: K must be a real CRS matrix");
    REQUIRE(K->nrows == AT->n() && K->ncols == AT->n(), "radjoint: K and AT differ in size");
    REQUIRE(s >= 1, "radjoint: s must be positive");
    if (s > MAXS) throw unsupported_error("radjoint: s > 16 is not supported by the GPU path");
    SolveOpts o;
    if (tolerance) {
      REQUIRE(*tolerance >= 0, "Illegal value for parameter tolerance");
      o.tol = *tolerance;
    }
    const long n = AT->n();
    o.maxit = maximum_iterations ? *maximum_iterations : (int)std::min<long>(2 * n, 1000);
    o.PT = find_shadow(AT, s);
    cudaStream_t st = AT->stream;
    Staged sv(AT, sizeof(double) * n), sg(AT, sizeof(double) * K->nnz);
    const double* d_g = (const double*)sv.in(g);
    const double* d_x = (const double*)sv.in(x);
    double* d_lam = (double*)sv.out(lambda);
    double* d_grad = grad ? (double*)sg.out(grad) : nullptr;
    DBuf mu(sizeof(double) * n, st), t1(sizeof(double) * n, st), t2(sizeof(double) * n, st);
    // A^T mu = g with IDR(s) on the adjoint operator, then lambda = scaleback(AT, g, mu)
    IdrsGpu<double> solver(*AT, 64, s, 1);
    solver.solve(d_g, mu.as<double>(), o);
    op_scaleback<double>(*AT, 64, AT->alpha_p, AT->degree, mu.as<double>(), d_lam, t1.as<double>(),
                         t2.as<double>(), nullptr, st);
    if (d_grad) sparse_outer_grad(*K, d_lam, d_x, d_grad, st);
    auto h = solver.state();
    sv.finish(lambda, d_lam);
    if (d_grad) sg.finish(grad, d_grad);
    IDRS_CUDA(cudaStreamSynchronize(st));
    if (flag) *flag = h.info;
    if (relres) *relres = h.relres;
    if (iterations) *iterations = h.iter;
    return IDRS_OK;
  });
}

}  // extern "C"

// RIDRS_RITZ / CIDRS_RITZ (ritz_module.f90:268-556): IDRS with the
// Hessenberg output, then omega and the recycle space.  T: double or c128;
// H, omega, U0 have the kind of T (complex interleaved).
template <class T>
static int ritz_t(idrs_matrix A, const double* b, int s, idrs_matrix M, const double* tolerance,
                  const int* maximum_iterations, const int* variant, int* flag, double* relres,
                  int* iterations, const double* x0, double* U0, int dimU0, double* omega,
                  int n_omega, double* resvec, int resvec_len, double* H, int ldh, int nh,
                  int* nritz, double* x) {
  constexpr bool cplx = traits<T>::is_cplx;
  constexpr int vw = cplx ? 2 : 1;
  REQUIRE(A && A->cplx == cplx && b && x, "idrs_ritz: bad arguments");
  REQUIRE(!M || M->cplx == cplx, "idrs_ritz: M must have the kind of A");
  long n = A->n();
  if (tolerance) REQUIRE(*tolerance >= 0, "Illegal value for parameter tolerance");
  int maxit = maximum_iterations ? *maximum_iterations : (int)std::min<long>(2 * n, 1000);
  REQUIRE(maxit >= 1, "idrs_ritz: maximum_iterations must be positive");
  if (resvec) REQUIRE(resvec_len >= maxit + 1, "Length of vector with residual norms too small, should be maxit+1");
  if (U0 && dimU0 > 0) REQUIRE(dimU0 <= MAXS, "idrs_ritz: dimension of U0 larger than 16");
  std::vector<double> Hf((size_t)vw * (maxit + 1) * maxit, 0.0);
  std::vector<double> zeros;
  const double* xs = x0;
  if (!xs && !A->device_pointers) { zeros.assign((size_t)vw * n, 0.0); xs = zeros.data(); }
  int conv = -1, iter = 0, method = variant ? *variant : 1;
  double rel = 1.0;
  std::vector<double> resnrm(maxit + 1);
  int st = run_idrs<T>(A, b, s, M, tolerance, &maxit, &method, &conv, &rel, &iter, xs, nullptr,
                       nullptr, 0, resnrm.data(), maxit + 1, Hf.data(), maxit + 1, maxit, x);
  if (st) return st;
  const int nr = (iter / (s + 1)) * s + iter % (s + 1);
  if (flag) *flag = conv;
  if (relres) *relres = rel;
  if (iterations) *iterations = iter;
  if (nritz) *nritz = nr;
  if (resvec) std::copy(resnrm.begin(), resnrm.end(), resvec);
  const T* Ht = (const T*)Hf.data();
  if (omega && n_omega > 0) {
    REQUIRE(nr >= n_omega, "Too many parameters omega requested, reduce omega.");
    if constexpr (cplx) ritz_omega((const cd*)Hf.data(), maxit + 1, n_omega, (cd*)omega);
    else ritz_omega(Hf.data(), maxit + 1, n_omega, omega);
  }
  if (U0 && dimU0 > 0) {
    REQUIRE(nr >= dimU0, "Recycle space is too large, reduce dimension of U0.");
    cudaStream_t cs = A->stream;
    std::vector<T> vec((size_t)nr * dimU0);
    std::vector<double> resval(dimU0);
    if constexpr (cplx) {
      // the first dimU0 Schur vectors of QR_eig (ritz_module.f90:367-368)
      std::vector<cd> Vs((size_t)nr * nr), ev(nr);
      int conv_eig = 0;
      qr_eig((const cd*)Hf.data(), maxit + 1, nr, ev.data(), &conv_eig, Vs.data());
      for (int j = 0; j < dimU0; ++j)
        for (int i = 0; i < nr; ++i) vec[i + (size_t)nr * j] = c128(Vs[i + (size_t)nr * j].real(), Vs[i + (size_t)nr * j].imag());
    } else {
      si_power(Hf.data(), maxit + 1, nr, dimU0, 0.0, kSiPowerSeed, (double*)vec.data());
    }
    Staged sb(A, sizeof(T) * n), su(A, sizeof(T) * n * dimU0);
    const T* d_b = (const T*)sb.in(b);
    T* d_U = (T*)su.out(U0);
    Operator* Mp = (M && M->dkind != 0) ? M : nullptr;
    compute_u0<T>(*A, Mp, Ht, maxit + 1, nr, vec.data(), dimU0, d_b, d_U, resval.data(), cs);
    if (Mp)
      for (int j = 0; j < dimU0; ++j) {
        DBuf tmp(sizeof(T) * n, cs);
        op_precon<T>(*Mp, 64, d_U + (size_t)n * j, tmp.as<T>(), nullptr, cs);
        IDRS_CUDA(cudaMemcpyAsync(d_U + (size_t)n * j, tmp.p, sizeof(T) * n, cudaMemcpyDeviceToDevice, cs));
      }
    int dep = global_qr<T>(n, dimU0, d_U, nullptr, A->red, cs);
    REQUIRE(dep == 0, " V has dependent columns ");
    su.finish(U0, d_U);
    IDRS_CUDA(cudaStreamSynchronize(cs));
  }
  if (H) {
    REQUIRE((long)ldh * nh <= (long)(maxit + 1) * maxit && ldh <= maxit + 1 && nh <= maxit,
            "Dimensions of Hessenberg matrix too large");
    for (int j = 0; j < nh; ++j)
      for (int i = 0; i < ldh; ++i)
        for (int c = 0; c < vw; ++c)
          H[vw * (i + (size_t)ldh * j) + c] = Hf[vw * (i + (size_t)(maxit + 1) * j) + c];
  }
  return IDRS_OK;
}

extern "C" {

int idrs_ridrs_ritz(idrs_matrix A, const double* b, int s, idrs_matrix M,
                    const double* tolerance, const int* maximum_iterations, const int* variant,
                    int* flag, double* relres, int* iterations, const double* x0, double* U0,
                    int dimU0, double* omega, int n_omega, double* resvec, int resvec_len,
                    double* H, int ldh, int nh, int* nritz, double* x) {
  return guard([&] {
    return ritz_t<double>(A, b, s, M, tolerance, maximum_iterations, variant, flag, relres, iterations,
                          x0, U0, dimU0, omega, n_omega, resvec, resvec_len, H, ldh, nh, nritz, x);
  });
}

int idrs_cidrs_ritz(idrs_matrix A, const double* b, int s, idrs_matrix M,
                    const double* tolerance, const int* maximum_iterations, const int* variant,
                    int* flag, double* relres, int* iterations, const double* x0, double* U0,
                    int dimU0, double* omega, int n_omega, double* resvec, int resvec_len,
                    double* H, int ldh, int nh, int* nritz, double* x) {
  return guard([&] {
    return ritz_t<c128>(A, b, s, M, tolerance, maximum_iterations, variant, flag, relres, iterations,
                        x0, U0, dimU0, omega, n_omega, resvec, resvec_len, H, ldh, nh, nritz, x);
  });
}

}  // extern "C"

// ------------------------------------------------------------- pp_idrs
namespace {

using clk = std::chrono::steady_clock;

// One pp_idrs job (pp_idrs_module.f90): the operator built from K (M, C, P,
// seed, shift, V), its device buffers and what the set-up solves produced
// (x0, omega, U0).  T: double (RPP_*) or c128 (CPP_*).
template <class T>
struct PPJob {
  idrs_matrix A = nullptr;
  long n = 0;          // vector length (2 nn for the block system)
  long nn = 0;         // rows of K
  bool block = false;  // multishift with C: the 2 x 2 block system
  cudaStream_t cs = nullptr;
  DBuf d_x0, d_y, t1, t2, r, res;
  std::vector<T> omega;  // allocated when the initial solve ran
  DBuf U0;
  bool have_U0 = false;
  ~PPJob() {
    // device buffers go back on the operator's stream before it is destroyed
    d_x0 = DBuf(); d_y = DBuf(); t1 = DBuf(); t2 = DBuf(); r = DBuf(); res = DBuf(); U0 = DBuf();
    if (A) idrs_matrix_free(A);
  }
};

template <class T> constexpr bool kCplx = traits<T>::is_cplx;

// stores the real part of a reduction result (|w|^2 of a real or complex w)
__device__ inline double re_of(double v) { return v; }
__device__ inline double re_of(c128 v) { return v.x; }
template <class W> struct TStoreRe {
  double* out;
  __device__ void operator()(const W* v) const { *out = re_of(v[0]); }
};

// y = y + a x
template <class T>
__global__ void k_axpy(long n, T a, const T* __restrict__ x, T* y) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (long)blockDim.x)
    y[i] = y[i] + a * x[i];
}
template <class T>
void axpy(long n, T a, const T* x, T* y, cudaStream_t st) {
  k_axpy<T><<<stream_grid(n), kThreads, 0, st>>>(n, a, x, y);
  IDRS_LAUNCH_CHECK();
}

// real_matrix.inc / complex_matrix.inc (+ make_deflation when V is given)
template <class T>
int pp_open(PPJob<T>& J, idrs_user_matrix K, idrs_user_matrix P, const idrs_pp_inputs* in,
            bool multishift, const idrs_pp_options* opt) {
  REQUIRE(K, "pp_idrs: K is required");
  REQUIRE(opt->s >= 1, "rpp_idrs: s must be positive");
  REQUIRE(std::isfinite(opt->fp64_check_tol) && opt->fp64_check_tol >= 0.0,
          "pp_idrs: fp64_check_tol must be 0 (no check) or a positive tolerance");
  REQUIRE(opt->n_omega >= 0, "rpp_idrs: n_omega must not be negative");
  idrs_user_matrix M = in ? in->M : nullptr, C = in ? in->C : nullptr;
  int st = idrs_matrix_create_ext(K, M, C, P, kCplx<T> ? 1 : 0, in ? in->seed : nullptr,
                                  in ? in->shift : nullptr, multishift ? 1 : 0, &J.A);
  if (st) return st;
  J.n = J.A->n();
  J.nn = K->nrows;
  J.block = multishift && C;
  J.cs = J.A->stream;
  const size_t vb = sizeof(T) * J.n;
  J.d_x0 = DBuf(vb, J.cs);
  J.d_y = DBuf(vb, J.cs);
  J.t1 = DBuf(vb, J.cs);
  J.t2 = DBuf(vb, J.cs);
  J.r = DBuf(vb, J.cs);
  J.res = DBuf(16, J.cs);
  IDRS_CUDA(cudaMemsetAsync(J.d_x0.p, 0, vb, J.cs));
  J.A->device_pointers = true;
  return IDRS_OK;
}

// `if (present(V)) call make_deflation(A, V)` with a host V (n x k)
template <class T>
int pp_deflate(PPJob<T>& J, const idrs_pp_inputs* in) {
  if (!in || !in->V || in->n_deflation <= 0) return IDRS_OK;
  J.A->device_pointers = false;
  int st = idrs_make_deflation(J.A, in->V, in->n_deflation);
  J.A->device_pointers = true;
  return st;
}

// IDRS_RITZ for the set-up solves: real -> idrs_ridrs_ritz; complex -> IDRS
// with the Hessenberg output and the complex omega ordering.
template <class T>
int pp_ritz(PPJob<T>& J, const T* pb, int s, double tol, int maxit, T* x, double* H, int ldh,
            int nh, int n_omega, T* omega, double* U0, int dimU0, int* flag, double* relres,
            int* iter, int* nritz) {
  int one = 1;
  auto fn = kCplx<T> ? idrs_cidrs_ritz : idrs_ridrs_ritz;
  return fn(J.A, (const double*)pb, s, nullptr, &tol, &maxit, &one, flag, relres, iter, nullptr, U0,
            dimU0, n_omega > 0 ? (double*)omega : nullptr, n_omega, nullptr, 0, H, ldh, nh, nritz,
            (double*)x);
}

// real_preconditioner.inc / complex_preconditioner.inc: the initial
// IDRS_RITZ solve (x0, H and, with n_omega > 0, omega) and the polynomial
// preconditioner.  center / foci: 1 / 2 values of the kind of T.
template <class T>
int pp_setup(PPJob<T>& J, const T* pb, const double* center, const double* foci,
             const idrs_pp_options* opt, idrs_pp_report& rep) {
  const int s = opt->s;
  constexpr int vw = kCplx<T> ? 2 : 1;
  REQUIRE(opt->poly_eval == IDRS_POLY_HORNER || opt->poly_eval == IDRS_POLY_RECURRENCE,
          "pp_idrs: poly_eval must be IDRS_POLY_HORNER or IDRS_POLY_RECURRENCE");
  J.A->poly_eval = opt->poly_eval;
  int preconditioner = opt->degree == 0 ? 0 : opt->preconditioner;
  bool estimate = preconditioner != 0;
  if (preconditioner == 1 && center) estimate = false;
  if (preconditioner == 2 && foci) estimate = false;
  const bool initial = estimate || opt->n_omega > 0;
  std::vector<double> H;
  int ldh = 0;
  if (initial) {
    int ini_iter = opt->n_ritz + opt->n_ritz / s;
    ldh = ini_iter + 1;
    H.assign((size_t)vw * ldh * ini_iter, 0.0);
    J.omega.assign(std::max(opt->n_omega, 0), T(0.0));
    int flag = -1, iter = 0, nr = 0;
    double rel = 1;
    int st = pp_ritz<T>(J, pb, s, opt->tol, ini_iter, J.d_x0.template as<T>(), H.data(), ldh, ini_iter,
                        opt->n_omega, J.omega.data(), nullptr, 0, &flag, &rel, &iter, &nr);
    if (st) return st;
    rep.ritz_iterations = iter;
    rep.nritz = nr;
  }
  if (estimate) {
    if constexpr (kCplx<T>) {
      std::vector<std::complex<double>> Hc((size_t)ldh * std::max(rep.nritz, 1));
      for (size_t q = 0; q < Hc.size() && 2 * q + 1 < H.size(); ++q) Hc[q] = {H[2 * q], H[2 * q + 1]};
      std::complex<double> f[2], c;
      analyse_spectrum(Hc.data(), ldh, rep.nritz, f, &c, nullptr);
      rep.foci[0] = f[0].real(); rep.foci[1] = f[1].real(); rep.center = c.real();
      rep.foci_imag[0] = f[0].imag(); rep.foci_imag[1] = f[1].imag(); rep.center_imag = c.imag();
    } else {
      analyse_spectrum(H.data(), ldh, rep.nritz, rep.foci, &rep.center, nullptr);
    }
    return set_preconditioner(J.A, preconditioner, opt->degree, nullptr, nullptr, H.data(), ldh, rep.nritz);
  }
  double f[4] = {0.15, 0.0, 1.85, 0.0}, c[2] = {1.0, 0.0};
  if (kCplx<T>) {
    if (foci) for (int q = 0; q < 4; ++q) f[q] = foci[q];
    if (center) { c[0] = center[0]; c[1] = center[1]; }
    rep.foci[0] = f[0]; rep.foci[1] = f[2]; rep.center = c[0];
    rep.foci_imag[0] = f[1]; rep.foci_imag[1] = f[3]; rep.center_imag = c[1];
  } else {
    f[1] = 1.85;
    if (foci) { f[0] = foci[0]; f[1] = foci[1]; }
    if (center) c[0] = *center;
    rep.foci[0] = f[0]; rep.foci[1] = f[1]; rep.center = c[0];
  }
  return set_preconditioner(J.A, preconditioner, opt->degree, f, c, nullptr, 0, 0);
}

// recycle.inc: x0 = IDRS_RITZ(A, b, s, tol, maxit, variant 1) with U0 (n x s)
template <class T>
int pp_recycle(PPJob<T>& J, const T* pb, const idrs_pp_options* opt, idrs_pp_report& rep) {
  const int s = opt->s;
  J.U0 = DBuf(sizeof(T) * J.n * s, J.cs);
  int nr = 0;
  int st = pp_ritz<T>(J, pb, s, opt->tol, opt->maxit, J.d_x0.template as<T>(), nullptr, 0, 0, 0, nullptr,
                      (double*)J.U0.template as<T>(), s, &rep.recycle_flag, &rep.recycle_relres,
                      &rep.recycle_iterations, &nr);
  if (st) return st;
  J.have_U0 = true;
  return IDRS_OK;
}

// |b - S x| / |b| with S the unscaled system matrix at the seed (the
// assembled K + seed C + seed^2 M, or K - seed M, ...), run_idrs.inc:44-59
template <class T>
double true_relres(PPJob<T>& J, const T* pb, const T* px) {
  using W = typename traits<T>::wide;
  cudaStream_t cs = J.cs;
  idrs_matrix A = J.A;
  spmv<T>(A->k64, px, J.r.template as<T>(), T(-1.0), T(1.0), pb, nullptr, cs);
  if (!A->seed_folded && (A->seed.x != 0.0 || A->seed.y != 0.0)) {
    // K x - seed x with an unassembled seed
    axpy<T>(J.n, narrow<T>(A->seed), px, J.r.template as<T>(), cs);
  }
  launch_fused<1, T>(J.n, BNorm<T>{J.r.template as<T>()}, TStoreRe<typename traits<T>::wide>{J.res.template as<double>()}, A->red, nullptr, cs);
  launch_fused<1, T>(J.n, BNorm<T>{pb}, TStoreRe<typename traits<T>::wide>{J.res.template as<double>() + 1}, A->red, nullptr, cs);
  double h[2] = {0, 0};
  IDRS_CUDA(cudaMemcpyAsync(h, J.res.p, 16, cudaMemcpyDeviceToHost, cs));
  IDRS_CUDA(cudaStreamSynchronize(cs));
  (void)sizeof(W);
  return std::sqrt(h[0]) / std::sqrt(h[1]);
}

// One solve of run_idrs.inc:9-60 / run_mr_idrs.inc:15-72 from x0 (then
// x0 = y), x = scaleback(A, b, y) and the original system's relative residual.
template <class T>
int pp_solve(PPJob<T>& J, const T* pb, T* px, const idrs_pp_options* opt, idrs_pp_report& rep) {
  idrs_matrix A = J.A;
  const long n = J.n;
  const int s = opt->s;
  double tol = opt->tol;
  int maxit = opt->maxit, st = 0;
  const double* om = J.omega.empty() ? nullptr : (const double*)J.omega.data();
  const int n_om = (int)J.omega.size();
  // Pmul(A, b): the deflated right-hand side
  const T* rb = pb;
  if (A->defl && A->defl->k > 0) {
    deflation_pmul<T>(*A->defl, pb, J.t1.template as<T>(), T(1.0), T(0.0), nullptr, nullptr, J.cs);
    rb = J.t1.template as<T>();
  }
  if (opt->method == 0) {
    int in_s = opt->in_s, in_it = opt->in_it, prec = opt->inner_precision ? opt->inner_precision : 64;
    double in_tol = opt->in_tol;
    st = run_qmridr<T, typename std::conditional<kCplx<T>, c64, float>::type>(
        A, (const double*)rb, s, nullptr, &tol, &maxit, &rep.flag, &rep.relres_solver, &rep.iterations,
        &in_s, &in_tol, &in_it, (const double*)J.d_x0.template as<T>(), om, n_om, nullptr, 0, &prec,
        (double*)J.d_y.template as<T>());
    rep.inner_solves = A->last_inner_calls;
    rep.inner_iterations = A->last_inner_total;
    rep.inner_max = A->last_inner_max;
  } else {
    int variant = opt->method == 2 ? 2 : 1;
    st = run_idrs<T>(A, (const double*)rb, s, nullptr, &tol, &maxit, &variant, &rep.flag,
                     &rep.relres_solver, &rep.iterations, (const double*)J.d_x0.template as<T>(),
                     J.have_U0 ? (const double*)J.U0.template as<T>() : nullptr, om, n_om, nullptr, 0, nullptr, 0, 0,
                     (double*)J.d_y.template as<T>());
  }
  if (st) return st;
  cudaStream_t cs = J.cs;
  // x0 = y (the warm start of the next right-hand side); x = scaleback(A, b, y)
  IDRS_CUDA(cudaMemcpyAsync(J.d_x0.p, J.d_y.p, sizeof(T) * n, cudaMemcpyDeviceToDevice, cs));
  op_scaleback<T>(*A, 64, A->alpha_p, A->degree, J.d_y.template as<T>(), px, J.t1.template as<T>(), J.t2.template as<T>(), nullptr,
                  cs, pb);
  rep.relres_original = true_relres<T>(J, pb, px);
  return IDRS_OK;
}

// ||x - xr|| / ||xr|| on the device (J.r is the scratch vector)
template <class T>
double rel_diff(PPJob<T>& J, const T* x, const T* xr) {
  cudaStream_t cs = J.cs;
  T* d = J.r.template as<T>();
  IDRS_CUDA(cudaMemcpyAsync(d, x, sizeof(T) * J.n, cudaMemcpyDeviceToDevice, cs));
  axpy<T>(J.n, T(-1.0), xr, d, cs);
  using W = typename traits<T>::wide;
  launch_fused<1, T>(J.n, BNorm<T>{d}, TStoreRe<W>{J.res.template as<double>()}, J.A->red, nullptr, cs);
  launch_fused<1, T>(J.n, BNorm<T>{xr}, TStoreRe<W>{J.res.template as<double>() + 1}, J.A->red, nullptr, cs);
  double h[2] = {0, 0};
  IDRS_CUDA(cudaMemcpyAsync(h, J.res.p, 16, cudaMemcpyDeviceToHost, cs));
  IDRS_CUDA(cudaStreamSynchronize(cs));
  return std::sqrt(h[0]) / std::sqrt(h[1]);
}

// The FP64 solve a result is checked against (no counterpart in the
// reference): the same preconditioned system solved again from x0 = 0 by the
// FP64 form of the method (QMRIDR(s) without inner solves, or IDR(s)) to
// opt->fp64_check_tol, with at least min(2n, 5000) iterations;
// rel_err_vs_fp64 = ||x - x64|| / ||x64||.  The warm start of the next
// right-hand side (J.d_x0) is kept.
// the iteration bound of the check's FP64 solve (at least)
int fp64_check_maxit(long n) { return (int)std::min<long>(2 * n, 5000); }

void no_fp64_check(idrs_pp_report& rep) {
  rep.rel_err_vs_fp64 = -1.0;
  rep.fp64_relres_original = -1.0;
  rep.fp64_flag = -1;
  rep.fp64_iterations = 0;
  rep.seconds_fp64_check = 0.0;
}

template <class T>
int pp_fp64_check(PPJob<T>& J, const T* pb, const T* px, const idrs_pp_options* opt, idrs_pp_report& rep) {
  no_fp64_check(rep);
  if (!(opt->fp64_check_tol > 0.0)) return IDRS_OK;
  auto t0 = clk::now();
  const size_t vb = sizeof(T) * J.n;
  DBuf keep(vb, J.cs), xr(vb, J.cs);
  IDRS_CUDA(cudaMemcpyAsync(keep.p, J.d_x0.p, vb, cudaMemcpyDeviceToDevice, J.cs));
  IDRS_CUDA(cudaMemsetAsync(J.d_x0.p, 0, vb, J.cs));
  idrs_pp_options o = *opt;
  o.tol = opt->fp64_check_tol;
  o.maxit = std::max(opt->maxit, fp64_check_maxit(J.n));  // a mixed call bounds outer iterations only
  o.in_it = 0;
  o.inner_precision = 64;
  idrs_pp_report r{};
  int st = pp_solve<T>(J, pb, xr.template as<T>(), &o, r);
  if (st) return st;
  rep.rel_err_vs_fp64 = rel_diff<T>(J, px, xr.template as<T>());
  rep.fp64_relres_original = r.relres_original;
  rep.fp64_flag = r.flag;
  rep.fp64_iterations = r.iterations;
  IDRS_CUDA(cudaMemcpyAsync(J.d_x0.p, keep.p, vb, cudaMemcpyDeviceToDevice, J.cs));
  IDRS_CUDA(cudaStreamSynchronize(J.cs));
  rep.seconds_fp64_check = std::chrono::duration<double>(clk::now() - t0).count();
  return IDRS_OK;
}

}  // namespace

extern "C" {

int idrs_rpp_idrs(idrs_user_matrix K, const double* b, idrs_user_matrix P, const double* center,
                  const double* foci, const idrs_pp_options* opt, idrs_pp_report* report,
                  double* x) {
  return idrs_rpp_idrs_ext(K, b, P, center, foci, nullptr, opt, report, x);
}

int idrs_rpp_mr_idrs(idrs_user_matrix K, int nrhs, const double* b_all, idrs_user_matrix P,
                     const double* center, const double* foci, const idrs_pp_options* opt,
                     idrs_pp_report* reports, double* x_all) {
  return idrs_rpp_mr_idrs_ext(K, nrhs, b_all, P, center, foci, nullptr, opt, reports, x_all);
}

}  // extern "C"

namespace {

template <class T>
int pp_idrs_t(idrs_user_matrix K, const double* b, idrs_user_matrix P, const double* center,
              const double* foci, const idrs_pp_inputs* in, const idrs_pp_options* opt,
              idrs_pp_report* report, double* x) {
  REQUIRE(K && b && opt && x, "pp_idrs: bad arguments");
  auto t0 = clk::now();
  PPJob<T> J;
  int st = pp_open<T>(J, K, P, in, false, opt);
  if (st) return st;
  const long n = J.n;
  const bool dev = opt->device_pointers != 0;
  DBuf hb, hx;
  const T* pb = (const T*)b;
  T* px = (T*)x;
  if (!dev) {
    hb = DBuf(sizeof(T) * n, J.cs);
    hx = DBuf(sizeof(T) * n, J.cs);
    IDRS_CUDA(cudaMemcpyAsync(hb.p, b, sizeof(T) * n, cudaMemcpyHostToDevice, J.cs));
    pb = hb.template as<T>();
    px = hx.template as<T>();
  }
  idrs_pp_report rep{};
  st = pp_setup<T>(J, pb, center, foci, opt, rep);
  if (st) return st;
  st = pp_deflate<T>(J, in);  // after the preconditioner (pp_idrs_module.f90:108-111, :154-157)
  if (st) return st;
  IDRS_CUDA(cudaStreamSynchronize(J.cs));
  auto t1 = clk::now();
  st = pp_solve<T>(J, pb, px, opt, rep);
  if (st) return st;
  if (!dev) IDRS_CUDA(cudaMemcpyAsync(x, px, sizeof(T) * n, cudaMemcpyDeviceToHost, J.cs));
  IDRS_CUDA(cudaStreamSynchronize(J.cs));
  auto t2 = clk::now();
  rep.seconds_setup = std::chrono::duration<double>(t1 - t0).count();
  rep.seconds_solve = std::chrono::duration<double>(t2 - t1).count();
  rep.seconds_total = std::chrono::duration<double>(t2 - t0).count();
  st = pp_fp64_check<T>(J, pb, px, opt, rep);
  if (st) return st;
  if (report) *report = rep;
  return IDRS_OK;
}

template <class T>
int pp_mr_idrs_t(idrs_user_matrix K, int nrhs, const double* b_all, idrs_user_matrix P,
                 const double* center, const double* foci, const idrs_pp_inputs* in,
                 const idrs_pp_options* opt, idrs_pp_report* reports, double* x_all) {
  REQUIRE(K && b_all && opt && x_all && nrhs >= 1, "pp_mr_idrs: bad arguments");
  auto t0 = clk::now();
  PPJob<T> J;
  int st = pp_open<T>(J, K, P, in, false, opt);
  if (st) return st;
  const long n = J.n;
  const bool dev = opt->device_pointers != 0;
  // one right-hand side on the device at a time (host arrays are staged per column)
  DBuf hb, hx;
  if (!dev) { hb = DBuf(sizeof(T) * n, J.cs); hx = DBuf(sizeof(T) * n, J.cs); }
  const T* B = (const T*)b_all;
  T* X = (T*)x_all;
  auto column_b = [&](int irhs) -> const T* {
    if (dev) return B + (size_t)n * irhs;
    IDRS_CUDA(cudaMemcpyAsync(hb.p, B + (size_t)n * irhs, sizeof(T) * n, cudaMemcpyHostToDevice, J.cs));
    return hb.template as<T>();
  };
  idrs_pp_report base{};
  // RPP_MR_IDRS deflates before the preconditioner set-up, CPP_MR_IDRS after
  // it (pp_idrs_module.f90:260-266 and :204-207)
  if (!kCplx<T>) {
    st = pp_deflate<T>(J, in);
    if (st) return st;
  }
  st = pp_setup<T>(J, column_b(0), center, foci, opt, base);
  if (st) return st;
  if (kCplx<T>) {
    st = pp_deflate<T>(J, in);
    if (st) return st;
  }
  if (opt->recycle) {
    st = pp_recycle<T>(J, column_b(0), opt, base);
    if (st) return st;
  }
  IDRS_CUDA(cudaStreamSynchronize(J.cs));
  auto t1 = clk::now();
  const double setup = std::chrono::duration<double>(t1 - t0).count();
  for (int irhs = 0; irhs < nrhs; ++irhs) {
    auto ts = clk::now();
    idrs_pp_report rep = base;
    const T* pb = column_b(irhs);
    T* px = dev ? X + (size_t)n * irhs : hx.template as<T>();
    st = pp_solve<T>(J, pb, px, opt, rep);
    if (st) return st;
    if (!dev)
      IDRS_CUDA(cudaMemcpyAsync(X + (size_t)n * irhs, px, sizeof(T) * n, cudaMemcpyDeviceToHost, J.cs));
    IDRS_CUDA(cudaStreamSynchronize(J.cs));
    auto te = clk::now();
    rep.seconds_setup = setup;
    rep.seconds_solve = std::chrono::duration<double>(te - ts).count();
    rep.seconds_total = std::chrono::duration<double>(te - t0).count();
    st = pp_fp64_check<T>(J, pb, px, opt, rep);
    if (st) return st;
    if (reports) reports[irhs] = rep;
  }
  return IDRS_OK;
}

// r = rhs - K s - sigma C s - sigma^2 M s (and the other forms of
// run_ms_idrs.inc:35-58), |r| / |rhs|, on the device with the user matrices
template <class T>
double ms_true_relres(PPJob<T>& J, idrs_user_matrix K, const idrs_pp_inputs* in, c128 sigma,
                      const T* rhs, const T* sol, T* r, T* u) {
  cudaStream_t cs = J.cs;
  const long nn = J.nn;
  const T sg = narrow<T>(sigma);
  const T zero = T(0.0);
  idrs_user_matrix M = in ? in->M : nullptr, C = in ? in->C : nullptr;
  spmv<T>(K->view64(), sol, r, T(-1.0), T(1.0), rhs, nullptr, cs);  // r = rhs - K s
  if (M && C) {
    spmv<T>(C->view64(), sol, u, T(1.0), zero, nullptr, nullptr, cs);
    axpy<T>(nn, zero - sg, u, r, cs);
    spmv<T>(M->view64(), sol, u, T(1.0), zero, nullptr, nullptr, cs);
    axpy<T>(nn, zero - sg * sg, u, r, cs);
  } else if (C) {
    spmv<T>(C->view64(), sol, u, T(1.0), zero, nullptr, nullptr, cs);
    axpy<T>(nn, zero - sg, u, r, cs);
    axpy<T>(nn, zero - sg * sg, sol, r, cs);
  } else if (M) {
    spmv<T>(M->view64(), sol, u, T(1.0), zero, nullptr, nullptr, cs);
    axpy<T>(nn, sg, u, r, cs);
  } else {
    axpy<T>(nn, sg, sol, r, cs);
  }
  launch_fused<1, T>(nn, BNorm<T>{r}, TStoreRe<typename traits<T>::wide>{J.res.template as<double>()}, J.A->red, nullptr, cs);
  launch_fused<1, T>(nn, BNorm<T>{rhs}, TStoreRe<typename traits<T>::wide>{J.res.template as<double>() + 1}, J.A->red, nullptr, cs);
  double h[2] = {0, 0};
  IDRS_CUDA(cudaMemcpyAsync(h, J.res.p, 16, cudaMemcpyDeviceToHost, cs));
  IDRS_CUDA(cudaStreamSynchronize(cs));
  return std::sqrt(h[0]) / std::sqrt(h[1]);
}

// RPP_MS_IDRS / CPP_MS_IDRS (pp_idrs_module.f90:281-409, run_ms_idrs.inc) and
// RPP_MS_MR_IDRS / CPP_MS_MR_IDRS (:411-..., run_ms_mr_idrs.inc): b = [-rhs; 0]
// for the block system, set-up on the first right-hand side, ms_parameters,
// then per right-hand side MSIDRS or MSQMRIDR on Pmul(b), scaleback, the
// solution (second half for the block system) and the true residuals.  The
// sequence form scales back with the deflated b, as run_ms_mr_idrs.inc does.
template <class T>
int pp_ms_t(idrs_user_matrix K, int nrhs, const double* rhs_all, int n_sigma, const double* sigma,
            idrs_user_matrix P, const double* center, const double* foci, const idrs_pp_inputs* in,
            const idrs_pp_options* opt, idrs_pp_report* reports, double* relres_sigma, double* x,
            bool sequence) {
  REQUIRE(K && rhs_all && sigma && opt && x && n_sigma >= 1 && nrhs >= 1, "pp_ms_idrs: bad arguments");
  REQUIRE(!opt->device_pointers, "pp_ms_idrs: host arrays only");
  auto t0 = clk::now();
  PPJob<T> J;
  int st = pp_open<T>(J, K, P, in, true, opt);
  if (st) return st;
  const long n = J.n, nn = J.nn;
  cudaStream_t cs = J.cs;
  DBuf db(sizeof(T) * n, cs), drhs(sizeof(T) * nn, cs), dY(sizeof(T) * n * n_sigma, cs),
      dX(sizeof(T) * n * n_sigma, cs), du(sizeof(T) * nn, cs);
  auto load_rhs = [&](int irhs) {  // b = rhs, or [-rhs; 0] for the block system
    IDRS_CUDA(cudaMemcpyAsync(drhs.p, (const T*)rhs_all + (size_t)nn * irhs, sizeof(T) * nn,
                              cudaMemcpyHostToDevice, cs));
    if (J.block) {
      IDRS_CUDA(cudaMemsetAsync(db.p, 0, sizeof(T) * n, cs));
      axpy<T>(nn, T(-1.0), drhs.template as<T>(), db.template as<T>(), cs);
    } else {
      IDRS_CUDA(cudaMemcpyAsync(db.p, drhs.p, sizeof(T) * nn, cudaMemcpyDeviceToDevice, cs));
    }
  };
  load_rhs(0);
  idrs_pp_report base{};
  st = pp_setup<T>(J, db.template as<T>(), center, foci, opt, base);
  if (st) return st;
  st = pp_deflate<T>(J, in);
  if (st) return st;
  IDRS_CUDA(cudaStreamSynchronize(cs));
  auto t1 = clk::now();
  const double setup = std::chrono::duration<double>(t1 - t0).count();
  constexpr int vw = kCplx<T> ? 2 : 1;
  std::vector<double> sp((size_t)vw * n_sigma);
  st = ms_parameters(J.A, n_sigma, sigma, sp.data(), kCplx<T>);
  if (st) return st;
  const double* om = J.omega.empty() ? nullptr : (const double*)J.omega.data();
  const int n_om = (int)J.omega.size();
  for (int irhs = 0; irhs < nrhs; ++irhs) {
    auto ts = clk::now();
    idrs_pp_report rep = base;
    if (irhs > 0) load_rhs(irhs);
    const T* rb = db.template as<T>();
    if (J.A->defl && J.A->defl->k > 0) {
      deflation_pmul<T>(*J.A->defl, db.template as<T>(), J.t1.template as<T>(), T(1.0), T(0.0),
                        nullptr, nullptr, cs);
      rb = J.t1.template as<T>();
    }
    double tol = opt->tol;
    int maxit = opt->maxit;
    std::vector<double> rel(n_sigma, 1.0);
    if (opt->method == 0) {
      int in_s = opt->in_s, in_it = opt->in_it, prec = opt->inner_precision ? opt->inner_precision : 64;
      double in_tol = opt->in_tol;
      st = run_msqmridr<T, typename std::conditional<kCplx<T>, c64, float>::type>(
          J.A, (const double*)rb, n_sigma, sp.data(), opt->s, nullptr, &tol, &maxit, &rep.flag,
          rel.data(), &rep.iterations, &in_s, &in_tol, &in_it, om, n_om, nullptr, 0, &prec,
          (double*)dY.template as<T>());
    } else {
      int variant = opt->method == 2 ? 2 : 1;
      st = run_msidrs<T>(J.A, (const double*)rb, n_sigma, sp.data(), opt->s, nullptr, &tol, &maxit,
                         &variant, &rep.flag, rel.data(), &rep.iterations, om, n_om, nullptr, 0,
                         nullptr, (double*)dY.template as<T>());
    }
    if (st) return st;
    rep.relres_solver = *std::max_element(rel.begin(), rel.end());
    st = ms_scaleback_t<T>(J.A, n_sigma, sigma, (const double*)(sequence ? rb : db.template as<T>()),
                           (const double*)dY.template as<T>(), (double*)dX.template as<T>());
    if (st) return st;
    double worst = 0;
    for (int k = 0; k < n_sigma; ++k) {
      const T* sol = dX.template as<T>() + (size_t)n * k + (J.block ? nn : 0);
      const c128 sg = kCplx<T> ? c128(sigma[2 * k], sigma[2 * k + 1]) : c128(sigma[k], 0.0);
      const double rr = ms_true_relres<T>(J, K, in, sg, drhs.template as<T>(), sol,
                                          J.r.template as<T>(), du.template as<T>());
      if (relres_sigma) relres_sigma[k + (size_t)n_sigma * irhs] = rr;
      worst = std::max(worst, rr);
      IDRS_CUDA(cudaMemcpyAsync((T*)x + (size_t)nn * (k + (size_t)n_sigma * irhs), sol, sizeof(T) * nn,
                                cudaMemcpyDeviceToHost, cs));
    }
    IDRS_CUDA(cudaStreamSynchronize(cs));
    rep.relres_original = worst;
    auto te = clk::now();
    rep.seconds_setup = setup;
    rep.seconds_solve = std::chrono::duration<double>(te - ts).count();
    rep.seconds_total = std::chrono::duration<double>(te - t0).count();
    no_fp64_check(rep);  // the multishift pipelines have no built-in check
    if (reports) reports[irhs] = rep;
  }
  return IDRS_OK;
}

}  // namespace

extern "C" {

int idrs_rpp_idrs_ext(idrs_user_matrix K, const double* b, idrs_user_matrix P, const double* center,
                      const double* foci, const idrs_pp_inputs* in, const idrs_pp_options* opt,
                      idrs_pp_report* report, double* x) {
  return guard([&] { return pp_idrs_t<double>(K, b, P, center, foci, in, opt, report, x); });
}
int idrs_cpp_idrs(idrs_user_matrix K, const double* b, idrs_user_matrix P, const double* center,
                  const double* foci, const idrs_pp_inputs* in, const idrs_pp_options* opt,
                  idrs_pp_report* report, double* x) {
  return guard([&] { return pp_idrs_t<c128>(K, b, P, center, foci, in, opt, report, x); });
}
int idrs_rpp_mr_idrs_ext(idrs_user_matrix K, int nrhs, const double* b_all, idrs_user_matrix P,
                         const double* center, const double* foci, const idrs_pp_inputs* in,
                         const idrs_pp_options* opt, idrs_pp_report* reports, double* x_all) {
  return guard([&] { return pp_mr_idrs_t<double>(K, nrhs, b_all, P, center, foci, in, opt, reports, x_all); });
}
int idrs_cpp_mr_idrs(idrs_user_matrix K, int nrhs, const double* b_all, idrs_user_matrix P,
                     const double* center, const double* foci, const idrs_pp_inputs* in,
                     const idrs_pp_options* opt, idrs_pp_report* reports, double* x_all) {
  return guard([&] { return pp_mr_idrs_t<c128>(K, nrhs, b_all, P, center, foci, in, opt, reports, x_all); });
}
int idrs_rpp_ms_idrs(idrs_user_matrix K, const double* rhs, int n_sigma, const double* sigma,
                     idrs_user_matrix P, const double* center, const double* foci,
                     const idrs_pp_inputs* in, const idrs_pp_options* opt, idrs_pp_report* report,
                     double* relres, double* x) {
  return guard([&] {
    return pp_ms_t<double>(K, 1, rhs, n_sigma, sigma, P, center, foci, in, opt, report, relres, x, false);
  });
}
int idrs_cpp_ms_idrs(idrs_user_matrix K, const double* rhs, int n_sigma, const double* sigma,
                     idrs_user_matrix P, const double* center, const double* foci,
                     const idrs_pp_inputs* in, const idrs_pp_options* opt, idrs_pp_report* report,
                     double* relres, double* x) {
  return guard([&] {
    return pp_ms_t<c128>(K, 1, rhs, n_sigma, sigma, P, center, foci, in, opt, report, relres, x, false);
  });
}
int idrs_rpp_ms_mr_idrs(idrs_user_matrix K, int nrhs, const double* rhs, int n_sigma,
                        const double* sigma, idrs_user_matrix P, const double* center,
                        const double* foci, const idrs_pp_inputs* in, const idrs_pp_options* opt,
                        idrs_pp_report* reports, double* relres, double* x) {
  return guard([&] {
    return pp_ms_t<double>(K, nrhs, rhs, n_sigma, sigma, P, center, foci, in, opt, reports, relres, x, true);
  });
}
int idrs_cpp_ms_mr_idrs(idrs_user_matrix K, int nrhs, const double* rhs, int n_sigma,
                        const double* sigma, idrs_user_matrix P, const double* center,
                        const double* foci, const idrs_pp_inputs* in, const idrs_pp_options* opt,
                        idrs_pp_report* reports, double* relres, double* x) {
  return guard([&] {
    return pp_ms_t<c128>(K, nrhs, rhs, n_sigma, sigma, P, center, foci, in, opt, reports, relres, x, true);
  });
}

}  // extern "C"
