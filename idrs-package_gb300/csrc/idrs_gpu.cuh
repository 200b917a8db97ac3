// idrs_gpu.cuh -- IDR(s) and QMRIDR(s) on the device.
//
// The host code mirrors the control flow of M/IDRS/idrs.inc and
// M/IDRS/qmridr.inc, but it never waits for a scalar: each vector pass is one
// fused kernel whose last block runs the reference's scalar work (the tails
// below) on the device and writes the coefficients of the next pass into the
// solver state.  The host enqueues whole cycles ahead and polls the device's
// stop flag one cycle behind (pinned memory + event), so the GPU never idles
// on a round trip.  Kernels launched after the solver stopped return at once.
#pragma once

#include <algorithm>
#include <vector>

#include "fused.cuh"
#include "matrix.cuh"

namespace idrs {

constexpr int MAXS = 16;  // largest shadow-space dimension of the GPU path

// Literal constants of the reference: default-real literals widened to
// real64 (e.g. `tol = 1e-6`, `kappa = 0.7`, `om = sqrt(2.)`).
constexpr double kDefaultTol = (double)1e-6f;
constexpr double kKappa = (double)0.7f;
constexpr double kInnerTolDefault = (double)1.e-1f;
constexpr double kDblMin = 2.2250738585072014e-308;  // tiny(1._rp)
constexpr double kDblEps = 2.220446049250313e-16;    // epsilon(1._rp)

__host__ __device__ inline double sqrt_default_real(int k) { return (double)sqrtf((float)k); }

template <class W> __device__ inline W wdiv(W a, W b) { return a / b; }

// ---------------------------------------------------------------------------
// solver states (device memory)
// ---------------------------------------------------------------------------
template <class W>
struct IdrsState {
  int info, stop, early, iter, ii, jj, maxit, method, s, out_H, nritz, n_omega;
  // x += beta_k U_k of the steps of the current cycle is deferred to the
  // omega step's pass: xpend steps are pending (xdone = 1 when none are)
  int xpend, xdone;
  double tol, tolb, normb, normr, kappa, relres, rho;
  W om;
  W M[MAXS * MAXS];
  W f[MAXS], mu[MAXS], alpha[MAXS], beta[MAXS], gamma[MAXS];
  W* H;
  int ldH;
  double* resvec;
  const W* omega;
};

template <class W>
struct QmrState {
  int info, stop, early, iter, jj, maxit, s, n_omega;
  int inner_calls, inner_total, inner_max;  // statistics of the inner solves
  double tol, tolb, normb, normg, normr, kappa, relres;
  W om, phi_n, phi_n1;
  W M[MAXS * MAXS];
  W mu[MAXS], gamma[MAXS], beta[MAXS];
  W c[MAXS + 2], h[MAXS + 2], rs[MAXS + 3], cs[MAXS + 2], sn[MAXS + 2];
  double* resvec;
  const W* omega;
};

// Options of one solve (device pointers; NULL == not present).
struct SolveOpts {
  double tol = kDefaultTol;
  int maxit = -1;         // -1: min(2n, 1000)
  int method = 1;         // idrs variant
  Operator* M1 = nullptr; // preconditioner "v/M1" (diagonal) or null
  const void* x0 = nullptr;
  const void* U0 = nullptr;
  const void* omega = nullptr;
  int n_omega = 0;
  double* resvec = nullptr;
  int resvec_len = 0;
  void* H = nullptr;
  int ldH = 0, nritz = 0;
  const void* PT = nullptr;  // injected shadow space (device, wide type, s x n)
  uint64_t p_seed = 1;
  // QMRIDR
  int in_s = 4, in_it = 0, in_prec = 64;
  double in_tol = kInnerTolDefault;
  // inner-solver mode
  bool inner = false;
  const int* outer_stop = nullptr;
};

// ---------------------------------------------------------------------------
// generic bodies
// ---------------------------------------------------------------------------

// r = b (optional copy), x = 0 (optional); acc0 = |b|^2, acc1 = |r|^2
template <class T>
struct BInit {
  const T* b; T* r; T* x; bool copy, zero_x;
  using Shared = NoShared;
  __device__ void prepare(Shared&) const {}
  template <int ND, class A>
  __device__ void operator()(long i, Shared&, A (&acc)[ND]) const {
    T bi = b[i];
    T ri = copy ? bi : r[i];
    if (copy) r[i] = ri;
    if (zero_x) x[i] = T(0);
    acc_add(acc[0], abs2_(bi));
    acc_add(acc[1], abs2_(ri));
  }
};

// acc_d = sum_i PT_d[i] * w[i]   (matmul(PT, w), no conjugation)
template <class T>
struct BPdot {
  const T* PT; long ld; const T* w; int nd;
  using Shared = NoShared;
  static constexpr bool kPack = true;
  bool pack_ok() const { return aligned_f4(PT) && aligned_f4(w) && ld % 4 == 0; }
  __device__ void prepare(Shared&) const {}
  template <int W, int ND, class A>
  __device__ void run(long i, Shared&, A (&acc)[ND]) const {
    const Pk<T, W> wi = pk_ld<W>(w, i);
#pragma unroll
    for (int d = 0; d < ND; ++d)
      if (d < nd) pk_acc_mul(acc[d], pk_ld<W>(PT + d * ld, i), wi);
  }
};

// acc0 = |w|^2
template <class T>
struct BNorm {
  const T* w;
  using Shared = NoShared;
  __device__ void prepare(Shared&) const {}
  template <int ND, class A>
  __device__ void operator()(long i, Shared&, A (&acc)[ND]) const { acc_add(acc[0], abs2_(w[i])); }
};

// COMP_OM dots: acc0 = (t,r) = sum conj(t) r, acc1 = (t,t), acc2 = (r,r)
template <class T>
struct BOmDots {
  const T* t; const T* r;
  using Shared = NoShared;
  static constexpr bool kPack = true;
  bool pack_ok() const { return aligned_f4(t) && aligned_f4(r); }
  __device__ void prepare(Shared&) const {}
  template <int W, int ND, class A>
  __device__ void run(long i, Shared&, A (&acc)[ND]) const {
    const Pk<T, W> ti = pk_ld<W>(t, i), ri = pk_ld<W>(r, i);
    pk_acc_dot(acc[0], ti, ri);
    pk_acc_abs2(acc[1], ti);
    pk_acc_abs2(acc[2], ri);
  }
};

// ---------------------------------------------------------------------------
// shadow space: MAKE_P (idrs_module.f90:839-937) on the device
// ---------------------------------------------------------------------------
template <class T>
__global__ void k_gen_p(long n, int rows, uint64_t seed, T* PT, long ld) {
  long tot = (long)rows * n;
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < tot; q += gridDim.x * (long)blockDim.x) {
    long i = q / rows;
    int j = (int)(q - i * rows);
    uint64_t k = (uint64_t)i * (uint64_t)rows + (uint64_t)j;
    double re = uniform01(seed, k);
    if constexpr (traits<T>::is_cplx) {
      double im = uniform01(seed, (uint64_t)rows * (uint64_t)n + k);
      PT[j * ld + i] = narrow<T>(c128(re, im));
    } else {
      PT[j * ld + i] = narrow<T>(re);
    }
  }
}

// acc_q = dot_product(P_q, P_j) = sum conj(P_q) P_j, q < j
template <class T>
struct BGsDots {
  const T* PT; long ld; int j;
  using Shared = NoShared;
  __device__ void prepare(Shared&) const {}
  template <int ND, class A>
  __device__ void operator()(long i, Shared&, A (&acc)[ND]) const {
    T pj = PT[j * ld + i];
#pragma unroll
    for (int d = 0; d < ND; ++d)
      if (d < j) acc_add(acc[d], conj_(PT[d * ld + i]) * pj);
  }
};

template <class T, class W>
struct BGsUpd {
  T* PT; long ld; int j; const W* alpha;
  struct Shared { T a[MAXS]; };
  __device__ void prepare(Shared& sh) const {
    for (int q = threadIdx.x; q < j; q += blockDim.x) sh.a[q] = narrow<T>(alpha[q]);
  }
  template <int ND, class A>
  __device__ void operator()(long i, Shared& sh, A (&acc)[ND]) const {
    T p = PT[j * ld + i];
    for (int q = 0; q < j; ++q) p = p - sh.a[q] * PT[q * ld + i];
    PT[j * ld + i] = p;
    acc_add(acc[0], abs2_(p));
  }
};

// p /= rho as a multiplication by the reciprocal (one FP64 division per
// thread instead of one per element: GB300's FP64 division is a sequence of
// FP64 instructions; the row changes by at most 1 ulp)
template <class T>
__global__ void k_div_row(long n, T* p, const double* rho, bool conj_it) {
  const auto inv = narrow<typename traits<T>::real>(1.0 / *rho);
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (long)blockDim.x) {
    T v = p[i] * inv;
    p[i] = conj_it ? conj_(v) : v;
  }
}
template <class T>
__global__ void k_conj_copy(long n, const T* a, T* b) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (long)blockDim.x) b[i] = conj_(a[i]);
}

template <class W> struct TStoreAlpha {
  W* alpha; int cnt;
  __device__ void operator()(const W* v) const {
    for (int q = 0; q < cnt; ++q) alpha[q] = v[q];
  }
};
struct TStoreRho {
  double* rho;
  template <class W> __device__ void operator()(const W* v) const { *rho = sqrt(real_(v[0])); }
};

// Generates and orthonormalises the shadow space PT (rows x n, row j at
// PT + j*ld) in the precision of T.  method 1: s random orthonormal rows;
// 2: conj(r); 3/4: one random normalised row (stored conjugated so that the
// unconjugated P-dot kernel computes dot_product(PT(1,:), w)).
template <class T, class W>
void make_shadow(int method, int rows, long n, uint64_t seed, const T* r, T* PT, long ld,
                 W* alpha_scratch, double* rho_scratch, RedBuf rb, cudaStream_t st) {
  if (method == 2) {
    k_conj_copy<T><<<stream_grid(n), kThreads, 0, st>>>(n, r, PT);
    IDRS_LAUNCH_CHECK();
    return;
  }
  k_gen_p<T><<<stream_grid((long)rows * n), kThreads, 0, st>>>(n, rows, seed, PT, ld);
  IDRS_LAUNCH_CHECK();
  for (int j = 0; j < rows; ++j) {
    if (j > 0) launch_fused_nd<T>(j, n, BGsDots<T>{PT, ld, j}, TStoreAlpha<W>{alpha_scratch, j}, rb, nullptr, st);
    launch_fused<1, T>(n, BGsUpd<T, W>{PT, ld, j, alpha_scratch}, TStoreRho{rho_scratch}, rb, nullptr, st);
    bool conj_it = (method >= 3) && traits<T>::is_cplx;
    k_div_row<T><<<stream_grid(n), kThreads, 0, st>>>(n, PT + j * ld, rho_scratch, conj_it);
    IDRS_LAUNCH_CHECK();
  }
}

// ---------------------------------------------------------------------------
// IDR(s) bodies and tails (idrs.inc:140-301)
// ---------------------------------------------------------------------------
template <class T, class W>
struct BBuildU {  // U_k = om*(r - sum_{q>=k} g_q G_q) + sum_{q>=k} g_q U_q   (idrs.inc:159-177)
  const T* r; const T* G; T* U; long ld; int k, s; const IdrsState<W>* st; T* vout;
  struct Shared { T g[MAXS]; T om; };
  __device__ void prepare(Shared& sh) const {
    for (int q = threadIdx.x; q < s; q += blockDim.x) sh.g[q] = narrow<T>(st->gamma[q]);
    if (threadIdx.x == 0) sh.om = narrow<T>(st->om);
  }
  static constexpr bool kPack = true;
  bool pack_ok() const {
    return aligned_f4(r) && aligned_f4(G) && aligned_f4(U) && (!vout || aligned_f4(vout)) && ld % 4 == 0;
  }
  template <int L, int ND, class A>
  __device__ void run(long i, Shared& sh, A (&)[ND]) const {
    Pk<T, L> v = pk_ld<L>(r, i);
#pragma unroll 4
    for (int q = k; q < s; ++q) v = pk_msub(v, sh.g[q], pk_ld<L>(G + q * ld, i));
    if (vout) { pk_st<L>(vout, i, v); return; }  // preconditioned variant: v only
    Pk<T, L> t = pk_scale(sh.om, v);
#pragma unroll 4
    for (int q = k; q < s; ++q) t = pk_madd(t, sh.g[q], pk_ld<L>(U + q * ld, i));
    pk_st<L>(U + k * ld, i, t);
  }
};
template <class T, class W>
struct BCombineU {  // U_k = om*t + sum_{q>=k} g_q U_q  (t = v/M1)
  const T* t; T* U; long ld; int k, s; const IdrsState<W>* st;
  struct Shared { T g[MAXS]; T om; };
  __device__ void prepare(Shared& sh) const {
    for (int q = threadIdx.x; q < s; q += blockDim.x) sh.g[q] = narrow<T>(st->gamma[q]);
    if (threadIdx.x == 0) sh.om = narrow<T>(st->om);
  }
  template <int ND, class A>
  __device__ void operator()(long i, Shared& sh, A (&)[ND]) const {
    T u = sh.om * t[i];
    for (int q = k; q < s; ++q) u = u + sh.g[q] * U[q * ld + i];
    U[k * ld + i] = u;
  }
};

template <class T, class W>
struct BIdrUpd {  // bi-orthogonalise G_k,U_k; r -= beta G_k; acc0 = |r|^2 (x += beta U_k: BOmUpd / BXFlush)
  T* G; T* U; long ld; int k; T* r; const IdrsState<W>* st;
  struct Shared { T a[MAXS]; T beta; };
  __device__ void prepare(Shared& sh) const {
    for (int q = threadIdx.x; q < k; q += blockDim.x) sh.a[q] = narrow<T>(st->alpha[q]);
    if (threadIdx.x == 0) sh.beta = narrow<T>(st->beta[k]);
  }
  static constexpr bool kPack = true;
  bool pack_ok() const { return aligned_f4(G) && aligned_f4(U) && aligned_f4(r) && ld % 4 == 0; }
  template <int L, int ND, class A>
  __device__ void run(long i, Shared& sh, A (&acc)[ND]) const {
    Pk<T, L> g = pk_ld<L>(G + k * ld, i);
    if (k > 0) {  // step 0 has nothing to orthogonalise against: G_0, U_0 stay as they are
      Pk<T, L> u = pk_ld<L>(U + k * ld, i);
#pragma unroll 4
      for (int q = 0; q < k; ++q) {
        g = pk_msub(g, sh.a[q], pk_ld<L>(G + q * ld, i));
        u = pk_msub(u, sh.a[q], pk_ld<L>(U + q * ld, i));
      }
      pk_st<L>(G + k * ld, i, g);
      pk_st<L>(U + k * ld, i, u);
    }
    const Pk<T, L> rr = pk_msub(pk_ld<L>(r, i), sh.beta, g);
    pk_st<L>(r, i, rr);
    pk_acc_abs2(acc[0], rr);
  }
};

// x += beta_q U_q for the q < n pending steps, in step order (so x is rounded
// exactly as if each step had updated it)
template <class T, class W>
struct XPending {
  T b[MAXS];
  int n;
  __device__ void load(const IdrsState<W>* st, int nmax) {
    if (threadIdx.x == 0) n = min(st->xpend, nmax);
    for (int q = threadIdx.x; q < nmax; q += blockDim.x) b[q] = narrow<T>(st->beta[q]);
  }
};
template <int L, class T, class W>
__device__ __forceinline__ Pk<T, L> x_pending(Pk<T, L> xi, const XPending<T, W>& p, const T* U, long ld, long i) {
  for (int q = 0; q < p.n; ++q) xi = pk_madd(xi, p.b[q], pk_ld<L>(U + q * ld, i));
  return xi;
}

template <class T, class W>
struct BXFlush {  // the deferred x += beta_q U_q of a cycle the solve stopped in
  T* x; const T* U; long ld; int s; const IdrsState<W>* st;
  struct Shared { XPending<T, W> p; };
  __device__ void prepare(Shared& sh) const { sh.p.load(st, s); }
  static constexpr bool kPack = true;
  bool pack_ok() const { return aligned_f4(x) && aligned_f4(U) && ld % 4 == 0; }
  template <int L, int ND, class A>
  __device__ void run(long i, Shared& sh, A (&)[ND]) const {
    pk_st<L>(x, i, x_pending<L>(pk_ld<L>(x, i), sh.p, U, ld, i));
  }
};

template <class T, class W>
struct BOmUpd {  // r -= om t; x += beta_q U_q (the cycle's steps) + om v; acc0 = |r|^2, acc_{1+j} = PT_j . r
  T* r; const T* t; T* x; const T* v; const T* PT; long ld; int s; const W* om; const T* U;
  const IdrsState<W>* st;
  struct Shared { T om; XPending<T, W> p; };
  static constexpr bool kPack = true;
  bool pack_ok() const {
    return aligned_f4(r) && aligned_f4(t) && aligned_f4(x) && aligned_f4(v) && aligned_f4(PT) &&
           aligned_f4(U) && ld % 4 == 0;
  }
  __device__ void prepare(Shared& sh) const {
    if (threadIdx.x == 0) sh.om = narrow<T>(*om);
    sh.p.load(st, s);
  }
  template <int L, int ND, class A>
  __device__ void run(long i, Shared& sh, A (&acc)[ND]) const {
    const Pk<T, L> vi = pk_ld<L>(v, i);
    const Pk<T, L> ri = pk_msub(pk_ld<L>(r, i), sh.om, pk_ld<L>(t, i));
    pk_st<L>(x, i, pk_madd(x_pending<L>(pk_ld<L>(x, i), sh.p, U, ld, i), sh.om, vi));
    pk_st<L>(r, i, ri);
    pk_acc_abs2(acc[0], ri);
#pragma unroll
    for (int d = 1; d < ND; ++d)
      if (d <= s) pk_acc_mul(acc[d], pk_ld<L>(PT + (d - 1) * ld, i), ri);
  }
};

template <class W>
__device__ inline W& Mat(W* M, int i, int j) { return M[i + MAXS * j]; }
template <class W>
__device__ inline W& H1(W* H, int ld, int i1, int j1) { return H[(i1 - 1) + (long)ld * (j1 - 1)]; }

// gamma for steps k..s-1 (0-based): lower-triangular solve of idrs.inc:159-164
template <class W>
__device__ inline void idrs_gamma(IdrsState<W>* st, int k) {
  int s = st->s;
  for (int i = k; i < s; ++i) {
    W g = st->f[i];
    for (int j = k; j < i; ++j) g = g - Mat(st->M, i, j) * st->gamma[j];
    st->gamma[i] = g / Mat(st->M, i, i);
  }
}

template <class W> struct TIdrsInit {
  IdrsState<W>* st;
  __device__ void operator()(const W* v) const {
    st->normb = sqrt(real_(v[0]));
    st->tolb = st->tol * st->normb;
    st->normr = sqrt(real_(v[1]));
    if (st->resvec) st->resvec[0] = st->normr;
    if (st->normr <= st->tolb) {
      st->info = 0; st->iter = 0; st->relres = st->normr / st->normb;
      st->early = 1; st->stop = 1;
    }
  }
};
template <class W> struct TIdrsF0 {
  IdrsState<W>* st;
  __device__ void operator()(const W* v) const { for (int j = 0; j < st->s; ++j) st->f[j] = v[j]; }
};
template <class W> struct TIdrsMu {  // idrs.inc:152 + 179-222
  IdrsState<W>* st; int k;
  __device__ void operator()(const W* v) const {
    const int s = st->s;
    st->ii += 1;
    const int ii = st->ii;
    const bool hh = st->out_H && ii <= st->nritz;
    if (st->jj > 0 && hh)
      for (int q = k; q < s; ++q) H1(st->H, st->ldH, ii - s + (q - k), ii) = -st->gamma[q] / st->beta[q];
    W mu[MAXS];
    for (int j = 0; j < s; ++j) mu[j] = v[j];
    for (int i = 0; i < k; ++i) {
      W a = mu[i];
      for (int j = 0; j < i; ++j) a = a - Mat(st->M, i, j) * st->alpha[j];
      a = a / Mat(st->M, i, i);
      st->alpha[i] = a;
      for (int q = k; q < s; ++q) mu[q] = mu[q] - Mat(st->M, q, i) * a;
    }
    for (int q = k; q < s; ++q) Mat(st->M, q, k) = mu[q];
    if (hh && k > 0)
      for (int i = 0; i < k; ++i) H1(st->H, st->ldH, ii - k + i, ii) = st->alpha[i] / st->beta[i];
    if (abs_(Mat(st->M, k, k)) <= kDblMin) { st->info = 3; st->stop = 1; return; }
    st->beta[k] = st->f[k] / Mat(st->M, k, k);
  }
};
template <class W> struct TIdrsNorm {  // idrs.inc:226-249
  IdrsState<W>* st; int k;
  __device__ void operator()(const W* v) const {
    const int s = st->s;
    st->xpend = k + 1;  // x += beta_q U_q, q <= k, still to come
    st->xdone = 0;
    if (k < s - 1)
      for (int q = k + 1; q < s; ++q) st->f[q] = st->f[q] - st->beta[k] * Mat(st->M, q, k);
    const int ii = st->ii;
    if (st->out_H && ii <= st->nritz) {
      H1(st->H, st->ldH, ii, ii) = W(1.0) / st->beta[k];
      int l = max(1, ii - s);
      for (int q = ii + 1; q >= l + 1; --q) H1(st->H, st->ldH, q, ii) = H1(st->H, st->ldH, q, ii) - H1(st->H, st->ldH, q - 1, ii);
      for (int q = l; q <= ii + 1; ++q) H1(st->H, st->ldH, q, ii) = H1(st->H, st->ldH, q, ii) / st->om;
    }
    st->normr = sqrt(real_(v[0]));
    st->iter += 1;
    if (st->resvec) st->resvec[st->iter] = st->normr;
    if (st->normr < st->tolb) { st->info = 0; st->stop = 1; return; }
    if (st->iter == st->maxit) { st->info = 1; st->stop = 1; return; }
    if (k < s - 1 && st->jj > 0) idrs_gamma(st, k + 1);
  }
};
template <class W> struct TIdrsOm {  // idrs.inc:260, 273-284 with COMP_OM idrs_module.f90:719-785
  IdrsState<W>* st;
  __device__ void operator()(const W* v) const {
    st->jj += 1;
    W om;
    if (st->n_omega > 0) {
      int i = st->jj % st->n_omega;
      if (i == 0) i = st->n_omega;
      om = st->omega[i - 1];
    } else if (st->kappa == 0.0) {
      om = v[0] / v[1];
    } else {
      W b1 = v[2], b2 = v[1], b3 = v[0];
      double rho = abs_(b3) / sqrt(abs_(b1 * b2));
      om = b3 / b2;
      if (rho < st->kappa) om = om * W(st->kappa) / W(rho);
    }
    st->om = om;
    if (abs_(om) <= kDblEps) { st->info = 3; st->stop = 1; }
  }
};
template <class W> struct TIdrsNormOm {  // idrs.inc:291-299, then f = P_DOT of the next cycle
  IdrsState<W>* st;
  __device__ void operator()(const W* v) const {
    st->xpend = 0;  // BOmUpd applied the cycle's x updates
    st->xdone = 1;
    st->normr = sqrt(real_(v[0]));
    st->iter += 1;
    if (st->resvec) st->resvec[st->iter] = st->normr;
    if (st->normr < st->tolb) { st->info = 0; st->stop = 1; return; }
    if (st->iter == st->maxit) { st->info = 1; st->stop = 1; return; }
    for (int j = 0; j < st->s; ++j) st->f[j] = v[1 + j];
    idrs_gamma(st, 0);
  }
};
template <class W> struct TIdrsFinal {  // idrs.inc:304-310
  IdrsState<W>* st;
  __device__ void operator()(const W* v) const {
    st->normr = sqrt(real_(v[0]));
    if (st->info == 0 && st->normr > st->tolb) st->info = 2;
    st->relres = st->normr / st->normb;
  }
};

template <class W>
__global__ void k_idrs_state_init(IdrsState<W>* st, IdrsState<W> init, const int* outer_stop) {
  if (outer_stop && *(volatile const int*)outer_stop) return;
  *st = init;
}
template <class W>
__global__ void k_set_stop(int* stop) { *stop = 1; }
// after BXFlush: no x update is pending any more
template <class W>
__global__ void k_xflush_done(IdrsState<W>* st) {
  st->xpend = 0;
  st->xdone = 1;
}

// ---------------------------------------------------------------------------
// IDR(s) driver
// ---------------------------------------------------------------------------
template <class T>
class IdrsGpu {
 public:
  using W = typename traits<T>::wide;
  IdrsGpu(Operator& A, int prec, int s, int method);
  ~IdrsGpu();
  // Enqueue one solve of A x = b (device pointers).  In inner mode nothing
  // waits on the host and the final true residual is omitted (it only sets
  // the flag, which the outer method never reads).
  void solve(const T* b, T* x, const SolveOpts& o);
  // Copy the device state back (after the stream was synchronised).
  IdrsState<W> state();

  Operator& A;
  int prec, s, rows, method;
  long n;
  cudaStream_t st;
  RedBuf rb;
  T *G = nullptr, *U = nullptr, *r = nullptr, *v = nullptr, *t = nullptr, *t1 = nullptr, *t2 = nullptr,
    *t3 = nullptr, *t4 = nullptr, *PT = nullptr;
  IdrsState<W>* d_st = nullptr;
  int* h_stop = nullptr;  // pinned, 2 slots
  cudaEvent_t ev[2];
  // the cycles after the first one, captured once per solve and replayed;
  // an inner solver keeps the graph for the next inner solve into the same x
  // (its operator and work vectors do not change during the outer solve)
  cudaGraphExec_t cycle_graph = nullptr;
  long cycle_launches = 0;
  const T* graph_x = nullptr;
  bool p_ready = false;
  const void* p_injected = nullptr;

 private:
  void enqueue_cycle(const T* b, T* x, const SolveOpts& o, int cycle, bool inispace);
  bool capture_cycle(const T* b, T* x, const SolveOpts& o, bool inispace);
  void matvec(const T* in, T* out, const int* skip, T fa = T(1), T fcv = T(0), const T* fv = nullptr);
};

// ---------------------------------------------------------------------------
// QMRIDR(s) bodies and tails (qmridr.inc:129-254)
// ---------------------------------------------------------------------------
template <class T, class W, class S = QmrState<W>>
struct BQv {  // v = gn - sum_i gamma_i G_i (logical G_1..G_s)
  const T* gn; const T* pool; long ld; int gmap[MAXS]; int s; T* v; const S* st;
  struct Shared { T g[MAXS]; };
  __device__ void prepare(Shared& sh) const {
    for (int q = threadIdx.x; q < s; q += blockDim.x) sh.g[q] = narrow<T>(st->gamma[q]);
  }
  template <int ND, class A>
  __device__ void operator()(long i, Shared& sh, A (&)[ND]) const {
    T vv = gn[i];
    for (int q = 0; q < s; ++q) vv = vv - sh.g[q] * pool[gmap[q] * ld + i];
    v[i] = vv;
  }
};

// One modified Gram-Schmidt pass: gn' = gn - c*y (c = 1/om on y = v with a
// division, or beta_prev on y = G_prev); acc0 = (G_next, gn') or |gn'|^2.
template <class T, class W, class S = QmrState<W>>
struct BMgs {
  T* gn; const T* y; const T* gnext; bool div_by_om; int prev; const S* st;
  struct Shared { T c; };
  __device__ void prepare(Shared& sh) const {
    // v/om as v*(1/om): one FP64 multiply per element instead of a division
    if (threadIdx.x == 0) sh.c = div_by_om ? narrow<T>(W(1.0) / st->om) : narrow<T>(st->beta[prev]);
  }
  template <int ND, class A>
  __device__ void operator()(long i, Shared& sh, A (&acc)[ND]) const {
    T g = gn[i] - y[i] * sh.c;
    gn[i] = g;
    if (gnext) acc_add(acc[0], conj_(gnext[i]) * g);
    else acc_add(acc[0], abs2_(g));
  }
};

// wn = (vt - W r_sigma(1:s+1)) / r_sigma(s+2) into the evicted W slot;
// x += phi_n wn; gn /= normg; acc_j = PT_j . gn (next iteration's mu)
template <class T, class W>
struct BQw {
  const T* vt; T* wpool; long ld; int wmap[MAXS + 1]; int s; T* x; T* gn; const T* PT; const QmrState<W>* st;
  struct Shared { T rs[MAXS + 1]; T rd; T phi; typename traits<T>::real inorm; };
  __device__ void prepare(Shared& sh) const {
    for (int q = threadIdx.x; q <= s; q += blockDim.x) sh.rs[q] = narrow<T>(st->rs[q]);
    if (threadIdx.x == 0) {
      sh.rd = narrow<T>(W(1.0) / st->rs[s + 1]);  // reciprocals: no per-element divisions
      sh.phi = narrow<T>(st->phi_n);
      sh.inorm = (typename traits<T>::real)(1.0 / st->normg);
    }
  }
  template <int ND, class A>
  __device__ void operator()(long i, Shared& sh, A (&acc)[ND]) const {
    T a = T(0);
    for (int q = 0; q <= s; ++q) a = a + wpool[wmap[q] * ld + i] * sh.rs[q];
    T wn = (vt[i] - a) * sh.rd;
    wpool[wmap[0] * ld + i] = wn;
    x[i] = x[i] + sh.phi * wn;
    T g = gn[i] * sh.inorm;
    gn[i] = g;
#pragma unroll
    for (int d = 0; d < ND; ++d)
      if (d < s) acc_add(acc[d], PT[d * ld + i] * g);
  }
};
// gn /= normg; acc_j = PT_j . gn   (start of the iteration loop)
template <class T, class W, class S = QmrState<W>>
struct BQstart {
  T* gn; const T* PT; long ld; int s; const S* st;
  struct Shared { typename traits<T>::real inorm; };
  __device__ void prepare(Shared& sh) const { if (threadIdx.x == 0) sh.inorm = (typename traits<T>::real)(1.0 / st->normg); }
  template <int ND, class A>
  __device__ void operator()(long i, Shared& sh, A (&acc)[ND]) const {
    T g = gn[i] * sh.inorm;
    gn[i] = g;
#pragma unroll
    for (int d = 0; d < ND; ++d)
      if (d < s) acc_add(acc[d], PT[d * ld + i] * g);
  }
};

// Gaussian elimination with partial pivoting (RSOLVE, dense_la_module.f90:644-681)
template <class W>
__device__ inline void solve_small(int n, const W* M, const W* b, W* x) {
  W A[MAXS * (MAXS + 1)];
#define AA(i, j) A[(i) + MAXS * (j)]
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) AA(i, j) = M[i + MAXS * j];
  for (int i = 0; i < n; ++i) AA(i, n) = b[i];
  for (int j = 0; j < n - 1; ++j) {
    int k = j;
    double best = abs_(AA(j, j));
    for (int i = j + 1; i < n; ++i)
      if (abs_(AA(i, j)) > best) { best = abs_(AA(i, j)); k = i; }
    for (int c = 0; c <= n; ++c) { W t = AA(k, c); AA(k, c) = AA(j, c); AA(j, c) = t; }
    for (int i = j + 1; i < n; ++i) {
      W p = AA(i, j) / AA(j, j);
      for (int c = j + 1; c <= n; ++c) AA(i, c) = AA(i, c) - AA(j, c) * p;
    }
  }
  for (int i = n - 1; i >= 0; --i) {
    W p = AA(i, n);
    for (int j = i + 1; j < n; ++j) p = p - AA(i, j) * AA(j, n);
    AA(i, n) = p / AA(i, i);
  }
  for (int i = 0; i < n; ++i) x[i] = AA(i, n);
#undef AA
}

// GROT (dense_la_module.f90:683-742)
__device__ inline void grot(double a, double b, double& c, double& s, double& r) {
  if (fabs(a) < kDblEps) { c = 0.0; s = 1.0; r = b; }
  else {
    double rho = hypot(fabs(a), fabs(b));
    double alpha = a / fabs(a);
    c = fabs(a) / rho; s = alpha * b / rho; r = alpha * rho;
  }
}
__device__ inline void grot(c128 a, c128 b, c128& c, c128& s, c128& r) {
  if (abs_(a) < kDblEps) { c = c128(0.0); s = c128(1.0); r = b; }
  else {
    double rho = hypot(abs_(a), abs_(b));
    c128 alpha = a / abs_(a);
    c = c128(abs_(a) / rho); s = alpha * conj_(b) / rho; r = alpha * rho;
  }
}

// Start of a QMRIDR iteration (qmridr.inc:134-158): mu in v, iter advanced.
template <class W>
__device__ inline void qmr_prepare(QmrState<W>* st, const W* mu) {
  const int s = st->s;
  st->iter += 1;
  for (int q = 0; q < s + 2; ++q) st->c[q] = W(0.0);
  st->c[s] = W(1.0);
  for (int q = 0; q < s; ++q) st->mu[q] = mu[q];
  if (st->iter > s) {
    solve_small(s, st->M, st->mu, st->gamma);
    for (int q = 0; q < s; ++q) st->c[q] = -st->gamma[q];
  }
  for (int j = 0; j < s - 1; ++j)
    for (int i = 0; i < s; ++i) Mat(st->M, i, j) = Mat(st->M, i, j + 1);
  for (int i = 0; i < s; ++i) Mat(st->M, i, s - 1) = st->mu[i];
}

template <class W> struct TQmrInit {  // qmridr.inc:81-96, 119-120
  QmrState<W>* st;
  __device__ void operator()(const W* v) const {
    st->normb = sqrt(real_(v[0]));
    st->tolb = st->tol * st->normb;
    st->normg = sqrt(real_(v[1]));
    st->normr = st->normg;
    if (st->resvec) st->resvec[0] = st->normr;
    st->phi_n = W(0.0);
    st->phi_n1 = W(st->normg);
    if (st->normg <= st->tolb) {
      st->info = 0; st->iter = 0; st->relres = st->normg / st->normb;
      st->early = 1; st->stop = 1;
    }
  }
};
template <class W> struct TQmrStart {
  QmrState<W>* st;
  __device__ void operator()(const W* v) const { qmr_prepare(st, v); }
};
template <class W> struct TQmrOm {  // qmridr.inc:179-193
  QmrState<W>* st;
  __device__ void operator()(const W* v) const {
    W om;
    if (st->n_omega > 0) {
      int i = st->jj % st->n_omega;
      if (i == 0) i = st->n_omega;
      om = st->omega[i - 1];
    } else {
      W b1 = v[2], b2 = v[1], b3 = v[0];
      double rho = abs_(b3) / sqrt(abs_(b1 * b2));
      om = b3 / b2;
      if (rho < st->kappa) om = om * W(st->kappa) / W(rho);
    }
    st->om = om;
    if (abs_(om) <= kDblEps) { st->info = 3; st->stop = 1; return; }
    st->jj += 1;
  }
};
template <class W> struct TQmrBeta {  // qmridr.inc:197-203, one MGS coefficient
  QmrState<W>* st; int i; bool first;
  __device__ void operator()(const W* v) const {
    const int s = st->s;
    if (first) for (int q = 0; q < s + 2; ++q) st->h[q] = st->c[q] / st->om;
    st->beta[i] = v[0];
    st->h[i + 1] = st->h[i + 1] + v[0];
  }
};
template <class W> struct TQmrNorm {  // qmridr.inc:206-237
  QmrState<W>* st; bool first;
  __device__ void operator()(const W* v) const {
    const int s = st->s;
    if (first) for (int q = 0; q < s + 2; ++q) st->h[q] = st->c[q] / st->om;
    st->normg = sqrt(real_(v[0]));
    st->h[s + 1] = W(st->normg);
    W* rs = st->rs;
    rs[0] = W(0.0);
    for (int q = 0; q < s + 2; ++q) rs[q + 1] = st->h[q];
    int low = max(1, s + 3 - st->iter);
    for (int l = low; l <= s + 1; ++l) {
      W tau = rs[l - 1];
      rs[l - 1] = st->cs[l - 1] * tau + st->sn[l - 1] * rs[l];
      rs[l] = -conj_(st->sn[l - 1]) * tau + st->cs[l - 1] * rs[l];
    }
    W tau = rs[s + 1];
    grot(tau, rs[s + 2], st->cs[s + 1], st->sn[s + 1], rs[s + 1]);
    st->phi_n = st->cs[s + 1] * st->phi_n1;
    st->phi_n1 = -conj_(st->sn[s + 1]) * st->phi_n1;
    for (int q = 0; q < s + 1; ++q) { st->cs[q] = st->cs[q + 1]; st->sn[q] = st->sn[q + 1]; }
    if (abs_(rs[s + 1]) < kDblEps) { st->info = 3; st->stop = 1; }
  }
};
template <class W> struct TQmrW {  // qmridr.inc:243-252, then the next iteration's start
  QmrState<W>* st;
  __device__ void operator()(const W* v) const {
    st->normr = abs_(st->phi_n1) * sqrt_default_real(st->jj + 1);
    if (st->resvec) st->resvec[st->iter] = st->normr;
    if (st->normr < st->tolb) { st->info = 0; st->stop = 1; return; }
    if (st->iter == st->maxit) { st->info = 1; st->stop = 1; return; }
    qmr_prepare(st, v);
  }
};
template <class W> struct TQmrFinal {  // qmridr.inc:256-262
  QmrState<W>* st;
  __device__ void operator()(const W* v) const {
    st->normr = sqrt(real_(v[0]));
    if (st->info == 0 && st->normr >= st->tolb) st->info = 2;
    st->relres = st->normr / st->normb;
  }
};

// adds the iteration count of the inner solve that just ran (skipped once the
// outer solve has stopped: the inner state was not re-initialised then)
template <class W, class Win>
__global__ void k_inner_stats(QmrState<W>* st, const IdrsState<Win>* in) {
  if (st->stop) return;
  st->inner_calls += 1;
  st->inner_total += in->iter;
  st->inner_max = max(st->inner_max, in->iter);
}

template <class T, class Tin>
class QmrGpu {
 public:
  using W = typename traits<T>::wide;
  QmrGpu(Operator& A, int s, const SolveOpts& o);
  ~QmrGpu();
  void solve(const T* b, T* x, const SolveOpts& o);
  QmrState<W> state();

  Operator& A;
  int s;
  long n;
  cudaStream_t st;
  RedBuf rb;
  T *gpool = nullptr, *wpool = nullptr, *v = nullptr, *vt = nullptr, *t1 = nullptr, *t2 = nullptr, *t3 = nullptr,
    *PT = nullptr;
  Tin *v_in = nullptr, *vt_in = nullptr;
  IdrsGpu<Tin>* inner = nullptr;
  QmrState<W>* d_st = nullptr;
  W* d_scratch = nullptr;
  double* d_rho = nullptr;
  int* h_stop = nullptr;
  cudaEvent_t ev[2];
};

}  // namespace idrs
