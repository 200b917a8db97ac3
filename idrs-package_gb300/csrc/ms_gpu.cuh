// ms_gpu.cuh -- multishift IDR(s) (M/IDRS/msidrs.inc) and multishift
// QMRIDR(s) (M/IDRS/msqmridr.inc) on the device.
//
// One Krylov space serves every shift sigma_k.  The per-shift recurrences
// (LU pivots l_sigma, Givens rotations, collinearity factors phi) are scalar
// work done by the tails on the device, and all per-shift vector updates of
// an iteration run in ONE pass over the shared vectors: each element of v,
// v0 (or vtilde) is read once and every shift's W block and solution column
// x(:,k) is updated from it.
//
// The reference tests convergence after its shift loop has updated x, so a
// tail that detects convergence sets `stop_next`; the shift pass still runs
// and the next commit turns stop_next into stop.
#pragma once

#include "idrs_gpu.cuh"

namespace idrs {

constexpr int MAXSIG = 64;  // shifts per solve (inner MSIDRS of MSQMRIDR: n_sigma + 1)

// Scalar options of one multishift solve (kernel argument of the state init).
struct MsArgs {
  int maxit, s, ns, n_omega, ldr, in_it;
  double tol, kappa;
  double* resvec;     // resvec(ldr, ns), column-major, or null
  const void* omega;  // user omegas (wide type) or null
  const void* cf;     // MSQMRIDR: colfac of the inner MSIDRS (wide type, ns + 1)
};

template <class W>
struct MsIdrsState {
  int info, stop, stop_next, early, iter, jj, maxit, s, ns, n_omega, ldr;
  double tol, tolb, normb, normg, kappa, rho;
  W om;
  W M[MAXS * MAXS];
  W f[MAXS], alpha[MAXS], gamma[MAXS], h[MAXS + 3];
  W l_sigma[(MAXS + 2) * MAXSIG];  // column ks: l_sigma(1:s+2, ks)
  W phi[MAXSIG], om_sigma[MAXSIG], sigma[MAXSIG];
  double normr[MAXSIG];
  W cw[(MAXS + 1) * MAXSIG];  // shift pass, per shift: the v0 coefficient, then s W coefficients
  W cinv[MAXSIG], cphi[MAXSIG];
  double* resvec;
  const W* omega;
};

template <class W>
struct MsQmrState {
  int info, stop, stop_next, early, iter, jj, maxit, s, ns, n_omega, ldr, in_it;
  double tol, tolb, normb, normg, kappa;
  W om;
  W M[MAXS * MAXS];
  W mu[MAXS], gamma[MAXS], beta[MAXS], c[MAXS + 2], h[MAXS + 2];
  W sigma[MAXSIG], phi_n[MAXSIG], phi_n1[MAXSIG];
  W cs[(MAXS + 2) * MAXSIG], sn[(MAXS + 2) * MAXSIG];
  W rsw[(MAXS + 1) * MAXSIG];  // shift pass: r_sigma(1:s+1) per shift
  W rinv[MAXSIG];              // 1 / r_sigma(s+2)
  int active[MAXSIG];          // shift updated in this iteration
  int converged[MAXSIG];
  int wbase[MAXSIG];           // slot of W(:,1) in the shift's circular window of s+1
  double normr[MAXSIG];
  double* resvec;
  const W* omega;
  const W* cf;
};

// Zeroes the state with the whole block; thread 0 then sets the options.
// Skipped when an enclosing solve has stopped (the state keeps stop = 1).
template <class S>
__device__ inline bool ms_zero_state(S* st, const int* outer_stop) {
  if (outer_stop && *(volatile const int*)outer_stop) return false;
  unsigned int* p = reinterpret_cast<unsigned int*>(st);
  for (size_t q = threadIdx.x; q < sizeof(S) / sizeof(unsigned int); q += blockDim.x) p[q] = 0u;
  __syncthreads();
  return threadIdx.x == 0;
}

template <class W>
__global__ void k_msidrs_init(MsIdrsState<W>* st, MsArgs a, const W* sigma, const int* outer_stop) {
  if (!ms_zero_state(st, outer_stop)) return;
  st->info = -1;
  st->maxit = a.maxit; st->s = a.s; st->ns = a.ns; st->n_omega = a.n_omega; st->ldr = a.ldr;
  st->tol = a.tol; st->kappa = a.kappa;
  st->resvec = a.resvec;
  st->omega = (const W*)a.omega;
  const W om = W(sqrt_default_real(2));  // om = sqrt(2.) (msidrs.inc:102)
  st->om = om;
  for (int ks = 0; ks < a.ns; ++ks) {
    st->sigma[ks] = sigma[ks];
    st->om_sigma[ks] = om / (W(1.0) - om * sigma[ks]);
    st->phi[ks] = W(1.0);
  }
}

template <class W>
__global__ void k_msqmr_init(MsQmrState<W>* st, MsArgs a, const W* sigma) {
  if (!ms_zero_state(st, nullptr)) return;
  st->info = -1;
  st->maxit = a.maxit; st->s = a.s; st->ns = a.ns; st->n_omega = a.n_omega; st->ldr = a.ldr;
  st->in_it = a.in_it;
  st->tol = a.tol; st->kappa = a.kappa;
  st->resvec = a.resvec;
  st->omega = (const W*)a.omega;
  st->cf = (const W*)a.cf;
  st->om = W(sqrt_default_real(2));
  for (int ks = 0; ks < a.ns; ++ks) st->sigma[ks] = sigma[ks];
}

template <class W>
__device__ inline W& Ls(MsIdrsState<W>* st, int i1, int ks) { return st->l_sigma[(i1 - 1) + (MAXS + 2) * ks]; }

// ================================================================== MSIDRS
// Start of step k (0-based; msidrs.inc:131-150): iter += 1, gamma from the
// lower-triangular M, M(k:s,k) = f(k:s), breakdown test.
template <class W>
__device__ inline void msidrs_prep(MsIdrsState<W>* st, int k) {
  const int s = st->s;
  st->iter += 1;
  if (st->jj > 0) {
    for (int i = k; i < s; ++i) {
      W g = st->f[i];
      for (int j = k; j < i; ++j) g = g - Mat(st->M, i, j) * st->gamma[j];
      st->gamma[i] = g / Mat(st->M, i, i);
    }
  }
  for (int q = k; q < s; ++q) Mat(st->M, q, k) = st->f[q];
  if (abs_(Mat(st->M, k, k)) <= kDblMin) { st->info = 3; st->stop = 1; }
}

template <class W> struct TMsInit {  // msidrs.inc:66-84
  MsIdrsState<W>* st;
  __device__ void operator()(const W* v) const {
    st->normb = sqrt(real_(v[0]));
    st->tolb = st->tol * st->normb;
    st->normg = st->normb;
    for (int ks = 0; ks < st->ns; ++ks) {
      st->normr[ks] = st->normg;
      if (st->resvec) st->resvec[(long)st->ldr * ks] = st->normg;
    }
    if (st->normg <= st->tolb) { st->info = 0; st->iter = 0; st->early = 1; st->stop = 1; }
  }
};

template <class W> struct TMsF0 {  // f = P_DOT(PT, gn) of the first cycle, then step 1's start
  MsIdrsState<W>* st;
  __device__ void operator()(const W* v) const {
    for (int j = 0; j < st->s; ++j) st->f[j] = v[j];
    msidrs_prep(st, 0);
  }
};

// v = gn - sum_{q >= kq} gamma_q G_q   (kq = s in the first cycle: v = gn)
template <class T, class W>
struct BMsV {
  const T* gn; const T* pool; long ld; int gmap[MAXS]; int kq, s; T* v; const MsIdrsState<W>* st;
  struct Shared { T g[MAXS]; };
  __device__ void prepare(Shared& sh) const {
    for (int q = threadIdx.x; q < s; q += blockDim.x) sh.g[q] = narrow<T>(st->gamma[q]);
  }
  template <int ND, class A>
  __device__ void operator()(long i, Shared& sh, A (&)[ND]) const {
    T vv = gn[i];
    for (int q = kq; q < s; ++q) vv = vv - sh.g[q] * pool[gmap[q] * ld + i];
    v[i] = vv;
  }
};

// gn = v - om t; acc = [|gn|^2 when with_norm], PT_j . gn
template <class T, class W>
struct BMsGn {
  const T* v; const T* t; T* gn; const T* PT; long ld; int s; const W* om; bool with_norm;
  struct Shared { T om; };
  __device__ void prepare(Shared& sh) const { if (threadIdx.x == 0) sh.om = narrow<T>(*om); }
  template <int ND, class A>
  __device__ void operator()(long i, Shared& sh, A (&acc)[ND]) const {
    const T g = v[i] - sh.om * t[i];
    gn[i] = g;
    const int o = with_norm ? 1 : 0;
    if (with_norm) acc_add(acc[0], abs2_(g));
#pragma unroll
    for (int d = 0; d < ND; ++d)
      if (d >= o && d < s + o) acc_add(acc[d], PT[(d - o) * ld + i] * g);
  }
};

template <class W> struct TMsAlpha {  // msidrs.inc:166-178, scalar part
  MsIdrsState<W>* st; int k;
  __device__ void operator()(const W* v) const {
    const int s = st->s;
    for (int j = 0; j < s; ++j) st->f[j] = v[j];
    for (int q = 0; q < s; ++q) st->alpha[q] = W(0.0);
    for (int i = 0; i <= k; ++i) {
      W a = st->f[i];
      for (int j = 0; j < i; ++j) a = a - Mat(st->M, i, j) * st->alpha[j];
      a = a / Mat(st->M, i, i);
      st->alpha[i] = a;
      for (int q = k + 1; q < s; ++q) st->f[q] = st->f[q] - Mat(st->M, q, i) * a;
    }
  }
};

// gn -= sum_{q <= k} alpha_q G_q; acc0 = |gn|^2
template <class T, class W>
struct BMsOrth {
  T* gn; const T* pool; long ld; int gmap[MAXS]; int k; const MsIdrsState<W>* st;
  struct Shared { T a[MAXS]; };
  __device__ void prepare(Shared& sh) const {
    for (int q = threadIdx.x; q <= k; q += blockDim.x) sh.a[q] = narrow<T>(st->alpha[q]);
  }
  template <int ND, class A>
  __device__ void operator()(long i, Shared& sh, A (&acc)[ND]) const {
    T g = gn[i];
    for (int q = 0; q <= k; ++q) g = g - pool[gmap[q] * ld + i] * sh.a[q];
    gn[i] = g;
    acc_add(acc[0], abs2_(g));
  }
};

template <class W> struct TMsStep {  // msidrs.inc:179-247: h, every shift's LU update, convergence
  MsIdrsState<W>* st; int k;
  __device__ void operator()(const W* v) const {
    const int s = st->s, ns = st->ns, k1 = k + 1;  // k1: the reference's 1-based k
    st->normg = sqrt(real_(v[0]));
    W* h = st->h;
    for (int q = 0; q < s + 3; ++q) h[q] = W(0.0);
    if (st->jj > 0)
      for (int q = 1; q <= s - k1 + 1; ++q) h[q - 1] = -st->gamma[k1 + q - 2];
    for (int q = 1; q <= k1; ++q) h[s + 2 - k1 + q - 1] = h[s + 2 - k1 + q - 1] - st->alpha[q - 1];
    h[s + 1] = h[s + 1] + W(1.0);
    h[s + 2] = W(-1.0);
    for (int q = 0; q < s + 3; ++q) h[q] = h[q] / st->om;
    double mx = 0.0;
    for (int ks = 0; ks < ns; ++ks) {
      W u[MAXS + 2];
      for (int q = 0; q < s + 2; ++q) u[q] = h[q];
      if (st->jj > 0)
        for (int q = 1; q <= s - k1 + 1; ++q) u[q - 1] = u[q - 1] + st->sigma[ks] * st->gamma[k1 + q - 2];
      u[s + 1] = u[s + 1] - st->sigma[ks];
      for (int q = 1; q <= s + 1; ++q) Ls(st, q, ks) = Ls(st, q + 1, ks);
      for (int j = 2; j <= s + 2; ++j) u[j - 1] = u[j - 1] - Ls(st, j - 1, ks) * u[j - 2];
      Ls(st, s + 2, ks) = W(-1.0) / (st->om * u[s + 1]);
      W* cw = st->cw + (MAXS + 1) * ks;
      cw[0] = st->om_sigma[ks] * u[s + 1 - k1];
      for (int i = 1; i <= s; ++i) cw[i] = (i < k1) ? u[s + 1 - k1 + i] : u[i - k1];
      st->cinv[ks] = W(1.0) / u[s + 1];
      st->cphi[ks] = st->phi[ks];
      st->phi[ks] = -Ls(st, s + 2, ks) * st->phi[ks];
      st->normr[ks] = st->normg * abs_(st->phi[ks]);
      if (st->resvec) st->resvec[st->iter + (long)st->ldr * ks] = st->normr[ks];
      if (st->normr[ks] > mx) mx = st->normr[ks];
    }
    if (mx < st->tolb) { st->info = 0; st->stop_next = 1; }
    else if (st->iter == st->maxit) { st->info = 1; st->stop_next = 1; }
  }
};

// Every shift in one pass: t = v - c0 v0 - sum_i c_i W_i; W_k = t / u(s+2); x += phi W_k
template <class T, class W>
struct BMsShift {
  const T* v; const T* v0; T* Wb; T* x; long ld; int s, ns, k; const MsIdrsState<W>* st;
  struct Shared { T cw[(MAXS + 1) * MAXSIG]; T cinv[MAXSIG]; T cphi[MAXSIG]; };
  __device__ void prepare(Shared& sh) const {
    for (int q = threadIdx.x; q < ns; q += blockDim.x) {
      for (int j = 0; j <= s; ++j) sh.cw[(MAXS + 1) * q + j] = narrow<T>(st->cw[(MAXS + 1) * q + j]);
      sh.cinv[q] = narrow<T>(st->cinv[q]);
      sh.cphi[q] = narrow<T>(st->cphi[q]);
    }
  }
  template <int ND, class A>
  __device__ void operator()(long i, Shared& sh, A (&)[ND]) const {
    const T vi = v[i], v0i = v0[i];
    for (int ks = 0; ks < ns; ++ks) {
      const T* c = sh.cw + (MAXS + 1) * ks;
      T* Wk = Wb + (long)s * ks * ld;
      T t = vi - c[0] * v0i;
      for (int q = 0; q < s; ++q) t = t - Wk[q * ld + i] * c[1 + q];
      const T wk = t * sh.cinv[ks];
      Wk[k * ld + i] = wk;
      x[ks * ld + i] = x[ks * ld + i] + sh.cphi[ks] * wk;
    }
  }
};

// Between steps: commit a detected stop, or prepare step next_k, or (after
// the s steps) advance jj and iter for the omega step (msidrs.inc:255-257).
template <class W>
__global__ void k_msidrs_commit(MsIdrsState<W>* st, int next_k, int end_of_cycle) {
  if (st->stop) return;
  if (st->stop_next) { st->stop = 1; return; }
  if (end_of_cycle) {
    st->jj += 1;
    st->iter += 1;
  } else {
    msidrs_prep(st, next_k);
  }
}

template <class W> struct TMsOm {  // msidrs.inc:262-272 with COMP_OM idrs_module.f90:719-785
  MsIdrsState<W>* st;
  __device__ void operator()(const W* v) const {
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

template <class W> struct TMsGnOm {  // msidrs.inc:274-303; f = P_DOT(gn) of the next cycle
  MsIdrsState<W>* st;
  __device__ void operator()(const W* v) const {
    const int s = st->s, ns = st->ns;
    st->normg = sqrt(real_(v[0]));
    double mx = 0.0;
    for (int ks = 0; ks < ns; ++ks) {
      for (int q = 1; q <= s + 1; ++q) Ls(st, q, ks) = Ls(st, q + 1, ks);
      const W den = W(1.0) - st->om * st->sigma[ks];
      Ls(st, s + 2, ks) = W(-1.0) / den;
      st->om_sigma[ks] = st->om / den;
      st->cphi[ks] = st->phi[ks] * st->om_sigma[ks];
      st->phi[ks] = -Ls(st, s + 2, ks) * st->phi[ks];
      st->normr[ks] = st->normg * abs_(st->phi[ks]);
      if (st->resvec) st->resvec[st->iter + (long)st->ldr * ks] = st->normr[ks];
      if (st->normr[ks] > mx) mx = st->normr[ks];
    }
    for (int j = 0; j < s; ++j) st->f[j] = v[1 + j];
    if (mx < st->tolb) { st->info = 0; st->stop_next = 1; }
    else if (st->iter == st->maxit) { st->info = 1; st->stop_next = 1; }
  }
};

// x(:,ks) += cphi_ks v0 for every shift
template <class T, class W>
struct BMsX {
  const T* v0; T* x; long ld; int ns; const MsIdrsState<W>* st;
  struct Shared { T c[MAXSIG]; };
  __device__ void prepare(Shared& sh) const {
    for (int q = threadIdx.x; q < ns; q += blockDim.x) sh.c[q] = narrow<T>(st->cphi[q]);
  }
  template <int ND, class A>
  __device__ void operator()(long i, Shared& sh, A (&)[ND]) const {
    const T vi = v0[i];
    for (int ks = 0; ks < ns; ++ks) x[ks * ld + i] = x[ks * ld + i] + sh.c[ks] * vi;
  }
};

// true residual of one shift: r = (b - A y) + sigma x; acc0 = |r|^2
template <class T, class S>
struct BMsRes {
  const T* r; const T* x; int ks; const S* st;
  struct Shared { T sg; };
  __device__ void prepare(Shared& sh) const { if (threadIdx.x == 0) sh.sg = narrow<T>(st->sigma[ks]); }
  template <int ND, class A>
  __device__ void operator()(long i, Shared& sh, A (&acc)[ND]) const {
    const T t = r[i] + sh.sg * x[i];
    acc_add(acc[0], abs2_(t));
  }
};
struct TMsRes {
  double* normr; int ks;
  template <class W> __device__ void operator()(const W* v) const { normr[ks] = sqrt(real_(v[0])); }
};
// flag 2 when a true residual misses the tolerance (msidrs.inc:321, msqmridr.inc)
template <class S>
__global__ void k_ms_final(S* st) {
  if (st->early) return;
  double mx = st->normr[0];
  for (int ks = 1; ks < st->ns; ++ks) mx = fmax(mx, st->normr[ks]);
  if (st->info == 0 && mx >= st->tolb) st->info = 2;
}

template <class T>
class MsIdrsGpu {
 public:
  using W = typename traits<T>::wide;
  MsIdrsGpu(Operator& A, int prec, int s, int ns, int method);
  ~MsIdrsGpu();
  // x(n, ns) column-major (device); sigma: ns wide values (device).  In inner
  // mode (o.inner) the final true residuals are omitted and x is left in the
  // mass-preconditioned variable with the collinearity factors in the state
  // (colfac_dev), as the reference does when colfac is requested.
  void solve(const T* b, const W* sigma, T* x, const SolveOpts& o);
  MsIdrsState<W> state();
  const W* colfac_dev() const { return d_st->phi; }
  const int* stop_flag() const { return &d_st->stop; }

  Operator& A;
  int prec, s, ns, method, rows;
  long n;
  cudaStream_t st;
  RedBuf rb;
  T *pool = nullptr, *Wb = nullptr, *v = nullptr, *t = nullptr, *tm = nullptr, *t1 = nullptr,
    *t2 = nullptr, *t3 = nullptr, *t4 = nullptr, *PT = nullptr;
  MsIdrsState<W>* d_st = nullptr;
  int* h_stop = nullptr;
  cudaEvent_t ev[2];
  bool p_ready = false;

 private:
  void matvec(const T* in, T* out, const int* skip, T fa = T(1), T fcv = T(0), const T* fv = nullptr);
  // out = fa * A M1^-1 in + fcv * fv   (M1: mass matrix, may be null)
  void apply(Operator* M1, const T* in, T* out, const int* skip, T fa = T(1), T fcv = T(0),
             const T* fv = nullptr);
};

// ================================================================ MSQMRIDR
// Start of an iteration (msqmridr.inc:131-155): iter += 1, c, mu, gamma, M shift.
template <class W>
__device__ inline void msq_prepare(MsQmrState<W>* st, const W* mu) {
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

template <class W> struct TMsqInit {  // msqmridr.inc:84-125
  MsQmrState<W>* st;
  __device__ void operator()(const W* v) const {
    st->normb = sqrt(real_(v[0]));
    st->tolb = st->tol * st->normb;
    st->normg = st->normb;
    for (int ks = 0; ks < st->ns; ++ks) {
      st->normr[ks] = st->normg;
      st->phi_n[ks] = W(0.0);
      st->phi_n1[ks] = W(st->normg);
      if (st->resvec) st->resvec[(long)st->ldr * ks] = st->normg;
    }
    if (st->normg <= st->tolb) { st->info = 0; st->iter = 0; st->early = 1; st->stop = 1; }
  }
};
template <class W> struct TMsqPrep {
  MsQmrState<W>* st;
  __device__ void operator()(const W* v) const { msq_prepare(st, v); }
};
template <class W> struct TMsqOm {
  MsQmrState<W>* st;
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
template <class W> struct TMsqBeta {  // one modified Gram-Schmidt coefficient
  MsQmrState<W>* st; int i; bool first;
  __device__ void operator()(const W* v) const {
    const int s = st->s;
    if (first) for (int q = 0; q < s + 2; ++q) st->h[q] = st->c[q] / st->om;
    st->beta[i] = v[0];
    st->h[i + 1] = st->h[i + 1] + v[0];
  }
};
// normg, h(s+2), then every shift's Givens update (msqmridr.inc:210-262)
template <class W> struct TMsqNorm {
  MsQmrState<W>* st; bool first;
  __device__ void operator()(const W* v) const {
    const int s = st->s, ns = st->ns;
    if (first) for (int q = 0; q < s + 2; ++q) st->h[q] = st->c[q] / st->om;
    st->normg = sqrt(real_(v[0]));
    st->h[s + 1] = W(st->normg);
    bool broken = false;
    for (int ks = 0; ks < ns; ++ks) {
      st->active[ks] = 0;
      if (broken || st->converged[ks]) continue;
      W rs[MAXS + 3];
      rs[0] = W(0.0);
      if (st->in_it == 0) {
        for (int q = 0; q < s + 2; ++q) rs[q + 1] = st->h[q] - st->sigma[ks] * st->c[q];
      } else {
        const W eta = st->cf[ks] / st->cf[ns];
        for (int q = 0; q < s + 2; ++q) rs[q + 1] = eta * st->h[q] - (eta - W(1.0)) * st->c[q];
      }
      W* cs = st->cs + (MAXS + 2) * ks;
      W* sn = st->sn + (MAXS + 2) * ks;
      const int low = max(1, s + 3 - st->iter);
      for (int l = low; l <= s + 1; ++l) {
        const W tau = rs[l - 1];
        rs[l - 1] = cs[l - 1] * tau + sn[l - 1] * rs[l];
        rs[l] = -conj_(sn[l - 1]) * tau + cs[l - 1] * rs[l];
      }
      const W tau = rs[s + 1];
      grot(tau, rs[s + 2], cs[s + 1], sn[s + 1], rs[s + 1]);
      st->phi_n[ks] = cs[s + 1] * st->phi_n1[ks];
      st->phi_n1[ks] = -conj_(sn[s + 1]) * st->phi_n1[ks];
      for (int q = 0; q < s + 1; ++q) { cs[q] = cs[q + 1]; sn[q] = sn[q + 1]; }
      if (abs_(rs[s + 1]) < kDblEps) {
        st->info = 3;  // leaves the shift loop only; the cycle still completes
        broken = true;
        continue;
      }
      for (int q = 0; q <= s; ++q) st->rsw[(MAXS + 1) * ks + q] = rs[q];
      st->rinv[ks] = W(1.0) / rs[s + 1];
      st->active[ks] = 1;
      st->normr[ks] = abs_(st->phi_n1[ks]) * sqrt_default_real(st->jj + 1);
      st->converged[ks] = st->normr[ks] < st->tolb;
    }
    double mx = 0.0;
    for (int ks = 0; ks < ns; ++ks) {
      if (st->resvec) st->resvec[st->iter + (long)st->ldr * ks] = st->normr[ks];
      mx = fmax(mx, st->normr[ks]);
    }
    if (mx < st->tolb) { st->info = 0; st->stop_next = 1; }
    else if (st->iter == st->maxit) { st->info = 1; st->stop_next = 1; }
  }
};

// Every active shift: wn = (vt_ks - W r_sigma(1:s+1)) / r_sigma(s+2) into the
// evicted slot of its window, x_ks += phi_n wn; then gn /= normg and
// acc_j = PT_j . gn (the next iteration's mu).  vt_ld is 0 when every shift
// shares one vtilde (no inner solve).
template <class T, class Tv, class W>
struct BMsqW {
  const Tv* vt; long vt_ld; T* Wb; T* x; T* gn; const T* PT; long ld; int s, ns; const MsQmrState<W>* st;
  struct Shared {
    T rs[(MAXS + 1) * MAXSIG]; T rinv[MAXSIG]; T phi[MAXSIG]; int act[MAXSIG]; int base[MAXSIG];
    typename traits<T>::real inorm;
  };
  __device__ void prepare(Shared& sh) const {
    for (int q = threadIdx.x; q < ns; q += blockDim.x) {
      for (int j = 0; j <= s; ++j) sh.rs[(MAXS + 1) * q + j] = narrow<T>(st->rsw[(MAXS + 1) * q + j]);
      sh.rinv[q] = narrow<T>(st->rinv[q]);
      sh.phi[q] = narrow<T>(st->phi_n[q]);
      sh.act[q] = st->active[q];
      sh.base[q] = st->wbase[q];
    }
    if (threadIdx.x == 0) sh.inorm = (typename traits<T>::real)(1.0 / st->normg);
  }
  template <int ND, class A>
  __device__ void operator()(long i, Shared& sh, A (&acc)[ND]) const {
    for (int ks = 0; ks < ns; ++ks) {
      if (!sh.act[ks]) continue;
      const T* r = sh.rs + (MAXS + 1) * ks;
      T* Wk = Wb + (long)(s + 1) * ks * ld;
      const int b = sh.base[ks];
      T a = T(0);
      for (int q = 0; q <= s; ++q) {
        int slot = b + q;
        if (slot > s) slot -= s + 1;
        a = a + Wk[slot * ld + i] * r[q];
      }
      const T wn = (T(vt[ks * vt_ld + i]) - a) * sh.rinv[ks];
      Wk[b * ld + i] = wn;
      x[ks * ld + i] = x[ks * ld + i] + sh.phi[ks] * wn;
    }
    const T g = gn[i] * sh.inorm;
    gn[i] = g;
#pragma unroll
    for (int d = 0; d < ND; ++d)
      if (d < s) acc_add(acc[d], PT[d * ld + i] * g);
  }
};
// Rotates the windows of the updated shifts, then commits a stop, ends the
// while loop after a cycle with a shift breakdown, or starts the next iteration.
template <class W> struct TMsqW {
  MsQmrState<W>* st; bool last_in_cycle;
  __device__ void operator()(const W* v) const {
    for (int ks = 0; ks < st->ns; ++ks)
      if (st->active[ks]) st->wbase[ks] = (st->wbase[ks] == st->s) ? 0 : st->wbase[ks] + 1;
    if (st->stop_next) { st->stop = 1; return; }
    if (last_in_cycle && st->info >= 0) { st->stop = 1; return; }
    msq_prepare(st, v);
  }
};

template <class T, class Tin>
class MsQmrGpu {
 public:
  using W = typename traits<T>::wide;
  MsQmrGpu(Operator& A, int s, int ns, const SolveOpts& o);
  ~MsQmrGpu();
  void solve(const T* b, const W* sigma, T* x, const SolveOpts& o);
  MsQmrState<W> state();

  Operator& A;
  int s, ns;
  long n;
  cudaStream_t st;
  RedBuf rb;
  T *gpool = nullptr, *Wb = nullptr, *v = nullptr, *vt = nullptr, *t = nullptr, *tm = nullptr,
    *t1 = nullptr, *t2 = nullptr, *PT = nullptr;
  Tin *v_in = nullptr, *Vt = nullptr;  // inner solve input and its n x (ns+1) solutions
  W* sig0 = nullptr;                   // [sigma, 0]
  MsIdrsGpu<Tin>* inner = nullptr;
  MsQmrState<W>* d_st = nullptr;
  W* d_scratch = nullptr;
  double* d_rho = nullptr;
  int* h_stop = nullptr;
  cudaEvent_t ev[2];
};

}  // namespace idrs
