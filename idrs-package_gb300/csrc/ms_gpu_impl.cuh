// ms_gpu_impl.cuh -- host drivers of MsIdrsGpu<T> and MsQmrGpu<T,Tin>.
// Included by one translation unit per scalar kind.
#pragma once

#include <utility>

#include "idrs_gpu_impl.cuh"
#include "ms_gpu.cuh"

namespace idrs {

// ------------------------------------------------------------------ MSIDRS
template <class T>
MsIdrsGpu<T>::MsIdrsGpu(Operator& A_, int prec_, int s_, int ns_, int method_)
    : A(A_), prec(prec_), s(s_), ns(ns_), method(method_) {
  if (s < 1 || s > MAXS) throw std::runtime_error("msidrs: s out of range");
  if (ns < 1 || ns > MAXSIG) throw std::runtime_error("msidrs: number of shifts out of range");
  n = A.n();
  st = A.stream;
  rb = A.red;
  rows = (method == 1) ? s : 1;
  // pool: G_1..G_s, gn and v0, addressed through slot maps (no vector copies)
  pool = dalloc<T>((long)(s + 2) * n, st);
  Wb = dalloc<T>((long)s * ns * n, st);
  v = dalloc<T>(n, st);
  t = dalloc<T>(n, st);
  tm = dalloc<T>(n, st);
  t1 = dalloc<T>(n, st);
  t2 = dalloc<T>(n, st);
  if (prec == 32) {
    t3 = dalloc<T>(n, st);
    t4 = dalloc<T>(n, st);
  }
  PT = dalloc<T>((long)rows * n, st);
  IDRS_CUDA(cudaMallocAsync((void**)&d_st, sizeof(MsIdrsState<W>), st));
  IDRS_CUDA(cudaMemsetAsync(d_st, 0, sizeof(MsIdrsState<W>), st));
  k_set_stop<W><<<1, 1, 0, st>>>(&d_st->stop);
  IDRS_LAUNCH_CHECK();
  IDRS_CUDA(cudaMallocHost((void**)&h_stop, 2 * sizeof(int)));
  IDRS_CUDA(cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming));
  IDRS_CUDA(cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming));
}

template <class T>
MsIdrsGpu<T>::~MsIdrsGpu() {
  for (void* p : {(void*)pool, (void*)Wb, (void*)v, (void*)t, (void*)tm, (void*)t1, (void*)t2, (void*)t3,
                  (void*)t4, (void*)PT, (void*)d_st})
    if (p) cudaFreeAsync(p, st);
  if (h_stop) cudaFreeHost(h_stop);
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
}

template <class T>
void MsIdrsGpu<T>::matvec(const T* in, T* out, const int* skip, T fa, T fcv, const T* fv) {
  if (prec == 32 && A.jac.valid())
    op_chain_recur<T>(A.view(prec), A.jac, A.degree, in, out, t1, t2, t3, t4, skip, st, fa, fcv, fv);
  else
    op_chain<T>(A.view(prec), A.alpha_p, A.degree, in, out, t1, t2, skip, st, fa, fcv, fv);
}

template <class T>
void MsIdrsGpu<T>::apply(Operator* M1, const T* in, T* out, const int* skip, T fa, T fcv, const T* fv) {
  if (M1) {
    op_precon<T>(*M1, prec, in, tm, skip, st);
    matvec(tm, out, skip, fa, fcv, fv);
  } else {
    matvec(in, out, skip, fa, fcv, fv);
  }
}

template <class T>
void MsIdrsGpu<T>::solve(const T* b, const W* sigma, T* x, const SolveOpts& o) {
  const int maxit = o.maxit >= 0 ? o.maxit : (int)std::min<long>(2 * n, 1000);
  MsArgs a{};
  a.maxit = maxit;
  a.s = s;
  a.ns = ns;
  a.n_omega = o.omega ? o.n_omega : 0;
  a.ldr = o.resvec_len;
  a.tol = o.tol;
  a.kappa = (method == 1) ? kKappa : 0.0;  // msidrs.inc:87-94
  a.resvec = o.resvec;
  a.omega = o.omega;
  const int* ostop = o.inner ? o.outer_stop : nullptr;
  k_msidrs_init<W><<<1, kThreads, 0, st>>>(d_st, a, sigma, ostop);
  IDRS_LAUNCH_CHECK();
  const int* stop = &d_st->stop;
  const int* early = &d_st->early;
  Operator* M1 = (o.M1 && o.M1->dkind != 0) ? o.M1 : nullptr;

  // slots of the pool: gmap[0..s-1] = G_1..G_s, then gn and v0
  int gmap[MAXS];
  for (int q = 0; q < s; ++q) gmap[q] = q;
  int gn_slot = s, v0_slot = s + 1;
  auto P = [&](int slot) { return pool + (long)slot * n; };
  // W = 0, v0 = 0, x = 0 (msidrs.inc:53, 97-101)
  IDRS_CUDA(cudaMemsetAsync(Wb, 0, sizeof(T) * (size_t)s * ns * n, st));
  IDRS_CUDA(cudaMemsetAsync(P(v0_slot), 0, sizeof(T) * (size_t)n, st));
  IDRS_CUDA(cudaMemsetAsync(x, 0, sizeof(T) * (size_t)ns * n, st));
  launch_fused<2, T>(n, BInit<T>{b, P(gn_slot), nullptr, true, false}, TMsInit<W>{d_st}, rb, stop, st);
  if (o.PT && method != 2) {
    k_narrow_copy<T><<<stream_grid((long)rows * n), kThreads, 0, st>>>((long)rows * n, (const W*)o.PT, PT);
    IDRS_LAUNCH_CHECK();
    p_ready = false;
  } else if (method == 2 || !p_ready) {
    make_shadow<T, W>(method, rows, n, o.p_seed, P(gn_slot), PT, n, d_st->alpha, &d_st->rho, rb, st);
    p_ready = (method != 2);
  }
  launch_fused_nd<T>(s, n, BPdot<T>{PT, n, P(gn_slot), s}, TMsF0<W>{d_st}, rb, stop, st);

  const int max_cycles = o.inner ? (maxit + s) / (s + 1) : (maxit > 0 ? maxit / (s + 1) + 2 : 1 << 30);
  for (int c = 0; c < max_cycles; ++c) {
    const bool first = (c == 0);
    for (int k = 0; k < s; ++k) {
      BMsV<T, W> bv{P(gn_slot), pool, n, {}, first ? s : k, s, v, d_st};
      for (int q = 0; q < s; ++q) bv.gmap[q] = gmap[q];
      launch_fused<0, T>(n, bv, NoTail(), rb, stop, st);
      // G_k = gn: the old gn buffer becomes G_k, the old G_k buffer takes the new gn
      const int fresh = gmap[k];
      gmap[k] = gn_slot;
      gn_slot = fresh;
      apply(M1, v, t, stop);
      launch_fused_nd<T>(s, n, BMsGn<T, W>{v, t, P(gn_slot), PT, n, s, &d_st->om, false},
                         TMsAlpha<W>{d_st, k}, rb, stop, st);
      BMsOrth<T, W> bo{P(gn_slot), pool, n, {}, k, d_st};
      for (int q = 0; q < s; ++q) bo.gmap[q] = gmap[q];
      launch_fused<1, T>(n, bo, TMsStep<W>{d_st, k}, rb, stop, st);
      launch_fused<0, T>(n, BMsShift<T, W>{v, P(v0_slot), Wb, x, n, s, ns, k, d_st}, NoTail(), rb, stop, st);
      k_msidrs_commit<W><<<1, 1, 0, st>>>(d_st, k + 1, k == s - 1 ? 1 : 0);
      IDRS_LAUNCH_CHECK();
    }
    // omega step: v = gn, t = A v, gn = v - om t, v0 = v (msidrs.inc:255-303)
    apply(M1, P(gn_slot), t, stop);
    launch_fused<3, T>(n, BOmDots<T>{t, P(gn_slot)}, TMsOm<W>{d_st}, rb, stop, st);
    launch_fused_nd<T>(s + 1, n, BMsGn<T, W>{P(gn_slot), t, P(v0_slot), PT, n, s, &d_st->om, true},
                       TMsGnOm<W>{d_st}, rb, stop, st);
    std::swap(gn_slot, v0_slot);
    launch_fused<0, T>(n, BMsX<T, W>{P(v0_slot), x, n, ns, d_st}, NoTail(), rb, stop, st);
    k_msidrs_commit<W><<<1, 1, 0, st>>>(d_st, 0, 0);
    IDRS_LAUNCH_CHECK();

    IDRS_CUDA(cudaMemcpyAsync(&h_stop[c & 1], stop, sizeof(int), cudaMemcpyDeviceToHost, st));
    IDRS_CUDA(cudaEventRecord(ev[c & 1], st));
    if (c >= 1) {
      IDRS_CUDA(cudaEventSynchronize(ev[(c - 1) & 1]));
      if (h_stop[(c - 1) & 1]) break;
    }
  }
  if (o.inner) return;
  // true residuals b - A y + sigma x per shift (msidrs.inc:306-316)
  for (int ks = 0; ks < ns; ++ks) {
    T* xs = x + (long)ks * n;
    apply(M1, xs, t, early, T(-1), T(1), b);
    launch_fused<1, T>(n, BMsRes<T, MsIdrsState<W>>{t, xs, ks, d_st}, TMsRes{d_st->normr, ks}, rb, early, st);
  }
  k_ms_final<<<1, 1, 0, st>>>(d_st);
  IDRS_LAUNCH_CHECK();
  if (M1)
    for (int ks = 0; ks < ns; ++ks) {
      T* xs = x + (long)ks * n;
      op_precon<T>(*M1, prec, xs, tm, early, st);
      vec_copy<T>(n, tm, xs, early, st);
    }
}

template <class T>
MsIdrsState<typename traits<T>::wide> MsIdrsGpu<T>::state() {
  MsIdrsState<W> h;
  IDRS_CUDA(cudaMemcpyAsync(&h, d_st, sizeof(h), cudaMemcpyDeviceToHost, st));
  IDRS_CUDA(cudaStreamSynchronize(st));
  return h;
}

// ---------------------------------------------------------------- MSQMRIDR
template <class T, class Tin>
MsQmrGpu<T, Tin>::MsQmrGpu(Operator& A_, int s_, int ns_, const SolveOpts& o) : A(A_), s(s_), ns(ns_) {
  if (s < 1 || s > MAXS) throw std::runtime_error("msqmridr: s out of range");
  if (ns < 1 || ns + 1 > MAXSIG) throw std::runtime_error("msqmridr: number of shifts out of range");
  n = A.n();
  st = A.stream;
  rb = A.red;
  gpool = dalloc<T>((long)(s + 1) * n, st);
  Wb = dalloc<T>((long)(s + 1) * ns * n, st);
  v = dalloc<T>(n, st);
  t = dalloc<T>(n, st);
  tm = dalloc<T>(n, st);
  t1 = dalloc<T>(n, st);
  t2 = dalloc<T>(n, st);
  PT = dalloc<T>((long)s * n, st);
  IDRS_CUDA(cudaMallocAsync((void**)&d_st, sizeof(MsQmrState<W>), st));
  IDRS_CUDA(cudaMemsetAsync(d_st, 0, sizeof(MsQmrState<W>), st));
  IDRS_CUDA(cudaMallocAsync((void**)&d_scratch, sizeof(W) * MAXS, st));
  IDRS_CUDA(cudaMallocAsync((void**)&d_rho, sizeof(double), st));
  if (o.in_it > 0) {
    inner = new MsIdrsGpu<Tin>(A, prec_of<Tin>(), o.in_s, ns + 1, 1);
    Vt = dalloc<Tin>((long)(ns + 1) * n, st);
    sig0 = dalloc<W>(ns + 1, st);
    if (!std::is_same<T, Tin>::value) {
      v_in = dalloc<Tin>(n, st);
      vt = dalloc<T>(n, st);
    }
  }
  IDRS_CUDA(cudaMallocHost((void**)&h_stop, 2 * sizeof(int)));
  IDRS_CUDA(cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming));
  IDRS_CUDA(cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming));
}

template <class T, class Tin>
MsQmrGpu<T, Tin>::~MsQmrGpu() {
  delete inner;
  for (void* p : {(void*)gpool, (void*)Wb, (void*)v, (void*)vt, (void*)t, (void*)tm, (void*)t1, (void*)t2,
                  (void*)PT, (void*)v_in, (void*)Vt, (void*)sig0, (void*)d_st, (void*)d_scratch, (void*)d_rho})
    if (p) cudaFreeAsync(p, st);
  if (h_stop) cudaFreeHost(h_stop);
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
}

template <class T, class Tin>
void MsQmrGpu<T, Tin>::solve(const T* b, const W* sigma, T* x, const SolveOpts& o) {
  const int maxit = o.maxit >= 0 ? o.maxit : (int)std::min<long>(2 * n, 1000);
  MsArgs a{};
  a.maxit = maxit;
  a.s = s;
  a.ns = ns;
  a.n_omega = o.omega ? o.n_omega : 0;
  a.ldr = o.resvec_len;
  a.in_it = o.in_it;
  a.tol = o.tol;
  a.kappa = kKappa;
  a.resvec = o.resvec;
  a.omega = o.omega;
  a.cf = inner ? (const void*)inner->colfac_dev() : nullptr;
  k_msqmr_init<W><<<1, kThreads, 0, st>>>(d_st, a, sigma);
  IDRS_LAUNCH_CHECK();
  const int* stop = &d_st->stop;
  const int* early = &d_st->early;
  Operator* M1 = (o.M1 && o.M1->dkind != 0) ? o.M1 : nullptr;
  if (inner) {  // shifts of the inner solve: [sigma, 0] (msqmridr.inc:165-170)
    IDRS_CUDA(cudaMemcpyAsync(sig0, sigma, sizeof(W) * ns, cudaMemcpyDeviceToDevice, st));
    IDRS_CUDA(cudaMemsetAsync(sig0 + ns, 0, sizeof(W), st));
  }
  int gmap[MAXS];
  for (int q = 0; q < s; ++q) gmap[q] = q;
  int gn_idx = s;
  auto G = [&](int idx) { return gpool + (long)idx * n; };
  IDRS_CUDA(cudaMemsetAsync(Wb, 0, sizeof(T) * (size_t)(s + 1) * ns * n, st));
  IDRS_CUDA(cudaMemsetAsync(x, 0, sizeof(T) * (size_t)ns * n, st));
  T* gn = G(gn_idx);
  auto matvec = [&](const T* in, T* out, const int* skip, T fa, T fcv, const T* fv) {
    if (M1) {
      op_precon<T>(*M1, 64, in, tm, skip, st);
      in = tm;
    }
    op_chain<T>(A.view(64), A.alpha_p, A.degree, in, out, t1, t2, skip, st, fa, fcv, fv);
  };
  launch_fused<2, T>(n, BInit<T>{b, gn, nullptr, true, false}, TMsqInit<W>{d_st}, rb, stop, st);
  if (o.PT) {
    k_narrow_copy<T><<<stream_grid((long)s * n), kThreads, 0, st>>>((long)s * n, (const W*)o.PT, PT);
    IDRS_LAUNCH_CHECK();
  } else {
    make_shadow<T, W>(1, s, n, o.p_seed, gn, PT, n, d_scratch, d_rho, rb, st);
  }
  using S = MsQmrState<W>;
  launch_fused_nd<T>(s, n, BQstart<T, W, S>{gn, PT, n, s, d_st}, TMsqPrep<W>{d_st}, rb, stop, st);

  SolveOpts io;
  io.tol = o.in_tol;
  io.maxit = o.in_it;
  io.M1 = o.M1;
  io.inner = true;
  io.outer_stop = stop;
  io.p_seed = o.p_seed;

  const int max_cycles = maxit > 0 ? maxit / (s + 1) + 2 : 1 << 30;
  int it = 0;
  for (int c = 0; c < max_cycles; ++c) {
    for (int k = 1; k <= s + 1; ++k) {
      ++it;
      gn = G(gn_idx);
      const T* vptr = gn;
      if (it > s) {
        BQv<T, W, S> bq{gn, gpool, n, {}, s, v, d_st};
        for (int q = 0; q < s; ++q) bq.gmap[q] = gmap[q];
        launch_fused<0, T>(n, bq, NoTail(), rb, stop, st);
        vptr = v;
      }
      // G(:,1:s-1) = G(:,2:s); G(:,s) = gn  (buffer rotation, no copy)
      const int old_first = gmap[0];
      for (int q = 0; q < s - 1; ++q) gmap[q] = gmap[q + 1];
      gmap[s - 1] = gn_idx;
      gn_idx = old_first;
      gn = G(gn_idx);
      // preconditioning: inner MSIDRS on [sigma, 0] or vtilde = v
      const T* vtm = vptr;  // the vector the operator is applied to
      if (inner) {
        if constexpr (std::is_same<T, Tin>::value) {
          inner->solve(vptr, sig0, Vt, io);
          vtm = Vt + (long)ns * n;
        } else {
          vec_convert<T, Tin>(n, vptr, v_in, stop, st);
          inner->solve(v_in, sig0, Vt, io);
          vec_convert<Tin, T>(n, Vt + (long)ns * n, vt, stop, st);
          vtm = vt;
        }
      }
      matvec(vtm, gn, stop, T(1), T(0), nullptr);
      if (k == s + 1) launch_fused<3, T>(n, BOmDots<T>{gn, vptr}, TMsqOm<W>{d_st}, rb, stop, st);
      // gn = gn - v/om, then modified Gram-Schmidt (msqmridr.inc:190-209)
      if (k < s + 1) {
        for (int idx = 0; idx < k; ++idx) {
          const int i = s - k + idx;
          const T* y = (idx == 0) ? vptr : G(gmap[i - 1]);
          launch_fused<1, T>(n, BMgs<T, W, S>{gn, y, G(gmap[i]), idx == 0, i - 1, d_st},
                             TMsqBeta<W>{d_st, i, idx == 0}, rb, stop, st);
        }
        launch_fused<1, T>(n, BMgs<T, W, S>{gn, G(gmap[s - 1]), nullptr, false, s - 1, d_st},
                           TMsqNorm<W>{d_st, false}, rb, stop, st);
      } else {
        launch_fused<1, T>(n, BMgs<T, W, S>{gn, vptr, nullptr, true, 0, d_st}, TMsqNorm<W>{d_st, true},
                           rb, stop, st);
      }
      // every shift's wn and x, normalise gn, next mu
      const bool last = (k == s + 1);
      if (inner)
        launch_fused_nd<T>(s, n, BMsqW<T, Tin, W>{Vt, n, Wb, x, gn, PT, n, s, ns, d_st},
                           TMsqW<W>{d_st, last}, rb, stop, st);
      else
        launch_fused_nd<T>(s, n, BMsqW<T, T, W>{vptr, 0, Wb, x, gn, PT, n, s, ns, d_st},
                           TMsqW<W>{d_st, last}, rb, stop, st);
    }
    IDRS_CUDA(cudaMemcpyAsync(&h_stop[c & 1], stop, sizeof(int), cudaMemcpyDeviceToHost, st));
    IDRS_CUDA(cudaEventRecord(ev[c & 1], st));
    if (c >= 1) {
      IDRS_CUDA(cudaEventSynchronize(ev[(c - 1) & 1]));
      if (h_stop[(c - 1) & 1]) break;
    }
  }
  // true residuals per shift, then x = M1^-1 x (msqmridr.inc, end)
  for (int ks = 0; ks < ns; ++ks) {
    T* xs = x + (long)ks * n;
    matvec(xs, t, early, T(-1), T(1), b);
    launch_fused<1, T>(n, BMsRes<T, S>{t, xs, ks, d_st}, TMsRes{d_st->normr, ks}, rb, early, st);
  }
  k_ms_final<<<1, 1, 0, st>>>(d_st);
  IDRS_LAUNCH_CHECK();
  if (M1)
    for (int ks = 0; ks < ns; ++ks) {
      T* xs = x + (long)ks * n;
      op_precon<T>(*M1, 64, xs, tm, early, st);
      vec_copy<T>(n, tm, xs, early, st);
    }
}

template <class T, class Tin>
MsQmrState<typename traits<T>::wide> MsQmrGpu<T, Tin>::state() {
  MsQmrState<W> h;
  IDRS_CUDA(cudaMemcpyAsync(&h, d_st, sizeof(h), cudaMemcpyDeviceToHost, st));
  IDRS_CUDA(cudaStreamSynchronize(st));
  return h;
}

}  // namespace idrs
