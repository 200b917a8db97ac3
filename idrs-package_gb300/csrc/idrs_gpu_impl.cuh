// idrs_gpu_impl.cuh -- host drivers of IdrsGpu<T> and QmrGpu<T,Tin>.
// Included by one translation unit per precision.
#pragma once

#include "idrs_gpu.cuh"
#include "stencil_dot.cuh"

namespace idrs {

template <class T> static inline int prec_of() { return (sizeof(typename traits<T>::real) == 4) ? 32 : 64; }

template <class T>
static T* dalloc(long n, cudaStream_t st) {
  T* p = nullptr;
  IDRS_CUDA(cudaMallocAsync((void**)&p, sizeof(T) * (size_t)std::max<long>(n, 1), st));
  return p;
}

// ------------------------------------------------------------------ IDR(s)
template <class T>
IdrsGpu<T>::IdrsGpu(Operator& A_, int prec_, int s_, int method_)
    : A(A_), prec(prec_), s(s_), method(method_) {
  n = A.n();
  st = A.stream;
  rb = A.red;
  rows = (method == 1) ? s : 1;
  G = dalloc<T>((long)s * n, st);
  U = dalloc<T>((long)s * n, st);
  r = dalloc<T>(n, st);
  v = dalloc<T>(n, st);
  t = dalloc<T>(n, st);
  t1 = dalloc<T>(n, st);
  t2 = dalloc<T>(n, st);
  if (prec == 32) {
    t3 = dalloc<T>(n, st);
    t4 = dalloc<T>(n, st);
  } else if (use_recurrence(A, prec)) {
    t3 = dalloc<T>(n, st);  // the fp64 recurrence rotates three vectors
  }
  PT = dalloc<T>((long)rows * n, st);
  IDRS_CUDA(cudaMallocAsync((void**)&d_st, sizeof(IdrsState<W>), st));
  IDRS_CUDA(cudaMemsetAsync(d_st, 0, sizeof(IdrsState<W>), st));
  k_set_stop<W><<<1, 1, 0, st>>>(&d_st->stop);
  IDRS_LAUNCH_CHECK();
  IDRS_CUDA(cudaMallocHost((void**)&h_stop, 2 * sizeof(int)));
  IDRS_CUDA(cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming));
  IDRS_CUDA(cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming));
}

template <class T>
IdrsGpu<T>::~IdrsGpu() {
  for (void* p : {(void*)G, (void*)U, (void*)r, (void*)v, (void*)t, (void*)t1, (void*)t2, (void*)t3, (void*)t4,
                  (void*)PT, (void*)d_st})
    if (p) cudaFreeAsync(p, st);
  if (h_stop) cudaFreeHost(h_stop);
  if (cycle_graph) cudaGraphExecDestroy(cycle_graph);
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
}

// Every IDR(s) cycle after the first launches the same kernels with the same
// arguments (fixed vectors, coefficients read from the device state, the
// stop flag read by each kernel), so a solve captures one such cycle as a
// CUDA graph and replays it: one launch per cycle instead of one per pass,
// which is what bounds small problems (2 MB vectors at 64^3).  The inner
// solves of a flexible QMRIDR(s) all write the same x, so the graph captured
// by the first one serves the whole outer solve.
// Anything the capture cannot hold ends it with an error; the solve then
// launches its cycles directly.  Returns whether the graph is ready.
// IDRS_CYCLE_GRAPHS=0 in the environment launches every cycle directly
// (read once per process; for comparisons)
inline bool cycle_graphs_enabled() {
  static const bool on = [] {
    const char* e = getenv("IDRS_CYCLE_GRAPHS");
    return !(e && e[0] == '0');
  }();
  return on;
}

template <class T>
bool IdrsGpu<T>::capture_cycle(const T* b, T* x, const SolveOpts& o, bool inispace) {
  if (cycle_graph) return true;
  cudaGraph_t g = nullptr;
  if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  const long l0 = launch_count();
  bool ok = true;
  try {
    enqueue_cycle(b, x, o, 1, inispace);
  } catch (const cuda_error&) {
    ok = false;
  }
  const cudaError_t e = cudaStreamEndCapture(st, &g);
  const long captured = launch_count() - l0;
  uncount_launches(captured);  // captured, not run: each replay counts them
  if (!ok || e != cudaSuccess || !g || cudaGraphInstantiate(&cycle_graph, g, 0) != cudaSuccess) {
    cudaGetLastError();
    if (g) cudaGraphDestroy(g);
    cycle_graph = nullptr;
    return false;
  }
  cudaGraphDestroy(g);
  cycle_launches = captured;
  graph_x = x;
  return true;
}

template <class T>
void IdrsGpu<T>::matvec(const T* in, T* out, const int* skip, T fa, T fcv, const T* fv) {
  // fp32 evaluates the polynomial by its stable three-term recurrence; fp64
  // keeps the monomial Horner form of rpolpre (matrix_module.f90:266-284)
  // unless the operator asks for the recurrence (poly_eval 1)
  op_apply<T>(A, prec, in, out, t1, t2, t3, t4, skip, st, fa, fcv, fv);
}

template <class T>
__global__ void k_narrow_copy(long n, const typename traits<T>::wide* a, T* b) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += gridDim.x * (long)blockDim.x)
    b[i] = narrow<T>(a[i]);
}

template <class T>
void IdrsGpu<T>::solve(const T* b, T* x, const SolveOpts& o) {
  if (s < 1 || s > MAXS) throw std::runtime_error("idrs: s out of range");
  const int maxit = o.maxit >= 0 ? o.maxit : (int)std::min<long>(2 * n, 1000);
  IdrsState<W> init{};
  init.info = -1;
  init.maxit = maxit;
  init.method = method;
  init.s = s;
  init.tol = o.tol;
  init.kappa = (method == 1 || method == 3) ? kKappa : 0.0;
  init.out_H = (o.H != nullptr && o.nritz > 0) ? 1 : 0;
  init.nritz = o.nritz;
  init.H = (W*)o.H;
  init.ldH = o.ldH;
  init.resvec = o.resvec;
  init.omega = (const W*)o.omega;
  init.n_omega = o.omega ? o.n_omega : 0;
  init.om = W(1.0);
  init.relres = 1.0;
  init.xpend = 0;
  init.xdone = 1;
  const int* ostop = o.inner ? o.outer_stop : nullptr;
  k_idrs_state_init<W><<<1, 1, 0, st>>>(d_st, init, ostop);
  IDRS_LAUNCH_CHECK();
  const int* stop = &d_st->stop;
  const int* early = &d_st->early;
  const bool have_x0 = (o.x0 != nullptr);
  const bool inispace = (o.U0 != nullptr);
  if (have_x0) {
    vec_copy<T>(n, (const T*)o.x0, x, stop, st);
    matvec(x, r, stop, T(-1), T(1), b);  // r = b - A x
  }
  launch_fused<2, T>(n, BInit<T>{b, r, x, !have_x0, !have_x0}, TIdrsInit<W>{d_st}, rb, stop, st);
  if (inispace) vec_copy<T>((long)s * n, (const T*)o.U0, U, stop, st);
  // shadow space
  if (o.PT && method != 2) {
    k_narrow_copy<T><<<stream_grid((long)rows * n), kThreads, 0, st>>>((long)rows * n, (const W*)o.PT, PT);
    IDRS_LAUNCH_CHECK();
    p_ready = false;
  } else if (method == 2 || !p_ready) {
    make_shadow<T, W>(method, rows, n, o.p_seed, r, PT, n, d_st->alpha, &d_st->rho, rb, st);
    p_ready = (method != 2);
  }
  launch_fused_nd<T>(s, n, BPdot<T>{PT, n, r, s}, TIdrsF0<W>{d_st}, rb, stop, st);
  // maxit <= 0 never ends the reference loop by count; the host then relies
  // on the device stop flag alone.
  const int max_cycles = o.inner ? (maxit + s) / (s + 1) : (maxit > 0 ? maxit / (s + 1) + 2 : 1 << 30);
  // One cycle of look-ahead: cycle c is queued before the host waits for the
  // stop flag of cycle c-1, so the GPU never waits for the host.  An inner
  // solve polls too (its outer iteration waits for its result anyway) so that
  // it launches no cycles beyond the one after convergence.
  const bool lu = A.P && (A.P->which_precon == 2 || A.P->which_precon == 3);
  bool graphs = cycle_graphs_enabled() && !(o.M1 && o.M1->dkind != 0) && !lu && !(A.defl && A.defl->k > 0);
  if (cycle_graph && !(o.inner && graphs && x == graph_x)) {
    cudaGraphExecDestroy(cycle_graph);  // captured for another solve's vectors
    cycle_graph = nullptr;
  }
  for (int c = 0; c < max_cycles; ++c) {
    if (c >= 1 && graphs) graphs = capture_cycle(b, x, o, inispace);
    if (c >= 1 && graphs) {
      IDRS_CUDA(cudaGraphLaunch(cycle_graph, st));
      for (long q = 0; q < cycle_launches; ++q) count_launch();
    } else {
      enqueue_cycle(b, x, o, c, inispace);
    }
    IDRS_CUDA(cudaMemcpyAsync(&h_stop[c & 1], stop, sizeof(int), cudaMemcpyDeviceToHost, st));
    IDRS_CUDA(cudaEventRecord(ev[c & 1], st));
    if (c >= 1) {
      IDRS_CUDA(cudaEventSynchronize(ev[(c - 1) & 1]));
      if (h_stop[(c - 1) & 1]) break;
    }
  }
  // x updates of the steps of a cycle the solve stopped in (skipped when none
  // is pending)
  launch_fused<0, T>(n, BXFlush<T, W>{x, U, n, s, d_st}, NoTail(), rb, &d_st->xdone, st);
  k_xflush_done<W><<<1, 1, 0, st>>>(d_st);
  IDRS_LAUNCH_CHECK();
  if (!o.inner) {
    matvec(x, r, early, T(-1), T(1), b);  // true residual b - A x (idrs.inc:304)
    launch_fused<1, T>(n, BNorm<T>{r}, TIdrsFinal<W>{d_st}, rb, early, st);
  }
}

template <class T>
void IdrsGpu<T>::enqueue_cycle(const T* b, T* x, const SolveOpts& o, int cycle, bool inispace) {
  (void)b;
  const int* stop = &d_st->stop;
  const bool first = (cycle == 0);
  Operator* M1 = (o.M1 && o.M1->dkind != 0) ? o.M1 : nullptr;
  for (int k = 0; k < s; ++k) {
    T* Gk = G + (long)k * n;
    T* Uk = U + (long)k * n;
    if (first) {
      if (!inispace) {
        if (M1) op_precon<T>(*M1, prec, r, Uk, stop, st);
        else vec_copy<T>(n, r, Uk, stop, st);
      }
    } else if (M1) {
      launch_fused<0, T>(n, BBuildU<T, W>{r, G, U, n, k, s, d_st, v}, NoTail(), rb, stop, st);
      op_precon<T>(*M1, prec, v, t, stop, st);
      launch_fused<0, T>(n, BCombineU<T, W>{t, U, n, k, s, d_st}, NoTail(), rb, stop, st);
    } else {
      launch_fused<0, T>(n, BBuildU<T, W>{r, G, U, n, k, s, d_st, nullptr}, NoTail(), rb, stop, st);
    }
    // G_k = A U_k and mu = P^T G_k: on the fp32 stencil the projection is
    // accumulated by the chain's last pass (G_k is not read back)
    bool fused = false;
    if constexpr (std::is_same<T, float>::value)
      fused = prec == 32 && chain_with_pdot(A, Uk, Gk, t1, t2, t3, t4, PT, n, s, rb, TIdrsMu<W>{d_st, k}, stop, st);
    if (!fused) {
      matvec(Uk, Gk, stop);
      launch_fused_nd<T>(s, n, BPdot<T>{PT, n, Gk, s}, TIdrsMu<W>{d_st, k}, rb, stop, st);
    }
    launch_fused<1, T>(n, BIdrUpd<T, W>{G, U, n, k, r, d_st}, TIdrsNorm<W>{d_st, k}, rb, stop, st);
  }
  // omega step (idrs.inc:254-299)
  const T* vv = r;
  if (M1) {
    op_precon<T>(*M1, prec, r, v, stop, st);
    vv = v;
  }
  // t = A vv and t.r, t.t, r.r: on the fp32 stencil accumulated by the
  // chain's last pass (t is not read back for them)
  bool fused = false;
  if constexpr (std::is_same<T, float>::value)
    fused = prec == 32 && chain_with_pdot<TIdrsOm<W>, true>(A, vv, t, t1, t2, t3, t4, r, n, 1, rb, TIdrsOm<W>{d_st},
                                                            stop, st);
  if (!fused) {
    matvec(vv, t, stop);
    launch_fused<3, T>(n, BOmDots<T>{t, r}, TIdrsOm<W>{d_st}, rb, stop, st);
  }
  launch_fused_nd<T>(s + 1, n, BOmUpd<T, W>{r, t, x, vv, PT, n, s, &d_st->om, U, d_st}, TIdrsNormOm<W>{d_st}, rb,
                     stop, st);
}

template <class T>
IdrsState<typename traits<T>::wide> IdrsGpu<T>::state() {
  IdrsState<W> h;
  IDRS_CUDA(cudaMemcpyAsync(&h, d_st, sizeof(h), cudaMemcpyDeviceToHost, st));
  IDRS_CUDA(cudaStreamSynchronize(st));
  return h;
}

// ----------------------------------------------------------------- QMRIDR(s)
template <class T, class Tin>
QmrGpu<T, Tin>::QmrGpu(Operator& A_, int s_, const SolveOpts& o) : A(A_), s(s_) {
  n = A.n();
  st = A.stream;
  rb = A.red;
  gpool = dalloc<T>((long)(s + 1) * n, st);
  wpool = dalloc<T>((long)(s + 1) * n, st);
  v = dalloc<T>(n, st);
  vt = dalloc<T>(n, st);
  t1 = dalloc<T>(n, st);
  t2 = dalloc<T>(n, st);
  if (use_recurrence(A, 64)) t3 = dalloc<T>(n, st);
  PT = dalloc<T>((long)s * n, st);
  IDRS_CUDA(cudaMallocAsync((void**)&d_st, sizeof(QmrState<W>), st));
  IDRS_CUDA(cudaMemsetAsync(d_st, 0, sizeof(QmrState<W>), st));
  IDRS_CUDA(cudaMallocAsync((void**)&d_scratch, sizeof(W) * MAXS, st));
  IDRS_CUDA(cudaMallocAsync((void**)&d_rho, sizeof(double), st));
  if (o.in_it > 0) {
    inner = new IdrsGpu<Tin>(A, prec_of<Tin>(), o.in_s, 1);
    if (!std::is_same<T, Tin>::value) {
      v_in = dalloc<Tin>(n, st);
      vt_in = dalloc<Tin>(n, st);
    }
  }
  IDRS_CUDA(cudaMallocHost((void**)&h_stop, 2 * sizeof(int)));
  IDRS_CUDA(cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming));
  IDRS_CUDA(cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming));
}

template <class T, class Tin>
QmrGpu<T, Tin>::~QmrGpu() {
  delete inner;
  for (void* p : {(void*)gpool, (void*)wpool, (void*)v, (void*)vt, (void*)t1, (void*)t2, (void*)t3, (void*)PT,
                  (void*)d_st, (void*)d_scratch, (void*)d_rho, (void*)v_in, (void*)vt_in})
    if (p) cudaFreeAsync(p, st);
  if (h_stop) cudaFreeHost(h_stop);
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
}

template <class T, class Tin>
void QmrGpu<T, Tin>::solve(const T* b, T* x, const SolveOpts& o) {
  if (s < 1 || s > MAXS) throw std::runtime_error("qmridr: s out of range");
  const int maxit = o.maxit >= 0 ? o.maxit : (int)std::min<long>(2 * n, 1000);
  QmrState<W> init{};
  init.info = -1;
  init.maxit = maxit;
  init.s = s;
  init.tol = o.tol;
  init.kappa = kKappa;
  init.om = W(1.0);
  init.relres = 1.0;
  init.resvec = o.resvec;
  init.omega = (const W*)o.omega;
  init.n_omega = o.omega ? o.n_omega : 0;
  IDRS_CUDA(cudaMemcpyAsync(d_st, &init, sizeof(init), cudaMemcpyHostToDevice, st));
  const int* stop = &d_st->stop;
  const int* early = &d_st->early;
  int gmap[MAXS], wmap[MAXS + 1];
  for (int q = 0; q < s; ++q) gmap[q] = q;
  int gn_idx = s;
  for (int q = 0; q <= s; ++q) wmap[q] = q;
  auto G = [&](int idx) { return gpool + (long)idx * n; };
  IDRS_CUDA(cudaMemsetAsync(wpool, 0, sizeof(T) * (size_t)(s + 1) * n, st));
  T* gn = G(gn_idx);
  const bool have_x0 = (o.x0 != nullptr);
  auto matvec = [&](const T* in, T* out, const int* skip, T fa, T fcv, const T* fv) {
    op_apply<T>(A, 64, in, out, t1, t2, t3, nullptr, skip, st, fa, fcv, fv);
  };
  if (have_x0) {
    vec_copy<T>(n, (const T*)o.x0, x, stop, st);
    matvec(x, gn, stop, T(-1), T(1), b);
  }
  launch_fused<2, T>(n, BInit<T>{b, gn, x, !have_x0, !have_x0}, TQmrInit<W>{d_st}, rb, stop, st);
  if (o.PT) {
    k_narrow_copy<T><<<stream_grid((long)s * n), kThreads, 0, st>>>((long)s * n, (const W*)o.PT, PT);
    IDRS_LAUNCH_CHECK();
  } else {
    make_shadow<T, W>(1, s, n, o.p_seed, gn, PT, n, d_scratch, d_rho, rb, st);
  }
  launch_fused_nd<T>(s, n, BQstart<T, W>{gn, PT, n, s, d_st}, TQmrStart<W>{d_st}, rb, stop, st);

  SolveOpts io;
  io.tol = o.in_tol;
  io.maxit = o.in_it;
  io.M1 = o.M1;
  io.inner = true;
  io.outer_stop = stop;
  io.p_seed = o.p_seed;
  Operator* M1 = (o.M1 && o.M1->dkind != 0) ? o.M1 : nullptr;

  const int max_cycles = maxit > 0 ? maxit / (s + 1) + 2 : 1 << 30;
  int it = 0;
  for (int c = 0; c < max_cycles; ++c) {
    for (int k = 1; k <= s + 1; ++k) {
      ++it;
      gn = G(gn_idx);
      const T* vptr = gn;
      if (it > s) {
        BQv<T, W> bq{gn, gpool, n, {}, s, v, d_st};
        for (int q = 0; q < s; ++q) bq.gmap[q] = gmap[q];
        launch_fused<0, T>(n, bq, NoTail(), rb, stop, st);
        vptr = v;
      }
      // G(:,1:s-1) = G(:,2:s); G(:,s) = gn  (buffer rotation, no copy)
      int old_first = gmap[0];
      for (int q = 0; q < s - 1; ++q) gmap[q] = gmap[q + 1];
      gmap[s - 1] = gn_idx;
      gn_idx = old_first;
      gn = G(gn_idx);
      // preconditioning (qmridr.inc:161-173)
      const T* vtptr = vptr;
      if (o.in_it == 0) {
        if (M1) { op_precon<T>(*M1, 64, vptr, vt, stop, st); vtptr = vt; }
      } else {
        if constexpr (std::is_same<T, Tin>::value) {
          inner->solve(vptr, vt, io);
        } else {
          vec_convert<T, Tin>(n, vptr, v_in, stop, st);
          inner->solve(v_in, vt_in, io);
          vec_convert<Tin, T>(n, vt_in, vt, stop, st);
        }
        k_inner_stats<<<1, 1, 0, st>>>(d_st, inner->d_st);
        IDRS_LAUNCH_CHECK();
        vtptr = vt;
      }
      matvec(vtptr, gn, stop, T(1), T(0), nullptr);
      if (k == s + 1) launch_fused<3, T>(n, BOmDots<T>{gn, vptr}, TQmrOm<W>{d_st}, rb, stop, st);
      // gn = gn - v/om, then modified Gram-Schmidt (qmridr.inc:194-208)
      if (k < s + 1) {
        for (int idx = 0; idx < k; ++idx) {
          int i = s - k + idx;
          const T* y = (idx == 0) ? vptr : G(gmap[i - 1]);
          launch_fused<1, T>(n, BMgs<T, W>{gn, y, G(gmap[i]), idx == 0, i - 1, d_st},
                             TQmrBeta<W>{d_st, i, idx == 0}, rb, stop, st);
        }
        launch_fused<1, T>(n, BMgs<T, W>{gn, G(gmap[s - 1]), nullptr, false, s - 1, d_st},
                           TQmrNorm<W>{d_st, false}, rb, stop, st);
      } else {
        launch_fused<1, T>(n, BMgs<T, W>{gn, vptr, nullptr, true, 0, d_st}, TQmrNorm<W>{d_st, true},
                           rb, stop, st);
      }
      // wn, x, normalise gn, next mu (qmridr.inc:206-252)
      BQw<T, W> bw{vtptr, wpool, n, {}, s, x, gn, PT, d_st};
      for (int q = 0; q <= s; ++q) bw.wmap[q] = wmap[q];
      launch_fused_nd<T>(s, n, bw, TQmrW<W>{d_st}, rb, stop, st);
      int wfirst = wmap[0];
      for (int q = 0; q < s; ++q) wmap[q] = wmap[q + 1];
      wmap[s] = wfirst;
    }
    IDRS_CUDA(cudaMemcpyAsync(&h_stop[c & 1], stop, sizeof(int), cudaMemcpyDeviceToHost, st));
    IDRS_CUDA(cudaEventRecord(ev[c & 1], st));
    if (c >= 1) {
      IDRS_CUDA(cudaEventSynchronize(ev[(c - 1) & 1]));
      if (h_stop[(c - 1) & 1]) break;
    }
  }
  gn = G(gn_idx);
  matvec(x, gn, early, T(-1), T(1), b);
  launch_fused<1, T>(n, BNorm<T>{gn}, TQmrFinal<W>{d_st}, rb, early, st);
}

template <class T, class Tin>
QmrState<typename traits<T>::wide> QmrGpu<T, Tin>::state() {
  QmrState<W> h;
  IDRS_CUDA(cudaMemcpyAsync(&h, d_st, sizeof(h), cudaMemcpyDeviceToHost, st));
  IDRS_CUDA(cudaStreamSynchronize(st));
  return h;
}

}  // namespace idrs
