"""Multishift solvers on the GPU (MSIDRS, MSQMRIDR; msidrs.inc, msqmridr.inc)
against the oracle on the same inputs, through the C ABI.

Problems: the 7-point Laplacian on an 8^3 grid (complex operator) with the
shifts of the multishift workload, sigma_k = (2 pi f_k)^2 (1 - 0.05i):
  * "definite" shifts, Re(sigma) in [1.2, 4] * lambda_max (K - sigma I is
    negative definite, well conditioned): converged solutions must agree with
    the oracle to 10 * tol;
  * "indefinite" shifts, Re(sigma) in [0.1, 0.9] * lambda_max: residual
    histories are compared over the first 12 iterations (rtol 1e-8, the
    rounding of fused reductions differs) and every true residual must meet
    the tolerance; x itself is compared to 10 * tol * cond(K - sigma I).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N1 = 8


@pytest.fixture(scope="module")
def P(gpu):
    return gpu.problems


def _rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


def _laplace(gpu, oracle, P, n=N1, cplx=True):
    coef = P.laplace_coefficients(n)
    K = gpu.stencil7_format(n, n, n, coef)
    Ko = oracle.stencil7_format(n, n, n, coef)
    return K, Ko, gpu.Matrix(K, complex=cplx), oracle.Matrix(Ko, cplx=cplx)


def _shifts(P, kind, n_shifts=4, n=N1):
    lo, hi = (1.2, 4.0) if kind == "definite" else (0.1, 0.9)
    sig, lam = P.multishift_shifts(n, n_shifts=n_shifts, lo=lo, hi=hi)
    return sig, lam


def _dense_laplace(P, n=N1):
    coef = P.laplace_coefficients(n)
    rp, ci, vals = P.stencil_to_crs(n, n, n, coef)
    N = n ** 3
    D = np.zeros((N, N))
    for i in range(N):
        D[i, ci[rp[i] - 1:rp[i + 1] - 1] - 1] = vals[rp[i] - 1:rp[i + 1] - 1]
    return D


def _maxit(N):
    return min(2 * N, 1000)


# ------------------------------------------------------------------ MSIDRS
@pytest.mark.parametrize("s", [2, 4, 8])
def test_msidrs_matches_oracle(gpu, oracle, P, s):
    K, Ko, A, Ao = _laplace(gpu, oracle, P)
    N = N1 ** 3
    b = P.complex_unit_normal(N)
    PT = oracle.make_p(s, N, seed=11, cplx=True)
    A.set_shadow(s, PT)
    tol = 1e-8
    sig, _ = _shifts(P, "indefinite")
    g = gpu.MSIDRS(A, b, sig, s, tolerance=tol, resvec=True, colfac=True)
    o = oracle.msidrs(Ao, b, sig, s, tolerance=tol, PT=PT, resvec_len=_maxit(N) + 1,
                      colfac_len=len(sig))
    assert g.flag == o.flag == 0
    np.testing.assert_allclose(g.resvec[:13], o.resvec[:13], rtol=1e-8)
    # indefinite shifts: ~200 iterations amplify the rounding differences
    assert abs(g.iterations - o.iterations) <= max(s + 1, 0.15 * o.iterations)
    assert np.max(g.relres) <= tol
    D = _dense_laplace(P)
    for k in range(len(sig)):
        Ak = D - sig[k] * np.eye(N)
        cond = np.linalg.cond(Ak)
        assert _rel(g.x[:, k], o.x[:, k]) <= 10 * tol * cond
    # definite shifts: converged solutions agree to 10 * tol
    sd, _ = _shifts(P, "definite", n_shifts=6)
    g = gpu.MSIDRS(A, b, sd, s, tolerance=tol)
    o = oracle.msidrs(Ao, b, sd, s, tolerance=tol, PT=PT)
    assert g.flag == o.flag == 0 and np.max(g.relres) <= tol
    assert g.iterations == o.iterations
    for k in range(len(sd)):
        assert _rel(g.x[:, k], o.x[:, k]) <= 10 * tol


def test_msidrs_colfac_and_history(gpu, oracle, P):
    """colfac (the collinearity factors phi, msidrs.inc:329) and the full
    residual history of every shift over a short run."""
    K, Ko, A, Ao = _laplace(gpu, oracle, P)
    N = N1 ** 3
    b = P.complex_unit_normal(N, seed=3)
    PT = oracle.make_p(4, N, seed=2, cplx=True)
    A.set_shadow(4, PT)
    sig, _ = _shifts(P, "indefinite", n_shifts=5)
    sig = np.concatenate([sig, [0.0]])
    g = gpu.MSIDRS(A, b, sig, 4, tolerance=0.1, maximum_iterations=10, resvec=True, colfac=True)
    o = oracle.msidrs(Ao, b, sig, 4, tolerance=0.1, maximum_iterations=10, PT=PT,
                      resvec_len=11, colfac_len=len(sig))
    assert g.flag == o.flag and g.iterations == o.iterations
    np.testing.assert_allclose(g.resvec, o.resvec, rtol=1e-9)
    np.testing.assert_allclose(g.colfac, o.colfac, rtol=1e-9)
    np.testing.assert_allclose(g.relres, o.relres, rtol=1e-9)
    np.testing.assert_allclose(g.x, o.x, rtol=1e-9, atol=1e-12 * np.abs(o.x).max())


def test_msbicgstab_variant(gpu, oracle, P):
    K, Ko, A, Ao = _laplace(gpu, oracle, P)
    N = N1 ** 3
    b = P.complex_unit_normal(N)
    sd, _ = _shifts(P, "definite", n_shifts=6)
    tol = 1e-8
    g = gpu.MSIDRS(A, b, sd, 1, variant=2, tolerance=tol, resvec=True)
    o = oracle.msidrs(Ao, b, sd, 1, variant=2, tolerance=tol, resvec_len=_maxit(N) + 1)
    assert g.flag == o.flag == 0 and np.max(g.relres) <= tol
    np.testing.assert_allclose(g.resvec[:13], o.resvec[:13], rtol=1e-8)
    for k in range(len(sd)):
        assert _rel(g.x[:, k], o.x[:, k]) <= 10 * tol


def test_msidrs_real_and_mass(gpu, oracle, P):
    """Real shifts on the real convection-diffusion operator; then the mass
    matrix argument M1 (diagonal scaling), msidrs.inc:151-160, 306-327."""
    n = 8
    N = n ** 3
    coef = P.cdr_coefficients(n)
    K = gpu.stencil7_format(n, n, n, coef)
    Ko = oracle.stencil7_format(n, n, n, coef)
    A, Ao = gpu.Matrix(K), oracle.Matrix(Ko)
    b = Ko.mv(np.ones(N))
    PT = oracle.make_p(4, N, seed=4)
    A.set_shadow(4, PT)
    sig = -np.array([0.0, 50.0, 200.0, 1000.0])
    tol = 1e-9
    g = gpu.MSIDRS(A, b, sig, 4, tolerance=tol, resvec=True)
    o = oracle.msidrs(Ao, b, sig, 4, tolerance=tol, PT=PT, resvec_len=_maxit(N) + 1)
    assert g.flag == o.flag == 0 and np.max(g.relres) <= tol
    np.testing.assert_allclose(g.resvec[:13], o.resvec[:13], rtol=1e-8)
    for k in range(len(sig)):
        assert _rel(g.x[:, k], o.x[:, k]) <= 10 * tol
    M1 = gpu.Matrix(K, P=gpu.real_precon(1, K))
    M1o = oracle.Matrix(Ko, oracle.real_precon(1, Ko))
    g = gpu.MSIDRS(A, b, sig, 4, M1=M1, tolerance=tol, resvec=True)
    o = oracle.msidrs(Ao, b, sig, 4, M1=M1o, tolerance=tol, PT=PT, resvec_len=_maxit(N) + 1)
    assert g.flag == o.flag
    np.testing.assert_allclose(g.resvec[:13], o.resvec[:13], rtol=1e-8)
    for k in range(len(sig)):
        assert _rel(g.x[:, k], o.x[:, k]) <= 1e-6


# ---------------------------------------------------------------- MSQMRIDR
@pytest.mark.parametrize("s", [1, 4, 8])
def test_msqmridr_matches_oracle(gpu, oracle, P, s):
    K, Ko, A, Ao = _laplace(gpu, oracle, P)
    N = N1 ** 3
    b = P.complex_unit_normal(N)
    PT = oracle.make_p(s, N, seed=5, cplx=True)
    A.set_shadow(s, PT)
    tol = 1e-8
    sd, _ = _shifts(P, "definite", n_shifts=6)
    g = gpu.MSQMRIDR(A, b, sd, s, tolerance=tol, resvec=True)
    o = oracle.msqmridr(Ao, b, sd, s, tolerance=tol, PT=PT, resvec_len=_maxit(N) + 1)
    assert g.flag == o.flag == 0 and np.max(g.relres) <= tol
    assert g.iterations == o.iterations
    np.testing.assert_allclose(g.resvec[:13], o.resvec[:13], rtol=1e-8)
    for k in range(len(sd)):
        assert _rel(g.x[:, k], o.x[:, k]) <= 10 * tol
    if s >= 4:
        si, _ = _shifts(P, "indefinite")
        g = gpu.MSQMRIDR(A, b, si, s, tolerance=tol, resvec=True)
        o = oracle.msqmridr(Ao, b, si, s, tolerance=tol, PT=PT, resvec_len=_maxit(N) + 1)
        assert g.flag == o.flag == 0 and np.max(g.relres) <= tol
        np.testing.assert_allclose(g.resvec[:13], o.resvec[:13], rtol=1e-8)
        assert abs(g.iterations - o.iterations) <= max(s + 1, 0.15 * o.iterations)


@pytest.mark.parametrize("prec", [64, 32])
def test_msqmridr_nested_inner_msidrs(gpu, oracle, P, prec):
    """MSQMRIDR(4) with MSIDRS(4) on [sigma, 0] as flexible preconditioner
    (msqmridr.inc:162-175, eta = cf/cf(n_sigma+1)).  Compared with the FP64
    oracle solve.

    With a complex64 inner solve the outer recurrences still assume that the
    inner residuals of all shifts are collinear (r_k = eta_k r_0); fp32
    arithmetic keeps that only to ~1e-7, so the shifted systems stop near
    1e-7 (flag 2) while the outer recurrence reports convergence."""
    K, Ko, A, Ao = _laplace(gpu, oracle, P)
    N = N1 ** 3
    b = P.complex_unit_normal(N)
    tol = 1e-8
    sd, _ = _shifts(P, "definite", n_shifts=6)
    kw = dict(tolerance=tol, inner_s=4, inner_iterations=10, inner_tolerance=0.1)
    g = gpu.MSQMRIDR(A, b, sd, 4, inner_precision=prec, **kw)
    o = oracle.msqmridr(Ao, b, sd, 4, **kw)
    # the per-shift masks of the result (no reference counterpart)
    assert not g.nonfinite_mask.any()
    np.testing.assert_array_equal(g.converged_mask, g.relres <= tol)
    if prec == 64:
        assert g.converged_mask.all()
        assert g.flag == o.flag == 0 and np.max(g.relres) <= tol
        assert g.iterations == o.iterations
        for k in range(len(sd)):
            assert _rel(g.x[:, k], o.x[:, k]) <= 10 * tol
    else:
        assert g.flag in (0, 2) and np.max(g.relres) <= 1e-6
        for k in range(len(sd)):
            assert _rel(g.x[:, k], o.x[:, k]) <= 1e-5


def test_msqmridr_real(gpu, oracle, P):
    n = 8
    N = n ** 3
    coef = P.cdr_coefficients(n)
    K = gpu.stencil7_format(n, n, n, coef)
    Ko = oracle.stencil7_format(n, n, n, coef)
    A, Ao = gpu.Matrix(K), oracle.Matrix(Ko)
    b = Ko.mv(np.ones(N))
    sig = -np.array([0.0, 50.0, 200.0, 1000.0])
    tol = 1e-9
    PT = oracle.make_p(4, N, seed=8)
    A.set_shadow(4, PT)
    g = gpu.MSQMRIDR(A, b, sig, 4, tolerance=tol, resvec=True)
    o = oracle.msqmridr(Ao, b, sig, 4, tolerance=tol, PT=PT, resvec_len=_maxit(N) + 1)
    assert g.flag == o.flag == 0 and g.iterations == o.iterations
    np.testing.assert_allclose(g.resvec[:13], o.resvec[:13], rtol=1e-8)
    for k in range(len(sig)):
        assert _rel(g.x[:, k], o.x[:, k]) <= 10 * tol
    # fp32 inner: the unshifted system converges, the shifted ones stop at the
    # fp32 collinearity level of the inner residuals
    g = gpu.MSQMRIDR(A, b, sig, 4, tolerance=tol, inner_s=2, inner_iterations=6, inner_precision=32)
    assert g.flag in (0, 2) and g.relres[0] <= tol and np.max(g.relres) <= 1e-3


def test_multishift_neumann_pipeline(gpu, oracle, P):
    """The multishift pipeline of run_ms_mr_idrs.inc: Neumann polynomial
    preconditioner, ms_parameters, MSQMRIDR on the preconditioned shifts,
    scaleback; the original systems (K - sigma_k I) x_k = b are checked."""
    K, Ko, A, Ao = _laplace(gpu, oracle, P)
    N = N1 ** 3
    b = P.complex_unit_normal(N)
    sd, lam = _shifts(P, "definite", n_shifts=6)
    A.preconditioner(1, 4, center=lam / 2)
    Ao.preconditioner(1, 4, center=lam / 2)
    sp = A.ms_parameters(sd)
    np.testing.assert_allclose(sp, Ao.ms_parameters(sd), rtol=1e-12)
    tol = 1e-9
    g = gpu.MSQMRIDR(A, b, sp, 4, tolerance=tol)
    o = oracle.msqmridr(Ao, b, sp, 4, tolerance=tol)
    assert g.flag == o.flag == 0
    X = A.ms_scaleback(sd, b, g.x)
    Xo = Ao.ms_scaleback(o.x)
    for k in range(len(sd)):
        r = b - K * X[:, k] + sd[k] * X[:, k]
        assert np.linalg.norm(r) <= 1e-7 * np.linalg.norm(b)
        assert _rel(X[:, k], Xo[:, k]) <= 1e-7


def test_multishift_flags_and_errors(gpu, P):
    n = 6
    K = gpu.stencil7_format(n, n, n, P.laplace_coefficients(n))
    A = gpu.Matrix(K, complex=True)
    N = n ** 3
    b = P.complex_unit_normal(N)
    sig, _ = P.multishift_shifts(n, n_shifts=3, lo=1.2, hi=4.0)
    r = gpu.MSIDRS(A, np.zeros(N), sig, 4, resvec=True)
    assert r.flag == 0 and r.iterations == 0 and np.all(r.x == 0)
    r = gpu.MSQMRIDR(A, np.zeros(N), sig, 4)
    assert r.flag == 0 and r.iterations == 0 and np.all(r.x == 0)
    r = gpu.MSIDRS(A, b, sig, 4, tolerance=1e-14, maximum_iterations=3)
    assert r.flag == 1 and r.iterations == 3
    r = gpu.MSQMRIDR(A, b, sig, 4, tolerance=1e-14, maximum_iterations=7)
    assert r.flag == 1 and r.iterations == 7
    with pytest.raises(gpu.IDRSError) as e:
        gpu.MSIDRS(A, b, sig, 4, tolerance=-1.0)
    assert e.value.status == 1 and "tolerance" in str(e.value)
    with pytest.raises(gpu.IDRSError) as e:
        gpu.MSIDRS(A, b, sig, 17)
    assert e.value.status == 5
    with pytest.raises(gpu.IDRSError) as e:
        gpu.MSIDRS(A, b, np.linspace(1, 2, 65) * (1 + 0j), 2)
    assert e.value.status == 5
    with pytest.raises(gpu.IDRSError) as e:
        gpu.MSIDRS(A, b, sig, 4, variant=2)
    assert e.value.status == 1
    with pytest.raises(gpu.IDRSError) as e:
        gpu.MSQMRIDR(A, b, np.linspace(1, 2, 64) * (1 + 0j), 2)
    assert e.value.status == 5
    with pytest.raises(gpu.IDRSError):
        gpu.MSQMRIDR(A, b, sig, 4, inner_s=0, inner_iterations=3)
    with pytest.raises(gpu.IDRSError):
        gpu.MSIDRS(A, b, [], 4)
