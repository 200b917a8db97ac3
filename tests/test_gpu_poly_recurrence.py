"""fp64 products, IDR(s) and the PP_IDRS pipeline with the polynomial
preconditioner evaluated by the three-term recurrence of its Jacobi matrix
(idrs_matrix_set_poly_eval / pp options poly_eval = 1; Chebyshev and Neumann,
matrix_module.f90:851-941) instead of the reference's Horner rpolpre
(:266-284), against the oracle's restatement of the same recurrence."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P(gpu):
    return gpu.problems


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _ops(gpu, oracle, P, fmt, n):
    coef = P.cdr_coefficients(n)
    N = n ** 3
    if fmt == "stencil":
        K, Ko = gpu.stencil7_format(n, n, n, coef), oracle.stencil7_format(n, n, n, coef)
    else:
        rp, ci, vals = P.stencil_to_crs(n, n, n, coef)
        K, Ko = gpu.crs_format(N, N, rp, ci, rval=vals), oracle.crs_format(N, N, rp, ci, vals)
    return N, K, Ko


@pytest.mark.parametrize("fmt", ["stencil", "crs"])
@pytest.mark.parametrize("prec,degree,kw", [(2, 8, dict(foci=[0.05, 1.9])), (1, 4, dict(center=1.0)),
                                            (2, 1, dict(foci=[0.2, 1.8]))])
def test_fp64_recurrence_products(gpu, oracle, P, fmt, prec, degree, kw):
    """A*v and scaleback(A, b, y) with the recurrence: GPU against the oracle
    (rtol 1e-12: the same recurrence, rounded in another order), and against
    Horner (the same polynomial: agreement to the cancellation of Horner)."""
    n = 14
    N, K, Ko = _ops(gpu, oracle, P, fmt, n)
    A = gpu.Matrix(K, P=gpu.real_precon(1, K))
    Ao = oracle.Matrix(Ko, P=oracle.real_precon(1, Ko))
    A.preconditioner(prec, degree, **kw)
    Ao.preconditioner(prec, degree, **kw)
    v = np.random.default_rng(degree).standard_normal(N)
    w_h, y_h = A * v, A.scaleback(v, v)
    A.set_poly_eval(gpu.POLY_RECURRENCE)
    Ao.set_poly_eval(1)
    w, y = A * v, A.scaleback(v, v)
    wo, yo = Ao.matvec(v), Ao.scaleback(v, v)
    np.testing.assert_allclose(w, wo, rtol=1e-12, atol=1e-12 * np.abs(wo).max())
    np.testing.assert_allclose(y, yo, rtol=1e-12, atol=1e-12 * np.abs(yo).max())
    assert _rel(w, w_h) <= 1e-10 and _rel(y, y_h) <= 1e-10
    A.set_poly_eval(gpu.POLY_HORNER)
    np.testing.assert_array_equal(A * v, w_h)


def test_fp64_recurrence_idrs_matches_oracle(gpu, oracle, P):
    """IDR(4) on the Chebyshev(4)-preconditioned CRS operator with the
    recurrence, shadow space injected: residual history and solution."""
    n = 10
    N, K, Ko = _ops(gpu, oracle, P, "crs", n)
    A = gpu.Matrix(K, P=gpu.real_precon(1, K))
    Ao = oracle.Matrix(Ko, P=oracle.real_precon(1, Ko))
    for M in (A, Ao):
        M.preconditioner(2, 4, foci=[0.05, 1.9])
    A.set_poly_eval(gpu.POLY_RECURRENCE)
    Ao.set_poly_eval(1)
    b = Ko.mv(np.ones(N))
    PT = oracle.make_p(4, N, seed=3)
    A.set_shadow(4, PT)
    g = gpu.IDRS(A, b, 4, tolerance=1e-10, resvec=True)
    o = oracle.idrs(Ao, b, 4, tolerance=1e-10, PT=PT, resvec_len=min(2 * N, 1000) + 1)
    assert g.flag == o.flag == 0
    assert abs(g.iterations - o.iterations) <= 5
    k = min(12, g.iterations)
    np.testing.assert_allclose(g.resvec[:k], o.resvec[:k], rtol=1e-8)
    xg, xo = A.scaleback(b, g.x), Ao.scaleback(b, o.x)
    assert _rel(xg, xo) <= 1e-9


def test_pp_idrs_qmridr_recurrence_matches_oracle(gpu, oracle, P):
    """PP_IDRS: Ritz-estimated Chebyshev(8), diagonal scaling, QMRIDR(8) with
    poly_eval = 1 on both sides; the fp64 solve meets 1e-8 on the original
    system and x agrees with the oracle's to 10 tol."""
    n = 14
    coef = P.cdr_coefficients(n)
    N = n ** 3
    K, Ko = gpu.stencil7_format(n, n, n, coef), oracle.stencil7_format(n, n, n, coef)
    b = Ko.mv(np.ones(N))
    kw = dict(method=0, s=8, tol=1e-8, preconditioner=2, degree=8, n_ritz=20, poly_eval=1)
    g = gpu.PP_IDRS(K, b, P=gpu.real_precon(1, K), **kw)
    o = oracle.pp_idrs(Ko, b, P=oracle.real_precon(1, Ko), **kw)
    assert g.flag == o.flag == 0 and g.nritz == o.nritz == 20
    np.testing.assert_allclose(g.foci, o.foci, rtol=1e-6)
    assert abs(g.iterations - o.iterations) <= 9
    assert g.relres_original <= 1e-8 * 1.01 and o.relres_original <= 1e-8 * 1.01
    assert _rel(g.x, o.x) <= 1e-7


def test_poly_eval_rejects_bad_modes(gpu, P):
    K = gpu.stencil7_format(4, 4, 4, P.cdr_coefficients(4))
    A = gpu.Matrix(K)
    with pytest.raises(gpu.IDRSError):
        A.set_poly_eval(2)
    with pytest.raises(gpu.IDRSError):
        gpu.PP_IDRS(K, np.ones(64), method=0, s=2, tol=1e-6, poly_eval=5)
