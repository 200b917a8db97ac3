"""Deflation on the GPU (make_deflation, Pmul, add_deflation;
matrix_module.f90:1284-1623) against the oracle: the projector, a deflated
IDR(s) solve with its scale-back, a deflated QMRIDR solve, and the
multishift projector I - V V^H on an invariant subspace."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P(gpu):
    return gpu.problems


def _cdr(gpu, oracle, P, n):
    N = n ** 3
    rp, ci, kv = P.stencil_to_crs(n, n, n, P.cdr_coefficients(n))
    rows = np.repeat(np.arange(N), np.diff(rp))
    D = np.zeros((N, N))
    D[rows, ci - 1] = kv
    return (N, gpu.crs_format(N, N, rp, ci, rval=kv), oracle.crs_format(N, N, rp, ci, kv), D)


@pytest.mark.parametrize("cplx", [False, True])
def test_pmul_matches_oracle(gpu, oracle, P, cplx):
    N, Kg, Ko, _ = _cdr(gpu, oracle, P, 6)
    rng = np.random.default_rng(1)
    V = rng.standard_normal((N, 4)) + (1j * rng.standard_normal((N, 4)) if cplx else 0)
    if cplx:
        A = gpu.Matrix(Kg, P=gpu.complex_precon(1, Kg), complex=True)
        Ao = oracle.Matrix(Ko, P=oracle.complex_precon(1, Ko), cplx=True)
    else:
        A = gpu.Matrix(Kg, P=gpu.real_precon(1, Kg))
        Ao = oracle.Matrix(Ko, P=oracle.real_precon(1, Ko))
    A.make_deflation(V)
    Ao.make_deflation(V)
    w = rng.standard_normal(N) + (1j * rng.standard_normal(N) if cplx else 0)
    np.testing.assert_allclose(A.pmul(w), Ao.pmul(w), rtol=1e-11, atol=1e-11)
    np.testing.assert_allclose(A * w, Ao.matvec(w), rtol=1e-11, atol=1e-11)
    b = rng.standard_normal(N) + (1j * rng.standard_normal(N) if cplx else 0)
    np.testing.assert_allclose(A.scaleback(b, w), Ao.scaleback(b, w), rtol=1e-11, atol=1e-13)
    A.make_deflation(None)
    np.testing.assert_array_equal(A.pmul(w), w)


@pytest.mark.parametrize("method", ["idrs", "qmridr"])
def test_deflated_solve_matches_oracle(gpu, oracle, P, method):
    N, Kg, Ko, D = _cdr(gpu, oracle, P, 10)
    rng = np.random.default_rng(2)
    V = rng.standard_normal((N, 3))
    A = gpu.Matrix(Kg, P=gpu.real_precon(1, Kg))
    Ao = oracle.Matrix(Ko, P=oracle.real_precon(1, Ko))
    A.make_deflation(V)
    Ao.make_deflation(V)
    b = rng.standard_normal(N)
    pb = Ao.pmul(b)
    if method == "idrs":
        g = gpu.IDRS(A, pb, 4, tolerance=1e-10, maximum_iterations=3000)
        o = oracle.idrs(Ao, pb, 4, tolerance=1e-10, maximum_iterations=3000)
    else:
        g = gpu.QMRIDR(A, pb, 4, tolerance=1e-10, maximum_iterations=3000)
        o = oracle.qmridr(Ao, pb, 4, tolerance=1e-10, maximum_iterations=3000)
    assert g.flag == o.flag == 0
    assert abs(g.iterations - o.iterations) <= max(3, 0.05 * o.iterations)
    x, xo = A.scaleback(b, g.x), Ao.scaleback(b, o.x)
    np.testing.assert_allclose(x, xo, rtol=0, atol=1e-7 * np.abs(xo).max())
    assert np.linalg.norm(b - D @ x) <= 1e-8 * np.linalg.norm(b)
    with pytest.raises(gpu.IDRSError):  # no deflated fp32 operator
        gpu.QMRIDR(A, pb, 4, tolerance=1e-8, inner_iterations=20, inner_precision=32)


def test_multishift_deflation_invariant_subspace(gpu, oracle, P):
    N, Kg, Ko, D = _cdr(gpu, oracle, P, 6)
    As = D / np.diag(D)[None, :]
    ev, EV = np.linalg.eig(As)
    V, _ = np.linalg.qr(EV[:, np.argsort(np.abs(ev))[:2]])
    A = gpu.Matrix(Kg, P=gpu.complex_precon(1, Kg), complex=True, multishift=True)
    Ao = oracle.Matrix(Ko, P=oracle.complex_precon(1, Ko), cplx=True, multishift=True)
    A.make_deflation(V)
    Ao.make_deflation(V)
    rng = np.random.default_rng(3)
    b = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    sig = np.array([0.1, 0.3 + 0.1j, -0.2j])
    sp, spo = A.ms_parameters(sig), Ao.ms_parameters(sig)
    pb = A.pmul(b)
    np.testing.assert_allclose(pb, Ao.pmul(b), rtol=1e-12, atol=1e-12)
    g = gpu.MSIDRS(A, pb, sp, 4, tolerance=1e-10, maximum_iterations=3000)
    o = oracle.msidrs(Ao, Ao.pmul(b), spo, 4, tolerance=1e-10, maximum_iterations=3000)
    assert g.flag == o.flag == 0
    assert abs(g.iterations - o.iterations) <= 3
    X = A.ms_scaleback(sig, b, g.x)
    Xo = Ao.ms_scaleback(o.x, b)
    np.testing.assert_allclose(X, Xo, rtol=0, atol=1e-7 * np.abs(Xo).max())
    Dm = np.diag(np.diag(D))
    for k, s in enumerate(sig):
        assert np.linalg.norm(b - (D - s * Dm) @ X[:, k]) <= 1e-8 * np.linalg.norm(b)
