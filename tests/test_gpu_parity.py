"""CUDA path (through the C ABI) against the oracle on the same inputs.

Tolerances: products and single vector passes rtol 1e-12; iteration
histories with an injected shared shadow space rtol 1e-8 over the first 12
iterations (rounding differs: fused reductions sum in a different order, and
non-monotone IDR(s) histories amplify it to ~1e-9 by iteration 12);
converged solutions ||x - x_ref|| <= 10 * tol * ||x_ref|| with the true
relative residual <= tol (the parity contract of the solve path).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P(gpu):
    return gpu.problems


def _cdr(P, n):
    coef = P.cdr_coefficients(n)
    rp, ci, vals = P.stencil_to_crs(n, n, n, coef)
    return coef, rp, ci, vals


def _rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


# ----------------------------------------------------------------- products
def test_user_mv_all_formats(gpu, oracle, P):
    rng = np.random.default_rng(3)
    n = 9
    coef, rp, ci, vals = _cdr(P, n)
    N = n ** 3
    v = rng.standard_normal(N)
    vc = v + 1j * rng.standard_normal(N)
    K = gpu.crs_format(N, N, rp, ci, rval=vals)
    Ko = oracle.crs_format(N, N, rp, ci, vals)
    np.testing.assert_allclose(K * v, Ko.mv(v), rtol=1e-12, atol=1e-9)
    np.testing.assert_allclose(K * vc, Ko.mv(vc), rtol=1e-12, atol=1e-9)
    S = gpu.stencil7_format(n, n, n, coef)
    np.testing.assert_allclose(S * v, Ko.mv(v), rtol=1e-12, atol=1e-9)
    np.testing.assert_allclose(S * vc, Ko.mv(vc), rtol=1e-12, atol=1e-9)
    # COO in a shuffled order
    rows = np.repeat(np.arange(N), np.diff(rp)) + 1
    perm = rng.permutation(len(vals))
    C_ = gpu.coo_format(N, N, len(vals), rows[perm], ci[perm], rval=vals[perm])
    Co = oracle.coo_format(N, N, rows[perm], ci[perm], vals[perm])
    np.testing.assert_allclose(C_ * v, Co.mv(v), rtol=1e-12, atol=1e-9)
    # complex CRS values
    cv = vals + 1j * rng.standard_normal(len(vals))
    Kc = gpu.crs_format(N, N, rp, ci, cval=cv)
    Kco = oracle.crs_format(N, N, rp, ci, cv)
    np.testing.assert_allclose(Kc * vc, Kco.mv(vc), rtol=1e-12, atol=1e-9)
    # CDS and dense
    m = 40
    hb = 3
    band = rng.standard_normal((m, 2 * hb + 1))
    D = gpu.cds_format(m, m, hb, rband=band)
    Do = oracle.cds_format(m, m, hb, band)
    w = rng.standard_normal(m)
    np.testing.assert_allclose(D * w, Do.mv(w), rtol=1e-12, atol=1e-12)
    M = rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m))
    Dm = gpu.dense_format(cmat=M)
    np.testing.assert_allclose(Dm * (w + 0j), M @ w, rtol=1e-12, atol=1e-12)


def test_empty_rows_and_pattern_only(gpu, oracle):
    N = 6
    rp = np.array([1, 1, 3, 3, 4, 4, 6])  # rows 0, 2 and 4 empty
    ci = np.array([1, 2, 3, 5, 6])
    K = gpu.crs_format(N, N, rp, ci)
    Ko = oracle.crs_format(N, N, rp, ci)
    v = np.arange(1.0, N + 1)
    np.testing.assert_allclose(K * v, Ko.mv(v))
    assert (K * v)[0] == 0.0


def test_operator_polynomial_and_scaling(gpu, oracle, P):
    """A*v = K D^-1 p(K D^-1) v (matrix_module.f90:152-284), v/A, scaleback."""
    n = 8
    coef, rp, ci, vals = _cdr(P, n)
    N = n ** 3
    v = np.random.default_rng(5).standard_normal(N)
    for fmt in ("crs", "stencil"):
        if fmt == "crs":
            K = gpu.crs_format(N, N, rp, ci, rval=vals)
        else:
            K = gpu.stencil7_format(n, n, n, coef)
        Ko = oracle.crs_format(N, N, rp, ci, vals)
        Dp = gpu.real_precon(1, K)
        Do = oracle.real_precon(1, Ko)
        A = gpu.Matrix(K, P=Dp)
        Ao = oracle.Matrix(Ko, Do)
        A.preconditioner(2, 5, foci=[0.2, 1.8])
        Ao.preconditioner(2, 5, foci=[0.2, 1.8])
        np.testing.assert_allclose(A.alpha_p, oracle.chebyshev(5, np.array([0.2, 1.8])), rtol=1e-13)
        np.testing.assert_allclose(A * v, Ao.matvec(v), rtol=1e-11, atol=1e-11 * np.abs(Ao.matvec(v)).max())
        np.testing.assert_allclose(v / A, Ao.precon(v), rtol=1e-14)
        np.testing.assert_allclose(A.scaleback(v, v), Ao.scaleback(v, v), rtol=1e-11,
                                   atol=1e-12 * np.abs(Ao.scaleback(v, v)).max())
    np.testing.assert_allclose(gpu.real_diagonal(gpu.crs_format(N, N, rp, ci, rval=vals)),
                               oracle.real_diagonal(oracle.crs_format(N, N, rp, ci, vals)))


# -------------------------------------------------------------------- IDRS
@pytest.mark.parametrize("s", [1, 2, 4, 8])
def test_idrs_matches_oracle_step_by_step(gpu, oracle, P, s):
    n = 10
    coef, rp, ci, vals = _cdr(P, n)
    N = n ** 3
    K = gpu.crs_format(N, N, rp, ci, rval=vals)
    A = gpu.Matrix(K)
    Ko = oracle.crs_format(N, N, rp, ci, vals)
    Ao = oracle.Matrix(Ko)
    b = Ko.mv(np.ones(N))
    PT = oracle.make_p(s, N, seed=7)
    A.set_shadow(s, PT)
    tol = 1e-8
    g = gpu.IDRS(A, b, s, tolerance=tol, resvec=True, H=12)
    o = oracle.idrs(Ao, b, s, tolerance=tol, PT=PT, resvec_len=min(2 * N, 1000) + 1, H_shape=(13, 12))
    assert g.flag == 0 and o.flag == 0
    assert g.relres <= tol
    k = min(12, g.iterations, o.iterations)
    np.testing.assert_allclose(g.resvec[:k + 1], o.resvec[:k + 1], rtol=1e-8)
    assert abs(g.iterations - o.iterations) <= 2
    assert _rel(g.x, o.x) <= 10 * tol
    np.testing.assert_allclose(g.x, 1.0, atol=1e-6)
    np.testing.assert_allclose(g.H, o.H, rtol=1e-8, atol=1e-8 * np.abs(o.H).max())


def test_bicgstab_variant(gpu, oracle, P):
    import os
    rp, ci, vals, b = P.toeplitz_real()
    A = gpu.Matrix(gpu.crs_format(60, 60, rp, ci, rval=vals))
    g = gpu.IDRS(A, b, 1, variant=2, tolerance=1e-14, maximum_iterations=80, resvec=True)
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "bicgstab_toeplitz_real.npz"))
    np.testing.assert_allclose(g.resvec[2:2 * 12 + 1:2], d["resnorm"][:12], rtol=1e-9)


@pytest.mark.parametrize("s", [1, 2, 4, 8])
def test_finite_termination_gpu(gpu, P, s):
    """E/TOEPLITZ/toeplitz.f90:134-138 on the CUDA path."""
    rp, ci, vals, b = P.toeplitz_real()
    A = gpu.Matrix(gpu.crs_format(60, 60, rp, ci, rval=vals))
    r = gpu.IDRS(A, b, s, tolerance=1e-8, maximum_iterations=4000)
    assert r.flag == 0 and r.iterations <= 60 + 60 // s and r.relres < 1e-8
    q = gpu.QMRIDR(A, b, s, tolerance=1e-8, maximum_iterations=4000)
    assert q.flag == 0 and q.iterations <= 60 + 60 // s and q.relres < 1e-8


@pytest.mark.parametrize("s", [1, 4, 8, 16])
def test_complex_toeplitz_gpu(gpu, oracle, P, s):
    rp, ci, vals, b = P.toeplitz_complex()
    A = gpu.Matrix(gpu.crs_format(200, 200, rp, ci, cval=vals), complex=True)
    Ao = oracle.Matrix(oracle.crs_format(200, 200, rp, ci, vals), cplx=True)
    PT = oracle.make_p(s, 200, seed=3, cplx=True)
    A.set_shadow(s, PT)
    g = gpu.IDRS(A, b, s, tolerance=1e-12, maximum_iterations=4000, resvec=True)
    o = oracle.idrs(Ao, b, s, tolerance=1e-12, maximum_iterations=4000, PT=PT, resvec_len=4001)
    assert g.flag == 0 and g.relres < 1e-12
    np.testing.assert_allclose(g.resvec[:10], o.resvec[:10], rtol=1e-9)
    assert _rel(g.x, o.x) <= 1e-10
    q = gpu.QMRIDR(A, b, s, tolerance=1e-12, maximum_iterations=4000)
    qo = oracle.qmridr(Ao, b, s, tolerance=1e-12, maximum_iterations=4000, PT=PT)
    assert q.flag == 0 and q.relres < 1e-12
    assert _rel(q.x, qo.x) <= 1e-10


# ------------------------------------------------------------------ QMRIDR
@pytest.mark.parametrize("s", [1, 4, 8])
def test_qmridr_matches_oracle(gpu, oracle, P, s):
    n = 10
    coef, rp, ci, vals = _cdr(P, n)
    N = n ** 3
    K = gpu.stencil7_format(n, n, n, coef)
    A = gpu.Matrix(K, P=gpu.real_precon(1, K))
    Ko = oracle.stencil7_format(n, n, n, coef)
    Ao = oracle.Matrix(Ko, oracle.real_precon(1, Ko))
    A.preconditioner(2, 4, foci=[0.05, 1.9])
    Ao.preconditioner(2, 4, foci=[0.05, 1.9])
    b = Ko.mv(np.ones(N))
    PT = oracle.make_p(s, N, seed=5)
    A.set_shadow(s, PT)
    tol = 1e-9
    g = gpu.QMRIDR(A, b, s, tolerance=tol, resvec=True)
    o = oracle.qmridr(Ao, b, s, tolerance=tol, PT=PT, resvec_len=min(2 * N, 1000) + 1)
    assert g.flag == 0 and o.flag == 0
    k = min(12, g.iterations)
    np.testing.assert_allclose(g.resvec[:k + 1], o.resvec[:k + 1], rtol=1e-8)
    assert _rel(g.x, o.x) <= 10 * tol
    assert g.relres <= tol


@pytest.mark.parametrize("prec", [64, 32])
def test_qmridr_flexible_inner(gpu, oracle, P, prec):
    """QMRIDR(8) with an inner IDR(4) (qmridr.inc:161-173); fp32 inner for
    the mixed form.  Compared with the FP64 oracle solve."""
    n = 12
    coef, rp, ci, vals = _cdr(P, n)
    N = n ** 3
    K = gpu.stencil7_format(n, n, n, coef)
    A = gpu.Matrix(K, P=gpu.real_precon(1, K))
    Ko = oracle.stencil7_format(n, n, n, coef)
    Ao = oracle.Matrix(Ko, oracle.real_precon(1, Ko))
    b = Ko.mv(np.ones(N))
    tol = 1e-8
    g = gpu.QMRIDR(A, b, 8, tolerance=tol, inner_s=4, inner_iterations=10, inner_tolerance=0.1,
                   inner_precision=prec)
    o = oracle.qmridr(Ao, b, 8, tolerance=tol, inner_s=4, inner_iterations=10, inner_tolerance=0.1)
    assert g.flag == 0 and g.relres <= tol
    assert _rel(g.x, o.x) <= 10 * tol
    if prec == 64:
        # The inner solve stops after 10 iterations at a 0.3-ish relative
        # residual, so the flexible outer iteration amplifies rounding.
        assert abs(g.iterations - o.iterations) <= max(4, int(0.35 * o.iterations))


# -------------------------------------------------------- options & errors
def test_options_x0_omega_M1(gpu, oracle, P):
    n = 8
    coef, rp, ci, vals = _cdr(P, n)
    N = n ** 3
    K = gpu.crs_format(N, N, rp, ci, rval=vals)
    A = gpu.Matrix(K)
    Ko = oracle.crs_format(N, N, rp, ci, vals)
    Ao = oracle.Matrix(Ko)
    b = Ko.mv(np.ones(N))
    PT = oracle.make_p(4, N, seed=2)
    A.set_shadow(4, PT)
    x0 = np.full(N, 0.5)
    omega = np.array([1e-3, 2e-3, 5e-4])
    g = gpu.IDRS(A, b, 4, tolerance=1e-8, x0=x0, omega=omega, resvec=True)
    o = oracle.idrs(Ao, b, 4, tolerance=1e-8, x0=x0, omega=omega, PT=PT, resvec_len=min(2 * N, 1000) + 1)
    np.testing.assert_allclose(g.resvec[:9], o.resvec[:9], rtol=1e-9)
    assert g.flag == o.flag
    # M1 = diagonal scaling used as the preconditioner argument
    M1 = gpu.Matrix(K, P=gpu.real_precon(1, K))
    M1o = oracle.Matrix(Ko, oracle.real_precon(1, Ko))
    g = gpu.IDRS(A, b, 4, M1=M1, tolerance=1e-8, resvec=True)
    o = oracle.idrs(Ao, b, 4, M1=M1o, tolerance=1e-8, PT=PT, resvec_len=min(2 * N, 1000) + 1)
    np.testing.assert_allclose(g.resvec[:9], o.resvec[:9], rtol=1e-9)
    assert g.flag == 0 and _rel(g.x, o.x) <= 1e-7


def test_flags_and_errors(gpu, P):
    rp, ci, vals, b = P.toeplitz_real()
    A = gpu.Matrix(gpu.crs_format(60, 60, rp, ci, rval=vals))
    r = gpu.IDRS(A, b, 4, tolerance=1e-12, maximum_iterations=5)
    assert r.flag == 1 and r.iterations == 5
    r = gpu.IDRS(A, np.zeros(60), 4)
    assert r.flag == 0 and r.iterations == 0 and np.all(r.x == 0)
    with pytest.raises(gpu.IDRSError) as e:
        gpu.IDRS(A, b, 4, tolerance=-1.0)
    assert e.value.status == 1 and "tolerance" in str(e.value)
    with pytest.raises(gpu.IDRSError) as e:
        gpu.IDRS(A, b, 17)
    assert e.value.status == 5
    with pytest.raises(gpu.IDRSError):
        gpu.QMRIDR(A, b, 4, inner_s=0, inner_iterations=3)
    bn = b.copy()
    bn[3] = np.nan
    r = gpu.IDRS(A, bn, 2, maximum_iterations=6)
    assert r.flag == 1 and not np.isfinite(r.relres)


def test_pp_idrs_matches_oracle(gpu, oracle, P):
    """PP_IDRS: Ritz-estimated Chebyshev(8) with diagonal scaling, QMRIDR(8)."""
    n = 14
    coef = P.cdr_coefficients(n)
    N = n ** 3
    K = gpu.stencil7_format(n, n, n, coef)
    Ko = oracle.stencil7_format(n, n, n, coef)
    b = Ko.mv(np.ones(N))
    g = gpu.PP_IDRS(K, b, P=gpu.real_precon(1, K), method=0, s=8, tol=1e-8, preconditioner=2,
                    degree=8, n_ritz=20)
    o = oracle.pp_idrs(Ko, b, P=oracle.real_precon(1, Ko), method=0, s=8, tol=1e-8,
                       preconditioner=2, degree=8, n_ritz=20)
    assert g.flag == 0 and g.nritz == o.nritz == 20
    np.testing.assert_allclose(g.foci, o.foci, rtol=1e-6)
    assert g.relres_original <= 1e-8 * 1.01
    assert _rel(g.x, o.x) <= 1e-7


def test_mixed_precision_with_chebyshev(gpu, P):
    """fp32 inner IDR(4) on a Chebyshev(8)-preconditioned operator (the
    polynomial evaluated by its stable Jacobi recurrence) inside the FP64
    QMRIDR(8): converges to 1e-8 in a few outer iterations."""
    n = 32
    coef = P.cdr_coefficients(n)
    N = n ** 3
    K = gpu.stencil7_format(n, n, n, coef)
    b = K * np.ones(N)
    r = gpu.PP_IDRS(K, b, P=gpu.real_precon(1, K), method=0, s=8, tol=1e-8, maxit=60, preconditioner=2,
                    degree=8, n_ritz=20, in_s=4, in_it=300, in_tol=1e-2, inner_precision=32)
    assert r.flag == 0 and r.iterations <= 10
    assert r.relres_original <= 1.01e-8
    np.testing.assert_allclose(r.x, 1.0, atol=1e-6)


@pytest.mark.parametrize("dims", [(12, 12, 12), (256, 3, 5), (20, 9, 33), (30, 30, 30), (260, 4, 4), (4, 1, 7),
                                  (64, 7, 9), (8, 5, 3), (128, 33, 20), (16, 16, 16), (256, 17, 6)])
@pytest.mark.parametrize("poly", ["chebyshev", "neumann"])
def test_fp32_chain_matches_fp64(gpu, P, dims, poly):
    """The fp32 operator of the inner solves (polynomial by its recurrence,
    two stencil steps per pass where nx <= 256 -- eight x-points per thread
    for nx % 8 == 0, four for nx % 4 == 0 -- single steps otherwise) against
    the fp64 operator: agreement to fp32 accuracy."""
    nx, ny, nz = dims
    coef = P.cdr_coefficients(max(nx, ny, nz))
    K = gpu.stencil7_format(nx, ny, nz, coef)
    A = gpu.Matrix(K, P=gpu.real_precon(1, K))
    if poly == "chebyshev":
        A.preconditioner(2, 8, foci=[0.05, 1.9])
    else:
        A.preconditioner(1, 6, center=1.0)
    v = np.random.default_rng(nx + ny + nz).standard_normal(nx * ny * nz)
    w64 = A * v
    w32 = A.matvec32(v)
    assert _rel(w32, w64) <= 2e-5
