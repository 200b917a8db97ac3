"""Every mixed-precision result states its relative error against an FP64
solve (fp64_check): PP_IDRS / PP_MR_IDRS run the FP64 form of the method
(QMRIDR(s) without inner solves) from x0 = 0 inside the library; QMRIDR,
MSQMRIDR and PP_MS_IDRS call it a second time from Python.  Checked here: the
reported error against an independent FP64 solve, the correctness bar
||x - x64|| <= 10 tol ||x64||, the defaults (on for mixed host calls, off for
FP64 and device-pointer calls) and that a sequence keeps its warm starts."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-8


@pytest.fixture(scope="module")
def prob(gpu):
    n = 24
    K = gpu.stencil7_format(n, n, n, gpu.problems.cdr_coefficients(n))
    return K, gpu.real_precon(1, K), K * np.ones(n ** 3)


MIXED = dict(method=0, s=8, maxit=60, preconditioner=2, degree=8, n_ritz=20, in_s=4, in_it=40,
             in_tol=1e-2, inner_precision=32, poly_eval=1)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_pp_idrs_mixed_states_its_error(gpu, prob):
    K, D, b = prob
    r = gpu.PP_IDRS(K, b, P=D, tol=TOL, **MIXED)
    assert r.flag == 0 and r.relres_original <= TOL
    assert r.fp64_flag == 0 and r.fp64_relres_original <= 1e-11 * 1.01
    assert 0 < r.rel_err_vs_fp64 <= 10 * TOL
    assert r.seconds_fp64_check > 0
    # against an FP64 solve made separately (started from the Ritz set-up's
    # x0, so it differs from the library's x64 only at the 1e-11 level)
    q = gpu.PP_IDRS(K, b, P=D, tol=1e-11, method=0, s=8, maxit=1000, preconditioner=2, degree=8,
                    n_ritz=20, poly_eval=1)
    assert q.rel_err_vs_fp64 is None  # an FP64 call is not checked by default
    assert abs(r.rel_err_vs_fp64 - _rel(r.x, q.x)) <= 1e-9 + 0.05 * r.rel_err_vs_fp64
    # the check changes neither the solution nor the solve
    r0 = gpu.PP_IDRS(K, b, P=D, tol=TOL, fp64_check=False, **MIXED)
    assert r0.rel_err_vs_fp64 is None
    np.testing.assert_array_equal(r0.x, r.x)
    assert r0.iterations == r.iterations and r0.inner_iterations == r.inner_iterations


def test_device_pointer_calls_check_on_request(gpu, prob):
    import torch
    K, D, b = prob
    bd = torch.from_numpy(b).cuda()
    xd = torch.empty_like(bd)
    r = gpu.PP_IDRS(K, bd.data_ptr(), P=D, tol=TOL, x_out=xd.data_ptr(), **MIXED)
    assert r.rel_err_vs_fp64 is None
    r = gpu.PP_IDRS(K, bd.data_ptr(), P=D, tol=TOL, x_out=xd.data_ptr(), fp64_check=True, **MIXED)
    assert r.fp64_flag == 0 and 0 < r.rel_err_vs_fp64 <= 10 * TOL


def test_pp_mr_idrs_checks_every_rhs_and_keeps_warm_starts(gpu, prob):
    K, D, b = prob
    rng = np.random.default_rng(4)
    B = np.stack([b, b * (1 + 0.1 * rng.standard_normal(len(b)))], axis=1)
    r = gpu.PP_MR_IDRS(K, B, P=D, tol=TOL, **MIXED)
    r0 = gpu.PP_MR_IDRS(K, B, P=D, tol=TOL, fp64_check=False, **MIXED)
    assert r0.rel_err_vs_fp64 is None
    assert list(r.fp64_flags) == [0, 0]
    assert np.all(r.rel_err_vs_fp64 > 0) and np.all(r.rel_err_vs_fp64 <= 10 * TOL)
    np.testing.assert_array_equal(r.iterations, r0.iterations)
    np.testing.assert_array_equal(r.x, r0.x)


def test_qmridr_and_msqmridr_state_their_errors(gpu, prob):
    K, D, b = prob
    A = gpu.Matrix(K, P=D)
    A.preconditioner(2, 8, foci=[0.05, 1.9])
    q = gpu.QMRIDR(A, b, 8, tolerance=TOL, maximum_iterations=60, inner_s=4, inner_iterations=40,
                   inner_tolerance=1e-2, inner_precision=32)
    assert q.flag == 0 and q.fp64_flag == 0
    # the check's own call: FP64 QMRIDR(8) to 1e-11 with min(2n, 5000) iterations
    x64 = gpu.QMRIDR(A, b, 8, tolerance=1e-11, maximum_iterations=5000).x
    assert q.rel_err_vs_fp64 == pytest.approx(_rel(q.x, x64), rel=1e-12)
    assert 0 < q.rel_err_vs_fp64 <= 1e-6
    n = 12
    Ks = gpu.stencil7_format(n, n, n, gpu.problems.laplace_coefficients(n))
    Am = gpu.Matrix(Ks, complex=True)
    bm = gpu.problems.complex_unit_normal(n ** 3)
    sig, _ = gpu.problems.multishift_shifts(n, n_shifts=4, lo=1.2, hi=4.0)
    m = gpu.MSQMRIDR(Am, bm, sig, 4, tolerance=TOL, maximum_iterations=200, inner_s=4,
                     inner_iterations=20, inner_tolerance=0.1, inner_precision=32)
    assert m.rel_err_vs_fp64.shape == (4,) and np.all(np.isfinite(m.rel_err_vs_fp64))
    m64 = gpu.MSQMRIDR(Am, bm, sig, 4, tolerance=1e-11, maximum_iterations=min(2 * n ** 3, 5000))
    np.testing.assert_allclose(m.rel_err_vs_fp64, np.linalg.norm(m.x - m64.x, axis=0)
                               / np.linalg.norm(m64.x, axis=0), rtol=1e-12)
    assert gpu.MSQMRIDR(Am, bm, sig, 4, tolerance=TOL, maximum_iterations=50).get("rel_err_vs_fp64") is None


def test_bad_check_tolerance_is_rejected(gpu, prob):
    K, D, b = prob
    with pytest.raises(gpu.IDRSError):
        gpu.PP_IDRS(K, b, P=D, tol=TOL, fp64_check=-1e-3, **MIXED)


def test_complex_pipeline_states_its_error(gpu, oracle):
    """CPP_IDRS (damped Helmholtz, seed 2 pi i, Neumann(4)) with QMRIDR(4) and
    a complex64 inner IDR(4): the check runs the complex FP64 form."""
    from test_gpu_pp import _helmholtz
    n, K, M, C, b = _helmholtz(gpu, oracle)
    kw = dict(method=0, s=4, tol=TOL, maxit=200, preconditioner=1, degree=4, n_ritz=12, in_s=4,
              in_it=20, in_tol=1e-2, inner_precision=32, M=M[0], C_=C[0], seed=2j * np.pi)
    g = gpu.PP_IDRS(K[0], b.astype(complex), **kw)
    assert g.flag == 0 and g.relres_original <= 2 * TOL
    assert g.fp64_flag == 0 and 0 < g.rel_err_vs_fp64 <= 1e-5
    q = gpu.PP_IDRS(K[0], b.astype(complex), **dict(kw, inner_precision=64, in_it=0, tol=1e-11, maxit=5000))
    assert q.flag == 0
    # both FP64 solutions carry errors of order kappa * 1e-11 of their own
    assert abs(g.rel_err_vs_fp64 - _rel(g.x, q.x)) <= 1e-8 + 0.05 * g.rel_err_vs_fp64
