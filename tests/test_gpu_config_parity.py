"""The production path against the oracle: the shadow space the device draws
itself (MAKE_P, idrs_module.f90:839-937: seeded uniform numbers, then
Gram-Schmidt) instead of one injected into both, and the 64^3 configuration
(IDR(4), tol 1e-8, CRS, N = 262,144, 1,810,432 nonzeros) at its full size."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P(gpu):
    return gpu.problems


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _cdr_crs(gpu, oracle, P, n):
    rp, ci, vals = P.stencil_to_crs(n, n, n, P.cdr_coefficients(n))
    N = n ** 3
    return N, gpu.crs_format(N, N, rp, ci, rval=vals), oracle.crs_format(N, N, rp, ci, vals)


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("s", [1, 4, 8])
def test_device_shadow_space_matches_oracle(gpu, oracle, P, s, cplx):
    """No set_shadow: the GPU's k_gen_p + fused Gram-Schmidt and the oracle's
    make_p draw the same counter-based numbers (seed 1), so the residual
    histories agree step by step; a different P would part them after the
    first cycle."""
    N, K, Ko = _cdr_crs(gpu, oracle, P, 10)
    A, Ao = gpu.Matrix(K, complex=cplx), oracle.Matrix(Ko, cplx=cplx)
    rng = np.random.default_rng(s + 10 * cplx)
    b = rng.standard_normal(N) + (1j * rng.standard_normal(N) if cplx else 0)
    g = gpu.IDRS(A, b, s, tolerance=1e-10, resvec=True)
    o = oracle.idrs(Ao, b, s, tolerance=1e-10, resvec_len=min(2 * N, 1000) + 1)
    assert g.flag == o.flag == 0
    k = min(12, g.iterations, o.iterations)
    np.testing.assert_allclose(g.resvec[:k], o.resvec[:k], rtol=1e-8)
    assert abs(g.iterations - o.iterations) <= s + 1
    assert _rel(g.x, o.x) <= 1e-9


def test_device_shadow_space_qmridr_matches_oracle(gpu, oracle, P):
    """The same for QMRIDR(4) (qmridr.inc builds P from the first residual's
    space the same way)."""
    N, K, Ko = _cdr_crs(gpu, oracle, P, 10)
    A, Ao = gpu.Matrix(K), oracle.Matrix(Ko)
    b = Ko.mv(np.ones(N))
    g = gpu.QMRIDR(A, b, 4, tolerance=1e-10, resvec=True)
    o = oracle.qmridr(Ao, b, 4, tolerance=1e-10, resvec_len=min(2 * N, 1000) + 1)
    assert g.flag == o.flag == 0
    k = min(12, g.iterations, o.iterations)
    np.testing.assert_allclose(g.resvec[:k], o.resvec[:k], rtol=1e-8)
    assert _rel(g.x, o.x) <= 1e-9


def test_cfg1_idr4_64cube_matches_oracle(gpu, oracle, P):
    """64^3 convection-diffusion, beta = 10, h = 1/65, CRS (N = 262,144,
    nnz = 1,810,432), b = A 1, x0 = 0, IDR(4), tol 1e-8, FP64, production
    shadow space: both reach the tolerance on the true residual, their
    iteration counts differ by at most s + 1 and the solutions agree to
    10 tol."""
    rp = P.stencil_to_crs(64, 64, 64, P.cdr_coefficients(64))[0]
    assert rp[-1] - 1 == 1810432
    N, K, Ko = _cdr_crs(gpu, oracle, P, 64)
    A, Ao = gpu.Matrix(K), oracle.Matrix(Ko)
    b = Ko.mv(np.ones(N))
    g = gpu.IDRS(A, b, 4, tolerance=1e-8, resvec=True)
    o = oracle.idrs(Ao, b, 4, tolerance=1e-8, resvec_len=min(2 * N, 1000) + 1)
    assert g.flag == o.flag == 0
    assert g.relres <= 1e-8 and o.relres <= 1e-8
    assert abs(g.iterations - o.iterations) <= 5
    k = min(12, g.iterations)
    np.testing.assert_allclose(g.resvec[:k], o.resvec[:k], rtol=1e-8)
    assert _rel(g.x, o.x) <= 1e-7
    np.testing.assert_allclose(g.x, 1.0, atol=1e-5)
