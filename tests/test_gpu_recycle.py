"""Recycling on the GPU: IDRS_RITZ's omega and U0 outputs (ritz_module.f90:
389-556) and the multi right-hand-side pipeline PP_MR_IDRS
(pp_idrs_module.f90:222-279, recycle.inc, run_mr_idrs.inc), against the
oracle on the same inputs (the shadow space and the SI_power start block come
from the generator the oracle shares)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P(gpu):
    return gpu.problems


def _cdr(gpu, oracle, P, n):
    coef = P.cdr_coefficients(n)
    rp, ci, vals = P.stencil_to_crs(n, n, n, coef)
    N = n ** 3
    return (gpu.crs_format(N, N, rp, ci, rval=vals), oracle.crs_format(N, N, rp, ci, vals),
            gpu.stencil7_format(n, n, n, coef), oracle.stencil7_format(n, n, n, coef))


@pytest.mark.parametrize("n,s", [(10, 4), (16, 8), (12, 2)])
def test_idrs_ritz_outputs_match_oracle(gpu, oracle, P, n, s):
    Kg, Ko, _, _ = _cdr(gpu, oracle, P, n)
    b = np.random.default_rng(n + s).standard_normal(n ** 3)
    A, Ao = gpu.Matrix(Kg), oracle.Matrix(Ko)
    n_om = 2 * s
    g = gpu.IDRS_RITZ(A, b, s, tolerance=1e-8, n_omega=n_om, dimU0=s, resvec=True,
                      H_shape=(21, 20))
    o = oracle.idrs_ritz(Ao, b, s, tolerance=1e-8, n_omega=n_om, dimU0=s, H_shape=(21, 20))
    assert g.flag == o.flag == 0
    assert abs(g.iterations - o.iterations) <= 1
    assert g.nritz == (g.iterations // (s + 1)) * s + g.iterations % (s + 1)
    np.testing.assert_allclose(g.H, o.H, rtol=1e-9, atol=1e-9 * np.abs(o.H).max())
    # conjugate Ritz pairs give equal omegas and equal |p|: the greedy order
    # of tied entries follows rounding, so the sets are compared
    assert g.omega[0] == pytest.approx(o.omega[0], rel=1e-9)
    np.testing.assert_allclose(np.sort(g.omega), np.sort(o.omega), rtol=1e-9)
    assert np.abs(g.U0.T @ g.U0 - np.eye(s)).max() < 1e-12
    if g.iterations == o.iterations:
        np.testing.assert_allclose(g.U0, o.U0, rtol=0, atol=1e-7)
    # the same subspace either way: projector distance
    d = g.U0 @ (g.U0.T @ o.U0) - o.U0
    assert np.linalg.norm(d) < 1e-6
    assert g.resvec[0] == pytest.approx(np.linalg.norm(b), rel=1e-13)
    np.testing.assert_allclose(g.x, o.x, rtol=0, atol=1e-7 * np.abs(o.x).max())


def test_idrs_ritz_errors(gpu, oracle, P):
    Kg, _, _, _ = _cdr(gpu, oracle, P, 8)
    A = gpu.Matrix(Kg)
    b = np.ones(8 ** 3)
    with pytest.raises(gpu.IDRSError):  # more omegas than Ritz values
        gpu.IDRS_RITZ(A, b, 4, tolerance=1e-8, maximum_iterations=3, n_omega=6)
    with pytest.raises(gpu.IDRSError):  # recycle space larger than the Krylov space
        gpu.IDRS_RITZ(A, b, 4, tolerance=1e-8, maximum_iterations=3, dimU0=4)
    with pytest.raises(gpu.IDRSError):
        gpu.IDRS_RITZ(A, b, 4, tolerance=-1.0)


def test_idrs_with_recycled_u0_matches_oracle(gpu, oracle, P):
    """IDRS started from a recycle space (idrs.inc:56-64: U = U0 in G_0)."""
    n, s = 12, 4
    Kg, Ko, _, _ = _cdr(gpu, oracle, P, n)
    rng = np.random.default_rng(3)
    b1, b2 = rng.standard_normal(n ** 3), rng.standard_normal(n ** 3)
    A, Ao = gpu.Matrix(Kg), oracle.Matrix(Ko)
    U0 = oracle.idrs_ritz(Ao, b1, s, tolerance=1e-8, dimU0=s).U0
    g = gpu.IDRS(A, b2, s, tolerance=1e-8, U0=U0)
    o = oracle.idrs(Ao, b2, s, tolerance=1e-8, U0=U0)
    assert g.flag == o.flag == 0
    assert abs(g.iterations - o.iterations) <= 1
    np.testing.assert_allclose(g.x, o.x, rtol=0, atol=1e-6 * np.abs(o.x).max())


# Ritz omegas come from the initial solve on the operator without the
# polynomial preconditioner (real_preconditioner.inc:22-34), so they are
# exercised without one; 32 of them keep the cyclic omega polynomial stable.
CASES = [dict(method=1, recycle=False, n_omega=0, preconditioner=2, degree=4, n_ritz=12),
         dict(method=1, recycle=True, n_omega=0, preconditioner=2, degree=4, n_ritz=12),
         dict(method=0, recycle=False, n_omega=0, preconditioner=2, degree=4, n_ritz=12),
         dict(method=1, recycle=False, n_omega=32, preconditioner=0, n_ritz=32),
         dict(method=1, recycle=True, n_omega=32, preconditioner=0, n_ritz=32)]


@pytest.mark.parametrize("case", CASES)
def test_pp_mr_idrs_matches_oracle(gpu, oracle, P, case):
    n = 12
    _, _, Sg, So = _cdr(gpu, oracle, P, n)
    rng = np.random.default_rng(7)
    B = rng.standard_normal((n ** 3, 4))
    B[:, 3] = B[:, 2]  # repeats its predecessor: the warm start already solves it
    recycle = case["recycle"]
    kw = dict(s=4, tol=1e-8, in_s=2, in_it=20, in_tol=1e-2, **case)
    g = gpu.PP_MR_IDRS(Sg, B, P=gpu.real_precon(1, Sg), **kw)
    o = oracle.pp_mr_idrs(So, B, P=oracle.real_precon(1, So), **kw)
    assert list(g.flags) == list(o.flags) == [0, 0, 0, 0]
    assert g.nritz == o.nritz
    assert np.all(np.abs(g.iterations - o.iterations) <= np.maximum(2, 0.1 * o.iterations))
    assert g.iterations[3] <= 1
    if recycle:
        assert g.recycle_flag == 0 and abs(g.recycle_iterations - o.recycle_iterations) <= 1
        assert g.iterations[0] == 0
    assert np.all(g.relres_original < 2e-8)
    for j in range(4):
        np.testing.assert_allclose(g.x[:, j], o.x[:, j], rtol=0,
                                   atol=1e-6 * np.abs(o.x[:, j]).max())


def test_pp_mr_idrs_device_pointers(gpu, P):
    torch = pytest.importorskip("torch")
    n = 12
    coef = P.cdr_coefficients(n)
    S = gpu.stencil7_format(n, n, n, coef)
    rng = np.random.default_rng(2)
    B = np.asfortranarray(rng.standard_normal((n ** 3, 3)))
    h = gpu.PP_MR_IDRS(S, B, s=4, tol=1e-8, recycle=True)
    Bd = torch.tensor(B.T.copy(), device="cuda")  # row j of Bd = column j of B
    Xd = torch.zeros_like(Bd)
    d = gpu.PP_MR_IDRS(S, Bd.data_ptr(), s=4, tol=1e-8, recycle=True, nrhs=3,
                       x_out=Xd.data_ptr())
    torch.cuda.synchronize()
    assert list(d.iterations) == list(h.iterations)
    np.testing.assert_array_equal(Xd.cpu().numpy().T, h.x)


def test_complex_idrs_ritz_outputs_match_oracle(gpu, oracle, P):
    """CIDRS_RITZ (ritz_module.f90:268-387): complex omegas and the recycle
    space from the Schur vectors of the complex Hessenberg matrix."""
    n, s = 8, 4
    Kg, Ko, _, _ = _cdr(gpu, oracle, P, n)
    seed = 1.0 + 2.0j
    A = gpu.Matrix(Kg, seed=seed, complex=True)
    Ao = oracle.Matrix(Ko, seed=seed, cplx=True)
    rng = np.random.default_rng(0)
    b = rng.standard_normal(n ** 3) + 1j * rng.standard_normal(n ** 3)
    g = gpu.IDRS_RITZ(A, b, s, tolerance=1e-8, n_omega=6, dimU0=s, H_shape=(21, 20))
    o = oracle.idrs_ritz(Ao, b, s, tolerance=1e-8, n_omega=6, dimU0=s, H_shape=(21, 20))
    assert g.flag == o.flag == 0 and abs(g.iterations - o.iterations) <= 1
    np.testing.assert_allclose(g.H, o.H, rtol=1e-9, atol=1e-9 * np.abs(o.H).max())
    np.testing.assert_allclose(np.sort_complex(g.omega), np.sort_complex(o.omega), rtol=1e-8)
    assert np.abs(g.U0.conj().T @ g.U0 - np.eye(s)).max() < 1e-12
    d = g.U0 @ (g.U0.conj().T @ o.U0) - o.U0
    assert np.linalg.norm(d) < 1e-6


def test_complex_pp_mr_idrs_recycle(gpu, oracle, P):
    """CPP_MR_IDRS with recycle: the recycle solve already solves rhs 1, the
    sequence meets the tolerance, and the result matches the same steps
    composed from the oracle."""
    n = 8
    Sg, So, _, _ = _cdr(gpu, oracle, P, n)  # CRS: a complex seed needs stored values
    rng = np.random.default_rng(9)
    B = rng.standard_normal((n ** 3, 3)) + 1j * rng.standard_normal((n ** 3, 3))
    seed = 0.5 + 1.0j
    g = gpu.PP_MR_IDRS(Sg, B, seed=seed, s=4, tol=1e-8, recycle=True)
    assert list(g.flags) == [0, 0, 0] and g.iterations[0] == 0
    assert np.all(g.relres_original < 2e-8)
    A = oracle.Matrix(So, seed=seed, cplx=True)
    r = oracle.idrs_ritz(A, B[:, 0], 4, tolerance=1e-8, maximum_iterations=1000, dimU0=4)
    assert abs(g.recycle_iterations - r.iterations) <= 1
    x0 = r.x
    for j in range(3):
        o = oracle.idrs(A, B[:, j], 4, tolerance=1e-8, x0=x0, U0=r.U0)
        x0 = o.x
        np.testing.assert_allclose(g.x[:, j], o.x, rtol=0, atol=1e-6 * np.abs(o.x).max())
