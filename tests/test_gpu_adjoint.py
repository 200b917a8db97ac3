"""Adjoint path on the GPU (idrs_crs_transpose, idrs_rsparse_outer_grad,
idrs_radjoint) against the oracle and against central finite differences.

Loss L = 1/2 ||x - x_t||^2 with A x = b (A = convection-diffusion CRS):
dL/db = lambda with A^T lambda = x - x_t, dL/dA_ij = -lambda_i x_j.
Finite differences use eps = 1e-6 and the exact rearrangement
L(+) - L(-) = (x - x_t).(d+ - d-) + (|d+|^2 - |d-|^2)/2 with d = x(+-) - x
obtained from one solve of the perturbed system each (A(+-) d = r(+-)), so
that no large loss values cancel; target agreement 1e-5 relative.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P(gpu):
    return gpu.problems


def _cdr_crs(P, n):
    coef = P.cdr_coefficients(n)
    rp, ci, vals = P.stencil_to_crs(n, n, n, coef)
    return rp, ci, vals


def _dense(rp, ci, vals, n):
    D = np.zeros((n, n))
    for i in range(n):
        for p in range(rp[i] - 1, rp[i + 1] - 1):
            D[i, ci[p] - 1] += vals[p]
    return D


def test_crs_transpose_matches_oracle(gpu, oracle):
    """Random rectangular-free square CRS with empty rows, empty columns and
    duplicate entries; K^T v compared with the oracle's serial transpose."""
    rng = np.random.default_rng(5)
    n = 300
    lens = rng.integers(0, 9, n)
    lens[::17] = 0
    rp = np.concatenate([[1], 1 + np.cumsum(lens)]).astype(np.int32)
    nnz = int(rp[-1] - 1)
    cols = rng.integers(1, n + 1, nnz)
    cols[cols % 29 == 0] = 1  # crowd column 1, leave others empty
    ci = cols.astype(np.int32)
    vals = rng.standard_normal(nnz)
    K = gpu.crs_format(n, n, rp, ci, rval=vals)
    Ko = oracle.crs_format(n, n, rp, ci, vals)
    KT = gpu.crs_transpose(K)
    KTo = oracle.crs_transpose(Ko)
    v = rng.standard_normal(n)
    np.testing.assert_allclose(KT * v, KTo.mv(v), rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(KT * v, _dense(rp, ci, vals, n).T @ v, rtol=1e-12, atol=1e-12)
    # complex values
    cv = vals + 1j * rng.standard_normal(nnz)
    Kc = gpu.crs_format(n, n, rp, ci, cval=cv)
    vc = v + 1j * rng.standard_normal(n)
    np.testing.assert_allclose(gpu.crs_transpose(Kc) * vc, oracle.crs_transpose(
        oracle.crs_format(n, n, rp, ci, cv)).mv(vc), rtol=1e-13, atol=1e-13)


def test_crs_transpose_stencil_matrix(gpu, oracle, P):
    n = 24
    N = n ** 3
    rp, ci, vals = _cdr_crs(P, n)
    K = gpu.crs_format(N, N, rp, ci, rval=vals)
    KT = gpu.crs_transpose(K)
    v = np.random.default_rng(1).standard_normal(N)
    KTo = oracle.crs_transpose(oracle.crs_format(N, N, rp, ci, vals))
    np.testing.assert_allclose(KT * v, KTo.mv(v), rtol=1e-13, atol=1e-9)
    # (K^T)^T = K
    np.testing.assert_allclose(gpu.crs_transpose(KT) * v, K * v, rtol=1e-13, atol=1e-9)


def test_sparse_outer_grad_exact(gpu, oracle, P):
    n = 20
    N = n ** 3
    rp, ci, vals = _cdr_crs(P, n)
    rng = np.random.default_rng(2)
    lam, x = rng.standard_normal(N), rng.standard_normal(N)
    K = gpu.crs_format(N, N, rp, ci, rval=vals)
    g = gpu.sparse_outer_grad(gpu.Matrix(K), lam, x)
    go = oracle.sparse_outer_grad(oracle.crs_format(N, N, rp, ci, vals), lam, x, len(vals))
    np.testing.assert_array_equal(g, go)


def test_sparse_outer_grad_ragged_blocks(gpu):
    """Row blocks whose nonzeros fit the shared-memory row ids and blocks that
    overflow them (a 256-row block with more than 4096 nonzeros takes the
    binary search), empty rows and a row count that is not a multiple of the
    block's 256 rows: bitwise equal to -lambda_i x_j in numpy."""
    rng = np.random.default_rng(11)
    n = 5000
    L = rng.integers(0, 12, n)
    L[1024:2048] = rng.integers(10, 40, 1024)  # these blocks overflow the row ids
    L[rng.integers(0, n, 200)] = 0
    rp = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(L, out=rp[1:])
    assert rp[1280] - rp[1024] > 4096 and rp[256] - rp[0] <= 4096
    ci = rng.integers(0, n, int(rp[-1]))
    vals = rng.standard_normal(int(rp[-1]))
    K = gpu.crs_format(n, n, (rp + 1).astype(np.int32), (ci + 1).astype(np.int32), rval=vals)
    lam, x = rng.standard_normal(n), rng.standard_normal(n)
    g = gpu.sparse_outer_grad(gpu.Matrix(K), lam, x)
    rows = np.repeat(np.arange(n), L)
    np.testing.assert_array_equal(g, -lam[rows] * x[ci])


def _setup(gpu, P, n, seed=9):
    N = n ** 3
    rp, ci, vals = _cdr_crs(P, n)
    rng = np.random.default_rng(seed)
    b, xt = rng.standard_normal(N), rng.standard_normal(N)
    return N, rp, ci, vals, b, xt


def test_adjoint_matches_oracle(gpu, oracle, P):
    n = 16
    N, rp, ci, vals, b, xt = _setup(gpu, P, n)
    tol = 1e-10
    K = gpu.crs_format(N, N, rp, ci, rval=vals)
    r = gpu.IDRS(gpu.Matrix(K), b, 4, tolerance=tol)
    assert r.flag == 0
    g = r.x - xt
    AT = gpu.Matrix(gpu.crs_transpose(K))
    a = gpu.ADJOINT(AT, K, r.x, g, 4, tolerance=tol)
    assert a.flag == 0 and a.relres <= tol
    Ko = oracle.crs_format(N, N, rp, ci, vals)
    xo = oracle.idrs(oracle.Matrix(Ko), b, 4, tolerance=tol).x
    lo = oracle.idrs(oracle.Matrix(oracle.crs_transpose(Ko)), xo - xt, 4, tolerance=tol).x
    go = oracle.sparse_outer_grad(Ko, lo, xo, len(vals))
    D = _dense(rp, ci, vals, N)
    kappa = np.linalg.cond(D)
    assert np.linalg.norm(a.lam - lo) <= 10 * tol * kappa * np.linalg.norm(lo)
    assert np.linalg.norm(a.grad - go) <= 10 * tol * kappa * np.linalg.norm(go)
    # against a direct FP64 solve
    x_ref = np.linalg.solve(D, b)
    l_ref = np.linalg.solve(D.T, x_ref - xt)
    assert np.linalg.norm(a.lam - l_ref) <= 10 * tol * kappa * np.linalg.norm(l_ref)
    # diagonal scaling on the adjoint operator: lambda = scaleback(AT, g, mu)
    KT = gpu.crs_transpose(K)
    ATs = gpu.Matrix(KT, P=gpu.real_precon(1, KT))
    a2 = gpu.ADJOINT(ATs, K, r.x, g, 4, tolerance=tol)
    assert a2.flag == 0
    assert np.linalg.norm(a2.lam - l_ref) <= 10 * tol * kappa * np.linalg.norm(l_ref)


def test_adjoint_finite_differences(gpu, P):
    n = 16
    N, rp, ci, vals, b, xt = _setup(gpu, P, n, seed=4)
    eps, tol = 1e-6, 1e-12
    K = gpu.crs_format(N, N, rp, ci, rval=vals)
    A = gpu.Matrix(K)
    x = gpu.IDRS(A, b, 4, tolerance=tol, maximum_iterations=4000).x
    a = gpu.ADJOINT(gpu.Matrix(gpu.crs_transpose(K)), K, x, x - xt, 4, tolerance=tol,
                    maximum_iterations=4000)
    rng = np.random.default_rng(0)
    res = x - xt

    def central(d_plus, d_minus):
        return (res @ (d_plus - d_minus) + 0.5 * (d_plus @ d_plus - d_minus @ d_minus)) / (2 * eps)

    def solve(Am, rhs):
        r = gpu.IDRS(Am, rhs, 4, tolerance=tol, maximum_iterations=4000)
        assert r.flag == 0
        return r.x

    for k in rng.choice(N, 8, replace=False):  # b entries: A d = +-eps e_k
        e = np.zeros(N)
        e[k] = eps
        fd = central(solve(A, e), solve(A, -e))
        assert abs(fd - a.lam[k]) <= 1e-5 * abs(a.lam[k])
    rows = np.repeat(np.arange(N), np.diff(rp))
    for p in rng.choice(len(vals), 8, replace=False):  # A entries: A(+-) d = -+eps x_j e_i
        i, j = rows[p], ci[p] - 1
        d = []
        for sgn in (1.0, -1.0):
            v2 = vals.copy()
            v2[p] += sgn * eps
            Ap = gpu.Matrix(gpu.crs_format(N, N, rp, ci, rval=v2))
            rhs = np.zeros(N)
            rhs[i] = -sgn * eps * x[j]
            d.append(solve(Ap, rhs))
        fd = central(d[0], d[1])
        assert abs(fd - a.grad[p]) <= 1e-5 * abs(a.grad[p])


def test_autograd_harness_gradcheck(gpu, P):
    torch = pytest.importorskip("torch")
    from importlib import import_module
    ag = import_module(gpu.__name__ + ".autograd")
    n = 4
    N = n ** 3
    rp, ci, vals = _cdr_crs(P, n)
    rng = np.random.default_rng(3)
    v = torch.tensor(vals, dtype=torch.float64, requires_grad=True)
    b = torch.tensor(rng.standard_normal(N), dtype=torch.float64, requires_grad=True)
    xt = torch.tensor(rng.standard_normal(N), dtype=torch.float64)

    def loss(v, b):
        x = ag.crs_solve(v, b, rp, ci, s=4, tol=1e-13)
        return 0.5 * ((x - xt) ** 2).sum()

    assert torch.autograd.gradcheck(loss, (v, b), eps=1e-6, atol=1e-7, rtol=1e-5)
