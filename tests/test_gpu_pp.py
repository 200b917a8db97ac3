"""The pp_idrs pipelines with every optional input (M, C, seed, shift, V),
real and complex, single, sequence and multishift (pp_idrs_module.f90,
real/complex_matrix.inc, real/complex_preconditioner.inc, run_idrs.inc,
run_mr_idrs.inc, run_ms_idrs.inc), against the same steps composed from the
oracle's restated routines."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _helmholtz(gpu, oracle, m=14):
    """2-D damped Helmholtz pieces: K (5-point stiffness), M (lumped mass),
    C (boundary damping), all CRS, for the GPU and the oracle."""
    h = 1.0 / (m - 1)
    n = m * m
    idx = lambda x, y: y * m + x
    rows, cols, vals = [], [], []
    for y in range(m):
        for x in range(m):
            i = idx(x, y)
            rows.append(i); cols.append(i); vals.append(4.0)
            for dx, dy in ((-1, 0), (1, 0), (0, -1), (0, 1)):
                if 0 <= x + dx < m and 0 <= y + dy < m:
                    rows.append(i); cols.append(idx(x + dx, y + dy)); vals.append(-1.0)
    bnd = {idx(x, y) for y in range(m) for x in range(m) if x in (0, m - 1) or y in (0, m - 1)}

    def crs(r, c, v):
        r, c, v = np.asarray(r), np.asarray(c), np.asarray(v, dtype=float)
        order = np.lexsort((c, r))
        r, c, v = r[order], c[order], v[order]
        rp = np.concatenate([[1], 1 + np.cumsum(np.bincount(r, minlength=n))]).astype(np.int32)
        return (gpu.crs_format(n, n, rp, (c + 1).astype(np.int32), rval=v),
                oracle.crs_format(n, n, rp, (c + 1).astype(np.int32), v))
    K = crs(rows, cols, vals)
    M = crs(range(n), range(n), [h * h] * n)
    bl = sorted(bnd)
    C = crs(bl, bl, [h] * len(bl))
    b = np.zeros(n)
    b[idx(m // 3, m // 2)] = 1.0
    return n, K, M, C, b


def test_cpp_idrs_single_frequency(gpu, oracle):
    """CPP_IDRS(K, b, M, C, seed = 2 pi f i), Ritz-estimated Neumann(4)."""
    n, K, M, C, b = _helmholtz(gpu, oracle)
    seed = 2j * np.pi
    kw = dict(s=4, tol=1e-8, maxit=3000, preconditioner=1, degree=4, n_ritz=12)
    g = gpu.PP_IDRS(K[0], b.astype(complex), M=M[0], C_=C[0], seed=seed, **kw)
    # the same steps from the oracle
    A = oracle.Matrix(K[1], M=M[1], C_=C[1], seed=seed, cplx=True)
    ini = 12 + 12 // 4
    bc = b.astype(complex)
    r = oracle.idrs(A, bc, 4, tolerance=1e-8, maximum_iterations=ini, variant=1, H_shape=(ini + 1, ini))
    nr = (r.iterations // 5) * 4 + r.iterations % 5
    assert g.nritz == nr
    A.preconditioner(1, 4, H=r.H[:nr, :nr])
    o = oracle.idrs(A, bc, 4, tolerance=1e-8, maximum_iterations=3000, x0=r.x)
    xo = A.scaleback(bc, o.x)
    assert g.flag == o.flag == 0 and abs(g.iterations - o.iterations) <= 2
    np.testing.assert_allclose(g.x, xo, rtol=0, atol=1e-6 * np.abs(xo).max())
    assert g.relres_original < 2e-8
    D = oracle.Matrix(K[1], M=M[1], C_=C[1], seed=seed, cplx=True)
    assert np.linalg.norm(bc - D.matvec(g.x)) <= 2e-8 * np.linalg.norm(bc)


@pytest.mark.parametrize("method", [1, 0])
def test_cpp_ms_idrs_block_system(gpu, oracle, method):
    """CPP_MS_IDRS with M, C, P = diag(M), seed = the last shift: the block
    system, solutions = second halves, true residuals per frequency."""
    n, K, M, C, b = _helmholtz(gpu, oracle, m=12)
    sigma = 2j * np.pi * np.array([1.0, 2.0, 3.0])
    Pg = gpu.complex_precon(1, M[0])
    g = gpu.PP_MS_IDRS(K[0], b.astype(complex), sigma, P=Pg, M=M[0], C_=C[0], seed=sigma[-1], s=4,
                       tol=1e-8, maxit=4000, method=method)
    assert g.flag == 0
    assert np.all(g.relres_sigma < 1e-6)
    A = oracle.Matrix(K[1], P=oracle.complex_precon(1, M[1]), M=M[1], C_=C[1], seed=sigma[-1],
                      cplx=True, multishift=True)
    bb = np.concatenate([-b.astype(complex), np.zeros(n)])
    sp = A.ms_parameters(sigma)
    o = (oracle.msidrs if method == 1 else oracle.msqmridr)(A, bb, sp, 4, tolerance=1e-8,
                                                             maximum_iterations=4000)
    X = A.ms_scaleback(o.x, bb)[n:, :]
    # ~500 iterations on an indefinite complex problem: rounding moves the count
    assert abs(g.iterations - o.iterations) <= max(5, 0.25 * o.iterations)
    np.testing.assert_allclose(g.x, X, rtol=0, atol=1e-5 * np.abs(X).max())
    for k, s in enumerate(sigma):
        D = oracle.Matrix(K[1], M=M[1], C_=C[1], seed=s, cplx=True)
        rr = np.linalg.norm(b - D.matvec(g.x[:, k])) / np.linalg.norm(b)
        assert rr == pytest.approx(g.relres_sigma[k], rel=1e-3, abs=1e-12)


def test_rpp_ms_idrs_shifted_laplacian(gpu, oracle):
    """RPP_MS_IDRS without M and C: (K - sigma I) x = rhs for real shifts."""
    n, K, M, C, b = _helmholtz(gpu, oracle, m=12)
    sigma = np.array([-0.5, -1.0, -2.0])
    g = gpu.PP_MS_IDRS(K[0], b, sigma, s=4, tol=1e-10, maxit=2000)
    assert g.flag == 0 and np.all(g.relres_sigma < 1e-9)
    A = oracle.Matrix(K[1])
    o = oracle.msidrs(A, b, A.ms_parameters(sigma), 4, tolerance=1e-10, maximum_iterations=2000)
    np.testing.assert_allclose(g.x, A.ms_scaleback(o.x, b), rtol=0, atol=1e-8 * np.abs(g.x).max())


def test_rpp_idrs_with_deflation(gpu, oracle):
    """RPP_IDRS(K, b, P, V): Pmul(b), the deflated solve, add_deflation."""
    n, K, M, C, b = _helmholtz(gpu, oracle, m=16)
    rng = np.random.default_rng(3)
    V = rng.standard_normal((n, 2))
    b = rng.standard_normal(n)
    g = gpu.PP_IDRS(K[0], b, P=gpu.real_precon(1, K[0]), V=V, s=4, tol=1e-10, maxit=3000)
    A = oracle.Matrix(K[1], P=oracle.real_precon(1, K[1]))
    A.make_deflation(V)
    o = oracle.idrs(A, A.pmul(b), 4, tolerance=1e-10, maximum_iterations=3000)
    xo = A.scaleback(b, o.x)
    assert g.flag == o.flag == 0 and abs(g.iterations - o.iterations) <= 2
    np.testing.assert_allclose(g.x, xo, rtol=0, atol=1e-8 * np.abs(xo).max())
    assert g.relres_original < 1e-9


def test_cpp_mr_idrs_sequence(gpu, oracle):
    """CPP_MR_IDRS: a complex sequence with warm starts."""
    n, K, M, C, b = _helmholtz(gpu, oracle, m=12)
    rng = np.random.default_rng(4)
    B = rng.standard_normal((n, 3)) + 1j * rng.standard_normal((n, 3))
    seed = 1.0j
    g = gpu.PP_MR_IDRS(K[0], B, M=M[0], C_=C[0], seed=seed, s=4, tol=1e-8, maxit=3000)
    assert list(g.flags) == [0, 0, 0] and np.all(g.relres_original < 2e-8)
    A = oracle.Matrix(K[1], M=M[1], C_=C[1], seed=seed, cplx=True)
    D = A
    for j in range(3):
        assert np.linalg.norm(B[:, j] - D.matvec(g.x[:, j])) <= 2e-8 * np.linalg.norm(B[:, j])


def test_cpp_ms_mr_idrs_sequence(gpu, oracle):
    """CPP_MS_MR_IDRS: two right-hand sides through one multishift set-up; each
    agrees with the single-rhs pipeline and meets the tolerance for every shift."""
    n, K, M, C, b = _helmholtz(gpu, oracle, m=10)
    rng = np.random.default_rng(5)
    R = rng.standard_normal((n, 2)) + 0j
    sigma = 2j * np.pi * np.array([1.0, 2.0])
    kw = dict(P=gpu.complex_precon(1, M[0]), M=M[0], C_=C[0], seed=sigma[-1], s=4, tol=1e-9,
              maxit=4000)
    g = gpu.PP_MS_IDRS(K[0], R, sigma, **kw)
    assert list(g.flags) == [0, 0] and g.x.shape == (n, 2, 2)
    assert np.all(g.relres_sigma < 1e-7)
    for j in range(2):
        one = gpu.PP_MS_IDRS(K[0], R[:, j], sigma, **kw)
        np.testing.assert_allclose(g.x[:, :, j], one.x, rtol=1e-12, atol=1e-12 * np.abs(one.x).max())
