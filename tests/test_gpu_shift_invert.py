"""Shift-and-invert on the GPU: dense (which_precon 2) and band (3) LU
preconditioners of K + shift C + shift^2 M (user_module.f90:1383-1602),
factored and solved on the device, and the multishift solve that uses one
at `shift` (matrix_module.f90:402-483, :724-766), against the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P(gpu):
    return gpu.problems


def _mats(gpu, oracle, P, n, seed=4):
    N = n ** 3
    rp, ci, kv = P.stencil_to_crs(n, n, n, P.cdr_coefficients(n))
    rows = np.repeat(np.arange(N), np.diff(rp))
    D = np.zeros((N, N))
    D[rows, ci - 1] = kv
    rng = np.random.default_rng(seed)
    Md = np.diag(rng.uniform(1.0, 2.0, N)) + np.diag(np.full(N - 1, 0.1), 1) + np.diag(np.full(N - 1, 0.1), -1)
    Cd = np.diag(rng.uniform(0.0, 0.5, N))

    def both(Dm):
        r, c = np.nonzero(Dm)
        rp_ = np.concatenate([[1], 1 + np.cumsum(np.bincount(r, minlength=N))]).astype(np.int32)
        return (gpu.crs_format(N, N, rp_, (c + 1).astype(np.int32), rval=Dm[r, c]),
                oracle.crs_format(N, N, rp_, (c + 1).astype(np.int32), Dm[r, c]))
    K = (gpu.crs_format(N, N, rp, ci, rval=kv), oracle.crs_format(N, N, rp, ci, kv))
    return N, D, Md, Cd, K, both(Md), both(Cd), rng


@pytest.mark.parametrize("which", [2, 3])
@pytest.mark.parametrize("form", ["none", "K", "M", "MC"])
@pytest.mark.parametrize("cplx", [False, True])
def test_lu_precon_matches_oracle(gpu, oracle, P, which, form, cplx):
    N, D, Md, Cd, K, M, C, rng = _mats(gpu, oracle, P, 5)
    sh = 2.5 + (1.5j if cplx else 0)
    kg, ko = {}, {}
    if form != "none":
        kg["shift"] = ko["shift"] = sh
    if form in ("M", "MC"):
        kg["M"], ko["M"] = M
    if form == "MC":
        kg["C_"], ko["C_"] = C
    if cplx:
        Pg, Po = gpu.complex_precon(which, K[0], **kg), oracle.complex_precon(which, K[1], **ko)
    else:
        Pg, Po = gpu.real_precon(which, K[0], **kg), oracle.real_precon(which, K[1], **ko)
    A, Ao = gpu.Matrix(K[0], P=Pg, complex=cplx), oracle.Matrix(K[1], P=Po, cplx=cplx)
    v = rng.standard_normal(N) + (1j * rng.standard_normal(N) if cplx else 0)
    np.testing.assert_allclose(v / A, Ao.precon(v), rtol=1e-11, atol=1e-14)
    np.testing.assert_allclose(A * v, Ao.matvec(v), rtol=1e-11, atol=1e-11)


def test_lu_preconditioned_idrs_matches_oracle(gpu, oracle, P):
    """IDR(4) on K P^-1 with the band LU of K - 30 I: x = P^-1 y solves K x = b."""
    N, D, Md, Cd, K, M, C, rng = _mats(gpu, oracle, P, 8)
    A = gpu.Matrix(K[0], P=gpu.real_precon(3, K[0], shift=30.0))
    Ao = oracle.Matrix(K[1], P=oracle.real_precon(3, K[1], shift=30.0))
    b = rng.standard_normal(N)
    g = gpu.IDRS(A, b, 4, tolerance=1e-10)
    o = oracle.idrs(Ao, b, 4, tolerance=1e-10)
    assert g.flag == o.flag == 0 and abs(g.iterations - o.iterations) <= 2
    x = A.scaleback(b, g.x)
    np.testing.assert_allclose(x, Ao.scaleback(b, o.x), rtol=0, atol=1e-8 * np.abs(x).max())
    assert np.linalg.norm(b - D @ x) <= 1e-9 * np.linalg.norm(b)
    with pytest.raises(gpu.IDRSError):  # no shift-and-invert in the fp32 operator
        gpu.QMRIDR(A, b, 4, tolerance=1e-8, inner_iterations=20, inner_precision=32)


@pytest.mark.parametrize("which", [2, 3])
def test_shift_and_invert_multishift_matches_oracle(gpu, oracle, P, which):
    N, D, Md, Cd, K, M, C, rng = _mats(gpu, oracle, P, 5, seed=6)
    seed, shift = 0.0, -60.0
    A = gpu.Matrix(K[0], P=gpu.complex_precon(which, K[0], shift=shift, M=M[0]), M=M[0], seed=seed,
                   shift=shift, complex=True, multishift=True)
    Ao = oracle.Matrix(K[1], P=oracle.complex_precon(which, K[1], shift=shift, M=M[1]), M=M[1],
                       seed=seed, shift=shift, cplx=True, multishift=True)
    sig = np.array([10.0, 20.0 + 5j, -5.0])
    sp, spo = A.ms_parameters(sig), Ao.ms_parameters(sig)
    np.testing.assert_allclose(sp, spo, rtol=1e-15)
    b = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    g = gpu.MSIDRS(A, b, sp, 4, tolerance=1e-11, maximum_iterations=2000)
    o = oracle.msidrs(Ao, b, spo, 4, tolerance=1e-11, maximum_iterations=2000)
    assert g.flag == o.flag == 0 and abs(g.iterations - o.iterations) <= 2
    X = A.ms_scaleback(sig, b, g.x)
    np.testing.assert_allclose(X, Ao.ms_scaleback(o.x, b), rtol=0, atol=1e-8 * np.abs(X).max())
    for k, s in enumerate(sig):
        assert np.linalg.norm(b - (D - s * Md) @ X[:, k]) <= 1e-9 * np.linalg.norm(b)
    with pytest.raises(gpu.IDRSError):  # the shift may not equal a shift of the problem
        A.ms_parameters(np.array([shift, 1.0]))


def test_zero_pivot_is_an_error(gpu):
    rp = np.array([1, 2, 3], np.int32)
    ci = np.array([2, 1], np.int32)
    K = gpu.crs_format(2, 2, rp, ci, rval=np.array([1.0, 1.0]))
    for which in (2, 3):
        with pytest.raises(gpu.IDRSError):
            gpu.real_precon(which, K)


def test_block_shift_and_invert_matches_oracle(gpu, oracle, P):
    """Damped multishift problem on the 2 x 2 block system with rprecon's
    shift-and-invert block form (matrix_module.f90:318-345): GPU and oracle
    agree and every (K + sigma C + sigma^2 M) x = rhs is solved."""
    N, D, Md, Cd, K, M, C, rng = _mats(gpu, oracle, P, 4, seed=8)
    tau = 3.0 + 2.0j
    sig = np.array([1.0 + 1.0j, 2.0 + 0.5j, 4.0 + 1.0j])
    A = gpu.Matrix(K[0], P=gpu.complex_precon(3, K[0], shift=tau, M=M[0], C_=C[0]), M=M[0], C_=C[0],
                   seed=sig[-1], shift=tau, complex=True, multishift=True)
    Ao = oracle.Matrix(K[1], P=oracle.complex_precon(3, K[1], shift=tau, M=M[1], C_=C[1]), M=M[1],
                       C_=C[1], seed=sig[-1], shift=tau, cplx=True, multishift=True)
    assert A.n == Ao.n == 2 * N
    v = rng.standard_normal(2 * N) + 1j * rng.standard_normal(2 * N)
    np.testing.assert_allclose(v / A, Ao.precon(v), rtol=1e-11, atol=1e-14)
    np.testing.assert_allclose(A * v, Ao.matvec(v), rtol=1e-11, atol=1e-11)
    rhs = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    b = np.concatenate([-rhs, np.zeros(N)])
    sp, spo = A.ms_parameters(sig), Ao.ms_parameters(sig)
    g = gpu.MSIDRS(A, b, sp, 4, tolerance=1e-11, maximum_iterations=3000)
    o = oracle.msidrs(Ao, b, spo, 4, tolerance=1e-11, maximum_iterations=3000)
    assert g.flag == o.flag == 0 and abs(g.iterations - o.iterations) <= 2
    X = A.ms_scaleback(sig, b, g.x)[N:, :]
    np.testing.assert_allclose(X, Ao.ms_scaleback(o.x, b)[N:, :], rtol=0, atol=1e-8 * np.abs(X).max())
    for k, s in enumerate(sig):
        S = D + s * Cd + s ** 2 * Md
        assert np.linalg.norm(rhs - S @ X[:, k]) <= 1e-8 * np.linalg.norm(rhs)


def _band_crs(pkg, n, hb, rng, cplx):
    """random diagonally dominant band matrix (CRS, 1-based) and its dense copy"""
    A = np.zeros((n, n), complex if cplx else float)
    for i in range(n):
        lo, hi = max(0, i - hb), min(n, i + hb + 1)
        A[i, lo:hi] = rng.standard_normal(hi - lo) + (1j * rng.standard_normal(hi - lo) if cplx else 0)
        A[i, i] += 2.0 * hb + 2.0
    r, c = np.nonzero(A)
    rp = np.concatenate([[1], 1 + np.cumsum(np.bincount(r, minlength=n))]).astype(np.int32)
    kw = {"cval": A[r, c]} if cplx else {"rval": A[r, c]}
    return A, pkg.crs_format(n, n, rp, (c + 1).astype(np.int32), **kw), (rp, (c + 1).astype(np.int32), A[r, c])


@pytest.mark.parametrize("n,hb,cplx", [(1000, 1, False), (333, 17, True), (95, 94, False), (700, 600, False),
                                       (700, 600, True), (2048, 64, True)])
def test_band_lu_shapes_match_oracle(gpu, oracle, n, hb, cplx):
    """Band LU solves across the staged kernel's shapes (chunk widths 32, 16 and
    8, ragged last chunk, half band n - 1) and the unstaged kernel of wide
    complex bands (600 x 2 threads > one block): GPU = oracle and A x = v."""
    rng = np.random.default_rng(n + hb)
    A, Kg, (rp, ci, vals) = _band_crs(gpu, n, hb, rng, cplx)
    Ko = oracle.crs_format(n, n, rp, ci, vals)
    if cplx:
        Pg, Po = gpu.complex_precon(3, Kg), oracle.complex_precon(3, Ko)
    else:
        Pg, Po = gpu.real_precon(3, Kg), oracle.real_precon(3, Ko)
    Ag, Ao = gpu.Matrix(Kg, P=Pg, complex=cplx), oracle.Matrix(Ko, P=Po, cplx=cplx)
    for _ in range(2):
        v = rng.standard_normal(n) + (1j * rng.standard_normal(n) if cplx else 0)
        w = v / Ag
        np.testing.assert_allclose(w, Ao.precon(v), rtol=1e-11, atol=1e-14)
        np.testing.assert_allclose(A @ w, v, rtol=1e-10, atol=1e-12)
