"""The reference's RANDOM examples on the GPU (E/RANDOM/band_real.f90:39-82,
band_complex.f90, dense_real.f90, dense_complex.f90:38-71): A given in band
(cds_format) or dense (dense_format) storage, P = its band / dense LU
(real_precon / complex_precon 3 / 2, built on the device from those formats),
b = A 1.  The preconditioner matches the oracle's and the solve returns 1."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _random_example(kind, n, hb, rng):
    """uniform random band (entries outside the matrix zeroed) or dense matrix"""
    cplx = kind.endswith("complex")
    if kind.startswith("band"):
        R = rng.uniform(size=(n, 2 * hb + 1)) + (1j * rng.uniform(size=(n, 2 * hb + 1)) if cplx else 0)
        A = np.zeros((n, n), R.dtype)
        for d in range(-hb, hb + 1):
            for i in range(n):
                if 0 <= i + d < n:
                    A[i, i + d] = R[i, d + hb]
                else:
                    R[i, d + hb] = 0
        return A, R, cplx
    A = rng.uniform(size=(n, n)) + (1j * rng.uniform(size=(n, n)) if cplx else 0)
    return A, A, cplx


@pytest.mark.parametrize("kind", ["band_real", "band_complex", "dense_real", "dense_complex"])
def test_random_examples_match_oracle(gpu, oracle, kind):
    rng = np.random.default_rng({"band_real": 1, "band_complex": 2, "dense_real": 3, "dense_complex": 4}[kind])
    band = kind.startswith("band")
    n, hb = (400, 6) if band else (120, 0)
    A, R, cplx = _random_example(kind, n, hb, rng)
    if band:
        Kg = gpu.cds_format(n, n, hb, **({"cband": R} if cplx else {"rband": R}))
        Ko = oracle.cds_format(n, n, hb, R)
    else:
        Kg = gpu.dense_format(**({"cmat": R} if cplx else {"rmat": R}))
        Ko = oracle.dense_format(R)
    which = 3 if band else 2
    if cplx:
        Pg, Po = gpu.complex_precon(which, Kg), oracle.complex_precon(which, Ko)
    else:
        Pg, Po = gpu.real_precon(which, Kg), oracle.real_precon(which, Ko)
    Ag, Ao = gpu.Matrix(Kg, P=Pg, complex=cplx), oracle.Matrix(Ko, P=Po, cplx=cplx)
    v = rng.standard_normal(n) + (1j * rng.standard_normal(n) if cplx else 0)
    xg, xo = v / Ag, Ao.precon(v)
    if band:
        # the band solve scales U's columns by 1/U(k,k) first (one rounding
        # more per entry than the oracle's divisions); growth is small here
        np.testing.assert_allclose(xg, xo, rtol=1e-10, atol=1e-12)
    else:
        # dense: the factor and the solve are the same FMAs and Smith
        # divisions in the same order on both sides, so they agree to the
        # last bit.  Without pivoting the growth max|U|/max|A| is 1.8e4
        # (dense_real): one rounding more per update (product, then
        # difference) already moves the solution by 5e-9 relative, so the
        # comparison is tight on purpose.
        np.testing.assert_allclose(xg, xo, rtol=1e-13, atol=0)
    # backward error of the GPU solve against A itself: measured 1.5e-13
    # (dense_real) and 1.5e-15 (dense_complex); n eps max(|L||U|)/max|A|
    # bounds it by 1.4e-9 in the worst case
    berr = np.linalg.norm(A @ xg - v) / (np.linalg.norm(A, 2) * np.linalg.norm(xg))
    assert berr <= 1e-12, berr
    b = A @ np.ones(n)
    r = gpu.IDRS(Ag, b, 4, tolerance=1e-10)
    assert r.flag == 0
    np.testing.assert_allclose(Ag.scaleback(b, r.x), 1.0, atol=1e-6)


def test_band_lu_of_a_dense_matrix_is_a_zero_pivot(gpu):
    """A dense matrix has no band form in the reference (real_band leaves it
    zero), so its band LU meets a zero pivot -- as in the reference."""
    K = gpu.dense_format(rmat=np.eye(3) * 2.0)
    with pytest.raises(gpu.IDRSError):
        gpu.real_precon(3, K)


@pytest.mark.parametrize("n", [600, 1208])
@pytest.mark.parametrize("cplx", [False, True])
def test_blocked_dense_lu_matches_oracle(gpu, oracle, cplx, n):
    """Dense LU from n = 256 on runs on all SMs in blocks of 16 pivots (panel,
    block row, trailing tiles) with the same operations per entry in the same
    order as the one-CTA factorisation and the oracle: the dense-LU
    preconditioner agrees with the oracle's to rounding of the solve alone.
    Neither n is a multiple of the block; at n = 1208 the first blocks' trailing
    updates run in 64 x 64 tiles (ragged at the edge), the later ones in 16 x
    16.  The matrix is the RANDOM examples' uniform matrix made diagonally
    dominant, so the solve is well posed."""
    rng = np.random.default_rng((21 if cplx else 20) + n)
    A = rng.uniform(size=(n, n)) + (1j * rng.uniform(size=(n, n)) if cplx else 0)
    A = A + n * np.eye(n)
    if cplx:
        Kg, Ko = gpu.dense_format(cmat=A), oracle.dense_format(A)
        Pg, Po = gpu.complex_precon(2, Kg), oracle.complex_precon(2, Ko)
    else:
        Kg, Ko = gpu.dense_format(rmat=A), oracle.dense_format(A)
        Pg, Po = gpu.real_precon(2, Kg), oracle.real_precon(2, Ko)
    Ag, Ao = gpu.Matrix(Kg, P=Pg, complex=cplx), oracle.Matrix(Ko, P=Po, cplx=cplx)
    v = rng.standard_normal(n) + (1j * rng.standard_normal(n) if cplx else 0)
    xg, xo = v / Ag, Ao.precon(v)
    np.testing.assert_allclose(xg, xo, rtol=1e-13, atol=0)
    berr = np.linalg.norm(A @ xg - v) / (np.linalg.norm(A, 2) * np.linalg.norm(xg))
    assert berr <= 1e-13, berr


def test_blocked_dense_lu_zero_pivot(gpu):
    """A pivot that stays exactly zero (row and column 300 are zero left of
    and above the diagonal, and the diagonal entry is zero) stops the blocked
    factorisation with the reference's error."""
    n = 600
    A = np.eye(n) * 4.0 + np.triu(np.full((n, n), 0.01), 1)
    A[300, :] = 0.0
    A[:, 300] = 0.0
    A[300, 301:] = 1.0
    K = gpu.dense_format(rmat=A)
    with pytest.raises(gpu.IDRSError):
        gpu.real_precon(2, K)


@pytest.mark.parametrize("kind", ["band_real", "band_complex"])
def test_blocked_band_lu_matches_oracle(gpu, oracle, kind):
    """Band LU with n >= 256 and hb >= 16 runs in blocks of 16 pivots on all
    SMs with the one-CTA kernel's operations per entry in its order; n = 1000
    and hb = 40 (neither a multiple of the block) as the RANDOM band example
    builds them plus 2 hb on the diagonal (moderate growth without
    pivoting), compared with the oracle as the one-CTA band test is."""
    rng = np.random.default_rng({"band_real": 31, "band_complex": 32}[kind])
    n, hb = 1000, 40
    A, R, cplx = _random_example(kind, n, hb, rng)
    R[:, hb] += 2 * hb
    A = A + 2 * hb * np.eye(n)
    Kg = gpu.cds_format(n, n, hb, **({"cband": R} if cplx else {"rband": R}))
    Ko = oracle.cds_format(n, n, hb, R)
    if cplx:
        Pg, Po = gpu.complex_precon(3, Kg), oracle.complex_precon(3, Ko)
    else:
        Pg, Po = gpu.real_precon(3, Kg), oracle.real_precon(3, Ko)
    Ag, Ao = gpu.Matrix(Kg, P=Pg, complex=cplx), oracle.Matrix(Ko, P=Po, cplx=cplx)
    v = rng.standard_normal(n) + (1j * rng.standard_normal(n) if cplx else 0)
    xg, xo = v / Ag, Ao.precon(v)
    np.testing.assert_allclose(xg, xo, rtol=1e-10, atol=1e-12 * np.abs(xo).max())
    berr = np.linalg.norm(A @ xg - v) / (np.linalg.norm(A, 2) * np.linalg.norm(xg))
    assert berr <= 1e-12, berr
