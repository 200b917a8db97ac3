"""Operators with mass and damping matrices (real_mv / complex_mv,
matrix_module.f90:170-264) and the 2x2 block system of a multishift problem
with damping, against the oracle: products, IDR(s) solves with a seed, and
MSIDRS on the block system."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P(gpu):
    return gpu.problems


def _mass_crs(n):
    """1-D consistent mass pattern on the grid ordering (tridiagonal)."""
    rp, ci, vals = [1], [], []
    for i in range(n):
        for j, v in ((i - 1, 1.0 / 6), (i, 4.0 / 6), (i + 1, 1.0 / 6)):
            if 0 <= j < n:
                ci.append(j + 1)
                vals.append(v)
        rp.append(len(ci) + 1)
    return np.array(rp, np.int32), np.array(ci, np.int32), np.array(vals)


def _system(gpu, oracle, P, n=8, cvals=False):
    N = n ** 3
    rp, ci, kv = P.stencil_to_crs(n, n, n, P.cdr_coefficients(n))
    mrp, mci, mv = _mass_crs(N)
    cv = 0.05 * kv
    if cvals:
        cv = cv * (1 + 0.3j)
    G = dict(K=gpu.crs_format(N, N, rp, ci, rval=kv), M=gpu.crs_format(N, N, mrp, mci, rval=mv),
             C=gpu.crs_format(N, N, rp, ci, cval=cv) if cvals else gpu.crs_format(N, N, rp, ci, rval=cv))
    O = dict(K=oracle.crs_format(N, N, rp, ci, kv), M=oracle.crs_format(N, N, mrp, mci, mv),
             C=oracle.crs_format(N, N, rp, ci, cv))
    G["P"], O["P"] = gpu.real_precon(1, G["K"]), oracle.real_precon(1, O["K"])
    return N, G, O


FORMS = [  # (use M, use C, multishift, seed)
    (True, True, False, 3.0), (False, True, False, -2.0), (True, False, False, 5.0),
    (True, True, False, 0.0), (True, True, True, 4.0), (False, True, True, 4.0),
    (True, True, True, 0.0)]


@pytest.mark.parametrize("useM,useC,ms,seed", FORMS)
@pytest.mark.parametrize("scaled", [False, True])
def test_system_products_match_oracle(gpu, oracle, P, useM, useC, ms, seed, scaled):
    N, G, O = _system(gpu, oracle, P)
    kw_g = dict(M=G["M"] if useM else None, C_=G["C"] if useC else None, multishift=ms,
                seed=seed, P=G["P"] if scaled else None)
    kw_o = dict(M=O["M"] if useM else None, C_=O["C"] if useC else None, multishift=ms,
                seed=seed, P=O["P"] if scaled else None)
    A, Ao = gpu.Matrix(G["K"], **kw_g), oracle.Matrix(O["K"], **kw_o)
    assert A.n == Ao.n == (2 * N if ms and useC else N)
    v = np.random.default_rng(1).standard_normal(A.n)
    ref = Ao.matvec(v)
    np.testing.assert_allclose(A * v, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
    np.testing.assert_allclose(v / A, Ao.precon(v), rtol=1e-14, atol=0)


@pytest.mark.parametrize("seed", [0.7 + 0.4j, -1.5 + 2.0j])
def test_system_complex_seed_products(gpu, oracle, P, seed):
    N, G, O = _system(gpu, oracle, P, cvals=True)
    for ms in (False, True):
        A = gpu.Matrix(G["K"], M=G["M"], C_=G["C"], seed=seed, complex=True, multishift=ms)
        Ao = oracle.Matrix(O["K"], M=O["M"], C_=O["C"], seed=seed, cplx=True, multishift=ms)
        rng = np.random.default_rng(2)
        v = rng.standard_normal(A.n) + 1j * rng.standard_normal(A.n)
        ref = Ao.matvec(v)
        np.testing.assert_allclose(A * v, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


def test_idrs_with_mass_and_damping_matches_oracle(gpu, oracle, P):
    """(K + seed C + seed^2 M) x = b with diagonal scaling, IDR(4)."""
    N, G, O = _system(gpu, oracle, P, n=10)
    seed = 2.0
    A = gpu.Matrix(G["K"], P=G["P"], M=G["M"], C_=G["C"], seed=seed)
    Ao = oracle.Matrix(O["K"], P=O["P"], M=O["M"], C_=O["C"], seed=seed)
    b = np.random.default_rng(4).standard_normal(N)
    g = gpu.IDRS(A, b, 4, tolerance=1e-10)
    o = oracle.idrs(Ao, b, 4, tolerance=1e-10)
    assert g.flag == o.flag == 0 and abs(g.iterations - o.iterations) <= 2
    xg, xo = A.scaleback(b, g.x), Ao.scaleback(b, o.x)
    np.testing.assert_allclose(xg, xo, rtol=0, atol=1e-8 * np.abs(xo).max())
    # the assembled operator is the reference's sum of products
    D = oracle.Matrix(O["K"], M=O["M"], C_=O["C"], seed=seed)
    assert np.linalg.norm(b - D.matvec(xg)) <= 2e-10 * np.linalg.norm(b) * 10


def test_msidrs_block_system_matches_oracle(gpu, oracle, P):
    """MSIDRS on the 2n x 2n block system of a damped problem (the multishift
    form of K + sigma C + sigma^2 M with complex shifts)."""
    N, G, O = _system(gpu, oracle, P, n=6)
    A = gpu.Matrix(G["K"], M=G["M"], C_=G["C"], complex=True, multishift=True)
    Ao = oracle.Matrix(O["K"], M=O["M"], C_=O["C"], cplx=True, multishift=True)
    rng = np.random.default_rng(5)
    b = rng.standard_normal(2 * N) + 1j * rng.standard_normal(2 * N)
    sigma = np.array([0.5 + 0.1j, 1.0 - 0.2j, 2.0 + 0.5j])
    g = gpu.MSIDRS(A, b, sigma, 4, tolerance=1e-8, maximum_iterations=3000)
    o = oracle.msidrs(Ao, b, sigma, 4, tolerance=1e-8, maximum_iterations=3000)
    assert g.flag == o.flag == 0
    assert abs(g.iterations - o.iterations) <= max(5, 0.1 * o.iterations)
    X = g.x
    for k, s in enumerate(sigma):
        r = b - (Ao.matvec(X[:, k]) - s * X[:, k])
        assert np.linalg.norm(r) <= 1e-7 * np.linalg.norm(b)


def test_system_rejects_unsupported_formats(gpu, P):
    n = 6
    coef = P.cdr_coefficients(n)
    S = gpu.stencil7_format(n, n, n, coef)
    rp, ci, kv = P.stencil_to_crs(n, n, n, coef)
    Mc = gpu.crs_format(n ** 3, n ** 3, rp, ci, rval=kv)
    with pytest.raises(gpu.IDRSError):
        gpu.Matrix(S, M=Mc, seed=1.0)


@pytest.mark.parametrize("useM,useC", [(True, True), (False, True), (True, False), (False, False)])
@pytest.mark.parametrize("shift", [None, 2.5, 1.0 - 0.5j])
def test_diagonal_precon_with_mass_and_damping(gpu, oracle, P, useM, useC, shift):
    """REAL_PRECON / COMPLEX_PRECON(1, K, M, C, shift): v / A with A = the
    identity operator scaled by that diagonal, against the oracle."""
    N, G, O = _system(gpu, oracle, P, n=6)
    cplx = isinstance(shift, complex)
    kg = dict(M=G["M"] if useM else None, C_=G["C"] if useC else None, shift=shift)
    ko = dict(M=O["M"] if useM else None, C_=O["C"] if useC else None, shift=shift)
    if cplx:
        Pg, Po = gpu.complex_precon(1, G["K"], **kg), oracle.complex_precon(1, O["K"], **ko)
    else:
        Pg, Po = gpu.real_precon(1, G["K"], **kg), oracle.real_precon(1, O["K"], **ko)
    A = gpu.Matrix(G["K"], P=Pg, complex=cplx)
    Ao = oracle.Matrix(O["K"], P=Po, cplx=cplx)
    v = np.random.default_rng(8).standard_normal(N) * (1 + 0.5j if cplx else 1)
    np.testing.assert_allclose(v / A, Ao.precon(v), rtol=1e-15, atol=0)
