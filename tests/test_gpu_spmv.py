"""Load-balanced sparse products on the GPU: CRS with power-law rows (the
long-row segment plan) and the COO segmented reduction, against the oracle's
serial products (rcrs_mv user_module.f90:376-450, rcoo_mv :525-585), then the
PageRank system solved through them.  Products rtol 1e-12 (the summation
order differs); solutions 10 * tol * cond-free bound via the true residual."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P(gpu):
    return gpu.problems


def _power_law(n, seed, max_len=6000):
    rng = np.random.default_rng(seed)
    lens = np.minimum(rng.zipf(1.7, n), max_len)
    lens[rng.random(n) < 0.05] = 0  # empty rows
    lens[3] = max_len                # at least one row spanning many segments
    rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    ci = rng.integers(0, n, rp[-1])
    vals = rng.standard_normal(rp[-1])
    return (rp + 1).astype(np.int32), (ci + 1).astype(np.int32), vals


@pytest.mark.parametrize("seed", [1, 2])
def test_crs_long_rows(gpu, oracle, seed):
    n = 20000
    rp, ci, vals = _power_law(n, seed)
    rng = np.random.default_rng(seed + 10)
    v = rng.standard_normal(n)
    vc = v + 1j * rng.standard_normal(n)
    K = gpu.crs_format(n, n, rp, ci, rval=vals)
    Ko = oracle.crs_format(n, n, rp, ci, vals)
    np.testing.assert_allclose(K * v, Ko.mv(v), rtol=1e-12, atol=1e-10)
    np.testing.assert_allclose(K * vc, Ko.mv(vc), rtol=1e-12, atol=1e-10)
    cv = vals + 1j * rng.standard_normal(len(vals))
    Kc = gpu.crs_format(n, n, rp, ci, cval=cv)
    np.testing.assert_allclose(Kc * vc, oracle.crs_format(n, n, rp, ci, cv).mv(vc), rtol=1e-12, atol=1e-10)
    # the operator path (scaled copy, epilogue terms) and fp32 view through
    # the transposed matrix's plan
    A = gpu.Matrix(K)
    np.testing.assert_allclose(A * v, Ko.mv(v), rtol=1e-12, atol=1e-10)
    KT = gpu.crs_transpose(K)
    np.testing.assert_allclose(KT * v, oracle.crs_transpose(Ko).mv(v), rtol=1e-12, atol=1e-10)


@pytest.mark.parametrize("seed", [3, 4])
def test_coo_segmented_reduction(gpu, oracle, seed):
    n = 20000
    rp, ci, vals = _power_law(n, seed)
    rows = np.repeat(np.arange(n), np.diff(rp)) + 1
    rng = np.random.default_rng(seed)
    perm = rng.permutation(len(vals))
    Kc = gpu.coo_format(n, n, len(vals), rows[perm], ci[perm], rval=vals[perm])
    Ko = oracle.coo_format(n, n, rows[perm], ci[perm], vals[perm])
    v = rng.standard_normal(n)
    np.testing.assert_allclose(Kc * v, Ko.mv(v), rtol=1e-12, atol=1e-10)
    vc = v + 1j * rng.standard_normal(n)
    np.testing.assert_allclose(Kc * vc, Ko.mv(vc), rtol=1e-12, atol=1e-10)
    # a single dense row (one row spans every warp share) and a diagonal
    m = 5000
    one = gpu.coo_format(m, m, m, np.ones(m, np.int32), np.arange(1, m + 1, dtype=np.int32),
                         rval=np.linspace(0, 1, m))
    w = rng.standard_normal(m)
    out = one * w
    assert abs(out[0] - np.linspace(0, 1, m) @ w) <= 1e-12 * m and np.all(out[1:] == 0)
    diag = gpu.coo_format(m, m, m, np.arange(1, m + 1, dtype=np.int32), np.arange(1, m + 1, dtype=np.int32),
                          rval=np.full(m, 2.0))
    np.testing.assert_array_equal(diag * w, 2.0 * w)


def test_pagerank_solve(gpu, oracle, P):
    """(I - alpha P^T) x = (1-alpha)/N 1 on a seeded power-law graph
    (pagerank.f90:87-179): IDR(2) / IDR(8) fp64 and the mixed form (fp32 inner
    IDR(s) under FP64 QMRIDR) against the oracle, tol 1e-10."""
    n = 50000
    rp, ci, vals, b = P.pagerank_crs(n)
    K = gpu.crs_format(n, n, rp, ci, rval=vals)
    Ko = oracle.crs_format(n, n, rp, ci, vals)
    A, Ao = gpu.Matrix(K), oracle.Matrix(Ko)
    tol = 1e-10
    for s in (2, 8):
        g = gpu.IDRS(A, b, s, tolerance=tol)
        o = oracle.idrs(Ao, b, s, tolerance=tol)
        assert g.flag == o.flag == 0 and g.relres <= tol
        assert abs(g.iterations - o.iterations) <= s + 1
        assert np.linalg.norm(g.x - o.x) <= 10 * tol * np.linalg.norm(o.x)
        m = gpu.QMRIDR(A, b, s, tolerance=tol, inner_s=s, inner_iterations=50, inner_tolerance=1e-3,
                       inner_precision=32)
        assert m.flag == 0 and m.relres <= tol
        assert np.linalg.norm(m.x - o.x) <= 10 * tol * np.linalg.norm(o.x)
