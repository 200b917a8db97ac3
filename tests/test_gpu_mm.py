"""Matrix Market fixtures through the GPU path, the way the reference's
E/MATRIX_MARKET examples use them (wedge_sommerfeld.f90, stommel.f90), on
problems of the same kind written here: a damped Helmholtz problem with
stiffness, mass and boundary-damping matrices (single frequency, and all
frequencies at once on the 2x2 block system), and a nonsymmetric
convection-diffusion matrix with a block of right-hand sides solved as a
sequence (PP_MR_IDRS).  GPU results against the oracle on the same data."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _write_sym(path, n, rows, cols, vals):
    """symmetric coordinate file from the lower triangle."""
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real symmetric\n")
        keep = [(i, j, v) for i, j, v in zip(rows, cols, vals) if j <= i]
        f.write(f"{n} {n} {len(keep)}\n")
        for i, j, v in keep:
            f.write(f"{i} {j} {v:.17e}\n")
    return str(path)


def _write_array(path, B):
    B = np.atleast_2d(B.T).T
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix array real general\n")
        f.write(f"{B.shape[0]} {B.shape[1]}\n")
        for v in B.ravel(order="F"):
            f.write(f"{v:.17e}\n")
    return str(path)


def _helmholtz(tmp_path, m=20):
    """2-D unit square, m x m nodes: K = 5-point stiffness, M = lumped mass,
    C = damping on the boundary nodes (first-order absorbing condition)."""
    h = 1.0 / (m - 1)
    n = m * m
    idx = lambda x, y: y * m + x + 1
    kr, kc, kv = [], [], []
    for y in range(m):
        for x in range(m):
            i = idx(x, y)
            kr.append(i); kc.append(i); kv.append(4.0)
            for dx, dy in ((-1, 0), (1, 0), (0, -1), (0, 1)):
                if 0 <= x + dx < m and 0 <= y + dy < m:
                    kr.append(i); kc.append(idx(x + dx, y + dy)); kv.append(-1.0)
    bnd = [idx(x, y) for y in range(m) for x in range(m) if x in (0, m - 1) or y in (0, m - 1)]
    files = dict(
        K=_write_sym(tmp_path / "w_K.mtx", n, kr, kc, kv),
        M=_write_sym(tmp_path / "w_M.mtx", n, range(1, n + 1), range(1, n + 1), [h * h] * n),
        C=_write_sym(tmp_path / "w_C.mtx", n, bnd, bnd, [h] * len(bnd)))
    b = np.zeros(n)
    b[idx(m // 3, m // 2) - 1] = 1.0
    files["b"] = _write_array(tmp_path / "w_b.mtx", b)
    return n, files


def _oracle_matrix(oracle, r, n):
    if "row_ptr" in r:
        return oracle.crs_format(n, n, r.row_ptr, r.col_ind, r.vals)
    return oracle.coo_format(n, n, r.indx, r.jndx, r.vals)


@pytest.mark.parametrize("freq", [1.0, 2.0])
def test_wedge_like_single_frequency(gpu, oracle, tmp_path, freq):
    """wedge_sommerfeld.f90 without -multi: (K + sigma C + sigma^2 M) x = b,
    sigma = 2 pi f i, K read as CRS and C, M as COO like the example."""
    n, F = _helmholtz(tmp_path)
    K, Cm, M = gpu.mm_matrix(F["K"], "crs"), gpu.mm_matrix(F["C"]), gpu.mm_matrix(F["M"])
    b = gpu.mm_read(F["b"]).vals[:, 0].astype(np.complex128)
    sigma = 2j * np.pi * freq
    A = gpu.Matrix(K, M=M, C_=Cm, seed=sigma, complex=True)
    Ao = oracle.Matrix(_oracle_matrix(oracle, gpu.mm_read(F["K"], "crs"), n),
                       M=_oracle_matrix(oracle, gpu.mm_read(F["M"]), n),
                       C_=_oracle_matrix(oracle, gpu.mm_read(F["C"]), n), seed=sigma, cplx=True)
    g = gpu.IDRS(A, b, 4, tolerance=1e-8, maximum_iterations=4000)
    o = oracle.idrs(Ao, b, 4, tolerance=1e-8, maximum_iterations=4000)
    assert g.flag == o.flag == 0
    assert abs(g.iterations - o.iterations) <= max(3, 0.05 * o.iterations)
    np.testing.assert_allclose(g.x, o.x, rtol=0, atol=1e-6 * np.abs(o.x).max())
    assert np.linalg.norm(b - Ao.matvec(g.x)) <= 2e-8 * np.linalg.norm(b)


def test_wedge_like_all_frequencies_block_system(gpu, oracle, tmp_path):
    """wedge_sommerfeld.f90 -multi: the block system with P = diag(M),
    seed = the last shift, MSIDRS on the shifted systems, x = the second
    half of each scaled-back solution (run_ms_idrs.inc)."""
    n, F = _helmholtz(tmp_path, m=16)
    K, Cm, M = gpu.mm_matrix(F["K"], "crs"), gpu.mm_matrix(F["C"]), gpu.mm_matrix(F["M"])
    rhs = gpu.mm_read(F["b"]).vals[:, 0].astype(np.complex128)
    freqs = np.array([1.0, 2.0, 4.0])
    sigma = 2j * np.pi * freqs
    P = gpu.complex_precon(1, M)
    A = gpu.Matrix(K, P=P, M=M, C_=Cm, seed=sigma[-1], complex=True, multishift=True)
    Ko, Mo, Co = (_oracle_matrix(oracle, gpu.mm_read(F[k], "crs" if k == "K" else None), n)
                  for k in ("K", "M", "C"))
    Ao = oracle.Matrix(Ko, P=oracle.complex_precon(1, Mo), M=Mo, C_=Co, seed=sigma[-1], cplx=True,
                       multishift=True)
    b = np.concatenate([-rhs, np.zeros(n)])
    sp, spo = A.ms_parameters(sigma), Ao.ms_parameters(sigma)
    np.testing.assert_allclose(sp, spo, rtol=1e-15)
    g = gpu.MSIDRS(A, b, sp, 4, tolerance=1e-8, maximum_iterations=4000)
    o = oracle.msidrs(Ao, b, spo, 4, tolerance=1e-8, maximum_iterations=4000)
    assert g.flag == o.flag == 0
    assert abs(g.iterations - o.iterations) <= max(3, 0.05 * o.iterations)
    X = A.ms_scaleback(sigma, b, g.x)[n:, :]
    Xo = Ao.ms_scaleback(o.x)[n:, :]
    np.testing.assert_allclose(X, Xo, rtol=0, atol=1e-6 * np.abs(Xo).max())
    for k, s in enumerate(sigma):  # (K + s C + s^2 M) x = rhs
        D = oracle.Matrix(Ko, M=Mo, C_=Co, seed=s, cplx=True)
        assert np.linalg.norm(rhs - D.matvec(X[:, k])) <= 1e-6 * np.linalg.norm(rhs)


def test_stommel_like_sequence(gpu, oracle, tmp_path):
    """stommel.f90: K read as COO, a block of right-hand sides from an array
    file, P = real_precon(1, K), x = pp_idrs(K, b, P=P) over all columns."""
    m = 30
    n = m * m
    h = 1.0 / (m + 1)
    rows, cols, vals = [], [], []
    for y in range(m):
        for x in range(m):
            i = y * m + x + 1
            for (dx, dy), v in (((0, 0), 4.0), ((-1, 0), -1 - 20 * h), ((1, 0), -1 + 20 * h),
                                ((0, -1), -1.0), ((0, 1), -1.0)):
                if 0 <= x + dx < m and 0 <= y + dy < m:
                    rows.append(i); cols.append(i + dx + dy * m); vals.append(v)
    path = tmp_path / "st.mtx"
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real general\n% convection-diffusion\n")
        f.write(f"{n} {n} {len(rows)}\n")
        for i, j, v in zip(rows, cols, vals):
            f.write(f"{i} {j} {v:.17e}\n")
    B = np.random.default_rng(12).standard_normal((n, 3))
    bpath = _write_array(tmp_path / "st_b.mtx", B)
    K = gpu.mm_matrix(str(path), "coo")
    Bm = gpu.mm_read(bpath).vals
    r = gpu.mm_read(str(path))
    Ko = oracle.coo_format(n, n, r.indx, r.jndx, r.vals)
    g = gpu.PP_MR_IDRS(K, Bm, P=gpu.real_precon(1, K), s=4, tol=1e-8)
    o = oracle.pp_mr_idrs(Ko, Bm, P=oracle.real_precon(1, Ko), s=4, tol=1e-8)
    assert list(g.flags) == list(o.flags) == [0, 0, 0]
    assert np.all(np.abs(g.iterations - o.iterations) <= 3)
    np.testing.assert_allclose(g.x, o.x, rtol=0, atol=1e-6 * np.abs(o.x).max())
    assert np.all(g.relres_original < 2e-8)
