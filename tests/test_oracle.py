"""The oracle (CPU restatement) against the golden fixtures and the
reference's own known-answer examples.  CPU only."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


@pytest.fixture(scope="module")
def P(pkg):
    return pkg.problems


def _toeplitz_real(O, P):
    rp, ci, vals, b = P.toeplitz_real()
    return O.Matrix(O.crs_format(60, 60, rp, ci, vals)), b


def _toeplitz_complex(O, P):
    rp, ci, vals, b = P.toeplitz_complex()
    return O.Matrix(O.crs_format(200, 200, rp, ci, vals), cplx=True), b


def test_bicgstab_variant_matches_scipy_real(oracle, P):
    """IDRS variant 2 is BiCGSTAB (idrs_module.f90:13-15): its residual after
    every omega step follows scipy's bicgstab (tests/golden)."""
    d = np.load(os.path.join(GOLD, "bicgstab_toeplitz_real.npz"))
    A, b = _toeplitz_real(oracle, P)
    r = oracle.idrs(A, b, 1, variant=2, tolerance=1e-14, maximum_iterations=80, resvec_len=81)
    k = 12
    ours = r.resvec[2:2 * k + 1:2]
    np.testing.assert_allclose(ours, d["resnorm"][:k], rtol=1e-10)
    assert abs(r.resvec[0] - d["normb"]) <= 1e-14 * d["normb"]


def test_bicgstab_variant_matches_scipy_complex(oracle, P):
    d = np.load(os.path.join(GOLD, "bicgstab_toeplitz_complex.npz"))
    A, b = _toeplitz_complex(oracle, P)
    r = oracle.idrs(A, b, 1, variant=2, tolerance=1e-14, maximum_iterations=80, resvec_len=81)
    k = 8
    np.testing.assert_allclose(r.resvec[2:2 * k + 1:2], d["resnorm"][:k], rtol=1e-9)


@pytest.mark.parametrize("s", [1, 2, 4, 8])
def test_finite_termination_real_toeplitz(oracle, P, s):
    """E/TOEPLITZ/toeplitz.f90:134-138: IDR(s) terminates within N + N/s."""
    A, b = _toeplitz_real(oracle, P)
    r = oracle.idrs(A, b, s, tolerance=1e-8, maximum_iterations=4000)
    assert r.flag == 0
    assert r.iterations <= 60 + 60 // s
    assert r.relres < 1e-8
    q = oracle.qmridr(A, b, s, tolerance=1e-8, maximum_iterations=4000)
    assert q.flag == 0 and q.iterations <= 60 + 60 // s and q.relres < 1e-8


@pytest.mark.parametrize("s", [1, 2, 4, 8, 16, 32, 64])
def test_complex_toeplitz_accuracy(oracle, P, s):
    """E/TOEPLITZ/toeplitz.f90:20-93: tol 1e-12, flag 0."""
    A, b = _toeplitz_complex(oracle, P)
    r = oracle.idrs(A, b, s, tolerance=1e-12, maximum_iterations=4000)
    assert r.flag == 0 and r.relres < 1e-12
    q = oracle.qmridr(A, b, s, tolerance=1e-12, maximum_iterations=4000)
    assert q.flag == 0 and q.relres < 1e-12


def test_chebyshev_and_neumann_polynomials(oracle):
    """matrix_module.f90:851-1019: r(t) = 1 - t p(t) equals the closed-form
    Chebyshev / Neumann residual polynomial."""
    g = np.load(os.path.join(GOLD, "poly.npz"))
    t = g["t"]
    for d in (1, 2, 4, 8, 12):
        a = oracle.chebyshev(d, g["foci"])
        r = 1 - t * np.polyval(a[::-1], t)
        np.testing.assert_allclose(r, g[f"cheb_{d}"], atol=1e-9)
    for d in (1, 3, 6):
        a = oracle.neumann(d, float(g["center"]))
        r = 1 - t * np.polyval(a[::-1], t)
        np.testing.assert_allclose(r, g[f"neu_{d}"], atol=1e-12)


def test_qr_eig_and_solve(oracle):
    """dense_la_module.f90: QR_eig against numpy eigenvalues, SOLVE against
    numpy.linalg.solve, GROT in BLAS rotg style."""
    g = np.load(os.path.join(GOLD, "dense.npz"))
    e, conv = oracle.qr_eig(g["H"])
    assert conv == 12
    ref = g["eig"]
    for z in ref:
        assert np.min(np.abs(e - z)) < 1e-10 * max(1.0, abs(z))
    np.testing.assert_allclose(oracle.solve(g["M"], g["rhs"]), g["x"], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(oracle.solve(g["Mc"], g["rhsc"]), g["xc"], rtol=1e-12, atol=1e-12)
    c, s, r = oracle.grot(3.0, 4.0)
    assert (c, s, r) == pytest.approx((0.6, 0.8, 5.0))
    assert oracle.grot(0.0, 2.0) == (0.0, 1.0, 2.0)


def test_known_solution_cdr(oracle, P):
    """b = A*1 => x = 1 (E/RANDOM/band_real.f90:77-79 style) on the 3-D
    convection-diffusion operator, CRS and stencil formats agree."""
    n = 10
    coef = P.cdr_coefficients(n)
    rp, ci, vals = P.stencil_to_crs(n, n, n, coef)
    K = oracle.crs_format(n ** 3, n ** 3, rp, ci, vals)
    S = oracle.stencil7_format(n, n, n, coef)
    v = np.random.default_rng(1).standard_normal(n ** 3)
    np.testing.assert_allclose(K.mv(v), S.mv(v), rtol=1e-13, atol=1e-9)
    np.testing.assert_allclose(S.mv(v), P.stencil_apply(n, n, n, coef, v), rtol=1e-13, atol=1e-9)
    b = K.mv(np.ones(n ** 3))
    r = oracle.idrs(oracle.Matrix(K), b, 4, tolerance=1e-10)
    assert r.flag == 0
    np.testing.assert_allclose(r.x, 1.0, atol=1e-8)


def test_problem_sizes(P):
    """The 64^3 CRS operator has the nonzero count of the benchmark config."""
    rp, ci, vals = P.stencil_to_crs(64, 64, 64, P.cdr_coefficients(64))
    assert rp[-1] - 1 == 1_810_432
    c = P.cdr_coefficients(64)
    h = 1 / 65
    assert c[0] == pytest.approx(6 / h**2)
    assert c[2] == pytest.approx(-1 / h**2 + 5 / h)
    assert c[1] == pytest.approx(-1 / h**2 - 5 / h)


def test_flags_and_errors(oracle, P):
    A, b = _toeplitz_real(oracle, P)
    r = oracle.idrs(A, b, 4, tolerance=1e-12, maximum_iterations=5)
    assert r.flag == 1 and r.iterations == 5
    with pytest.raises(ValueError):
        oracle.idrs(A, b, 4, tolerance=-1.0)
    r = oracle.idrs(A, np.zeros(60), 4)
    assert r.flag == 0 and r.iterations == 0


def test_pp_idrs_pipeline(oracle, P):
    """PP_IDRS with Ritz-estimated Chebyshev(8) and diagonal scaling."""
    n = 12
    coef = P.cdr_coefficients(n)
    S = oracle.stencil7_format(n, n, n, coef)
    D = oracle.real_precon(1, S)
    b = S.mv(np.ones(n ** 3))
    r = oracle.pp_idrs(S, b, P=D, method=0, s=8, tol=1e-8, preconditioner=2, degree=8, n_ritz=20)
    assert r.flag == 0 and r.relres_original < 1e-8 * 1.0001 or r.relres_original < 2e-8
    np.testing.assert_allclose(r.x, 1.0, atol=1e-6)


def test_nested_msqmridr_single_precision_inner_floor(oracle, P):
    """The nested MSQMRIDR(4) with MSIDRS(4) inner (msqmridr.inc:162-175)
    forms every shift's residual from the inner collinearity factors.  With
    the inner results rounded to single precision (the oracle's
    inner_round32 probe, as a complex64 inner solve hands them on) the
    shifted systems stop near 3e-8 with flag 2, where the exact nested solve
    reaches 1e-8 on every shift: the floor of the complex64 inner form is the
    method's, not the GPU's arithmetic."""
    n = 10
    N = n ** 3
    K = oracle.stencil7_format(n, n, n, P.laplace_coefficients(n))
    A = oracle.Matrix(K, cplx=True)
    b = P.complex_unit_normal(N)
    sd, _ = P.multishift_shifts(n, n_shifts=6, lo=1.2, hi=4.0)
    kw = dict(tolerance=1e-8, inner_s=4, inner_iterations=10, inner_tolerance=0.1, maximum_iterations=200)

    def true_relres(x):
        return np.array([np.linalg.norm(b - (K.mv(x[:, k]) - sd[k] * x[:, k])) / np.linalg.norm(b)
                         for k in range(len(sd))])
    exact = oracle.msqmridr(A, b, sd, 4, **kw)
    rounded = oracle.msqmridr(A, b, sd, 4, inner_round32=True, **kw)
    assert exact.flag == 0 and np.all(true_relres(exact.x) <= 1e-8)
    rr = true_relres(rounded.x)
    assert rounded.flag == 2 and np.all(rr > 1e-8) and np.all(rr < 1e-6)


def test_multishift_oracle(oracle, P):
    """MSIDRS / MSQMRIDR on a small shifted Laplacian: every shifted system's
    true residual meets the tolerance."""
    n = 8
    K = oracle.stencil7_format(n, n, n, P.laplace_coefficients(n))
    A = oracle.Matrix(K, cplx=True)
    sig, _ = P.multishift_shifts(n, n_shifts=4, lo=0.1, hi=0.9)
    b = P.complex_unit_normal(n ** 3)
    r = oracle.msidrs(A, b, sig, 4, tolerance=1e-8, maximum_iterations=2000)
    assert r.flag == 0 and np.max(r.relres) < 1e-8
    q = oracle.msqmridr(A, b, sig, 4, tolerance=1e-8, maximum_iterations=2000)
    assert q.flag == 0 and np.max(q.relres) < 1e-8


def test_adjoint_oracle(oracle, P):
    """The FP64 reference gradient: transposed CRS equals the dense transpose,
    lambda solves A^T lambda = x - x_t, and -lambda_i x_j matches central
    differences of L = 1/2 ||x - x_t||^2 on a few entries (dense FP64 solves)."""
    n = 6
    N = n ** 3
    coef = P.cdr_coefficients(n)
    rp, ci, vals = P.stencil_to_crs(n, n, n, coef)
    rows = np.repeat(np.arange(N), np.diff(rp))
    D = np.zeros((N, N))
    D[rows, ci - 1] = vals
    Ko = oracle.crs_format(N, N, rp, ci, vals)
    KT = oracle.crs_transpose(Ko)
    v = np.random.default_rng(0).standard_normal(N)
    np.testing.assert_allclose(KT.mv(v), D.T @ v, rtol=1e-13, atol=1e-12)
    rng = np.random.default_rng(1)
    b, xt = rng.standard_normal(N), rng.standard_normal(N)
    x = oracle.idrs(oracle.Matrix(Ko), b, 4, tolerance=1e-13).x
    lam = oracle.idrs(oracle.Matrix(KT), x - xt, 4, tolerance=1e-13).x
    g = oracle.sparse_outer_grad(Ko, lam, x, len(vals))
    np.testing.assert_array_equal(g, -lam[rows] * x[ci - 1])
    eps = 1e-6
    res = x - xt

    def central(dp, dm):
        # L(+) - L(-) with d = x(+-) - x, rearranged so no large losses cancel
        return (res @ (dp - dm) + 0.5 * (dp @ dp - dm @ dm)) / (2 * eps)

    for p in (0, 17, 333, len(vals) - 1):
        i, j = rows[p], ci[p] - 1
        d = []
        for sgn in (1.0, -1.0):
            Dp = D.copy()
            Dp[i, j] += sgn * eps
            rhs = np.zeros(N)
            rhs[i] = -sgn * eps * x[j]
            d.append(np.linalg.solve(Dp, rhs))
        assert abs(central(*d) - g[p]) <= 1e-5 * abs(g[p])
    for k in (3, 100):
        e = np.zeros(N)
        e[k] = eps
        fd = central(np.linalg.solve(D, e), np.linalg.solve(D, -e))
        assert abs(fd - lam[k]) <= 1e-5 * abs(lam[k])


# --------------------------------------------------------------------------
# recycling: IDRS_RITZ's omega and U0 outputs, PP_MR_IDRS
# --------------------------------------------------------------------------
def _mgs(V, refine):
    """Modified Gram-Schmidt QR (refine sweeps per column), numpy."""
    Q = np.array(V, dtype=float, copy=True)
    R = np.zeros((V.shape[1], V.shape[1]))
    for j in range(V.shape[1]):
        for _ in range(refine):
            for i in range(j):
                t = Q[:, i] @ Q[:, j]
                Q[:, j] -= t * Q[:, i]
                R[i, j] += t
        R[j, j] = np.linalg.norm(Q[:, j])
        Q[:, j] /= R[j, j]
    return Q, R


def _ritz_problem(oracle, P, n=10, s=4, seed=0):
    coef = P.cdr_coefficients(n)
    rp, ci, vals = P.stencil_to_crs(n, n, n, coef)
    K = oracle.crs_format(n ** 3, n ** 3, rp, ci, vals)
    b = np.random.default_rng(seed).standard_normal(n ** 3)
    return K, oracle.Matrix(K), b


def test_si_power_matches_numpy(oracle, P):
    """RSI_power (dense_la_module.f90:531-603) restated in numpy from the same
    counter-based start block: block inverse iteration with MGS(refine 2)
    re-orthonormalisation until the summed column lengths change by <= 1e-3
    of the start block's."""
    K, A, b = _ritz_problem(oracle, P)
    s = 4
    r = oracle.idrs(A, b, s, tolerance=1e-8, maximum_iterations=200, H_shape=(201, 200))
    nr = (r.iterations // (s + 1)) * s + r.iterations % (s + 1)
    Hn = r.H[:nr, :nr]
    Q, R = _mgs(Hn, 2)
    X = np.array([oracle.uniform(2, k) for k in range(nr * s)]).reshape(s, nr).T
    Qs, Rs = _mgs(X, 2)
    tr0 = told = np.trace(Rs)
    for _ in range(1000):
        Qs, Rs = _mgs(np.linalg.solve(np.triu(R), Q.T @ Qs), 2)
        err = abs(np.trace(Rs) - told) / tr0
        told = np.trace(Rs)
        if err <= 1e-3:
            break
    np.testing.assert_allclose(oracle.si_power(Hn, s), Qs, rtol=0, atol=1e-10)


def test_ritz_omega_and_u0_match_numpy(oracle, P):
    """IDRS_RITZ's omega ordering (ritz_module.f90:497-520) and the recycle
    space (compute_U0 :100-160 + global QR :66-96) restated in numpy."""
    K, A, b = _ritz_problem(oracle, P)
    s, n_om = 4, 6
    r = oracle.idrs_ritz(A, b, s, tolerance=1e-8, n_omega=n_om, dimU0=s)
    h = oracle.idrs(A, b, s, tolerance=1e-8, H_shape=(1001, 1000))
    assert r.iterations == h.iterations and r.flag == 0
    nr = r.nritz
    H = h.H
    # omega: Ritz values of H(1:n_omega,1:n_omega) in QR_eig's order, greedy |p|
    rv, _ = oracle.qr_eig(H[:n_om, :n_om])
    om = 1.0 / np.where(np.abs(rv.real) < np.finfo(float).eps, 1.0, rv.real)
    p = np.ones(n_om)
    for i in range(n_om):
        m = i + int(np.argmax(np.abs(p[i:])))
        om[i], om[m] = om[m], om[i]
        p *= 1.0 - rv.real * om[i]
    np.testing.assert_allclose(r.omega, om, rtol=1e-12)
    # U0: Krylov basis rebuilt from the Hessenberg recurrence, then MGS
    vec = oracle.si_power(H[:nr, :nr], s)
    V = [b.copy()]
    U = np.zeros((len(b), s))
    for i in range(nr):
        U += np.outer(V[i], vec[i])
        low = max(0, i - s)
        acc = sum(V[l] * H[l, i] for l in range(low, i + 1))
        V.append((A.matvec(V[i]) - acc) / H[i + 1, i])
    U /= np.linalg.norm(U, axis=0)
    Q, _ = _mgs(U, 1)
    np.testing.assert_allclose(r.U0, Q, rtol=0, atol=1e-9)
    assert np.abs(r.U0.T @ r.U0 - np.eye(s)).max() < 1e-12
    with pytest.raises(ValueError):  # more omegas than Ritz values
        oracle.idrs_ritz(A, b, s, tolerance=1e-8, maximum_iterations=3, n_omega=6)


def test_pp_mr_idrs_oracle(oracle, P):
    """PP_MR_IDRS: every right-hand side meets the tolerance on the original
    system; the warm start makes a repeated right-hand side free, and the
    recycle solve already solves b_all(:,1)."""
    n = 10
    coef = P.cdr_coefficients(n)
    S = oracle.stencil7_format(n, n, n, coef)
    D = oracle.real_precon(1, S)
    rng = np.random.default_rng(1)
    B = rng.standard_normal((n ** 3, 3))
    B = np.column_stack([B, B[:, 1]])  # rhs 4 repeats rhs 2
    r = oracle.pp_mr_idrs(S, B, P=D, s=4, tol=1e-8, preconditioner=2, degree=4, n_ritz=12,
                          n_omega=3)
    assert list(r.flags) == [0, 0, 0, 0]
    assert np.all(r.relres_original < 1e-7)
    for j in range(B.shape[1]):
        res = B[:, j] - S.mv(r.x[:, j])
        assert np.linalg.norm(res) <= 1e-7 * np.linalg.norm(B[:, j])
    rr = oracle.pp_mr_idrs(S, B[:, :2], P=D, s=4, tol=1e-8, recycle=True)
    assert rr.recycle_flag == 0 and rr.recycle_iterations > 0
    assert rr.iterations[0] == 0 and rr.flags[1] == 0
    same = oracle.pp_mr_idrs(S, np.column_stack([B[:, 0], B[:, 0]]), s=4, tol=1e-8)
    assert same.iterations[1] <= 1


@pytest.mark.parametrize("useM,useC,ms,seed", [
    (True, True, False, 3.0), (False, True, False, -2.0), (True, False, False, 5.0),
    (False, False, False, 1.5), (True, True, False, 0.0), (True, True, True, 4.0),
    (False, True, True, 4.0), (True, True, True, 0.0), (False, True, True, 0.0)])
def test_system_operator_oracle_matches_dense(oracle, P, useM, useC, ms, seed):
    """real_mv (matrix_module.f90:218-264) with mass/damping matrices and the
    2x2 block system, against dense numpy matrices (with diagonal scaling)."""
    n = 4
    N = n ** 3
    rp, ci, kv = P.stencil_to_crs(n, n, n, P.cdr_coefficients(n))
    rows = np.repeat(np.arange(N), np.diff(rp))
    Kd = np.zeros((N, N)); Kd[rows, ci - 1] = kv
    rng = np.random.default_rng(3)
    Md = np.diag(rng.uniform(1, 2, N)) + 0.1 * np.diag(rng.uniform(0, 1, N - 1), 1)
    Cd = 0.05 * Kd + 0.01 * np.diag(rng.uniform(0, 1, N - 1), -1)

    def crs(D):
        r, c = np.nonzero(D)
        rp_ = np.concatenate([[1], 1 + np.cumsum(np.bincount(r, minlength=N))]).astype(np.int32)
        return oracle.crs_format(N, N, rp_, (c + 1).astype(np.int32), D[r, c])
    K, M, Cm = crs(Kd), crs(Md), crs(Cd)
    Pd = oracle.real_precon(1, K)
    A = oracle.Matrix(K, P=Pd, M=M if useM else None, C_=Cm if useC else None, seed=seed,
                      multishift=ms)
    dinv = 1.0 / np.diag(Kd)
    I = np.eye(N)
    if ms and useC:
        top = -Cd - (seed * Md if (useM and seed) else seed * I)
        S = np.block([[top, -Kd], [I, -seed * I]])
        dv = np.concatenate([dinv, np.ones(N)])
    else:
        if seed == 0:
            S = Kd
        elif useC:
            S = Kd + seed * Cd + seed ** 2 * (Md if useM else I)
        elif useM:
            S = Kd - seed * Md
        else:
            S = Kd - seed * I
        dv = dinv
    v = rng.standard_normal(A.n)
    np.testing.assert_allclose(A.matvec(v), S @ (dv * v), rtol=1e-12, atol=1e-10)
    np.testing.assert_allclose(A.precon(v), dv * v, rtol=1e-15)


@pytest.mark.parametrize("useM,useC", [(True, True), (False, True), (True, False), (False, False)])
@pytest.mark.parametrize("shift", [None, 2.5, 1.0 - 0.5j])
def test_precon_with_mass_and_damping_oracle(oracle, P, useM, useC, shift):
    """REAL_PRECON / COMPLEX_PRECON(1, K, M, C, shift) (user_module.f90:1352-1381):
    each matrix's diagonal with zeros -> 1, combined by the shift."""
    n = 4
    N = n ** 3
    rp, ci, kv = P.stencil_to_crs(n, n, n, P.cdr_coefficients(n))
    K = oracle.crs_format(N, N, rp, ci, kv)
    dm = np.where(np.arange(N) % 3 == 0, 0.0, 1.5)    # zeros become 1
    dc = np.where(np.arange(N) % 4 == 0, 0.3, 0.0)
    ii = np.arange(1, N + 2, dtype=np.int32)
    M = oracle.crs_format(N, N, ii, ii[:-1], dm)
    C = oracle.crs_format(N, N, ii, ii[:-1], dc)
    cplx = isinstance(shift, complex)
    fn = oracle.complex_precon if cplx else oracle.real_precon
    Pm = fn(1, K, shift=shift, M=M if useM else None, C_=C if useC else None)
    fix = lambda d: np.where(d == 0, 1.0, d)
    dK = fix(np.array([kv[p] for i in range(N) for p in range(rp[i] - 1, rp[i + 1] - 1)
                       if ci[p] - 1 == i]))
    s = 0.0 if shift is None else shift
    if shift is None:
        D = dK
    elif useM and useC:
        D = dK + s * fix(dc) + s ** 2 * fix(dm)
    elif useC:
        D = dK + s * fix(dc) + s ** 2
    elif useM:
        D = dK - s * fix(dm)
    else:
        D = dK - s
    A = oracle.Matrix(K, P=Pm, cplx=cplx)
    v = np.random.default_rng(1).standard_normal(N) + (0.5j if cplx else 0)
    np.testing.assert_allclose(A.precon(v), v / D, rtol=1e-15)


def _scaled_cdr(oracle, P, n=6):
    N = n ** 3
    rp, ci, kv = P.stencil_to_crs(n, n, n, P.cdr_coefficients(n))
    rows = np.repeat(np.arange(N), np.diff(rp))
    D = np.zeros((N, N))
    D[rows, ci - 1] = kv
    K = oracle.crs_format(N, N, rp, ci, kv)
    return N, K, D, D / np.diag(D)[None, :]   # As = K D^-1


def test_deflation_oracle(oracle, P):
    """make_deflation / Pmul / add_deflation (matrix_module.f90:1284-1623)
    against dense numpy; a deflated solve recovers the solution of A x = b;
    the multishift projector I - V V^H with V spanning an invariant subspace
    gives every shifted system's solution."""
    N, K, D, As = _scaled_cdr(oracle, P)
    rng = np.random.default_rng(0)
    V = rng.standard_normal((N, 3))
    A = oracle.Matrix(K, P=oracle.real_precon(1, K))
    A.make_deflation(V)
    w = rng.standard_normal(N)
    AV = As @ V
    np.testing.assert_allclose(A.pmul(w), w - AV @ np.linalg.solve(V.T @ AV, V.T @ w), atol=1e-12)
    b = rng.standard_normal(N)
    r = oracle.idrs(A, A.pmul(b), 4, tolerance=1e-11, maximum_iterations=2000)
    x = A.scaleback(b, r.x)
    assert r.flag == 0 and np.linalg.norm(b - D @ x) <= 1e-9 * np.linalg.norm(b)
    # complex, multishift: I - V V^H, V an orthonormal basis of an invariant subspace of As
    ev, EV = np.linalg.eig(As)
    Vi, _ = np.linalg.qr(EV[:, np.argsort(np.abs(ev))[:2]])
    Ac = oracle.Matrix(K, P=oracle.complex_precon(1, K), cplx=True, multishift=True)
    Ac.make_deflation(Vi)
    wc = w + 1j * rng.standard_normal(N)
    np.testing.assert_allclose(Ac.pmul(wc), wc - Vi @ (Vi.conj().T @ wc), atol=1e-12)
    bc = b + 1j * rng.standard_normal(N)
    sig = np.array([0.1, 0.3 + 0.1j])
    o = oracle.msidrs(Ac, Ac.pmul(bc), Ac.ms_parameters(sig), 4, tolerance=1e-11,
                      maximum_iterations=3000)
    X = Ac.ms_scaleback(o.x, bc)
    Dm = np.diag(np.diag(D))
    for k, s in enumerate(sig):  # (K D^-1 - s) y = b  <=>  (K - s D) x = b
        assert np.linalg.norm(bc - (D - s * Dm) @ X[:, k]) <= 1e-9 * np.linalg.norm(bc)


def _mass_and_damping(oracle, N, rng):
    """a tridiagonal mass matrix and a diagonal damping matrix, CRS, plus dense copies"""
    Md = np.diag(rng.uniform(1.0, 2.0, N)) + np.diag(np.full(N - 1, 0.1), 1) + np.diag(np.full(N - 1, 0.1), -1)
    Cd = np.diag(rng.uniform(0.0, 0.5, N))

    def crs(Dm):
        r, c = np.nonzero(Dm)
        rp = np.concatenate([[1], 1 + np.cumsum(np.bincount(r, minlength=N))]).astype(np.int32)
        return oracle.crs_format(N, N, rp, (c + 1).astype(np.int32), Dm[r, c])
    return crs(Md), Md, crs(Cd), Cd


@pytest.mark.parametrize("which", [2, 3])
@pytest.mark.parametrize("form", ["none", "K", "M", "C", "MC"])
def test_lu_preconditioners_oracle(oracle, P, which, form):
    """REAL_PRECON(2 dense LU / 3 band LU, K[, M, C, shift]) (user_module.f90:1383-1463):
    v / P solves with the shifted matrix."""
    N, K, D, _ = _scaled_cdr(oracle, P, n=4)
    rng = np.random.default_rng(4)
    M, Md, C, Cd = _mass_and_damping(oracle, N, rng)
    sh = 2.5
    kw, S = {}, D.copy()
    if form == "K":
        kw, S = dict(shift=sh), D - sh * np.eye(N)
    elif form == "M":
        kw, S = dict(shift=sh, M=M), D - sh * Md
    elif form == "C":
        kw, S = dict(shift=sh, C_=C), D + sh * Cd + sh ** 2 * np.eye(N)
    elif form == "MC":
        kw, S = dict(shift=sh, M=M, C_=C), D + sh * Cd + sh ** 2 * Md
    Pm = oracle.real_precon(which, K, **kw)
    A = oracle.Matrix(K, P=Pm)
    v = rng.standard_normal(N)
    np.testing.assert_allclose(A.precon(v), np.linalg.solve(S, v), rtol=1e-10, atol=1e-13)


def test_shift_and_invert_multishift_oracle(oracle, P):
    """Multishift with a band-LU shift-and-invert preconditioner at `shift`
    (matrix_module.f90:402-483, :724-766): the shifted systems
    (K - sigma M) x = b all come out of one MSIDRS run."""
    N, K, D, _ = _scaled_cdr(oracle, P, n=5)
    rng = np.random.default_rng(6)
    M, Md, _, _ = _mass_and_damping(oracle, N, rng)
    seed, shift = 0.0, -60.0
    Pm = oracle.complex_precon(3, K, shift=shift, M=M)
    A = oracle.Matrix(K, P=Pm, M=M, seed=seed, shift=shift, cplx=True, multishift=True)
    sig = np.array([10.0, 20.0 + 5j, -5.0])
    sp = A.ms_parameters(sig)
    np.testing.assert_allclose(sp, (sig - seed) / (sig - shift), rtol=1e-15)
    b = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    o = oracle.msidrs(A, b, sp, 4, tolerance=1e-11, maximum_iterations=2000)
    assert o.flag == 0
    X = A.ms_scaleback(o.x, b)
    for k, s in enumerate(sig):
        assert np.linalg.norm(b - (D - s * Md) @ X[:, k]) <= 1e-9 * np.linalg.norm(b)


def test_block_shift_and_invert_oracle(oracle, P):
    """The damped multishift problem (K + sigma C + sigma^2 M) x = rhs on the
    2 x 2 block system with rprecon's shift-and-invert block form
    (matrix_module.f90:318-345): every frequency from one MSIDRS run."""
    N, K, D, _ = _scaled_cdr(oracle, P, n=4)
    rng = np.random.default_rng(8)
    M, Md, C, Cd = _mass_and_damping(oracle, N, rng)
    tau = 3.0 + 2.0j
    Pm = oracle.complex_precon(3, K, shift=tau, M=M, C_=C)
    sig = np.array([1.0 + 1.0j, 2.0 + 0.5j, 4.0 + 1.0j])
    seed = sig[-1]
    A = oracle.Matrix(K, P=Pm, M=M, C_=C, seed=seed, shift=tau, cplx=True, multishift=True)
    rhs = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    b = np.concatenate([-rhs, np.zeros(N)])
    sp = A.ms_parameters(sig)
    o = oracle.msidrs(A, b, sp, 4, tolerance=1e-11, maximum_iterations=3000)
    assert o.flag == 0
    X = A.ms_scaleback(o.x, b)[N:, :]
    for k, s in enumerate(sig):
        S = D + s * Cd + s ** 2 * Md
        assert np.linalg.norm(rhs - S @ X[:, k]) <= 1e-8 * np.linalg.norm(rhs)


@pytest.mark.parametrize("n,hb,cplx", [(1000, 1, False), (333, 17, True), (95, 94, False), (300, 250, True)])
def test_band_lu_oracle_wide_and_ragged_bands(oracle, n, hb, cplx):
    """The oracle's band LU (band_LU_solve, user_module.f90:2181-2336) on the
    band shapes the GPU solves are checked with: tridiagonal, odd n, half band
    n - 1 and wide complex bands -- against numpy solves."""
    rng = np.random.default_rng(n + hb)
    A = np.zeros((n, n), complex if cplx else float)
    for i in range(n):
        lo, hi = max(0, i - hb), min(n, i + hb + 1)
        A[i, lo:hi] = rng.standard_normal(hi - lo) + (1j * rng.standard_normal(hi - lo) if cplx else 0)
        A[i, i] += 2.0 * hb + 2.0
    r, c = np.nonzero(A)
    rp = np.concatenate([[1], 1 + np.cumsum(np.bincount(r, minlength=n))]).astype(np.int32)
    K = oracle.crs_format(n, n, rp, (c + 1).astype(np.int32), A[r, c])
    Pm = oracle.complex_precon(3, K) if cplx else oracle.real_precon(3, K)
    Ao = oracle.Matrix(K, P=Pm, cplx=cplx)
    v = rng.standard_normal(n) + (1j * rng.standard_normal(n) if cplx else 0)
    np.testing.assert_allclose(Ao.precon(v), np.linalg.solve(A, v), rtol=1e-10, atol=1e-13)


def _random_example(kind, n, hb, rng):
    """E/RANDOM: uniform random band (CDS, entries outside the matrix zeroed,
    band_real.f90:58-70) or dense matrix (dense_complex.f90:56-64); returns
    the dense copy, the band or matrix as stored, and whether it is complex."""
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
def test_random_examples_oracle(oracle, kind):
    """The reference's RANDOM examples (band_real.f90:39-82, dense_complex.f90:
    38-71): A from cds_format / dense_format, b = A 1, P = its band / dense LU
    (real_precon 3 / 2), the solution of A x = b is 1."""
    rng = np.random.default_rng({"band_real": 1, "band_complex": 2, "dense_real": 3, "dense_complex": 4}[kind])
    n, hb = (400, 6) if kind.startswith("band") else (120, 0)
    A, R, cplx = _random_example(kind, n, hb, rng)
    K = oracle.cds_format(n, n, hb, R) if kind.startswith("band") else oracle.dense_format(R)
    which = 3 if kind.startswith("band") else 2
    P = oracle.complex_precon(which, K) if cplx else oracle.real_precon(which, K)
    Ao = oracle.Matrix(K, P=P, cplx=cplx)
    v = rng.standard_normal(n) + (1j * rng.standard_normal(n) if cplx else 0)
    x = Ao.precon(v)
    np.testing.assert_allclose(x, np.linalg.solve(A, v), rtol=1e-8, atol=1e-10)
    # the unpivoted LU is backward stable up to its growth: measured 1.5e-13
    # (dense_real, growth 1.8e4), 1.5e-15 (dense_complex) and smaller for the bands
    berr = np.linalg.norm(A @ x - v) / (np.linalg.norm(A, 2) * np.linalg.norm(x))
    assert berr <= 1e-12, berr
    b = A @ np.ones(n)
    r = oracle.idrs(Ao, b, 4, tolerance=1e-10)  # pp_idrs without a polynomial: IDR(4) on A P^-1
    assert r.flag == 0
    np.testing.assert_allclose(Ao.scaleback(b, r.x), 1.0, atol=1e-6)


@pytest.mark.parametrize("prec,kw", [(2, dict(foci=[0.05, 1.9])), (1, dict(center=1.0))])
@pytest.mark.parametrize("degree", [1, 2, 8])
def test_recurrence_evaluation_oracle(oracle, P, prec, kw, degree):
    """The Jacobi three-term recurrence of the Chebyshev / Neumann polynomial
    (matrix_module.f90:851-941) gives the same A p(A) v and D^-1 p(A) y as
    the reference's Horner rpolpre (:266-284) and the dense closed form."""
    N, K, D, As = _scaled_cdr(oracle, P)
    rng = np.random.default_rng(degree)
    v = rng.standard_normal(N)
    A = oracle.Matrix(K, P=oracle.real_precon(1, K))
    A.preconditioner(prec, degree, **kw)
    a = oracle.chebyshev(degree, kw["foci"]) if prec == 2 else oracle.neumann(degree, kw["center"])
    pv = sum(a[k] * np.linalg.matrix_power(As, k) @ v for k in range(degree + 1))
    w_h = A.matvec(v)
    y_h = A.scaleback(v, v)
    A.set_poly_eval(1)
    w_r = A.matvec(v)
    y_r = A.scaleback(v, v)
    np.testing.assert_allclose(w_r, As @ pv, rtol=1e-10, atol=1e-10 * np.abs(As @ pv).max())
    np.testing.assert_allclose(w_r, w_h, rtol=1e-10, atol=1e-10 * np.abs(w_h).max())
    dinv = 1.0 / np.diag(D)
    np.testing.assert_allclose(y_r, dinv * pv, rtol=1e-10, atol=1e-10 * np.abs(dinv * pv).max())
    np.testing.assert_allclose(y_r, y_h, rtol=1e-10, atol=1e-10 * np.abs(y_h).max())
