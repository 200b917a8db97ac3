"""IDR(s) solves that stop inside a cycle, on the GPU against the oracle.

The device applies the x update of each IDR(s) step (x += beta_k U_k,
idrs.inc:220) together with the omega step's (idrs.inc:289-290) in one pass,
and the steps of a cycle that the solve stopped in afterwards.  Stopping after
every iteration count of the first cycles (maximum_iterations = 1 .. 3(s+1))
with one shared shadow space must give the oracle's x (which updates x at every
step, as the reference) to rounding, for real and complex systems, with and
without a preconditioner M1 and an initial guess.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P(gpu):
    return gpu.problems


def _rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("s", [1, 2, 4])
def test_stop_inside_a_cycle_real(gpu, oracle, P, s):
    n = 8
    N = n ** 3
    rp, ci, vals = P.stencil_to_crs(n, n, n, P.cdr_coefficients(n))
    K = gpu.crs_format(N, N, rp, ci, rval=vals)
    Ko = oracle.crs_format(N, N, rp, ci, vals)
    A, Ao = gpu.Matrix(K), oracle.Matrix(Ko)
    b = Ko.mv(np.ones(N))
    PT = oracle.make_p(s, N, seed=11)
    A.set_shadow(s, PT)
    for it in range(1, 3 * (s + 1) + 1):
        g = gpu.IDRS(A, b, s, tolerance=1e-14, maximum_iterations=it)
        o = oracle.idrs(Ao, b, s, tolerance=1e-14, maximum_iterations=it, PT=PT)
        assert g.flag == 1 and o.flag == 1 and g.iterations == o.iterations == it
        # the solutions after `it` steps: rounding of the fused reductions only
        assert _rel(g.x, o.x) <= 1e-9, (s, it, _rel(g.x, o.x))


def test_stop_inside_a_cycle_x0_and_M1(gpu, oracle, P):
    s, n = 4, 8
    N = n ** 3
    rp, ci, vals = P.stencil_to_crs(n, n, n, P.cdr_coefficients(n))
    K = gpu.crs_format(N, N, rp, ci, rval=vals)
    Ko = oracle.crs_format(N, N, rp, ci, vals)
    A, Ao = gpu.Matrix(K), oracle.Matrix(Ko)
    M1 = gpu.Matrix(K, P=gpu.real_precon(1, K))
    M1o = oracle.Matrix(Ko, oracle.real_precon(1, Ko))
    b = Ko.mv(np.ones(N))
    x0 = np.random.default_rng(5).standard_normal(N)
    PT = oracle.make_p(s, N, seed=13)
    A.set_shadow(s, PT)
    for it in (3, 5, 7, 9):
        g = gpu.IDRS(A, b, s, M1=M1, x0=x0, tolerance=1e-14, maximum_iterations=it)
        o = oracle.idrs(Ao, b, s, M1=M1o, x0=x0, tolerance=1e-14, maximum_iterations=it, PT=PT)
        assert g.iterations == o.iterations == it
        assert _rel(g.x, o.x) <= 1e-9, (it, _rel(g.x, o.x))


@pytest.mark.parametrize("s", [2, 4])
def test_stop_inside_a_cycle_complex(gpu, oracle, P, s):
    rp, ci, vals, b = P.toeplitz_complex()
    N = len(b)
    A = gpu.Matrix(gpu.crs_format(N, N, rp, ci, cval=vals), complex=True)
    Ao = oracle.Matrix(oracle.crs_format(N, N, rp, ci, vals), cplx=True)
    PT = oracle.make_p(s, N, seed=17, cplx=True)
    A.set_shadow(s, PT)
    for it in range(1, 2 * (s + 1) + 2):
        g = gpu.IDRS(A, b, s, tolerance=1e-14, maximum_iterations=it)
        o = oracle.idrs(Ao, b, s, tolerance=1e-14, maximum_iterations=it, PT=PT)
        assert g.iterations == o.iterations == it
        assert _rel(g.x, o.x) <= 1e-9, (s, it, _rel(g.x, o.x))


def test_time_matvec_graph(gpu, P):
    """The product timed as a replayed CUDA graph (the roofline figure of the
    bench) and launched directly: both positive, of the same size."""
    n = 64
    S = gpu.stencil7_format(n, n, n, P.cdr_coefficients(n))
    A = gpu.Matrix(S, P=gpu.real_precon(1, S))
    A.preconditioner(2, 8, foci=[0.05, 1.9])
    for prec in (32, 64):
        direct, _ = A.time_matvec(prec, 2, 5)
        graph = A.time_matvec_graph(prec, 2, 5)
        assert direct > 0 and graph > 0
        assert 0.2 < graph / direct < 5.0
