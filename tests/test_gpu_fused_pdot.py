"""The projection P^T G_k of the fp32 inner IDR(s) accumulated by the last
pass of the stencil chain (k_stencil7_f4_dot) against the separate pass
(IDRS_FUSED_PDOT=0, in a child process): G_k is bitwise the same and the
inner products differ only in their summation order, so the flexible
QMRIDR(8)'s outer residuals agree closely and the solves meet 1e-8 alike."""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
import __graft_entry__ as g
pkg = g.load_package(); pkg.load()
n = 24
K = pkg.stencil7_format(n, n, n, pkg.problems.cdr_coefficients(n))
b = K * np.ones(n ** 3)
out = []
for in_s, in_it in ((4, 6), (4, 40), (2, 40)):
    r = pkg.PP_IDRS(K, b, P=pkg.real_precon(1, K), method=0, s=8, tol=1e-8, maxit=60, preconditioner=2,
                    degree=8, n_ritz=20, in_s=in_s, in_it=in_it, in_tol=1e-2, inner_precision=32, poly_eval=1,
                    fp64_check=False)
    out += [r.x, np.array([r.flag, r.iterations, r.inner_iterations, r.relres_original])]
A = pkg.Matrix(K, P=pkg.real_precon(1, K))
A.preconditioner(2, 8, foci=[0.05, 1.9])
for inner in (1, 8):
    q = pkg.QMRIDR(A, b, 8, tolerance=1e-8, maximum_iterations=3, inner_s=4, inner_iterations=inner,
                   inner_tolerance=1e-12, inner_precision=32, resvec=True, fp64_check=False)
    out.append(q.resvec[:4])
np.savez(sys.argv[2], *out)
"""


def _run(tmp_path, fused):
    path = str(tmp_path / ("fused" if fused else "plain")) + ".npz"
    env = dict(os.environ, IDRS_FUSED_PDOT="1" if fused else "0")
    subprocess.run([sys.executable, "-c", CHILD, ROOT, path], env=env, check=True, timeout=600)
    d = np.load(path)
    return [d[f"arr_{i}"] for i in range(len(d.files))]


def test_fused_projection_matches_separate_pass(gpu, tmp_path):
    f, p = _run(tmp_path, True), _run(tmp_path, False)
    for k in (0, 2, 4):  # PP_IDRS mixed: IDR(4) short and long inner solves, IDR(2)
        xf, sf, xp, sp = f[k], f[k + 1], p[k], p[k + 1]
        assert sf[0] == sp[0] == 0 and sf[3] <= 1e-8 and sp[3] <= 1e-8
        assert np.linalg.norm(xf - xp) / np.linalg.norm(xp) <= 1e-7
    # outer residuals of three QMRIDR(8) iterations: with one fp32 inner
    # iteration each the two forms differ only by the rounding of the
    # projection's sum; with eight inner iterations that difference grows
    # through the inner solve (measured 1.1e-4 after one outer iteration,
    # 1.7e-3 after three); a wrong projection would differ by O(1)
    np.testing.assert_allclose(f[6], p[6], rtol=1e-5)
    np.testing.assert_allclose(f[7], p[7], rtol=1e-2)
