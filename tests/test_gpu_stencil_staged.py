"""The fp32 stencil pair whose xin / u / v rows are staged in shared memory
by bulk asynchronous copies (k_stencil7_f8x2t) computes every point with the
same FMAs as the unstaged pair (k_stencil7_f8x2): the two products agree bit
for bit.  The unstaged kernel runs in a child process started with
IDRS_STAGED_PAIR=0 (the choice is made once per process)."""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHAPES = [(256, 17, 6), (64, 7, 9), (8, 5, 3), (128, 33, 20), (16, 16, 16), (256, 3, 5), (96, 40, 31)]

CHILD = r"""
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
import __graft_entry__ as g
pkg = g.load_package(); pkg.load()
out = []
for nx, ny, nz in %r:
    coef = pkg.problems.cdr_coefficients(max(nx, ny, nz))
    K = pkg.stencil7_format(nx, ny, nz, coef)
    for poly in ("chebyshev", "neumann"):
        A = pkg.Matrix(K, P=pkg.real_precon(1, K))
        if poly == "chebyshev":
            A.preconditioner(2, 8, foci=[0.05, 1.9])
        else:
            A.preconditioner(1, 6, center=1.0)
        v = np.random.default_rng(nx + ny + nz).standard_normal(nx * ny * nz)
        out.append(A.matvec32(v))
np.savez(sys.argv[2], *out)
"""


def _products(tmp_path, staged):
    path = str(tmp_path / ("staged" if staged else "plain")) + ".npz"
    env = dict(os.environ, IDRS_STAGED_PAIR="1" if staged else "0")
    subprocess.run([sys.executable, "-c", CHILD % (SHAPES,), ROOT, path], env=env, check=True, timeout=600)
    d = np.load(path)
    return [d[f"arr_{i}"] for i in range(len(d.files))]


def test_staged_pair_equals_unstaged_bitwise(gpu, tmp_path):
    staged = _products(tmp_path, True)
    plain = _products(tmp_path, False)
    assert len(staged) == len(plain) == 2 * len(SHAPES)
    for a, b in zip(staged, plain):
        assert np.all(np.isfinite(a))
        np.testing.assert_array_equal(a, b)
