"""IDR(s) cycles replayed from a captured CUDA graph (standalone solves, and
the inner solves of a flexible QMRIDR(s), which share one graph per outer
solve) against the same cycles launched one by one (IDRS_CYCLE_GRAPHS=0, in a
child process): the graph runs the same kernels with the same arguments, so
solutions, residual histories and iteration counts agree bit for bit, and the
library's launch counter reports the same launches.  Direct launches with and
without programmatic dependent launch (IDRS_PDL=0) agree bit for bit too."""
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
P = pkg.problems
lib = pkg.lib()
l0 = lib.idrs_launch_count()
out = []
n = 20
rp, ci, vals = P.stencil_to_crs(n, n, n, P.cdr_coefficients(n))
K = pkg.crs_format(n ** 3, n ** 3, rp, ci, rval=vals)
A = pkg.Matrix(K, P=pkg.real_precon(1, K))
A.preconditioner(2, 4, foci=[0.05, 1.9])
b = K * np.ones(n ** 3)
for s in (1, 4):
    r = pkg.IDRS(A, b, s, tolerance=1e-8, resvec=True)
    out += [r.x, r.resvec, np.array([r.flag, r.iterations])]
m = 24
S = pkg.stencil7_format(m, m, m, P.cdr_coefficients(m))
bs = S * np.ones(m ** 3)
for prec in (32, 64):
    r = pkg.PP_IDRS(S, bs, P=pkg.real_precon(1, S), method=0, s=8, tol=1e-8, maxit=60, preconditioner=2,
                    degree=8, n_ritz=20, in_s=4, in_it=40, in_tol=1e-2, inner_precision=prec, poly_eval=1)
    out += [r.x, np.array([r.flag, r.iterations, r.inner_iterations, r.relres_original])]
B = pkg.Matrix(S, P=pkg.real_precon(1, S))
B.preconditioner(2, 8, foci=[0.05, 1.9])
q = pkg.QMRIDR(B, bs, 8, tolerance=1e-8, maximum_iterations=12, inner_s=4, inner_iterations=20,
               inner_tolerance=1e-3, inner_precision=32, resvec=True)
out += [q.x, q.resvec]
out.append(np.array([lib.idrs_launch_count() - l0]))
np.savez(sys.argv[2], *out)
"""


def _run(tmp_path, graphs, pdl=True):
    path = str(tmp_path / (("graphs" if graphs else "direct") + ("" if pdl else "_nopdl"))) + ".npz"
    env = dict(os.environ, IDRS_CYCLE_GRAPHS="1" if graphs else "0", IDRS_PDL="1" if pdl else "0")
    subprocess.run([sys.executable, "-c", CHILD, ROOT, path], env=env, check=True, timeout=600)
    d = np.load(path)
    return [d[f"arr_{i}"] for i in range(len(d.files))]


def test_cycle_graphs_equal_direct_launches(gpu, tmp_path):
    gr, di = _run(tmp_path, True), _run(tmp_path, False)
    assert len(gr) == len(di) == 13
    for a, b in zip(gr, di):
        assert np.all(np.isfinite(a))
        np.testing.assert_array_equal(a, b)
    assert gr[2][0] == gr[5][0] == 0  # standalone IDR(1), IDR(4) converged
    assert gr[7][0] == gr[9][0] == 0 and gr[7][2] > 0  # mixed PP_IDRS ran inner solves
    assert gr[12][0] > 0


def test_programmatic_launch_equals_stream_order(gpu, tmp_path):
    """Direct launches with programmatic dependent launch (the default) and
    without it (IDRS_PDL=0): every kernel launched so waits for its
    predecessor before it reads anything, so the results agree bit for bit."""
    on, off = _run(tmp_path, False, True), _run(tmp_path, False, False)
    assert len(on) == len(off) == 13
    for a, b in zip(on, off):
        np.testing.assert_array_equal(a, b)
