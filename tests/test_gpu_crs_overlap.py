"""The long-row bin of a length-binned CRS matrix run on a side stream beside
the short and middle bins (forked from and joined to the caller's stream)
against all bins on one stream (IDRS_CRS_OVERLAP=0, in a child process).  The
bins write disjoint rows, so fp64 and fp32 products, an IDR(s) solve (whose
captured cycle graph holds the fork and the join) and a mixed QMRIDR(s) solve
agree bit for bit, with the same launch count."""
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


def ragged(n, seed):
    # power-law rows (mean <= 16: one lane per row and the length bins), some
    # empty, a few longer than the 256-nonzero segments
    rng = np.random.default_rng(seed)
    L = np.minimum(rng.zipf(1.8, n), 2000)
    L[rng.integers(0, n, n // 20)] = 0
    L[rng.integers(0, n, 4)] = 700
    rp = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(L, out=rp[1:])
    ci = rng.integers(0, n, int(rp[-1]))
    vals = rng.standard_normal(int(rp[-1]))
    return (rp + 1).astype(np.int32), (ci + 1).astype(np.int32), vals


for rp, ci, vals in [P.pagerank_crs(50001)[:3], ragged(3001, 1), ragged(70000, 3)]:
    n = len(rp) - 1
    K = pkg.crs_format(n, n, rp, ci, rval=vals)
    A = pkg.Matrix(K)
    v = np.random.default_rng(n).standard_normal(n)
    out += [K * v, A.matvec32(v)]
rp, ci, vals, b = P.pagerank_crs(50001)
n = len(b)
A = pkg.Matrix(pkg.crs_format(n, n, rp, ci, rval=vals))
r = pkg.IDRS(A, b, 4, tolerance=1e-10, resvec=True)
out += [r.x, r.resvec]
q = pkg.QMRIDR(A, b, 4, tolerance=1e-10, maximum_iterations=50, inner_s=4, inner_iterations=20,
               inner_tolerance=1e-3, inner_precision=32, resvec=True, fp64_check=False)
out += [q.x, q.resvec]
out.append(np.array([lib.idrs_launch_count() - l0]))
np.savez(sys.argv[2], *out)
"""


def _run(tmp_path, overlap):
    path = str(tmp_path / ("overlap" if overlap else "serial")) + ".npz"
    env = dict(os.environ, IDRS_CRS_OVERLAP="1" if overlap else "0")
    subprocess.run([sys.executable, "-c", CHILD, ROOT, path], env=env, check=True, timeout=600)
    d = np.load(path)
    return [d[f"arr_{i}"] for i in range(len(d.files))]


def test_long_bin_on_side_stream_equals_one_stream(gpu, tmp_path):
    ov, se = _run(tmp_path, True), _run(tmp_path, False)
    assert len(ov) == len(se) == 11
    for a, b in zip(ov, se):
        assert np.all(np.isfinite(a))
        np.testing.assert_array_equal(a, b)
