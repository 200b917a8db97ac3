"""Synthetic test problems of the IDRS solve path (numpy only).

These generate, with fixed seeds, the operators and right-hand sides of the
workloads the package is measured and checked on:

* ``cdr_coefficients`` -- 7-point central-difference convection-diffusion-
  reaction stencil on the unit cube with Dirichlet boundaries, the operator of
  E/STENCIL/user_module.f90:520-567 (``cdr_matrix``) with caller-chosen
  diffusion ``eps``, convection ``beta`` and reaction ``r``.
* ``stencil_to_crs`` -- the same operator assembled as a CRS matrix,
  out-of-domain neighbours omitted (64^3: 1,810,432 nonzeros).
* ``laplace_coefficients`` -- 7-point Dirichlet Laplacian (c = 6/h^2).
* ``pagerank_crs`` -- (I - alpha*G/D) in CRS with power-law row lengths,
  following E/PAGERANK/pagerank.f90:87-134 for the structure.
* ``toeplitz_real`` / ``toeplitz_complex`` -- the two Toeplitz problems of
  E/TOEPLITZ/toeplitz.f90:20-177.

Grid ordering is x fastest, as in the reshape of E/STENCIL/user_module.f90:78.
Index arrays returned for the *_format calls are 1-based like the Fortran API.
"""
from __future__ import annotations

import numpy as np

STENCIL_ORDER = ("c", "w", "e", "s", "n", "f", "b")


def cdr_coefficients(n, eps=1.0, beta=(10.0, 10.0, 10.0), r=0.0, ny=None, nz=None):
    """Coefficients (c, w, e, s, n, f, b) of cdr_matrix (user_module.f90:548-556)
    on an n x ny x nz interior grid of the unit cube, h = 1/(n+1) per direction."""
    ny = n if ny is None else ny
    nz = n if nz is None else nz
    hx, hy, hz = 1.0 / (n + 1), 1.0 / (ny + 1), 1.0 / (nz + 1)
    bx, by, bz = beta
    c = 2.0 * eps / hx**2 + 2.0 * eps / hy**2 + 2.0 * eps / hz**2 + r
    e = -eps / hx**2 + bx / (2.0 * hx)
    w = -eps / hx**2 - bx / (2.0 * hx)
    nn = -eps / hy**2 + by / (2.0 * hy)
    s = -eps / hy**2 - by / (2.0 * hy)
    b = -eps / hz**2 + bz / (2.0 * hz)
    f = -eps / hz**2 - bz / (2.0 * hz)
    return np.array([c, w, e, s, nn, f, b], dtype=np.float64)


def laplace_coefficients(n):
    """7-point Dirichlet Laplacian (-Delta), h = 1/(n+1): c = 6/h^2, others -1/h^2."""
    h = 1.0 / (n + 1)
    return np.array([6.0 / h**2] + [-1.0 / h**2] * 6, dtype=np.float64)


def stencil_to_crs(nx, ny, nz, coef):
    """Assemble the 7-point stencil as CRS (1-based), columns ascending per row:
    f, s, w, c, e, n, b.  Out-of-domain neighbours are omitted."""
    c, w, e, s, n_, f, b = [float(v) for v in coef]
    N = nx * ny * nz
    idx = np.arange(N, dtype=np.int64)
    i = idx % nx
    j = (idx // nx) % ny
    k = idx // (nx * ny)
    offs = [(-nx * ny, f, k > 0), (-nx, s, j > 0), (-1, w, i > 0), (0, c, np.ones(N, bool)),
            (1, e, i < nx - 1), (nx, n_, j < ny - 1), (nx * ny, b, k < nz - 1)]
    valid = np.stack([m for _, _, m in offs], axis=1)          # N x 7
    cols = idx[:, None] + np.array([o for o, _, _ in offs])[None, :]
    vals = np.broadcast_to(np.array([v for _, v, _ in offs]), (N, 7))
    counts = valid.sum(axis=1)
    row_ptr = np.zeros(N + 1, dtype=np.int64)
    np.cumsum(counts, out=row_ptr[1:])
    col_ind = cols[valid].astype(np.int32) + 1
    values = np.ascontiguousarray(vals[valid], dtype=np.float64)
    return (row_ptr + 1).astype(np.int32), col_ind, values


def stencil_apply(nx, ny, nz, coef, v):
    """Reference numpy application of the stencil (for quick checks)."""
    c, w, e, s, n_, f, b = coef
    V = np.asarray(v).reshape(nz, ny, nx)
    P = np.zeros((nz + 2, ny + 2, nx + 2), dtype=V.dtype)
    P[1:-1, 1:-1, 1:-1] = V
    out = (c * P[1:-1, 1:-1, 1:-1] + w * P[1:-1, 1:-1, :-2] + e * P[1:-1, 1:-1, 2:]
           + s * P[1:-1, :-2, 1:-1] + n_ * P[1:-1, 2:, 1:-1] + f * P[:-2, 1:-1, 1:-1]
           + b * P[2:, 1:-1, 1:-1])
    return out.reshape(-1)


def crs_apply(row_ptr1, col_ind1, values, v):
    """Reference numpy CRS product (1-based arrays)."""
    rp = np.asarray(row_ptr1, dtype=np.int64) - 1
    ci = np.asarray(col_ind1, dtype=np.int64) - 1
    prod = np.asarray(values) * np.asarray(v)[ci]
    out = np.add.reduceat(prod, rp[:-1]) if len(prod) else np.zeros(len(rp) - 1, prod.dtype)
    out[np.diff(rp) == 0] = 0
    return out


def model_solution(nx, ny, nz):
    """x_model = sqrt(xyz(1-x)(1-y)(1-z)) of E/STENCIL/user_module.f90:652-673."""
    hx, hy, hz = 1.0 / (nx + 1), 1.0 / (ny + 1), 1.0 / (nz + 1)
    x = hx * np.arange(1, nx + 1)
    y = hy * np.arange(1, ny + 1)
    z = hz * np.arange(1, nz + 1)
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    return np.sqrt(X * Y * Z * (1 - X) * (1 - Y) * (1 - Z)).reshape(-1)


def zipf_row_lengths(nrows, seed=2024, exponent=2.1, mean=12.0, max_len=None):
    """Power-law row lengths: L = max(1, floor(kappa * Z)), Z ~ Zipf(exponent) on
    {1, 2, ...}, kappa chosen once (by bisection on the sample) so that the
    sample mean is `mean`.  Capped at max_len (default nrows // 4)."""
    rng = np.random.default_rng(seed)
    max_len = nrows // 4 if max_len is None else max_len
    z = rng.zipf(exponent, size=nrows).astype(np.float64)
    z = np.minimum(z, max_len)
    lo, hi = 0.5, 8.0
    for _ in range(60):
        kap = 0.5 * (lo + hi)
        m = np.maximum(1, np.minimum(np.floor(kap * z), max_len)).mean()
        if m < mean:
            lo = kap
        else:
            hi = kap
    L = np.maximum(1, np.minimum(np.floor(hi * z), max_len)).astype(np.int64)
    return L


def pagerank_crs(nrows, alpha=0.85, seed=2024, exponent=2.1, mean=12.0):
    """CRS (1-based) of I - alpha*G/D for a seeded random graph.

    Row i lists nnz_row(i) uniformly random columns (the in-links of node i),
    nnz_row ~ power law (zipf_row_lengths); G/D has value 1/outlinks(col),
    outlinks = nonzeros per column, 0 -> 1 for dangling columns, exactly as
    E/PAGERANK/pagerank.f90:87-134.  The identity diagonal is stored first in
    every row.  Returns (row_ptr1, col_ind1, values, b) with b = (1-alpha)/N.
    """
    rng = np.random.default_rng(seed + 1)
    L = zipf_row_lengths(nrows, seed=seed, exponent=exponent, mean=mean)
    nnz_g = int(L.sum())
    cols = rng.integers(0, nrows, size=nnz_g, dtype=np.int64)
    outlinks = np.bincount(cols, minlength=nrows).astype(np.float64)
    outlinks[outlinks == 0] = 1.0
    gvals = 1.0 / outlinks[cols]
    counts = L + 1
    row_ptr = np.zeros(nrows + 1, dtype=np.int64)
    np.cumsum(counts, out=row_ptr[1:])
    col_ind = np.empty(int(row_ptr[-1]), dtype=np.int64)
    values = np.empty(int(row_ptr[-1]), dtype=np.float64)
    diag_pos = row_ptr[:-1]
    col_ind[diag_pos] = np.arange(nrows)
    values[diag_pos] = 1.0
    mask = np.ones(int(row_ptr[-1]), dtype=bool)
    mask[diag_pos] = False
    col_ind[mask] = cols
    values[mask] = -alpha * gvals
    b = np.full(nrows, (1.0 - alpha) / nrows)
    return (row_ptr + 1).astype(np.int32), (col_ind + 1).astype(np.int32), values, b


def toeplitz_real(N=60, Pe=0.5):
    """1-D convection-diffusion of E/TOEPLITZ/toeplitz.f90:95-128 as CRS (1-based).
    Diagonals -1: -1-Pe, 0: 2, +1: -1+Pe; b(1) = 1+Pe, b(N) = 1-Pe."""
    diags = {-1: -1.0 - Pe, 0: 2.0, 1: -1.0 + Pe}
    rp, ci, vals = _toeplitz_crs(N, diags, np.float64)
    b = np.zeros(N)
    b[0] = 1.0 + Pe
    b[-1] = 1.0 - Pe
    return rp, ci, vals, b


def toeplitz_complex(N=200):
    """Complex Toeplitz of E/TOEPLITZ/toeplitz.f90:41-45 as CRS (1-based).
    Diagonals -1: 3.6i, 0: 4, 2: 1, 3: 0.7; b = i."""
    diags = {-1: 3.6j, 0: 4.0 + 0j, 2: 1.0 + 0j, 3: 0.7 + 0j}
    rp, ci, vals = _toeplitz_crs(N, diags, np.complex128)
    b = np.full(N, 1j)
    return rp, ci, vals, b


def _toeplitz_crs(N, diags, dtype):
    rows, cols, vals = [], [], []
    for i in range(N):
        for d in sorted(diags):
            j = i + d
            if 0 <= j < N:
                rows.append(i)
                cols.append(j)
                vals.append(diags[d])
    rows = np.array(rows)
    counts = np.bincount(rows, minlength=N)
    rp = np.zeros(N + 1, dtype=np.int64)
    np.cumsum(counts, out=rp[1:])
    return (rp + 1).astype(np.int32), np.array(cols, dtype=np.int32) + 1, np.array(vals, dtype=dtype)


def multishift_shifts(n, n_shifts=16, damping=0.05, lo=0.1, hi=4.0):
    """Shifts sigma_k = (2 pi f_k)^2 (1 - damping*i) with f_k evenly spaced so
    that Re(sigma_k) spans [lo, hi] * lambda_max of the 7-point Dirichlet
    Laplacian, lambda_max = (12/h^2) sin^2(n pi h / 2), h = 1/(n+1)."""
    h = 1.0 / (n + 1)
    lam_max = 12.0 / h**2 * np.sin(n * np.pi * h / 2.0) ** 2
    fmin = np.sqrt(lo * lam_max) / (2 * np.pi)
    fmax = np.sqrt(hi * lam_max) / (2 * np.pi)
    f = np.linspace(fmin, fmax, n_shifts)
    return (2 * np.pi * f) ** 2 * (1 - damping * 1j), lam_max


def complex_unit_normal(N, seed=7):
    rng = np.random.default_rng(seed)
    b = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    return b / np.linalg.norm(b)
