"""Generates the golden fixtures of tests/golden from independent implementations.

The IDRS reference (Fortran 2018) cannot be compiled here and commits no
outputs, so the oracle is pinned against independent restatements of the
same mathematics:
  * bicgstab_*.npz  -- scipy.sparse.linalg.bicgstab residual norms after each
                       full BiCGSTAB step on the reference's two Toeplitz test
                       problems (E/TOEPLITZ/toeplitz.f90:20-177).  IDRS
                       variant 2 is mathematically BiCGSTAB
                       (idrs_module.f90:13-15), so its resvec at the end of
                       every omega step must follow these numbers.
  * poly.npz        -- Chebyshev and Neumann residual polynomials evaluated
                       with numpy.polynomial (closed forms), for checking the
                       coefficients of matrix_module.f90:851-1019.
  * dense.npz       -- numpy eigenvalues / linear solves for QR_eig and SOLVE.
Run:  python tests/golden/make_golden.py   (needs scipy; writes the .npz files)
"""
import os
import sys

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "idrs-package_gb300"))
import problems as P  # noqa: E402


def _csr(rp, ci, vals, n):
    return sp.csr_matrix((vals, np.asarray(ci) - 1, np.asarray(rp) - 1), shape=(n, n))


def bicgstab_history(A, b, maxiter):
    hist = []
    nb = np.linalg.norm(b)

    def cb(xk):
        hist.append(np.linalg.norm(b - A @ xk))

    spla.bicgstab(A, b, x0=np.zeros_like(b), rtol=1e-300, atol=0.0, maxiter=maxiter, callback=cb)
    return np.array(hist), nb


def main():
    rp, ci, vals, b = P.toeplitz_real()
    A = _csr(rp, ci, vals, 60)
    h, nb = bicgstab_history(A, b, 40)
    np.savez(os.path.join(HERE, "bicgstab_toeplitz_real.npz"), resnorm=h, normb=nb)
    rp, ci, vals, b = P.toeplitz_complex()
    A = _csr(rp, ci, vals, 200)
    h, nb = bicgstab_history(A, b, 40)
    np.savez(os.path.join(HERE, "bicgstab_toeplitz_complex.npz"), resnorm=h, normb=nb)

    # residual polynomials r(t) = 1 - t p(t)
    t = np.linspace(0.05, 2.0, 41)
    foci = np.array([0.3, 1.9])
    theta, delta = foci.mean(), (foci[1] - foci[0]) / 2
    cheb = {}
    for d in (1, 2, 4, 8, 12):
        Tk = np.polynomial.chebyshev.Chebyshev.basis(d + 1)
        cheb[f"cheb_{d}"] = Tk((theta - t) / delta) / Tk(theta / delta)
    center = 1.1
    neu = {f"neu_{d}": (1 - t / center) ** (d + 1) for d in (1, 3, 6)}
    np.savez(os.path.join(HERE, "poly.npz"), t=t, foci=foci, center=center, **cheb, **neu)

    rng = np.random.default_rng(11)
    H = np.triu(rng.standard_normal((12, 12)), -1) + np.diag(np.arange(1, 13) * 1.0)
    Hs = H + H.T * 0.0
    eig = np.linalg.eigvals(Hs)
    M = rng.standard_normal((8, 8))
    rhs = rng.standard_normal(8)
    Mc = M + 1j * rng.standard_normal((8, 8))
    rhsc = rhs + 1j * rng.standard_normal(8)
    np.savez(os.path.join(HERE, "dense.npz"), H=Hs, eig=eig, M=M, rhs=rhs, x=np.linalg.solve(M, rhs),
             Mc=Mc, rhsc=rhsc, xc=np.linalg.solve(Mc, rhsc))


if __name__ == "__main__":
    main()
