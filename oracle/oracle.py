"""ctypes wrapper of the oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY.  The oracle is the CPU restatement of the IDRS
package's solve path that the CUDA library is checked against; see oracle.h
for its parity status.  Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg import this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

c_int_p = C.POINTER(C.c_int)
c_dbl_p = C.POINTER(C.c_double)


class Opts(C.Structure):
    _fields_ = [
        ("tolerance", c_dbl_p),
        ("maximum_iterations", c_int_p),
        ("variant", c_int_p),
        ("M1", C.c_void_p),
        ("inner_s", c_int_p),
        ("inner_tolerance", c_dbl_p),
        ("inner_iterations", c_int_p),
        ("x0", C.c_void_p),
        ("U0", C.c_void_p),
        ("omega", C.c_void_p),
        ("n_omega", C.c_int),
        ("PT", C.c_void_p),
        ("flag", c_int_p),
        ("relres", c_dbl_p),
        ("iterations", c_int_p),
        ("resvec", c_dbl_p),
        ("resvec_len", C.c_int),
        ("H", C.c_void_p),
        ("H_rows", C.c_int),
        ("H_cols", C.c_int),
        ("colfac", C.c_void_p),
        ("p_seed", C.c_uint64),
        ("skip_inner_true_residual", C.c_int),
        ("inner_round32", C.c_int),
    ]


class PPArgs(C.Structure):
    _fields_ = [
        ("method", C.c_int), ("s", C.c_int), ("maxit", C.c_int), ("in_s", C.c_int),
        ("in_it", C.c_int), ("preconditioner", C.c_int), ("degree", C.c_int),
        ("n_ritz", C.c_int),
        ("tol", C.c_double), ("in_tol", C.c_double),
        ("foci", c_dbl_p), ("center", c_dbl_p),
        ("p_seed", C.c_uint64),
        ("flag", C.c_int), ("iterations", C.c_int), ("ritz_iterations", C.c_int),
        ("nritz_used", C.c_int),
        ("relres_solver", C.c_double), ("relres_original", C.c_double),
        ("foci_used", C.c_double * 2), ("center_used", C.c_double),
        ("alpha_p", C.c_double * 64),
        ("seconds_setup", C.c_double), ("seconds_solve", C.c_double),
        ("n_omega", C.c_int), ("recycle", C.c_int),
        ("si_seed", C.c_uint64),
        ("omega_used", C.c_double * 64),
        ("recycle_flag", C.c_int), ("recycle_iterations", C.c_int),
        ("recycle_relres", C.c_double),
        ("flags", c_int_p), ("iters", c_int_p),
        ("relres_solver_all", c_dbl_p), ("relres_original_all", c_dbl_p),
        ("poly_eval", C.c_int),
    ]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc + OpenMP)."""
    if force or not os.path.exists(_LIB_PATH) or _stale():
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def _stale() -> bool:
    t = os.path.getmtime(_LIB_PATH)
    for f in ("oracle.c", "oracle_core.inc", "oracle.h", "Makefile"):
        if os.path.getmtime(os.path.join(_HERE, f)) > t:
            return True
    return False


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(_LIB_PATH)
        _lib.or_uniform.restype = C.c_double
        _lib.or_uniform.argtypes = [C.c_uint64, C.c_uint64]
        for name in ("or_norm_r", "or_norm_c"):
            getattr(_lib, name).restype = C.c_double
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _ip(v):
    return None if v is None else C.pointer(C.c_int(int(v)))


def _dp(v):
    return None if v is None else C.pointer(C.c_double(float(v)))


def set_threads(n: int) -> None:
    lib().or_set_threads(int(n))


def get_threads() -> int:
    return int(lib().or_get_threads())


def uniform(seed: int, index: int) -> float:
    return float(lib().or_uniform(seed, index))


# --------------------------------------------------------------------------
# user matrices
# --------------------------------------------------------------------------
class UserMatrix:
    """Owning handle of an oracle user_matrix."""

    def __init__(self, ptr, n, keep=()):
        self.ptr = ptr
        self.n = n
        self._keep = keep

    def __del__(self):
        if getattr(self, "ptr", None) and _lib is not None:
            _lib.or_umat_free(self.ptr)
            self.ptr = None

    def mv(self, v):
        v = np.ascontiguousarray(v)
        w = np.empty(self.n, dtype=v.dtype)
        fn = lib().or_user_mv_c if np.iscomplexobj(v) else lib().or_user_mv_r
        fn(self.ptr, _p(v), _p(w))
        return w


def _vals(values):
    if values is None:
        return None, None
    values = np.ascontiguousarray(values)
    if np.iscomplexobj(values):
        return None, values.astype(np.complex128)
    return values.astype(np.float64), None


def crs_format(nrows, ncols, row_ptr1, col_ind1, values=None) -> UserMatrix:
    rp = np.ascontiguousarray(row_ptr1, dtype=np.int32)
    ci = np.ascontiguousarray(col_ind1, dtype=np.int32)
    rv, cv = _vals(values)
    out = C.c_void_p()
    st = lib().or_crs_format(int(nrows), int(ncols), _p(rp), _p(ci), _p(rv), _p(cv), C.byref(out))
    if st:
        raise ValueError(f"or_crs_format status {st}")
    return UserMatrix(out, nrows)


def coo_format(nrows, ncols, indx1, jndx1, values=None) -> UserMatrix:
    ii = np.ascontiguousarray(indx1, dtype=np.int32)
    jj = np.ascontiguousarray(jndx1, dtype=np.int32)
    rv, cv = _vals(values)
    out = C.c_void_p()
    st = lib().or_coo_format(int(nrows), int(ncols), len(ii), _p(ii), _p(jj), _p(rv), _p(cv),
                             C.byref(out))
    if st:
        raise ValueError(f"or_coo_format status {st}")
    return UserMatrix(out, nrows)


def cds_format(nrows, ncols, half_band, band) -> UserMatrix:
    rv, cv = _vals(np.asfortranarray(band).ravel(order="F"))
    out = C.c_void_p()
    st = lib().or_cds_format(int(nrows), int(ncols), int(half_band), _p(rv), _p(cv), C.byref(out))
    if st:
        raise ValueError(f"or_cds_format status {st}")
    return UserMatrix(out, nrows)


def dense_format(mat) -> UserMatrix:
    mat = np.asarray(mat)
    rv, cv = _vals(mat.ravel(order="F"))
    out = C.c_void_p()
    st = lib().or_dense_format(mat.shape[0], mat.shape[1], _p(rv), _p(cv), C.byref(out))
    if st:
        raise ValueError(f"or_dense_format status {st}")
    return UserMatrix(out, mat.shape[0])


def stencil7_format(nx, ny, nz, coef) -> UserMatrix:
    c = np.ascontiguousarray(coef, dtype=np.float64)
    out = C.c_void_p()
    st = lib().or_stencil7_format(int(nx), int(ny), int(nz), _p(c), C.byref(out))
    if st:
        raise ValueError(f"or_stencil7_format status {st}")
    return UserMatrix(out, nx * ny * nz, keep=(c,))


def complex_precon(which, K: UserMatrix, shift=None, M: UserMatrix | None = None,
                   C_: UserMatrix | None = None) -> UserMatrix:
    out = C.c_void_p()
    sh = None if shift is None else np.array([np.real(shift), np.imag(shift)])
    st = lib().or_complex_precon_ext(int(which), K.ptr, M.ptr if M else None,
                                     C_.ptr if C_ else None, _p(sh), C.byref(out))
    if st:
        raise ValueError(f"or_complex_precon status {st}")
    return UserMatrix(out, K.n)


def real_precon(which, K: UserMatrix, shift=None, M: UserMatrix | None = None,
                C_: UserMatrix | None = None) -> UserMatrix:
    out = C.c_void_p()
    st = lib().or_real_precon_ext(int(which), K.ptr, M.ptr if M else None, C_.ptr if C_ else None,
                                  _dp(shift), C.byref(out))
    if st:
        raise ValueError(f"or_real_precon status {st}")
    return UserMatrix(out, K.n)


def real_diagonal(K: UserMatrix):
    d = np.empty(K.n)
    lib().or_real_diagonal(K.ptr, _p(d))
    return d


# --------------------------------------------------------------------------
# type(matrix)
# --------------------------------------------------------------------------
class Matrix:
    def __init__(self, K: UserMatrix, P: UserMatrix | None = None, seed=None, cplx=False,
                 M: UserMatrix | None = None, C_: UserMatrix | None = None, multishift=False,
                 shift=None):
        self.K, self.P, self.cplx = K, P, cplx
        self.M, self.C = M, C_  # keep the user matrices alive
        block = bool(multishift) and C_ is not None
        self.n = 2 * K.n if block else K.n
        sd = None
        if seed is not None:
            sd = np.array([np.real(seed), np.imag(seed)], dtype=np.float64)
        sh = None
        if shift is not None:
            sh = np.array([np.real(shift), np.imag(shift)], dtype=np.float64)
        out = C.c_void_p()
        st = lib().or_matrix_create_ext(K.ptr, M.ptr if M else None, C_.ptr if C_ else None,
                                        P.ptr if P else None, _p(sd), _p(sh), int(cplx),
                                        int(bool(multishift)), C.byref(out))
        if st:
            raise ValueError(f"or_matrix_create status {st}")
        self.ptr = out

    def __del__(self):
        if getattr(self, "ptr", None) and _lib is not None:
            _lib.or_matrix_free(self.ptr)
            self.ptr = None

    def preconditioner(self, preconditioner, degree, foci=None, center=None, H=None):
        if self.cplx:
            f = None if foci is None else np.ascontiguousarray(foci, dtype=np.complex128)
            c = None if center is None else np.array([center], dtype=np.complex128)
            Hf = None if H is None else np.asfortranarray(H, dtype=np.complex128)
            fn = lib().or_complex_preconditioner
        else:
            f = None if foci is None else np.ascontiguousarray(foci, dtype=np.float64)
            c = None if center is None else np.array([center], dtype=np.float64)
            Hf = None if H is None else np.asfortranarray(H, dtype=np.float64)
            fn = lib().or_real_preconditioner
        ldh = 0 if Hf is None else Hf.shape[0]
        nh = 0 if Hf is None else Hf.shape[1]
        st = fn(self.ptr, int(preconditioner), int(degree), _p(f), _p(c), _p(Hf), ldh, nh)
        if st:
            raise ValueError(f"preconditioner status {st}")

    def set_poly_eval(self, mode):
        """0: Horner (the reference's rpolpre), 1: the Jacobi three-term recurrence."""
        st = lib().or_matrix_set_poly_eval(self.ptr, int(mode))
        if st:
            raise ValueError(f"set_poly_eval status {st}")

    def ms_parameters(self, sigma):
        sigma = np.ascontiguousarray(sigma, dtype=np.complex128 if self.cplx else np.float64)
        sp = np.empty_like(sigma)
        fn = lib().or_complex_ms_parameters if self.cplx else lib().or_real_ms_parameters
        fn(self.ptr, len(sigma), _p(sigma), _p(sp))
        return sp

    def matvec(self, v):
        v = np.ascontiguousarray(v, dtype=np.complex128 if self.cplx else np.float64)
        w = np.empty_like(v)
        fn = lib().or_matvec_c if self.cplx else lib().or_matvec_r
        fn(self.ptr, len(v), _p(v), _p(w))
        return w

    def precon(self, v):
        v = np.ascontiguousarray(v, dtype=np.complex128 if self.cplx else np.float64)
        w = np.empty_like(v)
        fn = lib().or_precon_c if self.cplx else lib().or_precon_r
        fn(self.ptr, len(v), _p(v), _p(w))
        return w

    def scaleback(self, b, y):
        y = np.ascontiguousarray(y, dtype=np.complex128 if self.cplx else np.float64)
        b = np.ascontiguousarray(b, dtype=y.dtype)
        x = np.empty_like(y)
        fn = lib().or_scaleback_c if self.cplx else lib().or_scaleback_r
        fn(self.ptr, len(y), _p(b), _p(y), _p(x))
        return x

    def ms_scaleback(self, Y, b=None):
        dt = np.complex128 if self.cplx else np.float64
        Y = np.asfortranarray(Y, dtype=dt)
        X = np.empty_like(Y, order="F")
        bb = None if b is None else np.ascontiguousarray(b, dtype=dt)
        fn = lib().or_ms_scaleback_b_c if self.cplx else lib().or_ms_scaleback_b_r
        fn(self.ptr, Y.shape[0], Y.shape[1], _p(bb), _p(Y), _p(X))
        return X

    def make_deflation(self, V):
        """make_deflation(A, V) (matrix_module.f90:1284-1346); V is n x k."""
        V = np.asfortranarray(V, dtype=np.complex128 if self.cplx else np.float64)
        self._V = V
        fn = lib().or_make_deflation_c if self.cplx else lib().or_make_deflation_r
        st = fn(self.ptr, V.shape[0], _p(V), V.shape[1])
        if st:
            raise ValueError(f"or_make_deflation status {st}")

    def pmul(self, v):
        v = np.ascontiguousarray(v, dtype=np.complex128 if self.cplx else np.float64)
        w = np.empty_like(v)
        fn = lib().or_pmul_c if self.cplx else lib().or_pmul_r
        fn(self.ptr, len(v), _p(v), _p(w))
        return w


# --------------------------------------------------------------------------
# solvers
# --------------------------------------------------------------------------
class Result(dict):
    __getattr__ = dict.__getitem__


def _opts(n, dt, *, tolerance=None, maximum_iterations=None, variant=None, M1=None,
          inner_s=None, inner_tolerance=None, inner_iterations=None, x0=None, U0=None,
          omega=None, PT=None, resvec_len=None, n_sigma=1, H_shape=None, colfac_len=None,
          p_seed=1, inner_round32=False):
    keep = []
    o = Opts()
    o.tolerance = _dp(tolerance)
    o.maximum_iterations = _ip(maximum_iterations)
    o.variant = _ip(variant)
    o.M1 = M1.ptr if M1 is not None else None
    o.inner_s = _ip(inner_s)
    o.inner_tolerance = _dp(inner_tolerance)
    o.inner_iterations = _ip(inner_iterations)
    for name, arr in (("x0", x0), ("U0", U0), ("omega", omega), ("PT", PT)):
        if arr is not None:
            a = np.asfortranarray(arr, dtype=dt) if name == "U0" else np.ascontiguousarray(arr, dtype=dt)
            keep.append(a)
            setattr(o, name, _p(a))
            if name == "omega":
                o.n_omega = a.size
    flag, relres, iters = C.c_int(-99), (C.c_double * n_sigma)(), C.c_int(-1)
    o.flag = C.pointer(flag)
    o.relres = C.cast(relres, c_dbl_p)
    o.iterations = C.pointer(iters)
    resvec = None
    if resvec_len:
        resvec = np.zeros((resvec_len, n_sigma), order="F")
        o.resvec = resvec.ctypes.data_as(c_dbl_p)
        o.resvec_len = resvec_len
    H = None
    if H_shape:
        H = np.zeros(H_shape, dtype=dt, order="F")
        o.H = _p(H)
        o.H_rows, o.H_cols = H_shape
    colfac = None
    if colfac_len:
        colfac = np.zeros(colfac_len, dtype=dt)
        o.colfac = _p(colfac)
    o.p_seed = p_seed
    o.inner_round32 = int(bool(inner_round32))  # MSQMRIDR probe: nested results rounded to fp32
    return o, keep, (flag, relres, iters, resvec, H, colfac)


def _result(x, outs, n_sigma=1):
    flag, relres, iters, resvec, H, colfac = outs
    r = Result(x=x, flag=flag.value, iterations=iters.value,
               relres=relres[0] if n_sigma == 1 else np.array(relres[:]))
    if resvec is not None:
        r["resvec"] = resvec[:, 0] if n_sigma == 1 else resvec
    if H is not None:
        r["H"] = H
    if colfac is not None:
        r["colfac"] = colfac
    return r


def idrs(A: Matrix, b, s, **kw):
    dt = np.complex128 if A.cplx else np.float64
    b = np.ascontiguousarray(b, dtype=dt)
    o, keep, outs = _opts(len(b), dt, **kw)
    x = np.empty_like(b)
    fn = lib().or_idrs_c if A.cplx else lib().or_idrs_r
    st = fn(A.ptr, len(b), _p(b), int(s), C.byref(o), _p(x))
    if st:
        raise ValueError(f"or_idrs status {st}")
    return _result(x, outs)


def qmridr(A: Matrix, b, s, **kw):
    dt = np.complex128 if A.cplx else np.float64
    b = np.ascontiguousarray(b, dtype=dt)
    o, keep, outs = _opts(len(b), dt, **kw)
    x = np.empty_like(b)
    fn = lib().or_qmridr_c if A.cplx else lib().or_qmridr_r
    st = fn(A.ptr, len(b), _p(b), int(s), C.byref(o), _p(x))
    if st:
        raise ValueError(f"or_qmridr status {st}")
    return _result(x, outs)


def msidrs(A: Matrix, b, sigma, s, **kw):
    dt = np.complex128 if A.cplx else np.float64
    b = np.ascontiguousarray(b, dtype=dt)
    sigma = np.ascontiguousarray(sigma, dtype=dt)
    kw.setdefault("colfac_len", None)
    o, keep, outs = _opts(len(b), dt, n_sigma=len(sigma), **kw)
    x = np.empty((len(b), len(sigma)), dtype=dt, order="F")
    fn = lib().or_msidrs_c if A.cplx else lib().or_msidrs_r
    st = fn(A.ptr, len(b), _p(b), len(sigma), _p(sigma), int(s), C.byref(o), _p(x))
    if st:
        raise ValueError(f"or_msidrs status {st}")
    return _result(x, outs, n_sigma=len(sigma))


def msqmridr(A: Matrix, b, sigma, s, **kw):
    dt = np.complex128 if A.cplx else np.float64
    b = np.ascontiguousarray(b, dtype=dt)
    sigma = np.ascontiguousarray(sigma, dtype=dt)
    o, keep, outs = _opts(len(b), dt, n_sigma=len(sigma), **kw)
    x = np.empty((len(b), len(sigma)), dtype=dt, order="F")
    fn = lib().or_msqmridr_c if A.cplx else lib().or_msqmridr_r
    st = fn(A.ptr, len(b), _p(b), len(sigma), _p(sigma), int(s), C.byref(o), _p(x))
    if st:
        raise ValueError(f"or_msqmridr status {st}")
    return _result(x, outs, n_sigma=len(sigma))


def make_p(s, n, method=1, seed=1, r=None, cplx=False):
    dt = np.complex128 if cplx else np.float64
    rows = s if method == 1 else 1
    PT = np.empty((rows, n), dtype=dt)
    rr = np.ascontiguousarray(r if r is not None else np.zeros(n), dtype=dt)
    fn = lib().or_make_p_c if cplx else lib().or_make_p_r
    fn(int(s), int(n), int(method), C.c_uint64(seed), _p(rr), _p(PT))
    return PT


def norm(w):
    w = np.ascontiguousarray(w)
    if np.iscomplexobj(w):
        return float(lib().or_norm_c(len(w), _p(w.astype(np.complex128))))
    return float(lib().or_norm_r(len(w), _p(w.astype(np.float64))))


# --------------------------------------------------------------------------
# dense LA and polynomial helpers
# --------------------------------------------------------------------------
def qr_eig(H):
    H = np.asfortranarray(H)
    n = H.shape[1]
    eig = np.empty(n, dtype=np.complex128)
    conv = C.c_int(0)
    if np.iscomplexobj(H):
        lib().or_cqr_eig(_p(H.astype(np.complex128, order="F")), H.shape[0], n, _p(eig), C.byref(conv))
    else:
        lib().or_rqr_eig(_p(H.astype(np.float64, order="F")), H.shape[0], n, _p(eig), C.byref(conv))
    return eig, conv.value


def solve(A, b):
    A = np.asfortranarray(A)
    b = np.ascontiguousarray(b)
    if np.iscomplexobj(A) or np.iscomplexobj(b):
        A = A.astype(np.complex128, order="F"); b = b.astype(np.complex128)
        x = np.empty_like(b)
        lib().or_csolve(len(b), _p(A), _p(b), _p(x))
    else:
        A = A.astype(np.float64, order="F"); b = b.astype(np.float64)
        x = np.empty_like(b)
        lib().or_rsolve(len(b), _p(A), _p(b), _p(x))
    return x


class _Cplx(C.Structure):
    """By-value C99 double _Complex (same calling convention as two doubles)."""
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


def grot(a, b):
    if np.iscomplexobj(a) or np.iscomplexobj(b):
        c, s, r = (np.zeros(1, np.complex128) for _ in range(3))
        f = lib().or_cgrot
        f.argtypes = [_Cplx, _Cplx, C.c_void_p, C.c_void_p, C.c_void_p]
        f(_Cplx(np.real(a), np.imag(a)), _Cplx(np.real(b), np.imag(b)), _p(c), _p(s), _p(r))
        return c[0], s[0], r[0]
    c, s, r = C.c_double(), C.c_double(), C.c_double()
    lib().or_rgrot(C.c_double(a), C.c_double(b), C.byref(c), C.byref(s), C.byref(r))
    return c.value, s.value, r.value


def chebyshev(degree, foci):
    if np.iscomplexobj(foci):
        a = np.empty(degree + 1, np.complex128)
        lib().or_cchebyshev(int(degree), _p(np.ascontiguousarray(foci, np.complex128)), _p(a))
    else:
        a = np.empty(degree + 1)
        lib().or_rchebyshev(int(degree), _p(np.ascontiguousarray(foci, np.float64)), _p(a))
    return a


def neumann(degree, center):
    if np.iscomplexobj(center):
        a = np.empty(degree + 1, np.complex128)
        f = lib().or_cneumann
        f.argtypes = [C.c_int, _Cplx, C.c_void_p]
        f(int(degree), _Cplx(np.real(center), np.imag(center)), _p(a))
    else:
        a = np.empty(degree + 1)
        lib().or_rneumann(int(degree), C.c_double(center), _p(a))
    return a


def analyse_spectrum(H):
    H = np.asfortranarray(H, dtype=np.float64)
    f = np.empty(2); c = C.c_double(); sh = C.c_double()
    lib().or_ranalyse_spectrum(_p(H), H.shape[0], H.shape[1], _p(f), C.byref(c), C.byref(sh))
    return f, c.value, sh.value


def _pp_args(method, s, tol, maxit, in_s, in_tol, in_it, preconditioner, degree, n_ritz, foci,
             center, p_seed, n_omega=0, recycle=False, si_seed=0, poly_eval=0):
    a = PPArgs()
    a.method, a.s, a.maxit, a.in_s, a.in_it = method, s, maxit, in_s, in_it
    a.preconditioner, a.degree, a.n_ritz = preconditioner, degree, n_ritz
    a.tol, a.in_tol = tol, in_tol
    keep = []
    if foci is not None:
        f = (C.c_double * 2)(*foci); keep.append(f); a.foci = C.cast(f, c_dbl_p)
    if center is not None:
        c = C.c_double(center); keep.append(c); a.center = C.pointer(c)
    a.p_seed = p_seed
    a.n_omega, a.recycle, a.si_seed = int(n_omega), int(bool(recycle)), int(si_seed)
    a.poly_eval = int(poly_eval)
    return a, keep


def _pp_common(a, degree):
    return dict(ritz_iterations=a.ritz_iterations, nritz=a.nritz_used,
                foci=tuple(a.foci_used), center=a.center_used,
                alpha_p=np.array(a.alpha_p[: degree + 1]),
                omega=np.array(a.omega_used[: a.n_omega]),
                seconds_setup=a.seconds_setup, seconds_solve=a.seconds_solve)


def pp_idrs(K: UserMatrix, b, *, P: UserMatrix | None = None, method=1, s=4, tol=1e-6, maxit=1000,
            in_s=4, in_tol=0.1, in_it=0, preconditioner=0, degree=0, n_ritz=32, foci=None,
            center=None, p_seed=1, n_omega=0, poly_eval=0):
    a, keep = _pp_args(method, s, tol, maxit, in_s, in_tol, in_it, preconditioner, degree, n_ritz,
                       foci, center, p_seed, n_omega, poly_eval=poly_eval)
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.empty_like(b)
    st = lib().or_pp_idrs_r(K.ptr, P.ptr if P else None, len(b), _p(b), C.byref(a), _p(x))
    if st:
        raise ValueError(f"or_pp_idrs status {st}")
    return Result(x=x, flag=a.flag, iterations=a.iterations, relres=a.relres_solver,
                  relres_original=a.relres_original, **_pp_common(a, degree))


def pp_mr_idrs(K: UserMatrix, b_all, *, P: UserMatrix | None = None, method=1, s=4, tol=1e-6,
               maxit=1000, in_s=4, in_tol=0.1, in_it=0, preconditioner=0, degree=0, n_ritz=32,
               foci=None, center=None, p_seed=1, n_omega=0, recycle=False, si_seed=0):
    """PP_MR_IDRS (pp_idrs_module.f90:222-279): b_all is n x nrhs."""
    a, keep = _pp_args(method, s, tol, maxit, in_s, in_tol, in_it, preconditioner, degree, n_ritz,
                       foci, center, p_seed, n_omega, recycle, si_seed)
    b_all = np.asfortranarray(b_all, dtype=np.float64)
    n, nrhs = b_all.shape
    x_all = np.zeros((n, nrhs), order="F")
    flags, iters = np.zeros(nrhs, np.int32), np.zeros(nrhs, np.int32)
    rel, relo = np.zeros(nrhs), np.zeros(nrhs)
    a.flags, a.iters = flags.ctypes.data_as(c_int_p), iters.ctypes.data_as(c_int_p)
    a.relres_solver_all, a.relres_original_all = rel.ctypes.data_as(c_dbl_p), relo.ctypes.data_as(c_dbl_p)
    st = lib().or_pp_mr_idrs_r(K.ptr, P.ptr if P else None, n, nrhs, _p(b_all), C.byref(a), _p(x_all))
    if st:
        raise ValueError(f"or_pp_mr_idrs status {st}")
    return Result(x=x_all, flags=flags, iterations=iters, relres=rel, relres_original=relo,
                  recycle_flag=a.recycle_flag, recycle_iterations=a.recycle_iterations,
                  recycle_relres=a.recycle_relres, **_pp_common(a, degree))


def idrs_ritz(A: Matrix, b, s, *, n_omega=0, dimU0=0, si_seed=0, H_shape=None, **kw):
    """IDRS_RITZ (ritz_module.f90:268-556, real or complex) with its H, omega and U0 outputs."""
    dt = np.complex128 if A.cplx else np.float64
    b = np.ascontiguousarray(b, dtype=dt)
    o, keep, outs = _opts(len(b), dt, H_shape=H_shape, **kw)
    x = np.empty_like(b)
    nritz = C.c_int(0)
    om = np.zeros(max(n_omega, 1), dtype=dt)
    U0 = np.zeros((len(b), max(dimU0, 1)), dtype=dt, order="F")
    if A.cplx:
        st = lib().or_idrs_ritz_cx(A.ptr, len(b), _p(b), int(s), C.byref(o), _p(x), C.byref(nritz),
                                   _p(om) if n_omega else None, int(n_omega),
                                   _p(U0) if dimU0 else None, int(dimU0))
    else:
        st = lib().or_idrs_ritz_rx(A.ptr, len(b), _p(b), int(s), C.byref(o), _p(x), C.byref(nritz),
                                   _p(om) if n_omega else None, int(n_omega),
                                   _p(U0) if dimU0 else None, int(dimU0), C.c_uint64(si_seed))
    if st:
        raise ValueError(f"or_idrs_ritz status {st}")
    r = _result(x, outs)
    r["nritz"] = nritz.value
    if n_omega:
        r["omega"] = om
    if dimU0:
        r["U0"] = U0
    return r


def si_power(H, s, shift=0.0, seed=2):
    """RSI_power (dense_la_module.f90:531-603); H is n x n."""
    H = np.asfortranarray(H, dtype=np.float64)
    n = H.shape[1]
    vec = np.zeros((n, s), order="F")
    st = lib().or_rsi_power(_p(H), H.shape[0], n, int(s), C.c_double(shift), C.c_uint64(seed), _p(vec))
    if st:
        raise ValueError(f"or_rsi_power status {st}")
    return vec


def global_qr(V):
    V = np.asfortranarray(V, dtype=np.float64)
    n, s = V.shape
    Q = np.zeros((n, s), order="F")
    R = np.zeros((s, s), order="F")
    st = lib().or_rglobal_qr(n, s, _p(V), _p(Q), _p(R))
    if st:
        raise ValueError("V has dependent columns")
    return Q, R


def ritz_omega(H, n_omega):
    H = np.asfortranarray(H, dtype=np.float64)
    om = np.zeros(n_omega)
    lib().or_ritz_omega(_p(H), H.shape[0], int(n_omega), _p(om))
    return om


def crs_transpose(K: UserMatrix) -> UserMatrix:
    out = C.c_void_p()
    st = lib().or_crs_transpose(K.ptr, C.byref(out))
    if st:
        raise ValueError(f"or_crs_transpose status {st}")
    return UserMatrix(out, K.n)


def sparse_outer_grad(K: UserMatrix, lam, x, nnz):
    g = np.empty(nnz)
    lib().or_sparse_outer_grad(K.ptr, _p(np.ascontiguousarray(lam, np.float64)),
                               _p(np.ascontiguousarray(x, np.float64)), _p(g))
    return g
