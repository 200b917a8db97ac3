"""Python host mirror of the IDRS package's Fortran API over the C ABI.

The names, argument meanings and error behaviour follow the Fortran modules
(M/ = IDRS/MODULES of the IDRS package):

  user_module   : crs_format, coo_format, cds_format, dense_format,
                  stencil7_format (matrix-free stencil of E/STENCIL),
                  real_precon / complex_precon, real_diagonal, UserMatrix * v
  matrix_module : Matrix (type(matrix)), real_preconditioner /
                  complex_preconditioner, ms_parameters, A * v, v / A,
                  scaleback
  idrs_module   : IDRS, QMRIDR, MSIDRS, MSQMRIDR, NORM, INPROD (and IDRS_RITZ,
                  PP_IDRS)

Every call goes through libidrs_gb300.so (CUDA, sm_103a).  There is no CPU
fallback: importing this module raises if the library is missing, and a
failing C call raises IDRSError with the library's message, the equivalent
of the reference's `error stop`.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libidrs_gb300.so")

IDRS_OK, IDRS_ERR_ARG, IDRS_ERR_CUDA, IDRS_ERR_ALLOC, IDRS_ERR_STATE, IDRS_ERR_UNSUPPORTED = range(6)
POINTER_HOST, POINTER_DEVICE = 0, 1
# fp64 evaluation of the polynomial preconditioner (idrs_matrix_set_poly_eval)
POLY_HORNER, POLY_RECURRENCE = 0, 1


class IDRSError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"[status {status}] {msg}")
        self.status = status


_lib = None
_i = C.c_int
_d = C.c_double
_vp = C.c_void_p
_ip = C.POINTER(C.c_int)
_dp = C.POINTER(C.c_double)

# C prototypes (include/idrs_gb300.h)
_PROTOS = {
    "idrs_last_error": (C.c_char_p, []),
    "idrs_version": (_i, []),
    "idrs_launch_count": (C.c_long, []),
    "idrs_pp_struct_size": (C.c_long, [_i]),
    "idrs_crs_format": (_i, [_i, _i, _vp, _vp, _vp, _vp, _vp]),
    "idrs_coo_format": (_i, [_i, _i, _i, _vp, _vp, _vp, _vp, _vp]),
    "idrs_cds_format": (_i, [_i, _i, _i, _vp, _vp, _vp]),
    "idrs_dense_format": (_i, [_i, _i, _vp, _vp, _vp]),
    "idrs_mm_matrix": (_i, [C.c_char_p, C.c_char_p, _vp]),
    "idrs_mm_read": (_i, [C.c_char_p, C.c_char_p, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "idrs_stencil7_format": (_i, [_i, _i, _i, _vp, _vp]),
    "idrs_real_precon": (_i, [_i, _vp, _vp, _vp]),
    "idrs_complex_precon": (_i, [_i, _vp, _vp, _vp]),
    "idrs_real_precon_ext": (_i, [_i, _vp, _vp, _vp, _vp, _vp]),
    "idrs_complex_precon_ext": (_i, [_i, _vp, _vp, _vp, _vp, _vp]),
    "idrs_real_diagonal": (_i, [_vp, _vp]),
    "idrs_complex_diagonal": (_i, [_vp, _vp]),
    "idrs_ruser_mv": (_i, [_vp, _vp, _vp]),
    "idrs_cuser_mv": (_i, [_vp, _vp, _vp]),
    "idrs_user_matrix_free": (_i, [_vp]),
    "idrs_matrix_create": (_i, [_vp, _vp, _i, _vp, _vp]),
    "idrs_matrix_create_ext": (_i, [_vp, _vp, _vp, _vp, _i, _vp, _vp, _i, _vp]),
    "idrs_make_deflation": (_i, [_vp, _vp, _i]),
    "idrs_rpmul": (_i, [_vp, _vp, _vp]),
    "idrs_cpmul": (_i, [_vp, _vp, _vp]),
    "idrs_matrix_free": (_i, [_vp]),
    "idrs_matrix_set_stream": (_i, [_vp, _vp]),
    "idrs_matrix_set_pointer_mode": (_i, [_vp, _i]),
    "idrs_matrix_set_poly_eval": (_i, [_vp, _i]),
    "idrs_matrix_set_shadow": (_i, [_vp, _i, _vp]),
    "idrs_real_preconditioner": (_i, [_vp, _i, _i, _vp, _vp, _vp, _i, _i]),
    "idrs_complex_preconditioner": (_i, [_vp, _i, _i, _vp, _vp, _vp, _i, _i]),
    "idrs_matrix_get_alpha": (_i, [_vp, _vp, _vp]),
    "idrs_real_ms_parameters": (_i, [_vp, _i, _vp, _vp]),
    "idrs_complex_ms_parameters": (_i, [_vp, _i, _vp, _vp]),
    "idrs_rmatvec": (_i, [_vp, _vp, _vp]),
    "idrs_cmatvec": (_i, [_vp, _vp, _vp]),
    "idrs_rmatvec32": (_i, [_vp, _vp, _vp]),
    "idrs_rprecon": (_i, [_vp, _vp, _vp]),
    "idrs_cprecon": (_i, [_vp, _vp, _vp]),
    "idrs_rscaleback": (_i, [_vp, _vp, _vp, _vp]),
    "idrs_cscaleback": (_i, [_vp, _vp, _vp, _vp]),
    "idrs_ms_rscaleback": (_i, [_vp, _i, _vp, _vp, _vp, _vp]),
    "idrs_ms_cscaleback": (_i, [_vp, _i, _vp, _vp, _vp, _vp]),
    "idrs_time_matvec": (_i, [_vp, _i, _i, _i, _vp, _vp]),
    "idrs_time_matvec_graph": (_i, [_vp, _i, _i, _i, _vp]),
    "idrs_time_sparse_outer_grad": (_i, [_vp, _i, _i, _vp]),
    "idrs_ridrs": (_i, [_vp, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _vp,
                        _i, _vp, _i, _i, _vp]),
    "idrs_cidrs": (_i, [_vp, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _vp,
                        _i, _vp, _i, _i, _vp]),
    "idrs_rqmridr": (_i, [_vp, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                          _i, _vp, _i, _vp, _vp]),
    "idrs_cqmridr": (_i, [_vp, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                          _i, _vp, _i, _vp, _vp]),
    "idrs_rmsidrs": (_i, [_vp, _vp, _i, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _vp,
                          _i, _vp, _vp]),
    "idrs_cmsidrs": (_i, [_vp, _vp, _i, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _vp,
                          _i, _vp, _vp]),
    "idrs_rmsqmridr": (_i, [_vp, _vp, _i, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                            _vp, _i, _vp, _i, _vp, _vp]),
    "idrs_cmsqmridr": (_i, [_vp, _vp, _i, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                            _vp, _i, _vp, _i, _vp, _vp]),
    "idrs_solve_stats": (_i, [_vp, _vp, _vp, _vp]),
    "idrs_crs_transpose": (_i, [_vp, _vp]),
    "idrs_rsparse_outer_grad": (_i, [_vp, _vp, _vp, _vp]),
    "idrs_radjoint": (_i, [_vp, _vp, _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "idrs_rnorm": (_i, [_vp, _vp, _vp]),
    "idrs_cnorm": (_i, [_vp, _vp, _vp]),
    "idrs_rinprod": (_i, [_vp, _vp, _vp, _vp]),
    "idrs_cinprod": (_i, [_vp, _vp, _vp, _vp]),
    "idrs_rinprod_noalloc": (_i, [C.c_long, _vp, _vp, _vp, _vp]),
    "idrs_ridrs_ritz": (_i, [_vp, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _vp,
                             _i, _vp, _i, _vp, _i, _i, _vp, _vp]),
    "idrs_rpp_idrs": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "idrs_cidrs_ritz": (_i, [_vp, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _vp,
                             _i, _vp, _i, _vp, _i, _i, _vp, _vp]),
    "idrs_rpp_mr_idrs": (_i, [_vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "idrs_rpp_idrs_ext": (_i, [_vp] * 9),
    "idrs_cpp_idrs": (_i, [_vp] * 9),
    "idrs_rpp_mr_idrs_ext": (_i, [_vp, _i] + [_vp] * 8),
    "idrs_cpp_mr_idrs": (_i, [_vp, _i] + [_vp] * 8),
    "idrs_rpp_ms_idrs": (_i, [_vp, _vp, _i] + [_vp] * 9),
    "idrs_cpp_ms_idrs": (_i, [_vp, _vp, _i] + [_vp] * 9),
    "idrs_rpp_ms_mr_idrs": (_i, [_vp, _i, _vp, _i] + [_vp] * 9),
    "idrs_cpp_ms_mr_idrs": (_i, [_vp, _i, _vp, _i] + [_vp] * 9),
}


class PPOptions(C.Structure):
    _fields_ = [("method", C.c_int), ("s", C.c_int), ("tol", C.c_double), ("maxit", C.c_int),
                ("in_s", C.c_int), ("in_it", C.c_int), ("in_tol", C.c_double),
                ("preconditioner", C.c_int), ("degree", C.c_int), ("n_ritz", C.c_int),
                ("inner_precision", C.c_int), ("device_pointers", C.c_int),
                ("n_omega", C.c_int), ("recycle", C.c_int), ("poly_eval", C.c_int),
                ("fp64_check_tol", C.c_double)]


class PPReport(C.Structure):
    _fields_ = [("flag", C.c_int), ("iterations", C.c_int), ("ritz_iterations", C.c_int),
                ("nritz", C.c_int), ("relres_solver", C.c_double),
                ("relres_original", C.c_double), ("foci", C.c_double * 2), ("center", C.c_double),
                ("seconds_setup", C.c_double), ("seconds_solve", C.c_double),
                ("seconds_total", C.c_double), ("inner_solves", C.c_int),
                ("inner_iterations", C.c_int), ("inner_max", C.c_int),
                ("recycle_flag", C.c_int), ("recycle_iterations", C.c_int),
                ("recycle_relres", C.c_double), ("foci_imag", C.c_double * 2),
                ("center_imag", C.c_double), ("rel_err_vs_fp64", C.c_double),
                ("fp64_relres_original", C.c_double), ("fp64_flag", C.c_int),
                ("fp64_iterations", C.c_int), ("seconds_fp64_check", C.c_double)]


class PPInputs(C.Structure):
    """idrs_pp_inputs: M, C, seed, shift, V of pp_idrs (pointers; NULL = absent)."""
    _fields_ = [("M", C.c_void_p), ("C", C.c_void_p), ("seed", C.c_void_p),
                ("shift", C.c_void_p), ("V", C.c_void_p), ("n_deflation", C.c_int)]


def load(path: str | None = None):
    """Load libidrs_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise ImportError(f"libidrs_gb300.so not found at {path}: run "
                          "`python idrs-package_gb300/build.py` (or __graft_entry__.build())")
    lib = C.CDLL(path)
    for name, (res, args) in _PROTOS.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def lib():
    return _lib if _lib is not None else load()


def _check(status):
    if status != IDRS_OK:
        msg = lib().idrs_last_error()
        raise IDRSError(status, msg.decode() if msg else "")


def _p(a):
    if a is None:
        return None
    if isinstance(a, int):
        return a
    return a.ctypes.data


def _ref_int(v):
    return None if v is None else C.byref(C.c_int(int(v)))


def _ref_dbl(v):
    return None if v is None else C.byref(C.c_double(float(v)))


def _arr(a, cplx, n=None):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.complex128 if cplx else np.float64)
    if n is not None and a.size != n:
        raise ValueError(f"vector of length {a.size} where {n} entries are required")
    return a


class Result(dict):
    """x plus the optional outputs of the Fortran call (flag, relres, ...)."""
    __getattr__ = dict.__getitem__


# ---------------------------------------------------------------------------
# user_module
# ---------------------------------------------------------------------------
class UserMatrix:
    """type(user_matrix) (M/PP_MATRIX/user_module.f90:134-167), device resident."""

    __array_ufunc__ = None  # `v * K`, `v / K` must not broadcast element-wise

    def __init__(self, handle, nrows, ncols, cplx, nnz=None):
        self.handle, self.nrows, self.ncols, self.cplx = handle, nrows, ncols, cplx
        self.nnz = nnz

    def __del__(self):
        h = getattr(self, "handle", None)
        if h and _lib is not None:
            _lib.idrs_user_matrix_free(h)
            self.handle = None

    def __mul__(self, v):
        """K*v: ruser_mv / cuser_mv (user_module.f90:182-241)."""
        cplx = self.cplx or np.iscomplexobj(v)
        v = _arr(v, cplx, self.ncols)
        w = np.empty(self.nrows, dtype=v.dtype)
        fn = lib().idrs_cuser_mv if cplx else lib().idrs_ruser_mv
        _check(fn(self.handle, _p(v), _p(w)))
        return w


def _values(rval, cval):
    if cval is not None:
        return None, np.ascontiguousarray(cval, dtype=np.complex128)
    if rval is not None:
        rv = np.asarray(rval)
        if np.iscomplexobj(rv):
            return None, np.ascontiguousarray(rv, dtype=np.complex128)
        return np.ascontiguousarray(rv, dtype=np.float64), None
    return None, None


def crs_format(nrows, ncols, row_ptr, col_ind, rval=None, ival=None, cval=None) -> UserMatrix:
    """crs_format (user_module.f90:829-863); indices 1-based."""
    rp = np.ascontiguousarray(row_ptr, dtype=np.int32)
    ci = np.ascontiguousarray(col_ind, dtype=np.int32)
    if ival is not None and rval is None:
        rval = np.asarray(ival, dtype=np.float64)
    rv, cv = _values(rval, cval)
    h = C.c_void_p()
    _check(lib().idrs_crs_format(int(nrows), int(ncols), _p(rp), _p(ci), _p(rv), _p(cv), C.byref(h)))
    return UserMatrix(h.value, nrows, ncols, cv is not None, nnz=int(rp[nrows] - rp[0]))


def coo_format(nrows, ncols, nnz, indx, jndx, rval=None, ival=None, cval=None) -> UserMatrix:
    """coo_format (user_module.f90:865-898); indices 1-based."""
    ii = np.ascontiguousarray(indx[:nnz], dtype=np.int32)
    jj = np.ascontiguousarray(jndx[:nnz], dtype=np.int32)
    if ival is not None and rval is None:
        rval = np.asarray(ival, dtype=np.float64)
    rv, cv = _values(None if rval is None else np.asarray(rval)[:nnz],
                     None if cval is None else np.asarray(cval)[:nnz])
    h = C.c_void_p()
    _check(lib().idrs_coo_format(int(nrows), int(ncols), int(nnz), _p(ii), _p(jj), _p(rv), _p(cv),
                                 C.byref(h)))
    return UserMatrix(h.value, nrows, ncols, cv is not None)


def cds_format(nrows, ncols, half_band, rband=None, iband=None, cband=None) -> UserMatrix:
    """cds_format (user_module.f90:932-958); band shape (nrows, 2*half_band+1)."""
    if iband is not None and rband is None:
        rband = np.asarray(iband, dtype=np.float64)
    band = cband if cband is not None else rband
    rv = cv = None
    if band is not None:
        flat = np.asarray(band).reshape(nrows, 2 * half_band + 1).ravel(order="F")
        rv, cv = _values(None if np.iscomplexobj(flat) else flat, flat if np.iscomplexobj(flat) else None)
    h = C.c_void_p()
    _check(lib().idrs_cds_format(int(nrows), int(ncols), int(half_band), _p(rv), _p(cv), C.byref(h)))
    return UserMatrix(h.value, nrows, ncols, cv is not None)


def dense_format(rmat=None, imat=None, cmat=None) -> UserMatrix:
    """dense_format (user_module.f90:900-930)."""
    mat = cmat if cmat is not None else (rmat if rmat is not None else imat)
    mat = np.asarray(mat)
    flat = mat.ravel(order="F")
    rv, cv = _values(None if np.iscomplexobj(flat) else flat.astype(np.float64),
                     flat if np.iscomplexobj(flat) else None)
    h = C.c_void_p()
    _check(lib().idrs_dense_format(mat.shape[0], mat.shape[1], _p(rv), _p(cv), C.byref(h)))
    return UserMatrix(h.value, mat.shape[0], mat.shape[1], cv is not None)


def mm_read(mm_file, which_format=None) -> Result:
    """The conversion of mm_matrix (E/MATRIX_MARKET/mm_module.f90:48-154) into
    host arrays: rep ('coordinate'/'array'), field, nrows, ncols, nnz and
    row_ptr/col_ind ('crs'), indx/jndx ('coo', the default) and vals
    (array, column order, nrows x ncols).  Indices are 1-based."""
    f = os.fsencode(mm_file)
    w = None if which_format is None else which_format.encode()
    rep, field, nr, nc, nnz = C.c_int(), C.c_int(), C.c_int(), C.c_int(), C.c_long()
    _check(lib().idrs_mm_read(f, w, C.byref(rep), C.byref(field), C.byref(nr), C.byref(nc),
                              C.byref(nnz), None, None, None))
    cplx = field.value == 1
    crs = which_format is not None and which_format.lower() == "crs"
    n = nnz.value
    vals = np.zeros(n * (2 if cplx else 1))
    r = Result(rep="coordinate" if rep.value == 0 else "array",
               field=("real", "complex", "integer", "pattern")[field.value],
               nrows=nr.value, ncols=nc.value, nnz=n)
    if rep.value == 1:
        _check(lib().idrs_mm_read(f, w, None, None, None, None, None, None, None, _p(vals)))
        v = vals.view(np.complex128) if cplx else vals
        r["vals"] = v.reshape((nr.value, nc.value), order="F")
        return r
    ptr = np.zeros(nr.value + 1 if crs else n, np.int32)
    ind = np.zeros(n, np.int32)
    _check(lib().idrs_mm_read(f, w, None, None, None, None, None, _p(ptr), _p(ind), _p(vals)))
    v = vals.view(np.complex128) if cplx else vals
    if crs:
        r.update(row_ptr=ptr, col_ind=ind, vals=v)
    else:
        r.update(indx=ptr, jndx=ind, vals=v)
    return r


def mm_matrix(mm_file, which_format=None) -> UserMatrix:
    """A = mm_matrix(mm_file[, which_format]) (mm_module.f90:48-154): a COO
    (default) or CRS user_matrix for coordinate files, dense for arrays."""
    info = mm_read(mm_file, which_format)  # sizes and kind (host parse)
    h = C.c_void_p()
    w = None if which_format is None else which_format.encode()
    _check(lib().idrs_mm_matrix(os.fsencode(mm_file), w, C.byref(h)))
    return UserMatrix(h.value, info.nrows, info.ncols, info.field == "complex",
                      nnz=info.nnz if info.rep == "coordinate" else None)


def stencil7_format(nx, ny, nz, coef) -> UserMatrix:
    """Matrix-free 7-point stencil of E/STENCIL/user_module.f90 (coef c,w,e,s,n,f,b)."""
    c = np.ascontiguousarray(coef, dtype=np.float64)
    h = C.c_void_p()
    _check(lib().idrs_stencil7_format(int(nx), int(ny), int(nz), _p(c), C.byref(h)))
    n = nx * ny * nz
    return UserMatrix(h.value, n, n, False)


def real_precon(which_precon, K: UserMatrix, shift=None, M: UserMatrix | None = None,
                C_: UserMatrix | None = None) -> UserMatrix:
    """REAL_PRECON(which_precon, K[, M, C, shift]) (user_module.f90:1327-1463):
    0 none, 1 diagonal scaling, 2 dense LU, 3 band LU (of K + shift C +
    shift^2 M with a shift)."""
    h = C.c_void_p()
    _check(lib().idrs_real_precon_ext(int(which_precon), K.handle, M.handle if M else None,
                                      C_.handle if C_ else None, _ref_dbl(shift), C.byref(h)))
    return UserMatrix(h.value, K.nrows, K.ncols, False)


def complex_precon(which_precon, K: UserMatrix, shift=None, M: UserMatrix | None = None,
                   C_: UserMatrix | None = None) -> UserMatrix:
    """COMPLEX_PRECON(which_precon, K[, M, C, shift]) (user_module.f90:1465-1602)."""
    h = C.c_void_p()
    sh = None if shift is None else np.array([np.real(shift), np.imag(shift)])
    _check(lib().idrs_complex_precon_ext(int(which_precon), K.handle, M.handle if M else None,
                                         C_.handle if C_ else None, _p(sh), C.byref(h)))
    return UserMatrix(h.value, K.nrows, K.ncols, True)


def real_diagonal(K: UserMatrix):
    d = np.empty(K.nrows)
    _check(lib().idrs_real_diagonal(K.handle, _p(d)))
    return d


def complex_diagonal(K: UserMatrix):
    d = np.empty(K.nrows, dtype=np.complex128)
    _check(lib().idrs_complex_diagonal(K.handle, _p(d)))
    return d


# ---------------------------------------------------------------------------
# matrix_module
# ---------------------------------------------------------------------------
class Matrix:
    """type(matrix) (M/PP_MATRIX/matrix_module.f90:38-81): K, the mass and
    damping matrices M and C, the diagonal preconditioner P, the seed shift
    and the polynomial preconditioner.  With multishift and C the operator
    is the 2n x 2n block system (vectors of length 2n)."""

    __array_ufunc__ = None  # `v / A` must reach __rtruediv__ with the whole vector

    def __init__(self, K: UserMatrix, P: UserMatrix | None = None, seed=None, complex=False,
                 M: UserMatrix | None = None, C_: UserMatrix | None = None, multishift=False,
                 shift=None):
        self.K, self.P, self.cplx = K, P, bool(complex)
        block = bool(multishift) and C_ is not None
        self.n = 2 * K.nrows if block else K.nrows
        sd = None if seed is None else np.array([np.real(seed), np.imag(seed)], dtype=np.float64)
        sh = None if shift is None else np.array([np.real(shift), np.imag(shift)], dtype=np.float64)
        h = C.c_void_p()
        _check(lib().idrs_matrix_create_ext(K.handle, M.handle if M else None,
                                            C_.handle if C_ else None, P.handle if P else None,
                                            int(self.cplx), _p(sd), _p(sh), int(bool(multishift)),
                                            C.byref(h)))
        self.handle = h.value
        self.device_pointers = False

    def __del__(self):
        h = getattr(self, "handle", None)
        if h and _lib is not None:
            _lib.idrs_matrix_free(h)
            self.handle = None

    @property
    def dtype(self):
        return np.complex128 if self.cplx else np.float64

    def set_stream(self, stream_handle: int):
        _check(lib().idrs_matrix_set_stream(self.handle, C.c_void_p(stream_handle)))

    def set_pointer_mode(self, mode: int):
        _check(lib().idrs_matrix_set_pointer_mode(self.handle, int(mode)))
        self.device_pointers = mode == POINTER_DEVICE

    def set_poly_eval(self, mode: int):
        """POLY_HORNER (the reference's rpolpre) or POLY_RECURRENCE (the Jacobi
        three-term recurrence) for the fp64 products of this operator."""
        _check(lib().idrs_matrix_set_poly_eval(self.handle, int(mode)))

    def set_shadow(self, s, PT):
        """Inject the shadow space P (s x n, rows contiguous) for solves with this s."""
        pt = None if PT is None else np.ascontiguousarray(PT, dtype=self.dtype)
        _check(lib().idrs_matrix_set_shadow(self.handle, int(s), _p(pt)))

    def preconditioner(self, preconditioner=0, degree=0, foci=None, center=None, H=None):
        """real_preconditioner / complex_preconditioner (matrix_module.f90:551-722)."""
        dt = self.dtype
        f = None if foci is None else np.ascontiguousarray(foci, dtype=dt)
        c = None if center is None else np.array([center], dtype=dt)
        Hf = None if H is None else np.asfortranarray(H, dtype=dt)
        ldh, nh = (0, 0) if Hf is None else Hf.shape
        fn = lib().idrs_complex_preconditioner if self.cplx else lib().idrs_real_preconditioner
        _check(fn(self.handle, int(preconditioner), int(degree), _p(f), _p(c), _p(Hf), ldh, nh))

    real_preconditioner = preconditioner
    complex_preconditioner = preconditioner

    @property
    def alpha_p(self):
        deg = C.c_int()
        _check(lib().idrs_matrix_get_alpha(self.handle, None, C.byref(deg)))
        a = np.empty(deg.value + 1, dtype=self.dtype)
        _check(lib().idrs_matrix_get_alpha(self.handle, _p(a), None))
        return a

    def time_matvec(self, prec=64, warmup=3, reps=20):
        """CUDA-event time of one product A*v (ms) and of one SpMV launch (ms)."""
        a, b = C.c_double(), C.c_double()
        _check(lib().idrs_time_matvec(self.handle, int(prec), int(warmup), int(reps), C.byref(a),
                                      C.byref(b)))
        return a.value, b.value

    def time_matvec_graph(self, prec=64, warmup=3, reps=20):
        """CUDA-event time (ms) of one product A*v captured as a CUDA graph and
        replayed, as the IDR(s) cycles run their products."""
        a = C.c_double()
        _check(lib().idrs_time_matvec_graph(self.handle, int(prec), int(warmup), int(reps), C.byref(a)))
        return a.value

    def ms_parameters(self, sigma):
        sigma = np.ascontiguousarray(sigma, dtype=self.dtype)
        sp = np.empty_like(sigma)
        fn = lib().idrs_complex_ms_parameters if self.cplx else lib().idrs_real_ms_parameters
        _check(fn(self.handle, len(sigma), _p(sigma), _p(sp)))
        return sp

    def make_deflation(self, V):
        """make_deflation(A, V) (matrix_module.f90:1284-1346): V is n x k (k <= 16);
        None or k = 0 removes the deflation."""
        if V is None:
            _check(lib().idrs_make_deflation(self.handle, None, 0))
            return
        V = np.asfortranarray(V, dtype=self.dtype)
        if V.ndim != 2 or V.shape[0] != self.n:
            raise ValueError("V must be n x k")
        _check(lib().idrs_make_deflation(self.handle, _p(V), V.shape[1]))

    def pmul(self, v):
        """w = Pmul(A, v) (matrix_module.f90:1348-1418)."""
        v = _arr(v, self.cplx, self.n)
        w = np.empty_like(v)
        fn = lib().idrs_cpmul if self.cplx else lib().idrs_rpmul
        _check(fn(self.handle, _p(v), _p(w)))
        return w

    def matvec32(self, v):
        """A*v evaluated in fp32 (the operator of the fp32 inner solves), widened to fp64."""
        if self.cplx:
            raise IDRSError(IDRS_ERR_UNSUPPORTED, "matvec32: real matrices only")
        v = _arr(v, False, self.n)
        w = np.empty_like(v)
        _check(lib().idrs_rmatvec32(self.handle, _p(v), _p(w)))
        return w

    def __mul__(self, v):
        """A*v: rmatvec / cmatvec (matrix_module.f90:135-167)."""
        v = _arr(v, self.cplx, self.n)
        w = np.empty_like(v)
        fn = lib().idrs_cmatvec if self.cplx else lib().idrs_rmatvec
        _check(fn(self.handle, _p(v), _p(w)))
        return w

    def __rtruediv__(self, v):
        """v/A: rprecon / cprecon (matrix_module.f90:306-400)."""
        v = _arr(v, self.cplx, self.n)
        w = np.empty_like(v)
        fn = lib().idrs_cprecon if self.cplx else lib().idrs_rprecon
        _check(fn(self.handle, _p(v), _p(w)))
        return w

    def scaleback(self, b, y):
        """scaleback(A, b, y) (matrix_module.f90:811-849)."""
        y = _arr(y, self.cplx, self.n)
        b = _arr(b, self.cplx, self.n)
        x = np.empty_like(y)
        fn = lib().idrs_cscaleback if self.cplx else lib().idrs_rscaleback
        _check(fn(self.handle, _p(b), _p(y), _p(x)))
        return x

    def ms_scaleback(self, sigma, b, Y):
        """scaleback(A, sigma, b, y) (matrix_module.f90:724-809); Y is n x n_sigma."""
        Y = np.asfortranarray(Y, dtype=self.dtype)
        if Y.ndim != 2 or Y.shape[0] != self.n:
            raise ValueError("Y must be n x n_sigma")
        X = np.empty_like(Y, order="F")
        sg = np.ascontiguousarray(sigma, dtype=self.dtype)
        b = _arr(b, self.cplx)
        fn = lib().idrs_ms_cscaleback if self.cplx else lib().idrs_ms_rscaleback
        _check(fn(self.handle, Y.shape[1], _p(sg), _p(b), _p(Y), _p(X)))
        return X


# ---------------------------------------------------------------------------
# idrs_module
# ---------------------------------------------------------------------------
def _solver_common(A: Matrix, b):
    if A.device_pointers:
        raise ValueError("the numpy mirror works in host-pointer mode")
    return _arr(b, A.cplx, A.n)


def IDRS(A: Matrix, b, s, M1: Matrix | None = None, tolerance=None, maximum_iterations=None,
         variant=None, x0=None, U0=None, omega=None, resvec=False, H=None) -> Result:
    """x = IDRS(A, b, s, ...) (RIDRS/CIDRS, idrs_module.f90:107-251).

    resvec=True returns the residual history (maxit+1 entries); H=nritz
    returns the (nritz+1) x nritz Hessenberg matrix."""
    b = _solver_common(A, b)
    n = len(b)
    maxit = maximum_iterations if maximum_iterations is not None else min(2 * n, 1000)
    x = np.empty_like(b)
    flag, relres, iters = C.c_int(), C.c_double(), C.c_int()
    x0a = _arr(x0, A.cplx, n)
    U0a = None if U0 is None else np.asfortranarray(U0, dtype=A.dtype)
    if U0a is not None and U0a.shape != (n, s):
        raise ValueError("U0 must be n x s")
    om = _arr(omega, A.cplx)
    rv = np.zeros(maxit + 1) if resvec else None
    Hm = np.zeros((H + 1, H), dtype=A.dtype, order="F") if H else None
    fn = lib().idrs_cidrs if A.cplx else lib().idrs_ridrs
    _check(fn(A.handle, _p(b), int(s), M1.handle if M1 else None, _ref_dbl(tolerance),
              _ref_int(maximum_iterations), _ref_int(variant), C.byref(flag), C.byref(relres),
              C.byref(iters), _p(x0a), _p(U0a), _p(om), 0 if om is None else len(om), _p(rv),
              0 if rv is None else len(rv), _p(Hm), 0 if Hm is None else H + 1, H or 0, _p(x)))
    r = Result(x=x, flag=flag.value, relres=relres.value, iterations=iters.value)
    if rv is not None:
        r["resvec"] = rv
    if Hm is not None:
        r["H"] = Hm
    return r


def _rel_err(x, xr):
    """||x - xr|| / ||xr|| (per column of a multishift x)."""
    return np.linalg.norm(x - xr, axis=0) / np.linalg.norm(xr, axis=0)


def _is_mixed(inner_iterations, inner_precision):
    return bool(inner_iterations) and inner_iterations > 0 and inner_precision == 32


def _check_maxit(maxit, n):
    """Iteration bound of the FP64 check solve: a mixed call's bound counts
    outer iterations, so the check gets at least min(2n, 5000)."""
    return max(maxit or 0, min(2 * n, 5000))


def QMRIDR(A: Matrix, b, s, M1: Matrix | None = None, tolerance=None, maximum_iterations=None,
           inner_s=None, inner_tolerance=None, inner_iterations=None, x0=None, omega=None,
           resvec=False, inner_precision=None, fp64_check=None) -> Result:
    """x = QMRIDR(A, b, s, ...) (RQMRIDR/CQMRIDR, idrs_module.f90:253-408).
    inner_precision=32 runs the inner IDR(inner_s) in fp32 / complex64.

    fp64_check (see fp64_check_tolerance; by default on for the mixed form)
    adds rel_err_vs_fp64 = ||x - x64|| / ||x64||, x64 the FP64 QMRIDR(s)
    solution of the same system (no inner solves) at the check's tolerance,
    with its fp64_flag and fp64_iterations."""
    b = _solver_common(A, b)
    n = len(b)
    maxit = maximum_iterations if maximum_iterations is not None else min(2 * n, 1000)
    x = np.empty_like(b)
    flag, relres, iters = C.c_int(), C.c_double(), C.c_int()
    x0a = _arr(x0, A.cplx, n)
    om = _arr(omega, A.cplx)
    rv = np.zeros(maxit + 1) if resvec else None
    fn = lib().idrs_cqmridr if A.cplx else lib().idrs_rqmridr
    _check(fn(A.handle, _p(b), int(s), M1.handle if M1 else None, _ref_dbl(tolerance),
              _ref_int(maximum_iterations), C.byref(flag), C.byref(relres), C.byref(iters),
              _ref_int(inner_s), _ref_dbl(inner_tolerance), _ref_int(inner_iterations), _p(x0a),
              _p(om), 0 if om is None else len(om), _p(rv), 0 if rv is None else len(rv),
              _ref_int(inner_precision), _p(x)))
    r = Result(x=x, flag=flag.value, relres=relres.value, iterations=iters.value)
    if rv is not None:
        r["resvec"] = rv
    tc = fp64_check_tolerance(1e-6 if tolerance is None else tolerance, fp64_check,
                              _is_mixed(inner_iterations, inner_precision))
    if tc > 0:
        q = QMRIDR(A, b, s, M1=M1, tolerance=tc, maximum_iterations=_check_maxit(maximum_iterations, n),
                   omega=omega, inner_iterations=0, fp64_check=False)
        r.update(rel_err_vs_fp64=float(_rel_err(x, q.x)), fp64_flag=q.flag, fp64_iterations=q.iterations)
    return r


def _shift_masks(r: Result, tolerance):
    """Per-shift status of a multishift result (no counterpart in the
    reference, which reports one flag for all shifts and, like gfortran's
    maxval, lets a NaN residual pass the flag test): converged_mask[k] is
    relres[k] <= tol, nonfinite_mask[k] marks a shift whose residual or
    solution holds a NaN or an infinity (a breakdown of that shift)."""
    tol = 1e-6 if tolerance is None else float(tolerance)
    rel = np.asarray(r.relres, dtype=float)
    fin = np.isfinite(rel) & np.all(np.isfinite(r.x), axis=0)
    r["nonfinite_mask"] = ~fin
    r["converged_mask"] = fin & (rel <= tol)
    return r


def _shifts(A: Matrix, sigma):
    sig = np.ascontiguousarray(np.atleast_1d(sigma), dtype=np.complex128 if A.cplx else np.float64)
    if sig.ndim != 1 or len(sig) < 1:
        raise IDRSError(IDRS_ERR_ARG, "sigma must be a non-empty vector of shifts")
    return sig


def MSIDRS(A: Matrix, b, sigma, s, M1: Matrix | None = None, tolerance=None,
           maximum_iterations=None, variant=None, omega=None, resvec=False,
           colfac=False) -> Result:
    """x(:, k) = MSIDRS(A, b, sigma, s, ...) (RMSIDRS/CMSIDRS, idrs_module.f90:572-713):
    (A - sigma_k I) x_k = b for every shift; relres has one entry per shift."""
    b = _solver_common(A, b)
    n = len(b)
    sig = _shifts(A, sigma)
    ns = len(sig)
    maxit = maximum_iterations if maximum_iterations is not None else min(2 * n, 1000)
    x = np.empty((n, ns), dtype=b.dtype, order="F")
    flag, iters = C.c_int(), C.c_int()
    relres = np.ones(ns)
    om = _arr(omega, A.cplx)
    rv = np.zeros((maxit + 1, ns), order="F") if resvec else None
    cf = np.empty(ns, dtype=b.dtype) if colfac else None
    fn = lib().idrs_cmsidrs if A.cplx else lib().idrs_rmsidrs
    _check(fn(A.handle, _p(b), ns, _p(sig), int(s), M1.handle if M1 else None,
              _ref_dbl(tolerance), _ref_int(maximum_iterations), _ref_int(variant),
              C.byref(flag), _p(relres), C.byref(iters), _p(om), 0 if om is None else len(om),
              _p(rv), 0 if rv is None else maxit + 1, _p(cf), _p(x)))
    r = Result(x=x, flag=flag.value, relres=relres, iterations=iters.value)
    if rv is not None:
        r["resvec"] = rv
    if cf is not None:
        r["colfac"] = cf
    return _shift_masks(r, tolerance)


def MSQMRIDR(A: Matrix, b, sigma, s, M1: Matrix | None = None, tolerance=None,
             maximum_iterations=None, inner_s=None, inner_tolerance=None,
             inner_iterations=None, omega=None, resvec=False, inner_precision=None,
             fp64_check=None) -> Result:
    """x(:, k) = MSQMRIDR(A, b, sigma, s, ...) (RMSQMRIDR/CMSQMRIDR,
    idrs_module.f90:410-570).  inner_precision=32 runs the inner MSIDRS in
    fp32 / complex64.  fp64_check as in QMRIDR: rel_err_vs_fp64 per shift
    against the FP64 MSQMRIDR(s) solutions (no inner solves)."""
    b = _solver_common(A, b)
    n = len(b)
    sig = _shifts(A, sigma)
    ns = len(sig)
    maxit = maximum_iterations if maximum_iterations is not None else min(2 * n, 1000)
    x = np.empty((n, ns), dtype=b.dtype, order="F")
    flag, iters = C.c_int(), C.c_int()
    relres = np.ones(ns)
    om = _arr(omega, A.cplx)
    rv = np.zeros((maxit + 1, ns), order="F") if resvec else None
    fn = lib().idrs_cmsqmridr if A.cplx else lib().idrs_rmsqmridr
    _check(fn(A.handle, _p(b), ns, _p(sig), int(s), M1.handle if M1 else None,
              _ref_dbl(tolerance), _ref_int(maximum_iterations), C.byref(flag), _p(relres),
              C.byref(iters), _ref_int(inner_s), _ref_dbl(inner_tolerance),
              _ref_int(inner_iterations), _p(om), 0 if om is None else len(om), _p(rv),
              0 if rv is None else maxit + 1, _ref_int(inner_precision), _p(x)))
    r = Result(x=x, flag=flag.value, relres=relres, iterations=iters.value)
    if rv is not None:
        r["resvec"] = rv
    tc = fp64_check_tolerance(1e-6 if tolerance is None else tolerance, fp64_check,
                              _is_mixed(inner_iterations, inner_precision))
    if tc > 0:
        q = MSQMRIDR(A, b, sig, s, M1=M1, tolerance=tc, maximum_iterations=_check_maxit(maximum_iterations, n),
                     omega=omega, inner_iterations=0, fp64_check=False)
        r.update(rel_err_vs_fp64=_rel_err(x, q.x), fp64_flag=q.flag, fp64_iterations=q.iterations)
    return _shift_masks(r, tolerance)


# ------------------------------------------------------------------ adjoint
def crs_transpose(K: UserMatrix) -> UserMatrix:
    """K^T as a CRS user_matrix built on the device (no reference counterpart)."""
    h = C.c_void_p()
    _check(lib().idrs_crs_transpose(K.handle, C.byref(h)))
    return UserMatrix(h.value, K.ncols, K.nrows, K.cplx, nnz=K.nnz)


def sparse_outer_grad(A: Matrix, lam, x):
    """grad[p] = -lam_i x_j over the stored entries of A's CRS matrix, in storage order."""
    if A.K.nnz is None:
        raise IDRSError(IDRS_ERR_ARG, "sparse_outer_grad: CRS matrix required")
    lam = _arr(lam, False, A.n)
    x = _arr(x, False, A.n)
    g = np.empty(A.K.nnz)
    _check(lib().idrs_rsparse_outer_grad(A.handle, _p(lam), _p(x), _p(g)))
    return g


def ADJOINT(AT: Matrix, K: UserMatrix, x, g, s, tolerance=None, maximum_iterations=None,
            grad=True) -> Result:
    """Backward step of A x = b for a scalar loss with dL/dx = g: IDR(s) on the
    adjoint operator AT (from crs_transpose(K)) gives lambda = dL/db; grad is
    dL/dK over K's stored entries, -lambda_i x_j."""
    if K.nnz is None:
        raise IDRSError(IDRS_ERR_ARG, "ADJOINT: K must be a CRS user_matrix")
    x = _arr(x, False, AT.n)
    g = _arr(g, False, AT.n)
    lam = np.empty(AT.n)
    gr = np.empty(K.nnz) if grad else None
    flag, relres, iters = C.c_int(), C.c_double(), C.c_int()
    _check(lib().idrs_radjoint(AT.handle, K.handle, _p(x), _p(g), int(s), _ref_dbl(tolerance),
                               _ref_int(maximum_iterations), C.byref(flag), C.byref(relres),
                               C.byref(iters), _p(lam), _p(gr)))
    r = Result(lam=lam, flag=flag.value, relres=relres.value, iterations=iters.value)
    if gr is not None:
        r["grad"] = gr
    return r


def NORM(A: Matrix, w) -> float:
    w = _arr(w, A.cplx, A.n)
    out = np.zeros(1)
    fn = lib().idrs_cnorm if A.cplx else lib().idrs_rnorm
    _check(fn(A.handle, _p(w), _p(out)))
    return float(out[0])


def INPROD(A: Matrix, u, v):
    u = _arr(u, A.cplx, A.n)
    v = _arr(v, A.cplx, A.n)
    out = np.zeros(2)
    fn = lib().idrs_cinprod if A.cplx else lib().idrs_rinprod
    _check(fn(A.handle, _p(u), _p(v), _p(out)))
    return complex(out[0], out[1]) if A.cplx else float(out[0])


def IDRS_RITZ(A: Matrix, b, s, M: Matrix | None = None, tolerance=None, maximum_iterations=None,
              variant=None, x0=None, n_omega=0, dimU0=0, resvec=False, H_shape=None) -> Result:
    """x = IDRS_RITZ(A, b, s[, M, tolerance, maximum_iterations, variant, flag, relres,
    iterations, x0, U0, omega, resvec, H]) (ritz_module.f90:389-556).

    The reference's optional outputs are requested by size: n_omega (omega),
    dimU0 (the recycle space U0, n x dimU0), H_shape (H) and resvec."""
    b = _solver_common(A, b)
    x = np.empty_like(b)
    dt = A.dtype
    flag, relres, iters, nritz = C.c_int(), C.c_double(), C.c_int(), C.c_int()
    Hm = np.zeros(H_shape, dtype=dt, order="F") if H_shape else None
    om = np.zeros(n_omega, dtype=dt) if n_omega else None
    U0 = np.zeros((A.n, dimU0), dtype=dt, order="F") if dimU0 else None
    maxit = maximum_iterations if maximum_iterations is not None else min(2 * A.n, 1000)
    rv = np.zeros(maxit + 1) if resvec else None
    fn = lib().idrs_cidrs_ritz if A.cplx else lib().idrs_ridrs_ritz
    _check(fn(A.handle, _p(b), int(s), M.handle if M else None,
              _ref_dbl(tolerance), _ref_int(maximum_iterations),
              _ref_int(variant), C.byref(flag), C.byref(relres), C.byref(iters),
              _p(_arr(x0, A.cplx, A.n)), _p(U0), int(dimU0), _p(om), int(n_omega),
              _p(rv), 0 if rv is None else len(rv), _p(Hm),
              0 if Hm is None else H_shape[0], 0 if Hm is None else H_shape[1],
              C.byref(nritz), _p(x)))
    r = Result(x=x, flag=flag.value, relres=relres.value, iterations=iters.value, nritz=nritz.value)
    for key, val in (("H", Hm), ("omega", om), ("U0", U0), ("resvec", rv)):
        if val is not None:
            r[key] = val
    return r


def fp64_check_tolerance(tol, fp64_check, mixed, dev=False):
    """The tolerance of the FP64 solve that a result's relative error is
    measured against (0.0: no check).  fp64_check: None (default) checks every
    mixed-precision result (fp32 / complex64 inner solves) of a call with host
    arrays; True checks any result; False none; a float is the tolerance
    itself.  The default tolerance is tol * 1e-3 (at least 1e-14), tight
    enough that the FP64 solution's own error is small beside the 10 tol
    that a mixed result may differ from it."""
    if fp64_check is None:
        fp64_check = bool(mixed) and not dev
    if fp64_check is False:
        return 0.0
    if fp64_check is True:
        return max(float(tol) * 1e-3, 1e-14)
    t = float(fp64_check)
    if not t > 0.0:
        raise IDRSError(IDRS_ERR_ARG, "fp64_check must be None, a bool or a positive tolerance")
    return t


def _pp_options(method, s, tol, maxit, in_s, in_it, in_tol, preconditioner, degree, n_ritz,
                inner_precision, dev, n_omega, recycle, poly_eval=POLY_HORNER, fp64_check=False):
    mixed = method == 0 and in_it > 0 and inner_precision == 32
    return PPOptions(method, s, tol, maxit, in_s, in_it, in_tol, preconditioner, degree, n_ritz,
                     inner_precision, int(dev), int(n_omega), int(bool(recycle)), int(poly_eval),
                     fp64_check_tolerance(tol, fp64_check, mixed, dev))


def _pp_result(rep: PPReport, **extra) -> Result:
    foci = tuple(complex(rep.foci[q], rep.foci_imag[q]) if rep.foci_imag[q] else rep.foci[q]
                 for q in range(2))
    center = complex(rep.center, rep.center_imag) if rep.center_imag else rep.center
    return Result(flag=rep.flag, iterations=rep.iterations,
                  ritz_iterations=rep.ritz_iterations, nritz=rep.nritz,
                  relres=rep.relres_solver, relres_original=rep.relres_original,
                  foci=foci, center=center, seconds_setup=rep.seconds_setup,
                  seconds_solve=rep.seconds_solve, seconds_total=rep.seconds_total,
                  inner_solves=rep.inner_solves, inner_iterations=rep.inner_iterations,
                  inner_max=rep.inner_max, recycle_flag=rep.recycle_flag,
                  recycle_iterations=rep.recycle_iterations, recycle_relres=rep.recycle_relres,
                  **_fp64_fields(rep), **extra)


def _fp64_fields(rep: PPReport) -> dict:
    """rel_err_vs_fp64 (None without a check) and the FP64 solve's record."""
    if rep.fp64_flag < 0:
        return dict(rel_err_vs_fp64=None)
    return dict(rel_err_vs_fp64=rep.rel_err_vs_fp64, fp64_flag=rep.fp64_flag,
                fp64_iterations=rep.fp64_iterations, fp64_relres_original=rep.fp64_relres_original,
                seconds_fp64_check=rep.seconds_fp64_check)


def _pp_kind(K, b, M, C_, seed, shift, complex_):
    if complex_ is not None:
        return bool(complex_)
    return bool(K.cplx or (M is not None and M.cplx) or (C_ is not None and C_.cplx)
                or np.iscomplexobj(b) or np.iscomplexobj(seed) or np.iscomplexobj(shift))


def _pp_inputs(cplx, M, C_, seed, shift, V, keep):
    """idrs_pp_inputs (or None when every optional input is absent)."""
    if M is None and C_ is None and seed is None and shift is None and V is None:
        return None
    inp = PPInputs()
    inp.M = M.handle if M else None
    inp.C = C_.handle if C_ else None
    for name, v in (("seed", seed), ("shift", shift)):
        if v is not None:
            a = np.array([np.real(v), np.imag(v)], dtype=np.float64)
            keep.append(a)
            setattr(inp, name, a.ctypes.data)
    if V is not None:
        Va = np.asfortranarray(V, dtype=np.complex128 if cplx else np.float64)
        keep.append(Va)
        inp.V = Va.ctypes.data
        inp.n_deflation = Va.shape[1]
    keep.append(inp)
    return C.byref(inp)


def _pp_cf(cplx, center, foci):
    """center / foci in the pipeline's kind (complex: re/im pairs)."""
    dt = np.complex128 if cplx else np.float64
    c = None if center is None else np.asarray([center], dtype=dt)
    f = None if foci is None else np.ascontiguousarray(foci, dtype=dt)
    return c, f


def PP_IDRS(K: UserMatrix, b, P: UserMatrix | None = None, center=None, foci=None, *, method=1,
            s=4, tol=1e-6, maxit=1000, in_s=1, in_it=0, in_tol=0.1, preconditioner=0, degree=0,
            n_ritz=32, inner_precision=64, n_omega=0, M=None, C_=None, seed=None, shift=None,
            V=None, complex=None, x_out=None, poly_eval=0, fp64_check=None) -> Result:
    """x = pp_idrs(K, b[, M, C, P, center, foci, seed, shift, V]) (RPP_IDRS / CPP_IDRS,
    pp_idrs_module.f90:64-162); the command-line options of initialize.inc:4-31
    are keyword arguments.

    b may be a numpy array (host) or an int device address; with a device b,
    x_out must be the device address of the solution vector.  With a host b,
    x_out may be a contiguous numpy array of b's length and kind (for
    example pinned memory) that receives the solution.

    fp64_check (see fp64_check_tolerance; by default on for mixed-precision
    solves with host arrays) adds rel_err_vs_fp64 = ||x - x64|| / ||x64||
    against an FP64 solve of the same system, with that solve's fp64_flag,
    fp64_iterations and fp64_relres_original."""
    dev = isinstance(b, int)
    cplx = _pp_kind(K, None if dev else b, M, C_, seed, shift, complex)
    if dev:
        if not isinstance(x_out, int):
            raise ValueError("a device b needs a device x_out")
        x = x_out
    else:
        b = _arr(b, cplx, K.nrows)
        if x_out is None:
            x = np.empty_like(b)
        elif (isinstance(x_out, np.ndarray) and x_out.dtype == b.dtype and x_out.shape == b.shape
              and x_out.flags.c_contiguous and x_out.flags.writeable):
            x = x_out
        else:
            raise ValueError("x_out must be a writeable contiguous array of b's length and kind")
    o = _pp_options(method, s, tol, maxit, in_s, in_it, in_tol, preconditioner, degree, n_ritz,
                    inner_precision, dev, n_omega, False, poly_eval, fp64_check)
    rep = PPReport()
    keep = []
    c, f = _pp_cf(cplx, center, foci)
    inp = _pp_inputs(cplx, M, C_, seed, shift, V, keep)
    fn = lib().idrs_cpp_idrs if cplx else lib().idrs_rpp_idrs_ext
    _check(fn(K.handle, _p(b), P.handle if P else None, _p(c), _p(f), inp, C.byref(o), C.byref(rep),
              _p(x)))
    return _pp_result(rep, x=None if dev else x)


def PP_MR_IDRS(K: UserMatrix, b_all, P: UserMatrix | None = None, center=None, foci=None, *,
               method=1, s=4, tol=1e-6, maxit=1000, in_s=1, in_it=0, in_tol=0.1,
               preconditioner=0, degree=0, n_ritz=32, inner_precision=64, n_omega=0,
               recycle=False, M=None, C_=None, seed=None, shift=None, V=None, complex=None,
               nrhs=None, x_out=None, poly_eval=0, fp64_check=None) -> Result:
    """x_all = pp_idrs(K, b_all[, M, C, P, center, foci, seed, shift, V]) for a sequence
    of right-hand sides (RPP_MR_IDRS / CPP_MR_IDRS, pp_idrs_module.f90:164-279,
    recycle.inc, run_mr_idrs.inc).

    b_all: n x nrhs numpy array, or the int device address of a column-major
    n x nrhs array (then nrhs and the device address x_out are required).
    Returns x (n x nrhs, host case) and per right-hand side arrays flags,
    iterations, relres, relres_original, seconds_solve (and rel_err_vs_fp64
    with fp64_check, as in PP_IDRS)."""
    dev = isinstance(b_all, int)
    n = K.nrows
    cplx = _pp_kind(K, None if dev else b_all, M, C_, seed, shift, complex)
    dt = np.complex128 if cplx else np.float64
    if dev:
        if not isinstance(x_out, int) or not nrhs:
            raise ValueError("a device b_all needs nrhs and a device x_out")
        x = x_out
    else:
        b_all = np.asfortranarray(b_all, dtype=dt)
        if b_all.ndim != 2 or b_all.shape[0] != n:
            raise ValueError("b_all must be n x nrhs")
        nrhs = b_all.shape[1]
        x = np.zeros((n, nrhs), dtype=dt, order="F")
    o = _pp_options(method, s, tol, maxit, in_s, in_it, in_tol, preconditioner, degree, n_ritz,
                    inner_precision, dev, n_omega, recycle, poly_eval, fp64_check)
    reps = (PPReport * nrhs)()
    keep = []
    c, f = _pp_cf(cplx, center, foci)
    inp = _pp_inputs(cplx, M, C_, seed, shift, V, keep)
    fn = lib().idrs_cpp_mr_idrs if cplx else lib().idrs_rpp_mr_idrs_ext
    _check(fn(K.handle, int(nrhs), _p(b_all), P.handle if P else None, _p(c), _p(f), inp,
              C.byref(o), reps, _p(x)))
    r = _pp_result(reps[nrhs - 1], x=None if dev else x)
    r["flags"] = np.array([q.flag for q in reps])
    r["iterations"] = np.array([q.iterations for q in reps])
    r["relres"] = np.array([q.relres_solver for q in reps])
    r["relres_original"] = np.array([q.relres_original for q in reps])
    r["seconds_solve"] = np.array([q.seconds_solve for q in reps])
    if o.fp64_check_tol > 0:
        r["rel_err_vs_fp64"] = np.array([q.rel_err_vs_fp64 for q in reps])
        r["fp64_flags"] = np.array([q.fp64_flag for q in reps])
    return r


def PP_MS_IDRS(K: UserMatrix, rhs, sigma, P: UserMatrix | None = None, center=None, foci=None, *,
               method=1, s=4, tol=1e-6, maxit=1000, in_s=1, in_it=0, in_tol=0.1,
               preconditioner=0, degree=0, n_ritz=32, inner_precision=64, n_omega=0, M=None,
               C_=None, seed=None, shift=None, V=None, complex=None, fp64_check=None) -> Result:
    """x(n, n_sigma) = pp_idrs(K, rhs, sigma[, M, C, P, center, foci, seed, shift, V])
    (RPP_MS_IDRS / CPP_MS_IDRS with run_ms_idrs.inc).  With C the block system
    is solved and x is the second half of each solution.  relres_sigma: the
    true residual of every shifted system.  A 2-D rhs (n x nrhs) runs the
    sequence form RPP_MS_MR_IDRS / CPP_MS_MR_IDRS: x is n x n_sigma x nrhs,
    relres_sigma n_sigma x nrhs, flags and iterations per right-hand side.
    fp64_check as in PP_IDRS: rel_err_vs_fp64 per shift (and right-hand side)
    against the same pipeline in FP64 without inner solves."""
    r = _pp_ms_idrs(K, rhs, sigma, P, center, foci, method, s, tol, maxit, in_s, in_it, in_tol,
                    preconditioner, degree, n_ritz, inner_precision, n_omega, M, C_, seed, shift,
                    V, complex)
    tc = fp64_check_tolerance(tol, fp64_check, method == 0 and _is_mixed(in_it, inner_precision))
    if tc > 0:
        q = _pp_ms_idrs(K, rhs, sigma, P, center, foci, method, s, tc, _check_maxit(maxit, K.nrows),
                        in_s, 0, in_tol, preconditioner, degree, n_ritz, 64, n_omega, M, C_, seed,
                        shift, V, complex)
        r.update(rel_err_vs_fp64=_rel_err(r.x, q.x), fp64_flag=q.flag, fp64_iterations=q.iterations)
    return r


def _pp_ms_idrs(K, rhs, sigma, P, center, foci, method, s, tol, maxit, in_s, in_it, in_tol,
                preconditioner, degree, n_ritz, inner_precision, n_omega, M, C_, seed, shift, V,
                complex):
    cplx = _pp_kind(K, rhs, M, C_, seed, shift, complex) or np.iscomplexobj(sigma)
    dt = np.complex128 if cplx else np.float64
    seq = np.ndim(rhs) == 2
    rhs = np.asfortranarray(rhs, dtype=dt) if seq else _arr(rhs, cplx, K.nrows)
    if rhs.shape[0] != K.nrows:
        raise ValueError("rhs must have K.nrows rows")
    nrhs = rhs.shape[1] if seq else 1
    sig = np.ascontiguousarray(sigma, dtype=dt)
    ns = len(sig)
    x = np.zeros((K.nrows, ns, nrhs), dtype=dt, order="F")
    rel = np.zeros((ns, nrhs), order="F")
    o = _pp_options(method, s, tol, maxit, in_s, in_it, in_tol, preconditioner, degree, n_ritz,
                    inner_precision, False, n_omega, False)
    keep = []
    c, f = _pp_cf(cplx, center, foci)
    inp = _pp_inputs(cplx, M, C_, seed, shift, V, keep)
    if seq:
        reps = (PPReport * nrhs)()
        fn = lib().idrs_cpp_ms_mr_idrs if cplx else lib().idrs_rpp_ms_mr_idrs
        _check(fn(K.handle, int(nrhs), _p(rhs), ns, _p(sig), P.handle if P else None, _p(c), _p(f),
                  inp, C.byref(o), reps, _p(rel), _p(x)))
        r = _pp_result(reps[nrhs - 1], x=x, relres_sigma=rel)
        r["flags"] = np.array([q.flag for q in reps])
        r["iterations"] = np.array([q.iterations for q in reps])
        return r
    rep = PPReport()
    fn = lib().idrs_cpp_ms_idrs if cplx else lib().idrs_rpp_ms_idrs
    _check(fn(K.handle, _p(rhs), ns, _p(sig), P.handle if P else None, _p(c), _p(f), inp,
              C.byref(o), C.byref(rep), _p(rel), _p(x)))
    return _pp_result(rep, x=x[:, :, 0], relres_sigma=rel[:, 0])
