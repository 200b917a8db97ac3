"""idrs_gb300 -- GB300-native (sm_103a) implementation of the IDRS package's solve path.

The CUDA library (csrc/, built into _build/libidrs_gb300.so by build.py)
exports the C ABI of include/idrs_gb300.h; `api` mirrors the Fortran API on
top of it with ctypes, and `problems` generates the synthetic workloads.
This directory is loaded as the package `idrs_gb300` (its own name is not a
Python identifier).
"""
from . import build as build_recipe  # noqa: F401
from . import problems  # noqa: F401
from .api import (  # noqa: F401
    ADJOINT, IDRS, IDRS_RITZ, INPROD, MSIDRS, MSQMRIDR, NORM, PP_IDRS, PP_MR_IDRS, PP_MS_IDRS, QMRIDR,
    IDRSError,
    Matrix,
    POINTER_DEVICE, crs_transpose, sparse_outer_grad, mm_matrix, mm_read,
    POINTER_HOST, POLY_HORNER, POLY_RECURRENCE, Result, UserMatrix, cds_format, complex_diagonal, complex_precon, coo_format,
    crs_format, dense_format, lib, load, real_diagonal, real_precon, stencil7_format,
)
