"""Gradient-check harness: a torch.autograd.Function over the C ABI.

forward  : x = A(vals)^-1 b with IDR(s) (idrs_ridrs) for a fixed CRS pattern;
backward : lambda from IDR(s) on A^T (idrs_crs_transpose + idrs_radjoint),
           dL/db = lambda and dL/dvals = -lambda_i x_j over the pattern.

It exists to check the adjoint path against finite differences and
torch.autograd.gradcheck; tensors pass through host memory, so it is not a
training API.  Every call goes to libidrs_gb300.so (no CPU fallback).
"""
from __future__ import annotations

import numpy as np
import torch

from . import api


class CRSSolve(torch.autograd.Function):
    """x = A^-1 b, A in CRS with 1-based row_ptr / col_ind and values `vals`."""

    @staticmethod
    def forward(ctx, vals, b, row_ptr, col_ind, s=4, tol=1e-12, maxit=None):
        n = len(row_ptr) - 1
        v = vals.detach().to("cpu", torch.float64).numpy()
        bb = b.detach().to("cpu", torch.float64).numpy()
        K = api.crs_format(n, n, row_ptr, col_ind, rval=v)
        r = api.IDRS(api.Matrix(K), bb, s, tolerance=tol, maximum_iterations=maxit)
        if r.flag != 0:
            raise api.IDRSError(api.IDRS_ERR_STATE, f"forward solve ended with flag {r.flag}")
        ctx.K, ctx.x, ctx.s, ctx.tol, ctx.maxit = K, r.x, s, tol, maxit
        return torch.from_numpy(r.x.copy()).to(b.device)

    @staticmethod
    def backward(ctx, grad_x):
        KT = api.crs_transpose(ctx.K)
        AT = api.Matrix(KT)
        g = grad_x.detach().to("cpu", torch.float64).numpy()
        r = api.ADJOINT(AT, ctx.K, ctx.x, g, ctx.s, tolerance=ctx.tol, maximum_iterations=ctx.maxit)
        if r.flag != 0:
            raise api.IDRSError(api.IDRS_ERR_STATE, f"adjoint solve ended with flag {r.flag}")
        dev = grad_x.device
        return (torch.from_numpy(r.grad).to(dev), torch.from_numpy(r.lam).to(dev),
                None, None, None, None, None)


def crs_solve(vals, b, row_ptr, col_ind, s=4, tol=1e-12, maxit=None):
    return CRSSolve.apply(vals, b, np.asarray(row_ptr, np.int32), np.asarray(col_ind, np.int32), s,
                          tol, maxit)
