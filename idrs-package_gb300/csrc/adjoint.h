// adjoint.h -- the backward path of a solve A x = b with a CRS matrix A:
// the transposed CRS (for the adjoint solve A^T lambda = dL/dx) and the sparse
// outer-product gradient dL/dA_ij = -lambda_i x_j over A's nonzero pattern.
#pragma once

#include "matrix.cuh"

namespace idrs {

// K^T in CRS on the device.  Stable: row j of K^T lists the entries of column
// j of K in increasing row order (duplicates keep their order), so the result
// is the same on every run and equals a serial counting-sort transpose.
// T must be empty; on an exception T holds no device memory.
void crs_transpose(const UserMatrix& K, UserMatrix& T, cudaStream_t st);

// grad[p] = -lambda[i] * x[col[p]] for every stored entry p = (i, col[p]) of
// the CRS matrix K (real values).
void sparse_outer_grad(const UserMatrix& K, const double* lambda, const double* x, double* grad,
                       cudaStream_t st);

}  // namespace idrs
