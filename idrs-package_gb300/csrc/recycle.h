// recycle.h -- the recycling outputs of IDRS_RITZ (ritz_module.f90:389-556):
// the omega parameters from the Ritz values and the recycle space U0 (Schur
// vectors of the Hessenberg matrix by block shift-and-invert power iteration,
// the Krylov basis rebuilt on the device from the Hessenberg recurrence, and
// a global modified Gram-Schmidt QR of the result).
#pragma once

#include <complex>
#include <cstdint>

#include "matrix.cuh"

namespace idrs {

// Seed of the SI_power start block.  The reference draws it from
// RANDOM_NUMBER; here it is uniform01(kSiPowerSeed, i + n*j).
constexpr uint64_t kSiPowerSeed = 2;

// RSI_power (dense_la_module.f90:531-603): s Schur vectors of H(1:n,1:n)
// (column-major, leading dimension ldh) nearest `shift`; vec is n x s.
// Returns 0, or 1 for bad sizes.
int si_power(const double* H, int ldh, int n, int s, double shift, uint64_t seed, double* vec);

// omega(1:n_omega) = 1/Re(QR_eig(Hf(1:n_omega,1:n_omega))) (|Re| < eps -> 1),
// ordered greedily by the largest residual-polynomial value
// (ritz_module.f90:497-520).
void ritz_omega(const double* Hf, int ldh, int n_omega, double* omega);
// complex version (CIDRS_RITZ, ritz_module.f90:335-358): omega = 1/ritz
// (|ritz| < eps -> 1), p *= 1 - ritz omega(i)
void ritz_omega(const std::complex<double>* Hf, int ldh, int n_omega, std::complex<double>* omega);

// rcompute_U0 (ritz_module.f90:100-160) on the device: rebuilds v_1 = b,
// v_{i+1} = (A v_i - sum_{l=max(1,i-s)}^{i} v_l H(l,i)) / H(i+1,i) for
// i = 1..nritz and accumulates U(:,j) = sum_i eigvec(i,j) v_i.  With resnrm
// (host, length ns) the columns are normalised and the Ritz residual norms
// returned.  H (ldh >= nritz+1) and eigvec (nritz x ns) are host arrays;
// b and U (n x ns, leading dimension n) are device arrays.  M: optional
// preconditioner (the products are A (v / M)).
template <class T>
void compute_u0(Operator& A, Operator* M, const T* H, int ldh, int nritz, const T* eigvec, int ns,
                const T* b, T* U, double* resnrm, cudaStream_t st);

// global_RQR_factorization / global_CQR_factorization (ritz_module.f90:36-96):
// modified Gram-Schmidt with global inner products, in place on the device
// matrix Q (n x s, leading dimension n).  R (host, s x s) optional.  Returns
// 0, or the 1-based index of the first dependent column.
template <class T>
int global_qr(long n, int s, T* Q, T* R, RedBuf rb, cudaStream_t st);

}  // namespace idrs
