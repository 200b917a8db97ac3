// setup.h -- host set-up arithmetic of the polynomial preconditioners.
#pragma once
#include <complex>
#include <vector>

namespace idrs {
int compute_alpha(int degree, const double* H, int ldh, int nh, double* alpha);
int compute_alpha(int degree, const std::complex<double>* H, int ldh, int nh, std::complex<double>* alpha);
int neumann(int degree, double center, double* alpha);
int neumann(int degree, std::complex<double> center, std::complex<double>* alpha);
int chebyshev(int degree, const double* foci, double* alpha);
int chebyshev(int degree, const std::complex<double>* foci, std::complex<double>* alpha);
// Jacobi matrices ((degree+2) x (degree+1), column-major) of the residual
// polynomials; real problems pass real values with zero imaginary parts.
std::vector<std::complex<double>> neumann_jacobi(int degree, std::complex<double> center);
std::vector<std::complex<double>> chebyshev_jacobi(int degree, const std::complex<double>* foci);
void qr_eig(const double* H, int ldh, int n, std::complex<double>* eig, int* converged);
// complex: U (n x n, optional) receives the Schur vectors (CQR_eig's U)
void qr_eig(const std::complex<double>* H, int ldh, int n, std::complex<double>* eig, int* converged,
            std::complex<double>* U = nullptr);
void analyse_spectrum(const double* H, int ldh, int n, double* foci, double* center, double* shift);
void analyse_spectrum(const std::complex<double>* H, int ldh, int n, std::complex<double>* foci,
                      std::complex<double>* center, std::complex<double>* shift);
}  // namespace idrs
