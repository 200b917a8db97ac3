// setup.h -- host set-up arithmetic of the polynomial preconditioners.
#pragma once
#include <complex>

namespace idrs {
int compute_alpha(int degree, const double* H, int ldh, int nh, double* alpha);
int compute_alpha(int degree, const std::complex<double>* H, int ldh, int nh, std::complex<double>* alpha);
int neumann(int degree, double center, double* alpha);
int neumann(int degree, std::complex<double> center, std::complex<double>* alpha);
int chebyshev(int degree, const double* foci, double* alpha);
int chebyshev(int degree, const std::complex<double>* foci, std::complex<double>* alpha);
void qr_eig(const double* H, int ldh, int n, std::complex<double>* eig, int* converged);
void qr_eig(const std::complex<double>* H, int ldh, int n, std::complex<double>* eig, int* converged);
void analyse_spectrum(const double* H, int ldh, int n, double* foci, double* center, double* shift);
void analyse_spectrum(const std::complex<double>* H, int ldh, int n, std::complex<double>* foci,
                      std::complex<double>* center, std::complex<double>* shift);
}  // namespace idrs
