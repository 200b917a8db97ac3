// setup.cpp -- host-side set-up arithmetic of the polynomial preconditioners:
// Chebyshev / Neumann Jacobi matrices, the residual-polynomial coefficients,
// the QR eigenvalues of the Ritz Hessenberg matrix and the spectrum analysis
// that turns them into foci / a centre, and the multishift coefficients.
// All of it is O(degree^2) or O(nritz^3) scalar work done once per solve;
// it stays in fp64 on the host.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <complex>
#include <vector>

#include "setup.h"

namespace idrs {

using cd = std::complex<double>;

// compute_alpha: matrix_module.f90:983-1057.  J(ldh, >= degree+1) column-major.
template <class S>
static int compute_alpha_t(int degree, const S* H, int ldh, int nh, S* alpha) {
  if (degree == 0) { alpha[0] = S(1.0); return 0; }
  if (ldh < degree + 2 || nh < degree + 1) return 1;
  const int d2 = degree + 2;
  std::vector<S> r((size_t)d2 * d2, S(0.0));
  auto R = [&](int i, int c) -> S& { return r[i + (size_t)d2 * c]; };
  R(0, 0) = S(1.0);
  for (int i = 1; i <= degree + 1; ++i) {
    for (int c = 1; c <= degree + 1; ++c) R(i, c) = R(i - 1, c - 1);
    for (int j = 0; j <= i - 1; ++j) {
      S hji = H[j + (size_t)ldh * (i - 1)];
      for (int c = 0; c <= degree + 1; ++c) R(i, c) = R(i, c) - hji * R(j, c);
    }
    S hd = H[i + (size_t)ldh * (i - 1)];
    for (int c = 0; c <= degree + 1; ++c) R(i, c) = R(i, c) / hd;
  }
  for (int c = 1; c <= degree + 1; ++c) alpha[c - 1] = -R(degree + 1, c);
  return 0;
}

// Jacobi matrix of the Neumann residual polynomials: matrix_module.f90:851-875
template <class S>
static std::vector<S> neumann_jacobi_t(int degree, S center) {
  const int ld = degree + 2;
  std::vector<S> J((size_t)ld * (degree + 1), S(0.0));
  for (int i = 1; i <= degree + 1; ++i) {
    J[(i - 1) + (size_t)ld * (i - 1)] = center;
    J[i + (size_t)ld * (i - 1)] = -center;
  }
  return J;
}

// Jacobi matrix of the shifted and scaled Chebyshev residual polynomials:
// matrix_module.f90:903-941
template <class S>
static std::vector<S> chebyshev_jacobi_t(int degree, const S* foci) {
  S theta = (foci[0] + foci[1]) / 2.0;
  S delta = (foci[0] - foci[1]) / 2.0;
  S sigma = theta / delta;
  const int ld = degree + 2;
  std::vector<S> J((size_t)ld * (degree + 1), S(0.0));
  J[0] = theta;
  J[1] = -theta;
  S rho = S(1.0) / sigma;
  for (int i = 2; i <= degree + 1; ++i) {
    J[(i - 2) + (size_t)ld * (i - 1)] = -delta * rho / 2.0;
    J[(i - 1) + (size_t)ld * (i - 1)] = delta * sigma;
    J[i + (size_t)ld * (i - 1)] = -delta * sigma + delta * rho / 2.0;
    rho = S(1.0) / (2.0 * sigma - rho);
  }
  return J;
}

template <class S>
static int neumann_t(int degree, S center, S* alpha) {
  auto J = neumann_jacobi_t<S>(degree, center);
  return compute_alpha_t<S>(degree, J.data(), degree + 2, degree + 1, alpha);
}
template <class S>
static int chebyshev_t(int degree, const S* foci, S* alpha) {
  auto J = chebyshev_jacobi_t<S>(degree, foci);
  return compute_alpha_t<S>(degree, J.data(), degree + 2, degree + 1, alpha);
}

int compute_alpha(int degree, const double* H, int ldh, int nh, double* a) { return compute_alpha_t(degree, H, ldh, nh, a); }
int compute_alpha(int degree, const cd* H, int ldh, int nh, cd* a) { return compute_alpha_t(degree, H, ldh, nh, a); }
int neumann(int degree, double c, double* a) { return neumann_t(degree, c, a); }
int neumann(int degree, cd c, cd* a) { return neumann_t(degree, c, a); }
int chebyshev(int degree, const double* f, double* a) { return chebyshev_t(degree, f, a); }
int chebyshev(int degree, const cd* f, cd* a) { return chebyshev_t(degree, f, a); }
std::vector<cd> neumann_jacobi(int degree, cd center) { return neumann_jacobi_t<cd>(degree, center); }
std::vector<cd> chebyshev_jacobi(int degree, const cd* foci) { return chebyshev_jacobi_t<cd>(degree, foci); }

// CQR_factorization with refine = 2: dense_la_module.f90:42-83
static int cqr_factorization(int m, const cd* V, int ldv, cd* Q, cd* R) {
  for (int j = 0; j < m; ++j)
    for (int i = 0; i < m; ++i) { Q[i + m * j] = V[i + ldv * j]; R[i + m * j] = 0.0; }
  for (int j = 0; j < m; ++j) {
    for (int k = 0; k < 2; ++k)
      for (int i = 0; i < j; ++i) {
        cd t = 0.0;
        for (int q = 0; q < m; ++q) t += std::conj(Q[q + m * i]) * Q[q + m * j];
        for (int q = 0; q < m; ++q) Q[q + m * j] = Q[q + m * j] - t * Q[q + m * i];
        R[i + m * j] = R[i + m * j] + t;
      }
    double nr = 0.0;
    for (int q = 0; q < m; ++q) nr += std::norm(Q[q + m * j]);
    R[j + m * j] = R[j + m * j] + std::sqrt(nr);
    if (std::abs(R[j + m * j]) > DBL_MIN) {
      for (int q = 0; q < m; ++q) Q[q + m * j] = Q[q + m * j] / R[j + m * j];
    } else {
      return j + 1;
    }
  }
  return 0;
}

// RQR_eig / CQR_eig: dense_la_module.f90:192-403 (shifted QR iteration)
static void qr_eig_core(int n, std::vector<cd>& V, bool real_version, cd* eig, int* converged,
                        cd* U = nullptr) {
  int iter = 0, m = n, maxit = real_version ? 100 * n : 10 * n;
  const double tol = DBL_EPSILON;
  std::vector<cd> Q((size_t)n * n), R((size_t)n * n), RQ((size_t)n * n);
  auto VV = [&](int i, int j) -> cd& { return V[i + (size_t)n * j]; };
  std::vector<cd> UQ;
  if (U) {  // Schur vectors: U = I, then U(:, 1:m) = U(:, 1:m) Q after every step
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) U[i + (size_t)n * j] = (i == j) ? cd(1.0) : cd(0.0);
    UQ.resize((size_t)n * n);
  }
  cd shift = 0.0;
  if (real_version) {
    for (int i = 0; i < m; ++i) if (std::abs(VV(i, i)) > std::abs(shift)) shift = VV(i, i);
    shift = shift * cd(1.0, 1.0);
  } else {
    shift = VV(n - 1, n - 1);
  }
  while (m > 1 && iter < maxit) {
    for (int i = 0; i < m; ++i) VV(i, i) = VV(i, i) - shift;
    if (cqr_factorization(m, V.data(), n, Q.data(), R.data()) > 0) break;
    for (int j = 0; j < m; ++j)
      for (int i = 0; i < m; ++i) {
        cd acc = 0.0;
        for (int q = 0; q < m; ++q) acc += R[i + m * q] * Q[q + m * j];
        RQ[i + m * j] = acc;
      }
    for (int j = 0; j < m; ++j)
      for (int i = 0; i < m; ++i) VV(i, j) = RQ[i + m * j];
    for (int i = 0; i < m; ++i) VV(i, i) = VV(i, i) + shift;
    if (U) {
      for (int j = 0; j < m; ++j)
        for (int i = 0; i < n; ++i) {
          cd acc = 0.0;
          for (int q = 0; q < m; ++q) acc += U[i + (size_t)n * q] * Q[q + m * j];
          UQ[i + (size_t)n * j] = acc;
        }
      for (int j = 0; j < m; ++j)
        for (int i = 0; i < n; ++i) U[i + (size_t)n * j] = UQ[i + (size_t)n * j];
    }
    if (std::abs(VV(m - 1, m - 2)) < tol * std::abs(VV(m - 1, m - 1))) m = m - 1;
    if (real_version) {
      shift = 0.0;
      for (int i = 0; i < m; ++i) if (std::abs(VV(i, i)) > std::abs(shift)) shift = VV(i, i);
    } else {
      shift = VV(m - 1, m - 1);
    }
    iter = iter + 1;
  }
  for (int i = 0; i < n; ++i) eig[i] = VV(i, i);
  if (converged) *converged = n - m + 1;
}

void qr_eig(const double* H, int ldh, int n, cd* eig, int* converged) {
  std::vector<cd> V((size_t)n * n);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) V[i + (size_t)n * j] = H[i + (size_t)ldh * j];
  qr_eig_core(n, V, true, eig, converged);
}
void qr_eig(const cd* H, int ldh, int n, cd* eig, int* converged, cd* U) {
  std::vector<cd> V((size_t)n * n);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) V[i + (size_t)n * j] = H[i + (size_t)ldh * j];
  qr_eig_core(n, V, false, eig, converged, U);
}

// filter_ritzval: matrix_module.f90:1059-1077
static std::vector<int> filter_ritzval(const std::vector<cd>& rv) {
  const int n = (int)rv.size();
  cd center = 0.0;
  for (auto& z : rv) center += z;
  center /= (double)n;
  double sg = 0.0;
  for (auto& z : rv) sg += std::norm(z - center);
  sg = std::sqrt(sg / n);
  std::vector<int> out(n);
  for (int i = 0; i < n; ++i) out[i] = std::abs(rv[i] - center) > 1.5 * sg;
  return out;
}

struct Box { double left, right, bottom, top; };
static Box box_of(const std::vector<cd>& rv, const std::vector<int>& out) {
  Box b{INFINITY, -INFINITY, INFINITY, -INFINITY};
  for (size_t i = 0; i < rv.size(); ++i) {
    if (out[i]) continue;
    b.left = std::min(b.left, rv[i].real());
    b.right = std::max(b.right, rv[i].real());
    b.bottom = std::min(b.bottom, rv[i].imag());
    b.top = std::max(b.top, rv[i].imag());
  }
  return b;
}

// ranalyse_spectrum: matrix_module.f90:1079-1181
void analyse_spectrum(const double* H, int ldh, int n, double* foci, double* center,
                      double* shift) {
  std::vector<cd> rv(n);
  qr_eig(H, ldh, n, rv.data(), nullptr);
  auto out = filter_ritzval(rv);
  Box b = box_of(rv, out);
  double center_box = (b.right + b.left) / 2.0;
  double radius = -INFINITY;
  for (int i = 0; i < n; ++i) if (!out[i]) radius = std::max(radius, std::abs(rv[i] - center_box));
  double center_circle = center_box;
  if (std::abs(center_box) / radius < 1) center_circle = center_box / (std::abs(center_box) / radius);
  double shift_circle = center_box - center_circle;
  double x0 = (b.right - b.left) / 2.0, y0 = (b.top - b.bottom) / 2.0;
  double a = std::sqrt(x0 * (x0 + y0)), bb = std::sqrt(y0 * (x0 + y0));
  double center_ellipse = center_box;
  if (std::abs(center_box) / a < 1.0) center_ellipse = center_box / (std::abs(center_box) / a);
  double f1, f2;
  if (a > bb) {
    double c = std::sqrt(a * a - bb * bb);
    f1 = center_ellipse - c; f2 = center_ellipse + c;
  } else {
    double c = 0.15 * center_ellipse;
    f1 = center_ellipse - c; f2 = center_ellipse + c;
  }
  if (foci) { foci[0] = f1; foci[1] = f2; }
  if (center) *center = center_circle;
  if (shift) *shift = shift_circle;
}

// canalyse_spectrum: matrix_module.f90:1183-1282
void analyse_spectrum(const cd* H, int ldh, int n, cd* foci, cd* center, cd* shift) {
  std::vector<cd> rv(n);
  qr_eig(H, ldh, n, rv.data(), nullptr);
  auto out = filter_ritzval(rv);
  Box b = box_of(rv, out);
  cd center_box = cd(b.right + b.left, b.top + b.bottom) / 2.0;
  double radius = -INFINITY;
  for (int i = 0; i < n; ++i) if (!out[i]) radius = std::max(radius, std::abs(rv[i] - center_box));
  cd center_circle = center_box;
  if (std::abs(center_box) / radius < 1) center_circle = center_box / (std::abs(center_box) / radius);
  cd shift_circle = center_box - center_circle;
  double x0 = (b.right - b.left) / 2.0, y0 = (b.top - b.bottom) / 2.0;
  double a = std::sqrt(x0 * (x0 + y0)), bb = std::sqrt(y0 * (x0 + y0));
  cd center_ellipse = center_box;
  double q = std::pow(center_box.real() / a, 2) + std::pow(center_box.imag() / bb, 2);
  if (q < 1.0) center_ellipse = center_box / std::sqrt(q);
  cd f1, f2;
  if (a > bb) {
    double c = std::sqrt(a * a - bb * bb);
    f1 = center_ellipse - c; f2 = center_ellipse + c;
  } else {
    double c = std::sqrt(bb * bb - a * a);
    f1 = center_ellipse - cd(0, c); f2 = center_ellipse + cd(0, c);
  }
  if (foci) { foci[0] = f1; foci[1] = f2; }
  if (center) *center = center_circle;
  if (shift) *shift = shift_circle;
}

}  // namespace idrs
