/*
 * oracle.h -- CPU restatement of the IDRS package's solve path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the CUDA
 * implementation in idrs-package_gb300/.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg (and its `--impl reference` arm) may load it.
 * The product path never calls into it.
 *
 * Parity status: partially pinned.  The reference (Fortran 2018 + coarrays) has
 * no compiler in this environment and commits no golden outputs, and its shadow
 * space P comes from gfortran's RANDOM_NUMBER.  The restatement is pinned by
 *   - tests/golden fixtures made by independent implementations
 *     (scipy.sparse.linalg.bicgstab iterates for the deterministic BiCGSTAB
 *     variant, numpy Chebyshev/eigen/solve results), see tests/golden/make_golden.py;
 *   - the reference's own known-answer examples (Toeplitz finite termination
 *     N+N/s, b = A*1 => x = 1, the true-residual flag logic).
 *
 * Every routine follows the reference operation by operation and cites the
 * Fortran source it restates (paths relative to the IDRS-package root, with
 * IDRS/MODULES abbreviated M/ and IDRS/EXAMPLES abbreviated E/).
 *
 * Conventions: vectors are contiguous; complex values are C99 double _Complex
 * (layout-compatible with Fortran complex(real64) and numpy complex128);
 * index arrays handed to the *_format constructors are 1-based like the
 * Fortran API and stored 0-based.  Small matrices (M, H, W blocks) are
 * column-major like Fortran.
 */
#ifndef IDRS_ORACLE_H
#define IDRS_ORACLE_H

#include <complex.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef double _Complex or_cplx;

/* status codes (same meaning as the CUDA library's C-ABI) */
enum { OR_OK = 0, OR_EARG = 1, OR_EALLOC = 3, OR_EUNSUP = 5 };

/* user_matrix formats: M/PP_MATRIX/user_module.f90:134-167 (1..4) and the
 * matrix-free 7-point stencil of E/STENCIL/user_module.f90:39-187 (5). */
enum { OR_DENSE = 1, OR_CRS = 2, OR_COO = 3, OR_CDS = 4, OR_STENCIL7 = 5 };

typedef struct or_umat {
  int format, which_precon, nrows, ncols;
  int vals;                    /* 0: pattern only, 1: real, 2: complex */
  double *rmat; or_cplx *cmat; /* dense, column-major nrows x ncols */
  int *row_ptr, *col_ind;      /* CRS, 0-based */
  int nnz; int *indx, *jndx;   /* COO, 0-based */
  double *rval; or_cplx *cval; /* CRS/COO values */
  int half_band;               /* CDS: band(nrows, -hb:hb) column-major */
  double *rband; or_cplx *cband;
  int nx, ny, nz; double st[7];/* stencil coefficients c,w,e,s,n,f,b */
} or_umat;

typedef struct or_mat {
  const or_umat *K, *P;        /* P: user preconditioner (diagonal) or NULL */
  const or_umat *M, *C;        /* mass and damping matrices or NULL */
  int mass_matrix, damping_matrix, block_system;
  double rseed; or_cplx cseed;
  int preconditioner, degree;
  double *ralpha_p; or_cplx *calpha_p;   /* 0..degree */
  int n_sigma; double *ralpha_s; or_cplx *calpha_s; /* (degree+1) x n_sigma */
  void *sigma_s;               /* n_sigma shifts relative to the seed (ms_parameters) */
  void *sigma;                 /* the shifts of the last ms_parameters call */
  int multishift;              /* deflation projector I - V V^H */
  int shift_invert;            /* P is the LU of the matrix at `shift` */
  double rshift; or_cplx cshift;
  int n_deflation;             /* deflation: V, AV (n x k), V^H A V (k x k) */
  void *defl_V, *defl_AV, *defl_E;
  /* evaluation of the polynomial: 0 Horner (rpolpre), 1 the three-term
   * recurrence of its Jacobi matrix (no counterpart in the reference);
   * jac = (a_i, b_i, c_i), i = 1..degree+1, of the kind of the operator */
  int poly_eval;
  void *jac;
} or_mat;

/* Optional arguments of the solvers: a NULL pointer means "not present". */
typedef struct or_opts {
  const double *tolerance;
  const int *maximum_iterations;
  const int *variant;
  const or_mat *M1;
  const int *inner_s;
  const double *inner_tolerance;
  const int *inner_iterations;
  const void *x0;               /* n */
  const void *U0;               /* n x s column-major */
  const void *omega; int n_omega;
  const void *PT;               /* injected shadow space, s x n, row j contiguous */
  int *flag; double *relres; int *iterations;
  double *resvec; int resvec_len; /* msidrs/msqmridr: resvec_len x n_sigma */
  void *H; int H_rows, H_cols;  /* column-major */
  void *colfac;
  uint64_t p_seed;              /* seed of the shadow-space generator (default 1) */
  int skip_inner_true_residual; /* unused by the oracle (always faithful) */
  int inner_round32;            /* test probe, 0 = the reference: each nested MSIDRS result of
                                   MSQMRIDR (solutions and collinearity factors) rounded to
                                   single precision, the way a complex64 inner solve hands its
                                   output to the FP64 outer iteration */
} or_opts;

/* ---- counter-based uniform generator shared with the CUDA library ---- */
double or_uniform(uint64_t seed, uint64_t index);

/* ---- user_module ---- */
int or_crs_format(int nrows, int ncols, const int *row_ptr1, const int *col_ind1,
                  const double *rval, const double *cval, or_umat **out);
int or_coo_format(int nrows, int ncols, int nnz, const int *indx1, const int *jndx1,
                  const double *rval, const double *cval, or_umat **out);
int or_cds_format(int nrows, int ncols, int half_band, const double *rband,
                  const double *cband, or_umat **out);
int or_dense_format(int nrows, int ncols, const double *rmat, const double *cmat,
                    or_umat **out);
int or_stencil7_format(int nx, int ny, int nz, const double coef[7], or_umat **out);
int or_real_precon(int which_precon, const or_umat *K, const double *shift, or_umat **out);
int or_complex_precon(int which_precon, const or_umat *K, const double *shift, or_umat **out);
int or_real_precon_ext(int which_precon, const or_umat *K, const or_umat *M, const or_umat *C,
                       const double *shift, or_umat **out);
int or_complex_precon_ext(int which_precon, const or_umat *K, const or_umat *M, const or_umat *C,
                          const double *shift, or_umat **out);
int or_real_diagonal(const or_umat *K, double *D);
int or_complex_diagonal(const or_umat *K, or_cplx *D);
void or_umat_free(or_umat *A);
void or_user_mv_r(const or_umat *A, const double *v, double *w);
void or_user_mv_c(const or_umat *A, const or_cplx *v, or_cplx *w);
void or_user_precon_r(const or_umat *A, const double *v, double *w);
void or_user_precon_c(const or_umat *A, const or_cplx *v, or_cplx *w);

/* ---- matrix_module ---- */
int or_matrix_create(const or_umat *K, const or_umat *P, const double *seed, int cplx,
                     or_mat **out);
/* type(matrix) with mass M and damping C (real_matrix.inc:9-43): the 2x2
 * block system when multishift and C are both present (vectors of 2n); with
 * P and shift, P is a shift-and-invert preconditioner (the LU of
 * K + shift C + shift^2 M; for the block system rprecon's block form). */
int or_matrix_create_ext(const or_umat *K, const or_umat *M, const or_umat *C,
                         const or_umat *P, const double *seed, const double *shift, int cplx,
                         int multishift, or_mat **out);
/* 0: Horner (the reference), 1: the Jacobi three-term recurrence */
int or_matrix_set_poly_eval(or_mat *A, int mode);
void or_matrix_free(or_mat *A);
int or_real_preconditioner(or_mat *A, int preconditioner, int degree, const double *foci,
                           const double *center, const double *H, int ldh, int nh);
int or_complex_preconditioner(or_mat *A, int preconditioner, int degree, const or_cplx *foci,
                              const or_cplx *center, const or_cplx *H, int ldh, int nh);
int or_real_ms_parameters(or_mat *A, int n_sigma, const double *sigma, double *sigma_p);
int or_complex_ms_parameters(or_mat *A, int n_sigma, const or_cplx *sigma, or_cplx *sigma_p);
void or_matvec_r(const or_mat *A, int n, const double *v, double *w);
void or_matvec_c(const or_mat *A, int n, const or_cplx *v, or_cplx *w);
void or_precon_r(const or_mat *A, int n, const double *v, double *w);
void or_precon_c(const or_mat *A, int n, const or_cplx *v, or_cplx *w);
void or_scaleback_r(const or_mat *A, int n, const double *b, const double *y, double *x);
void or_scaleback_c(const or_mat *A, int n, const or_cplx *b, const or_cplx *y, or_cplx *x);
void or_ms_scaleback_r(const or_mat *A, int n, int n_sigma, const double *y, double *x);
void or_ms_scaleback_c(const or_mat *A, int n, int n_sigma, const or_cplx *y, or_cplx *x);
/* ms_scaleback with the right-hand side b (needed by a deflated operator) */
void or_ms_scaleback_b_r(const or_mat *A, int n, int n_sigma, const double *b, const double *y, double *x);
void or_ms_scaleback_b_c(const or_mat *A, int n, int n_sigma, const or_cplx *b, const or_cplx *y, or_cplx *x);
/* make_deflation (matrix_module.f90:1284-1346), Pmul (:1348-1418) and
 * add_deflation (:1420-1623).  The real projector uses AV like the complex
 * one (the reference's real branch subtracts V t instead). */
int or_make_deflation_r(or_mat *A, int n, const double *V, int k);
int or_make_deflation_c(or_mat *A, int n, const or_cplx *V, int k);
void or_pmul_r(const or_mat *A, int n, const double *v, double *w);
void or_pmul_c(const or_mat *A, int n, const or_cplx *v, or_cplx *w);
int or_rneumann(int degree, double center, double *alpha);
int or_rchebyshev(int degree, const double foci[2], double *alpha);
int or_rcompute_alpha(int degree, const double *H, int ldh, int nh, double *alpha);
int or_cneumann(int degree, or_cplx center, or_cplx *alpha);
int or_cchebyshev(int degree, const or_cplx foci[2], or_cplx *alpha);
int or_ccompute_alpha(int degree, const or_cplx *H, int ldh, int nh, or_cplx *alpha);
int or_ranalyse_spectrum(const double *H, int ldh, int n, double *foci, double *center,
                         double *shift);
int or_canalyse_spectrum(const or_cplx *H, int ldh, int n, or_cplx *foci, or_cplx *center,
                         or_cplx *shift);

/* ---- dense_la_module ---- */
int or_rqr_eig(const double *H, int ldh, int n, or_cplx *eig, int *converged);
int or_cqr_eig(const or_cplx *H, int ldh, int n, or_cplx *eig, int *converged);
void or_rsolve(int n, const double *A, const double *b, double *x);
void or_csolve(int n, const or_cplx *A, const or_cplx *b, or_cplx *x);
void or_rgrot(double a, double b, double *c, double *s, double *r);
void or_cgrot(or_cplx a, or_cplx b, or_cplx *c, or_cplx *s, or_cplx *r);

/* ---- idrs_module ---- */
double or_norm_r(int n, const double *w);
double or_norm_c(int n, const or_cplx *w);
int or_make_p_r(int s, int n, int method, uint64_t seed, const double *r, double *PT);
int or_make_p_c(int s, int n, int method, uint64_t seed, const or_cplx *r, or_cplx *PT);
int or_idrs_r(const or_mat *A, int n, const double *b, int s, const or_opts *o, double *x);
int or_idrs_c(const or_mat *A, int n, const or_cplx *b, int s, const or_opts *o, or_cplx *x);
int or_qmridr_r(const or_mat *A, int n, const double *b, int s, const or_opts *o, double *x);
int or_qmridr_c(const or_mat *A, int n, const or_cplx *b, int s, const or_opts *o, or_cplx *x);
int or_msidrs_r(const or_mat *A, int n, const double *b, int n_sigma, const double *sigma,
                int s, const or_opts *o, double *x);
int or_msidrs_c(const or_mat *A, int n, const or_cplx *b, int n_sigma, const or_cplx *sigma,
                int s, const or_opts *o, or_cplx *x);
int or_msqmridr_r(const or_mat *A, int n, const double *b, int n_sigma, const double *sigma,
                  int s, const or_opts *o, double *x);
int or_msqmridr_c(const or_mat *A, int n, const or_cplx *b, int n_sigma, const or_cplx *sigma,
                  int s, const or_opts *o, or_cplx *x);

/* ---- ritz_module ----
 * or_idrs_ritz_rx: IDRS_RITZ with the H output (o->H), omega(n_omega) and
 * the recycle space U0(n x dimU0) (NULL / 0: not requested).  si_seed seeds
 * the start block of SI_power (0: seed 2). */
int or_idrs_ritz_r(const or_mat *A, int n, const double *b, int s, const or_opts *o,
                   double *x, int *nritz);
int or_idrs_ritz_rx(const or_mat *A, int n, const double *b, int s, const or_opts *o,
                    double *x, int *nritz, double *omega, int n_omega, double *U0, int dimU0,
                    uint64_t si_seed);
int or_rsi_power(const double *H, int ldh, int n, int s, double shift, uint64_t seed,
                 double *vec);
int or_rcompute_U0(const or_mat *A, const or_mat *M, int n, const double *H, int ldh, int nritz,
                   const double *eigvec, int ns, const double *b, double *U0, double *resnrm);
int or_rglobal_qr(int n, int s, const double *V, double *Q, double *R);
int or_ritz_omega(const double *Hf, int ldh, int n_omega, double *omega);
int or_ritz_omega_c(const or_cplx *Hf, int ldh, int n_omega, or_cplx *omega);
int or_ccompute_U0(const or_mat *A, const or_mat *M, int n, const or_cplx *H, int ldh, int nritz,
                   const or_cplx *eigvec, int ns, const or_cplx *b, or_cplx *U0, double *resnrm);
int or_cglobal_qr(int n, int s, const or_cplx *V, or_cplx *Q, or_cplx *R);
/* CIDRS_RITZ: complex IDRS_RITZ with H (o->H), omega and U0 (Schur vectors) */
int or_idrs_ritz_cx(const or_mat *A, int n, const or_cplx *b, int s, const or_opts *o,
                    or_cplx *x, int *nritz, or_cplx *omega, int n_omega, or_cplx *U0, int dimU0);

/* ---- pp_idrs pipeline (real, single right-hand side) ----
 * method: 1 idrs, 2 bicgstab, 0 qmridr.  preconditioner: 0 none, 1 neumann,
 * 2 chebyshev, 3 hessenberg.  foci/center: NULL => estimated from n_ritz Ritz values. */
typedef struct or_pp_args {
  int method, s, maxit, in_s, in_it, preconditioner, degree, n_ritz;
  double tol, in_tol;
  const double *foci, *center;
  uint64_t p_seed;
  /* outputs */
  int flag, iterations, ritz_iterations, nritz_used;
  double relres_solver, relres_original;
  double foci_used[2], center_used;
  double alpha_p[64];
  double seconds_setup, seconds_solve; /* wall clock of the set-up and the solve */
  /* -omega and -recycle (initialize.inc:162-163) */
  int n_omega, recycle;
  uint64_t si_seed;
  double omega_used[64];
  int recycle_flag, recycle_iterations;
  double recycle_relres;
  /* per right-hand side outputs of or_pp_mr_idrs_r (arrays of nrhs; may be NULL) */
  int *flags, *iters;
  double *relres_solver_all, *relres_original_all;
  int poly_eval;               /* as or_mat.poly_eval, for the pipeline's operator */
} or_pp_args;
int or_pp_idrs_r(const or_umat *K, const or_umat *P, int n, const double *b, or_pp_args *a,
                 double *x);
/* PP_MR_IDRS (real): pp_idrs_module.f90:222-279 with real_preconditioner.inc,
 * recycle.inc and run_mr_idrs.inc.  b_all, x_all: n x nrhs column-major. */
int or_pp_mr_idrs_r(const or_umat *K, const or_umat *P, int n, int nrhs, const double *b_all,
                    or_pp_args *a, double *x_all);

/* ---- adjoint (new; no counterpart in the reference) ----
 * grad = -lambda_i * x_j over the CRS pattern of K. */
void or_sparse_outer_grad(const or_umat *K, const double *lambda, const double *x, double *g);
int or_crs_transpose(const or_umat *K, or_umat **out);

/* runtime controls */
void or_set_threads(int nthreads);
int or_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
