/*
 * idrs_gb300.h -- C ABI of the GB300-native IDRS solve path.
 *
 * Drop-in boundary for the Fortran 2018 API of the IDRS package
 * (mbvangijzen/IDRS-package).  Each entry point names the Fortran interface
 * it replaces (path:line in the IDRS package; M/ = IDRS/MODULES).  A Fortran
 * ISO_C_BINDING module (idrs-package_gb300/fortran/idrs_gb300_module.f90)
 * binds these with the reference's module and routine names.
 *
 * Conventions
 *  - Every function returns an int status: IDRS_OK (0) or an error code; the
 *    message of the last error on the calling thread is idrs_last_error().
 *    The library never aborts the process (the reference's `error stop`
 *    becomes a status code; the Fortran shim turns it back into error stop).
 *  - Fortran OPTIONAL arguments are pointers: NULL means "not present", which
 *    is what an OPTIONAL dummy of a BIND(C) interface passes when absent.
 *  - Real vectors are double*, complex vectors are double* holding
 *    interleaved (re, im) pairs (Fortran complex(real64), C99 double _Complex).
 *  - Index arrays are 1-based int32, as in the Fortran API.
 *  - Vector arguments of the solver, matvec and scaleback calls are host
 *    pointers by default (copied in and out, never retained).  After
 *    idrs_matrix_set_pointer_mode(A, IDRS_POINTER_DEVICE) they are device
 *    pointers on the current CUDA device.
 *  - One CUDA stream per idrs_matrix handle (idrs_matrix_set_stream).
 *  - Small matrices (H, U0, multishift x(n, n_sigma), resvec(maxit+1,
 *    n_sigma)) are column-major like Fortran.
 */
#ifndef IDRS_GB300_H
#define IDRS_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define IDRS_OK 0
#define IDRS_ERR_ARG 1         /* illegal argument (reference: error stop / stop) */
#define IDRS_ERR_CUDA 2        /* CUDA runtime error, or a staged (TMA) copy that never completed */
#define IDRS_ERR_ALLOC 3       /* out of device or host memory */
#define IDRS_ERR_STATE 4       /* handle used in the wrong state */
#define IDRS_ERR_UNSUPPORTED 5 /* valid in the reference, not in this build */

#define IDRS_POINTER_HOST 0
#define IDRS_POINTER_DEVICE 1

/* type(user_matrix): M/PP_MATRIX/user_module.f90:134-167 */
typedef struct idrs_user_matrix_s *idrs_user_matrix;
/* type(matrix): M/PP_MATRIX/matrix_module.f90:38-81 */
typedef struct idrs_matrix_s *idrs_matrix;

const char *idrs_last_error(void);
int idrs_version(void);
/* Number of CUDA kernels this library has launched in this process
 * (measurement helper; no counterpart in the reference). */
long idrs_launch_count(void);

/* ---------------------------------------------------------------------- */
/* user_module                                                            */
/* ---------------------------------------------------------------------- */

/* crs_format(nrows, ncols, row_ptr, col_ind[, rval, ival, cval]):
 * user_module.f90:829-863.  rval (real) or cval (complex) or neither
 * (pattern only, all values 1). */
int idrs_crs_format(int nrows, int ncols, const int *row_ptr, const int *col_ind,
                    const double *rval, const double *cval, idrs_user_matrix *K);
/* coo_format(nrows, ncols, nnz, indx, jndx[, rval, ival, cval]): user_module.f90:865-898 */
int idrs_coo_format(int nrows, int ncols, int nnz, const int *indx, const int *jndx,
                    const double *rval, const double *cval, idrs_user_matrix *K);
/* cds_format(nrows, ncols, half_band[, rband, iband, cband]): user_module.f90:932-958.
 * band(nrows, -half_band:half_band) column-major. */
int idrs_cds_format(int nrows, int ncols, int half_band, const double *rband,
                    const double *cband, idrs_user_matrix *K);
/* dense_format([rmat, imat, cmat]): user_module.f90:900-930 (column-major) */
int idrs_dense_format(int nrows, int ncols, const double *rmat, const double *cmat,
                      idrs_user_matrix *K);
/* Matrix-free 7-point stencil user_matrix of E/STENCIL/user_module.f90:39-187
 * (Dirichlet boundaries, x fastest).  coef = {c, w, e, s, n, f, b}. */
int idrs_stencil7_format(int nx, int ny, int nz, const double *coef, idrs_user_matrix *K);
/* REAL_PRECON(which_precon, K[, M, C, shift]): user_module.f90:1327-1463.
 * which_precon 0 (none) or 1 (diagonal scaling, D(K) - shift). */
int idrs_real_precon(int which_precon, idrs_user_matrix K, const double *shift,
                     idrs_user_matrix *P);
/* COMPLEX_PRECON: user_module.f90:1465-1603 (shift = {re, im}) */
int idrs_complex_precon(int which_precon, idrs_user_matrix K, const double *shift,
                        idrs_user_matrix *P);
/* The same with mass M and damping C (NULL = absent), user_module.f90:1327-1602.
 * which_precon 1: with a shift the diagonal of K + shift C + shift^2 M (C only:
 * + shift^2; M only: K - shift M), each matrix's diagonal with zeros -> 1.
 * which_precon 2 / 3: the dense / band LU factor (no pivoting, as the
 * reference; a zero pivot is IDRS_ERR_ARG) of that shifted matrix, factored
 * on the device; K, M, C may be CRS, COO, CDS or dense (as in the reference,
 * a CDS matrix has no dense form and a dense matrix no band form: they add
 * nothing there).  v/P is then two triangular solves on the device. */
int idrs_real_precon_ext(int which_precon, idrs_user_matrix K, idrs_user_matrix M,
                         idrs_user_matrix C, const double *shift, idrs_user_matrix *P);
int idrs_complex_precon_ext(int which_precon, idrs_user_matrix K, idrs_user_matrix M,
                            idrs_user_matrix C, const double *shift, idrs_user_matrix *P);
/* real_diagonal(K) / complex_diagonal(K): user_module.f90:960-1047, 1049-1136 */
int idrs_real_diagonal(idrs_user_matrix K, double *D);
int idrs_complex_diagonal(idrs_user_matrix K, double *D);
/* operator(*) of user_matrix: ruser_mv / cuser_mv, user_module.f90:182-241 (host vectors) */
int idrs_ruser_mv(idrs_user_matrix K, const double *v, double *w);
int idrs_cuser_mv(idrs_user_matrix K, const double *v, double *w);
int idrs_user_matrix_free(idrs_user_matrix K);

/* ---------------------------------------------------------------------- */
/* Matrix Market input: E/MATRIX_MARKET/mm_module.f90:48-154 (mm_matrix)  */
/* ---------------------------------------------------------------------- */
/* A = mm_matrix(mm_file[, which_format]): coordinate files become a COO
 * (which_format NULL or "coo", the reference's default) or CRS ("crs")
 * user_matrix, array files a dense one.  Symmetric, skew-symmetric and
 * Hermitian files are expanded; complex entries pass through single
 * precision and integer entries become reals, as in the reference. */
int idrs_mm_matrix(const char *mm_file, const char *which_format, idrs_user_matrix *A);
/* The same conversion into host arrays (no GPU needed).  Call once with
 * ptr = ind = vals = NULL for the sizes, then with arrays of those sizes.
 * rep: 0 coordinate, 1 array; field: 0 real, 1 complex, 2 integer, 3 pattern.
 * coordinate "crs": ptr = row_ptr (nrows+1), ind = col_ind (nnz), 1-based;
 * coordinate "coo": ptr = indx (nnz), ind = jndx (nnz), 1-based;
 * array: nnz = nrows*ncols values in column order (ptr, ind unused);
 * vals: nnz reals, or 2*nnz interleaved re/im for complex. */
int idrs_mm_read(const char *mm_file, const char *which_format, int *rep, int *field, int *nrows,
                 int *ncols, long *nnz, int *ptr, int *ind, double *vals);

/* ---------------------------------------------------------------------- */
/* matrix_module                                                          */
/* ---------------------------------------------------------------------- */

/* A%K = K, A%P = P, A%rseed/cseed = seed: M/PP_IDRS/real_matrix.inc:9-58.
 * is_complex selects the real (r*) or complex (c*) specifics; seed = {re[, im]}. */
int idrs_matrix_create(idrs_user_matrix K, idrs_user_matrix P, int is_complex,
                       const double *seed, idrs_matrix *A);
/* The same with mass M and damping C (real_matrix.inc:9-43; NULL = absent)
 * and the multishift flag.  real_mv/complex_mv (matrix_module.f90:170-264):
 *   seed 0: K;  C and M: K + seed C + seed^2 M;  C: K + seed C + seed^2 I;
 *   M: K - seed M;  multishift with C: the 2n x 2n block system
 *   [-C - seed M, -K; I, -seed I] (without M: -seed I in the (1,1) block),
 *   whose vectors have length 2n and whose diagonal scaling is [P; 1].
 * The combination is assembled once into one CRS matrix (K, M, C must be
 * CRS or COO; others: IDRS_ERR_UNSUPPORTED), so each product is one SpMV.
 * With a shift-and-invert P (which_precon 2/3) and `shift` (NULL = absent),
 * A%shift_invert holds (real_matrix.inc:23-29): every product is
 * K' (P^-1 v), ms_parameters uses (sigma - seed)/(sigma - shift) and the
 * multishift scaleback the factor (seed - shift)/(sigma - shift).  For the
 * block system P is the LU of K + shift C + shift^2 M (n x n) and v/A is
 * rprecon's block form (matrix_module.f90:318-345). */
int idrs_matrix_create_ext(idrs_user_matrix K, idrs_user_matrix M, idrs_user_matrix C,
                           idrs_user_matrix P, int is_complex, const double *seed,
                           const double *shift, int multishift, idrs_matrix *A);
int idrs_matrix_free(idrs_matrix A);
int idrs_matrix_set_stream(idrs_matrix A, void *cuda_stream);
int idrs_matrix_set_pointer_mode(idrs_matrix A, int mode);
/* How fp64 products evaluate the polynomial preconditioner (no counterpart
 * in the reference, which always uses rpolpre's Horner scheme on the
 * monomial coefficients, matrix_module.f90:266-284):
 *   IDRS_POLY_HORNER (default): Horner, as the reference;
 *   IDRS_POLY_RECURRENCE: the three-term recurrence of the polynomial's
 *     tridiagonal Jacobi matrix (Chebyshev and Neumann, matrix_module.f90:
 *     851-941), for A*v, IDRS/QMRIDR and scaleback.  A degree-8 Chebyshev
 *     polynomial fitted to a wide spectrum has monomial coefficients of
 *     +-10^3..10^4 with alternating signs, so Horner cancels digits and the
 *     true residual of an fp64 solve stalls above 1e-8 at 256^3; the
 *     recurrence keeps its iterates of the size of A^-1 v.
 * fp32 products always use the recurrence.  Multishift solves, their
 * per-shift scale-back, the recycle space and operators with deflation or a
 * shift-and-invert preconditioner keep Horner, as does the Hessenberg
 * polynomial (no Jacobi matrix). */
#define IDRS_POLY_HORNER 0
#define IDRS_POLY_RECURRENCE 1
int idrs_matrix_set_poly_eval(idrs_matrix A, int mode);
/* Injects the shadow space used by solves with this s (row j of PT is
 * PT + j*n, real or interleaved complex).  PT = NULL removes it.  The
 * reference draws P from gfortran's RANDOM_NUMBER (idrs_module.f90:839-937);
 * without an injected P this library draws it from a documented seeded
 * generator (splitmix64), shared with the CPU oracle. */
int idrs_matrix_set_shadow(idrs_matrix A, int s, const double *PT);

/* real_preconditioner(A, preconditioner, degree[, foci, center, H]):
 * matrix_module.f90:551-635.  preconditioner 0 none, 1 Neumann, 2 Chebyshev,
 * 3 Hessenberg.  H(ldh, nh) column-major. */
int idrs_real_preconditioner(idrs_matrix A, int preconditioner, int degree, const double *foci,
                             const double *center, const double *H, int ldh, int nh);
/* complex_preconditioner: matrix_module.f90:637-722 (complex foci[2], center, H) */
int idrs_complex_preconditioner(idrs_matrix A, int preconditioner, int degree,
                                const double *foci, const double *center, const double *H,
                                int ldh, int nh);
/* Polynomial coefficients alpha_p(0:degree) currently held by A. */
int idrs_matrix_get_alpha(idrs_matrix A, double *alpha, int *degree);
/* ms_parameters(A, sigma, sigma_p): matrix_module.f90:402-549 */
int idrs_real_ms_parameters(idrs_matrix A, int n_sigma, const double *sigma, double *sigma_p);
int idrs_complex_ms_parameters(idrs_matrix A, int n_sigma, const double *sigma,
                               double *sigma_p);
/* operator(*): rmatvec / cmatvec, matrix_module.f90:135-167 */
int idrs_rmatvec(idrs_matrix A, const double *v, double *w);
int idrs_cmatvec(idrs_matrix A, const double *v, double *w);
/* A*v evaluated in fp32, the operator of the fp32 inner solves (new, no
 * reference counterpart): v is rounded to fp32, the polynomial is applied by
 * its stable recurrence when A holds a Chebyshev/Neumann preconditioner, and
 * w is returned widened to fp64. */
int idrs_rmatvec32(idrs_matrix A, const double *v, double *w);
/* operator(/): rprecon / cprecon, matrix_module.f90:306-400  (w = v/A) */
int idrs_rprecon(idrs_matrix A, const double *v, double *w);
int idrs_cprecon(idrs_matrix A, const double *v, double *w);
/* make_deflation(A, V): matrix_module.f90:1284-1346.  V(n, k), k <= 16,
 * column-major (complex: interleaved), host or device per the pointer mode;
 * stores V, A V = real_mv(A, V) and V^H A V; k = 0 removes the deflation.
 * From then on A*v is Pmul(real_mv(polpre(v))) (matrix_module.f90:152-167)
 * and scaleback adds the deflated components (add_deflation, :1420-1623).
 * Pmul is I - AV (V^H A V)^-1 V^H, or I - V V^H for a multishift operator
 * (idrs_matrix_create_ext with multishift = 1).  The reference's real branch
 * subtracts V t instead of AV t (matrix_module.f90:1415); this library uses
 * AV for both kinds.  Not available with fp32 inner solves. */
int idrs_make_deflation(idrs_matrix A, const double *V, int k);
/* w = Pmul(A, v): matrix_module.f90:1348-1418 */
int idrs_rpmul(idrs_matrix A, const double *v, double *w);
int idrs_cpmul(idrs_matrix A, const double *v, double *w);
/* scaleback(A, b, y): matrix_module.f90:811-849 */
int idrs_rscaleback(idrs_matrix A, const double *b, const double *y, double *x);
int idrs_cscaleback(idrs_matrix A, const double *b, const double *y, double *x);
/* scaleback(A, sigma, b, y) (multishift): matrix_module.f90:724-809 */
int idrs_ms_rscaleback(idrs_matrix A, int n_sigma, const double *sigma, const double *b,
                       const double *y, double *x);
int idrs_ms_cscaleback(idrs_matrix A, int n_sigma, const double *sigma, const double *b,
                       const double *y, double *x);

/* Measurement helper (no counterpart in the reference): runs `reps` products
 * w = A*v of the operator chain (degree+1 SpMV launches) in precision prec
 * (64 or 32) on A's stream, after `warmup` untimed ones, on internal vectors
 * of length n, and returns the CUDA-event time per product and per launch.
 * Each vector is larger than the GPU's L2 for n >= 2^24 (fp64). */
int idrs_time_matvec(idrs_matrix A, int prec, int warmup, int reps, double *ms_per_product,
                     double *ms_per_launch);
/* The same products as idrs_time_matvec, captured once as a CUDA graph and
 * replayed `reps` times between CUDA events (no counterpart in the
 * reference): the product as the IDR(s) cycles run it, whose captured cycles
 * are replayed graphs too.  warmup >= 1 (the products before the capture
 * allocate the operator's lazily created work arrays). */
int idrs_time_matvec_graph(idrs_matrix A, int prec, int warmup, int reps, double *ms_per_product);
/* Device time of the sparse gradient kernel (idrs_rsparse_outer_grad) on A's
 * CRS matrix: reps launches back to back on A's stream between CUDA events,
 * after warmup launches, with vectors the call allocates (no host copies, no
 * synchronisation between launches).  No reference counterpart. */
int idrs_time_sparse_outer_grad(idrs_matrix A, int warmup, int reps, double *ms_per_call);

/* ---------------------------------------------------------------------- */
/* idrs_module                                                            */
/* ---------------------------------------------------------------------- */

/* x = IDRS(A, b, s[, M1, tolerance, maximum_iterations, variant, flag, relres,
 *          iterations, x0, U0, omega, resvec, H]):
 * RIDRS idrs_module.f90:180-251, CIDRS :107-178, body M/IDRS/idrs.inc.
 * U0(n, s) column-major; omega(n_omega); resvec(resvec_len >= maxit+1);
 * H(nritz+1, nritz) column-major with ldh = nritz+1. */
int idrs_ridrs(idrs_matrix A, const double *b, int s, idrs_matrix M1, const double *tolerance,
               const int *maximum_iterations, const int *variant, int *flag, double *relres,
               int *iterations, const double *x0, const double *U0, const double *omega,
               int n_omega, double *resvec, int resvec_len, double *H, int ldh, int nritz,
               double *x);
int idrs_cidrs(idrs_matrix A, const double *b, int s, idrs_matrix M1, const double *tolerance,
               const int *maximum_iterations, const int *variant, int *flag, double *relres,
               int *iterations, const double *x0, const double *U0, const double *omega,
               int n_omega, double *resvec, int resvec_len, double *H, int ldh, int nritz,
               double *x);

/* x = QMRIDR(A, b, s[, M1, tolerance, maximum_iterations, flag, relres,
 *            iterations, inner_s, inner_tolerance, inner_iterations, x0, omega,
 *            resvec]): RQMRIDR idrs_module.f90:331-408, CQMRIDR :253-329,
 * body M/IDRS/qmridr.inc.  inner_precision (new, optional): 64 (default) or
 * 32 -- the inner IDR(inner_s) and its operator run in fp32 (complex64). */
int idrs_rqmridr(idrs_matrix A, const double *b, int s, idrs_matrix M1,
                 const double *tolerance, const int *maximum_iterations, int *flag,
                 double *relres, int *iterations, const int *inner_s,
                 const double *inner_tolerance, const int *inner_iterations, const double *x0,
                 const double *omega, int n_omega, double *resvec, int resvec_len,
                 const int *inner_precision, double *x);
int idrs_cqmridr(idrs_matrix A, const double *b, int s, idrs_matrix M1,
                 const double *tolerance, const int *maximum_iterations, int *flag,
                 double *relres, int *iterations, const int *inner_s,
                 const double *inner_tolerance, const int *inner_iterations, const double *x0,
                 const double *omega, int n_omega, double *resvec, int resvec_len,
                 const int *inner_precision, double *x);

/* x(n, n_sigma) = MSIDRS(A, b, sigma, s[, M1, tolerance, maximum_iterations,
 *                 variant, flag, relres, iterations, omega, resvec, colfac]):
 * RMSIDRS idrs_module.f90:572-641, CMSIDRS :643-713, body M/IDRS/msidrs.inc.
 * Solves (A - sigma_k I) x_k = b for every shift.  sigma(n_sigma) and
 * omega(n_omega) have the kind of b (complex: interleaved re/im);
 * relres(n_sigma); resvec(resvec_len, n_sigma) column-major with
 * resvec_len >= maxit+1; colfac(n_sigma) of the kind of b; x column-major.
 * variant 1: MSIDRS(s), 2: MSBiCGSTAB (s = 1).  n_sigma <= 64. */
int idrs_rmsidrs(idrs_matrix A, const double *b, int n_sigma, const double *sigma, int s,
                 idrs_matrix M1, const double *tolerance, const int *maximum_iterations,
                 const int *variant, int *flag, double *relres, int *iterations,
                 const double *omega, int n_omega, double *resvec, int resvec_len, double *colfac,
                 double *x);
int idrs_cmsidrs(idrs_matrix A, const double *b, int n_sigma, const double *sigma, int s,
                 idrs_matrix M1, const double *tolerance, const int *maximum_iterations,
                 const int *variant, int *flag, double *relres, int *iterations,
                 const double *omega, int n_omega, double *resvec, int resvec_len, double *colfac,
                 double *x);

/* x(n, n_sigma) = MSQMRIDR(A, b, sigma, s[, M1, tolerance, maximum_iterations,
 *                   flag, relres, iterations, inner_s, inner_tolerance,
 *                   inner_iterations, omega, resvec]):
 * RMSQMRIDR idrs_module.f90:491-570, CMSQMRIDR :410-489, body
 * M/IDRS/msqmridr.inc.  With inner_iterations > 0 each iteration runs
 * MSIDRS(inner_s) on the shifts [sigma, 0] as flexible preconditioner;
 * inner_precision (new, optional): 64 (default) or 32 -- that inner solve and
 * its operator run in fp32 (complex64).  n_sigma <= 63. */
int idrs_rmsqmridr(idrs_matrix A, const double *b, int n_sigma, const double *sigma, int s,
                   idrs_matrix M1, const double *tolerance, const int *maximum_iterations,
                   int *flag, double *relres, int *iterations, const int *inner_s,
                   const double *inner_tolerance, const int *inner_iterations,
                   const double *omega, int n_omega, double *resvec, int resvec_len,
                   const int *inner_precision, double *x);
int idrs_cmsqmridr(idrs_matrix A, const double *b, int n_sigma, const double *sigma, int s,
                   idrs_matrix M1, const double *tolerance, const int *maximum_iterations,
                   int *flag, double *relres, int *iterations, const int *inner_s,
                   const double *inner_tolerance, const int *inner_iterations,
                   const double *omega, int n_omega, double *resvec, int resvec_len,
                   const int *inner_precision, double *x);

/* Statistics of the last QMRIDR solve with inner iterations on handle A (new,
 * no reference counterpart): number of inner solves, their total and largest
 * iteration counts. */
int idrs_solve_stats(idrs_matrix A, int *inner_solves, int *inner_iterations, int *inner_max);

/* ---------------------------------------------------------------------- */
/* Adjoint (backward) path of A x = b with a real CRS matrix A = K.  No    */
/* counterpart in the reference, which has no adjoint (its compliance      */
/* sensitivities, E/TOP/top_opt.f90:209-224, are written by hand for a     */
/* self-adjoint problem).  For a scalar loss L(x):                         */
/*   K^T lambda = dL/dx,  dL/db = lambda,  dL/dK_ij = -lambda_i x_j.       */
/* ---------------------------------------------------------------------- */
/* K^T as a new CRS user_matrix (device; stable: ascending rows of K). */
int idrs_crs_transpose(idrs_user_matrix K, idrs_user_matrix *KT);
/* grad(nnz) = -lambda_i x_j over the stored entries of A's CRS matrix K, in
 * K's storage order; vectors follow A's pointer mode and stream. */
int idrs_rsparse_outer_grad(idrs_matrix A, const double *lambda, const double *x, double *grad);
/* One backward step: IDR(s) on the adjoint operator AT (built from K^T,
 * optionally with its own preconditioner and seed) for AT lambda = g
 * (g = dL/dx), lambda = scaleback(AT, g, mu); then, if grad is given,
 * grad(nnz) = -lambda_i x_j over K's pattern.  flag/relres/iterations are
 * those of the adjoint solve.  Pointer mode and stream are AT's. */
int idrs_radjoint(idrs_matrix AT, idrs_user_matrix K, const double *x, const double *g, int s,
                  const double *tolerance, const int *maximum_iterations, int *flag,
                  double *relres, int *iterations, double *lambda, double *grad);

/* NORM(w): idrs_module.f90:787-811;  INPROD(u, v): idrs_module.f90:813-837 */
int idrs_rnorm(idrs_matrix A, const double *w, double *norm);
int idrs_cnorm(idrs_matrix A, const double *w, double *norm);
int idrs_rinprod(idrs_matrix A, const double *u, const double *v, double *uv);
int idrs_cinprod(idrs_matrix A, const double *u, const double *v, double *uv);

/* INPROD(u, v) = sum u_i v_i of two real device vectors of length n, written
 * to the device double *uv, without allocating any device memory.  No
 * counterpart in the reference: it serves callers that cannot call
 * cudaMalloc (their device memory belongs to another allocator, or their
 * policy forbids allocating after start-up).  Its scratch is a static
 * 128 KiB device array held by every GPU that loads this library, so n is
 * limited to 67,108,864 (IDRS_ERR_ARG beyond).  The first call on each device
 * performs a one-time set-up; make it before any stream capture.  The call
 * is asynchronous on `stream` (a cudaStream_t, NULL for the default stream);
 * calls that overlap on the GPU share the scratch and race.  u, v and uv must
 * be device memory of the current device (or managed memory); other pointers
 * return IDRS_ERR_ARG before anything is launched. */
int idrs_rinprod_noalloc(long n, const double *u, const double *v, double *uv, void *stream);

/* x = IDRS_RITZ(A, b, s[, M, tolerance, maximum_iterations, variant, flag,
 *               relres, iterations, x0, U0, omega, resvec, H]): ritz_module.f90:389-556.
 * Runs IDRS with the Hessenberg output Hf and returns, besides x:
 *  - H(ldh, nh) = Hf(1:ldh, 1:nh) (NULL: not wanted);
 *  - *nritz = (iter/(s+1))*s + mod(iter,s+1);
 *  - omega(n_omega): 1/Re of the Ritz values of Hf(1:n_omega,1:n_omega),
 *    ordered greedily (n_omega > nritz: IDRS_ERR_ARG, as the reference's stop);
 *  - U0(n, dimU0), dimU0 <= 16: the recycle space, an orthonormal basis of
 *    the Krylov combination of the dimU0 Schur vectors of Hf(1:nritz,1:nritz)
 *    nearest 0 (SI_power, compute_U0, global QR).  The reference starts
 *    SI_power from RANDOM_NUMBER; this library from a fixed counter-based
 *    uniform block (seed 2).  U0 follows the pointer mode of A (host or device).
 * resvec(resvec_len >= maxit+1) receives the residual norms. */
int idrs_ridrs_ritz(idrs_matrix A, const double *b, int s, idrs_matrix M,
                    const double *tolerance, const int *maximum_iterations, const int *variant,
                    int *flag, double *relres, int *iterations, const double *x0, double *U0,
                    int dimU0, double *omega, int n_omega, double *resvec, int resvec_len,
                    double *H, int ldh, int nh, int *nritz, double *x);
/* CIDRS_RITZ (ritz_module.f90:268-387): the same for a complex A (b, x, x0,
 * U0, omega and H interleaved).  omega = 1/ritz ordered greedily with the
 * complex Ritz values; U0 from the first dimU0 Schur vectors of QR_eig. */
int idrs_cidrs_ritz(idrs_matrix A, const double *b, int s, idrs_matrix M,
                    const double *tolerance, const int *maximum_iterations, const int *variant,
                    int *flag, double *relres, int *iterations, const double *x0, double *U0,
                    int dimU0, double *omega, int n_omega, double *resvec, int resvec_len,
                    double *H, int ldh, int nh, int *nritz, double *x);

/* ---------------------------------------------------------------------- */
/* pp_idrs: M/PP_IDRS/pp_idrs_module.f90:118-162 (RPP_IDRS) with            */
/* real_matrix.inc, real_preconditioner.inc:10-34 and run_idrs.inc:9-60.  */
/* The reference reads its options from the command line                 */
/* (initialize.inc:4-31); here they are a struct.                         */
/* ---------------------------------------------------------------------- */
typedef struct idrs_pp_options {
  int method;          /* 1 idrs, 2 bicgstab, 0 qmridr */
  int s;
  double tol;
  int maxit;
  int in_s, in_it;
  double in_tol;
  int preconditioner;  /* 0 none, 1 neumann, 2 chebyshev, 3 hessenberg */
  int degree;
  int n_ritz;          /* -ritz (default 32) */
  int inner_precision; /* 64 or 32 */
  int device_pointers; /* 1: b and x are device pointers */
  int n_omega;         /* -omega: number of Ritz-value omegas (default 0) */
  int recycle;         /* -recycle: 1 builds the s-dimensional recycle space U0 */
  int poly_eval;       /* IDRS_POLY_HORNER (0, the reference) or IDRS_POLY_RECURRENCE for
                          the fp64 products (see idrs_matrix_set_poly_eval); no
                          counterpart in the reference */
  double fp64_check_tol; /* > 0: after each solve, solve the same preconditioned system
                            again from x0 = 0 with the FP64 form of the method (no inner
                            solves; at least min(2n, 5000) iterations) to this tolerance
                            and report the relative error of x against that solution
                            (report->rel_err_vs_fp64); 0: no check.  Not counted in
                            seconds_solve.  No counterpart in the reference. */
} idrs_pp_options;

typedef struct idrs_pp_report {
  int flag, iterations, ritz_iterations, nritz;
  double relres_solver, relres_original;
  double foci[2], center;
  double seconds_setup, seconds_solve, seconds_total;
  int inner_solves, inner_iterations, inner_max;  /* flexible QMRIDR: inner IDR(s) statistics */
  int recycle_flag, recycle_iterations;            /* the recycle.inc solve (recycle = 1) */
  double recycle_relres;
  double foci_imag[2], center_imag;                 /* complex pipelines: imaginary parts */
  /* opt->fp64_check_tol > 0: ||x - x64|| / ||x64|| against the FP64 solve x64,
   * and that solve's flag, iterations, true residual and wall time; otherwise
   * rel_err_vs_fp64 = fp64_relres_original = -1 and fp64_flag = -1 */
  double rel_err_vs_fp64, fp64_relres_original;
  int fp64_flag, fp64_iterations;
  double seconds_fp64_check;
} idrs_pp_report;

/* sizeof(idrs_pp_options) (which 0), sizeof(idrs_pp_report) (1) or
 * sizeof(idrs_pp_inputs) (2), for bindings that declare the structs
 * themselves; 0 for another value.  Needs no GPU. */
long idrs_pp_struct_size(int which);

/* The optional inputs of pp_idrs beyond P, center and foci
 * (pp_idrs_module.f90: M, C, seed, shift, V); NULL = all absent.  seed and
 * shift have the kind of the pipeline (complex: {re, im}); V is n x
 * n_deflation (host, complex interleaved).  With P and shift, P is a
 * shift-and-invert preconditioner (which_precon 2 or 3). */
typedef struct idrs_pp_inputs {
  idrs_user_matrix M, C;
  const double *seed, *shift;
  const double *V;
  int n_deflation;
} idrs_pp_inputs;

int idrs_rpp_idrs(idrs_user_matrix K, const double *b, idrs_user_matrix P, const double *center,
                  const double *foci, const idrs_pp_options *opt, idrs_pp_report *report,
                  double *x);

/* pp_idrs with every optional input: RPP_IDRS / CPP_IDRS (pp_idrs_module.f90:
 * 64-162; complex: center 2 and foci 4 doubles, b and x interleaved).  The
 * complex pipelines compute the Ritz omegas and the recycle space like CIDRS_RITZ. */
int idrs_rpp_idrs_ext(idrs_user_matrix K, const double *b, idrs_user_matrix P, const double *center,
                      const double *foci, const idrs_pp_inputs *in, const idrs_pp_options *opt,
                      idrs_pp_report *report, double *x);
int idrs_cpp_idrs(idrs_user_matrix K, const double *b, idrs_user_matrix P, const double *center,
                  const double *foci, const idrs_pp_inputs *in, const idrs_pp_options *opt,
                  idrs_pp_report *report, double *x);

/* x_all = pp_idrs(K, b_all[, P, center, foci]) for nrhs right-hand sides:
 * RPP_MR_IDRS (pp_idrs_module.f90:222-279) with real_preconditioner.inc,
 * recycle.inc and run_mr_idrs.inc.  The set-up solves use b_all(:,1); the
 * systems are then solved in order, each started from the previous
 * (preconditioned) solution, with U0 (opt->recycle, IDRS only) and omega
 * (opt->n_omega).  b_all and x_all are n x nrhs column-major, host or (with
 * opt->device_pointers) device arrays.  reports: nrhs entries or NULL. */
int idrs_rpp_mr_idrs(idrs_user_matrix K, int nrhs, const double *b_all, idrs_user_matrix P,
                     const double *center, const double *foci, const idrs_pp_options *opt,
                     idrs_pp_report *reports, double *x_all);
/* the same with every optional input (RPP_MR_IDRS / CPP_MR_IDRS,
 * pp_idrs_module.f90:164-279) */
int idrs_rpp_mr_idrs_ext(idrs_user_matrix K, int nrhs, const double *b_all, idrs_user_matrix P,
                         const double *center, const double *foci, const idrs_pp_inputs *in,
                         const idrs_pp_options *opt, idrs_pp_report *reports, double *x_all);
int idrs_cpp_mr_idrs(idrs_user_matrix K, int nrhs, const double *b_all, idrs_user_matrix P,
                     const double *center, const double *foci, const idrs_pp_inputs *in,
                     const idrs_pp_options *opt, idrs_pp_report *reports, double *x_all);

/* x(n, n_sigma) = pp_idrs(K, rhs, sigma[, M, C, P, center, foci, seed, shift,
 * V]): RPP_MS_IDRS / CPP_MS_IDRS with run_ms_idrs.inc.  With C the operator is
 * the 2n x 2n block system, b = [-rhs; 0] and x the second half of each
 * solution.  method 1/2 runs MSIDRS, 0 MSQMRIDR.  relres(n_sigma): the true
 * residuals |rhs - K x - sigma C x - sigma^2 M x| / |rhs| (and the other
 * forms); report->relres_original is their maximum.  Host arrays only. */
int idrs_rpp_ms_idrs(idrs_user_matrix K, const double *rhs, int n_sigma, const double *sigma,
                     idrs_user_matrix P, const double *center, const double *foci,
                     const idrs_pp_inputs *in, const idrs_pp_options *opt, idrs_pp_report *report,
                     double *relres, double *x);
int idrs_cpp_ms_idrs(idrs_user_matrix K, const double *rhs, int n_sigma, const double *sigma,
                     idrs_user_matrix P, const double *center, const double *foci,
                     const idrs_pp_inputs *in, const idrs_pp_options *opt, idrs_pp_report *report,
                     double *relres, double *x);
/* x(n, n_sigma, nrhs) = pp_idrs(K, rhs(n, nrhs), sigma[, ...]): RPP_MS_MR_IDRS /
 * CPP_MS_MR_IDRS with run_ms_mr_idrs.inc: one set-up (on rhs(:,1)) and one
 * ms_parameters, then one multishift solve per right-hand side.
 * reports(nrhs), relres(n_sigma, nrhs). */
int idrs_rpp_ms_mr_idrs(idrs_user_matrix K, int nrhs, const double *rhs, int n_sigma,
                        const double *sigma, idrs_user_matrix P, const double *center,
                        const double *foci, const idrs_pp_inputs *in, const idrs_pp_options *opt,
                        idrs_pp_report *reports, double *relres, double *x);
int idrs_cpp_ms_mr_idrs(idrs_user_matrix K, int nrhs, const double *rhs, int n_sigma,
                        const double *sigma, idrs_user_matrix P, const double *center,
                        const double *foci, const idrs_pp_inputs *in, const idrs_pp_options *opt,
                        idrs_pp_report *reports, double *relres, double *x);

#ifdef __cplusplus
}
#endif
#endif
