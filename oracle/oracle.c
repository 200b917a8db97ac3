/*
 * oracle.c -- CPU restatement of the IDRS package's solve path.
 *
 * TEST INFRASTRUCTURE ONLY (parity checker and CPU baseline); see oracle.h
 * for the rules on who may load it and for the parity status.
 */
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_NCHUNK 64
#define OR_MAXS 64

/* ------------------------------------------------------------------------ */
/* shadow-space generator: splitmix64 of the element index, shared bit for  */
/* bit with the CUDA library (csrc/common.cuh idrs_uniform).                */
/* ------------------------------------------------------------------------ */
static inline uint64_t or_splitmix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
double or_uniform(uint64_t seed, uint64_t index) {
  uint64_t z = or_splitmix64(index ^ or_splitmix64(seed));
  return (double)(z >> 11) * 0x1.0p-53;
}

void or_set_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
}
int or_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* GROT: M/IDRS/dense_la_module.f90:683-742 (BLAS rotg style)              */
/* ------------------------------------------------------------------------ */
void or_rgrot(double a, double b, double *c, double *s, double *r) {
  if (fabs(a) < DBL_EPSILON) {
    *c = 0.; *s = 1.; *r = b;
  } else {
    double rho = hypot(fabs(a), fabs(b));
    double alpha = a / fabs(a);
    *c = fabs(a) / rho;
    *s = alpha * b / rho;
    *r = alpha * rho;
  }
}
void or_cgrot(or_cplx a, or_cplx b, or_cplx *c, or_cplx *s, or_cplx *r) {
  if (cabs(a) < DBL_EPSILON) {
    *c = 0.; *s = 1.; *r = b;
  } else {
    double rho = hypot(cabs(a), cabs(b));
    or_cplx alpha = a / cabs(a);
    *c = cabs(a) / rho;
    *s = alpha * conj(b) / rho;
    *r = alpha * rho;
  }
}
static void or_grot__r(double a, double b, double *c, double *s, double *r) { or_rgrot(a, b, c, s, r); }
static void or_grot__c(or_cplx a, or_cplx b, or_cplx *c, or_cplx *s, or_cplx *r) { or_cgrot(a, b, c, s, r); }

/* ------------------------------------------------------------------------ */
/* LU arithmetic (LU_decomp / LU_solve, user_module.f90:1604-1831): every   */
/* multiply-subtract as FMAs and every complex division as Smith's          */
/* algorithm with FMAs, in the order the CUDA library uses (csrc/lu.cu      */
/* lu_msub / lu_div), so factors and solutions agree bit for bit.  Without  */
/* pivoting the elimination's growth turns the difference between one       */
/* rounding and two into relative differences near 5e-9 on a uniform       */
/* random 120 x 120 matrix.  l is the factor's entry.                       */
/* ------------------------------------------------------------------------ */
static inline double or_lu_msub_r(double a, double l, double b) { return fma(-l, b, a); }
static inline or_cplx or_lu_msub_c(or_cplx a, or_cplx l, or_cplx b) {
  double ax = creal(a), ay = cimag(a), lx = creal(l), ly = cimag(l), bx = creal(b), by = cimag(b);
  return CMPLX(fma(ly, by, fma(-lx, bx, ax)), fma(-ly, bx, fma(-lx, by, ay)));
}
static inline or_cplx or_lu_div_c(or_cplx a, or_cplx b) {
  double ax = creal(a), ay = cimag(a), bx = creal(b), by = cimag(b);
  if (fabs(bx) >= fabs(by)) {
    double r = by / bx, d = fma(by, r, bx);
    return CMPLX(fma(ay, r, ax) / d, fma(-ax, r, ay) / d);
  }
  double r = bx / by, d = fma(bx, r, by);
  return CMPLX(fma(ax, r, ay) / d, fma(ay, r, -ax) / d);
}

/* ------------------------------------------------------------------------ */
/* element-type-generic part                                                */
/* ------------------------------------------------------------------------ */
#define T double
#define SFX(name) name##_r
#define CONJ(x) (x)
#define ABSV(x) fabs(x)
#define IS_CPLX 0
#define LU_MSUB(a, l, b) or_lu_msub_r(a, l, b)
#define LU_DIV(a, b) ((a) / (b))
#include "oracle_core.inc"
#undef T
#undef SFX
#undef CONJ
#undef ABSV
#undef IS_CPLX
#undef LU_MSUB
#undef LU_DIV

#define T or_cplx
#define SFX(name) name##_c
#define CONJ(x) conj(x)
#define ABSV(x) cabs(x)
#define IS_CPLX 1
#define LU_MSUB(a, l, b) or_lu_msub_c(a, l, b)
#define LU_DIV(a, b) or_lu_div_c(a, b)
#include "oracle_core.inc"
#undef T
#undef SFX
#undef LU_MSUB
#undef LU_DIV
#undef CONJ
#undef ABSV
#undef IS_CPLX

void or_rsolve(int n, const double *A, const double *b, double *x) { or_solve__r(n, A, b, x); }
void or_csolve(int n, const or_cplx *A, const or_cplx *b, or_cplx *x) { or_solve__c(n, A, b, x); }

/* ------------------------------------------------------------------------ */
/* user_module constructors: M/PP_MATRIX/user_module.f90:829-958            */
/* ------------------------------------------------------------------------ */
static or_umat *umat_new(int format, int nrows, int ncols) {
  or_umat *A = calloc(1, sizeof(or_umat));
  if (!A) return NULL;
  A->format = format; A->nrows = nrows; A->ncols = ncols;
  return A;
}

/* crs_format: user_module.f90:829-863.  Indices arrive 1-based.  The
 * reference's quirk of storing ival into rval (:860) is immaterial here:
 * integer matrices arrive as real values. */
int or_crs_format(int nrows, int ncols, const int *row_ptr1, const int *col_ind1,
                  const double *rval, const double *cval, or_umat **out) {
  if (nrows < 0 || ncols < 0 || !row_ptr1 || !out) return OR_EARG;
  int nnz = row_ptr1[nrows] - row_ptr1[0];
  if (nnz < 0) return OR_EARG;
  or_umat *A = umat_new(OR_CRS, nrows, ncols);
  A->nnz = nnz;
  A->row_ptr = malloc(sizeof(int) * (nrows + 1));
  A->col_ind = malloc(sizeof(int) * (nnz > 0 ? nnz : 1));
  for (int i = 0; i <= nrows; ++i) A->row_ptr[i] = row_ptr1[i] - row_ptr1[0];
  for (int k = 0; k < nnz; ++k) {
    int c = col_ind1[k] - 1;
    if (c < 0 || c >= ncols) { or_umat_free(A); return OR_EARG; }
    A->col_ind[k] = c;
  }
  if (cval) {
    A->vals = 2; A->cval = malloc(sizeof(or_cplx) * (nnz > 0 ? nnz : 1));
    memcpy(A->cval, cval, sizeof(or_cplx) * nnz);
  } else if (rval) {
    A->vals = 1; A->rval = malloc(sizeof(double) * (nnz > 0 ? nnz : 1));
    memcpy(A->rval, rval, sizeof(double) * nnz);
  }
  *out = A;
  return OR_OK;
}

/* coo_format: user_module.f90:865-898 */
int or_coo_format(int nrows, int ncols, int nnz, const int *indx1, const int *jndx1,
                  const double *rval, const double *cval, or_umat **out) {
  if (nrows < 0 || ncols < 0 || nnz < 0 || !out) return OR_EARG;
  or_umat *A = umat_new(OR_COO, nrows, ncols);
  A->nnz = nnz;
  A->indx = malloc(sizeof(int) * (nnz > 0 ? nnz : 1));
  A->jndx = malloc(sizeof(int) * (nnz > 0 ? nnz : 1));
  for (int k = 0; k < nnz; ++k) {
    A->indx[k] = indx1[k] - 1; A->jndx[k] = jndx1[k] - 1;
    if (A->indx[k] < 0 || A->indx[k] >= nrows || A->jndx[k] < 0 || A->jndx[k] >= ncols) {
      or_umat_free(A); return OR_EARG;
    }
  }
  if (cval) {
    A->vals = 2; A->cval = malloc(sizeof(or_cplx) * (nnz > 0 ? nnz : 1));
    memcpy(A->cval, cval, sizeof(or_cplx) * nnz);
  } else if (rval) {
    A->vals = 1; A->rval = malloc(sizeof(double) * (nnz > 0 ? nnz : 1));
    memcpy(A->rval, rval, sizeof(double) * nnz);
  }
  *out = A;
  return OR_OK;
}

/* cds_format: user_module.f90:932-958 (band(nrows,-hb:hb), column-major) */
int or_cds_format(int nrows, int ncols, int half_band, const double *rband,
                  const double *cband, or_umat **out) {
  if (nrows < 0 || half_band < 0 || !out) return OR_EARG;
  or_umat *A = umat_new(OR_CDS, nrows, ncols);
  A->half_band = half_band;
  size_t cnt = (size_t)nrows * (2 * half_band + 1);
  if (cband) {
    A->vals = 2; A->cband = malloc(sizeof(or_cplx) * (cnt ? cnt : 1));
    memcpy(A->cband, cband, sizeof(or_cplx) * cnt);
  } else if (rband) {
    A->vals = 1; A->rband = malloc(sizeof(double) * (cnt ? cnt : 1));
    memcpy(A->rband, rband, sizeof(double) * cnt);
  }
  *out = A;
  return OR_OK;
}

/* dense_format: user_module.f90:900-930 */
int or_dense_format(int nrows, int ncols, const double *rmat, const double *cmat,
                    or_umat **out) {
  if (nrows < 0 || ncols < 0 || !out) return OR_EARG;
  or_umat *A = umat_new(OR_DENSE, nrows, ncols);
  size_t cnt = (size_t)nrows * ncols;
  if (cmat) {
    A->vals = 2; A->cmat = malloc(sizeof(or_cplx) * (cnt ? cnt : 1));
    memcpy(A->cmat, cmat, sizeof(or_cplx) * cnt);
  } else {
    A->vals = 1; A->rmat = malloc(sizeof(double) * (cnt ? cnt : 1));
    if (rmat) memcpy(A->rmat, rmat, sizeof(double) * cnt); else memset(A->rmat, 0, sizeof(double) * cnt);
  }
  *out = A;
  return OR_OK;
}

/* matrix-free stencil: E/STENCIL/user_module.f90:39-63 (coefficients c,w,e,s,n,f,b) */
int or_stencil7_format(int nx, int ny, int nz, const double coef[7], or_umat **out) {
  if (nx < 1 || ny < 1 || nz < 1 || !coef || !out) return OR_EARG;
  or_umat *A = umat_new(OR_STENCIL7, nx * ny * nz, nx * ny * nz);
  A->nx = nx; A->ny = ny; A->nz = nz; A->vals = 1;
  memcpy(A->st, coef, sizeof(double) * 7);
  *out = A;
  return OR_OK;
}

void or_umat_free(or_umat *A) {
  if (!A) return;
  free(A->rmat); free(A->cmat); free(A->row_ptr); free(A->col_ind); free(A->indx);
  free(A->jndx); free(A->rval); free(A->cval); free(A->rband); free(A->cband);
  free(A);
}

/* real_diagonal: user_module.f90:960-1047 (single image: phi == me always).
 * The stencil format (an extension) has the constant diagonal c. */
int or_real_diagonal(const or_umat *A, double *D) {
  int n = A->nrows;
  for (int i = 0; i < n; ++i) D[i] = 0.;
  switch (A->format) {
  case OR_DENSE:
    if (A->rmat) for (int i = 0; i < n; ++i) D[i] = A->rmat[i + (size_t)n * i];
    break;
  case OR_CRS:
    for (int i = 0; i < n; ++i)
      for (int j = A->row_ptr[i]; j < A->row_ptr[i + 1]; ++j)
        if (A->col_ind[j] == i) D[i] += (A->vals == 1) ? A->rval[j] : (A->vals == 0 ? 1. : creal(A->cval[j]));
    break;
  case OR_COO:
    for (int k = 0; k < A->nnz; ++k)
      if (A->indx[k] == A->jndx[k]) D[A->indx[k]] += (A->vals == 1) ? A->rval[k] : (A->vals == 0 ? 1. : creal(A->cval[k]));
    break;
  case OR_CDS:
    if (A->rband) for (int i = 0; i < n; ++i) D[i] = A->rband[i + (size_t)n * A->half_band];
    else for (int i = 0; i < n; ++i) D[i] = 1.;
    break;
  case OR_STENCIL7:
    for (int i = 0; i < n; ++i) D[i] = A->st[0];
    break;
  }
  for (int i = 0; i < n; ++i) if (D[i] == 0) D[i] = 1.;
  return OR_OK;
}
int or_complex_diagonal(const or_umat *A, or_cplx *D) {
  int n = A->nrows;
  for (int i = 0; i < n; ++i) D[i] = 0.;
  switch (A->format) {
  case OR_DENSE:
    for (int i = 0; i < n; ++i) D[i] = A->cmat ? A->cmat[i + (size_t)n * i] : A->rmat[i + (size_t)n * i];
    break;
  case OR_CRS:
    for (int i = 0; i < n; ++i)
      for (int j = A->row_ptr[i]; j < A->row_ptr[i + 1]; ++j)
        if (A->col_ind[j] == i) D[i] += (A->vals == 2) ? A->cval[j] : (A->vals == 1 ? A->rval[j] : 1.);
    break;
  case OR_COO:
    for (int k = 0; k < A->nnz; ++k)
      if (A->indx[k] == A->jndx[k]) D[A->indx[k]] += (A->vals == 2) ? A->cval[k] : (A->vals == 1 ? A->rval[k] : 1.);
    break;
  case OR_CDS:
    for (int i = 0; i < n; ++i)
      D[i] = A->cband ? A->cband[i + (size_t)n * A->half_band] : (A->rband ? A->rband[i + (size_t)n * A->half_band] : 1.);
    break;
  case OR_STENCIL7:
    for (int i = 0; i < n; ++i) D[i] = A->st[0];
    break;
  }
  for (int i = 0; i < n; ++i) if (D[i] == 0) D[i] = 1.;
  return OR_OK;
}

/* REAL_PRECON: user_module.f90:1327-1381, which_precon = 1 (diagonal
 * scaling, optionally shifted: D(K) - shift).  Dense/band LU are out of scope. */
/* ------------------------------------------------------------------------ */
/* Shift-and-invert preconditioners, which_precon 2 (dense LU) and 3 (band  */
/* LU): user_module.f90:1383-1463, :1520-1602, real_dense :1163-1235,      */
/* get_band :1833-1872, real_band :1981-2066, LU_decomp :1604-1701,         */
/* band_LU_decomp :2068-2179.  Values are combined in complex arithmetic    */
/* and stored by kind.                                                      */
/* ------------------------------------------------------------------------ */
static or_cplx umat_val(const or_umat *A, long k) {
  if (A->vals == 2) return A->cval[k];
  if (A->vals == 1) return A->rval[k];
  return 1.;
}

/* real_dense / complex_dense: dense (all), CRS, COO; other formats give zeros */
static void to_dense(const or_umat *A, or_cplx *D) {
  long n = A->nrows;
  for (long i = 0; i < n * (long)A->ncols; ++i) D[i] = 0;
  if (A->format == OR_DENSE) {
    for (long i = 0; i < n * (long)A->ncols; ++i) D[i] = A->cmat ? A->cmat[i] : (A->rmat ? A->rmat[i] : 0.);
  } else if (A->format == OR_CRS) {
    for (long i = 0; i < n; ++i)
      for (int k = A->row_ptr[i]; k < A->row_ptr[i + 1]; ++k) D[i + n * A->col_ind[k]] += umat_val(A, k);
  } else if (A->format == OR_COO) {
    for (long k = 0; k < A->nnz; ++k) D[A->indx[k] + n * A->jndx[k]] += umat_val(A, k);
  }
}

/* get_band */
static int band_of(const or_umat *A) {
  int hb = 0;
  if (A->format == OR_DENSE) return A->ncols;
  if (A->format == OR_CRS) {
    for (int i = 0; i < A->nrows; ++i)
      for (int k = A->row_ptr[i]; k < A->row_ptr[i + 1]; ++k) {
        int d = abs(A->col_ind[k] - i);
        if (d > hb) hb = d;
      }
  } else if (A->format == OR_COO) {
    for (long k = 0; k < A->nnz; ++k) {
      int d = abs(A->jndx[k] - A->indx[k]);
      if (d > hb) hb = d;
    }
  } else if (A->format == OR_CDS) {
    hb = A->half_band;
  }
  return hb;
}

/* real_band / complex_band: B(n, -hb:hb) from CRS, COO, CDS; dense gives zeros */
static void to_band(const or_umat *A, int hb, or_cplx *B) {
  long n = A->nrows, w = 2L * hb + 1;
  for (long i = 0; i < n * w; ++i) B[i] = 0;
  if (A->format == OR_CRS) {
    for (long i = 0; i < n; ++i)
      for (int k = A->row_ptr[i]; k < A->row_ptr[i + 1]; ++k)
        B[i + n * ((long)(A->col_ind[k] - i) + hb)] += umat_val(A, k);
  } else if (A->format == OR_COO) {
    for (long k = 0; k < A->nnz; ++k)
      B[A->indx[k] + n * ((long)(A->jndx[k] - A->indx[k]) + hb)] += umat_val(A, k);
  } else if (A->format == OR_CDS) {
    int h = A->half_band;
    for (long d = -h; d <= h; ++d)
      for (long i = 0; i < n; ++i) {
        or_cplx v = A->cband ? A->cband[i + n * (d + h)] : (A->rband ? A->rband[i + n * (d + h)] : 1.);
        B[i + n * (d + hb)] = v;
      }
  }
}

/* the shifted matrix K + shift C + shift^2 M (C only: + shift^2 I; M only:
 * K - shift M; neither: K - shift I), element by element like the reference */
static void combine(long cnt, or_cplx *S, const or_cplx *Cd, const or_cplx *Md, int hasC, int hasM,
                    or_cplx sh) {
  for (long i = 0; i < cnt; ++i) {
    if (hasM && hasC) S[i] = S[i] + sh * Cd[i] + (sh * sh) * Md[i];
    else if (hasC) S[i] = S[i] + sh * Cd[i];
    else if (hasM) S[i] = S[i] - sh * Md[i];
  }
}

/* LU_decomp without pivoting (real and complex factors: real matrices are
 * factored in real arithmetic); returns OR_EARG on a zero pivot */
#define OR_LU_DENSE(SUF, V, DIV, MSUB)                                          \
  static int lu_decomp_dense_##SUF(long n, V *LU) {                             \
    for (long k = 0; k < n; ++k) {                                              \
      V p = LU[k + n * k];                                                      \
      if (p == 0) return OR_EARG; /* 'Pivot equal to zero in LU decomposition' */ \
      for (long i = k + 1; i < n; ++i) {                                        \
        if (LU[i + n * k] == 0) continue;                                       \
        LU[i + n * k] = DIV(LU[i + n * k], p);                                  \
        V l = LU[i + n * k];                                                    \
        for (long j = k + 1; j < n; ++j) LU[i + n * j] = MSUB(LU[i + n * j], l, LU[k + n * j]); \
      }                                                                         \
    }                                                                           \
    return OR_OK;                                                               \
  }
/* band_LU_decomp without pivoting on B(n, -hb:hb) */
#define OR_LU_BAND(SUF, V, DIV, MSUB)                                           \
  static int lu_decomp_band_##SUF(long n, int hb, V *B) {                       \
    for (long k = 0; k < n - 1; ++k) {                                          \
      V p = B[k + n * (long)hb];                                                \
      if (p == 0) return OR_EARG;                                               \
      long last = k + hb < n - 1 ? k + hb : n - 1;                              \
      for (long i = k + 1; i <= last; ++i) {                                    \
        long dia = k - i;                                                       \
        V *bi = B + i + n * (dia + hb);                                         \
        *bi = DIV(*bi, p);                                                      \
        V l = *bi;                                                              \
        for (long j = 1; j <= hb; ++j)                                          \
          B[i + n * (dia + j + hb)] = MSUB(B[i + n * (dia + j + hb)], l, B[k + n * (j + hb)]); \
      }                                                                         \
    }                                                                           \
    return OR_OK;                                                               \
  }
#define OR_DIV_R(a, b) ((a) / (b))
OR_LU_DENSE(r, double, OR_DIV_R, or_lu_msub_r)
OR_LU_DENSE(c, or_cplx, or_lu_div_c, or_lu_msub_c)
OR_LU_BAND(r, double, OR_DIV_R, or_lu_msub_r)
OR_LU_BAND(c, or_cplx, or_lu_div_c, or_lu_msub_c)
#undef OR_DIV_R

static int lu_precon(int which, const or_umat *K, const or_umat *M, const or_umat *C,
                     const double *shift, int cplx, or_umat *P) {
  long n = K->nrows;
  or_cplx sh = 0;
  if (shift) sh = cplx ? shift[0] + I * shift[1] : shift[0];
  int st = OR_OK;
  if (which == 2) {
    long cnt = n * n;
    or_cplx *S = malloc(sizeof(or_cplx) * (cnt ? cnt : 1)), *Cd = NULL, *Md = NULL;
    to_dense(K, S);
    if (shift) {
      if (C) { Cd = malloc(sizeof(or_cplx) * (cnt ? cnt : 1)); to_dense(C, Cd); }
      if (M) { Md = malloc(sizeof(or_cplx) * (cnt ? cnt : 1)); to_dense(M, Md); }
      combine(cnt, S, Cd, Md, C != NULL, M != NULL, sh);
      if (C && !M) for (long i = 0; i < n; ++i) S[i + n * i] += sh * sh;
      if (!C && !M) for (long i = 0; i < n; ++i) S[i + n * i] -= sh;
    }
    P->format = OR_DENSE;
    if (cplx) { st = lu_decomp_dense_c(n, S); P->vals = 2; P->cmat = S; S = NULL; }
    else {
      P->vals = 1; P->rmat = malloc(sizeof(double) * (cnt ? cnt : 1));
      for (long i = 0; i < cnt; ++i) P->rmat[i] = creal(S[i]);
      st = lu_decomp_dense_r(n, P->rmat);
    }
    free(S); free(Cd); free(Md);
  } else {
    int hb = band_of(K);
    if (shift && C && band_of(C) > hb) hb = band_of(C);
    if (shift && M && band_of(M) > hb) hb = band_of(M);
    long cnt = n * (2L * hb + 1);
    or_cplx *S = malloc(sizeof(or_cplx) * (cnt ? cnt : 1)), *Cd = NULL, *Md = NULL;
    to_band(K, hb, S);
    if (shift) {
      if (C) { Cd = malloc(sizeof(or_cplx) * (cnt ? cnt : 1)); to_band(C, hb, Cd); }
      if (M) { Md = malloc(sizeof(or_cplx) * (cnt ? cnt : 1)); to_band(M, hb, Md); }
      combine(cnt, S, Cd, Md, C != NULL, M != NULL, sh);
      if (C && !M) for (long i = 0; i < n; ++i) S[i + n * hb] += sh * sh;
      if (!C && !M) for (long i = 0; i < n; ++i) S[i + n * hb] -= sh;
    }
    P->format = OR_CDS;
    P->half_band = hb;
    if (cplx) { st = lu_decomp_band_c(n, hb, S); P->vals = 2; P->cband = S; S = NULL; }
    else {
      P->vals = 1; P->rband = malloc(sizeof(double) * (cnt ? cnt : 1));
      for (long i = 0; i < cnt; ++i) P->rband[i] = creal(S[i]);
      st = lu_decomp_band_r(n, hb, P->rband);
    }
    free(S); free(Cd); free(Md);
  }
  return st;
}

/* REAL_PRECON / COMPLEX_PRECON, which_precon 0/1: user_module.f90:1327-1381 and
 * :1465-1520.  The diagonal of K, or with a shift that of K + shift C +
 * shift^2 M (C only: + shift^2; M only: K - shift M; neither: K - shift), each
 * matrix's diagonal taken with its zeros replaced by 1 (real_diagonal). */
int or_real_precon_ext(int which_precon, const or_umat *K, const or_umat *M, const or_umat *C,
                       const double *shift, or_umat **out) {
  if (!K || !out) return OR_EARG;
  or_umat *P = umat_new(0, K->nrows, K->ncols);
  P->which_precon = which_precon;
  int n = K->nrows;
  if (which_precon == 1) {
    P->format = OR_CDS; P->half_band = 0; P->vals = 1;
    P->rband = malloc(sizeof(double) * (n > 0 ? n : 1));
    double *D = P->rband;
    or_real_diagonal(K, D);
    if (shift) {
      double sh = *shift;
      double *dc = malloc(sizeof(double) * (n > 0 ? n : 1)), *dm = malloc(sizeof(double) * (n > 0 ? n : 1));
      if (C) or_real_diagonal(C, dc);
      if (M) or_real_diagonal(M, dm);
      for (int i = 0; i < n; ++i) {
        if (M && C) D[i] = D[i] + sh * dc[i] + (sh * sh) * dm[i];
        else if (C) D[i] = (D[i] + sh * dc[i]) + sh * sh;
        else if (M) D[i] = D[i] - sh * dm[i];
        else D[i] = D[i] - sh;
      }
      free(dc); free(dm);
    }
  } else if (which_precon == 2 || which_precon == 3) {
    int st = lu_precon(which_precon, K, M, C, shift, 0, P);
    if (st != OR_OK) { or_umat_free(P); return st; }
  } else if (which_precon != 0) {
    or_umat_free(P); return OR_EUNSUP;
  }
  *out = P;
  return OR_OK;
}
int or_complex_precon_ext(int which_precon, const or_umat *K, const or_umat *M, const or_umat *C,
                          const double *shift, or_umat **out) {
  if (!K || !out) return OR_EARG;
  or_umat *P = umat_new(0, K->nrows, K->ncols);
  P->which_precon = which_precon;
  int n = K->nrows;
  if (which_precon == 1) {
    P->format = OR_CDS; P->half_band = 0; P->vals = 2;
    P->cband = malloc(sizeof(or_cplx) * (n > 0 ? n : 1));
    or_cplx *D = P->cband;
    or_complex_diagonal(K, D);
    if (shift) {
      or_cplx sh = shift[0] + I * shift[1];
      or_cplx *dc = malloc(sizeof(or_cplx) * (n > 0 ? n : 1)), *dm = malloc(sizeof(or_cplx) * (n > 0 ? n : 1));
      if (C) or_complex_diagonal(C, dc);
      if (M) or_complex_diagonal(M, dm);
      for (int i = 0; i < n; ++i) {
        if (M && C) D[i] = D[i] + sh * dc[i] + (sh * sh) * dm[i];
        else if (C) D[i] = (D[i] + sh * dc[i]) + sh * sh;
        else if (M) D[i] = D[i] - sh * dm[i];
        else D[i] = D[i] - sh;
      }
      free(dc); free(dm);
    }
  } else if (which_precon == 2 || which_precon == 3) {
    int st = lu_precon(which_precon, K, M, C, shift, 1, P);
    if (st != OR_OK) { or_umat_free(P); return st; }
  } else if (which_precon != 0) {
    or_umat_free(P); return OR_EUNSUP;
  }
  *out = P;
  return OR_OK;
}
int or_real_precon(int which_precon, const or_umat *K, const double *shift, or_umat **out) {
  return or_real_precon_ext(which_precon, K, NULL, NULL, shift, out);
}
int or_complex_precon(int which_precon, const or_umat *K, const double *shift, or_umat **out) {
  return or_complex_precon_ext(which_precon, K, NULL, NULL, shift, out);
}

/* ------------------------------------------------------------------------ */
/* type(matrix): M/PP_MATRIX/matrix_module.f90:38-81                        */
/* ------------------------------------------------------------------------ */
int or_matrix_create_ext(const or_umat *K, const or_umat *M, const or_umat *C,
                         const or_umat *P, const double *seed, const double *shift, int cplx,
                         int multishift, or_mat **out) {
  int st = or_matrix_create(K, P, seed, cplx, out);
  if (st != OR_OK) return st;
  if (P && shift) {
    (*out)->shift_invert = 1;
    if (cplx) (*out)->cshift = shift[0] + I * shift[1];
    else (*out)->rshift = shift[0];
  }
  (*out)->M = M; (*out)->C = C;
  (*out)->mass_matrix = M != NULL;
  (*out)->damping_matrix = C != NULL;
  (*out)->block_system = multishift && C != NULL;
  (*out)->multishift = multishift != 0;
  return OR_OK;
}

int or_matrix_create(const or_umat *K, const or_umat *P, const double *seed, int cplx, or_mat **out) {
  if (!K || !out) return OR_EARG;
  or_mat *A = calloc(1, sizeof(or_mat));
  A->K = K; A->P = P;
  if (seed) {
    if (cplx) A->cseed = seed[0] + I * seed[1];
    else A->rseed = seed[0];
  }
  *out = A;
  return OR_OK;
}
int or_matrix_set_poly_eval(or_mat *A, int mode) {
  if (!A || (mode != 0 && mode != 1)) return OR_EARG;
  A->poly_eval = mode;
  return OR_OK;
}
void or_matrix_free(or_mat *A) {
  if (!A) return;
  free(A->ralpha_p); free(A->calpha_p); free(A->ralpha_s); free(A->calpha_s);
  free(A->sigma_s); free(A->sigma); free(A->defl_V); free(A->defl_AV); free(A->defl_E);
  free(A->jac);
  free(A);
}

/* ------------------------------------------------------------------------ */
/* Polynomial preconditioners: matrix_module.f90:851-1019                   */
/* ------------------------------------------------------------------------ */
#define DEF_COMPUTE_ALPHA(NAME, TT)                                                     \
  int NAME(int degree, const TT *H, int ldh, int nh, TT *alpha) {                      \
    if (degree == 0) { alpha[0] = 1.; return OR_OK; }                                  \
    if (ldh < degree + 2 || nh < degree + 1) return OR_EARG;                            \
    int d2 = degree + 2;                                                                \
    TT *r = calloc((size_t)d2 * d2, sizeof(TT));                                        \
    r[0] = 1.;                                                                           \
    for (int i = 1; i <= degree + 1; ++i) {                                             \
      for (int c = 1; c <= degree + 1; ++c) r[i + d2 * c] = r[(i - 1) + d2 * (c - 1)];  \
      for (int j = 0; j <= i - 1; ++j) {                                                \
        TT hji = H[j + (size_t)ldh * (i - 1)];                                          \
        for (int c = 0; c <= degree + 1; ++c) r[i + d2 * c] = r[i + d2 * c] - hji * r[j + d2 * c]; \
      }                                                                                 \
      TT hd = H[i + (size_t)ldh * (i - 1)];                                             \
      for (int c = 0; c <= degree + 1; ++c) r[i + d2 * c] = r[i + d2 * c] / hd;          \
    }                                                                                   \
    for (int c = 1; c <= degree + 1; ++c) alpha[c - 1] = -r[(degree + 1) + d2 * c];     \
    free(r);                                                                            \
    return OR_OK;                                                                       \
  }
/* rcompute_alpha: matrix_module.f90:983-1019 */
DEF_COMPUTE_ALPHA(or_rcompute_alpha, double)
/* ccompute_alpha: matrix_module.f90:1021-1057 */
DEF_COMPUTE_ALPHA(or_ccompute_alpha, or_cplx)

/* The Jacobi matrix's tridiagonal columns (a_i, b_i, c_i) = (J(i-1,i),
 * J(i,i), J(i+1,i)), i = 1..degree+1, kept for the recurrence evaluation */
#define DEF_JCOLS(NAME, TT)                                                             \
  static void NAME(int degree, const TT *J, TT *cols) {                                 \
    int ld = degree + 2;                                                                \
    if (!cols) return;                                                                  \
    for (int i = 1; i <= degree + 1; ++i) {                                             \
      cols[3 * (i - 1)] = i >= 2 ? J[(i - 2) + ld * (i - 1)] : 0;                       \
      cols[3 * (i - 1) + 1] = J[(i - 1) + ld * (i - 1)];                                \
      cols[3 * (i - 1) + 2] = J[i + ld * (i - 1)];                                      \
    }                                                                                   \
  }
DEF_JCOLS(or_jcols_r, double)
DEF_JCOLS(or_jcols_c, or_cplx)

#define DEF_NEUMANN(NAME, TT, CA, JC)                                                   \
  int NAME##_j(int degree, TT center, TT *alpha, TT *cols) {                            \
    int ld = degree + 2;                                                                \
    TT *J = calloc((size_t)ld * (degree + 1), sizeof(TT));                              \
    for (int i = 1; i <= degree + 1; ++i) {                                             \
      J[(i - 1) + ld * (i - 1)] = center;                                               \
      J[i + ld * (i - 1)] = -center;                                                    \
    }                                                                                   \
    int st = CA(degree, J, ld, degree + 1, alpha);                                      \
    JC(degree, J, cols);                                                                \
    free(J);                                                                            \
    return st;                                                                          \
  }                                                                                     \
  int NAME(int degree, TT center, TT *alpha) { return NAME##_j(degree, center, alpha, NULL); }
/* rneumann: matrix_module.f90:851-875; cneumann :877-901 */
DEF_NEUMANN(or_rneumann, double, or_rcompute_alpha, or_jcols_r)
DEF_NEUMANN(or_cneumann, or_cplx, or_ccompute_alpha, or_jcols_c)

#define DEF_CHEBYSHEV(NAME, TT, CA, JC)                                                 \
  int NAME##_j(int degree, const TT foci[2], TT *alpha, TT *cols) {                     \
    TT theta = (foci[0] + foci[1]) / 2.;                                                \
    TT delta = (foci[0] - foci[1]) / 2.;                                                \
    TT sigma = theta / delta;                                                           \
    int ld = degree + 2;                                                                \
    TT *J = calloc((size_t)ld * (degree + 1), sizeof(TT));                              \
    J[0] = theta;                                                                       \
    J[1] = -theta;                                                                      \
    TT rho = 1. / sigma;                                                                \
    for (int i = 2; i <= degree + 1; ++i) {                                             \
      J[(i - 2) + ld * (i - 1)] = -delta * rho / 2.;                                    \
      J[(i - 1) + ld * (i - 1)] = delta * sigma;                                        \
      J[i + ld * (i - 1)] = -delta * sigma + delta * rho / 2.;                          \
      rho = 1. / (2. * sigma - rho);                                                    \
    }                                                                                   \
    int st = CA(degree, J, ld, degree + 1, alpha);                                      \
    JC(degree, J, cols);                                                                \
    free(J);                                                                            \
    return st;                                                                          \
  }                                                                                     \
  int NAME(int degree, const TT foci[2], TT *alpha) { return NAME##_j(degree, foci, alpha, NULL); }
/* rchebyshev: matrix_module.f90:903-941; cchebyshev :943-981 */
DEF_CHEBYSHEV(or_rchebyshev, double, or_rcompute_alpha, or_jcols_r)
DEF_CHEBYSHEV(or_cchebyshev, or_cplx, or_ccompute_alpha, or_jcols_c)

/* ------------------------------------------------------------------------ */
/* QR eigenvalues: dense_la_module.f90:42-83 (CQR_factorization, refine=2), */
/* :192-293 (CQR_eig) and :295-403 (RQR_eig)                               */
/* ------------------------------------------------------------------------ */
static int cqr_factorization(int m, or_cplx *V, int ldv, or_cplx *Q, or_cplx *R) {
  for (int j = 0; j < m; ++j)
    for (int i = 0; i < m; ++i) { Q[i + m * j] = V[i + ldv * j]; R[i + m * j] = 0; }
  for (int j = 0; j < m; ++j) {
    for (int k = 0; k < 2; ++k)
      for (int i = 0; i < j; ++i) {
        or_cplx t = 0;
        for (int q = 0; q < m; ++q) t += conj(Q[q + m * i]) * Q[q + m * j];
        for (int q = 0; q < m; ++q) Q[q + m * j] = Q[q + m * j] - t * Q[q + m * i];
        R[i + m * j] = R[i + m * j] + t;
      }
    double nr = 0;
    for (int q = 0; q < m; ++q) { double a = cabs(Q[q + m * j]); nr += a * a; }
    R[j + m * j] = R[j + m * j] + sqrt(nr);
    if (cabs(R[j + m * j]) > DBL_MIN) {
      for (int q = 0; q < m; ++q) Q[q + m * j] = Q[q + m * j] / R[j + m * j];
    } else {
      return j + 1;
    }
  }
  return 0;
}

static int qr_eig_core_u(int n, or_cplx *V, int real_version, or_cplx *eig, int *converged,
                         or_cplx *U);
static int qr_eig_core(int n, or_cplx *V, int real_version, or_cplx *eig, int *converged) {
  return qr_eig_core_u(n, V, real_version, eig, converged, NULL);
}
/* U (optional): Schur vectors, U = I then U(:,1:m) = U(:,1:m) Q after each step
 * (CQR_eig, dense_la_module.f90:222-260) */
static int qr_eig_core_u(int n, or_cplx *V, int real_version, or_cplx *eig, int *converged,
                         or_cplx *U) {
  int iter = 0, m = n, maxit = real_version ? 100 * n : 10 * n;
  const double tol = DBL_EPSILON;
  or_cplx shift = 0;
  if (U)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) U[i + n * j] = (i == j) ? 1 : 0;
  or_cplx *Q = malloc(sizeof(or_cplx) * n * n), *R = malloc(sizeof(or_cplx) * n * n),
          *RQ = malloc(sizeof(or_cplx) * n * n);
#define VV(i, j) V[(i) + n * (j)]
  if (real_version) {
    for (int i = 0; i < m; ++i) if (cabs(VV(i, i)) > cabs(shift)) shift = VV(i, i);
    shift = shift * (1. + 1. * I);
  } else {
    shift = VV(n - 1, n - 1);
  }
  while (m > 1 && iter < maxit) {
    for (int i = 0; i < m; ++i) VV(i, i) = VV(i, i) - shift;
    int info = cqr_factorization(m, V, n, Q, R);
    if (info > 0) break;
    for (int j = 0; j < m; ++j)
      for (int i = 0; i < m; ++i) {
        or_cplx acc = 0;
        for (int q = 0; q < m; ++q) acc += R[i + m * q] * Q[q + m * j];
        RQ[i + m * j] = acc;
      }
    for (int j = 0; j < m; ++j)
      for (int i = 0; i < m; ++i) VV(i, j) = RQ[i + m * j];
    for (int i = 0; i < m; ++i) VV(i, i) = VV(i, i) + shift;
    if (U) {
      or_cplx *UQ = malloc(sizeof(or_cplx) * n * m);
      for (int j = 0; j < m; ++j)
        for (int i = 0; i < n; ++i) {
          or_cplx acc = 0;
          for (int q = 0; q < m; ++q) acc += U[i + n * q] * Q[q + m * j];
          UQ[i + n * j] = acc;
        }
      memcpy(U, UQ, sizeof(or_cplx) * n * m);
      free(UQ);
    }
    if (cabs(VV(m - 1, m - 2)) < tol * cabs(VV(m - 1, m - 1))) m = m - 1;
    if (real_version) {
      shift = 0;
      for (int i = 0; i < m; ++i) if (cabs(VV(i, i)) > cabs(shift)) shift = VV(i, i);
    } else {
      shift = VV(m - 1, m - 1);
    }
    iter = iter + 1;
  }
  for (int i = 0; i < n; ++i) eig[i] = VV(i, i);
  if (converged) *converged = n - m + 1;
#undef VV
  free(Q); free(R); free(RQ);
  return OR_OK;
}
int or_rqr_eig(const double *H, int ldh, int n, or_cplx *eig, int *converged) {
  or_cplx *V = malloc(sizeof(or_cplx) * n * n);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) V[i + n * j] = H[i + (size_t)ldh * j];
  int st = qr_eig_core(n, V, 1, eig, converged);
  free(V);
  return st;
}
int or_cqr_eig(const or_cplx *H, int ldh, int n, or_cplx *eig, int *converged) {
  or_cplx *V = malloc(sizeof(or_cplx) * n * n);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) V[i + n * j] = H[i + (size_t)ldh * j];
  int st = qr_eig_core(n, V, 0, eig, converged);
  free(V);
  return st;
}

/* filter_ritzval: matrix_module.f90:1059-1077 */
static void filter_ritzval(int n, const or_cplx *rv, int *outlier) {
  or_cplx center = 0;
  for (int i = 0; i < n; ++i) center += rv[i];
  center = center / n;
  double sg = 0;
  for (int i = 0; i < n; ++i) { double a = cabs(rv[i] - center); sg += a * a; }
  sg = sqrt(sg / n);
  for (int i = 0; i < n; ++i) outlier[i] = cabs(rv[i] - center) > 1.5 * sg;
}

/* ranalyse_spectrum: matrix_module.f90:1079-1181 */
int or_ranalyse_spectrum(const double *H, int ldh, int n, double *foci, double *center,
                         double *shift) {
  or_cplx *rv = malloc(sizeof(or_cplx) * n);
  int *out = malloc(sizeof(int) * n);
  or_rqr_eig(H, ldh, n, rv, NULL);
  filter_ritzval(n, rv, out);
  double left = INFINITY, right = -INFINITY, bottom = INFINITY, top = -INFINITY;
  for (int i = 0; i < n; ++i) {
    if (out[i]) continue;
    double re = creal(rv[i]), im = cimag(rv[i]);
    if (re < left) left = re;
    if (re > right) right = re;
    if (im < bottom) bottom = im;
    if (im > top) top = im;
  }
  double center_box = (right + left) / 2.;
  double radius = -INFINITY;
  for (int i = 0; i < n; ++i) if (!out[i]) { double a = cabs(rv[i] - center_box); if (a > radius) radius = a; }
  double center_circle = center_box;
  if (fabs(center_box) / radius < 1) {
    double correction = fabs(center_box) / radius;
    center_circle = center_box / correction;
  }
  double shift_circle = center_box - center_circle;
  double x0 = (right - left) / 2., y0 = (top - bottom) / 2.;
  double a = sqrt(x0 * (x0 + y0)), b = sqrt(y0 * (x0 + y0));
  double center_ellipse = center_box;
  if (fabs(center_box) / a < 1.) {
    double correction = fabs(center_box) / a;
    center_ellipse = center_box / correction;
  }
  double f1, f2;
  if (a > b) {
    double c = sqrt(a * a - b * b);
    f1 = center_ellipse - c; f2 = center_ellipse + c;
  } else {
    double c = 0.15 * center_ellipse;
    f1 = center_ellipse - c; f2 = center_ellipse + c;
  }
  if (foci) { foci[0] = f1; foci[1] = f2; }
  if (center) *center = center_circle;
  if (shift) *shift = shift_circle;
  free(rv); free(out);
  return OR_OK;
}

/* canalyse_spectrum: matrix_module.f90:1183-1282 */
int or_canalyse_spectrum(const or_cplx *H, int ldh, int n, or_cplx *foci, or_cplx *center,
                         or_cplx *shift) {
  or_cplx *rv = malloc(sizeof(or_cplx) * n);
  int *out = malloc(sizeof(int) * n);
  or_cqr_eig(H, ldh, n, rv, NULL);
  filter_ritzval(n, rv, out);
  double left = INFINITY, right = -INFINITY, bottom = INFINITY, top = -INFINITY;
  for (int i = 0; i < n; ++i) {
    if (out[i]) continue;
    double re = creal(rv[i]), im = cimag(rv[i]);
    if (re < left) left = re;
    if (re > right) right = re;
    if (im < bottom) bottom = im;
    if (im > top) top = im;
  }
  or_cplx center_box = ((right + left) + I * (top + bottom)) / 2.;
  double radius = -INFINITY;
  for (int i = 0; i < n; ++i) if (!out[i]) { double a = cabs(rv[i] - center_box); if (a > radius) radius = a; }
  or_cplx center_circle = center_box;
  if (cabs(center_box) / radius < 1) {
    double correction = cabs(center_box) / radius;
    center_circle = center_box / correction;
  }
  or_cplx shift_circle = center_box - center_circle;
  double x0 = (right - left) / 2., y0 = (top - bottom) / 2.;
  double a = sqrt(x0 * (x0 + y0)), b = sqrt(y0 * (x0 + y0));
  or_cplx center_ellipse = center_box;
  double q = pow(creal(center_box) / a, 2) + pow(cimag(center_box) / b, 2);
  if (q < 1.) center_ellipse = center_box / sqrt(q);
  or_cplx f1, f2;
  if (a > b) {
    double c = sqrt(a * a - b * b);
    f1 = center_ellipse - c; f2 = center_ellipse + c;
  } else {
    double c = sqrt(b * b - a * a);
    f1 = center_ellipse - I * c; f2 = center_ellipse + I * c;
  }
  if (foci) { foci[0] = f1; foci[1] = f2; }
  if (center) *center = center_circle;
  if (shift) *shift = shift_circle;
  free(rv); free(out);
  return OR_OK;
}

/* real_preconditioner: matrix_module.f90:551-635 */
int or_real_preconditioner(or_mat *A, int preconditioner, int degree, const double *foci,
                           const double *center, const double *H, int ldh, int nh) {
  A->preconditioner = preconditioner;
  A->degree = (preconditioner == 0) ? 0 : degree;
  free(A->ralpha_p); A->ralpha_p = NULL;
  free(A->jac); A->jac = NULL;
  if (preconditioner == 0) return OR_OK;
  A->ralpha_p = calloc(degree + 1, sizeof(double));
  if (preconditioner == 1) {
    double c;
    if (center) c = *center - A->rseed;
    else if (H) or_ranalyse_spectrum(H, ldh, nh, NULL, &c, NULL);
    else c = 1.;
    A->jac = calloc(3 * (size_t)(degree + 1), sizeof(double));
    return or_rneumann_j(degree, c, A->ralpha_p, A->jac);
  } else if (preconditioner == 2) {
    double f[2];
    if (foci) { f[0] = foci[0] - A->rseed; f[1] = foci[1] - A->rseed; }
    else if (H) or_ranalyse_spectrum(H, ldh, nh, f, NULL, NULL);
    else { f[0] = 0.25; f[1] = 1.75; }
    A->jac = calloc(3 * (size_t)(degree + 1), sizeof(double));
    return or_rchebyshev_j(degree, f, A->ralpha_p, A->jac);
  } else if (preconditioner == 3) {
    if (!H) return OR_EARG;
    return or_rcompute_alpha(degree, H, ldh, nh, A->ralpha_p);
  }
  return OR_EARG;
}
/* complex_preconditioner: matrix_module.f90:637-722 */
int or_complex_preconditioner(or_mat *A, int preconditioner, int degree, const or_cplx *foci,
                              const or_cplx *center, const or_cplx *H, int ldh, int nh) {
  A->preconditioner = preconditioner;
  A->degree = (preconditioner == 0) ? 0 : degree;
  free(A->calpha_p); A->calpha_p = NULL;
  free(A->jac); A->jac = NULL;
  if (preconditioner == 0) return OR_OK;
  A->calpha_p = calloc(degree + 1, sizeof(or_cplx));
  if (preconditioner == 1) {
    or_cplx c;
    if (center) c = *center - A->cseed;
    else if (H) or_canalyse_spectrum(H, ldh, nh, NULL, &c, NULL);
    else c = 1.;
    A->jac = calloc(3 * (size_t)(degree + 1), sizeof(or_cplx));
    return or_cneumann_j(degree, c, A->calpha_p, A->jac);
  } else if (preconditioner == 2) {
    or_cplx f[2];
    if (foci) { f[0] = foci[0] - A->cseed; f[1] = foci[1] - A->cseed; }
    else if (H) or_canalyse_spectrum(H, ldh, nh, f, NULL, NULL);
    else { f[0] = 0.25; f[1] = 1.75; }
    A->jac = calloc(3 * (size_t)(degree + 1), sizeof(or_cplx));
    return or_cchebyshev_j(degree, f, A->calpha_p, A->jac);
  } else if (preconditioner == 3) {
    if (!H) return OR_EARG;
    return or_ccompute_alpha(degree, H, ldh, nh, A->calpha_p);
  }
  return OR_EARG;
}

/* real_ms_parameters: matrix_module.f90:485-549 (no shift-and-invert) */
int or_real_ms_parameters(or_mat *A, int n_sigma, const double *sigma, double *sigma_p) {
  int d = A->degree;
  free(A->ralpha_s); A->ralpha_s = NULL; A->n_sigma = n_sigma;
  free(A->sigma_s); A->sigma_s = calloc(n_sigma > 0 ? n_sigma : 1, sizeof(double));
  free(A->sigma); A->sigma = calloc(n_sigma > 0 ? n_sigma : 1, sizeof(double));
  memcpy(A->sigma, sigma, sizeof(double) * n_sigma);
  if (A->shift_invert) {
    if (A->rshift == A->rseed) return OR_EARG;
    for (int i = 0; i < n_sigma; ++i) if (A->rshift == sigma[i]) return OR_EARG;
  }
  for (int i = 0; i < n_sigma; ++i) {
    double ss = A->shift_invert ? (sigma[i] - A->rseed) / (sigma[i] - A->rshift) : sigma[i] - A->rseed;
    ((double *)A->sigma_s)[i] = ss;
    if (d > 0) {
      if (!A->ralpha_s) A->ralpha_s = calloc((size_t)(d + 1) * n_sigma, sizeof(double));
      double *as = A->ralpha_s + (size_t)(d + 1) * i;
      as[d] = A->ralpha_p[d];
      for (int k = d - 1; k >= 0; --k) as[k] = A->ralpha_p[k] + ss * as[k + 1];
      sigma_p[i] = ss * as[0];
    } else sigma_p[i] = ss;
  }
  return OR_OK;
}
/* complex_ms_parameters: matrix_module.f90:402-483 */
int or_complex_ms_parameters(or_mat *A, int n_sigma, const or_cplx *sigma, or_cplx *sigma_p) {
  int d = A->degree;
  free(A->calpha_s); A->calpha_s = NULL; A->n_sigma = n_sigma;
  free(A->sigma_s); A->sigma_s = calloc(n_sigma > 0 ? n_sigma : 1, sizeof(or_cplx));
  free(A->sigma); A->sigma = calloc(n_sigma > 0 ? n_sigma : 1, sizeof(or_cplx));
  memcpy(A->sigma, sigma, sizeof(or_cplx) * n_sigma);
  if (A->shift_invert) {
    if (A->cshift == A->cseed) return OR_EARG;
    for (int i = 0; i < n_sigma; ++i) if (A->cshift == sigma[i]) return OR_EARG;
  }
  for (int i = 0; i < n_sigma; ++i) {
    or_cplx ss = A->shift_invert ? (sigma[i] - A->cseed) / (sigma[i] - A->cshift) : sigma[i] - A->cseed;
    ((or_cplx *)A->sigma_s)[i] = ss;
    if (d > 0) {
      if (!A->calpha_s) A->calpha_s = calloc((size_t)(d + 1) * n_sigma, sizeof(or_cplx));
      or_cplx *as = A->calpha_s + (size_t)(d + 1) * i;
      as[d] = A->calpha_p[d];
      for (int k = d - 1; k >= 0; --k) as[k] = A->calpha_p[k] + ss * as[k + 1];
      sigma_p[i] = ss * as[0];
    } else sigma_p[i] = ss;
  }
  return OR_OK;
}

/* ------------------------------------------------------------------------ */
/* Recycling helpers (real): dense_la_module.f90:84-124 (RQR_factorization, */
/* refine = 2), :159-190 (RQR_solve), :531-603 (RSI_power); ritz_module.f90 */
/* :66-96 (global_RQR_factorization), :100-160 (rcompute_U0) and :497-520   */
/* (the omega ordering of RIDRS_RITZ).                                      */
/* ------------------------------------------------------------------------ */
/* Q(m x n), R(n x n) column-major.  Returns 0, or the 1-based column that was
 * found dependent (Q and R are then partial, as in the reference). */
static int or_rqr_fact(int m, int n, const double *V, int ldv, double *Q, double *R) {
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) Q[i + (size_t)m * j] = V[i + (size_t)ldv * j];
  for (int i = 0; i < n * n; ++i) R[i] = 0;
  for (int j = 0; j < n; ++j) {
    double *qj = Q + (size_t)m * j;
    for (int k = 0; k < 2; ++k)
      for (int i = 0; i < j; ++i) {
        const double *qi = Q + (size_t)m * i;
        double t = 0;
        for (int q = 0; q < m; ++q) t += qi[q] * qj[q];
        for (int q = 0; q < m; ++q) qj[q] = qj[q] - t * qi[q];
        R[i + n * j] = R[i + n * j] + t;
      }
    double nr = 0;
    for (int q = 0; q < m; ++q) nr += qj[q] * qj[q];
    R[j + n * j] = sqrt(nr);
    if (R[j + n * j] > DBL_MIN) {
      for (int q = 0; q < m; ++q) qj[q] = qj[q] / R[j + n * j];
    } else {
      return j + 1;
    }
  }
  return 0;
}

/* X(n x s) = R^-1 Q^T B with Q(m x n), B(m x s) */
static void or_rqr_solve(int m, int n, int s, const double *Q, const double *R, const double *B,
                         double *X) {
  for (int c = 0; c < s; ++c)
    for (int i = 0; i < n; ++i) {
      double t = 0;
      for (int q = 0; q < m; ++q) t += Q[q + (size_t)m * i] * B[q + (size_t)m * c];
      X[i + (size_t)n * c] = t;
    }
  for (int j = n - 1; j >= 0; --j)
    for (int c = 0; c < s; ++c) {
      X[j + (size_t)n * c] = X[j + (size_t)n * c] / R[j + n * j];
      for (int i = 0; i < j; ++i) X[i + (size_t)n * c] = X[i + (size_t)n * c] - R[i + n * j] * X[j + (size_t)n * c];
    }
}

/* RSI_power: s Schur vectors of H(1:n,1:n) nearest `shift` by block
 * shift-and-invert power iteration.  The reference starts from
 * RANDOM_NUMBER; here the start block is or_uniform(seed, i + n*j). */
int or_rsi_power(const double *H, int ldh, int n, int s, double shift, uint64_t seed,
                 double *vec) {
  if (s < 1 || n < s) return OR_EARG;
  double *A = calloc((size_t)n * n, sizeof(double)), *Q = malloc(sizeof(double) * n * n),
         *R = malloc(sizeof(double) * n * n), *sv = malloc(sizeof(double) * n * s),
         *Qs = malloc(sizeof(double) * n * s), *Rs = malloc(sizeof(double) * s * s);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) A[i + (size_t)n * j] = H[i + (size_t)ldh * j];
  for (int i = 0; i < n; ++i) A[i + (size_t)n * i] = A[i + (size_t)n * i] - shift;
  or_rqr_fact(n, n, A, n, Q, R);
  for (long k = 0; k < (long)n * s; ++k) sv[k] = or_uniform(seed, (uint64_t)k);
  or_rqr_fact(n, s, sv, n, Qs, Rs);
  double trace0 = 0;
  for (int i = 0; i < s; ++i) trace0 += Rs[i + s * i];
  double trace_old = trace0, err = 1;
  int iter = 0;
  while (err > 1e-3 && iter < 1000) {
    iter = iter + 1;
    or_rqr_solve(n, n, s, Q, R, Qs, sv);
    or_rqr_fact(n, s, sv, n, Qs, Rs);
    double trace = 0;
    for (int i = 0; i < s; ++i) trace += Rs[i + s * i];
    err = fabs(trace - trace_old) / trace0;
    trace_old = trace;
  }
  memcpy(vec, Qs, sizeof(double) * n * s);
  free(A); free(Q); free(R); free(sv); free(Qs); free(Rs);
  return OR_OK;
}

/* rcompute_U0: rebuild the Krylov basis v_1 = b, v_{i+1} = (A v_i -
 * sum_{l=max(1,i-s)}^{i} v_l H(l,i)) / H(i+1,i) from the Hessenberg matrix
 * H(ldh, >= nritz) and accumulate U0(:,j) = sum_i eigvec(i,j) v_i.  With
 * resnrm (length ns) the columns are normalised and the Ritz residual norms
 * returned.  M: optional preconditioner (A*(v/M)). */
int or_rcompute_U0(const or_mat *A, const or_mat *M, int n, const double *H, int ldh, int nritz,
                   const double *eigvec, int ns, const double *b, double *U0, double *resnrm) {
  const int s = ns;
  double *W = calloc((size_t)n * (s + 1), sizeof(double)), *v = malloc(sizeof(double) * n),
         *t = malloc(sizeof(double) * n), *u = malloc(sizeof(double) * n);
  int *ind = calloc(nritz + 1, sizeof(int));
  for (long q = 0; q < (long)n * s; ++q) U0[q] = 0;
  memcpy(v, b, sizeof(double) * n);
  int k = 0;
  for (int i = 1; i <= nritz; ++i) {
    k = k + 1;
    if (k > s + 1) k = 1;
    ind[i] = k;
    memcpy(W + (size_t)n * (k - 1), v, sizeof(double) * n);
    for (int j = 0; j < s; ++j) {
      double e = eigvec[(i - 1) + (size_t)nritz * j];
      double *uj = U0 + (size_t)n * j;
      for (int q = 0; q < n; ++q) uj[q] = uj[q] + e * v[q];
    }
    int low = i - s > 1 ? i - s : 1;
    if (M) {
      or_precon_r(M, n, v, u);
      or_matvec_r(A, n, u, t);
    } else {
      or_matvec_r(A, n, v, t);
    }
    double hd = H[i + (size_t)ldh * (i - 1)];
    for (int q = 0; q < n; ++q) {
      double acc = 0;
      for (int l = low; l <= i; ++l) acc += W[q + (size_t)n * (ind[l] - 1)] * H[(l - 1) + (size_t)ldh * (i - 1)];
      v[q] = (t[q] - acc) / hd;
    }
  }
  if (resnrm) {
    double nv = or_norm_r(n, v);
    for (int j = 0; j < s; ++j) {
      double *uj = U0 + (size_t)n * j;
      double nrm = or_norm_r(n, uj);
      for (int q = 0; q < n; ++q) uj[q] = uj[q] / nrm;
      resnrm[j] = nv * fabs(H[nritz + (size_t)ldh * (nritz - 1)]) *
                  fabs(eigvec[(nritz - 1) + (size_t)nritz * j]) / nrm;
    }
  }
  free(W); free(v); free(t); free(u); free(ind);
  return OR_OK;
}

/* global_RQR_factorization: modified Gram-Schmidt with global inner products.
 * Q(n x s) may alias V.  R(s x s) optional.  OR_EARG: dependent columns. */
int or_rglobal_qr(int n, int s, const double *V, double *Q, double *R) {
  if (Q != V) memcpy(Q, V, sizeof(double) * n * s);
  double *Rl = calloc((size_t)s * s, sizeof(double));
  int st = OR_OK;
  for (int j = 0; j < s && st == OR_OK; ++j) {
    double *qj = Q + (size_t)n * j;
    for (int i = 0; i < j; ++i) {
      const double *qi = Q + (size_t)n * i;
      double r = 0;
      for (int q = 0; q < n; ++q) r += qi[q] * qj[q];
      Rl[i + s * j] = r;
      for (int q = 0; q < n; ++q) qj[q] = qj[q] - r * qi[q];
    }
    Rl[j + s * j] = or_norm_r(n, qj);
    if (Rl[j + s * j] > DBL_MIN) {
      for (int q = 0; q < n; ++q) qj[q] = qj[q] / Rl[j + s * j];
    } else {
      st = OR_EARG;
    }
  }
  if (R) memcpy(R, Rl, sizeof(double) * s * s);
  free(Rl);
  return st;
}

/* omega = 1/Re(Ritz values of Hf(1:n_omega,1:n_omega)) (|Re| < eps -> 1),
 * ordered greedily: step i takes the omega whose Ritz value maximises |p|
 * over positions i..n_omega, then p *= 1 - Re(ritz) omega(i). */
int or_ritz_omega(const double *Hf, int ldh, int n_omega, double *omega) {
  if (n_omega < 1) return OR_EARG;
  or_cplx *rv = malloc(sizeof(or_cplx) * n_omega);
  double *p = malloc(sizeof(double) * n_omega);
  int converged = 0;
  or_rqr_eig(Hf, ldh, n_omega, rv, &converged);
  for (int i = 0; i < n_omega; ++i) {
    double w = creal(rv[i]);
    if (fabs(w) < DBL_EPSILON) w = 1.;
    omega[i] = 1. / w;
    p[i] = 1.;
  }
  for (int i = 0; i < n_omega; ++i) {
    int mp = i;
    for (int k = i + 1; k < n_omega; ++k)
      if (fabs(p[k]) > fabs(p[mp])) mp = k;
    double mo = omega[mp];
    omega[mp] = omega[i];
    omega[i] = mo;
    for (int k = 0; k < n_omega; ++k) p[k] = p[k] * (1. - creal(rv[k]) * omega[i]);
  }
  free(rv); free(p);
  return OR_OK;
}

/* complex versions: CIDRS_RITZ's omega (ritz_module.f90:335-358, 1/ritz,
 * complex p), ccompute_U0 (:162-223), global_CQR_factorization (:36-64) */
int or_ritz_omega_c(const or_cplx *Hf, int ldh, int n_omega, or_cplx *omega) {
  if (n_omega < 1) return OR_EARG;
  or_cplx *rv = malloc(sizeof(or_cplx) * n_omega), *p = malloc(sizeof(or_cplx) * n_omega);
  int converged = 0;
  or_cqr_eig(Hf, ldh, n_omega, rv, &converged);
  for (int i = 0; i < n_omega; ++i) {
    or_cplx w = rv[i];
    if (cabs(w) < DBL_EPSILON) w = 1.;
    omega[i] = 1. / w;
    p[i] = 1.;
  }
  for (int i = 0; i < n_omega; ++i) {
    int mp = i;
    for (int k = i + 1; k < n_omega; ++k)
      if (cabs(p[k]) > cabs(p[mp])) mp = k;
    or_cplx mo = omega[mp];
    omega[mp] = omega[i];
    omega[i] = mo;
    for (int k = 0; k < n_omega; ++k) p[k] = p[k] * (1. - rv[k] * omega[i]);
  }
  free(rv); free(p);
  return OR_OK;
}

int or_ccompute_U0(const or_mat *A, const or_mat *M, int n, const or_cplx *H, int ldh, int nritz,
                   const or_cplx *eigvec, int ns, const or_cplx *b, or_cplx *U0, double *resnrm) {
  const int s = ns;
  or_cplx *W = calloc((size_t)n * (s + 1), sizeof(or_cplx)), *v = malloc(sizeof(or_cplx) * n),
          *t = malloc(sizeof(or_cplx) * n), *u = malloc(sizeof(or_cplx) * n);
  int *ind = calloc(nritz + 1, sizeof(int));
  for (long q = 0; q < (long)n * s; ++q) U0[q] = 0;
  memcpy(v, b, sizeof(or_cplx) * n);
  int k = 0;
  for (int i = 1; i <= nritz; ++i) {
    k = k + 1;
    if (k > s + 1) k = 1;
    ind[i] = k;
    memcpy(W + (size_t)n * (k - 1), v, sizeof(or_cplx) * n);
    for (int j = 0; j < s; ++j) {
      or_cplx e = eigvec[(i - 1) + (size_t)nritz * j];
      or_cplx *uj = U0 + (size_t)n * j;
      for (int q = 0; q < n; ++q) uj[q] = uj[q] + e * v[q];
    }
    int low = i - s > 1 ? i - s : 1;
    if (M) {
      or_precon_c(M, n, v, u);
      or_matvec_c(A, n, u, t);
    } else {
      or_matvec_c(A, n, v, t);
    }
    or_cplx hd = H[i + (size_t)ldh * (i - 1)];
    for (int q = 0; q < n; ++q) {
      or_cplx acc = 0;
      for (int l = low; l <= i; ++l) acc += W[q + (size_t)n * (ind[l] - 1)] * H[(l - 1) + (size_t)ldh * (i - 1)];
      v[q] = (t[q] - acc) / hd;
    }
  }
  if (resnrm) {
    double nv = or_norm_c(n, v);
    for (int j = 0; j < s; ++j) {
      or_cplx *uj = U0 + (size_t)n * j;
      double nrm = or_norm_c(n, uj);
      for (int q = 0; q < n; ++q) uj[q] = uj[q] / nrm;
      resnrm[j] = nv * cabs(H[nritz + (size_t)ldh * (nritz - 1)]) *
                  cabs(eigvec[(nritz - 1) + (size_t)nritz * j]) / nrm;
    }
  }
  free(W); free(v); free(t); free(u); free(ind);
  return OR_OK;
}

int or_cglobal_qr(int n, int s, const or_cplx *V, or_cplx *Q, or_cplx *R) {
  if (Q != V) memcpy(Q, V, sizeof(or_cplx) * n * s);
  or_cplx *Rl = calloc((size_t)s * s, sizeof(or_cplx));
  int st = OR_OK;
  for (int j = 0; j < s && st == OR_OK; ++j) {
    or_cplx *qj = Q + (size_t)n * j;
    for (int i = 0; i < j; ++i) {
      const or_cplx *qi = Q + (size_t)n * i;
      or_cplx r = 0;
      for (int q = 0; q < n; ++q) r += conj(qi[q]) * qj[q];
      Rl[i + s * j] = r;
      for (int q = 0; q < n; ++q) qj[q] = qj[q] - r * qi[q];
    }
    Rl[j + s * j] = or_norm_c(n, qj);
    if (cabs(Rl[j + s * j]) > DBL_MIN) {
      for (int q = 0; q < n; ++q) qj[q] = qj[q] / Rl[j + s * j];
    } else {
      st = OR_EARG;
    }
  }
  if (R) memcpy(R, Rl, sizeof(or_cplx) * s * s);
  free(Rl);
  return st;
}

/* CIDRS_RITZ (ritz_module.f90:268-387): H, omega and U0 (Schur vectors) */
int or_idrs_ritz_cx(const or_mat *A, int n, const or_cplx *b, int s, const or_opts *o,
                    or_cplx *x, int *nritz, or_cplx *omega, int n_omega, or_cplx *U0, int dimU0) {
  double tol = (o && o->tolerance) ? *o->tolerance : (double)1e-6f;
  if (tol < 0) return OR_EARG;
  int maxit = (2 * n < 1000) ? 2 * n : 1000;
  if (o && o->maximum_iterations) maxit = *o->maximum_iterations;
  int method = (o && o->variant) ? *o->variant : 1;
  or_cplx *Hf = calloc((size_t)(maxit + 1) * maxit, sizeof(or_cplx));
  double *resnrm = calloc(maxit + 1, sizeof(double));
  or_cplx *xs = calloc(n, sizeof(or_cplx));
  if (o && o->x0) memcpy(xs, o->x0, sizeof(or_cplx) * n);
  int conv = -1, iter = 0; double relnrm = 1;
  or_opts io; memset(&io, 0, sizeof io);
  io.M1 = o ? o->M1 : NULL;
  io.tolerance = &tol; io.maximum_iterations = &maxit; io.variant = &method;
  io.flag = &conv; io.relres = &relnrm; io.iterations = &iter; io.x0 = xs;
  io.resvec = resnrm; io.resvec_len = maxit + 1;
  io.H = Hf; io.H_rows = maxit + 1; io.H_cols = maxit;
  io.PT = o ? o->PT : NULL; io.p_seed = o ? o->p_seed : 0;
  int st = or_idrs_c(A, n, b, s, &io, x);
  if (st != OR_OK) { free(Hf); free(resnrm); free(xs); return st; }
  const int nr = (iter / (s + 1)) * s + iter % (s + 1);
  if (nritz) *nritz = nr;
  if (o && o->flag) *o->flag = conv;
  if (o && o->relres) *o->relres = relnrm;
  if (o && o->iterations) *o->iterations = iter;
  if (o && o->H) {
    or_cplx *H = o->H;
    for (int j = 0; j < o->H_cols; ++j)
      for (int i = 0; i < o->H_rows; ++i) H[i + (size_t)o->H_rows * j] = Hf[i + (size_t)(maxit + 1) * j];
  }
  if (omega && n_omega > 0) {
    if (nr < n_omega) st = OR_EARG;
    else or_ritz_omega_c(Hf, maxit + 1, n_omega, omega);
  }
  if (st == OR_OK && U0 && dimU0 > 0) {
    if (nr < dimU0) st = OR_EARG;
    else {
      or_cplx *Vs = malloc(sizeof(or_cplx) * nr * nr), *ev = malloc(sizeof(or_cplx) * nr),
              *V = malloc(sizeof(or_cplx) * nr * nr), *U = malloc(sizeof(or_cplx) * n * dimU0);
      double *resval = malloc(sizeof(double) * dimU0);
      for (int j = 0; j < nr; ++j)
        for (int i = 0; i < nr; ++i) V[i + nr * j] = Hf[i + (size_t)(maxit + 1) * j];
      int cv = 0;
      qr_eig_core_u(nr, V, 0, ev, &cv, Vs);
      const or_mat *M = o ? o->M1 : NULL;
      or_ccompute_U0(A, M, n, Hf, maxit + 1, nr, Vs, dimU0, b, U, resval);
      if (M)
        for (int j = 0; j < dimU0; ++j) {
          or_precon_c(M, n, U + (size_t)n * j, U0);
          memcpy(U + (size_t)n * j, U0, sizeof(or_cplx) * n);
        }
      st = or_cglobal_qr(n, dimU0, U, U0, NULL);
      free(Vs); free(ev); free(V); free(U); free(resval);
    }
  }
  free(Hf); free(resnrm); free(xs);
  return st;
}

/* ------------------------------------------------------------------------ */
/* IDRS_RITZ: M/IDRS/ritz_module.f90:389-556 with its H, omega and U0       */
/* outputs (U0: SI_power Schur vectors of Hf, compute_U0, global QR).       */
/* ------------------------------------------------------------------------ */
int or_idrs_ritz_r(const or_mat *A, int n, const double *b, int s, const or_opts *o, double *x,
                   int *nritz) {
  return or_idrs_ritz_rx(A, n, b, s, o, x, nritz, NULL, 0, NULL, 0, 0);
}

int or_idrs_ritz_rx(const or_mat *A, int n, const double *b, int s, const or_opts *o, double *x,
                    int *nritz, double *omega, int n_omega, double *U0, int dimU0,
                    uint64_t si_seed) {
  double tol = (o && o->tolerance) ? *o->tolerance : (double)1e-6f;
  if (tol < 0) return OR_EARG;
  int maxit = (2 * n < 1000) ? 2 * n : 1000;
  if (o && o->maximum_iterations) maxit = *o->maximum_iterations;
  int method = (o && o->variant) ? *o->variant : 1;
  double *Hf = calloc((size_t)(maxit + 1) * maxit, sizeof(double));
  double *resnrm = calloc(maxit + 1, sizeof(double));
  double *xs = calloc(n, sizeof(double));
  if (o && o->x0) memcpy(xs, o->x0, sizeof(double) * n);
  int conv = -1, iter = 0; double relnrm = 1;
  or_opts io; memset(&io, 0, sizeof io);
  io.M1 = o ? o->M1 : NULL;
  io.tolerance = &tol; io.maximum_iterations = &maxit; io.variant = &method;
  io.flag = &conv; io.relres = &relnrm; io.iterations = &iter; io.x0 = xs;
  io.resvec = resnrm; io.resvec_len = maxit + 1;
  io.H = Hf; io.H_rows = maxit + 1; io.H_cols = maxit;
  io.PT = o ? o->PT : NULL; io.p_seed = o ? o->p_seed : 0;
  int st = or_idrs_r(A, n, b, s, &io, x);
  if (st != OR_OK) { free(Hf); free(resnrm); free(xs); return st; }
  const int nr = (iter / (s + 1)) * s + iter % (s + 1);
  if (nritz) *nritz = nr;
  if (o && o->flag) *o->flag = conv;
  if (o && o->relres) *o->relres = relnrm;
  if (o && o->iterations) *o->iterations = iter;
  if (o && o->resvec) memcpy(o->resvec, resnrm, sizeof(double) * (maxit + 1));
  if (o && o->H) {
    if ((long)o->H_rows * o->H_cols > (long)(maxit + 1) * maxit) { free(Hf); free(resnrm); free(xs); return OR_EARG; }
    double *H = o->H;
    for (int j = 0; j < o->H_cols; ++j)
      for (int i = 0; i < o->H_rows; ++i) H[i + (size_t)o->H_rows * j] = Hf[i + (size_t)(maxit + 1) * j];
  }
  if (omega && n_omega > 0) {
    if (nr < n_omega) st = OR_EARG;  /* "Too many parameters omega requested" */
    else or_ritz_omega(Hf, maxit + 1, n_omega, omega);
  }
  if (st == OR_OK && U0 && dimU0 > 0) {
    if (nr < dimU0) st = OR_EARG;    /* "Recycle space is too large" */
    else {
      double *vec = malloc(sizeof(double) * nr * dimU0), *U = malloc(sizeof(double) * n * dimU0),
             *resval = malloc(sizeof(double) * dimU0);
      or_rsi_power(Hf, maxit + 1, nr, dimU0, 0.0, si_seed ? si_seed : 2, vec);
      const or_mat *M = o ? o->M1 : NULL;
      or_rcompute_U0(A, M, n, Hf, maxit + 1, nr, vec, dimU0, b, U, resval);
      if (M)
        for (int j = 0; j < dimU0; ++j) {
          or_precon_r(M, n, U + (size_t)n * j, U0);
          memcpy(U + (size_t)n * j, U0, sizeof(double) * n);
        }
      st = or_rglobal_qr(n, dimU0, U, U0, NULL);
      free(vec); free(U); free(resval);
    }
  }
  free(Hf); free(resnrm); free(xs);
  return st;
}

/* ------------------------------------------------------------------------ */
/* PP_IDRS (real, single rhs): M/PP_IDRS/pp_idrs_module.f90:118-162 with    */
/* real_matrix.inc, real_preconditioner.inc:10-34 and run_idrs.inc:9-60.    */
/* ------------------------------------------------------------------------ */
static double or_wtime(void) {
#ifdef _OPENMP
  return omp_get_wtime();
#else
  return 0.0;
#endif
}

/* real_preconditioner.inc:10-34: the initial IDRS_RITZ solve (which also
 * yields x0 and, with n_omega > 0, the omega parameters) and the polynomial
 * preconditioner.  *omega is allocated when the initial solve ran. */
static int or_pp_setup_r(or_mat *A, int n, const double *b, or_pp_args *a, double *x0,
                         double **omega) {
  int preconditioner = a->degree == 0 ? 0 : a->preconditioner;
  int estimate = 1;
  if (preconditioner == 0) estimate = 0;
  if (preconditioner == 1 && a->center) estimate = 0;
  if (preconditioner == 2 && a->foci) estimate = 0;
  int initial = estimate || a->n_omega > 0;
  a->ritz_iterations = 0; a->nritz_used = 0;
  *omega = NULL;
  int st = OR_OK;
  double *H = NULL;
  int ldh = 0;
  if (initial) {
    int ini_iter = a->n_ritz + a->n_ritz / a->s;
    ldh = ini_iter + 1;
    H = calloc((size_t)ldh * ini_iter, sizeof(double));
    *omega = calloc(a->n_omega > 0 ? a->n_omega : 1, sizeof(double));
    int flag = -1, iter = 0, one = 1, nritz = 0; double relres = 1;
    or_opts o; memset(&o, 0, sizeof o);
    o.tolerance = &a->tol; o.maximum_iterations = &ini_iter; o.variant = &one;
    o.flag = &flag; o.relres = &relres; o.iterations = &iter;
    o.H = H; o.H_rows = ldh; o.H_cols = ini_iter; o.p_seed = a->p_seed;
    st = or_idrs_ritz_rx(A, n, b, a->s, &o, x0, &nritz, *omega, a->n_omega, NULL, 0, 0);
    a->ritz_iterations = iter;
    a->nritz_used = (iter / (a->s + 1)) * a->s + iter % (a->s + 1);
    for (int i = 0; i < a->n_omega && i < 64; ++i) a->omega_used[i] = (*omega)[i];
  }
  if (st == OR_OK) {
    if (estimate) {
      or_ranalyse_spectrum(H, ldh, a->nritz_used, a->foci_used, &a->center_used, NULL);
      st = or_real_preconditioner(A, preconditioner, a->degree, NULL, NULL, H, ldh, a->nritz_used);
    } else {
      double f[2] = {0.15, 1.85}, c = 1.;
      if (a->foci) { f[0] = a->foci[0]; f[1] = a->foci[1]; }
      if (a->center) c = *a->center;
      a->foci_used[0] = f[0]; a->foci_used[1] = f[1]; a->center_used = c;
      st = or_real_preconditioner(A, preconditioner, a->degree, f, &c, NULL, 0, 0);
    }
  }
  if (st == OR_OK)
    for (int i = 0; i <= A->degree && i < 64; ++i) a->alpha_p[i] = A->ralpha_p ? A->ralpha_p[i] : 1.;
  A->poly_eval = a->poly_eval;
  free(H);
  return st;
}

/* One solve of run_idrs.inc:9-60 / run_mr_idrs.inc:15-72: y from the
 * selected method with x0, U0 and omega, x = scaleback(A, b, y) and the
 * relative residual of the original system. */
static int or_pp_solve_r(const or_mat *A, const or_umat *K, int n, const double *b,
                         const or_pp_args *a, const double *x0, const double *U0,
                         const double *omega, double *y, double *x, int *flag, int *iter,
                         double *relres, double *relres_original) {
  or_opts o; memset(&o, 0, sizeof o);
  double tol = a->tol; int maxit = a->maxit, in_s = a->in_s, in_it = a->in_it;
  double in_tol = a->in_tol;
  o.tolerance = &tol; o.maximum_iterations = &maxit; o.x0 = x0; o.p_seed = a->p_seed;
  o.flag = flag; o.relres = relres; o.iterations = iter;
  if (omega && a->n_omega > 0) { o.omega = omega; o.n_omega = a->n_omega; }
  int variant = a->method == 2 ? 2 : 1, st;
  if (a->method == 0) {
    o.inner_s = &in_s; o.inner_tolerance = &in_tol; o.inner_iterations = &in_it;
    st = or_qmridr_r(A, n, b, a->s, &o, y);
  } else {
    o.variant = &variant;
    o.U0 = U0;
    st = or_idrs_r(A, n, b, a->s, &o, y);
  }
  if (st != OR_OK) return st;
  double *t = malloc(sizeof(double) * n);
  or_scaleback_r(A, n, b, y, x);
  or_user_mv_r(K, x, t);
  for (int i = 0; i < n; ++i) t[i] = b[i] - t[i];
  *relres_original = or_norm_r(n, t) / or_norm_r(n, b);
  free(t);
  return OR_OK;
}

int or_pp_idrs_r(const or_umat *K, const or_umat *P, int n, const double *b, or_pp_args *a,
                 double *x) {
  double t0 = or_wtime();
  or_mat *A;
  or_matrix_create(K, P, NULL, 0, &A);
  double *x0 = calloc(n, sizeof(double)), *y = malloc(sizeof(double) * n), *omega = NULL;
  int st = or_pp_setup_r(A, n, b, a, x0, &omega);
  double t1 = or_wtime();
  a->seconds_setup = t1 - t0;
  if (st == OR_OK)
    st = or_pp_solve_r(A, K, n, b, a, x0, NULL, omega, y, x, &a->flag, &a->iterations,
                       &a->relres_solver, &a->relres_original);
  a->seconds_solve = or_wtime() - t1;
  free(x0); free(y); free(omega);
  or_matrix_free(A);
  return st;
}

int or_pp_mr_idrs_r(const or_umat *K, const or_umat *P, int n, int nrhs, const double *b_all,
                    or_pp_args *a, double *x_all) {
  if (nrhs < 1) return OR_EARG;
  double t0 = or_wtime();
  or_mat *A;
  or_matrix_create(K, P, NULL, 0, &A);
  double *x0 = calloc(n, sizeof(double)), *y = malloc(sizeof(double) * n), *omega = NULL,
         *U0 = NULL;
  int st = or_pp_setup_r(A, n, b_all, a, x0, &omega);
  a->recycle_flag = 0; a->recycle_iterations = 0; a->recycle_relres = 0;
  if (st == OR_OK && a->recycle) {  /* recycle.inc */
    U0 = malloc(sizeof(double) * n * a->s);
    int one = 1, nritz = 0, maxit = a->maxit;
    double tol = a->tol;
    or_opts o; memset(&o, 0, sizeof o);
    o.tolerance = &tol; o.maximum_iterations = &maxit; o.variant = &one;
    o.flag = &a->recycle_flag; o.relres = &a->recycle_relres; o.iterations = &a->recycle_iterations;
    o.p_seed = a->p_seed;
    st = or_idrs_ritz_rx(A, n, b_all, a->s, &o, x0, &nritz, NULL, 0, U0, a->s, a->si_seed);
  }
  double t1 = or_wtime();
  a->seconds_setup = t1 - t0;
  for (int irhs = 0; irhs < nrhs && st == OR_OK; ++irhs) {
    const double *b = b_all + (size_t)n * irhs;
    int flag = -1, iter = 0; double rel = 1, relo = 1;
    st = or_pp_solve_r(A, K, n, b, a, x0, U0, omega, y, x_all + (size_t)n * irhs, &flag, &iter,
                       &rel, &relo);
    memcpy(x0, y, sizeof(double) * n);  /* warm start: the preconditioned solution */
    if (a->flags) a->flags[irhs] = flag;
    if (a->iters) a->iters[irhs] = iter;
    if (a->relres_solver_all) a->relres_solver_all[irhs] = rel;
    if (a->relres_original_all) a->relres_original_all[irhs] = relo;
    a->flag = flag; a->iterations = iter; a->relres_solver = rel; a->relres_original = relo;
  }
  a->seconds_solve = or_wtime() - t1;
  free(x0); free(y); free(omega); free(U0);
  or_matrix_free(A);
  return st;
}

/* ------------------------------------------------------------------------ */
/* Adjoint helpers (new; no counterpart in the reference)                   */
/* ------------------------------------------------------------------------ */
void or_sparse_outer_grad(const or_umat *K, const double *lambda, const double *x, double *g) {
  long n = K->nrows;
  _Pragma("omp parallel for schedule(static) if(n > 32768)")
  for (long i = 0; i < n; ++i)
    for (int j = K->row_ptr[i]; j < K->row_ptr[i + 1]; ++j) g[j] = -lambda[i] * x[K->col_ind[j]];
}
int or_crs_transpose(const or_umat *K, or_umat **out) {
  if (!K || K->format != OR_CRS || !out) return OR_EARG;
  int n = K->nrows, m = K->ncols, nnz = K->row_ptr[n];
  or_umat *A = umat_new(OR_CRS, m, n);
  A->nnz = nnz; A->vals = K->vals;
  A->row_ptr = calloc(m + 1, sizeof(int));
  A->col_ind = malloc(sizeof(int) * (nnz > 0 ? nnz : 1));
  if (K->vals == 1) A->rval = malloc(sizeof(double) * (nnz > 0 ? nnz : 1));
  if (K->vals == 2) A->cval = malloc(sizeof(or_cplx) * (nnz > 0 ? nnz : 1));
  for (int k = 0; k < nnz; ++k) A->row_ptr[K->col_ind[k] + 1]++;
  for (int j = 0; j < m; ++j) A->row_ptr[j + 1] += A->row_ptr[j];
  int *pos = malloc(sizeof(int) * (m > 0 ? m : 1));
  memcpy(pos, A->row_ptr, sizeof(int) * m);
  for (int i = 0; i < n; ++i)
    for (int k = K->row_ptr[i]; k < K->row_ptr[i + 1]; ++k) {
      int j = K->col_ind[k], p = pos[j]++;
      A->col_ind[p] = i;
      if (K->vals == 1) A->rval[p] = K->rval[k];
      if (K->vals == 2) A->cval[p] = K->cval[k];
    }
  free(pos);
  *out = A;
  return OR_OK;
}
