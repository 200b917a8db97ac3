// matrix.cuh -- device user_matrix, the composed operator and its SpMV chain.
//
// user_matrix (M/PP_MATRIX/user_module.f90:134-167) lives in HBM in one of
// the formats DENSE, CRS, COO (stored row-sorted, i.e. CRS with a stable
// order inside each row), CDS, or the matrix-free 7-point stencil of
// E/STENCIL/user_module.f90.  Indices are 0-based int32.
//
// type(matrix) (M/PP_MATRIX/matrix_module.f90:38-81) becomes `Operator`:
// the solver product A*v = K D^-1 p(K D^-1) v of rmatvec (:152-167), with
// the diagonal scaling D (user preconditioner, which_precon = 1) and the
// real seed shift folded into a scaled copy Ks = (K - seed I) D^-1 made once
// at set-up, and the polynomial evaluated by Horner with every step fused
// into one SpMV kernel: w_new = Ks w + alpha_k v (the epilogue).  So one
// solver matvec with a degree-d polynomial is d+1 SpMV launches and no
// separate vector passes.
#pragma once

#include <vector>

#include "common.cuh"

namespace idrs {

enum Format { FMT_NONE = 0, FMT_DENSE = 1, FMT_CRS = 2, FMT_COO = 3, FMT_CDS = 4, FMT_STENCIL7 = 5 };

// Read-only view of one matrix in one precision (values double/c128 for
// prec 64, float/c64 for prec 32; `vcplx` tells whether values are complex).
struct Deflation;

struct MatView {
  int format = FMT_NONE;
  int nrows = 0, ncols = 0;
  long nnz = 0;
  const int* rp = nullptr;
  const int* ci = nullptr;
  const void* val = nullptr;
  bool vcplx = false;
  int hb = 0;  // CDS half band
  int nx = 0, ny = 0, nz = 0;
  double st[7] = {0, 0, 0, 0, 0, 0, 0};  // stencil c,w,e,s,n,f,b
  int group = 8;                          // CRS lanes per row
  // CRS with skewed rows: length bins.  Rows up to bin_short nonzeros stay
  // with the row kernels; rows up to kBinLong in med_rows (sorted by length)
  // get kBinLanes lanes each; longer rows are cut into kSegNnz-nonzero warp
  // segments whose partial sums are added per row in a fixed order.
  int bin_short = 0, n_med = 0, n_long = 0, n_seg = 0;
  const int* med_rows = nullptr;
  const int* long_rows = nullptr;
  const int* seg_ptr = nullptr;
  void* partial = nullptr;
  // COO: nonzero-balanced segmented reduction: row of every entry, empty
  // rows, per-warp carries
  const int* ri = nullptr;
  int n_empty = 0;
  const int* empty_rows = nullptr;
  void* carry = nullptr;
  // deflation projector applied after the last product of a polynomial chain
  // (rmatvec = Pmul(real_mv(polpre v))); set on the fp64 view only
  const Deflation* defl = nullptr;
  // shift-and-invert preconditioner: every product is Ks (P^-1 v), the
  // triangular solves of P's LU factor into lu_tmp first (fp64 view only)
  const struct UserMatrix* lu = nullptr;
  void* lu_tmp = nullptr;
  // the block system's shift-and-invert form (rprecon, matrix_module.f90:
  // 318-345) needs C, M (n/2 x n/2), the shift and a 2 x n/2 scratch
  const struct UserMatrix* si_C = nullptr;
  const struct UserMatrix* si_M = nullptr;
  c128 si_shift;
  void* si_tmp = nullptr;
};

// Deflation of type(matrix) (matrix_module.f90:1284-1623): V (n x k), AV =
// real_mv(A, V) and E = V^H A V, all on the device (wide type).  Pmul is
// I - AV E^-1 V^H, or I - V V^H for a multishift operator.
struct Deflation {
  int k = 0;
  bool multishift = false;
  bool cplx = false;
  long n = 0;
  void* V = nullptr;
  void* AV = nullptr;
  void* E = nullptr;     // k x k with leading dimension 16 (the device solver's layout)
  void* coef = nullptr;  // 2 x 16 coefficient slots written by the reduction tails
  void* tmp = nullptr;   // n-vector scratch of the chain's last product
  void* tmp2 = nullptr;  // n-vector scratch of add_deflation
  RedBuf rb{nullptr, nullptr};
  cudaStream_t st = nullptr;
};

constexpr int kCooWarpNnz = 256;   // entries per warp of the segmented reduction (8 per lane)
constexpr int kBinShort = 8;       // CRS length bins (rows with one lane per row)
constexpr int kBinLanes = 4;       // lanes per row of the middle bin
constexpr int kBinLong = 256;      // longer rows: warp segments
constexpr int kSegNnz = 1024;      // nonzeros per warp segment of a long row

// Three diagonals of a tridiagonal Jacobi matrix J((d+2) x (d+1)):
// a[i-1] = J(i-1,i), b[i-1] = J(i,i), c[i-1] = J(i+1,i), i = 1..d+1.
struct JacobiCols {
  std::vector<c128> a, b, c;
  bool valid() const { return !c.empty(); }
};

// SpMV epilogue: y = a*(M x) + cx*x + cu*u + cv*v   (u, v may be null)
template <class T>
struct Epi {
  T a = T(1), cx = T(0), cu = T(0), cv = T(0);
  const T* u = nullptr;
  const T* v = nullptr;
};

struct UserMatrix {
  int format = FMT_NONE;
  int which_precon = 0;
  int nrows = 0, ncols = 0;
  int vals = 1;  // 0 pattern, 1 real, 2 complex
  long nnz = 0;
  int* row_ptr = nullptr;  // CRS / sorted COO
  int* col_ind = nullptr;
  void* val = nullptr;     // double or c128
  int half_band = 0;
  void* band = nullptr;    // CDS, column-major nrows x (2hb+1); band LU factor: lu.cu's layout
  void* mat = nullptr;     // dense, column-major
  int nx = 0, ny = 0, nz = 0;
  double st[7] = {0, 0, 0, 0, 0, 0, 0};
  // CRS / COO load-balancing data (see MatView)
  int bin_short = 0, n_med = 0, n_long = 0, n_seg = 0;
  int* med_rows = nullptr;
  int* long_rows = nullptr;
  int* seg_ptr = nullptr;
  void* partial = nullptr;   // 16 B per segment
  int* row_ind = nullptr;    // COO
  int n_empty = 0;
  int* empty_rows = nullptr; // COO rows without entries
  void* carry = nullptr;     // COO: 2 x 16 B per warp of kCooWarpNnz entries
  void* diag = nullptr;    // which_precon == 1: diagonal D (double or c128)
  bool diag_cplx = false;
  bool diag_uniform = false;  // D constant (stencil): value in diag_u
  c128 diag_u;
  int group = 8;
  int refcount = 1;

  MatView view64() const;
  long bytes() const;
};

void user_matrix_release(UserMatrix* K);

// Load balancing of CRS / COO matrices (rp: host copy of the 0-based row
// pointers).  CRS with a row longer than 32 * group nonzeros gets length bins
// (see MatView); every COO matrix uses the nonzero-balanced segmented
// reduction: the row index of every entry, the empty rows, the carries.
void build_row_plan(UserMatrix& M, const int* rp_host);
void build_coo_rows(UserMatrix& M, const int* rp_host);

// The composed operator of type(matrix).
struct Operator {
  UserMatrix* K = nullptr;
  UserMatrix* P = nullptr;  // diagonal preconditioner or null
  bool cplx = false;        // vectors complex?
  c128 seed;                // rseed / cseed
  bool seed_folded = false;  // the seed is part of an assembled system matrix K
  int preconditioner = 0, degree = 0;
  std::vector<c128> alpha_p;  // 0..degree
  JacobiCols jac;             // tridiagonal Jacobi matrix of the polynomial (Chebyshev/Neumann)
  // fp64 evaluation of p: 0 Horner on the monomial coefficients (rpolpre),
  // 1 the three-term recurrence of jac (fp32 products always use it)
  int poly_eval = 0;
  int n_sigma = 0;
  std::vector<c128> alpha_s;  // (degree+1) x n_sigma
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  bool device_pointers = false;

  // scaled operator Ks = (K - seed I) D^-1
  MatView ks64, ks32;         // ks32 built lazily
  void* ks_val64 = nullptr;   // owned scaled values (CRS/COO/CDS/dense)
  void* ks_val32 = nullptr;
  int dkind = 0;              // 0: no scaling, 1: uniform, 2: vector
  c128 dinv_u;                // uniform D^-1
  void* dinv64 = nullptr;     // vector D^-1 (double or c128)
  void* dinv32 = nullptr;
  bool dinv_cplx = false;
  MatView k64;                // unscaled K (original system residual)

  // injected shadow spaces, keyed by s
  std::vector<std::pair<int, void*>> shadows;  // device PT (s x n), wide type

  // reduction scratch for kernels launched on this operator's stream
  RedBuf red{nullptr, nullptr};

  // private partial-sum / carry buffers of the load-balanced kernels (so that
  // operators sharing a user_matrix may run concurrently)
  void* lb_partial = nullptr;
  void* lb_carry = nullptr;

  // statistics of the last flexible (QMRIDR) solve with inner iterations
  int last_inner_calls = 0, last_inner_total = 0, last_inner_max = 0;

  // multishift operator (deflation projector I - V V^H; block system with C)
  bool multishift = false;
  // shift-and-invert: P is the LU factor of the matrix at `shift`
  // (which_precon 2 dense, 3 band); lu_tmp is the solves' scratch vector
  bool shift_invert = false;
  c128 shift;
  void* lu_tmp = nullptr;
  // block system with shift-and-invert: C and M of the block form (held)
  UserMatrix* si_C = nullptr;
  UserMatrix* si_M = nullptr;
  void* si_tmp = nullptr;
  Deflation* defl = nullptr;
  // shifts relative to the seed of the last ms_parameters call (sigma_s)
  std::vector<c128> sigma_s;

  int n() const { return K->nrows; }
  const MatView& view(int prec);
};

// Does a product of precision prec evaluate p by its three-term recurrence?
// fp32: whenever p has a Jacobi matrix; fp64: on request (poly_eval 1), for
// operators without deflation and without a shift-and-invert LU factor.
inline bool use_recurrence(const Operator& A, int prec) {
  if (A.degree <= 0 || !A.jac.valid()) return false;
  if (prec == 32) return true;
  const bool lu = A.P && (A.P->which_precon == 2 || A.P->which_precon == 3);
  return A.poly_eval == 1 && !lu && !(A.defl && A.defl->k > 0);
}

int build_operator(Operator* A);  // (re)builds the scaled data; returns status
void operator_free(Operator* A);
RedBuf alloc_redbuf(cudaStream_t st);
void free_redbuf(RedBuf rb, cudaStream_t st);

// ---------------------------------------------------------------------------
// SpMV with the fused epilogue  y = a * (M x) + cv * v   (v may be null)
// ---------------------------------------------------------------------------
template <class T>
void spmv(const MatView& M, const T* x, T* y, T a, T cv, const T* v, const int* skip,
          cudaStream_t st);
template <class T>
void spmv_ex(const MatView& M, const T* x, T* y, const Epi<T>& e, const int* skip, cudaStream_t st);

// w = fa * Ks p(Ks) v + fcv * fv with p from its Jacobi three-term recurrence
// (numerically stable; used by the fp32 inner solves).  t1..t3: scratch; t4:
// optional fourth scratch vector that lets every pair of fp32 stencil steps
// run as one pass (with three, only pairs whose outputs overwrite none of
// their inputs are fused).
template <class T>
void op_chain_recur(const MatView& Ks, const JacobiCols& J, int degree, const T* v, T* w, T* t1,
                    T* t2, T* t3, T* t4, const int* skip, cudaStream_t st, T fa = T(1), T fcv = T(0),
                    const T* fv = nullptr);

// w = fa * Ks p(Ks) v + fcv * fv, p evaluated as use_recurrence() says
// (t3 null: Horner); t1..t4 as for op_chain_recur.
template <class T>
void op_apply(Operator& A, int prec, const T* v, T* w, T* t1, T* t2, T* t3, T* t4, const int* skip,
              cudaStream_t st, T fa = T(1), T fcv = T(0), const T* fv = nullptr);

// every step of op_chain_recur but the last product; returns the vector
// that product multiplies (y_{d+1}; v itself for degree 0)
template <class T>
const T* op_chain_recur_head(const MatView& Ks, const JacobiCols& J, int degree, const T* v, T* t1, T* t2, T* t3,
                             T* t4, const int* skip, cudaStream_t st);

// w = Ks p(Ks) v, then the final product gets the epilogue
//   w = fa * (Ks u) + fcv * fv.
// t1, t2: scratch vectors (length n).  alpha: polynomial coefficients (host).
template <class T>
void op_chain(const MatView& Ks, const std::vector<c128>& alpha, int degree, const T* v, T* w,
              T* t1, T* t2, const int* skip, cudaStream_t st, T fa = T(1), T fcv = T(0),
              const T* fv = nullptr);

// x = D^-1 p(Ks) y   (scaleback of matrix_module.f90:724-849); with a
// deflated operator and b, add_deflation (shift sigma_s) comes before D^-1
template <class T>
void op_scaleback(Operator& A, int prec, const std::vector<c128>& alpha, int degree,
                  const T* y, T* x, T* t1, T* t2, const int* skip, cudaStream_t st,
                  const T* b = nullptr, c128 sigma_s = c128(0.0, 0.0),
                  c128 factor = c128(1.0, 0.0));

// Shift-and-invert LU factors (lu.cu).  lu_build: P = the dense (which 2) or
// band (which 3) LU factor, without pivoting, of K + shift C + shift^2 M (C
// only: + shift^2 I; M only: K - shift M; no shift: K); throws on a zero
// pivot.  lu_solve: x = P^-1 b (x may equal b).
void lu_build(const UserMatrix& K, const UserMatrix* M, const UserMatrix* C, bool has_shift,
              c128 shift, int which, bool cplx, UserMatrix& P);
template <class T>
void lu_solve(const UserMatrix& P, const T* b, T* x, const int* skip, cudaStream_t st);
// w = v / A for the block system with a shift-and-invert P (n = 2 nn):
// t1 = v2, t2 = P^-1 (v1 + C v2 + shift M v2) (M absent: + shift v2),
// w1 = t1 - shift t2, w2 = -t2.  tmp: 2 nn scratch; w must not alias v.
template <class T>
void block_si_precon(const MatView& V, long nn, const T* v, T* w, const int* skip, cudaStream_t st);
// y = a * Ks (P^-1 x) + cv * v: real_mv of matrix_module.f90:218-264 on a
// view (the LU solve only with a shift-and-invert preconditioner)
template <class T>
void ks_mv(const MatView& Ks, const T* x, T* y, T a, T cv, const T* v, const int* skip,
           cudaStream_t st);

// Deflation (deflation.cu).  deflation_make: V (device, n x k, the
// operator's wide type) -> A.defl; k = 0 removes it.  deflation_pmul:
// out = fa * Pmul(w) + fcv * fv.  deflation_add: add_deflation with the
// shift sigma_s (0 for a single system): x = V Hs^-1 V^H b +
// (y - V Hs^-1 V^H (Ks y - sigma_s y)), Hs = E - sigma_s I.
void deflation_make(Operator& A, const void* V, int k);
void deflation_free(Deflation* D);
template <class T>
void deflation_pmul(const Deflation& D, const T* w, T* out, T fa, T fcv, const T* fv,
                    const int* skip, cudaStream_t st);
template <class T>
void deflation_add(Operator& A, c128 sigma_s, const T* b, const T* y, T* x, const int* skip,
                   cudaStream_t st);

// w = D^-1 v  (operator / of matrix_module.f90:306-352 for a standard system)
template <class T>
void op_precon(Operator& A, int prec, const T* v, T* w, const int* skip, cudaStream_t st);

// elementwise helpers
template <class T> void vec_copy(long n, const T* a, T* b, const int* skip, cudaStream_t st);
template <class T> void vec_scale_vec(long n, const void* d, bool dcplx, const T* a, T* b,
                                      const int* skip, cudaStream_t st);
template <class Tin, class Tout>
void vec_convert(long n, const Tin* a, Tout* b, const int* skip, cudaStream_t st);

// uniform [0,1) generator shared with the oracle (splitmix64 of the index)
__host__ __device__ inline uint64_t splitmix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__host__ __device__ inline double uniform01(uint64_t seed, uint64_t index) {
  uint64_t z = splitmix64(index ^ splitmix64(seed));
  return (double)(z >> 11) * 0x1.0p-53;
}

}  // namespace idrs
