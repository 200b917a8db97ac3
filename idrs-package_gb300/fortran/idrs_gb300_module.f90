!
! idrs_gb300_module.f90 -- Fortran 2018 drop-in for the IDRS package's solve path,
! bound with ISO_C_BINDING to libidrs_gb300.so (include/idrs_gb300.h).
!
! A program written against the reference modules
!     use user_module    ! crs_format, coo_format, cds_format, dense_format, real_precon, *
!     use matrix_module  ! type(matrix), real_preconditioner, *, /
!     use idrs_module    ! IDRS, QMRIDR, NORM, INPROD
! switches to the GB300 path by using this module instead; the generic names,
! argument order and optional arguments are those of
!     M/PP_MATRIX/user_module.f90:829-958, 1327-1463
!     M/PP_MATRIX/matrix_module.f90:135-167, 306-352, 551-635, 811-849
!     M/IDRS/idrs_module.f90:66-103, 107-408, 410-713, 787-837
! (IDRS package paths, M/ = IDRS/MODULES).  Beyond the reference: the adjoint
! path (crs_transpose, idrs_backward) for gradients of a scalar loss.  Also bound: mm_matrix
! (E/MATRIX_MARKET/mm_module.f90), make_deflation / Pmul, IDRS_RITZ and the real pp_idrs
! pipelines (single, sequence, multishift) with their options and report as bind(C)
! types.  Status codes of the C ABI become
! `error stop` with the library's message, as the reference stops on illegal
! arguments.  Index arrays are 1-based, as in the reference.
!
! The operator of type(matrix) is built from a user_matrix K, an optional
! diagonal preconditioner P and a seed, like M/PP_IDRS/real_matrix.inc:9-58.
!
module idrs_gb300_module

   use iso_c_binding
   implicit none

   private
   public :: user_matrix, matrix, crs_format, coo_format, cds_format, stencil7_format
   public :: real_precon, make_matrix, real_preconditioner, scaleback
   public :: operator(*), operator(/)
   public :: IDRS, QMRIDR, MSIDRS, MSQMRIDR, NORM, INPROD
   public :: crs_transpose, idrs_backward
   public :: mm_matrix, make_deflation, Pmul, IDRS_RITZ, pp_idrs
   public :: idrs_pp_options, idrs_pp_report

   type :: user_matrix
      type(c_ptr) :: h = c_null_ptr
      integer     :: nrows = 0, ncols = 0, nnz = 0
   end type user_matrix

   type :: matrix
      type(c_ptr) :: h = c_null_ptr
      integer     :: n = 0
   end type matrix

   interface operator(*)
      module procedure user_mv, rmatvec
   end interface
   interface operator(/)
      module procedure rprecon
   end interface
   interface IDRS
      module procedure RIDRS
   end interface
   interface IDRS_RITZ
      module procedure RIDRS_RITZ
   end interface
   interface pp_idrs
      module procedure RPP_IDRS, RPP_MR_IDRS, RPP_MS_IDRS
   end interface

   ! Options and report of the pp_idrs pipelines (the reference reads the
   ! options from the command line, M/PP_IDRS/initialize.inc:4-31); the members
   ! and their order are those of the C structs idrs_pp_options / _report.
   type, bind(C) :: idrs_pp_options
      integer(c_int) :: method = 1, s = 4
      real(c_double) :: tol = 1.0d-6
      integer(c_int) :: maxit = 1000, in_s = 1, in_it = 0
      real(c_double) :: in_tol = 0.1d0
      integer(c_int) :: preconditioner = 0, degree = 0, n_ritz = 32, inner_precision = 64
      integer(c_int) :: device_pointers = 0, n_omega = 0, recycle = 0
      ! 0: the reference's Horner evaluation of the polynomial in fp64,
      ! 1: its three-term recurrence (see idrs_matrix_set_poly_eval)
      integer(c_int) :: poly_eval = 0
      ! > 0: solve again in FP64 (no inner solves) to this tolerance and report
      ! the relative error against that solution (rel_err_vs_fp64)
      real(c_double) :: fp64_check_tol = 0.0d0
   end type idrs_pp_options

   type, bind(C) :: idrs_pp_report
      integer(c_int) :: flag, iterations, ritz_iterations, nritz
      real(c_double) :: relres_solver, relres_original
      real(c_double) :: foci(2), center
      real(c_double) :: seconds_setup, seconds_solve, seconds_total
      integer(c_int) :: inner_solves, inner_iterations, inner_max
      integer(c_int) :: recycle_flag, recycle_iterations
      real(c_double) :: recycle_relres
      real(c_double) :: foci_imag(2), center_imag
      real(c_double) :: rel_err_vs_fp64, fp64_relres_original
      integer(c_int) :: fp64_flag, fp64_iterations
      real(c_double) :: seconds_fp64_check
   end type idrs_pp_report

   type, bind(C) :: idrs_pp_inputs
      type(c_ptr) :: M = c_null_ptr, C = c_null_ptr, seed = c_null_ptr, shift = c_null_ptr
      type(c_ptr) :: V = c_null_ptr
      integer(c_int) :: n_deflation = 0
   end type idrs_pp_inputs
   interface QMRIDR
      module procedure RQMRIDR
   end interface
   interface MSIDRS
      module procedure RMSIDRS
   end interface
   interface MSQMRIDR
      module procedure RMSQMRIDR
   end interface
   interface NORM
      module procedure RNORM
   end interface
   interface INPROD
      module procedure RINPROD
   end interface

   ! ----------------------------------------------------------------- C ABI
   interface
      function c_last_error() bind(C, name='idrs_last_error') result(p)
         import :: c_ptr
         type(c_ptr) :: p
      end function
      integer(c_int) function c_crs_format(nrows, ncols, row_ptr, col_ind, rval, cval, K) &
            bind(C, name='idrs_crs_format')
         import :: c_int, c_double, c_ptr
         integer(c_int), value :: nrows, ncols
         integer(c_int), intent(in) :: row_ptr(*), col_ind(*)
         real(c_double), intent(in), optional :: rval(*)
         real(c_double), intent(in), optional :: cval(*)
         type(c_ptr), intent(out) :: K
      end function
      integer(c_int) function c_coo_format(nrows, ncols, nnz, indx, jndx, rval, cval, K) &
            bind(C, name='idrs_coo_format')
         import :: c_int, c_double, c_ptr
         integer(c_int), value :: nrows, ncols, nnz
         integer(c_int), intent(in) :: indx(*), jndx(*)
         real(c_double), intent(in), optional :: rval(*)
         real(c_double), intent(in), optional :: cval(*)
         type(c_ptr), intent(out) :: K
      end function
      integer(c_int) function c_cds_format(nrows, ncols, half_band, rband, cband, K) &
            bind(C, name='idrs_cds_format')
         import :: c_int, c_double, c_ptr
         integer(c_int), value :: nrows, ncols, half_band
         real(c_double), intent(in), optional :: rband(*)
         real(c_double), intent(in), optional :: cband(*)
         type(c_ptr), intent(out) :: K
      end function
      integer(c_int) function c_stencil7_format(nx, ny, nz, coef, K) &
            bind(C, name='idrs_stencil7_format')
         import :: c_int, c_double, c_ptr
         integer(c_int), value :: nx, ny, nz
         real(c_double), intent(in) :: coef(7)
         type(c_ptr), intent(out) :: K
      end function
      integer(c_int) function c_real_precon(which, K, shift, P) bind(C, name='idrs_real_precon')
         import :: c_int, c_double, c_ptr
         integer(c_int), value :: which
         type(c_ptr), value :: K
         real(c_double), intent(in), optional :: shift
         type(c_ptr), intent(out) :: P
      end function
      integer(c_int) function c_ruser_mv(K, v, w) bind(C, name='idrs_ruser_mv')
         import :: c_int, c_double, c_ptr
         type(c_ptr), value :: K
         real(c_double), intent(in) :: v(*)
         real(c_double), intent(out) :: w(*)
      end function
      integer(c_int) function c_matrix_create(K, P, is_complex, seed, A) &
            bind(C, name='idrs_matrix_create')
         import :: c_int, c_double, c_ptr
         type(c_ptr), value :: K, P
         integer(c_int), value :: is_complex
         real(c_double), intent(in), optional :: seed(*)
         type(c_ptr), intent(out) :: A
      end function
      integer(c_int) function c_real_preconditioner(A, preconditioner, degree, foci, center, &
            H, ldh, nh) bind(C, name='idrs_real_preconditioner')
         import :: c_int, c_double, c_ptr
         type(c_ptr), value :: A
         integer(c_int), value :: preconditioner, degree, ldh, nh
         real(c_double), intent(in), optional :: foci(2), center, H(*)
      end function
      integer(c_int) function c_rmatvec(A, v, w) bind(C, name='idrs_rmatvec')
         import :: c_int, c_double, c_ptr
         type(c_ptr), value :: A
         real(c_double), intent(in) :: v(*)
         real(c_double), intent(out) :: w(*)
      end function
      integer(c_int) function c_rprecon(A, v, w) bind(C, name='idrs_rprecon')
         import :: c_int, c_double, c_ptr
         type(c_ptr), value :: A
         real(c_double), intent(in) :: v(*)
         real(c_double), intent(out) :: w(*)
      end function
      integer(c_int) function c_rscaleback(A, b, y, x) bind(C, name='idrs_rscaleback')
         import :: c_int, c_double, c_ptr
         type(c_ptr), value :: A
         real(c_double), intent(in) :: b(*), y(*)
         real(c_double), intent(out) :: x(*)
      end function
      integer(c_int) function c_ridrs(A, b, s, M1, tolerance, maximum_iterations, variant, &
            flag, relres, iterations, x0, U0, omega, n_omega, resvec, resvec_len, H, ldh, &
            nritz, x) bind(C, name='idrs_ridrs')
         import :: c_int, c_double, c_ptr
         type(c_ptr), value :: A, M1
         real(c_double), intent(in) :: b(*)
         integer(c_int), value :: s, n_omega, resvec_len, ldh, nritz
         real(c_double), intent(in), optional :: tolerance
         integer(c_int), intent(in), optional :: maximum_iterations, variant
         integer(c_int), intent(out), optional :: flag, iterations
         real(c_double), intent(out), optional :: relres
         real(c_double), intent(in), optional :: x0(*), U0(*), omega(*)
         real(c_double), intent(out), optional :: resvec(*), H(*)
         real(c_double), intent(out) :: x(*)
      end function
      integer(c_int) function c_rqmridr(A, b, s, M1, tolerance, maximum_iterations, flag, &
            relres, iterations, inner_s, inner_tolerance, inner_iterations, x0, omega, n_omega, &
            resvec, resvec_len, inner_precision, x) bind(C, name='idrs_rqmridr')
         import :: c_int, c_double, c_ptr
         type(c_ptr), value :: A, M1
         real(c_double), intent(in) :: b(*)
         integer(c_int), value :: s, n_omega, resvec_len
         real(c_double), intent(in), optional :: tolerance, inner_tolerance
         integer(c_int), intent(in), optional :: maximum_iterations, inner_s, inner_iterations
         integer(c_int), intent(in), optional :: inner_precision
         integer(c_int), intent(out), optional :: flag, iterations
         real(c_double), intent(out), optional :: relres
         real(c_double), intent(in), optional :: x0(*), omega(*)
         real(c_double), intent(out), optional :: resvec(*)
         real(c_double), intent(out) :: x(*)
      end function
      integer(c_int) function c_rmsidrs(A, b, n_sigma, sigma, s, M1, tolerance, &
            maximum_iterations, variant, flag, relres, iterations, omega, n_omega, resvec, &
            resvec_len, colfac, x) bind(C, name='idrs_rmsidrs')
         import :: c_int, c_double, c_ptr
         type(c_ptr), value :: A, M1
         real(c_double), intent(in) :: b(*), sigma(*)
         integer(c_int), value :: n_sigma, s, n_omega, resvec_len
         real(c_double), intent(in), optional :: tolerance
         integer(c_int), intent(in), optional :: maximum_iterations, variant
         integer(c_int), intent(out), optional :: flag, iterations
         real(c_double), intent(out), optional :: relres(*), resvec(*), colfac(*)
         real(c_double), intent(in), optional :: omega(*)
         real(c_double), intent(out) :: x(*)
      end function
      integer(c_int) function c_rmsqmridr(A, b, n_sigma, sigma, s, M1, tolerance, &
            maximum_iterations, flag, relres, iterations, inner_s, inner_tolerance, &
            inner_iterations, omega, n_omega, resvec, resvec_len, inner_precision, x) &
            bind(C, name='idrs_rmsqmridr')
         import :: c_int, c_double, c_ptr
         type(c_ptr), value :: A, M1
         real(c_double), intent(in) :: b(*), sigma(*)
         integer(c_int), value :: n_sigma, s, n_omega, resvec_len
         real(c_double), intent(in), optional :: tolerance, inner_tolerance
         integer(c_int), intent(in), optional :: maximum_iterations, inner_s, inner_iterations
         integer(c_int), intent(in), optional :: inner_precision
         integer(c_int), intent(out), optional :: flag, iterations
         real(c_double), intent(out), optional :: relres(*), resvec(*)
         real(c_double), intent(in), optional :: omega(*)
         real(c_double), intent(out) :: x(*)
      end function
      integer(c_int) function c_crs_transpose(K, KT) bind(C, name='idrs_crs_transpose')
         import :: c_int, c_ptr
         type(c_ptr), value :: K
         type(c_ptr), intent(out) :: KT
      end function
      integer(c_int) function c_radjoint(AT, K, x, g, s, tolerance, maximum_iterations, flag, &
            relres, iterations, lambda, grad) bind(C, name='idrs_radjoint')
         import :: c_int, c_double, c_ptr
         type(c_ptr), value :: AT, K
         real(c_double), intent(in) :: x(*), g(*)
         integer(c_int), value :: s
         real(c_double), intent(in), optional :: tolerance
         integer(c_int), intent(in), optional :: maximum_iterations
         integer(c_int), intent(out), optional :: flag, iterations
         real(c_double), intent(out), optional :: relres
         real(c_double), intent(out) :: lambda(*)
         real(c_double), intent(out), optional :: grad(*)
      end function
      integer(c_int) function c_rnorm(A, w, nrm) bind(C, name='idrs_rnorm')
         import :: c_int, c_double, c_ptr
         type(c_ptr), value :: A
         real(c_double), intent(in) :: w(*)
         real(c_double), intent(out) :: nrm
      end function
      integer(c_int) function c_rinprod(A, u, v, uv) bind(C, name='idrs_rinprod')
         import :: c_int, c_double, c_ptr
         type(c_ptr), value :: A
         real(c_double), intent(in) :: u(*), v(*)
         real(c_double), intent(out) :: uv(2)
      end function
      integer(c_int) function c_real_precon_ext(which, K, M, C, shift, P) &
            bind(C, name='idrs_real_precon_ext')
         import :: c_int, c_double, c_ptr
         integer(c_int), value :: which
         type(c_ptr), value :: K, M, C
         real(c_double), intent(in), optional :: shift
         type(c_ptr), intent(out) :: P
      end function
      integer(c_int) function c_matrix_create_ext(K, M, C, P, is_complex, seed, shift, &
            multishift, A) bind(C, name='idrs_matrix_create_ext')
         import :: c_int, c_double, c_ptr
         type(c_ptr), value :: K, M, C, P
         integer(c_int), value :: is_complex, multishift
         real(c_double), intent(in), optional :: seed(*), shift(*)
         type(c_ptr), intent(out) :: A
      end function
      integer(c_int) function c_mm_matrix(mm_file, which_format, A) bind(C, name='idrs_mm_matrix')
         import :: c_int, c_char, c_ptr
         character(kind=c_char), intent(in) :: mm_file(*), which_format(*)
         type(c_ptr), intent(out) :: A
      end function
      integer(c_int) function c_mm_read(mm_file, which_format, rep, field, nrows, ncols, nnz, &
            ptr, ind, vals) bind(C, name='idrs_mm_read')
         import :: c_int, c_char, c_long, c_ptr
         character(kind=c_char), intent(in) :: mm_file(*), which_format(*)
         integer(c_int), intent(out) :: rep, field, nrows, ncols
         integer(c_long), intent(out) :: nnz
         type(c_ptr), value :: ptr, ind, vals
      end function
      integer(c_int) function c_make_deflation(A, V, k) bind(C, name='idrs_make_deflation')
         import :: c_int, c_double, c_ptr
         type(c_ptr), value :: A
         real(c_double), intent(in) :: V(*)
         integer(c_int), value :: k
      end function
      integer(c_int) function c_rpmul(A, v, w) bind(C, name='idrs_rpmul')
         import :: c_int, c_double, c_ptr
         type(c_ptr), value :: A
         real(c_double), intent(in) :: v(*)
         real(c_double), intent(out) :: w(*)
      end function
      integer(c_int) function c_ridrs_ritz(A, b, s, M, tolerance, maximum_iterations, variant, &
            flag, relres, iterations, x0, U0, dimU0, omega, n_omega, resvec, resvec_len, H, ldh, &
            nh, nritz, x) bind(C, name='idrs_ridrs_ritz')
         import :: c_int, c_double, c_ptr
         type(c_ptr), value :: A, M
         real(c_double), intent(in) :: b(*)
         integer(c_int), value :: s, dimU0, n_omega, resvec_len, ldh, nh
         real(c_double), intent(in), optional :: tolerance
         integer(c_int), intent(in), optional :: maximum_iterations, variant
         integer(c_int), intent(out), optional :: flag, iterations, nritz
         real(c_double), intent(out), optional :: relres
         real(c_double), intent(in), optional :: x0(*)
         real(c_double), intent(out), optional :: U0(*), omega(*), resvec(*), H(*)
         real(c_double), intent(out) :: x(*)
      end function
      integer(c_int) function c_rpp_idrs_ext(K, b, P, center, foci, inp, opt, report, x) &
            bind(C, name='idrs_rpp_idrs_ext')
         import :: c_int, c_double, c_ptr, idrs_pp_options, idrs_pp_report, idrs_pp_inputs
         type(c_ptr), value :: K, P
         real(c_double), intent(in) :: b(*)
         real(c_double), intent(in), optional :: center, foci(2)
         type(idrs_pp_inputs), intent(in) :: inp
         type(idrs_pp_options), intent(in) :: opt
         type(idrs_pp_report), intent(out) :: report
         real(c_double), intent(out) :: x(*)
      end function
      integer(c_int) function c_rpp_mr_idrs_ext(K, nrhs, b_all, P, center, foci, inp, opt, &
            reports, x_all) bind(C, name='idrs_rpp_mr_idrs_ext')
         import :: c_int, c_double, c_ptr, idrs_pp_options, idrs_pp_report, idrs_pp_inputs
         type(c_ptr), value :: K, P
         integer(c_int), value :: nrhs
         real(c_double), intent(in) :: b_all(*)
         real(c_double), intent(in), optional :: center, foci(2)
         type(idrs_pp_inputs), intent(in) :: inp
         type(idrs_pp_options), intent(in) :: opt
         type(idrs_pp_report), intent(out) :: reports(*)
         real(c_double), intent(out) :: x_all(*)
      end function
      integer(c_int) function c_rpp_ms_idrs(K, rhs, n_sigma, sigma, P, center, foci, inp, opt, &
            report, relres, x) bind(C, name='idrs_rpp_ms_idrs')
         import :: c_int, c_double, c_ptr, idrs_pp_options, idrs_pp_report, idrs_pp_inputs
         type(c_ptr), value :: K, P
         real(c_double), intent(in) :: rhs(*), sigma(*)
         integer(c_int), value :: n_sigma
         real(c_double), intent(in), optional :: center, foci(2)
         type(idrs_pp_inputs), intent(in) :: inp
         type(idrs_pp_options), intent(in) :: opt
         type(idrs_pp_report), intent(out) :: report
         real(c_double), intent(out) :: relres(*), x(*)
      end function
   end interface

contains

   subroutine check(status)
      integer(c_int), intent(in) :: status
      character(kind=c_char), pointer :: msg(:)
      character(len=512) :: text
      integer :: i
      if (status == 0) return
      call c_f_pointer(c_last_error(), msg, [512])
      text = ' '
      do i = 1, 512
         if (msg(i) == c_null_char) exit
         text(i:i) = msg(i)
      end do
      error stop trim(text)
   end subroutine check

   ! ------------------------------------------------------------ user_module
   function crs_format(nrows, ncols, row_ptr, col_ind, rval, ival, cval) result(A)
      integer, intent(in) :: nrows, ncols, row_ptr(:), col_ind(:)
      real(c_double), intent(in), optional :: rval(:)
      integer, intent(in), optional :: ival(:)
      complex(c_double_complex), intent(in), optional, target :: cval(:)
      type(user_matrix) :: A
      real(c_double), pointer :: cflat(:)
      if (present(cval)) then
         call c_f_pointer(c_loc(cval), cflat, [2*size(cval)])
         call check(c_crs_format(nrows, ncols, row_ptr, col_ind, cval=cflat, K=A%h))
      elseif (present(rval)) then
         call check(c_crs_format(nrows, ncols, row_ptr, col_ind, rval=rval, K=A%h))
      elseif (present(ival)) then
         call check(c_crs_format(nrows, ncols, row_ptr, col_ind, rval=real(ival, c_double), K=A%h))
      else
         call check(c_crs_format(nrows, ncols, row_ptr, col_ind, K=A%h))
      end if
      A%nrows = nrows
      A%ncols = ncols
      A%nnz = row_ptr(nrows+1) - row_ptr(1)
   end function crs_format

   function coo_format(nrows, ncols, nnz, indx, jndx, rval, ival, cval) result(A)
      integer, intent(in) :: nrows, ncols, nnz, indx(:), jndx(:)
      real(c_double), intent(in), optional :: rval(:)
      integer, intent(in), optional :: ival(:)
      complex(c_double_complex), intent(in), optional, target :: cval(:)
      type(user_matrix) :: A
      real(c_double), pointer :: cflat(:)
      if (present(cval)) then
         call c_f_pointer(c_loc(cval), cflat, [2*size(cval)])
         call check(c_coo_format(nrows, ncols, nnz, indx, jndx, cval=cflat, K=A%h))
      elseif (present(rval)) then
         call check(c_coo_format(nrows, ncols, nnz, indx, jndx, rval=rval, K=A%h))
      elseif (present(ival)) then
         call check(c_coo_format(nrows, ncols, nnz, indx, jndx, rval=real(ival, c_double), K=A%h))
      else
         call check(c_coo_format(nrows, ncols, nnz, indx, jndx, K=A%h))
      end if
      A%nrows = nrows
      A%ncols = ncols
   end function coo_format

   function cds_format(nrows, ncols, half_band, rband) result(A)
      integer, intent(in) :: nrows, ncols, half_band
      real(c_double), intent(in), optional :: rband(nrows, -half_band:half_band)
      type(user_matrix) :: A
      if (present(rband)) then
         call check(c_cds_format(nrows, ncols, half_band, rband=rband, K=A%h))
      else
         call check(c_cds_format(nrows, ncols, half_band, K=A%h))
      end if
      A%nrows = nrows
      A%ncols = ncols
   end function cds_format

   ! Matrix-free 7-point stencil of E/STENCIL/user_module.f90 (c, w, e, s, n, f, b)
   function stencil7_format(nx, ny, nz, coef) result(A)
      integer, intent(in) :: nx, ny, nz
      real(c_double), intent(in) :: coef(7)
      type(user_matrix) :: A
      call check(c_stencil7_format(nx, ny, nz, coef, A%h))
      A%nrows = nx*ny*nz
      A%ncols = A%nrows
   end function stencil7_format

   ! REAL_PRECON(which_precon, K, M, C, shift): user_module.f90:1327-1463
   ! (0 none, 1 diagonal, 2 dense LU, 3 band LU of K + shift C + shift^2 M)
   function real_precon(which_precon, K, M, C, shift) result(P)
      integer, intent(in) :: which_precon
      type(user_matrix), intent(in) :: K
      type(user_matrix), intent(in), optional :: M, C
      real(c_double), intent(in), optional :: shift
      type(user_matrix) :: P
      type(c_ptr) :: mh, ch
      mh = c_null_ptr
      ch = c_null_ptr
      if (present(M)) mh = M%h
      if (present(C)) ch = C%h
      call check(c_real_precon_ext(which_precon, K%h, mh, ch, shift, P%h))
      P%nrows = K%nrows
      P%ncols = K%ncols
   end function real_precon

   ! mm_matrix(mm_file, which_format): E/MATRIX_MARKET/mm_module.f90:48-154
   function mm_matrix(mm_file, which_format) result(A)
      character(len=*), intent(in) :: mm_file
      character(len=3), intent(in), optional :: which_format
      type(user_matrix) :: A
      character(kind=c_char, len=len(mm_file)+1) :: cfile
      character(kind=c_char, len=4) :: cfmt
      integer(c_int) :: rep, field, nrows, ncols
      integer(c_long) :: nnz
      cfile = trim(mm_file) // c_null_char
      cfmt = 'coo' // c_null_char
      if (present(which_format)) cfmt = which_format // c_null_char
      call check(c_mm_read(cfile, cfmt, rep, field, nrows, ncols, nnz, c_null_ptr, c_null_ptr, &
                           c_null_ptr))
      call check(c_mm_matrix(cfile, cfmt, A%h))
      A%nrows = nrows
      A%ncols = ncols
      A%nnz = int(nnz)
   end function mm_matrix

   function user_mv(K, v) result(w)
      type(user_matrix), intent(in) :: K
      real(c_double), intent(in) :: v(:)
      real(c_double) :: w(K%nrows)
      call check(c_ruser_mv(K%h, v, w))
   end function user_mv

   ! ---------------------------------------------------------- matrix_module
   ! A%K = K, A%M = M, A%C = C, A%P = P, A%rseed = seed, A%rshift = shift,
   ! A%multishift (real_matrix.inc:9-58); the block system when multishift and C
   function make_matrix(K, P, seed, M, C, shift, multishift) result(A)
      type(user_matrix), intent(in) :: K
      type(user_matrix), intent(in), optional :: P, M, C
      real(c_double), intent(in), optional :: seed, shift
      logical, intent(in), optional :: multishift
      type(matrix) :: A
      real(c_double) :: sd(2), sh(2)
      type(c_ptr) :: ph, mh, ch
      integer(c_int) :: ms
      ph = c_null_ptr
      mh = c_null_ptr
      ch = c_null_ptr
      if (present(P)) ph = P%h
      if (present(M)) mh = M%h
      if (present(C)) ch = C%h
      ms = 0
      if (present(multishift)) then
         if (multishift) ms = 1
      end if
      sd = 0
      sh = 0
      if (present(seed)) sd(1) = seed
      if (present(shift)) sh(1) = shift
      if (present(seed) .and. present(shift)) then
         call check(c_matrix_create_ext(K%h, mh, ch, ph, 0_c_int, sd, sh, ms, A%h))
      elseif (present(seed)) then
         call check(c_matrix_create_ext(K%h, mh, ch, ph, 0_c_int, seed=sd, multishift=ms, A=A%h))
      elseif (present(shift)) then
         call check(c_matrix_create_ext(K%h, mh, ch, ph, 0_c_int, shift=sh, multishift=ms, A=A%h))
      else
         call check(c_matrix_create_ext(K%h, mh, ch, ph, 0_c_int, multishift=ms, A=A%h))
      end if
      A%n = K%nrows
      if (ms == 1 .and. present(C)) A%n = 2 * K%nrows
   end function make_matrix

   ! make_deflation(A, V) and Pmul(A, v): matrix_module.f90:1284-1418
   subroutine make_deflation(A, V)
      type(matrix), intent(inout) :: A
      real(c_double), intent(in) :: V(:,:)
      call check(c_make_deflation(A%h, V, int(size(V,2), c_int)))
   end subroutine make_deflation

   function Pmul(A, v) result(w)
      type(matrix), intent(in) :: A
      real(c_double), intent(in) :: v(:)
      real(c_double) :: w(size(v))
      call check(c_rpmul(A%h, v, w))
   end function Pmul

   subroutine real_preconditioner(A, preconditioner, degree, foci, center, H)
      type(matrix), intent(inout) :: A
      integer, intent(in), optional :: preconditioner, degree
      real(c_double), intent(in), optional :: foci(2), center
      real(c_double), intent(in), optional :: H(:,:)
      integer :: pre, deg
      pre = 0
      deg = 0
      if (present(preconditioner)) pre = preconditioner
      if (present(degree)) deg = degree
      if (present(H)) then
         call check(c_real_preconditioner(A%h, pre, deg, foci, center, H, size(H,1), size(H,2)))
      else
         call check(c_real_preconditioner(A%h, pre, deg, foci, center, ldh=0, nh=0))
      end if
   end subroutine real_preconditioner

   function rmatvec(A, v) result(w)
      type(matrix), intent(in) :: A
      real(c_double), intent(in) :: v(:)
      real(c_double) :: w(size(v))
      call check(c_rmatvec(A%h, v, w))
   end function rmatvec

   function rprecon(v, A) result(w)
      real(c_double), intent(in) :: v(:)
      type(matrix), intent(in) :: A
      real(c_double) :: w(size(v))
      call check(c_rprecon(A%h, v, w))
   end function rprecon

   function scaleback(A, b, y) result(x)
      type(matrix), intent(in) :: A
      real(c_double), intent(in) :: b(:), y(:)
      real(c_double) :: x(size(y))
      call check(c_rscaleback(A%h, b, y, x))
   end function scaleback

   ! ------------------------------------------------------------ idrs_module
   function RIDRS(A, b, s, M1, tolerance, maximum_iterations, variant, flag, relres, &
                  iterations, x0, U0, omega, resvec, H) result(x)
      type(matrix), intent(in) :: A
      real(c_double), intent(in) :: b(:)
      integer, intent(in) :: s
      type(matrix), intent(in), optional :: M1
      real(c_double), intent(in), optional :: tolerance
      integer, intent(in), optional :: maximum_iterations, variant
      integer, intent(out), optional :: flag, iterations
      real(c_double), intent(out), optional :: relres
      real(c_double), intent(in), optional :: x0(:), omega(:)
      real(c_double), allocatable, intent(in), optional :: U0(:,:)
      real(c_double), intent(out), optional :: resvec(:), H(:,:)
      real(c_double) :: x(size(b))
      type(c_ptr) :: m1h
      integer :: n_omega, nres, ldh, nritz
      m1h = c_null_ptr
      if (present(M1)) m1h = M1%h
      n_omega = 0
      if (present(omega)) n_omega = size(omega)
      nres = 0
      if (present(resvec)) nres = size(resvec)
      ldh = 0
      nritz = 0
      if (present(H)) then
         ldh = size(H,1)
         nritz = size(H,2)
      end if
      if (present(U0)) then
         if (allocated(U0)) then
            call check(c_ridrs(A%h, b, s, m1h, tolerance, maximum_iterations, variant, flag, &
                 relres, iterations, x0, U0, omega, n_omega, resvec, nres, H, ldh, nritz, x))
            return
         end if
      end if
      call check(c_ridrs(A%h, b, s, m1h, tolerance, maximum_iterations, variant, flag, relres, &
           iterations, x0=x0, omega=omega, n_omega=n_omega, resvec=resvec, resvec_len=nres, &
           H=H, ldh=ldh, nritz=nritz, x=x))
   end function RIDRS

   function RQMRIDR(A, b, s, M1, tolerance, maximum_iterations, flag, relres, iterations, &
                    inner_s, inner_tolerance, inner_iterations, x0, omega, resvec, &
                    inner_precision) result(x)
      type(matrix), intent(in) :: A
      real(c_double), intent(in) :: b(:)
      integer, intent(in) :: s
      type(matrix), intent(in), optional :: M1
      real(c_double), intent(in), optional :: tolerance, inner_tolerance
      integer, intent(in), optional :: maximum_iterations, inner_s, inner_iterations
      integer, intent(in), optional :: inner_precision
      integer, intent(out), optional :: flag, iterations
      real(c_double), intent(out), optional :: relres
      real(c_double), intent(in), optional :: x0(:), omega(:)
      real(c_double), intent(out), optional :: resvec(:)
      real(c_double) :: x(size(b))
      type(c_ptr) :: m1h
      integer :: n_omega, nres
      m1h = c_null_ptr
      if (present(M1)) m1h = M1%h
      n_omega = 0
      if (present(omega)) n_omega = size(omega)
      nres = 0
      if (present(resvec)) nres = size(resvec)
      call check(c_rqmridr(A%h, b, s, m1h, tolerance, maximum_iterations, flag, relres, &
           iterations, inner_s, inner_tolerance, inner_iterations, x0, omega, n_omega, resvec, &
           nres, inner_precision, x))
   end function RQMRIDR

   function RMSIDRS(A, b, sigma, s, M1, tolerance, maximum_iterations, variant, flag, relres, &
                    iterations, omega, resvec, colfac) result(x)
      ! RMSIDRS, idrs_module.f90:572-641
      type(matrix), intent(in) :: A
      real(c_double), intent(in) :: b(:), sigma(:)
      integer, intent(in) :: s
      type(matrix), intent(in), optional :: M1
      real(c_double), intent(in), optional :: tolerance
      integer, intent(in), optional :: maximum_iterations, variant
      integer, intent(out), optional :: flag, iterations
      real(c_double), intent(out), optional :: relres(size(sigma)), colfac(size(sigma))
      real(c_double), intent(in), optional :: omega(:)
      real(c_double), intent(out), optional :: resvec(:,:)
      real(c_double) :: x(size(b), size(sigma))
      type(c_ptr) :: m1h
      integer :: n_omega, nres
      m1h = c_null_ptr
      if (present(M1)) m1h = M1%h
      n_omega = 0
      if (present(omega)) n_omega = size(omega)
      nres = 0
      if (present(resvec)) nres = size(resvec, 1)
      call check(c_rmsidrs(A%h, b, size(sigma), sigma, s, m1h, tolerance, maximum_iterations, &
           variant, flag, relres, iterations, omega, n_omega, resvec, nres, colfac, x))
   end function RMSIDRS

   function RMSQMRIDR(A, b, sigma, s, M1, tolerance, maximum_iterations, flag, relres, &
                      iterations, inner_s, inner_tolerance, inner_iterations, omega, resvec, &
                      inner_precision) result(x)
      ! RMSQMRIDR, idrs_module.f90:491-570
      type(matrix), intent(in) :: A
      real(c_double), intent(in) :: b(:), sigma(:)
      integer, intent(in) :: s
      type(matrix), intent(in), optional :: M1
      real(c_double), intent(in), optional :: tolerance, inner_tolerance
      integer, intent(in), optional :: maximum_iterations, inner_s, inner_iterations
      integer, intent(in), optional :: inner_precision
      integer, intent(out), optional :: flag, iterations
      real(c_double), intent(out), optional :: relres(size(sigma))
      real(c_double), intent(in), optional :: omega(:)
      real(c_double), intent(out), optional :: resvec(:,:)
      real(c_double) :: x(size(b), size(sigma))
      type(c_ptr) :: m1h
      integer :: n_omega, nres
      m1h = c_null_ptr
      if (present(M1)) m1h = M1%h
      n_omega = 0
      if (present(omega)) n_omega = size(omega)
      nres = 0
      if (present(resvec)) nres = size(resvec, 1)
      call check(c_rmsqmridr(A%h, b, size(sigma), sigma, s, m1h, tolerance, maximum_iterations, &
           flag, relres, iterations, inner_s, inner_tolerance, inner_iterations, omega, n_omega, &
           resvec, nres, inner_precision, x))
   end function RMSQMRIDR

   ! ---------------------------------------------------------------- adjoint
   function crs_transpose(K) result(KT)
      ! K^T as a new CRS user_matrix, built on the device
      type(user_matrix), intent(in) :: K
      type(user_matrix) :: KT
      call check(c_crs_transpose(K%h, KT%h))
      KT%nrows = K%ncols
      KT%ncols = K%nrows
      KT%nnz = K%nnz
   end function crs_transpose

   subroutine idrs_backward(AT, K, x, dLdx, s, dLdb, dLdK, tolerance, maximum_iterations, &
                            flag, relres, iterations)
      ! Backward step of A x = b, A = K (CRS), for a scalar loss L(x):
      ! AT lambda = dL/dx with IDR(s) on the adjoint operator AT (built from
      ! crs_transpose(K)), dL/db = lambda, dL/dK(p) = -lambda(i) x(j) over K's
      ! stored entries p = (i, j) in storage order.
      type(matrix), intent(in) :: AT
      type(user_matrix), intent(in) :: K
      real(c_double), intent(in) :: x(:), dLdx(:)
      integer, intent(in) :: s
      real(c_double), intent(out) :: dLdb(:)
      real(c_double), intent(out), optional :: dLdK(:)
      real(c_double), intent(in), optional :: tolerance
      integer, intent(in), optional :: maximum_iterations
      integer, intent(out), optional :: flag, iterations
      real(c_double), intent(out), optional :: relres
      if (present(dLdK)) then
         if (size(dLdK) /= K%nnz) error stop "idrs_backward: dLdK must have one entry per nonzero of K"
      end if
      call check(c_radjoint(AT%h, K%h, x, dLdx, s, tolerance, maximum_iterations, flag, relres, &
           iterations, dLdb, dLdK))
   end subroutine idrs_backward

   ! x = IDRS_RITZ(A, b, s, M, tolerance, maximum_iterations, variant, flag,
   ! relres, iterations, x0, U0, omega, resvec, H): ritz_module.f90:389-556
   function RIDRS_RITZ(A, b, s, M, tolerance, maximum_iterations, variant, flag, relres, &
                       iterations, x0, U0, omega, resvec, H) result(x)
      type(matrix), intent(in) :: A
      real(c_double), intent(in) :: b(:)
      integer, intent(in) :: s
      type(matrix), intent(in), optional :: M
      real(c_double), intent(in), optional :: tolerance
      integer, intent(in), optional :: maximum_iterations, variant
      integer, intent(out), optional :: flag, iterations
      real(c_double), intent(out), optional :: relres
      real(c_double), intent(in), optional :: x0(:)
      real(c_double), allocatable, intent(inout), optional :: U0(:,:)
      real(c_double), intent(out), optional :: omega(:), resvec(:), H(:,:)
      real(c_double) :: x(size(b))
      type(c_ptr) :: mh
      integer(c_int) :: dimU0, n_omega, nres, ldh, nh, nritz
      mh = c_null_ptr
      if (present(M)) mh = M%h
      dimU0 = 0
      n_omega = 0
      nres = 0
      ldh = 0
      nh = 0
      if (present(omega)) n_omega = size(omega)
      if (present(resvec)) nres = size(resvec)
      if (present(H)) then
         ldh = size(H,1)
         nh = size(H,2)
      end if
      if (present(U0)) then
         if (allocated(U0)) then
            dimU0 = size(U0,2)
            call check(c_ridrs_ritz(A%h, b, s, mh, tolerance, maximum_iterations, variant, flag, &
                 relres, iterations, x0, U0, dimU0, omega, n_omega, resvec, nres, H, ldh, nh, &
                 nritz, x))
            return
         end if
      end if
      call check(c_ridrs_ritz(A%h, b, s, mh, tolerance, maximum_iterations, variant, flag, relres, &
           iterations, x0=x0, dimU0=dimU0, omega=omega, n_omega=n_omega, resvec=resvec, &
           resvec_len=nres, H=H, ldh=ldh, nh=nh, nritz=nritz, x=x))
   end function RIDRS_RITZ

   ! the optional M, C, seed, shift, V of pp_idrs as the C struct
   subroutine pp_inputs(inp, M, C, seed, shift, V, sd, sh)
      type(idrs_pp_inputs), intent(out) :: inp
      type(user_matrix), intent(in), optional :: M, C
      real(c_double), intent(in), optional, target :: seed, shift
      real(c_double), intent(in), optional, target, contiguous :: V(:,:)
      real(c_double), intent(inout), target :: sd(2), sh(2)
      if (present(M)) inp%M = M%h
      if (present(C)) inp%C = C%h
      if (present(seed)) then
         sd(1) = seed
         inp%seed = c_loc(sd)
      end if
      if (present(shift)) then
         sh(1) = shift
         inp%shift = c_loc(sh)
      end if
      if (present(V)) then
         inp%V = c_loc(V)
         inp%n_deflation = size(V,2)
      end if
   end subroutine pp_inputs

   ! x = pp_idrs(K, b, opt, M, C, P, center, foci, seed, shift, V, report):
   ! RPP_IDRS, pp_idrs_module.f90:118-162
   function RPP_IDRS(K, b, opt, M, C, P, center, foci, seed, shift, V, report) result(x)
      type(user_matrix), intent(in) :: K
      real(c_double), intent(in) :: b(:)
      type(idrs_pp_options), intent(in) :: opt
      type(user_matrix), intent(in), optional :: M, C, P
      real(c_double), intent(in), optional :: center, foci(2), seed, shift
      real(c_double), intent(in), optional, target, contiguous :: V(:,:)
      type(idrs_pp_report), intent(out), optional :: report
      real(c_double) :: x(size(b))
      type(idrs_pp_inputs) :: inp
      type(idrs_pp_report) :: rep
      real(c_double), target :: sd(2), sh(2)
      type(c_ptr) :: ph
      sd = 0
      sh = 0
      ph = c_null_ptr
      if (present(P)) ph = P%h
      call pp_inputs(inp, M, C, seed, shift, V, sd, sh)
      call check(c_rpp_idrs_ext(K%h, b, ph, center, foci, inp, opt, rep, x))
      if (present(report)) report = rep
   end function RPP_IDRS

   ! x_all = pp_idrs(K, b_all, opt, ...): RPP_MR_IDRS, pp_idrs_module.f90:222-279
   function RPP_MR_IDRS(K, b_all, opt, M, C, P, center, foci, seed, shift, V, reports) result(x_all)
      type(user_matrix), intent(in) :: K
      real(c_double), intent(in) :: b_all(:,:)
      type(idrs_pp_options), intent(in) :: opt
      type(user_matrix), intent(in), optional :: M, C, P
      real(c_double), intent(in), optional :: center, foci(2), seed, shift
      real(c_double), intent(in), optional, target, contiguous :: V(:,:)
      type(idrs_pp_report), intent(out), optional :: reports(:)
      real(c_double) :: x_all(size(b_all,1), size(b_all,2))
      type(idrs_pp_inputs) :: inp
      type(idrs_pp_report) :: reps(size(b_all,2))
      real(c_double), target :: sd(2), sh(2)
      type(c_ptr) :: ph
      sd = 0
      sh = 0
      ph = c_null_ptr
      if (present(P)) ph = P%h
      call pp_inputs(inp, M, C, seed, shift, V, sd, sh)
      call check(c_rpp_mr_idrs_ext(K%h, int(size(b_all,2), c_int), b_all, ph, center, foci, inp, &
                                   opt, reps, x_all))
      if (present(reports)) reports = reps
   end function RPP_MR_IDRS

   ! x(:, 1:n_sigma) = pp_idrs(K, rhs, sigma, opt, ...): RPP_MS_IDRS, pp_idrs_module.f90:346-409
   function RPP_MS_IDRS(K, rhs, sigma, opt, M, C, P, center, foci, seed, shift, V, report, &
                        relres) result(x)
      type(user_matrix), intent(in) :: K
      real(c_double), intent(in) :: rhs(:), sigma(:)
      type(idrs_pp_options), intent(in) :: opt
      type(user_matrix), intent(in), optional :: M, C, P
      real(c_double), intent(in), optional :: center, foci(2), seed, shift
      real(c_double), intent(in), optional, target, contiguous :: V(:,:)
      type(idrs_pp_report), intent(out), optional :: report
      real(c_double), intent(out), optional :: relres(:)
      real(c_double) :: x(size(rhs), size(sigma))
      type(idrs_pp_inputs) :: inp
      type(idrs_pp_report) :: rep
      real(c_double) :: rel(size(sigma))
      real(c_double), target :: sd(2), sh(2)
      type(c_ptr) :: ph
      sd = 0
      sh = 0
      ph = c_null_ptr
      if (present(P)) ph = P%h
      call pp_inputs(inp, M, C, seed, shift, V, sd, sh)
      call check(c_rpp_ms_idrs(K%h, rhs, int(size(sigma), c_int), sigma, ph, center, foci, inp, &
                               opt, rep, rel, x))
      if (present(report)) report = rep
      if (present(relres)) relres = rel
   end function RPP_MS_IDRS

   function RNORM(A, w) result(nrm)
      type(matrix), intent(in) :: A
      real(c_double), intent(in) :: w(:)
      real(c_double) :: nrm
      call check(c_rnorm(A%h, w, nrm))
   end function RNORM

   function RINPROD(A, u, v) result(uv)
      type(matrix), intent(in) :: A
      real(c_double), intent(in) :: u(:), v(:)
      real(c_double) :: uv, buf(2)
      call check(c_rinprod(A%h, u, v, buf))
      uv = buf(1)
   end function RINPROD

end module idrs_gb300_module
