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
! path (crs_transpose, idrs_backward) for gradients of a scalar loss.  Status codes of the C ABI become
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

   function real_precon(which_precon, K, shift) result(P)
      integer, intent(in) :: which_precon
      type(user_matrix), intent(in) :: K
      real(c_double), intent(in), optional :: shift
      type(user_matrix) :: P
      call check(c_real_precon(which_precon, K%h, shift, P%h))
      P%nrows = K%nrows
      P%ncols = K%ncols
   end function real_precon

   function user_mv(K, v) result(w)
      type(user_matrix), intent(in) :: K
      real(c_double), intent(in) :: v(:)
      real(c_double) :: w(K%nrows)
      call check(c_ruser_mv(K%h, v, w))
   end function user_mv

   ! ---------------------------------------------------------- matrix_module
   ! A%K = K, A%P = P, A%rseed = seed (real_matrix.inc:9-58)
   function make_matrix(K, P, seed) result(A)
      type(user_matrix), intent(in) :: K
      type(user_matrix), intent(in), optional :: P
      real(c_double), intent(in), optional :: seed
      type(matrix) :: A
      real(c_double) :: sd(1)
      type(c_ptr) :: ph
      ph = c_null_ptr
      if (present(P)) ph = P%h
      if (present(seed)) then
         sd(1) = seed
         call check(c_matrix_create(K%h, ph, 0_c_int, sd, A%h))
      else
         call check(c_matrix_create(K%h, ph, 0_c_int, A=A%h))
      end if
      A%n = K%nrows
   end function make_matrix

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
