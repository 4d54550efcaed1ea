! gammcor_gpu.f90 -- Fortran (ISO_C_BINDING) interface to libgammcor_gpu.
!
! The bind(C) interfaces mirror include/gammcor_gpu.h. The wrappers below keep
! the names and argument lists of the reference routines they replace, so a
! call site in GAMMCOR changes only its routine name and passes device buffers
! where the reference passes scratch-file names (FFOO, FOFO):
!
!   AB_CAS_FOFO     abfofo.f90:8-10     -> AB_CAS_FOFO_GPU
!   ERPASYMM1       interpa.f:1652      -> ERPASYMM1_GPU
!   ACEneERPA_FOFO  abfofo.f90:3791-3792 -> ACENEERPA_FOFO_GPU
!   tran4_gen       tran.f90:313        -> TRAN4_GEN_GPU
!
! Host arrays keep their Fortran shapes; the wrappers copy them to and from
! the device with the CUDA runtime (cudaMalloc/cudaMemcpy/cudaFree, bound
! below). A status other than GC_OK stops the program with the library's
! message, as the reference stops on LAPACK failures (misc.f:563-600).
!
! No Fortran compiler exists where this library was built, so this file has
! not been compiled there.
module gammcor_gpu
  use iso_c_binding
  implicit none
  private :: check, to_dev, from_dev, dev_alloc, dev_free

  integer(c_int), parameter :: GC_OK = 0
  integer(c_int), parameter :: GC_PREC_FP64 = 0, GC_PREC_BF16X3 = 1, GC_PREC_BF16X6 = 2, &
                               GC_PREC_FP64TC5 = 3, GC_PREC_FP64TC6 = 4
  integer(c_int), parameter :: GC_ERPA_SYMM1 = 0, GC_ERPA_CHOLESKY = 1, &
                               GC_ERPA_CHOLESKY_REFINED = 2
  integer(c_int), parameter :: cudaMemcpyHostToDevice = 1, cudaMemcpyDeviceToHost = 2

  type, bind(C) :: gc_system
    integer(c_int) :: nbas, ninact, nact, ndimx, rank
    type(c_ptr) :: occ, xone, indn, rdm2act   ! host arrays (c_loc of the Fortran arrays)
    type(c_ptr) :: cmo_dev, lfac_dev          ! device arrays
  end type

  type, bind(C) :: gc_ac_params
    integer(c_int) :: ngrid, precision, erpa_mode, affine, nstreams, eig_emulation, eig_refine
    type(c_ptr) :: lambda, weight             ! c_null_ptr: Gauss-Legendre points on [0,1]
  end type

  ! the context the wrappers use (device 0, legacy default stream), made on first use
  type(c_ptr), save :: gpu_ctx = c_null_ptr

  interface
    integer(c_int) function gc_create(ctx, device, stream) bind(C, name="gc_create")
      import :: c_ptr, c_int
      type(c_ptr) :: ctx
      integer(c_int), value :: device
      type(c_ptr), value :: stream
    end function
    integer(c_int) function gc_destroy(ctx) bind(C, name="gc_destroy")
      import :: c_ptr, c_int
      type(c_ptr), value :: ctx
    end function
    type(c_ptr) function gc_last_error(ctx) bind(C, name="gc_last_error")
      import :: c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function gc_tran4_gen(ctx, nbas, na, ca, nb, cb, nc, cc, nd, cd, ao, out, prec) &
        bind(C, name="gc_tran4_gen")
      import :: c_ptr, c_int
      type(c_ptr), value :: ctx, ca, cb, cc, cd, ao, out
      integer(c_int), value :: nbas, na, nb, nc, nd, prec
    end function
    integer(c_int) function gc_ab_cas_fofo_ex(ctx, nbas, ninact, nact, ndimx, occ, ure, xone, indn, &
        rdm2act, ffoo, fofo, alpha, ab1, abplus, abmin, etot) bind(C, name="gc_ab_cas_fofo_ex")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: ctx, ffoo, fofo, abplus, abmin
      integer(c_int), value :: nbas, ninact, nact, ndimx, ab1
      real(c_double) :: occ(*), ure(*), xone(*), rdm2act(*), etot
      integer(c_int) :: indn(2,*)
      real(c_double), value :: alpha
    end function
    integer(c_int) function gc_erpasymm1(ctx, ndimx, abplus, abmin, eigvec, eig) &
        bind(C, name="gc_erpasymm1")
      import :: c_ptr, c_int
      type(c_ptr), value :: ctx, abplus, abmin, eigvec, eig
      integer(c_int), value :: ndimx
    end function
    integer(c_int) function gc_erpa_ex(ctx, ndimx, abplus, abmin, eigvec, eig, mode, prec) &
        bind(C, name="gc_erpa_ex")
      import :: c_ptr, c_int
      type(c_ptr), value :: ctx, abplus, abmin, eigvec, eig
      integer(c_int), value :: ndimx, mode, prec
    end function
    integer(c_int) function gc_ace_ne_erpa_fofo(ctx, nbas, ninact, nact, ndimx, occ, indn, eigvec, &
        eig, fofo, prec, w) bind(C, name="gc_ace_ne_erpa_fofo")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: ctx, eigvec, eig, fofo
      integer(c_int), value :: nbas, ninact, nact, ndimx, prec
      real(c_double) :: occ(*), w
      integer(c_int) :: indn(2,*)
    end function
    integer(c_int) function gc_acecorr(ctx, nbas, ninact, nact, ndimx, occ, xone, indn, rdm2act, &
        ffoo, fofo, ngrid, erpa_mode, prec, ecorr, ecas, w_out) bind(C, name="gc_acecorr")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: ctx, ffoo, fofo
      integer(c_int), value :: nbas, ninact, nact, ndimx, ngrid, erpa_mode, prec
      real(c_double) :: occ(*), xone(*), rdm2act(*), ecorr, ecas, w_out(*)
      integer(c_int) :: indn(2,*)
    end function
    integer(c_int) function gc_ac_energy_batched(ctx, nsys, sys, par, ecorr, ecas, w_lambda, &
        omega_stats, status) bind(C, name="gc_ac_energy_batched")
      import :: c_ptr, c_int, c_double, gc_system, gc_ac_params
      type(c_ptr), value :: ctx, w_lambda, omega_stats, status
      integer(c_int), value :: nsys
      type(gc_system) :: sys(*)
      type(gc_ac_params) :: par
      real(c_double) :: ecorr(*), ecas(*)
    end function
    ! context settings and timing (no counterpart in the reference)
    integer(c_int) function gc_set_eig_batch(ctx, on) bind(C, name="gc_set_eig_batch")
      import :: c_ptr, c_int
      type(c_ptr), value :: ctx
      integer(c_int), value :: on
    end function
    integer(c_int) function gc_set_gemm_tile(ctx, width) bind(C, name="gc_set_gemm_tile")
      import :: c_ptr, c_int
      type(c_ptr), value :: ctx
      integer(c_int), value :: width
    end function
    integer(c_int) function gc_set_phase_timing(ctx, on) bind(C, name="gc_set_phase_timing")
      import :: c_ptr, c_int
      type(c_ptr), value :: ctx
      integer(c_int), value :: on
    end function
    integer(c_int) function gc_phase_time(ctx, phase, ms, calls) bind(C, name="gc_phase_time")
      import :: c_ptr, c_int, c_double, c_long_long
      type(c_ptr), value :: ctx
      integer(c_int), value :: phase
      real(c_double) :: ms
      integer(c_long_long) :: calls
    end function
    integer(c_int) function gc_eig_time(ctx, ms, calls) bind(C, name="gc_eig_time")
      import :: c_ptr, c_int, c_double, c_long_long
      type(c_ptr), value :: ctx
      real(c_double) :: ms
      integer(c_long_long) :: calls
    end function
    ! CUDA runtime
    integer(c_int) function cudaMalloc(ptr, bytes) bind(C, name="cudaMalloc")
      import :: c_ptr, c_int, c_size_t
      type(c_ptr) :: ptr
      integer(c_size_t), value :: bytes
    end function
    integer(c_int) function cudaFree(ptr) bind(C, name="cudaFree")
      import :: c_ptr, c_int
      type(c_ptr), value :: ptr
    end function
    integer(c_int) function cudaMemcpy(dst, src, bytes, kind) bind(C, name="cudaMemcpy")
      import :: c_ptr, c_int, c_size_t
      type(c_ptr), value :: dst, src
      integer(c_size_t), value :: bytes
      integer(c_int), value :: kind
    end function
  end interface

contains

  subroutine check(status, where)
    integer(c_int), intent(in) :: status
    character(*), intent(in) :: where
    character(kind=c_char), pointer :: msg(:)
    integer :: n
    if (status == GC_OK) return
    call c_f_pointer(gc_last_error(gpu_ctx), msg, [512])
    n = 0
    do while (n < 512)
      if (msg(n + 1) == c_null_char) exit
      n = n + 1
    end do
    write(6, '(1x,a,": status ",i0,": ",512a)') where, status, msg(1:n)
    stop
  end subroutine

  subroutine context()
    if (.not. c_associated(gpu_ctx)) call check(gc_create(gpu_ctx, 0_c_int, c_null_ptr), "gc_create")
  end subroutine

  function dev_alloc(nelem) result(p)
    integer(c_size_t), intent(in) :: nelem
    type(c_ptr) :: p
    p = c_null_ptr
    if (cudaMalloc(p, 8_c_size_t * nelem) /= 0) stop "gammcor_gpu: cudaMalloc failed"
  end function

  subroutine dev_free(p)
    type(c_ptr), intent(inout) :: p
    if (c_associated(p)) then
      if (cudaFree(p) /= 0) stop "gammcor_gpu: cudaFree failed"
    end if
    p = c_null_ptr
  end subroutine

  subroutine to_dev(dev, host, nelem)
    type(c_ptr), intent(in) :: dev
    real(c_double), target, intent(in) :: host(*)
    integer(c_size_t), intent(in) :: nelem
    if (cudaMemcpy(dev, c_loc(host), 8_c_size_t * nelem, cudaMemcpyHostToDevice) /= 0) &
      stop "gammcor_gpu: cudaMemcpy to the device failed"
  end subroutine

  subroutine from_dev(host, dev, nelem)
    real(c_double), target, intent(inout) :: host(*)
    type(c_ptr), intent(in) :: dev
    integer(c_size_t), intent(in) :: nelem
    if (cudaMemcpy(c_loc(host), dev, 8_c_size_t * nelem, cudaMemcpyDeviceToHost) /= 0) &
      stop "gammcor_gpu: cudaMemcpy from the device failed"
  end subroutine

  ! tran4_gen(NBas,nA,CA,nB,CB,nC,CC,nD,CD,fname,srtfile), tran.f90:313: the output
  ! file and the AOTWOSORT file become device buffers (out_dev: nA*nB records of
  ! nC*nD doubles; ao_dev: ntr records of ntr doubles).
  subroutine TRAN4_GEN_GPU(NBas, nA, CA, nB, CB, nC, CC, nD, CD, out_dev, ao_dev)
    integer, intent(in) :: NBas, nA, nB, nC, nD
    real(c_double), intent(in) :: CA(NBas,nA), CB(NBas,nB), CC(NBas,nC), CD(NBas,nD)
    type(c_ptr), intent(in) :: out_dev, ao_dev
    type(c_ptr) :: da, db, dc, dd
    call context()
    da = dev_alloc(int(NBas, c_size_t) * nA)
    db = dev_alloc(int(NBas, c_size_t) * nB)
    dc = dev_alloc(int(NBas, c_size_t) * nC)
    dd = dev_alloc(int(NBas, c_size_t) * nD)
    call to_dev(da, CA, int(NBas, c_size_t) * nA)
    call to_dev(db, CB, int(NBas, c_size_t) * nB)
    call to_dev(dc, CC, int(NBas, c_size_t) * nC)
    call to_dev(dd, CD, int(NBas, c_size_t) * nD)
    call check(gc_tran4_gen(gpu_ctx, NBas, nA, da, nB, db, nC, dc, nD, dd, ao_dev, out_dev, &
                            GC_PREC_FP64), "tran4_gen")
    call dev_free(da); call dev_free(db); call dev_free(dc); call dev_free(dd)
  end subroutine

  ! AB_CAS_FOFO(ABPLUS,ABMIN,ETot,URe,Occ,XOne,IndN,IndX,IGemIN,NAct,INActive,NDimX,
  !             NBasis,NDim,NInte1,IntJFile,IntKFile,ACAlpha,AB1), abfofo.f90:8-10.
  ! IntJFile/IntKFile become the FFOO/FOFO device buffers; the active 2-RDM, which
  ! the reference reads from rdm2.dat, is passed as RDM2Act (its NAddrRDM packing,
  ! value/2 as AB_CAS_FOFO stores it). IndX must be the identity and IGemIN the
  ! inactive/active/virtual grouping, as ACCAS sets them.
  subroutine AB_CAS_FOFO_GPU(ABPLUS, ABMIN, ETot, URe, Occ, XOne, IndN, IndX, IGemIN, NAct, &
                             INActive, NDimX, NBasis, NDim, NInte1, ffoo_dev, fofo_dev, &
                             ACAlpha, AB1, RDM2Act)
    integer, intent(in) :: NAct, INActive, NDimX, NBasis, NDim, NInte1
    integer, intent(in) :: IndN(2,NDim), IndX(NDim), IGemIN(NBasis)
    real(c_double), intent(in) :: URe(NBasis,NBasis), Occ(NBasis), XOne(NInte1), ACAlpha
    real(c_double), intent(in) :: RDM2Act(*)
    logical, intent(in) :: AB1
    type(c_ptr), intent(in) :: ffoo_dev, fofo_dev
    real(c_double), intent(out) :: ABPLUS(NDimX,NDimX), ABMIN(NDimX,NDimX), ETot
    integer(c_int) :: ind(2,NDimX)
    type(c_ptr) :: dp, dm
    integer :: i
    call context()
    do i = 1, NDimX
      if (IndX(i) /= i) stop "AB_CAS_FOFO_GPU: IndX must be the identity"
    end do
    do i = 1, NBasis
      if ((i <= INActive .and. IGemIN(i) /= 1) .or. &
          (i > INActive .and. i <= INActive + NAct .and. IGemIN(i) /= 2) .or. &
          (i > INActive + NAct .and. IGemIN(i) /= 3)) stop "AB_CAS_FOFO_GPU: unexpected IGemIN"
    end do
    ind(:, 1:NDimX) = IndN(:, 1:NDimX)
    dp = dev_alloc(int(NDimX, c_size_t) * NDimX)
    dm = dev_alloc(int(NDimX, c_size_t) * NDimX)
    call check(gc_ab_cas_fofo_ex(gpu_ctx, NBasis, INActive, NAct, NDimX, Occ, URe, XOne, ind, &
                                 RDM2Act, ffoo_dev, fofo_dev, ACAlpha, merge(1_c_int, 0_c_int, AB1), &
                                 dp, dm, ETot), "AB_CAS_FOFO")
    call from_dev(ABPLUS, dp, int(NDimX, c_size_t) * NDimX)
    call from_dev(ABMIN, dm, int(NDimX, c_size_t) * NDimX)
    call dev_free(dp); call dev_free(dm)
  end subroutine

  ! ERPASYMM1(EigVecR,Eig,APLSQRT,ABMIN,NBasis,NDimX), interpa.f:1652: APLSQRT holds
  ! A+ on entry and A+^1/2 on return; ABMIN is symmetrised in place.
  subroutine ERPASYMM1_GPU(EigVecR, Eig, APLSQRT, ABMIN, NBasis, NDimX)
    integer, intent(in) :: NBasis, NDimX
    real(c_double), intent(inout) :: APLSQRT(NDimX,NDimX), ABMIN(NDimX,NDimX)
    real(c_double), intent(out) :: EigVecR(NDimX*NDimX), Eig(NDimX)
    type(c_ptr) :: dp, dm, dy, de
    integer(c_size_t) :: nn
    call context()
    nn = int(NDimX, c_size_t) * NDimX
    dp = dev_alloc(nn); dm = dev_alloc(nn); dy = dev_alloc(nn); de = dev_alloc(int(NDimX, c_size_t))
    call to_dev(dp, APLSQRT, nn)
    call to_dev(dm, ABMIN, nn)
    call check(gc_erpasymm1(gpu_ctx, NDimX, dp, dm, dy, de), "ERPASYMM1")
    call from_dev(APLSQRT, dp, nn)
    call from_dev(ABMIN, dm, nn)
    call from_dev(EigVecR, dy, nn)
    call from_dev(Eig, de, int(NDimX, c_size_t))
    call dev_free(dp); call dev_free(dm); call dev_free(dy); call dev_free(de)
  end subroutine

  ! ACEneERPA_FOFO(ECorr,EVec,EVal,Occ,IGem,IndN,IndX,NOccup,NDimX,NBasis,IntKFile),
  ! abfofo.f90:3791-3792: IntKFile becomes the FOFO device buffer; NAct is the
  ! number of active orbitals (NOccup = INActive + NAct).
  subroutine ACENEERPA_FOFO_GPU(ECorr, EVec, EVal, Occ, IGem, IndN, IndX, NOccup, NDimX, NBasis, &
                                fofo_dev, NAct)
    integer, intent(in) :: NOccup, NDimX, NBasis, NAct
    integer, intent(in) :: IGem(NBasis), IndN(2,NDimX), IndX(NDimX)
    real(c_double), intent(in) :: EVec(NDimX*NDimX), EVal(NDimX), Occ(NBasis)
    type(c_ptr), intent(in) :: fofo_dev
    real(c_double), intent(out) :: ECorr
    integer(c_int) :: ind(2,NDimX)
    type(c_ptr) :: dy, de
    integer :: i
    call context()
    do i = 1, NDimX
      if (IndX(i) /= i) stop "ACENEERPA_FOFO_GPU: IndX must be the identity"
    end do
    if (IGem(1) < 1) stop "ACENEERPA_FOFO_GPU: unexpected IGem"
    ind(:, 1:NDimX) = IndN(:, 1:NDimX)
    dy = dev_alloc(int(NDimX, c_size_t) * NDimX)
    de = dev_alloc(int(NDimX, c_size_t))
    call to_dev(dy, EVec, int(NDimX, c_size_t) * NDimX)
    call to_dev(de, EVal, int(NDimX, c_size_t))
    call check(gc_ace_ne_erpa_fofo(gpu_ctx, NBasis, NOccup - NAct, NAct, NDimX, Occ, ind, dy, de, &
                                   fofo_dev, GC_PREC_FP64, ECorr), "ACEneERPA_FOFO")
    call dev_free(dy); call dev_free(de)
  end subroutine

end module gammcor_gpu
