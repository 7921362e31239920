! surfatt_gpu.f90 -- ISO_C_BINDING interface of libsurfatt_gb300.so for the
! reference's Fortran drivers (forward_simulate, src/acqui.f90:91-161 and
! src/tomo2d.f90:158-201).
!
! NOT COMPILED in this repository: no Fortran compiler exists on the build
! machine or on the GPU machine.  tests/test_capi_cpu.py checks, with a C
! compiler, that the derived types below match the C structs of
! include/surfatt_gb300.h field by field (names, order, kinds and offsets).
!
! The unchanged drivers need none of this: they reach the drop-in symbols
! (fsm_uw_ps_lonlat_2d_, fsm_o1_jse_lonlat_2d_, mask_, ...) at link time.
! This module is for a driver that hands a whole gradient evaluation to the
! batched engine:
!
!   use surfatt_gpu
!   type(c_ptr) :: eng
!   type(surfatt_problem_t) :: pb     ! c_loc of period-slowest copies
!   type(surfatt_result_t) :: res     ! c_loc of the output arrays
!   ierr = surfatt_engine_create(eng, 0_c_int, 0_c_size_t)
!   ierr = surfatt_engine_load(eng, pb)                 ! once per inversion
!   ierr = surfatt_engine_update_velocity(eng, svel)    ! per iterate / trial
!   ierr = surfatt_engine_run(eng, SURFATT_MODE_3D, SURFATT_PREC_FP32)
!   ierr = surfatt_engine_results(eng, res)             ! waits for the run
!   call surfatt_engine_destroy(eng)
!
! The reference stores svel, m11, m12, m22 as (nperiod, nx, ny) with the
! period fastest (src/grid.f90:25-33); the engine wants each period's
! (nx, ny) plane contiguous (period slowest) -- transpose on the way in and
! out.  The MPI reductions after the loop (src/acqui.f90:152-160, 205-206)
! stay as they are; with one GPU per rank each rank loads its own block of
! the work list.
module surfatt_gpu
  use iso_c_binding
  implicit none

  enum, bind(c)
    enumerator :: SURFATT_OK = 0, SURFATT_SOURCE_ON_BOUNDARY = 1, SURFATT_BAD_ARG = 2
    enumerator :: SURFATT_NOT_CONVERGED = 3, SURFATT_OOM = 4, SURFATT_CUDA_ERROR = 5
    enumerator :: SURFATT_TIMEOUT = 6
  end enum
  enum, bind(c)
    enumerator :: SURFATT_MODE_FORWARD = 0, SURFATT_MODE_2D = 2, SURFATT_MODE_3D = 3
  end enum
  enum, bind(c)
    enumerator :: SURFATT_PREC_FP64 = 0, SURFATT_PREC_FP32 = 1
  end enum

  ! surfatt_problem_t (include/surfatt_gb300.h): one field per line, in the
  ! C struct's order
  type, bind(c) :: surfatt_problem_t
    integer(c_int) :: nperiod
    type(c_ptr) :: nx
    type(c_ptr) :: ny
    type(c_ptr) :: xoff
    type(c_ptr) :: yoff
    type(c_ptr) :: goff
    type(c_ptr) :: xgrid
    type(c_ptr) :: ygrid
    type(c_ptr) :: svel
    type(c_ptr) :: m11
    type(c_ptr) :: m12
    type(c_ptr) :: m22
    integer(c_int) :: nsolve
    type(c_ptr) :: pidx
    type(c_ptr) :: srcx
    type(c_ptr) :: srcy
    type(c_ptr) :: rec_off
    type(c_ptr) :: nrec
    type(c_ptr) :: recx
    type(c_ptr) :: recy
    type(c_ptr) :: tt
    type(c_ptr) :: weight
    type(c_ptr) :: path
    integer(c_int) :: npath
  end type surfatt_problem_t

  ! surfatt_result_t (include/surfatt_gb300.h)
  type, bind(c) :: surfatt_result_t
    type(c_ptr) :: adj_s
    type(c_ptr) :: adj_density
    type(c_ptr) :: chi
    type(c_ptr) :: tt_fwd
    type(c_ptr) :: status
    type(c_ptr) :: fwd_iters
    type(c_ptr) :: adj_iters
  end type surfatt_result_t

  interface
    integer(c_int) function surfatt_engine_create(eng, device, budget) &
        bind(c, name="surfatt_engine_create")
      import :: c_ptr, c_int, c_size_t
      type(c_ptr), intent(out) :: eng
      integer(c_int), value :: device
      integer(c_size_t), value :: budget
    end function

    integer(c_int) function surfatt_engine_load(eng, pb) bind(c, name="surfatt_engine_load")
      import :: c_ptr, c_int, surfatt_problem_t
      type(c_ptr), value :: eng
      type(surfatt_problem_t), intent(in) :: pb
    end function

    integer(c_int) function surfatt_engine_update_velocity(eng, svel) &
        bind(c, name="surfatt_engine_update_velocity")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: eng
      real(c_double), intent(in) :: svel(*)
    end function

    integer(c_int) function surfatt_engine_run(eng, mode, prec) bind(c, name="surfatt_engine_run")
      import :: c_ptr, c_int
      type(c_ptr), value :: eng
      integer(c_int), value :: mode, prec
    end function

    integer(c_int) function surfatt_engine_sync(eng) bind(c, name="surfatt_engine_sync")
      import :: c_ptr, c_int
      type(c_ptr), value :: eng
    end function

    integer(c_int) function surfatt_engine_results(eng, res) &
        bind(c, name="surfatt_engine_results")
      import :: c_ptr, c_int, surfatt_result_t
      type(c_ptr), value :: eng
      type(surfatt_result_t), intent(in) :: res
    end function

    integer(c_int) function surfatt_engine_smooth(eng, sigma, ker_s) &
        bind(c, name="surfatt_engine_smooth")
      import :: c_ptr, c_int, c_double
      type(c_ptr), value :: eng
      real(c_double), value :: sigma
      real(c_double), intent(out) :: ker_s(*)
    end function

    subroutine surfatt_engine_destroy(eng) bind(c, name="surfatt_engine_destroy")
      import :: c_ptr
      type(c_ptr), value :: eng
    end subroutine

    integer(c_int) function surfatt_last_status() bind(c, name="surfatt_last_status")
      import :: c_int
    end function

    subroutine surfatt_set_exit_on_boundary(enable) bind(c, name="surfatt_set_exit_on_boundary")
      import :: c_int
      integer(c_int), value :: enable
    end subroutine
  end interface
end module surfatt_gpu
