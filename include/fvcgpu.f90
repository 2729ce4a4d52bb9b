! fvcgpu.f90 -- Fortran 2003 (ISO_C_BINDING) interface to libfvcgpu.so.
!
! Two ways for the fortranFVCell Fortran host to reach the GPU solver:
!  1. leave src/Solver.f out of the build and link libfvcgpu.so: the
!     library exports `solver_`, the gfortran name of the reference's
!     `subroutine solver(ad,au,al,x,b,iax,ja,neq,nad,unsym,tol,maxit,
!     code,matriz,nlit)`, so the existing calls in Simple.f/Transporte.f
!     resolve to it unchanged;
!  2. `use fvcgpu` and call fvc_solver / fvc_solver_ex explicitly.
! LOGICAL unsym is passed as a 4-byte integer (gfortran's LOGICAL(4)).
module fvcgpu
  use iso_c_binding
  implicit none

  integer(c_int32_t), parameter :: FVC_OK = 0, FVC_ERR_NOCONV = 1, &
       FVC_ERR_BREAKDOWN = 2, FVC_ERR_NAN = 3, FVC_ERR_UNSUPPORTED = 4, &
       FVC_ERR_CUDA = 5, FVC_ERR_ARG = 6, FVC_ERR_TIMEOUT = 7
  integer(c_int32_t), parameter :: FVC_PREC_FP64 = 0, FVC_PREC_MIXED = 1

  type, bind(C) :: fvc_opts
     integer(c_int32_t) :: precision
     integer(c_int32_t) :: init
     real(c_double)     :: refine_tol
     real(c_double)     :: inner_tol
     integer(c_int32_t) :: max_refine
     integer(c_int32_t) :: block_threads
     integer(c_int32_t) :: blocks_per_sm
     integer(c_int32_t) :: stop_rule
     integer(c_int32_t) :: want_residual
     integer(c_int32_t) :: update_beta
     integer(c_int32_t) :: staging
     integer(c_int32_t) :: max_blocks
  end type fvc_opts

  type, bind(C) :: fvc_stats
     integer(c_int32_t) :: status
     integer(c_int32_t) :: iterations
     integer(c_int32_t) :: inner_iterations
     integer(c_int32_t) :: refinements
     real(c_double)     :: energy
     real(c_double)     :: conv
     real(c_double)     :: final_crit
     real(c_double)     :: rel_residual
     real(c_double)     :: solve_ms
  end type fvc_stats

  interface
     ! drop-in replacement of src/Solver.f:28-29 (all arguments by reference)
     subroutine fvc_solver(ad, au, al, x, b, iax, ja, neq, nad, unsym, tol, &
          maxit, code, matriz, nlit) bind(C, name="fvc_solver")
       import :: c_double, c_int32_t
       real(c_double)     :: ad(*), au(*), al(*), x(*), b(*)
       integer(c_int32_t) :: iax(*), ja(*)
       integer(c_int32_t) :: neq, nad, unsym, maxit, code, matriz, nlit
       real(c_double)     :: tol
     end subroutine fvc_solver

     subroutine fvc_opts_default(opts) bind(C, name="fvc_opts_default")
       import :: fvc_opts
       type(fvc_opts) :: opts
     end subroutine fvc_opts_default

     ! explicit options and statistics; never stops the program
     integer(c_int32_t) function fvc_solver_ex(ad, au, al, x, b, iax, ja, neq, &
          nad, unsym, tol, maxit, code, matriz, opts, stats) &
          bind(C, name="fvc_solver_ex")
       import :: c_double, c_int32_t, fvc_opts, fvc_stats
       real(c_double)     :: ad(*), au(*), al(*), x(*), b(*)
       integer(c_int32_t) :: iax(*), ja(*)
       integer(c_int32_t), value :: neq, nad, unsym, maxit, code, matriz
       real(c_double), value     :: tol
       type(fvc_opts)     :: opts
       type(fvc_stats)    :: stats
     end function fvc_solver_ex
  end interface
end module fvcgpu
