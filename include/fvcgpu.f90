! fvcgpu.f90 -- Fortran 2003 (ISO_C_BINDING) interface to libfvcgpu.so.
!
! Two ways for the fortranFVCell Fortran host to reach the GPU solver:
!  1. leave src/Solver.f out of the build and link libfvcgpu.so: the
!     library exports `solver_`, the gfortran name of the reference's
!     `subroutine solver(ad,au,al,x,b,iax,ja,neq,nad,unsym,tol,maxit,
!     code,matriz,nlit)`, so the existing calls in Simple.f/Transporte.f
!     resolve to it unchanged;
!  2. `use fvcgpu` and call fvc_solver / fvc_solver_ex explicitly;
!  3. hand the whole SIMPLE outer iteration to the GPU (fvc_simple_*): the
!     mesh arrays as Simple.f holds them (x, ix with the material last,
!     nelcon, num, pedge, sedge, e) go up once, each call runs outer
!     iterations on the device and returns the residual norms.
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
     integer(c_int32_t) :: fp32_layout
     integer(c_int32_t) :: cluster_size
  end type fvc_opts

  ! options of the SIMPLE outer iteration (fvc_simple_opts in fvcgpu.h)
  type, bind(C) :: fvc_simple_opts
     real(c_double)     :: dt, under_u, under_pc
     integer(c_int32_t) :: simple_c, bs, int_vel, matriz_u, code_u
     real(c_double)     :: tol_u
     integer(c_int32_t) :: matriz_pc, code_pc
     real(c_double)     :: tol_pc
     integer(c_int32_t) :: maxit, precision, precision_u
  end type fvc_simple_opts

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

     ! after each solve fn(line, user) receives the reference's unit-13
     ! line (a NUL-terminated C string); c_null_funptr turns it off
     subroutine fvc_set_solver_log(fn, user) bind(C, name="fvc_set_solver_log")
       import :: c_funptr, c_ptr
       type(c_funptr), value :: fn
       type(c_ptr), value    :: user
     end subroutine fvc_set_solver_log

     ! ---- the SIMPLE outer iteration on the GPU (fvc_simple_* of fvcgpu.h)
     subroutine fvc_simple_opts_default(opts) bind(C, name="fvc_simple_opts_default")
       import :: fvc_simple_opts
       type(fvc_simple_opts) :: opts
     end subroutine fvc_simple_opts_default

     ! s receives the loop handle; x(2,nnode), ix(nshared+1,numel),
     ! nelcon(nshared,numel), num(numel), pedge(nshared+1,numel),
     ! sedge(3,nshared+1,numel), e(10,nmat) as in Simple.f
     integer(c_int32_t) function fvc_simple_create(s, device, numel, nnode, &
          nshared, nmat, x, ix, nelcon, num, pedge, sedge, e, opts) &
          bind(C, name="fvc_simple_create")
       import :: c_ptr, c_double, c_int32_t, fvc_simple_opts
       type(c_ptr)                  :: s
       integer(c_int32_t), value    :: device, numel, nnode, nshared, nmat
       real(c_double)               :: x(*), sedge(*), e(*)
       integer(c_int32_t)           :: ix(*), nelcon(*), num(*), pedge(*)
       type(fvc_simple_opts)        :: opts
     end function fvc_simple_create

     ! nit outer iterations; res(3,nit) the cell-residual norms of u1, u2,
     ! p' and its(3,nit) the solver iterations (0: not solved)
     integer(c_int32_t) function fvc_simple_iterate(s, nit, res, its) &
          bind(C, name="fvc_simple_iterate")
       import :: c_ptr, c_double, c_int32_t
       type(c_ptr), value        :: s
       integer(c_int32_t), value :: nit
       real(c_double)            :: res(*)
       integer(c_int32_t)        :: its(*)
     end function fvc_simple_iterate

     ! on = 1: one CUDA graph launch per outer iteration (same results)
     integer(c_int32_t) function fvc_simple_set_graph(s, on) &
          bind(C, name="fvc_simple_set_graph")
       import :: c_ptr, c_int32_t
       type(c_ptr), value        :: s
       integer(c_int32_t), value :: on
     end function fvc_simple_set_graph

     ! the system the last outer iteration solved: which 1 u1, 2 u2, 3 p',
     ! 4 enthalpy; ad(numel), au(nja), b(numel) in equation order (c_loc of
     ! the arrays, or c_null_ptr); nja receives the length of au
     integer(c_int32_t) function fvc_simple_system(s, which, ad, au, b, nja) &
          bind(C, name="fvc_simple_system")
       import :: c_ptr, c_int32_t, c_int64_t
       type(c_ptr), value        :: s
       integer(c_int32_t), value :: which
       type(c_ptr), value        :: ad, au, b
       integer(c_int64_t)        :: nja
     end function fvc_simple_system

     integer(c_int32_t) function fvc_simple_time_step(s) &
          bind(C, name="fvc_simple_time_step")
       import :: c_ptr, c_int32_t
       type(c_ptr), value :: s
     end function fvc_simple_time_step

     ! ideal gas with the energy equation: pedgeE / sedgeE (nshared+1,numel),
     ! gravity (gx, gy), initial temperature t0
     integer(c_int32_t) function fvc_simple_energy(s, pedge_e, sedge_e, gx, gy, &
          t0) bind(C, name="fvc_simple_energy")
       import :: c_ptr, c_double, c_int32_t
       type(c_ptr), value        :: s
       integer(c_int32_t)        :: pedge_e(*)
       real(c_double)            :: sedge_e(*)
       real(c_double), value     :: gx, gy, t0
     end function fvc_simple_energy

     ! res(4,nit), its(4,nit): u1, u2, p', enthalpy
     integer(c_int32_t) function fvc_simple_iterate_energy(s, nit, res, its) &
          bind(C, name="fvc_simple_iterate_energy")
       import :: c_ptr, c_double, c_int32_t
       type(c_ptr), value        :: s
       integer(c_int32_t), value :: nit
       real(c_double)            :: res(*)
       integer(c_int32_t)        :: its(*)
     end function fvc_simple_iterate_energy

     ! w(2,numel), p(numel) to the host; c_loc() of an array or c_null_ptr
     integer(c_int32_t) function fvc_simple_fields(s, w, p) &
          bind(C, name="fvc_simple_fields")
       import :: c_ptr, c_int32_t
       type(c_ptr), value :: s, w, p
     end function fvc_simple_fields

     integer(c_int32_t) function fvc_simple_set_fields(s, w, p) &
          bind(C, name="fvc_simple_set_fields")
       import :: c_ptr, c_int32_t
       type(c_ptr), value :: s, w, p
     end function fvc_simple_set_fields

     ! the restart state saveSimple writes: w, w0, p, en, en0, ro(3,numel)
     integer(c_int32_t) function fvc_simple_get_state(s, w, w0, p, en, en0, ro) &
          bind(C, name="fvc_simple_get_state")
       import :: c_ptr, c_int32_t
       type(c_ptr), value :: s, w, w0, p, en, en0, ro
     end function fvc_simple_get_state

     integer(c_int32_t) function fvc_simple_set_state(s, w, w0, p, en, en0, ro) &
          bind(C, name="fvc_simple_set_state")
       import :: c_ptr, c_int32_t
       type(c_ptr), value :: s, w, w0, p, en, en0, ro
     end function fvc_simple_set_state

     integer(c_int32_t) function fvc_simple_destroy(s) &
          bind(C, name="fvc_simple_destroy")
       import :: c_ptr, c_int32_t
       type(c_ptr), value :: s
     end function fvc_simple_destroy
  end interface
end module fvcgpu
