!===============================================================================
! covof_gpu_bridge -- ISO_C_BINDING drop-in for the COVOF 2D Fortran driver.
!
! Forwards the two hot-path calls of a time step to libcovof_gpu.so
! (include/covof_gpu.h):
!   * sp_step_gpu(mesh, cfg, fields, dt, total_iters) replaces the body of
!     sim_solve_standard_projection (src/module_simulation.f90:2424-2666);
!     module_simulation.f90:559 calls it with (this%mesh, this%config,
!     this%fields, dt, total_iters) instead of this%solve_standard_projection.
!   * advect_vof_weymouth_yue_gpu(fields, mesh, cfg, dt) has the interface of
!     advect_vof_weymouth_yue (src/module_interface_vof.f90:1162-1166) and is
!     called from advect_vof (:802) in its place; the same subroutine runs the
!     CIAM or TVD transport when cfg%advection_method names it (:801-808).
!   * al_step_gpu(mesh, cfg, fields, dt, total_iters) replaces the Uzawa block
!     of the AUGMENTED_LAGRANGIAN / AAL branch (src/module_simulation.f90:
!     561-607).
!   * mono_step_gpu(mesh, cfg, fields, dt, total_iters) replaces the same
!     block for MONOLITHIC (one pass: assemble_preconditioner_blocks,
!     assemble_rhs, pack_vector, solve_linear_system, unpack_vector,
!     src/module_simulation.f90:552-583).
! The field arrays are contiguous allocatables dimensioned (0:nx+1, 0:ny+1),
! so their first elements are passed by reference with no copy-in.
!
! The handle (device buffers + stream) is created on the first call and
! re-created when the mesh size changes.  The Weymouth-Yue pass order is
! carried by the bridge's own step counter, which matches vof_step_count as
! long as every WY step goes through this bridge.
!
! Scope: one MPI rank, single domain; Euler or Gear, Picard or
! Adams-Bashforth; UPWIND / CENTERED / TVD_SUPERBEE convection; JACOBI,
! ILU0, SSOR or BLOCK_TRIANGULAR Krylov preconditioners; DIRICHLET or
! FREE_SLIP walls; no obstacle, markers, Newton linearisation or CAAL.
! Anything else stops with a message (the GPU path has no CPU fallback).
! The pressure Poisson runs the reference's own solver (SGS-PCG, 1e-7, 1000
! iterations) unless COVOF_GPU_POISSON asks for a faster one (make_params).
!===============================================================================
module covof_gpu_bridge
  use, intrinsic :: iso_c_binding
  use module_precision, only: dp
  use module_constants
  use module_mesh, only: mesh_2d_t
  use module_fields, only: flow_fields_t
  use module_config, only: config_t
  implicit none
  private

  public :: sp_step_gpu, advect_vof_weymouth_yue_gpu, al_step_gpu, mono_step_gpu, covof_gpu_finalize

  ! Mirror of covof_params (include/covof_gpu.h); bind(C) gives the C layout.
  type, bind(C) :: covof_params_t
     integer(c_int) :: nx, ny
     real(c_double) :: dx, dy
     integer(c_int) :: bc_type(4)
     real(c_double) :: bc_u(4), bc_v(4)
     integer(c_int) :: linear_solver, precond, use_precond, max_iter
     real(c_double) :: tol
     integer(c_int) :: enable_convection, convective_scheme
     integer(c_int) :: p_precond, p_max_iter, p_gauge, p_precision
     real(c_double) :: p_tol, p_inner_tol
     integer(c_int) :: p_inner_max_iter, p_max_refine
     integer(c_int) :: enable_two_phase, enable_surface_tension
     real(c_double) :: rho1, rho2, mu1, mu2, sigma, gx, gy
     integer(c_int) :: recon
     integer(c_int) :: p_inner_kind
     real(c_double) :: p_cheb_lo
     integer(c_int) :: p_mg_nu
     real(c_double) :: p_mg_cw
     integer(c_int) :: p_mg_tail
     integer(c_int) :: time_scheme
     integer(c_int) :: convective_linearization
     integer(c_int) :: enable_svof_smoothing
     real(c_double) :: svof_filter_width
     integer(c_int) :: enable_diffusion_smoothing
     integer(c_int) :: diffusion_smoothing_steps
     integer(c_int) :: advection_method
     integer(c_int) :: tvd_limiter
     integer(c_int) :: solver_type
     real(c_double) :: r_al
     integer(c_int) :: adaptative_al
     real(c_double) :: k_aal, l0_ref, t0_ref, u0_ref, p0_ref, ic_radius
     integer(c_int) :: uzawa_iter
     real(c_double) :: uzawa_tol
     integer(c_int) :: p_mg_nuc
  end type covof_params_t

  integer(c_int), parameter :: COVOF_OK = 0, COVOF_MAXITER = 1, COVOF_BREAKDOWN = 2
  ! Poisson arithmetic, preconditioner and inner kind codes (include/covof_gpu.h)
  integer(c_int), parameter :: COVOF_PREC_FP64 = 0, COVOF_PREC_MIXED = 1
  integer(c_int), parameter :: COVOF_PRECOND_JACOBI = 1, COVOF_PRECOND_SSOR = 2, COVOF_INNER_MG = 3
  integer(c_int), parameter :: COVOF_FIELD_U_NM1 = 14, COVOF_FIELD_V_NM1 = 15

  interface
     subroutine covof_params_default(p, nx, ny, lx, ly) bind(C, name="covof_params_default")
       import :: covof_params_t, c_int, c_double
       type(covof_params_t), intent(out) :: p
       integer(c_int), value :: nx, ny
       real(c_double), value :: lx, ly
     end subroutine covof_params_default

     integer(c_int) function covof_create(p, h) bind(C, name="covof_create")
       import :: covof_params_t, c_int, c_ptr
       type(covof_params_t), intent(in) :: p
       type(c_ptr), intent(out) :: h
     end function covof_create

     integer(c_int) function covof_destroy(h) bind(C, name="covof_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
     end function covof_destroy

     integer(c_int) function covof_sp_step(h, dt, u, v, p, rho_u, rho_v, mu, mu_node, &
                                           fx, fy, u_old, v_old, total_iters, relres) &
                                           bind(C, name="covof_sp_step")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       real(c_double), value :: dt
       real(c_double) :: u(*), v(*), p(*)
       real(c_double), intent(in) :: rho_u(*), rho_v(*), mu(*), mu_node(*), fx(*), fy(*)
       real(c_double), intent(in) :: u_old(*), v_old(*)
       integer(c_int), intent(out) :: total_iters
       real(c_double), intent(out) :: relres
     end function covof_sp_step

     integer(c_int) function covof_state_set(h, field, host) bind(C, name="covof_state_set")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       integer(c_int), value :: field
       real(c_double), intent(in) :: host(*)
     end function covof_state_set

     integer(c_int) function covof_set_has_nm1(h, has_nm1) bind(C, name="covof_set_has_nm1")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
       integer(c_int), value :: has_nm1
     end function covof_set_has_nm1

     integer(c_int) function covof_vof_wy_step(h, dt, x_first, u, v, c) &
                                               bind(C, name="covof_vof_wy_step")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       real(c_double), value :: dt
       integer(c_int), value :: x_first
       real(c_double), intent(in) :: u(*), v(*)
       real(c_double) :: c(*)
     end function covof_vof_wy_step

     integer(c_int) function covof_al_step(h, dt, u, v, p, rho, rho_u, rho_v, mu, mu_node, fx, fy, &
                                           u_old, v_old, total_iters, uzawa_done) bind(C, name="covof_al_step")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       real(c_double), value :: dt
       real(c_double) :: u(*), v(*), p(*)
       real(c_double), intent(in) :: rho(*), rho_u(*), rho_v(*), mu(*), mu_node(*), fx(*), fy(*)
       real(c_double), intent(in) :: u_old(*), v_old(*)
       integer(c_int), intent(out) :: total_iters, uzawa_done
     end function covof_al_step

     integer(c_int) function covof_monolithic_step(h, dt, u, v, p, rho_u, rho_v, mu, mu_node, fx, fy, &
                                                   u_old, v_old, iters) bind(C, name="covof_monolithic_step")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: h
       real(c_double), value :: dt
       real(c_double) :: u(*), v(*), p(*)
       real(c_double), intent(in) :: rho_u(*), rho_v(*), mu(*), mu_node(*), fx(*), fy(*)
       real(c_double), intent(in) :: u_old(*), v_old(*)
       integer(c_int), intent(out) :: iters
     end function covof_monolithic_step

     type(c_ptr) function covof_strerror(status) bind(C, name="covof_strerror")
       import :: c_int, c_ptr
       integer(c_int), value :: status
     end function covof_strerror
  end interface

  type(c_ptr), save :: handle = c_null_ptr
  integer, save :: handle_nx = -1, handle_ny = -1
  integer, save :: wy_step_count = 0

contains

  subroutine fail(where, status)
    character(len=*), intent(in) :: where
    integer(c_int), intent(in) :: status
    write(*, '(A,A,A,I0)') "covof_gpu_bridge: ", where, " failed, status ", status
    error stop 1
  end subroutine fail

  ! config_t (src/module_config.f90:31-184) -> covof_params
  subroutine make_params(mesh, cfg, p)
    type(mesh_2d_t), intent(in) :: mesh
    type(config_t), intent(in) :: cfg
    type(covof_params_t), intent(out) :: p
    character(len=32) :: choice
    integer :: env_st

    if (mesh%size /= 1) then
       write(*, '(A)') "covof_gpu_bridge: the GPU path runs one single-domain rank"
       error stop 1
    end if
    if (cfg%convective_linearization == CONV_LIN_NEWTON .or. &
        cfg%obs_enabled .or. cfg%enable_ssp_rk3_momentum .or. cfg%compressible .or. &
        cfg%use_markers .or. cfg%solver_type == SOLVER_CAAL) then
       write(*, '(A)') "covof_gpu_bridge: option outside the GPU path (no Newton/obstacle/markers/CAAL)"
       error stop 1
    end if
    call covof_params_default(p, int(mesh%nx_global, c_int), int(mesh%ny_global, c_int), &
                              real(mesh%lx, c_double), real(mesh%ly, c_double))
    p%dx = mesh%dx
    p%dy = mesh%dy
    p%bc_type = [cfg%bc_left%btype, cfg%bc_right%btype, cfg%bc_bottom%btype, cfg%bc_top%btype]
    p%bc_u = [cfg%bc_left%u, cfg%bc_right%u, cfg%bc_bottom%u, cfg%bc_top%u]
    p%bc_v = [cfg%bc_left%v, cfg%bc_right%v, cfg%bc_bottom%v, cfg%bc_top%v]
    p%linear_solver = cfg%linear_solver
    p%precond = cfg%precond_type
    p%use_precond = merge(1_c_int, 0_c_int, cfg%use_precond)
    p%max_iter = cfg%max_iter
    p%tol = cfg%tol
    p%enable_convection = merge(1_c_int, 0_c_int, cfg%enable_convection)
    p%convective_scheme = cfg%convective_scheme
    p%time_scheme = cfg%time_scheme
    p%convective_linearization = cfg%convective_linearization
    ! transport and interface smoothing (the smoothing itself stays in the
    ! Fortran advect_vof; the GPU entry points accept it too)
    select case (trim(cfg%advection_method))
    case ("WEYMOUTH_YUE")
       p%advection_method = 0
    case ("CIAM")
       p%advection_method = 1
    case default
       p%advection_method = 2
    end select
    select case (trim(cfg%tvd_limiter))
    case ("VAN_LEER")
       p%tvd_limiter = 1
    case ("MUSCL")
       p%tvd_limiter = 2
    case ("HRIC")
       p%tvd_limiter = 3
    case default
       p%tvd_limiter = 0
    end select
    p%enable_svof_smoothing = merge(1_c_int, 0_c_int, cfg%enable_svof_smoothing)
    p%svof_filter_width = cfg%svof_filter_width
    p%enable_diffusion_smoothing = merge(1_c_int, 0_c_int, cfg%enable_diffusion_smoothing)
    p%diffusion_smoothing_steps = cfg%diffusion_smoothing_steps
    ! coupling (src/module_config.f90:159-168)
    p%solver_type = cfg%solver_type
    p%r_al = cfg%r_al
    p%adaptative_al = merge(1_c_int, 0_c_int, cfg%adaptative_al)
    p%k_aal = cfg%k_aal
    p%l0_ref = cfg%l0_ref; p%t0_ref = cfg%t0_ref; p%u0_ref = cfg%u0_ref; p%p0_ref = cfg%p0_ref
    p%ic_radius = cfg%ic_radius
    p%uzawa_iter = cfg%uzawa_iter
    p%uzawa_tol = cfg%uzawa_tol
    ! Poisson: the reference's hard-coded tolerance and cap
    ! (src/module_simulation.f90:2437-2438) and, by default, its solver: PCG
    ! with the symmetric Gauss-Seidel sweep pair (poisson_ssor, :2709-2758),
    ! in FP64, so that the drop-in returns the reference's pressure.  The
    ! environment variable COVOF_GPU_POISSON picks a faster solver for the
    ! same system and stopping test instead: "jacobi" (FP64 Jacobi-PCG, the
    ! fused persistent kernel) or "mixed" (FP64 flexible CG on the true
    ! residual with an FP32 multigrid V-cycle; no iteration cap of 1000
    ! V-cycles is ever reached).  Both stop at the same ||r||/||b|| <= 1e-7,
    ! so their pressure differs from the reference's by the solvers'
    ! different truncation errors, not by more than the tolerance allows.
    p%p_tol = 1.0e-7_c_double
    p%p_max_iter = 1000
    p%p_precision = COVOF_PREC_FP64
    p%p_precond = COVOF_PRECOND_SSOR
    call get_environment_variable("COVOF_GPU_POISSON", choice, status=env_st)
    if (env_st == 0) then
       select case (trim(choice))
       case ("jacobi")
          p%p_precond = COVOF_PRECOND_JACOBI
       case ("mixed")
          p%p_precond = COVOF_PRECOND_JACOBI
          p%p_precision = COVOF_PREC_MIXED
          p%p_inner_kind = COVOF_INNER_MG
       case ("reference")
       case default
          write(*, '(A)') "covof_gpu_bridge: COVOF_GPU_POISSON is reference, jacobi or mixed"
          error stop 1
       end select
    end if
    p%enable_two_phase = merge(1_c_int, 0_c_int, cfg%enable_two_phase)
    p%enable_surface_tension = merge(1_c_int, 0_c_int, cfg%enable_surface_tension)
    p%rho1 = cfg%rho1; p%rho2 = cfg%rho2; p%mu1 = cfg%mu1; p%mu2 = cfg%mu2
    p%sigma = cfg%sigma; p%gx = cfg%gx; p%gy = cfg%gy
    if (trim(cfg%reconstruction_method) == "ELVIRA") then
       p%recon = 1
    else
       p%recon = 0
    end if
  end subroutine make_params

  subroutine ensure_handle(mesh, cfg)
    type(mesh_2d_t), intent(in) :: mesh
    type(config_t), intent(in) :: cfg
    type(covof_params_t) :: p
    integer(c_int) :: st
    if (c_associated(handle) .and. handle_nx == mesh%nx_local .and. handle_ny == mesh%ny_local) return
    if (c_associated(handle)) st = covof_destroy(handle)
    call make_params(mesh, cfg, p)
    st = covof_create(p, handle)
    if (st /= COVOF_OK) call fail("covof_create", st)
    handle_nx = mesh%nx_local
    handle_ny = mesh%ny_local
  end subroutine ensure_handle

  ! Drop-in for sim_solve_standard_projection (src/module_simulation.f90:2424-2666).
  subroutine sp_step_gpu(mesh, cfg, fields, dt, total_iters)
    type(mesh_2d_t), intent(in) :: mesh
    type(config_t), intent(in) :: cfg
    type(flow_fields_t), intent(inout) :: fields
    real(dp), intent(in) :: dt
    integer, intent(out) :: total_iters
    integer(c_int) :: st, it
    real(c_double) :: rr
    call ensure_handle(mesh, cfg)
    ! Gear / BDF2 and Adams-Bashforth read the n-1 history (fields%u_nm1,
    ! has_nm1, set by the loop at src/module_simulation.f90:508-520)
    if (cfg%time_scheme == TIME_SCHEME_GEAR .or. cfg%convective_linearization == CONV_LIN_ADAMS_BASHFORTH) then
       st = covof_state_set(handle, COVOF_FIELD_U_NM1, fields%u_nm1)
       if (st == COVOF_OK) st = covof_state_set(handle, COVOF_FIELD_V_NM1, fields%v_nm1)
       if (st == COVOF_OK) st = covof_set_has_nm1(handle, merge(1_c_int, 0_c_int, fields%has_nm1))
       if (st /= COVOF_OK) call fail("covof_state_set", st)
    end if
    st = covof_sp_step(handle, real(dt, c_double), fields%u, fields%v, fields%p, &
                       fields%rho_u, fields%rho_v, fields%mu, fields%mu_node, &
                       fields%fx_sigma, fields%fy_sigma, fields%u_old, fields%v_old, it, rr)
    ! The reference continues silently after MAXITER / BREAKDOWN
    ! (src/module_linear_solvers.f90:565,576); so does the bridge.
    if (st /= COVOF_OK .and. st /= COVOF_MAXITER .and. st /= COVOF_BREAKDOWN) call fail("covof_sp_step", st)
    total_iters = it
  end subroutine sp_step_gpu

  ! Drop-in for advect_vof_weymouth_yue (src/module_interface_vof.f90:1162-1377).
  subroutine advect_vof_weymouth_yue_gpu(fields, mesh, cfg, dt)
    type(flow_fields_t), intent(inout) :: fields
    type(mesh_2d_t), intent(in) :: mesh
    type(config_t), intent(in) :: cfg
    real(dp), intent(in) :: dt
    integer(c_int) :: st, x_first
    call ensure_handle(mesh, cfg)
    x_first = merge(1_c_int, 0_c_int, mod(wy_step_count, 2) == 0)
    st = covof_vof_wy_step(handle, real(dt, c_double), x_first, fields%u, fields%v, fields%C)
    if (st /= COVOF_OK) call fail("covof_vof_wy_step", st)
    wy_step_count = wy_step_count + 1
  end subroutine advect_vof_weymouth_yue_gpu

  ! Drop-in for the AUGMENTED_LAGRANGIAN / AAL branch of the loop body
  ! (src/module_simulation.f90:546-607): the GPU step builds the penalty
  ! field and the preconditioner diagonal and runs the Uzawa iterations.
  subroutine al_step_gpu(mesh, cfg, fields, dt, total_iters)
    type(mesh_2d_t), intent(in) :: mesh
    type(config_t), intent(in) :: cfg
    type(flow_fields_t), intent(inout) :: fields
    real(dp), intent(in) :: dt
    integer, intent(out) :: total_iters
    integer(c_int) :: st, it, ud
    call ensure_handle(mesh, cfg)
    if (cfg%time_scheme == TIME_SCHEME_GEAR .or. cfg%convective_linearization == CONV_LIN_ADAMS_BASHFORTH) then
       st = covof_state_set(handle, COVOF_FIELD_U_NM1, fields%u_nm1)
       if (st == COVOF_OK) st = covof_state_set(handle, COVOF_FIELD_V_NM1, fields%v_nm1)
       if (st == COVOF_OK) st = covof_set_has_nm1(handle, merge(1_c_int, 0_c_int, fields%has_nm1))
       if (st /= COVOF_OK) call fail("covof_state_set", st)
    end if
    st = covof_al_step(handle, real(dt, c_double), fields%u, fields%v, fields%p, fields%rho, &
                       fields%rho_u, fields%rho_v, fields%mu, fields%mu_node, &
                       fields%fx_sigma, fields%fy_sigma, fields%u_old, fields%v_old, it, ud)
    if (st /= COVOF_OK .and. st /= COVOF_MAXITER .and. st /= COVOF_BREAKDOWN) call fail("covof_al_step", st)
    total_iters = it
  end subroutine al_step_gpu

  ! Drop-in for the MONOLITHIC branch of the loop body (src/module_simulation.f90:
  ! 552-583, uzawa_max = 1): the coupled (u, v, p) solve on the GPU.
  subroutine mono_step_gpu(mesh, cfg, fields, dt, total_iters)
    type(mesh_2d_t), intent(in) :: mesh
    type(config_t), intent(in) :: cfg
    type(flow_fields_t), intent(inout) :: fields
    real(dp), intent(in) :: dt
    integer, intent(out) :: total_iters
    integer(c_int) :: st, it
    call ensure_handle(mesh, cfg)
    if (cfg%time_scheme == TIME_SCHEME_GEAR .or. cfg%convective_linearization == CONV_LIN_ADAMS_BASHFORTH) then
       st = covof_state_set(handle, COVOF_FIELD_U_NM1, fields%u_nm1)
       if (st == COVOF_OK) st = covof_state_set(handle, COVOF_FIELD_V_NM1, fields%v_nm1)
       if (st == COVOF_OK) st = covof_set_has_nm1(handle, merge(1_c_int, 0_c_int, fields%has_nm1))
       if (st /= COVOF_OK) call fail("covof_state_set", st)
    end if
    st = covof_monolithic_step(handle, real(dt, c_double), fields%u, fields%v, fields%p, &
                               fields%rho_u, fields%rho_v, fields%mu, fields%mu_node, &
                               fields%fx_sigma, fields%fy_sigma, fields%u_old, fields%v_old, it)
    if (st /= COVOF_OK .and. st /= COVOF_MAXITER .and. st /= COVOF_BREAKDOWN) call fail("covof_monolithic_step", st)
    total_iters = it
  end subroutine mono_step_gpu

  subroutine covof_gpu_finalize()
    integer(c_int) :: st
    if (c_associated(handle)) st = covof_destroy(handle)
    handle = c_null_ptr
  end subroutine covof_gpu_finalize

end module covof_gpu_bridge
