!> fen_gpu_mod: iso_c_binding interfaces of libfen_gb300.so (C ABI: include/fen_gpu.h).
!>
!> One interface per C entry point, argument for argument.  Host field arrays are passed as
!> assumed-size real(c_double) dummies, so FEN's contiguous allocatable arrays go in directly
!> (e.g. fen_upload(fen_ctx, FEN_U, v%x%f)); the library reads or writes them during the call
!> only.  Error codes are negative; fen_check prints the library's message and stops, as FEN
!> does on an unsupported configuration (src/IO.f90:12-30, src/poisson.f90:92-94).
!>
!> Standalone: needs only iso_c_binding.  FEN's own modules are used by fen_gpu_route.f90.
module fen_gpu_mod

    use, intrinsic :: iso_c_binding
    implicit none

    ! physical boundary conditions (grid.f90:41-46) and faces (scalar.f90:24-36)
    integer(c_int), parameter :: FEN_BC_PERIODIC = 0, FEN_BC_WALL = 1, FEN_BC_INFLOW = 2, &
                                 FEN_BC_OUTFLOW = 3
    integer(c_int), parameter :: FEN_LEFT = 0, FEN_RIGHT = 1, FEN_BOTTOM = 2, FEN_TOP = 3, &
                                 FEN_FRONT = 4, FEN_BACK = 5
    ! fields (navier_stokes_mod module state, navier_stokes.f90:36-37; multiphase.f90:25)
    integer(c_int), parameter :: FEN_U = 0, FEN_V = 1, FEN_W = 2, FEN_P = 3, FEN_PHI = 4, &
                                 FEN_DVO_X = 5, FEN_DVO_Y = 6, FEN_DVO_Z = 7, &
                                 FEN_S_X = 8, FEN_S_Y = 9, FEN_S_Z = 10, &
                                 FEN_RHO = 11, FEN_MU = 12, FEN_P_O = 13
    integer(c_int), parameter :: FEN_FP64 = 0, FEN_MIXED = 1
    integer(c_int), parameter :: FEN_OK = 0, FEN_ERR_ARG = -1, FEN_ERR_BC = -2, FEN_ERR_CUDA = -3, &
                                 FEN_ERR_NAN = -4, FEN_ERR_NOMEM = -5, FEN_ERR_STATE = -6

    type, bind(C) :: fen_params
        integer(c_int) :: dim, nx, ny, nz
        real(c_double) :: lx, ly, lz, origin(3)
        integer(c_int) :: bc(6), aniso
        real(c_double) :: density, viscosity, g(3), cfl
        integer(c_int) :: constant_cfl, precision, refine
    end type fen_params

    type, bind(C) :: fen_status
        real(c_double) :: dt, dt_o, maxdiv, maxcfl, maxvel, dt_visc
        integer(c_int) :: nan_detected, poisson_solver
    end type fen_status

    interface
        ! ---- context, transfers, boundary conditions ----------------------------------------
        integer(c_int) function fen_ctx_create(params, ctx) bind(C, name='fen_ctx_create')
            import :: c_int, c_ptr, fen_params
            type(fen_params), intent(in) :: params
            type(c_ptr), intent(out) :: ctx
        end function fen_ctx_create
        integer(c_int) function fen_ctx_destroy(ctx) bind(C, name='fen_ctx_destroy')
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
        end function fen_ctx_destroy
        type(c_ptr) function fen_last_error() bind(C, name='fen_last_error')
            import :: c_ptr
        end function fen_last_error
        integer(c_int) function fen_upload(ctx, field, host) bind(C, name='fen_upload')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: field
            real(c_double), intent(in) :: host(*)
        end function fen_upload
        integer(c_int) function fen_download(ctx, field, host) bind(C, name='fen_download')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: field
            real(c_double), intent(inout) :: host(*)
        end function fen_download
        integer(c_int) function fen_upload_gl(ctx, field, host, gl) bind(C, name='fen_upload_gl')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: field, gl
            real(c_double), intent(in) :: host(*)
        end function fen_upload_gl
        integer(c_int) function fen_download_gl(ctx, field, host, gl) bind(C, name='fen_download_gl')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: field, gl
            real(c_double), intent(inout) :: host(*)
        end function fen_download_gl
        integer(c_int) function fen_field_bounds(ctx, field, lo, hi) bind(C, name='fen_field_bounds')
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
            integer(c_int), value :: field
            integer(c_int), intent(out) :: lo(3), hi(3)
        end function fen_field_bounds
        integer(c_int) function fen_update_ghost_nodes(ctx, field) bind(C, name='fen_update_ghost_nodes')
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
            integer(c_int), value :: field
        end function fen_update_ghost_nodes
        integer(c_int) function fen_set_bc_values(ctx, field, face, values) bind(C, name='fen_set_bc_values')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: field, face
            real(c_double), intent(in) :: values(*)
        end function fen_set_bc_values
        integer(c_int) function fen_set_bc_type(ctx, field, face, btype) bind(C, name='fen_set_bc_type')
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
            integer(c_int), value :: field, face, btype
        end function fen_set_bc_type

        ! ---- time step --------------------------------------------------------------------
        integer(c_int) function fen_set_timestep(ctx, U, dt) bind(C, name='fen_set_timestep')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), value :: U
            real(c_double), intent(out) :: dt
        end function fen_set_timestep
        integer(c_int) function fen_set_dt_o(ctx, dt_o) bind(C, name='fen_set_dt_o')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), value :: dt_o
        end function fen_set_dt_o
        integer(c_int) function fen_advance_solution(ctx, step, dt) bind(C, name='fen_advance_solution')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: step
            real(c_double), intent(inout) :: dt
        end function fen_advance_solution
        integer(c_int) function fen_advance_n(ctx, nsteps, dt) bind(C, name='fen_advance_n')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: nsteps
            real(c_double), intent(inout) :: dt
        end function fen_advance_n
        integer(c_int) function fen_get_status(ctx, st) bind(C, name='fen_get_status')
            import :: c_int, c_ptr, fen_status
            type(c_ptr), value :: ctx
            type(fen_status), intent(out) :: st
        end function fen_get_status

        ! ---- poisson_mod and fields_mod ------------------------------------------------------
        integer(c_int) function fen_solve_poisson(ctx) bind(C, name='fen_solve_poisson')
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
        end function fen_solve_poisson
        integer(c_int) function fen_divergence(ctx, out) bind(C, name='fen_divergence')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: out(*)
        end function fen_divergence
        integer(c_int) function fen_explicit_terms(ctx, out) bind(C, name='fen_explicit_terms')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: out(*)
        end function fen_explicit_terms
        integer(c_int) function fen_gradient(ctx, field, gx, gy, gz) bind(C, name='fen_gradient')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: field
            real(c_double), intent(out) :: gx(*), gy(*), gz(*)
        end function fen_gradient
        integer(c_int) function fen_laplacian(ctx, field, out) bind(C, name='fen_laplacian')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: field
            real(c_double), intent(out) :: out(*)
        end function fen_laplacian
        integer(c_int) function fen_add_advection(ctx, rhs_x, rhs_y, rhs_z) bind(C, name='fen_add_advection')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(inout) :: rhs_x(*), rhs_y(*), rhs_z(*)
        end function fen_add_advection

        ! ---- solver_mod checkpoint and snapshots (file names NUL-terminated) ----------------
        integer(c_int) function fen_save_state(ctx, path) bind(C, name='fen_save_state')
            import :: c_int, c_ptr, c_char
            type(c_ptr), value :: ctx
            character(kind=c_char), intent(in) :: path(*)
        end function fen_save_state
        integer(c_int) function fen_load_state(ctx, path) bind(C, name='fen_load_state')
            import :: c_int, c_ptr, c_char
            type(c_ptr), value :: ctx
            character(kind=c_char), intent(in) :: path(*)
        end function fen_load_state
        integer(c_int) function fen_save_state_mf(ctx, path, vof) bind(C, name='fen_save_state_mf')
            import :: c_int, c_ptr, c_char, c_double
            type(c_ptr), value :: ctx
            character(kind=c_char), intent(in) :: path(*)
            real(c_double), intent(in) :: vof(*)
        end function fen_save_state_mf
        integer(c_int) function fen_load_state_mf(ctx, path, vof) bind(C, name='fen_load_state_mf')
            import :: c_int, c_ptr, c_char, c_double
            type(c_ptr), value :: ctx
            character(kind=c_char), intent(in) :: path(*)
            real(c_double), intent(out) :: vof(*)
        end function fen_load_state_mf
        integer(c_int) function fen_save_fields(ctx, dir, step) bind(C, name='fen_save_fields')
            import :: c_int, c_ptr, c_char
            type(c_ptr), value :: ctx
            character(kind=c_char), intent(in) :: dir(*)
            integer(c_int), value :: step
        end function fen_save_fields

        ! ---- discrete adjoint (no counterpart in FEN) ---------------------------------------
        integer(c_int) function fen_adjoint_setup(ctx, nsteps, every) bind(C, name='fen_adjoint_setup')
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
            integer(c_int), value :: nsteps, every
        end function fen_adjoint_setup
        integer(c_int) function fen_adjoint_forward(ctx, dt) bind(C, name='fen_adjoint_forward')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), value :: dt
        end function fen_adjoint_forward
        integer(c_int) function fen_adjoint_backward3(ctx, lam_u, lam_v, lam_w, g_u, g_v, g_w, ms) &
                bind(C, name='fen_adjoint_backward3')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(in) :: lam_u(*), lam_v(*), lam_w(*)
            real(c_double), intent(out) :: g_u(*), g_v(*), g_w(*), ms(2)
        end function fen_adjoint_backward3
        integer(c_int) function fen_adjoint_backward(ctx, lam_u, lam_v, g_u, g_v, ms) bind(C, name='fen_adjoint_backward')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(in) :: lam_u(*), lam_v(*)
            real(c_double), intent(out) :: g_u(*), g_v(*), ms(2)
        end function fen_adjoint_backward

        ! ---- variable properties (MF build) and IBM forcing (IBM build) ---------------------
        integer(c_int) function fen_set_split_pressure(ctx, rhomin) bind(C, name='fen_set_split_pressure')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), value :: rhomin
        end function fen_set_split_pressure
        integer(c_int) function fen_set_ibm_forcing(ctx, comp, npoints, ijk, nnbr, nbr_ijk, w, c0) &
                bind(C, name='fen_set_ibm_forcing')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: comp, npoints
            integer(c_int), intent(in) :: ijk(*), nnbr(*), nbr_ijk(*)
            real(c_double), intent(in) :: w(*), c0(*)
        end function fen_set_ibm_forcing
        integer(c_int) function fen_get_ibm_force(ctx, comp, fe) bind(C, name='fen_get_ibm_force')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: comp
            real(c_double), intent(out) :: fe(*)
        end function fen_get_ibm_force

        ! ---- device timing and counters -------------------------------------------------------
        integer(c_int) function fen_debug_checks(count, first) bind(C, name='fen_debug_checks')
            import :: c_int, c_long_long
            integer(c_long_long), intent(out) :: count, first
        end function fen_debug_checks
        integer(c_int) function fen_sync(ctx) bind(C, name='fen_sync')
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
        end function fen_sync
        integer(c_long_long) function fen_kernel_launches(ctx) bind(C, name='fen_kernel_launches')
            import :: c_long_long, c_ptr
            type(c_ptr), value :: ctx
        end function fen_kernel_launches
        integer(c_int) function fen_time_steps(ctx, nsteps, dt, ms) bind(C, name='fen_time_steps')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: nsteps
            real(c_double), value :: dt
            real(c_double), intent(out) :: ms
        end function fen_time_steps
        integer(c_int) function fen_profile_step(ctx, reps, dt, out) bind(C, name='fen_profile_step')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: reps
            real(c_double), value :: dt
            real(c_double), intent(out) :: out(8)
        end function fen_profile_step

        ! ---- allocation-free 2D periodic Poisson solve on caller-owned device arrays ----------
        integer(c_int) function fen_poisson_pp2d_noalloc(rhs, phi, nx, ny, lx, stream) &
                bind(C, name='fen_poisson_pp2d_noalloc')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: rhs, phi, stream
            integer(c_int), value :: nx, ny
            real(c_double), value :: lx
        end function fen_poisson_pp2d_noalloc

        ! ---- batched ensemble of 2D periodic runs (no counterpart in FEN) ---------------------
        integer(c_int) function fen_ensemble_create(nruns, n, viscosity, length, cfl, famp, fk, ens) &
                bind(C, name='fen_ensemble_create')
            import :: c_int, c_ptr, c_double
            integer(c_int), value :: nruns, fk
            integer(c_int), intent(in) :: n(*)
            real(c_double), intent(in) :: viscosity(*)
            real(c_double), value :: length, cfl, famp
            type(c_ptr), intent(out) :: ens
        end function fen_ensemble_create
        integer(c_int) function fen_ensemble_destroy(ens) bind(C, name='fen_ensemble_destroy')
            import :: c_int, c_ptr
            type(c_ptr), value :: ens
        end function fen_ensemble_destroy
        integer(c_int) function fen_ensemble_upload(ens, run, u, v, p) bind(C, name='fen_ensemble_upload')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ens
            integer(c_int), value :: run
            real(c_double), intent(in) :: u(*), v(*)
            type(c_ptr), value :: p   ! c_loc of the pressure, or c_null_ptr
        end function fen_ensemble_upload
        integer(c_int) function fen_ensemble_download(ens, run, u, v, p) bind(C, name='fen_ensemble_download')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ens
            integer(c_int), value :: run
            real(c_double), intent(out) :: u(*), v(*), p(*)
        end function fen_ensemble_download
        integer(c_int) function fen_ensemble_set_timestep(ens, U) bind(C, name='fen_ensemble_set_timestep')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ens
            real(c_double), value :: U
        end function fen_ensemble_set_timestep
        integer(c_int) function fen_ensemble_advance(ens, nsteps, ms) bind(C, name='fen_ensemble_advance')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ens
            integer(c_int), value :: nsteps
            real(c_double), intent(out) :: ms
        end function fen_ensemble_advance
        integer(c_int) function fen_ensemble_status(ens, run, out) bind(C, name='fen_ensemble_status')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ens
            integer(c_int), value :: run
            real(c_double), intent(out) :: out(8)  ! time, dt, dt_o, maxvel, ke, maxdiv, nan, viscosity
        end function fen_ensemble_status
        integer(c_int) function fen_ensemble_config(ens, threads, sizes, groups, nclasses, nclusters) &
                bind(C, name='fen_ensemble_config')
            import :: c_int, c_ptr
            type(c_ptr), value :: ens
            integer(c_int), intent(out) :: threads, sizes(*), groups(*), nclasses, nclusters
        end function fen_ensemble_config
        integer(c_int) function fen_ensemble_set_config(ens, threads, groups) bind(C, name='fen_ensemble_set_config')
            import :: c_int, c_ptr
            type(c_ptr), value :: ens
            integer(c_int), value :: threads
            integer(c_int), intent(in) :: groups(*)
        end function fen_ensemble_set_config
        integer(c_int) function fen_ensemble_tune(ens, steps, cache_path) bind(C, name='fen_ensemble_tune')
            import :: c_int, c_ptr, c_char
            type(c_ptr), value :: ens
            integer(c_int), value :: steps
            character(kind=c_char), intent(in) :: cache_path(*)
        end function fen_ensemble_tune
        integer(c_long_long) function fen_ensemble_launches(ens) bind(C, name='fen_ensemble_launches')
            import :: c_long_long, c_ptr
            type(c_ptr), value :: ens
        end function fen_ensemble_launches
        integer(c_int) function fen_ensemble_adjoint_setup(ens, nsteps, every) bind(C, name='fen_ensemble_adjoint_setup')
            import :: c_int, c_ptr
            type(c_ptr), value :: ens
            integer(c_int), value :: nsteps, every
        end function fen_ensemble_adjoint_setup
        integer(c_int) function fen_ensemble_adjoint_forward(ens, ms) bind(C, name='fen_ensemble_adjoint_forward')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ens
            real(c_double), intent(out) :: ms
        end function fen_ensemble_adjoint_forward
        integer(c_int) function fen_ensemble_adjoint_seed(ens, run, lam_u, lam_v) bind(C, name='fen_ensemble_adjoint_seed')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ens
            integer(c_int), value :: run
            real(c_double), intent(in) :: lam_u(*), lam_v(*)
        end function fen_ensemble_adjoint_seed
        integer(c_int) function fen_ensemble_adjoint_backward(ens, ms) bind(C, name='fen_ensemble_adjoint_backward')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ens
            real(c_double), intent(out) :: ms
        end function fen_ensemble_adjoint_backward
        integer(c_int) function fen_ensemble_adjoint_gradient(ens, run, g_u, g_v) &
                bind(C, name='fen_ensemble_adjoint_gradient')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ens
            integer(c_int), value :: run
            real(c_double), intent(out) :: g_u(*), g_v(*)
        end function fen_ensemble_adjoint_gradient
        integer(c_int) function fen_ensemble_adjoint_dts(ens, run, dt, dt_o) bind(C, name='fen_ensemble_adjoint_dts')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ens
            integer(c_int), value :: run
            real(c_double), intent(out) :: dt(*), dt_o(*)
        end function fen_ensemble_adjoint_dts
        integer(c_size_t) function fen_ensemble_smem_bytes(n, groups) bind(C, name='fen_ensemble_smem_bytes')
            import :: c_size_t, c_int
            integer(c_int), value :: n, groups
        end function fen_ensemble_smem_bytes

        ! C library strlen, to size the message of fen_last_error
        integer(c_size_t) function fen_c_strlen(s) bind(C, name='strlen')
            import :: c_size_t, c_ptr
            type(c_ptr), value :: s
        end function fen_c_strlen
    end interface

    !> The context of the one grid this process drives (one GPU per process).
    type(c_ptr) :: fen_ctx = c_null_ptr

contains

    !> Stop with the library's message when an entry point failed.
    subroutine fen_check(rc)
        use, intrinsic :: iso_fortran_env, only : error_unit
        integer(c_int), intent(in) :: rc
        character(kind=c_char), pointer :: msg(:)
        type(c_ptr) :: p
        integer :: n
        if (rc == FEN_OK) return
        p = fen_last_error()
        n = int(fen_c_strlen(p))
        call c_f_pointer(p, msg, [n])
        write(error_unit, '(a, i0, a, *(a))') 'fen_gpu error ', rc, ': ', msg(1:n)
        error stop 1
    end subroutine fen_check

end module fen_gpu_mod
