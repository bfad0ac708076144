!> fen_gpu_route_mod: routes FEN's projection-step hot path to libfen_gb300 (one GPU).
!>
!> Compiled with FEN's own sources and flags (mpif90 -cpp [-DDIM=3] [-DMF] [-DIBM]) after
!> fen_gpu_mod.f90.  A program keeps FEN's calls and adds one line after init_solver:
!>
!>     call init_solver(comp_grid)          ! FEN (solver.f90:34): host fields, plans
!>     call gpu_init_solver(comp_grid)      ! device context; re-points the procedure pointers
!>     call set_timestep(comp_grid, dt, U)  ! or gpu_set_timestep, see below
!>     do ... call advance_solution(comp_grid, step, dt) ... end do   ! runs on the GPU
!>
!> gpu_init_solver creates the context from comp_grid and navier_stokes_mod's density,
!> viscosity, g, CFL and constant_CFL, uploads FEN's current fields, and points
!> solver_mod::advance_solution (solver.f90:12-19, 28) and poisson_mod::solve_poisson
!> (poisson.f90:21-29) at the GPU routines below.  The host arrays stay FEN's: with
!> gpu_host_sync (default .true.) every advance_solution first uploads what programs write
!> between steps (v, p, S and the boundary values v%x%bc%top ..., e.g. lid_driven.f90:59,
!> isotropic.f90:114-152), then downloads v and p after the step, and it sets
!> navier_stokes_mod's maxdiv, maxCFL and dt_o, so FEN's print_solver_status, output and
!> steady-state checks work unchanged.  That mirror moves four or five fields each way per
!> step; with gpu_host_sync = .false. the device copies are authoritative between explicit
!> gpu_sync_to_device / gpu_sync_to_host calls and a step moves no field.
module fen_gpu_route_mod

    use, intrinsic :: iso_c_binding
    use precision_mod, only : dp
    use grid_mod     , only : grid
    use scalar_mod   , only : scalar
    use fen_gpu_mod

    implicit none

    private
    public :: gpu_init_solver, gpu_advance_solution, gpu_solve_poisson, gpu_set_timestep, &
              gpu_sync_to_device, gpu_sync_to_host, gpu_save_state, gpu_load_state, &
              gpu_destroy_solver, gpu_host_sync, gpu_precision

    !> Mirror FEN's host fields around every step (see above).
    logical, save :: gpu_host_sync = .true.
    !> Arithmetic form of the context: FEN_FP64 (the reference's arithmetic) or FEN_MIXED.
    integer(c_int), save :: gpu_precision = FEN_FP64

contains

    !> Physical boundary condition string of grid%boundary_conditions (grid.f90:41-46).
    integer(c_int) function bc_code(s)
        character(len=*), intent(in) :: s
        select case (s)
        case ('Periodic')
            bc_code = FEN_BC_PERIODIC
        case ('Wall')
            bc_code = FEN_BC_WALL
        case ('Inflow')
            bc_code = FEN_BC_INFLOW
        case ('Outflow')
            bc_code = FEN_BC_OUTFLOW
        case default
            bc_code = -1
        end select
    end function bc_code

    !===============================================================================================
    subroutine gpu_init_solver(comp_grid)
        use navier_stokes_mod, only : density, viscosity, g, CFL, constant_CFL
        use solver_mod       , only : advance_solution
        use poisson_mod      , only : solve_poisson
        use, intrinsic :: iso_fortran_env, only : error_unit

        type(grid), intent(in) :: comp_grid

        type(fen_params) :: prm
        integer :: q, nface

        nface = size(comp_grid%boundary_conditions)
        prm%dim = int(nface/2, c_int)
        prm%nx = int(comp_grid%Nx, c_int)
        prm%ny = int(comp_grid%Ny, c_int)
        prm%nz = int(comp_grid%Nz, c_int)
        prm%lx = comp_grid%Lx
        prm%ly = comp_grid%Ly
        prm%lz = comp_grid%Lz
        prm%origin = comp_grid%origin
        prm%bc = FEN_BC_PERIODIC
        do q = 1, nface
            prm%bc(q) = bc_code(comp_grid%boundary_conditions(q)%s)
            if (prm%bc(q) < 0) then
                write(error_unit, '(a)') 'fen_gpu: unknown boundary condition '//comp_grid%boundary_conditions(q)%s
                error stop 1
            endif
        end do
        prm%aniso = 0                 ! delta = Lx/Nx on every axis (grid.f90:140)
        prm%density = density
        prm%viscosity = viscosity
        prm%g = g
        prm%cfl = CFL
        prm%constant_cfl = merge(1_c_int, 0_c_int, constant_CFL)
        prm%precision = gpu_precision
        prm%refine = merge(1_c_int, 0_c_int, gpu_precision == FEN_MIXED)
        call fen_check(fen_ctx_create(prm, fen_ctx))
        call gpu_sync_to_device()

        advance_solution => gpu_advance_solution
        solve_poisson => gpu_solve_poisson
    end subroutine gpu_init_solver
    !===============================================================================================

    !===============================================================================================
    !> advance_solution on the GPU (navier_stokes_solver, navier_stokes.f90:50-136).
    subroutine gpu_advance_solution(comp_grid, step, dt)
        use navier_stokes_mod, only : maxdiv, maxCFL, dt_o

        type(grid), intent(in   ) :: comp_grid   ! the context holds the grid
        integer   , intent(in   ) :: step
        real(dp)  , intent(inout) :: dt

        type(fen_status) :: st

        if (gpu_host_sync) call upload_program_fields()
        call fen_check(fen_advance_solution(fen_ctx, int(step, c_int), dt))
        call fen_check(fen_get_status(fen_ctx, st))
        maxdiv = st%maxdiv
        maxCFL = st%maxcfl
        dt_o = st%dt_o
        if (gpu_host_sync) call download_state()
    end subroutine gpu_advance_solution
    !===============================================================================================

    !===============================================================================================
    !> solve_poisson(f) on the GPU for any scalar with FEN's boundary set of the grid
    !> (poisson.f90:21-29): the field goes up in its own ghost level and comes back solved.
    subroutine gpu_solve_poisson(f)
        type(scalar), intent(inout) :: f

        call fen_check(fen_upload_gl(fen_ctx, FEN_PHI, f%f, int(f%gl, c_int)))
        call fen_check(fen_solve_poisson(fen_ctx))
        call fen_check(fen_download_gl(fen_ctx, FEN_PHI, f%f, int(f%gl, c_int)))
    end subroutine gpu_solve_poisson
    !===============================================================================================

    !===============================================================================================
    !> set_timestep(comp_grid, dt, U) (navier_stokes.f90:623-666) on the context; also sets
    !> FEN's dt_o.
    subroutine gpu_set_timestep(comp_grid, dt, U)
        use navier_stokes_mod, only : dt_o

        type(grid), intent(in ) :: comp_grid
        real(dp)  , intent(out) :: dt
        real(dp)  , intent(in ) :: U

        call fen_check(fen_set_timestep(fen_ctx, U, dt))
        dt_o = dt
    end subroutine gpu_set_timestep
    !===============================================================================================

    !===============================================================================================
    !> Host -> device: every field of the step (v, p, the AB2 history dv_o, S) and the
    !> boundary values.
    subroutine gpu_sync_to_device()
        use navier_stokes_mod, only : dv_o

        call upload_program_fields()
        call fen_check(fen_upload(fen_ctx, FEN_DVO_X, dv_o%x%f))
        call fen_check(fen_upload(fen_ctx, FEN_DVO_Y, dv_o%y%f))
#if DIM==3
        call fen_check(fen_upload(fen_ctx, FEN_DVO_Z, dv_o%z%f))
#endif
    end subroutine gpu_sync_to_device

    !> Device -> host: v, p and dv_o.
    subroutine gpu_sync_to_host()
        use navier_stokes_mod, only : dv_o

        call download_state()
        call fen_check(fen_download(fen_ctx, FEN_DVO_X, dv_o%x%f))
        call fen_check(fen_download(fen_ctx, FEN_DVO_Y, dv_o%y%f))
#if DIM==3
        call fen_check(fen_download(fen_ctx, FEN_DVO_Z, dv_o%z%f))
#endif
    end subroutine gpu_sync_to_host

    !> What programs write between steps: v and p (with their ghosts, gl = 1), S as FEN
    !> allocates it (no ghosts, navier_stokes.f90:768) and the Dirichlet values of v.
    subroutine upload_program_fields()
        use navier_stokes_mod, only : v, p, S

        call fen_check(fen_upload(fen_ctx, FEN_U, v%x%f))
        call fen_check(fen_upload(fen_ctx, FEN_V, v%y%f))
#if DIM==3
        call fen_check(fen_upload(fen_ctx, FEN_W, v%z%f))
#endif
        call fen_check(fen_upload(fen_ctx, FEN_P, p%f))
        call fen_check(fen_upload(fen_ctx, FEN_S_X, S%x%f))
        call fen_check(fen_upload(fen_ctx, FEN_S_Y, S%y%f))
#if DIM==3
        call fen_check(fen_upload(fen_ctx, FEN_S_Z, S%z%f))
#endif
        call upload_bc_values(FEN_U, v%x)
        call upload_bc_values(FEN_V, v%y)
#if DIM==3
        call upload_bc_values(FEN_W, v%z)
#endif
    end subroutine upload_program_fields

    !> field%bc%left ... (scalar.f90:28-36, allocated over the ghosted face extents).
    subroutine upload_bc_values(fid, f)
        integer(c_int), intent(in) :: fid
        type(scalar)  , intent(in) :: f

        call fen_check(fen_set_bc_values(fen_ctx, fid, FEN_LEFT, f%bc%left))
        call fen_check(fen_set_bc_values(fen_ctx, fid, FEN_RIGHT, f%bc%right))
        call fen_check(fen_set_bc_values(fen_ctx, fid, FEN_BOTTOM, f%bc%bottom))
        call fen_check(fen_set_bc_values(fen_ctx, fid, FEN_TOP, f%bc%top))
#if DIM==3
        call fen_check(fen_set_bc_values(fen_ctx, fid, FEN_FRONT, f%bc%front))
        call fen_check(fen_set_bc_values(fen_ctx, fid, FEN_BACK, f%bc%back))
#endif
    end subroutine upload_bc_values

    subroutine download_state()
        use navier_stokes_mod, only : v, p

        call fen_check(fen_download(fen_ctx, FEN_U, v%x%f))
        call fen_check(fen_download(fen_ctx, FEN_V, v%y%f))
#if DIM==3
        call fen_check(fen_download(fen_ctx, FEN_W, v%z%f))
#endif
        call fen_check(fen_download(fen_ctx, FEN_P, p%f))
    end subroutine download_state
    !===============================================================================================

    !===============================================================================================
    !> save_state(step) / load_state(step) (solver.f90:160-329): FEN's file name and raw
    !> layout, written from and read into the device state.
    subroutine gpu_save_state(step)
        integer, intent(in) :: step
        character(len=7) :: sn

        write(sn, '(I0.7)') step
        call fen_check(fen_save_state(fen_ctx, 'data/state_'//sn//'.raw'//c_null_char))
    end subroutine gpu_save_state

    subroutine gpu_load_state(step)
        integer, intent(in) :: step
        character(len=7) :: sn

        write(sn, '(I0.7)') step
        call fen_check(fen_load_state(fen_ctx, 'data/state_'//sn//'.raw'//c_null_char))
        if (gpu_host_sync) call gpu_sync_to_host()
    end subroutine gpu_load_state
    !===============================================================================================

    !> destroy_solver's device part (solver.f90:333).
    subroutine gpu_destroy_solver()
        call fen_check(fen_ctx_destroy(fen_ctx))
        fen_ctx = c_null_ptr
    end subroutine gpu_destroy_solver

end module fen_gpu_route_mod
