! aderdg_gpu.f90 -- ISO_C_BINDING interface to libaderdg_gpu.so
! (include/aderdg_gpu.h) for the reference's Fortran driver.
!
! A maintainer adds this module to the reference's Makefile, `use`s it in
! main.f90 and replaces the per-cell phase loops of the time loop
! (Euler/main.f90:24-100) by the grid-level calls below; module arrays are
! passed unchanged (Fortran layout uh(nVar,N+1,N+1,IMAX,JMAX)).  No Fortran
! compiler exists on the build machines of this project, so this file is
! shipped uncompiled.
module aderdg_gpu
    use iso_c_binding
    implicit none

    integer(c_int), parameter :: ADERDG_OK = 0
    integer(c_int), parameter :: ADERDG_SYS_ADVDIFF = 0, ADERDG_SYS_EULER = 1, ADERDG_SYS_BN = 2
    integer(c_int), parameter :: ADERDG_FP64 = 0, ADERDG_FP32_MIXED = 1, ADERDG_FP32_WIDE = 2

    type, bind(C) :: aderdg_config
        integer(c_int) :: system, N, imax, jmax
        real(c_double) :: xl(2), xr(2)
        integer(c_int) :: bc(4)
        integer(c_int) :: bc_mode
        real(c_double) :: cfl, gamma
        real(c_double) :: gamma_s, gamma_g, pi_s, pi_g
        real(c_double) :: cx, cy, a
        integer(c_int) :: ad_flux_mode, limiter, precision
    end type aderdg_config

    interface
        integer(c_int) function aderdg_create(cfg, ctx) bind(C, name="aderdg_create")
            import :: c_int, c_ptr, aderdg_config
            type(aderdg_config), intent(in) :: cfg
            type(c_ptr), intent(out) :: ctx
        end function
        integer(c_int) function aderdg_destroy(ctx) bind(C, name="aderdg_destroy")
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
        end function
        integer(c_int) function aderdg_upload(ctx, uh) bind(C, name="aderdg_upload")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(in) :: uh(*)
        end function
        integer(c_int) function aderdg_init_limiter(ctx, lh_ic, n_limited) bind(C, name="aderdg_init_limiter")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(in) :: lh_ic(*)
            integer(c_int), intent(out) :: n_limited
        end function
        integer(c_int) function aderdg_download(ctx, uh, status) bind(C, name="aderdg_download")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: uh(*)
            integer(c_int), intent(out) :: status(*)
        end function
        integer(c_int) function aderdg_calc_time_step(ctx, time, tend, dt) bind(C, name="aderdg_calc_time_step")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), value :: time, tend
            real(c_double), intent(out) :: dt
        end function
        integer(c_int) function aderdg_limiter_prepare(ctx) bind(C, name="aderdg_limiter_prepare")
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
        end function
        integer(c_int) function aderdg_space_time_predictor(ctx) bind(C, name="aderdg_space_time_predictor")
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
        end function
        integer(c_int) function aderdg_volume_integral(ctx) bind(C, name="aderdg_volume_integral")
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
        end function
        integer(c_int) function aderdg_riemann_problem(ctx) bind(C, name="aderdg_riemann_problem")
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
        end function
        integer(c_int) function aderdg_surface_integral(ctx) bind(C, name="aderdg_surface_integral")
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
        end function
        integer(c_int) function aderdg_element_update(ctx, n_recompute) bind(C, name="aderdg_element_update")
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
            integer(c_int), intent(out) :: n_recompute
        end function
        integer(c_int) function aderdg_limiter(ctx) bind(C, name="aderdg_limiter")
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
        end function
        integer(c_int) function aderdg_step(ctx, time, tend, dt, n_recompute) bind(C, name="aderdg_step")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(inout) :: time
            real(c_double), value :: tend
            real(c_double), intent(out) :: dt
            integer(c_int), intent(out) :: n_recompute
        end function
        integer(c_int) function aderdg_run(ctx, time, tend, max_steps, sync_every, steps_done) bind(C, name="aderdg_run")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(inout) :: time
            real(c_double), value :: tend
            integer(c_int), value :: max_steps, sync_every
            integer(c_int), intent(out) :: steps_done
        end function
        integer(c_int) function aderdg_step_host(ctx, uh, time, tend, dt, n_recompute) bind(C, name="aderdg_step_host")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(inout) :: uh(*)
            real(c_double), intent(inout) :: time
            real(c_double), value :: tend
            real(c_double), intent(out) :: dt
            integer(c_int), intent(out) :: n_recompute
        end function
        ! write_data's field: cell-average primitive variables wh(nVar,IMAX,JMAX)
        integer(c_int) function aderdg_cell_averages(ctx, primitive, wh) bind(C, name="aderdg_cell_averages")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: primitive
            real(c_double), intent(out) :: wh(*)
        end function
        ! analyze_soln: norms(3) = max over cells of the cell-average error of variable var+1
        integer(c_int) function aderdg_error_norms(ctx, ic, params, var, norms) bind(C, name="aderdg_error_norms")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: ic, var
            real(c_double), intent(in) :: params(32)
            real(c_double), intent(out) :: norms(3)
        end function
        ! the initial field and the initial limiter evaluated on the device
        integer(c_int) function aderdg_initial_condition(ctx, ic, params, n_limited) &
                bind(C, name="aderdg_initial_condition")
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: ic
            real(c_double), intent(in) :: params(32)
            integer(c_int), intent(out) :: n_limited
        end function
        type(c_ptr) function aderdg_last_error(ctx) bind(C, name="aderdg_last_error")
            import :: c_ptr
            type(c_ptr), value :: ctx
        end function
    end interface
end module aderdg_gpu
