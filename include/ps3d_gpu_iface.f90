! ps3d_gpu_iface.f90 - Fortran (iso_c_binding) interface to libps3d_gpu.so,
! the C ABI of include/ps3d_gpu.h.
!
! The reference's driver binds the GPU path with this module; a stepper
! extension of base_stepper (src/stepper/advance.f90:31-59) then calls
! ps3d_gpu_advance from its step procedure (see the integration notes).  The
! host arrays of src/fields/fields.f90 ((0:nz, ny, nx, 3) column-major) are
! the ABI's host layout, so svor, vor and vel pass without a copy.
!
! Derived types mirror ps3d_gpu_config and ps3d_gpu_diag member for member;
! the status codes and enums are the #defines of the header.
module ps3d_gpu_iface
    use iso_c_binding
    implicit none

    integer(c_int), parameter :: PS3D_OK = 0, PS3D_ERR_INVALID_ARG = 1, PS3D_ERR_UNSUPPORTED_SIZE = 2, &
                                 PS3D_ERR_CUDA = 3, PS3D_ERR_OUT_OF_MEMORY = 4, PS3D_ERR_NOT_READY = 5, &
                                 PS3D_ERR_NONFINITE = 6, PS3D_ERR_DEVICE_LIMIT = 7, PS3D_ERR_NO_DEVICE = 8
    integer(c_int), parameter :: PS3D_PRE_CONSTANT = 0, PS3D_PRE_VORCH = 1, PS3D_PRE_BFMAX = 2, &
                                 PS3D_PRE_ROLL_MEAN_MAX_STRAIN = 3, PS3D_PRE_MAX_STRAIN = 4, &
                                 PS3D_PRE_US_MAX_STRAIN = 5, PS3D_PRE_ROLL_MEAN_BFMAX = 6
    integer(c_int), parameter :: PS3D_KOLMOGOROV = 0, PS3D_GEOPHYSICAL = 1, PS3D_HOU_LI = 0, PS3D_TWO_THIRDS = 1
    integer(c_int), parameter :: PS3D_IMPL_DIFF_RK4 = 0, PS3D_CN2 = 1
    integer(c_int), parameter :: PS3D_PRECISION_FP64 = 0, PS3D_PRECISION_MIXED = 1
    integer(c_int), parameter :: PS3D_FIELD_SVOR = 0, PS3D_FIELD_VOR = 1, PS3D_FIELD_VEL = 2, &
                                 PS3D_FIELD_SVEL = 3, PS3D_FIELD_SVORTS = 4, PS3D_FIELD_SBUOY = 5, &
                                 PS3D_FIELD_BUOY = 6, PS3D_FIELD_SBUOYS = 7
    integer(c_int), parameter :: PS3D_CLOSURE_EVERY_STAGE = 1, PS3D_CLOSURE_CLIP = 2, PS3D_CLOSURE_WALLS = 4

    type, bind(c) :: ps3d_gpu_config
        integer(c_int) :: nx, ny, nz
        integer(c_int) :: nnu
        real(c_double) :: lower(3)
        real(c_double) :: extent(3)
        real(c_double) :: prediss
        integer(c_int) :: pretype
        integer(c_int) :: length_scale
        integer(c_int) :: filtering
        integer(c_int) :: stepper
        real(c_double) :: cflmax
        real(c_double) :: alpha
        real(c_double) :: time_limit
        integer(c_int) :: roll_mean_win_size
        integer(c_int) :: nthreads
        integer(c_int) :: hold_source
        real(c_double) :: f_cor(3)
        integer(c_int) :: precision
        integer(c_int) :: device
        integer(c_int) :: buoyancy
        real(c_double) :: bfsq
        integer(c_int) :: bfsq_given
        integer(c_int) :: buoy_nnu
        real(c_double) :: buoy_prediss
        integer(c_int) :: buoy_pretype
        integer(c_int) :: buoy_length_scale
        integer(c_int) :: buoy_roll_mean_win_size
    end type ps3d_gpu_config

    type, bind(c) :: ps3d_gpu_diag
        real(c_double) :: t, dt
        real(c_double) :: ke, en, hel
        real(c_double) :: vortmax, vortrms, vorch
        real(c_double) :: vormean(3)
        real(c_double) :: ggmax, usggmax, lsggmax
        real(c_double) :: umax, vmax, wmax
        real(c_double) :: bfmax, rmv, pref
        real(c_double) :: rmb, bpref
    end type ps3d_gpu_diag

    interface
        ! ---- lifetime and errors
        integer(c_int) function ps3d_gpu_create(cfg, ctx) bind(c, name='ps3d_gpu_create')
            import :: c_int, c_ptr, ps3d_gpu_config
            type(ps3d_gpu_config), intent(in) :: cfg
            type(c_ptr), intent(out) :: ctx
        end function
        integer(c_int) function ps3d_gpu_destroy(ctx) bind(c, name='ps3d_gpu_destroy')
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
        end function
        type(c_ptr) function ps3d_gpu_strerror(status) bind(c, name='ps3d_gpu_strerror')
            import :: c_int, c_ptr
            integer(c_int), value :: status
        end function
        type(c_ptr) function ps3d_gpu_last_error(ctx) bind(c, name='ps3d_gpu_last_error')
            import :: c_ptr
            type(c_ptr), value :: ctx
        end function
        integer(c_int) function ps3d_gpu_synchronize(ctx) bind(c, name='ps3d_gpu_synchronize')
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
        end function

        ! ---- state transfer
        integer(c_int) function ps3d_gpu_set_field(ctx, which, host) bind(c, name='ps3d_gpu_set_field')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: which
            real(c_double), intent(in) :: host(*)
        end function
        integer(c_int) function ps3d_gpu_get_field(ctx, which, host) bind(c, name='ps3d_gpu_get_field')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: which
            real(c_double), intent(out) :: host(*)
        end function
        integer(c_int) function ps3d_gpu_set_ini_vor_mean(ctx, v) bind(c, name='ps3d_gpu_set_ini_vor_mean')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(in) :: v(2)
        end function
        integer(c_int) function ps3d_gpu_get_ini_vor_mean(ctx, v) bind(c, name='ps3d_gpu_get_ini_vor_mean')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: v(2)
        end function

        ! ---- set-up (setup_fields, init_diffusion)
        integer(c_int) function ps3d_gpu_setup_fields(ctx, vor, pert, te, en) bind(c, name='ps3d_gpu_setup_fields')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(in) :: vor(*)
            type(c_ptr), value :: pert          ! c_null_ptr or c_loc of a spectral perturbation
            real(c_double), intent(out) :: te, en
        end function
        integer(c_int) function ps3d_gpu_setup_fields_buoyancy(ctx, vor, pert, buoy, te, en) &
                bind(c, name='ps3d_gpu_setup_fields_buoyancy')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(in) :: vor(*)
            type(c_ptr), value :: pert
            real(c_double), intent(in) :: buoy(*)
            real(c_double), intent(out) :: te, en
        end function
        integer(c_int) function ps3d_gpu_init_diffusion(ctx, te, en) bind(c, name='ps3d_gpu_init_diffusion')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), value :: te, en
        end function

        ! ---- right-hand side and stepping (vor2vel, source, adapt, steppers)
        integer(c_int) function ps3d_gpu_vor2vel(ctx) bind(c, name='ps3d_gpu_vor2vel')
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
        end function
        integer(c_int) function ps3d_gpu_source(ctx) bind(c, name='ps3d_gpu_source')
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
        end function
        integer(c_int) function ps3d_gpu_adapt(ctx, t, dt, diag) bind(c, name='ps3d_gpu_adapt')
            import :: c_int, c_ptr, c_double, ps3d_gpu_diag
            type(c_ptr), value :: ctx
            real(c_double), value :: t
            real(c_double), intent(out) :: dt
            type(ps3d_gpu_diag), intent(out) :: diag
        end function
        integer(c_int) function ps3d_gpu_set_diffusion(ctx, dt, pref) bind(c, name='ps3d_gpu_set_diffusion')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), value :: dt, pref
        end function
        integer(c_int) function ps3d_gpu_step(ctx, t, dt) bind(c, name='ps3d_gpu_step')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(inout) :: t
            real(c_double), value :: dt
        end function
        integer(c_int) function ps3d_gpu_advance(ctx, t, nsteps, diag) bind(c, name='ps3d_gpu_advance')
            import :: c_int, c_ptr, c_double, ps3d_gpu_diag
            type(c_ptr), value :: ctx
            real(c_double), intent(inout) :: t
            integer(c_int), value :: nsteps
            type(ps3d_gpu_diag), intent(out) :: diag(*)
        end function
        integer(c_int) function ps3d_gpu_advance_host(ctx, svor, t, diag) bind(c, name='ps3d_gpu_advance_host')
            import :: c_int, c_ptr, c_double, ps3d_gpu_diag
            type(c_ptr), value :: ctx
            real(c_double), intent(inout) :: svor(*)
            real(c_double), intent(inout) :: t
            type(ps3d_gpu_diag), intent(out) :: diag
        end function
        integer(c_int) function ps3d_gpu_advance_graph(ctx, t, nsteps, diag, ms) bind(c, name='ps3d_gpu_advance_graph')
            import :: c_int, c_ptr, c_double, ps3d_gpu_diag
            type(c_ptr), value :: ctx
            real(c_double), intent(inout) :: t
            integer(c_int), value :: nsteps
            type(ps3d_gpu_diag), intent(out) :: diag
            real(c_double), intent(out) :: ms
        end function

        ! ---- diagnostics (field_diagnostics, fields_derived, genspec)
        integer(c_int) function ps3d_gpu_energy_series(ctx, ke, en, hel) bind(c, name='ps3d_gpu_energy_series')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: ke, en, hel
        end function
        integer(c_int) function ps3d_gpu_calc_vorticity_mean(ctx, v) bind(c, name='ps3d_gpu_calc_vorticity_mean')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: v(2)
        end function
        integer(c_int) function ps3d_gpu_adjust_vorticity_mean(ctx) bind(c, name='ps3d_gpu_adjust_vorticity_mean')
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx
        end function
        integer(c_int) function ps3d_gpu_derived_fields(ctx, pres, delta) bind(c, name='ps3d_gpu_derived_fields')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            real(c_double), intent(out) :: pres(*), delta(*)
        end function
        integer(c_int) function ps3d_gpu_ke_spectrum(ctx, nmax, spec, nbins, dk) bind(c, name='ps3d_gpu_ke_spectrum')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: ctx
            integer(c_int), value :: nmax
            real(c_double), intent(out) :: spec(*)
            integer(c_int), intent(out) :: nbins
            real(c_double), intent(out) :: dk
        end function

        ! ---- checkpoint (path: a NUL-terminated character array)
        integer(c_int) function ps3d_gpu_save_state(ctx, path, t) bind(c, name='ps3d_gpu_save_state')
            import :: c_int, c_ptr, c_char, c_double
            type(c_ptr), value :: ctx
            character(kind=c_char), intent(in) :: path(*)
            real(c_double), value :: t
        end function
        integer(c_int) function ps3d_gpu_load_state(ctx, path, t) bind(c, name='ps3d_gpu_load_state')
            import :: c_int, c_ptr, c_char, c_double
            type(c_ptr), value :: ctx
            character(kind=c_char), intent(in) :: path(*)
            real(c_double), intent(out) :: t
        end function

        ! ---- learned sub-grid closure
        integer(c_int) function ps3d_closure_create(nx, ny, nz, max_samples, device, seed, cl) &
                bind(c, name='ps3d_closure_create')
            import :: c_int, c_long_long, c_ptr
            integer(c_int), value :: nx, ny, nz, max_samples, device
            integer(c_long_long), value :: seed
            type(c_ptr), intent(out) :: cl
        end function
        integer(c_int) function ps3d_closure_destroy(cl) bind(c, name='ps3d_closure_destroy')
            import :: c_int, c_ptr
            type(c_ptr), value :: cl
        end function
        integer(c_int) function ps3d_closure_set_params(cl, params) bind(c, name='ps3d_closure_set_params')
            import :: c_int, c_ptr, c_float
            type(c_ptr), value :: cl
            real(c_float), intent(in) :: params(*)
        end function
        integer(c_int) function ps3d_closure_set_scale(cl, ct) bind(c, name='ps3d_closure_set_scale')
            import :: c_int, c_ptr, c_double
            type(c_ptr), value :: cl
            real(c_double), value :: ct
        end function
        integer(c_int) function ps3d_closure_set_engine(cl, engine) bind(c, name='ps3d_closure_set_engine')
            import :: c_int, c_ptr
            type(c_ptr), value :: cl
            integer(c_int), value :: engine
        end function
        integer(c_int) function ps3d_gpu_set_closure(ctx, cl, flags) bind(c, name='ps3d_gpu_set_closure')
            import :: c_int, c_ptr
            type(c_ptr), value :: ctx, cl
            integer(c_int), value :: flags
        end function
    end interface

contains

    ! a NUL-terminated C string (ps3d_gpu_strerror, ps3d_gpu_last_error) as a
    ! Fortran string, e.g. for mpi_stop messages
    function ps3d_c_string(p) result(s)
        type(c_ptr), intent(in) :: p
        character(:), allocatable :: s
        character(kind=c_char), pointer :: c(:)
        integer :: n
        s = ''
        if (.not. c_associated(p)) return
        call c_f_pointer(p, c, [65536])
        n = 0
        do while (n < 65536)
            if (c(n + 1) == c_null_char) exit
            n = n + 1
        end do
        allocate(character(n) :: s)
        s = transfer(c(1:n), s)
    end function ps3d_c_string

end module ps3d_gpu_iface
