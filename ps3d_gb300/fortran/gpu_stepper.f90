! gpu_stepper.f90 - a base_stepper (src/stepper/advance.f90:31-59) whose steps
! run on one GPU through libps3d_gpu.so (module ps3d_gpu_iface).
!
! Drop-in at the reference's plugin point: registered in the stepper factory
! of src/ps3d.f90:90-99 (e.g. stepper = 'gpu-rk4' or 'gpu-cn2'; the option
! holds 16 characters, options.f90:24), it keeps the reference's advance()
! unchanged.  advance() still runs its
! host vor2vel, adapt and source for the diagnostics and output; adapt calls
! set_diffusion(dt, pref, bpref) and advance then calls step(t, dt), which
!   1. sends the host svor (fields.f90; projected in place by the host
!      vor2vel) to the device,
!   2. evaluates vor2vel and source there (inversion.f90:23-388),
!   3. takes the step of impl_rk4.f90 / cn2.f90 with the host's dt and
!      prefactor, and
!   4. returns svor to the host.
! The state crosses the host link twice per step; a driver that wants the
! device to keep the state calls ps3d_gpu_advance (or ps3d_gpu_advance_graph)
! in place of advance() instead.  One MPI rank only (the ABI is one GPU).
module gpu_stepper_mod
    use iso_c_binding
    use advance_mod, only : base_stepper
    use ps3d_gpu_iface
    use parameters, only : nx, ny, nz, lower, extent
    use options, only : vor_visc, filtering, stepper, time
    use fields, only : svor, ini_vor_mean
    use constants, only : cflmax
    use physics, only : f_cor
    use mpi_utils, only : mpi_stop
    implicit none

    private
    public :: gpu_stepper

    type, extends(base_stepper) :: gpu_stepper
        type(c_ptr) :: ctx = c_null_ptr
    contains
        procedure :: set_diffusion => gpu_set_diffusion
        procedure :: setup => gpu_setup
        procedure :: step => gpu_step
        procedure :: release => gpu_release
    end type gpu_stepper

contains

    ! PS3D_PRE_* code of a visc_type%pretype string (options.f90:56-63)
    integer(c_int) function pretype_code(s) result(code)
        character(*), intent(in) :: s
        select case (trim(s))
        case ('constant')
            code = PS3D_PRE_CONSTANT
        case ('vorch')
            code = PS3D_PRE_VORCH
        case ('bfmax')
            code = PS3D_PRE_BFMAX
        case ('max-strain')
            code = PS3D_PRE_MAX_STRAIN
        case ('us-max-strain')
            code = PS3D_PRE_US_MAX_STRAIN
        case ('roll-mean-bfmax')
            code = PS3D_PRE_ROLL_MEAN_BFMAX
        case default
            code = PS3D_PRE_ROLL_MEAN_MAX_STRAIN
        end select
    end function pretype_code

    subroutine check(self, rc, what)
        class(gpu_stepper), intent(in) :: self
        integer(c_int),     intent(in) :: rc
        character(*),       intent(in) :: what
        if (rc /= PS3D_OK) then
            if (c_associated(self%ctx)) then
                call mpi_stop('gpu_stepper: ' // what // ': ' // ps3d_c_string(ps3d_gpu_last_error(self%ctx)))
            else
                call mpi_stop('gpu_stepper: ' // what // ': ' // ps3d_c_string(ps3d_gpu_strerror(rc)))
            endif
        endif
    end subroutine check

    ! called by pre_run after setup_fields (ps3d.f90:84-101): the context for
    ! this grid and namelist, the initial state, and the viscosity from the
    ! initial energy and enstrophy (utils.f90:168-182, evaluated on the device
    ! from the same state)
    subroutine gpu_setup(self)
        class(gpu_stepper), intent(inout) :: self
        type(ps3d_gpu_config) :: cfg
        real(c_double) :: te, en, hel
        cfg%nx = nx
        cfg%ny = ny
        cfg%nz = nz
        cfg%nnu = vor_visc%nnu
        cfg%lower = lower
        cfg%extent = extent
        cfg%prediss = vor_visc%prediss
        cfg%pretype = pretype_code(vor_visc%pretype)
        cfg%length_scale = merge(PS3D_GEOPHYSICAL, PS3D_KOLMOGOROV, trim(vor_visc%length_scale) == 'geophysical')
        cfg%filtering = merge(PS3D_TWO_THIRDS, PS3D_HOU_LI, trim(filtering) == '2/3-rule')
        cfg%stepper = merge(PS3D_CN2, PS3D_IMPL_DIFF_RK4, index(stepper, 'cn2') > 0)
        cfg%cflmax = cflmax
        cfg%alpha = time%alpha
        cfg%time_limit = time%limit
        cfg%roll_mean_win_size = vor_visc%roll_mean_win_size
        cfg%nthreads = 0
        cfg%hold_source = 0
        cfg%f_cor = f_cor
        cfg%precision = PS3D_PRECISION_FP64
        cfg%device = 0
        cfg%buoyancy = 0
        cfg%bfsq = 0.0d0
        cfg%bfsq_given = 0
        cfg%buoy_nnu = vor_visc%nnu
        cfg%buoy_prediss = vor_visc%prediss
        cfg%buoy_pretype = PS3D_PRE_BFMAX
        cfg%buoy_length_scale = PS3D_KOLMOGOROV
        cfg%buoy_roll_mean_win_size = vor_visc%roll_mean_win_size
        call check(self, ps3d_gpu_create(cfg, self%ctx), 'create')
        call check(self, ps3d_gpu_set_field(self%ctx, PS3D_FIELD_SVOR, svor), 'set_field')
        call check(self, ps3d_gpu_set_ini_vor_mean(self%ctx, ini_vor_mean), 'set_ini_vor_mean')
        call check(self, ps3d_gpu_vor2vel(self%ctx), 'vor2vel')
        call check(self, ps3d_gpu_energy_series(self%ctx, te, en, hel), 'energy_series')
        call check(self, ps3d_gpu_init_diffusion(self%ctx, te, en), 'init_diffusion')
    end subroutine gpu_setup

    ! called by adapt (advance.f90:367-375) with the step and the prefactor
    subroutine gpu_set_diffusion(self, dt, vorch, bf)
        class(gpu_stepper), intent(inout) :: self
        double precision,   intent(in)    :: dt
        double precision,   intent(in)    :: vorch
        double precision,   intent(in)    :: bf
        call check(self, ps3d_gpu_set_diffusion(self%ctx, dt, vorch), 'set_diffusion')
    end subroutine gpu_set_diffusion

    subroutine gpu_step(self, t, dt)
        class(gpu_stepper), intent(inout) :: self
        double precision,   intent(inout) :: t
        double precision,   intent(in)    :: dt
        call check(self, ps3d_gpu_set_field(self%ctx, PS3D_FIELD_SVOR, svor), 'set_field')
        call check(self, ps3d_gpu_vor2vel(self%ctx), 'vor2vel')
        call check(self, ps3d_gpu_source(self%ctx), 'source')
        call check(self, ps3d_gpu_step(self%ctx, t, dt), 'step')
        call check(self, ps3d_gpu_get_field(self%ctx, PS3D_FIELD_SVOR, svor), 'get_field')
    end subroutine gpu_step

    ! release the device context (post_run)
    subroutine gpu_release(self)
        class(gpu_stepper), intent(inout) :: self
        integer(c_int) :: rc
        if (c_associated(self%ctx)) rc = ps3d_gpu_destroy(self%ctx)
        self%ctx = c_null_ptr
    end subroutine gpu_release

end module gpu_stepper_mod
