!> @file m_gpu_bridge.f90
!! ISO_C_BINDING bridge from MicroFC's simulation host to the GB300 kernels
!! of libmfc_gpu.so (C ABI: include/mfc_gpu.h).
!!
!! Status: written for the reference's src/simulation tree, where it uses the
!! reference's m_derived_types, m_global_parameters and m_mpi_proxy modules.
!! It has not been compiled: no Fortran compiler exists where this library
!! is built and tested.  The same call sequence is exercised from C by
!! tests/c_host/p_main_host.c (test: tests/test_c_host.py), which binds
!! exactly the entry points declared below.
!!
!! Where the reference calls it (paths inside the MicroFC project):
!!   s_initialize_gpu_bridge   p_main.fpp:188-193, after s_initialize_derived_variables,
!!                             in place of the "!$acc update device(... q_cons_ts(1))"
!!   s_gpu_tvd_rk              m_time_steppers.fpp:129/197/271, the body of
!!                             s_{1st,2nd,3rd}_order_tvd_rk (one call per time step)
!!   s_gpu_compute_rhs         m_rhs.fpp:405, for hosts that keep their own integrator
!!   s_gpu_download_state      p_main.fpp:291-296, the save-step "!$acc update host"
!!                             and its NaN scan
!!   s_finalize_gpu_bridge     s_finalize_*_module
module m_gpu_bridge

    use iso_c_binding
    use m_derived_types        !< scalar_field
    use m_global_parameters    !< m, n, num_fluids, weno_order, weno_eps, time_stepper,
                               !! bc_x, bc_y, fluid_pp, x_cb, y_cb, dt, sys_size, buff_size,
                               !! Re_size, weno_Re_flux
    use m_mpi_proxy            !< s_mpi_abort

    implicit none

    private
    public :: s_initialize_gpu_bridge, s_gpu_tvd_rk, s_gpu_compute_rhs, &
              s_gpu_download_state, s_finalize_gpu_bridge

    integer(c_int32_t), parameter :: MFC_PREC_FP64 = 0, MFC_PREC_SPLIT = 1
    integer(c_int32_t), parameter :: MFC_FLAG_NAN = 1

    !> include/mfc_gpu.h: mfc_params (same member order and kinds)
    type, bind(C) :: mfc_params_t
        integer(c_int32_t) :: m, n, p
        integer(c_int32_t) :: num_fluids
        integer(c_int32_t) :: weno_order
        real(c_double) :: weno_eps
        integer(c_int32_t) :: time_stepper
        integer(c_int32_t) :: bc_x_beg, bc_x_end, bc_y_beg, bc_y_end, bc_z_beg, bc_z_end
        real(c_double) :: gammas(4), pi_infs(4)
        type(c_ptr) :: x_cb, y_cb, z_cb
        integer(c_int32_t) :: precision
        integer(c_int32_t) :: device
    end type mfc_params_t

    type(c_ptr) :: ctx = c_null_ptr     !< the device context (opaque mfc_gpu_ctx*)
    type(mfc_params_t), target :: prm

    interface
        integer(c_int) function mfc_gpu_init(params, ctx_out) bind(C, name='mfc_gpu_init')
            import :: mfc_params_t, c_int, c_ptr
            type(mfc_params_t), intent(in) :: params
            type(c_ptr), intent(out) :: ctx_out
        end function mfc_gpu_init

        integer(c_int) function mfc_gpu_upload(c, var, host_sf, ld_y, ld_z) bind(C, name='mfc_gpu_upload')
            import :: c_ptr, c_int, c_int64_t
            type(c_ptr), value :: c
            integer(c_int), value :: var
            type(c_ptr), value :: host_sf
            integer(c_int64_t), value :: ld_y, ld_z
        end function mfc_gpu_upload

        integer(c_int) function mfc_gpu_download(c, var, host_sf, ld_y, ld_z) bind(C, name='mfc_gpu_download')
            import :: c_ptr, c_int, c_int64_t
            type(c_ptr), value :: c
            integer(c_int), value :: var
            type(c_ptr), value :: host_sf
            integer(c_int64_t), value :: ld_y, ld_z
        end function mfc_gpu_download

        integer(c_int) function mfc_gpu_tvd_rk(c, dt_step, last_step) bind(C, name='mfc_gpu_tvd_rk')
            import :: c_ptr, c_int, c_double
            type(c_ptr), value :: c
            real(c_double), value :: dt_step
            integer(c_int), value :: last_step
        end function mfc_gpu_tvd_rk

        integer(c_int) function mfc_gpu_compute_rhs(c, rhs_out, prim_out) bind(C, name='mfc_gpu_compute_rhs')
            import :: c_ptr, c_int
            type(c_ptr), value :: c, rhs_out, prim_out
        end function mfc_gpu_compute_rhs

        integer(c_int) function mfc_gpu_status(c, flags, clear) bind(C, name='mfc_gpu_status')
            import :: c_ptr, c_int, c_int32_t
            type(c_ptr), value :: c
            integer(c_int32_t), intent(out) :: flags
            integer(c_int), value :: clear
        end function mfc_gpu_status

        integer(c_int) function mfc_gpu_finalize(c) bind(C, name='mfc_gpu_finalize')
            import :: c_ptr, c_int
            type(c_ptr), value :: c
        end function mfc_gpu_finalize

        type(c_ptr) function mfc_gpu_last_error() bind(C, name='mfc_gpu_last_error')
            import :: c_ptr
        end function mfc_gpu_last_error

        integer(c_int) function mfc_gpu_set_viscosity(c, re_shear, re_bulk) bind(C, name='mfc_gpu_set_viscosity')
            import :: c_ptr, c_int, c_double
            type(c_ptr), value :: c
            real(c_double), dimension(*), intent(in) :: re_shear, re_bulk
        end function mfc_gpu_set_viscosity

        integer(c_int) function mfc_gpu_set_viscous_gradients(c, weno_re_flux) &
            bind(C, name='mfc_gpu_set_viscous_gradients')
            import :: c_ptr, c_int
            type(c_ptr), value :: c
            integer(c_int), value :: weno_re_flux
        end function mfc_gpu_set_viscous_gradients
    end interface

contains

    !> Prints the library's message and aborts, as the reference does on a
    !! failed input check (m_start_up.fpp:108-109).
    subroutine s_check(ierr, what)
        integer(c_int), intent(in) :: ierr
        character(len=*), intent(in) :: what
        character(kind=c_char), pointer :: msg(:)
        integer :: i, k

        if (ierr == 0) return
        call c_f_pointer(mfc_gpu_last_error(), msg, [4096])
        k = 0
        do i = 1, 4096
            if (msg(i) == c_null_char) exit
            k = i
        end do
        print '(A,A,I0,A,4096A)', what, ': status ', ierr, ': ', msg(1:k)
        call s_mpi_abort()
    end subroutine s_check

    !> Creates the device context from the namelist globals and uploads
    !! q_cons_ts(1): each sf(-b:m+b, -b:n+b) is passed from sf(0, 0) with the
    !! leading dimension m + 2*buff_size + 1.  Viscous cases (a positive
    !! fluid_pp(i)%Re, Re_size > 0) pass the Reynolds numbers of every fluid,
    !! the unset ones as the namelist default (negative: no viscosity), and
    !! weno_Re_flux picks the WENO velocity gradients.
    subroutine s_initialize_gpu_bridge(q_cons_vf, device)
        type(scalar_field), dimension(sys_size), intent(in) :: q_cons_vf
        integer, intent(in) :: device
        real(c_double) :: re_shear(num_fluids), re_bulk(num_fluids)
        integer :: i

        prm%m = m; prm%n = n; prm%p = 0
        prm%num_fluids = num_fluids
        prm%weno_order = weno_order
        prm%weno_eps = weno_eps
        prm%time_stepper = time_stepper
        prm%bc_x_beg = bc_x%beg; prm%bc_x_end = bc_x%end
        prm%bc_y_beg = bc_y%beg; prm%bc_y_end = bc_y%end
        prm%bc_z_beg = -3; prm%bc_z_end = -3
        prm%gammas = 0d0; prm%pi_infs = 0d0
        do i = 1, num_fluids
            prm%gammas(i) = fluid_pp(i)%gamma
            prm%pi_infs(i) = fluid_pp(i)%pi_inf
        end do
        prm%x_cb = c_loc(x_cb(-1))
        prm%y_cb = c_null_ptr
        if (n > 0) prm%y_cb = c_loc(y_cb(-1))
        prm%z_cb = c_null_ptr
        prm%precision = MFC_PREC_FP64
        prm%device = device

        call s_check(mfc_gpu_init(prm, ctx), 'mfc_gpu_init')
        if (any(Re_size > 0)) then
            do i = 1, num_fluids
                re_shear(i) = fluid_pp(i)%Re(1)
                re_bulk(i) = fluid_pp(i)%Re(2)
            end do
            call s_check(mfc_gpu_set_viscosity(ctx, re_shear, re_bulk), 'mfc_gpu_set_viscosity')
            if (weno_Re_flux) call s_check(mfc_gpu_set_viscous_gradients(ctx, 1_c_int), &
                                           'mfc_gpu_set_viscous_gradients')
        end if
        do i = 1, sys_size
            call s_check(mfc_gpu_upload(ctx, i - 1, c_loc(q_cons_vf(i)%sf(0, 0)), &
                                        int(m + 2*buff_size + 1, c_int64_t), 0_c_int64_t), 'mfc_gpu_upload')
        end do
    end subroutine s_initialize_gpu_bridge

    !> One TVD-RK time step of q_cons_ts(1) on the device (the whole body of
    !! s_{1st,2nd,3rd}_order_tvd_rk); at t_step == t_step_stop it does
    !! nothing, as s_compute_rhs returns early there (m_rhs.fpp:452).
    subroutine s_gpu_tvd_rk(t_step)
        integer, intent(in) :: t_step

        call s_check(mfc_gpu_tvd_rk(ctx, dt, merge(1_c_int, 0_c_int, t_step == t_step_stop)), 'mfc_gpu_tvd_rk')
    end subroutine s_gpu_tvd_rk

    !> s_compute_rhs of q_cons_ts(1) into contiguous [sys_size][n+1][m+1]
    !! host arrays (either may be absent).
    subroutine s_gpu_compute_rhs(rhs, prim)
        real(c_double), dimension(:, :, :), target, optional, intent(out) :: rhs, prim
        type(c_ptr) :: r, q

        r = c_null_ptr; q = c_null_ptr
        if (present(rhs)) r = c_loc(rhs)
        if (present(prim)) q = c_loc(prim)
        call s_check(mfc_gpu_compute_rhs(ctx, r, q), 'mfc_gpu_compute_rhs')
    end subroutine s_gpu_compute_rhs

    !> Save step: the device's NaN flag replaces the host scan of
    !! p_main.fpp:297-306, then q_cons_ts(1) is copied back variable by
    !! variable for s_write_data_files.
    subroutine s_gpu_download_state(q_cons_vf)
        type(scalar_field), dimension(sys_size), intent(inout) :: q_cons_vf
        integer(c_int32_t) :: flags
        integer :: i

        call s_check(mfc_gpu_status(ctx, flags, 0_c_int), 'mfc_gpu_status')
        if (iand(flags, MFC_FLAG_NAN) /= 0) then
            print *, 'NaN or Inf in the conservative state'
            STOP "Error"
        end if
        do i = 1, sys_size
            call s_check(mfc_gpu_download(ctx, i - 1, c_loc(q_cons_vf(i)%sf(0, 0)), &
                                          int(m + 2*buff_size + 1, c_int64_t), 0_c_int64_t), 'mfc_gpu_download')
        end do
    end subroutine s_gpu_download_state

    subroutine s_finalize_gpu_bridge()
        if (c_associated(ctx)) call s_check(mfc_gpu_finalize(ctx), 'mfc_gpu_finalize')
        ctx = c_null_ptr
    end subroutine s_finalize_gpu_bridge

end module m_gpu_bridge
