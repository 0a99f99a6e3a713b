! pizza_gpu.f90 -- ISO_C_BINDING interface to libpizza_gb300.so (include/pizza_gpu.h).
!
! A GPU build of pizza.exe adds this module and calls it from time_loop in
! place of the stage body (src/step_time.f90:216-368).  Every entry point of
! pizza_gpu.h has one interface here, with the same name, argument order and
! meaning.  Conventions of the C side that matter to a Fortran caller:
!  - complex(c_double_complex) arrays are passed as they are: the library's
!    spectral layout is pizza's f(n_m, n_r) with n_m fastest;
!  - pointer arguments that the C side accepts as NULL are OPTIONAL here
!    (Fortran 2018 interoperability: an absent argument passes NULL);
!  - the handle is an opaque type(c_ptr);
!  - pz_explicit_terms* take DEVICE addresses (type(c_ptr), value), e.g. from
!    a CUDA Fortran or OpenACC host_data region;
!  - every function returns PZ_OK (0) or a negative PZ_E_* code.
! The layout of type(pz_config) is checked against the C struct by the
! library's CPU tests (field order, kinds, offsets).
module pizza_gpu
   use iso_c_binding
   implicit none

   integer(c_int), parameter :: PZ_OK = 0
   integer(c_int), parameter :: PZ_E_ARG = -1
   integer(c_int), parameter :: PZ_E_CUDA = -2
   integer(c_int), parameter :: PZ_E_SINGULAR = -3
   integer(c_int), parameter :: PZ_E_DT_TOO_SMALL = -4
   integer(c_int), parameter :: PZ_E_NONFINITE = -5
   integer(c_int), parameter :: PZ_E_UNSUPPORTED = -6
   integer(c_int), parameter :: PZ_E_NOMEM = -7

   ! time_scheme values (src/multistep_schemes.f90, src/dirk_schemes.f90)
   integer(c_int), parameter :: PZ_CNAB2 = 0, PZ_SBDF2 = 1, PZ_SBDF3 = 2, PZ_SBDF4 = 3
   integer(c_int), parameter :: PZ_CNLF = 4, PZ_MODCNAB = 5, PZ_TVB33 = 6
   integer(c_int), parameter :: PZ_ARS222 = 10, PZ_ARS232 = 11, PZ_ARS233 = 12, PZ_SSP222 = 13
   integer(c_int), parameter :: PZ_LSDIRK222 = 14, PZ_LZ232 = 15, PZ_CK232 = 16, PZ_ARS443 = 17
   integer(c_int), parameter :: PZ_BPR353 = 18, PZ_PC2 = 19, PZ_ARS343 = 20, PZ_MARS343 = 21
   integer(c_int), parameter :: PZ_SSP322 = 22, PZ_SSP332 = 23
   integer(c_int), parameter :: PZ_SSP433 = 24, PZ_DP1_242 = 25, PZ_DP2_242 = 26, PZ_LZ453 = 27
   integer(c_int), parameter :: PZ_KC343 = 28, PZ_KC564 = 29, PZ_KC785 = 30, PZ_DBM453 = 31

   integer(c_int), parameter :: PZ_SOLVE_INFLUENCE = 0, PZ_SOLVE_DIRECT = 1
   integer(c_int), parameter :: PZ_CHEB_COLL = 0, PZ_CHEB_INTEG = 1
   integer(c_int), parameter :: PZ_TS_VISC = 0, PZ_TS_ROT = 1
   integer(c_int), parameter :: PZ_SERIES_COLS = 22
   integer(c_int), parameter :: PZ_KERNEL_KINDS = 10
   integer(c_int), parameter :: PZ_NOALLOC_MAX_MN = 32768
   integer(c_int), parameter :: PZ_OBJ_EKIN3D = 0, PZ_OBJ_NUTOP = 1
   integer(c_int), parameter :: PZ_INTEG_OPS = 19
   integer(c_int), parameter :: PZ_TUNE_FAST_G = 0, PZ_TUNE_RLOOP_RG = 1, PZ_TUNE_LANES = 2

   ! One instance's namelist values, the C struct pz_config field by field.
   type, bind(c) :: pz_config
      integer(c_int) :: n_r_max, n_cheb_max, m_max, minc
      real(c_double) :: ra, ek, pr, radratio
      real(c_double) :: g0, g1, g2
      integer(c_int) :: ktopt, kbott
      integer(c_int) :: ktopv, kbotv
      integer(c_int) :: l_ek_pump
      integer(c_int) :: l_non_rot
      integer(c_int) :: l_temp_advz
      integer(c_int) :: time_scheme
      integer(c_int) :: matrix_solve
      integer(c_int) :: corio_imp
      integer(c_int) :: buo_imp
      real(c_double) :: dtMax
      real(c_double) :: courfac
      real(c_double) :: alpha
      real(c_double) :: dt_fac
      integer(c_int) :: cheb_method
      integer(c_int) :: time_scale
      integer(c_int) :: l_rerror_fix
      real(c_double) :: rerror_fac
      real(c_double) :: raxi, sc
      integer(c_int) :: ktopxi, kbotxi
      real(c_double) :: xicond_fac
   end type pz_config

   interface
      subroutine pz_config_default(cfg) bind(c, name='pz_config_default')
         import :: pz_config
         type(pz_config), intent(out) :: cfg
      end subroutine pz_config_default

      integer(c_int) function pz_create(cfgs, n_instances, out) bind(c, name='pz_create')
         import :: pz_config, c_int, c_ptr
         type(pz_config), intent(in) :: cfgs(*)
         integer(c_int), value :: n_instances
         type(c_ptr), intent(out) :: out
      end function pz_create

      integer(c_int) function pz_set_state(h, inst, us, up, temp) bind(c, name='pz_set_state')
         import :: c_ptr, c_int, c_double_complex
         type(c_ptr), value :: h
         integer(c_int), value :: inst
         complex(c_double_complex), intent(in), optional :: us(*), up(*), temp(*)
      end function pz_set_state

      integer(c_int) function pz_set_state_all(h, us, up, temp) bind(c, name='pz_set_state_all')
         import :: c_ptr, c_int, c_double_complex
         type(c_ptr), value :: h
         complex(c_double_complex), intent(in), optional :: us(*), up(*), temp(*)
      end function pz_set_state_all

      integer(c_int) function pz_set_state_xi(h, inst, us, up, temp, xi) bind(c, name='pz_set_state_xi')
         import :: c_ptr, c_int, c_double_complex
         type(c_ptr), value :: h
         integer(c_int), value :: inst
         complex(c_double_complex), intent(in), optional :: us(*), up(*), temp(*), xi(*)
      end function pz_set_state_xi

      integer(c_int) function pz_get_state_xi(h, inst, xi, dxi) bind(c, name='pz_get_state_xi')
         import :: c_ptr, c_int, c_double_complex
         type(c_ptr), value :: h
         integer(c_int), value :: inst
         complex(c_double_complex), intent(out), optional :: xi(*), dxi(*)
      end function pz_get_state_xi

      integer(c_int) function pz_step(h, n_steps) bind(c, name='pz_step')
         import :: c_ptr, c_int
         type(c_ptr), value :: h
         integer(c_int), value :: n_steps
      end function pz_step

      integer(c_int) function pz_sync(h) bind(c, name='pz_sync')
         import :: c_ptr, c_int
         type(c_ptr), value :: h
      end function pz_sync

      integer(c_int) function pz_get_state(h, inst, us, up, om, psi, temp, dtemp, time, dt) &
            bind(c, name='pz_get_state')
         import :: c_ptr, c_int, c_double, c_double_complex
         type(c_ptr), value :: h
         integer(c_int), value :: inst
         complex(c_double_complex), intent(out), optional :: us(*), up(*), om(*), psi(*), temp(*), dtemp(*)
         real(c_double), intent(out), optional :: time, dt
      end function pz_get_state

      integer(c_int) function pz_get_history(h, inst, field, kind, slot, out) bind(c, name='pz_get_history')
         import :: c_ptr, c_int, c_double_complex
         type(c_ptr), value :: h
         integer(c_int), value :: inst, field, kind, slot
         complex(c_double_complex), intent(out) :: out(*)
      end function pz_get_history

      integer(c_int) function pz_set_history(h, inst, field, kind, slot, in) bind(c, name='pz_set_history')
         import :: c_ptr, c_int, c_double_complex
         type(c_ptr), value :: h
         integer(c_int), value :: inst, field, kind, slot
         complex(c_double_complex), intent(in) :: in(*)
      end function pz_set_history

      integer(c_int) function pz_get_step_state(h, inst, time, dt, n_step) bind(c, name='pz_get_step_state')
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: h
         integer(c_int), value :: inst
         real(c_double), intent(out), optional :: time
         real(c_double), intent(out), optional :: dt(*)
         integer(c_int), intent(out), optional :: n_step
      end function pz_get_step_state

      integer(c_int) function pz_set_step_state(h, inst, time, dt, n_step) bind(c, name='pz_set_step_state')
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: h
         integer(c_int), value :: inst
         real(c_double), value :: time
         real(c_double), intent(in) :: dt(*)
         integer(c_int), value :: n_step
      end function pz_set_step_state

      integer(c_int) function pz_get_spectra(h, inst, out) bind(c, name='pz_get_spectra')
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: h
         integer(c_int), value :: inst
         real(c_double), intent(out) :: out(5, *)
      end function pz_get_spectra

      integer(c_int) function pz_get_spectra_2d(h, inst, out) bind(c, name='pz_get_spectra_2d')
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: h
         integer(c_int), value :: inst
         real(c_double), intent(out) :: out(*)
      end function pz_get_spectra_2d

      integer(c_int) function pz_balance_step(h, inst, vort, vp) bind(c, name='pz_balance_step')
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: h
         integer(c_int), value :: inst
         real(c_double), intent(out) :: vort(*), vp(*)
      end function pz_balance_step

      integer(c_int) function pz_set_restart_ab1(h, inst, l_ab1) bind(c, name='pz_set_restart_ab1')
         import :: c_ptr, c_int
         type(c_ptr), value :: h
         integer(c_int), value :: inst, l_ab1
      end function pz_set_restart_ab1

      ! rows(PZ_SERIES_COLS, n_rows): one time-series row per column of the array
      integer(c_int) function pz_get_series(h, inst, rows, n_rows) bind(c, name='pz_get_series')
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: h
         integer(c_int), value :: inst
         real(c_double), intent(out) :: rows(22, *)
         integer(c_int), intent(inout) :: n_rows
      end function pz_get_series

      integer(c_int) function pz_get_dims(h, inst, n_r_max, n_m_max, n_phi_max) bind(c, name='pz_get_dims')
         import :: c_ptr, c_int
         type(c_ptr), value :: h
         integer(c_int), value :: inst
         integer(c_int), intent(out), optional :: n_r_max, n_m_max, n_phi_max
      end function pz_get_dims

      integer(c_int) function pz_launches_per_step(h) bind(c, name='pz_launches_per_step')
         import :: c_ptr, c_int
         type(c_ptr), value :: h
      end function pz_launches_per_step

      ! rows(PZ_SERIES_COLS, n_instances)
      integer(c_int) function pz_latest_rows(h, rows) bind(c, name='pz_latest_rows')
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: h
         real(c_double), intent(out) :: rows(22, *)
      end function pz_latest_rows

      ! the cudaStream_t of the handle
      type(c_ptr) function pz_stream(h) bind(c, name='pz_stream')
         import :: c_ptr
         type(c_ptr), value :: h
      end function pz_stream

      integer(c_int) function pz_step_profile(h, n_steps, kernel_ms) bind(c, name='pz_step_profile')
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: h
         integer(c_int), value :: n_steps
         real(c_double), intent(out) :: kernel_ms(*)
      end function pz_step_profile

      ! a C string (c_f_pointer it into a character buffer)
      type(c_ptr) function pz_kernel_name(k) bind(c, name='pz_kernel_name')
         import :: c_ptr, c_int
         integer(c_int), value :: k
      end function pz_kernel_name

      ! device addresses of complex (n_m, n_r) arrays and of two n_r_max vectors
      integer(c_int) function pz_explicit_terms(h, inst, us, up, om, temp, dTdt_expl, dpsidt_expl, dtr, dth) &
            bind(c, name='pz_explicit_terms')
         import :: c_ptr, c_int
         type(c_ptr), value :: h
         integer(c_int), value :: inst
         type(c_ptr), value :: us, up, om, temp, dTdt_expl, dpsidt_expl, dtr, dth
      end function pz_explicit_terms

      integer(c_int) function pz_explicit_terms_noalloc(h, inst, us, up, om, temp, dTdt_expl, dpsidt_expl, &
            dtr, dth) bind(c, name='pz_explicit_terms_noalloc')
         import :: c_ptr, c_int
         type(c_ptr), value :: h
         integer(c_int), value :: inst
         type(c_ptr), value :: us, up, om, temp, dTdt_expl, dpsidt_expl, dtr, dth
      end function pz_explicit_terms_noalloc

      integer(c_int) function pz_adjoint_forward(h, objective, n_steps, n_window, checkpoint_every, dt_sched, &
            J, dt_used) bind(c, name='pz_adjoint_forward')
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: h
         integer(c_int), value :: objective, n_steps, n_window, checkpoint_every
         real(c_double), intent(in), optional :: dt_sched(*)
         real(c_double), intent(out), optional :: J(*), dt_used(*)
      end function pz_adjoint_forward

      integer(c_int) function pz_adjoint_backward(h, dJ_dtemp, dJ_dra) bind(c, name='pz_adjoint_backward')
         import :: c_ptr, c_int, c_double, c_double_complex
         type(c_ptr), value :: h
         complex(c_double_complex), intent(out), optional :: dJ_dtemp(*)
         real(c_double), intent(out), optional :: dJ_dra(*)
      end function pz_adjoint_backward

      integer(c_int) function pz_adjoint_grid_snapshots(h, enable) bind(c, name='pz_adjoint_grid_snapshots')
         import :: c_ptr, c_int
         type(c_ptr), value :: h
         integer(c_int), value :: enable
      end function pz_adjoint_grid_snapshots

      integer(c_int) function pz_set_ra(h, inst, ra) bind(c, name='pz_set_ra')
         import :: c_ptr, c_int, c_double
         type(c_ptr), value :: h
         integer(c_int), value :: inst
         real(c_double), value :: ra
      end function pz_set_ra

      integer(c_int) function pz_integ_operator(n_r_max, radratio, which, out, bandwidth) &
            bind(c, name='pz_integ_operator')
         import :: c_int, c_double
         integer(c_int), value :: n_r_max
         real(c_double), value :: radratio
         integer(c_int), value :: which
         real(c_double), intent(out) :: out(*)
         integer(c_int), intent(out) :: bandwidth
      end function pz_integ_operator

      integer(c_int) function pz_fast_path(enable) bind(c, name='pz_fast_path')
         import :: c_int
         integer(c_int), value :: enable
      end function pz_fast_path

      integer(c_int) function pz_integ_banded(enable) bind(c, name='pz_integ_banded')
         import :: c_int
         integer(c_int), value :: enable
      end function pz_integ_banded

      integer(c_int) function pz_tune_set(what, key, value) bind(c, name='pz_tune_set')
         import :: c_int
         integer(c_int), value :: what, key, value
      end function pz_tune_set

      integer(c_int) function pz_fast_eigen(n_r_max, radratio, m, lam, U) bind(c, name='pz_fast_eigen')
         import :: c_int, c_double
         integer(c_int), value :: n_r_max
         real(c_double), value :: radratio
         integer(c_int), value :: m
         real(c_double), intent(out) :: lam(*), U(*)
      end function pz_fast_eigen

      integer(c_int) function pz_probe_peaks(dfma_tflops, mma_bf16_tflops) bind(c, name='pz_probe_peaks')
         import :: c_int, c_double
         real(c_double), intent(out), optional :: dfma_tflops, mma_bf16_tflops
      end function pz_probe_peaks

      integer(c_int) function pz_destroy(h) bind(c, name='pz_destroy')
         import :: c_ptr, c_int
         type(c_ptr), value :: h
      end function pz_destroy

      type(c_ptr) function pz_last_error(h) bind(c, name='pz_last_error')
         import :: c_ptr
         type(c_ptr), value :: h
      end function pz_last_error
   end interface

contains

   ! pz_last_error as a Fortran string (at most len(msg) characters)
   subroutine pz_error_message(h, msg)
      type(c_ptr), intent(in) :: h
      character(len=*), intent(out) :: msg
      character(kind=c_char), pointer :: s(:)
      type(c_ptr) :: p
      integer :: i
      msg = ''
      p = pz_last_error(h)
      if (.not. c_associated(p)) return
      call c_f_pointer(p, s, [len(msg)])
      do i = 1, len(msg)
         if (s(i) == c_null_char) exit
         msg(i:i) = s(i)
      end do
   end subroutine pz_error_message

end module pizza_gpu
