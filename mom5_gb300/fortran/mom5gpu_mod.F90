!-----------------------------------------------------------------------
! mom5gpu_mod: ISO_C_BINDING interface to libmom5gpu.so (include/mom5gpu.h)
! and drop-in wrappers with the procedure names and dummy argument lists of
!   ocean_tracer_advect_mod : horz_advect_tracer, vert_advect_tracer
!                             (ocean_tracer_advect.F90:1898-1908, :2095-2104)
!   ocean_barotropic_mod    : update_ocean_barotropic, eta_and_pbot_tendency,
!                             eta_and_pbot_update
!                             (ocean_barotropic.F90:2763-2774, :2668, :2290)
!
! The device domain keeps the grid, the advection velocity and the tracer
! state resident.  The wrappers copy in only what the host changed since the
! last call (flags set by mom5gpu_mark_*), call the C entry point and copy the
! outputs the caller reads (th_tendency, Ext_mode fields) back.  Arrays are
! passed with their Fortran data-domain bounds (isd:ied, jsd:jed, ...), which
! is the layout the C ABI expects.
!
! Build (where a Fortran compiler exists):
!   gfortran -fdefault-real-8 -c mom5gpu_mod.F90   (after ocean_types_mod)
!   link with -L<repo>/mom5_gb300 -lmom5gpu -lcudart
!-----------------------------------------------------------------------
module mom5gpu_c
  use, intrinsic :: iso_c_binding
  implicit none
  public

  integer(c_int), parameter :: MOM5GPU_OK = 0
  integer(c_int), parameter :: MOM5GPU_BGRID = 1, MOM5GPU_CGRID = 2
  integer(c_int), parameter :: MOM5GPU_PRECISION_FP64 = 0, MOM5GPU_PRECISION_MIXED = 1
  ! field ids (enum mom5gpu_field)
  integer(c_int), parameter :: F_DXT = 1, F_DYT = 2, F_DXU = 3, F_DYU = 4, F_DXTE = 5, F_DYTE = 6, &
       F_DXTN = 7, F_DYTN = 8, F_DAT = 9, F_DATR = 10, F_DXUR = 11, F_DYUR = 12, F_DXTER = 13, &
       F_DYTNR = 14, F_DTE = 15, F_DTW = 16, F_DUS = 17, F_DUN = 18, F_DAUR = 19, F_CORIOLIS_F = 20, &
       F_UMASK1 = 21, F_TMASKEN_E1 = 22, F_TMASKEN_N1 = 23, F_TMASK = 40, F_UHRHO_ET = 50, &
       F_VHRHO_NT = 51, F_WRHO_BT = 52, F_RHO_DZT = 60, F_RHO_DZTR = 61, F_THICKU = 62, &
       F_THICKEN_E = 63, F_THICKEN_N = 64, F_TRACER = 70, F_TH_TENDENCY = 71, F_TMASK_LIMIT = 72, &
       F_ETA_T = 80, F_ETA_T_BAR = 81, F_ETA_U = 82, F_UDRHO_U = 83, F_UDRHO_V = 84, &
       F_CONV_RHO_UD_T = 85, F_DETA_DT = 86, F_FORCING_BT_U = 87, F_FORCING_BT_V = 88, &
       F_SOURCE = 89, F_ETA_SMOOTH = 90, F_PS = 91, F_GRAD_PS_X = 92, F_GRAD_PS_Y = 93, &
       F_PATM = 100, F_PME = 101, F_RIVER = 102, F_RHO_G = 103, &
       F_DXT_DXTER = 24, F_DYT_DYTER = 25, F_DXT_DXTNR = 26, F_DYT_DYTNR = 27, F_DIVERGE_T = 53, &
       F_RHO_DZU = 65, F_RHO_DZTEN_E = 66, F_RHO_DZTEN_N = 67, F_RHO_DZT_TENDENCY = 68, &
       F_MASS_SOURCE = 69, F_U_VEL = 110, F_V_VEL = 111, F_TMASKEN_E = 41, F_TMASKEN_N = 42, &
       F_TPME = 73, F_TRACER_ETA_SMOOTH = 74, F_PBOT_SMOOTH = 75, F_ACCEL_U = 112, F_ACCEL_V = 113, &
       F_SMF_U = 114, F_SMF_V = 115, F_BMF_U = 116, F_BMF_V = 117, &
       F_PSOM_S0 = 120, F_PSOM_SX = 121, F_PSOM_SXX = 122, F_PSOM_SY = 123, F_PSOM_SYY = 124, &
       F_PSOM_SZ = 125, F_PSOM_SZZ = 126, F_PSOM_SXY = 127, F_PSOM_SXZ = 128, F_PSOM_SYZ = 129, &
       F_UMASK = 130, F_DZT = 131, F_DZWT = 132, F_DZU = 133, F_DZWU = 134, F_RHO_DZUR = 135, &
       F_DZTEN_E = 136, F_DZTEN_N = 137, F_DEPTH_ZT = 138, F_DEPTH_ZWT = 139, F_DEPTH_ZU = 140, &
       F_DEPTH_ZWU = 141, F_MASS_U = 142, F_MASS_EN_E = 143, F_MASS_EN_N = 144, &
       F_DYUE = 150, F_DXUER = 151, F_DXUN = 152, F_DYUNR = 153, F_LAP_VISC_CEU = 154, F_LAP_VISC_CNU = 155, &
       F_BIH_VISC_CEU = 156, F_BIH_VISC_CNU = 157, F_LAP_CEU_BACK = 158, F_LAP_CNU_BACK = 159, &
       F_BIH_CEU_BACK = 160, F_BIH_CNU_BACK = 161, F_LAP_FRICTION_BT_U = 162, F_LAP_FRICTION_BT_V = 163, &
       F_BIH_FRICTION_BT_U = 164, F_BIH_FRICTION_BT_V = 165, F_BIH_DEL2_VEL_U = 166, F_BIH_DEL2_VEL_V = 167
  integer(c_int), parameter :: MOM5GPU_ADVECT_PSOM = 11
  integer, parameter :: MOM5GPU_FIXED_CHUNKS = 8

  type, bind(C) :: mom5gpu_dims
     integer(c_int) :: ni, nj, nk, cyclic_x, cyclic_y, num_prog_tracers, horz_grid
  end type mom5gpu_dims

  type, bind(C) :: mom5gpu_options
     integer(c_int) :: advect_sweby_all, limit_with_upwind, zero_tracer_advect_horz, zero_tracer_advect_vert
     integer(c_int) :: barotropic_time_stepping_A, barotropic_time_stepping_B, initsum_with_bar
     real(c_double) :: pred_corr_gamma, rho0, grav
     integer(c_int) :: precision
     integer(c_int) :: zero_forcing_bt, zero_nonlinear_forcing_bt
     integer(c_int) :: psom_limit_prather
     integer(c_int) :: udrho_lap, udrho_bih
     real(c_double) :: udrho_lap_vel_micom, udrho_bih_vel_micom
  end type mom5gpu_options

  interface
     subroutine mom5gpu_default_options(opt) bind(C, name="mom5gpu_default_options")
       import :: mom5gpu_options
       type(mom5gpu_options), intent(out) :: opt
     end subroutine
     integer(c_int) function mom5gpu_create(dims, opt, dom) bind(C, name="mom5gpu_create")
       import :: c_int, c_ptr, mom5gpu_dims, mom5gpu_options
       type(mom5gpu_dims), intent(in) :: dims
       type(mom5gpu_options), intent(in) :: opt
       type(c_ptr), intent(out) :: dom
     end function
     subroutine mom5gpu_destroy(dom) bind(C, name="mom5gpu_destroy")
       import :: c_ptr
       type(c_ptr), value :: dom
     end subroutine
     type(c_ptr) function mom5gpu_last_error(dom) bind(C, name="mom5gpu_last_error")
       import :: c_ptr
       type(c_ptr), value :: dom
     end function
     integer(c_int) function mom5gpu_set_field(dom, field, n, level, src, on_device) &
          bind(C, name="mom5gpu_set_field")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: dom
       integer(c_int), value :: field, n, level, on_device
       real(c_double), intent(in) :: src(*)
     end function
     integer(c_int) function mom5gpu_get_field(dom, field, n, level, dst, on_device) &
          bind(C, name="mom5gpu_get_field")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: dom
       integer(c_int), value :: field, n, level, on_device
       real(c_double), intent(out) :: dst(*)
     end function
     integer(c_int) function mom5gpu_set_vertical_grid(dom, dzt, zw, kmt) bind(C, name="mom5gpu_set_vertical_grid")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: dom
       real(c_double), intent(in) :: dzt(*), zw(*)
       integer(c_int), intent(in) :: kmt(*)
     end function
     integer(c_int) function mom5gpu_set_tracer_scheme(dom, n, horz, vert, tmin, tmax) &
          bind(C, name="mom5gpu_set_tracer_scheme")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: dom
       integer(c_int), value :: n, horz, vert
       real(c_double), value :: tmin, tmax
     end function
     integer(c_int) function mom5gpu_set_ppm_limiter(dom, n, lim) bind(C, name="mom5gpu_set_ppm_limiter")
       import :: c_int, c_ptr
       type(c_ptr), value :: dom
       integer(c_int), value :: n, lim
     end function
     integer(c_int) function mom5gpu_set_psom_limit(dom, n, on) bind(C, name="mom5gpu_set_psom_limit")
       import :: c_int, c_ptr
       type(c_ptr), value :: dom
       integer(c_int), value :: n, on
     end function
     integer(c_int) function mom5gpu_set_itt0(dom, itt0) bind(C, name="mom5gpu_set_itt0")
       import :: c_int, c_ptr, c_long
       type(c_ptr), value :: dom
       integer(c_long), value :: itt0
     end function
     integer(c_int) function mom5gpu_set_tracer_name(dom, n, name, restart_file) &
          bind(C, name="mom5gpu_set_tracer_name")
       import :: c_int, c_ptr, c_char
       type(c_ptr), value :: dom
       integer(c_int), value :: n
       character(kind=c_char), intent(in) :: name(*), restart_file(*)
     end function
     integer(c_int) function mom5gpu_write_restart(dom, dir, level) bind(C, name="mom5gpu_write_restart")
       import :: c_int, c_ptr, c_char
       type(c_ptr), value :: dom
       character(kind=c_char), intent(in) :: dir(*)
       integer(c_int), value :: level
     end function
     integer(c_int) function mom5gpu_read_restart(dom, dir, level) bind(C, name="mom5gpu_read_restart")
       import :: c_int, c_ptr, c_char
       type(c_ptr), value :: dom
       character(kind=c_char), intent(in) :: dir(*)
       integer(c_int), value :: level
     end function
     integer(c_int) function mom5gpu_tracer_advect_init(dom) bind(C, name="mom5gpu_tracer_advect_init")
       import :: c_int, c_ptr
       type(c_ptr), value :: dom
     end function
     integer(c_int) function mom5gpu_barotropic_init(dom, dtuv, dtbt) bind(C, name="mom5gpu_barotropic_init")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: dom
       real(c_double), value :: dtuv, dtbt
     end function
     integer(c_int) function mom5gpu_horz_advect_tracer(dom, n, taum1, tau, dtime) &
          bind(C, name="mom5gpu_horz_advect_tracer")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: dom
       integer(c_int), value :: n, taum1, tau
       real(c_double), value :: dtime
     end function
     integer(c_int) function mom5gpu_vert_advect_tracer(dom, n, taum1, tau, dtime) &
          bind(C, name="mom5gpu_vert_advect_tracer")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: dom
       integer(c_int), value :: n, taum1, tau
       real(c_double), value :: dtime
     end function
     integer(c_int) function mom5gpu_compute_tmask_limit(dom, tau, index_temp, index_salt) &
          bind(C, name="mom5gpu_compute_tmask_limit")
       import :: c_int, c_ptr
       type(c_ptr), value :: dom
       integer(c_int), value :: tau, index_temp, index_salt
     end function
     integer(c_int) function mom5gpu_zero_th_tendency(dom, n) bind(C, name="mom5gpu_zero_th_tendency")
       import :: c_int, c_ptr
       type(c_ptr), value :: dom
       integer(c_int), value :: n
     end function
     integer(c_int) function mom5gpu_update_tracer(dom, n, taum1, taup1, dtime) bind(C, name="mom5gpu_update_tracer")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: dom
       integer(c_int), value :: n, taum1, taup1
       real(c_double), value :: dtime
     end function
     integer(c_int) function mom5gpu_eta_and_pbot_tendency(dom, tau) bind(C, name="mom5gpu_eta_and_pbot_tendency")
       import :: c_int, c_ptr
       type(c_ptr), value :: dom
       integer(c_int), value :: tau
     end function
     integer(c_int) function mom5gpu_eta_and_pbot_update(dom, taum1, taup1, dtime) &
          bind(C, name="mom5gpu_eta_and_pbot_update")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: dom
       integer(c_int), value :: taum1, taup1
       real(c_double), value :: dtime
     end function
     integer(c_int) function mom5gpu_update_ocean_barotropic(dom, tau, taup1) &
          bind(C, name="mom5gpu_update_ocean_barotropic")
       import :: c_int, c_ptr
       type(c_ptr), value :: dom
       integer(c_int), value :: tau, taup1
     end function
     integer(c_int) function mom5gpu_ocean_advection_velocity(dom, tau) &
          bind(C, name="mom5gpu_ocean_advection_velocity")
       import :: c_int, c_ptr
       type(c_ptr), value :: dom
       integer(c_int), value :: tau
     end function
     integer(c_int) function mom5gpu_tracer_boundary_terms(dom, n) bind(C, name="mom5gpu_tracer_boundary_terms")
       import :: c_int, c_ptr
       type(c_ptr), value :: dom
       integer(c_int), value :: n
     end function
     integer(c_int) function mom5gpu_ocean_barotropic_forcing(dom) bind(C, name="mom5gpu_ocean_barotropic_forcing")
       import :: c_int, c_ptr
       type(c_ptr), value :: dom
     end function
     integer(c_int) function mom5gpu_ocean_barotropic_forcing_tau(dom, tau) &
          bind(C, name="mom5gpu_ocean_barotropic_forcing_tau")
       import :: c_int, c_ptr
       type(c_ptr), value :: dom
       integer(c_int), value :: tau
     end function
     integer(c_int) function mom5gpu_update_ucell_thickness(dom, taup1, vert_coordinate, linear_free_surface, &
          update_dzwu_k0) bind(C, name="mom5gpu_update_ucell_thickness")
       import :: c_int, c_ptr
       type(c_ptr), value :: dom
       integer(c_int), value :: taup1, vert_coordinate, linear_free_surface, update_dzwu_k0
     end function
     integer(c_int) function mom5gpu_global_tracer_content(dom, n, level, total) &
          bind(C, name="mom5gpu_global_tracer_content")
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: dom
       integer(c_int), value :: n, level
       real(c_double), intent(out) :: total
     end function
     integer(c_int) function mom5gpu_tracer_content_fixed(dom, n, level, acc) &
          bind(C, name="mom5gpu_tracer_content_fixed")
       import :: c_int, c_ptr, c_long_long, MOM5GPU_FIXED_CHUNKS
       type(c_ptr), value :: dom
       integer(c_int), value :: n, level
       integer(c_long_long), intent(out) :: acc(MOM5GPU_FIXED_CHUNKS)
     end function
     integer(c_int) function mom5gpu_fixed_to_double(acc, total) bind(C, name="mom5gpu_fixed_to_double")
       import :: c_int, c_long_long, c_double, MOM5GPU_FIXED_CHUNKS
       integer(c_long_long), intent(in) :: acc(MOM5GPU_FIXED_CHUNKS)
       real(c_double), intent(out) :: total
     end function
  end interface
end module mom5gpu_c


module mom5gpu_mod
  ! Drop-in wrappers.  ocean_tracer.F90:2300-2303 and ocean_model.F90:1752,
  ! :1819, :1941 call these exactly as they call the reference procedures once
  ! their use statements name this module instead of ocean_tracer_advect_mod
  ! and ocean_barotropic_mod.
  use, intrinsic :: iso_c_binding
  use mom5gpu_c
  use mpp_mod,          only: mpp_error, FATAL, mpp_sum
  use ocean_types_mod,  only: ocean_time_type, ocean_adv_vel_type, ocean_thickness_type, ocean_density_type, &
                              ocean_prog_tracer_type, ocean_external_mode_type, ocean_velocity_type, &
                              ocean_lagrangian_type, ocean_grid_type
  implicit none
  private

  public :: mom5gpu_attach, mom5gpu_mark_velocity_changed, mom5gpu_mark_state_changed
  public :: horz_advect_tracer, vert_advect_tracer
  public :: update_ocean_barotropic, eta_and_pbot_tendency, eta_and_pbot_update
  public :: ocean_advection_velocity, ocean_barotropic_forcing, device_restart_write
  public :: update_ucell_thickness, device_thickness_options, device_total_tracer

  ! ocean_thickness_nml switches and the vertical coordinate (ocean_parameters.F90:107-112)
  ! used by update_ucell_thickness; set once by the host driver
  integer(c_int), save :: thk_vert_coordinate = 1
  integer(c_int), save :: thk_linear_free_surface = 0, thk_update_dzwu_k0 = 1

  type(c_ptr), save :: dom = c_null_ptr
  logical, save :: velocity_dirty = .true.
  logical, save :: state_dirty = .true.
  logical, save :: velocity_on_device = .false.

contains

  subroutine check(st, where)
    integer(c_int), intent(in) :: st
    character(len=*), intent(in) :: where
    character(len=256), pointer :: msg
    type(c_ptr) :: p
    if (st /= MOM5GPU_OK) then
       p = mom5gpu_last_error(dom)
       call c_f_pointer(p, msg)
       call mpp_error(FATAL, 'mom5gpu ('//where//'): '//trim(msg(1:index(msg, c_null_char)-1)))
    endif
  end subroutine check

  ! total_tracer (ocean_tracer_diag.F90:2380-2415) of prognostic tracer n at
  ! time level `index`, the same on any processor count (the role of
  ! BITWISE_EXACT_SUM): each PE's device forms its exact fixed-point column
  ! sums, the integer accumulators are summed over the PEs (mpp_sum of
  ! integer(8), exact) and rounded once.
  function device_total_tracer(n, index) result(total)
    integer, intent(in) :: n, index
    real :: total
    integer(c_long_long) :: acc(MOM5GPU_FIXED_CHUNKS)
    real(c_double) :: t
    call check(mom5gpu_tracer_content_fixed(dom, int(n, c_int), int(index, c_int), acc), 'total_tracer')
    call mpp_sum(acc, MOM5GPU_FIXED_CHUNKS)
    call check(mom5gpu_fixed_to_double(acc, t), 'total_tracer')
    total = t
  end function device_total_tracer

  ! Called once from ocean_model_init after the grid and the first state exist:
  ! takes ownership of the device domain created by the host driver.
  subroutine mom5gpu_attach(handle)
    type(c_ptr), intent(in) :: handle
    dom = handle
  end subroutine mom5gpu_attach

  subroutine mom5gpu_mark_velocity_changed()
    velocity_dirty = .true.
  end subroutine mom5gpu_mark_velocity_changed

  subroutine mom5gpu_mark_state_changed()
    state_dirty = .true.
  end subroutine mom5gpu_mark_state_changed

  subroutine push_inputs(Time, Adv_vel, Thickness, T_prog)
    type(ocean_time_type),        intent(in) :: Time
    type(ocean_adv_vel_type),     intent(in) :: Adv_vel
    type(ocean_thickness_type),   intent(in) :: Thickness
    type(ocean_prog_tracer_type), intent(in) :: T_prog(:)
    integer :: n
    if (velocity_dirty) then
       if (.not. velocity_on_device) then
          call check(mom5gpu_set_field(dom, F_UHRHO_ET, 0, 0, Adv_vel%uhrho_et, 0), 'uhrho_et')
          call check(mom5gpu_set_field(dom, F_VHRHO_NT, 0, 0, Adv_vel%vhrho_nt, 0), 'vhrho_nt')
          call check(mom5gpu_set_field(dom, F_WRHO_BT, 0, 0, Adv_vel%wrho_bt, 0), 'wrho_bt')
       endif
       velocity_on_device = .false.
       call check(mom5gpu_set_field(dom, F_RHO_DZT, 0, Time%tau, Thickness%rho_dzt(:,:,:,Time%tau), 0), 'rho_dzt')
       call check(mom5gpu_set_field(dom, F_RHO_DZT, 0, Time%taum1, Thickness%rho_dzt(:,:,:,Time%taum1), 0), 'rho_dzt')
       call check(mom5gpu_set_field(dom, F_RHO_DZTR, 0, 0, Thickness%rho_dztr, 0), 'rho_dztr')
       velocity_dirty = .false.
    endif
    if (state_dirty) then
       do n = 1, size(T_prog)
          call check(mom5gpu_set_field(dom, F_TRACER, n, Time%taum1, T_prog(n)%field(:,:,:,Time%taum1), 0), 'T')
          if (Time%tau /= Time%taum1) &
             call check(mom5gpu_set_field(dom, F_TRACER, n, Time%tau, T_prog(n)%field(:,:,:,Time%tau), 0), 'T')
          call check(mom5gpu_set_field(dom, F_TH_TENDENCY, n, 0, T_prog(n)%th_tendency, 0), 'th_tendency')
       enddo
       state_dirty = .false.
    endif
  end subroutine push_inputs

  ! ocean_tracer_advect.F90:1898-1908
  subroutine horz_advect_tracer(Time, Adv_vel, Thickness, Dens, T_prog, Tracer, ntracer, dtime, store_flux)
    type(ocean_time_type),        intent(in)    :: Time
    type(ocean_adv_vel_type),     intent(in)    :: Adv_vel
    type(ocean_thickness_type),   intent(in)    :: Thickness
    type(ocean_density_type),     intent(in)    :: Dens
    type(ocean_prog_tracer_type), intent(inout) :: T_prog(:)
    type(ocean_prog_tracer_type), intent(inout) :: Tracer
    integer,                      intent(in)    :: ntracer
    real,                         intent(in)    :: dtime
    logical, optional,            intent(in)    :: store_flux
    call push_inputs(Time, Adv_vel, Thickness, T_prog)
    call check(mom5gpu_horz_advect_tracer(dom, int(ntracer, c_int), int(Time%taum1, c_int), int(Time%tau, c_int), &
         real(dtime, c_double)), 'horz_advect_tracer')
    call check(mom5gpu_get_field(dom, F_TH_TENDENCY, int(ntracer, c_int), 0, Tracer%th_tendency, 0), 'th_tendency')
  end subroutine horz_advect_tracer

  ! ocean_tracer_advect.F90:2095-2104
  subroutine vert_advect_tracer(Time, Adv_vel, Dens, Thickness, T_prog, Tracer, ntracer, dtime)
    type(ocean_time_type),        intent(in)    :: Time
    type(ocean_adv_vel_type),     intent(in)    :: Adv_vel
    type(ocean_density_type),     intent(in)    :: Dens
    type(ocean_thickness_type),   intent(in)    :: Thickness
    type(ocean_prog_tracer_type), intent(inout) :: T_prog(:)
    type(ocean_prog_tracer_type), intent(inout) :: Tracer
    integer,                      intent(in)    :: ntracer
    real,                         intent(in)    :: dtime
    call push_inputs(Time, Adv_vel, Thickness, T_prog)
    call check(mom5gpu_vert_advect_tracer(dom, int(ntracer, c_int), int(Time%taum1, c_int), int(Time%tau, c_int), &
         real(dtime, c_double)), 'vert_advect_tracer')
    call check(mom5gpu_get_field(dom, F_TH_TENDENCY, int(ntracer, c_int), 0, Tracer%th_tendency, 0), 'th_tendency')
    ! th_tendency is modified by other terms on the host before the next tracer call
    state_dirty = .true.
  end subroutine vert_advect_tracer

  ! ocean_barotropic.F90:2668
  subroutine eta_and_pbot_tendency(Time, pme, river, Ext_mode, use_blobs)
    type(ocean_time_type),          intent(in)    :: Time
    real, dimension(:,:),           intent(in)    :: pme, river
    type(ocean_external_mode_type), intent(inout) :: Ext_mode
    logical,                        intent(in)    :: use_blobs
    if (use_blobs) call mpp_error(FATAL, 'mom5gpu: use_blobs is outside the implemented path')
    call check(mom5gpu_set_field(dom, F_PME, 0, 0, pme, 0), 'pme')
    call check(mom5gpu_set_field(dom, F_RIVER, 0, 0, river, 0), 'river')
    call check(mom5gpu_set_field(dom, F_SOURCE, 0, 0, Ext_mode%source, 0), 'source')
    call check(mom5gpu_eta_and_pbot_tendency(dom, int(Time%tau, c_int)), 'eta_and_pbot_tendency')
    call check(mom5gpu_get_field(dom, F_DETA_DT, 0, 0, Ext_mode%deta_dt, 0), 'deta_dt')
  end subroutine eta_and_pbot_tendency

  ! ocean_barotropic.F90:2290
  subroutine eta_and_pbot_update(Time, Ext_mode)
    type(ocean_time_type),          intent(in)    :: Time
    type(ocean_external_mode_type), intent(inout) :: Ext_mode
    call check(mom5gpu_eta_and_pbot_update(dom, int(Time%taum1, c_int), int(Time%taup1, c_int), &
         real(Time%dtime_e, c_double)), 'eta_and_pbot_update')
    call check(mom5gpu_get_field(dom, F_ETA_T, 0, int(Time%taup1, c_int), Ext_mode%eta_t(:,:,Time%taup1), 0), 'eta_t')
  end subroutine eta_and_pbot_update

  ! ocean_barotropic.F90:2763-2774
  subroutine update_ocean_barotropic(Time, Dens, Thickness, Adv_vel, Ext_mode, patm, pme, river, use_blobs)
    type(ocean_time_type),          intent(in)    :: Time
    type(ocean_density_type),       intent(in)    :: Dens
    type(ocean_thickness_type),     intent(in)    :: Thickness
    type(ocean_adv_vel_type),       intent(in)    :: Adv_vel
    type(ocean_external_mode_type), intent(inout) :: Ext_mode
    real, dimension(:,:),           intent(in)    :: patm, pme, river
    logical,                        intent(in)    :: use_blobs
    integer(c_int) :: tau, taup1
    if (use_blobs) call mpp_error(FATAL, 'mom5gpu: use_blobs is outside the implemented path')
    tau = int(Time%tau, c_int)
    taup1 = int(Time%taup1, c_int)
    call check(mom5gpu_set_field(dom, F_PATM, 0, 0, patm, 0), 'patm')
    call check(mom5gpu_set_field(dom, F_PME, 0, 0, pme, 0), 'pme')
    call check(mom5gpu_set_field(dom, F_RIVER, 0, 0, river, 0), 'river')
    call check(mom5gpu_set_field(dom, F_FORCING_BT_U, 0, 0, Ext_mode%forcing_bt(:,:,1), 0), 'forcing_bt')
    call check(mom5gpu_set_field(dom, F_FORCING_BT_V, 0, 0, Ext_mode%forcing_bt(:,:,2), 0), 'forcing_bt')
    call check(mom5gpu_set_field(dom, F_THICKU, 0, tau, Thickness%thicku(:,:,Time%tau), 0), 'thicku')
    call check(mom5gpu_set_field(dom, F_SOURCE, 0, 0, Ext_mode%source, 0), 'source')
    call check(mom5gpu_set_field(dom, F_ETA_SMOOTH, 0, 0, Ext_mode%eta_smooth, 0), 'eta_smooth')
    call check(mom5gpu_update_ocean_barotropic(dom, tau, taup1), 'update_ocean_barotropic')
    call check(mom5gpu_get_field(dom, F_ETA_T_BAR, 0, taup1, Ext_mode%eta_t_bar(:,:,Time%taup1), 0), 'eta_t_bar')
    call check(mom5gpu_get_field(dom, F_UDRHO_U, 0, taup1, Ext_mode%udrho(:,:,1,Time%taup1), 0), 'udrho')
    call check(mom5gpu_get_field(dom, F_UDRHO_V, 0, taup1, Ext_mode%udrho(:,:,2,Time%taup1), 0), 'udrho')
    call check(mom5gpu_get_field(dom, F_CONV_RHO_UD_T, 0, taup1, Ext_mode%conv_rho_ud_t(:,:,Time%taup1), 0), 'conv')
    call check(mom5gpu_get_field(dom, F_ETA_U, 0, taup1, Ext_mode%eta_u(:,:,Time%taup1), 0), 'eta_u')
    call check(mom5gpu_get_field(dom, F_PS, 0, 0, Ext_mode%ps, 0), 'ps')
    call check(mom5gpu_get_field(dom, F_GRAD_PS_X, 0, 0, Ext_mode%grad_ps(:,:,1), 0), 'grad_ps')
    call check(mom5gpu_get_field(dom, F_GRAD_PS_Y, 0, 0, Ext_mode%grad_ps(:,:,2), 0), 'grad_ps')
  end subroutine update_ocean_barotropic

  ! ocean_advection_velocity.F90:568-579.  Computes the T-cell fluxes on the
  ! device (they stay there for the advection calls); the U-cell fluxes for
  ! momentum advection are left to the host's own routine.
  subroutine ocean_advection_velocity(Velocity, Time, Thickness, Dens, pme, river, Adv_vel, L_system, use_blobs)
    type(ocean_velocity_type),   intent(in)    :: Velocity
    type(ocean_time_type),       intent(in)    :: Time
    type(ocean_thickness_type),  intent(in)    :: Thickness
    type(ocean_density_type),    intent(in)    :: Dens
    real, dimension(:,:),        intent(in)    :: pme, river
    type(ocean_adv_vel_type),    intent(inout) :: Adv_vel
    type(ocean_lagrangian_type), intent(in)    :: L_system
    logical,                     intent(in)    :: use_blobs
    integer(c_int) :: tau
    if (use_blobs) call mpp_error(FATAL, 'mom5gpu: use_blobs is outside the implemented path')
    tau = int(Time%tau, c_int)
    call check(mom5gpu_set_field(dom, F_U_VEL, 0, tau, Velocity%u(:,:,:,1,Time%tau), 0), 'u')
    call check(mom5gpu_set_field(dom, F_V_VEL, 0, tau, Velocity%u(:,:,:,2,Time%tau), 0), 'v')
    call check(mom5gpu_set_field(dom, F_RHO_DZU, 0, tau, Thickness%rho_dzu(:,:,:,Time%tau), 0), 'rho_dzu')
    call check(mom5gpu_set_field(dom, F_RHO_DZT_TENDENCY, 0, 0, Thickness%rho_dzt_tendency, 0), 'rho_dzt_tendency')
    call check(mom5gpu_set_field(dom, F_MASS_SOURCE, 0, 0, Thickness%mass_source, 0), 'mass_source')
    call check(mom5gpu_set_field(dom, F_PME, 0, 0, pme, 0), 'pme')
    call check(mom5gpu_set_field(dom, F_RIVER, 0, 0, river, 0), 'river')
    call check(mom5gpu_ocean_advection_velocity(dom, tau), 'ocean_advection_velocity')
    call check(mom5gpu_get_field(dom, F_UHRHO_ET, 0, 0, Adv_vel%uhrho_et, 0), 'uhrho_et')
    call check(mom5gpu_get_field(dom, F_VHRHO_NT, 0, 0, Adv_vel%vhrho_nt, 0), 'vhrho_nt')
    call check(mom5gpu_get_field(dom, F_WRHO_BT, 0, 0, Adv_vel%wrho_bt, 0), 'wrho_bt')
    call check(mom5gpu_get_field(dom, F_DIVERGE_T, 0, 0, Adv_vel%diverge_t, 0), 'diverge_t')
    ! the device copy of the fluxes is current: the next advection call need
    ! not push them again (thickness is still pushed)
    velocity_on_device = .true.
  end subroutine ocean_advection_velocity

  ! ocean_barotropic.F90:3058-3062.  Velocity%accel, smf and bmf go to the device,
  ! Ext_mode%forcing_bt comes back (it also stays on the device for the subcycle).
  ! Grd%tmasken is copied once by the host driver (fields F_TMASKEN_E/N).
  subroutine ocean_barotropic_forcing(Time, Velocity, Ext_mode)
    type(ocean_time_type),          intent(in)    :: Time
    type(ocean_velocity_type),      intent(inout) :: Velocity
    type(ocean_external_mode_type), intent(inout) :: Ext_mode
    call check(mom5gpu_set_field(dom, F_ACCEL_U, 0, 0, Velocity%accel(:,:,:,1), 0), 'accel')
    call check(mom5gpu_set_field(dom, F_ACCEL_V, 0, 0, Velocity%accel(:,:,:,2), 0), 'accel')
    call check(mom5gpu_set_field(dom, F_SMF_U, 0, 0, Velocity%smf(:,:,1), 0), 'smf')
    call check(mom5gpu_set_field(dom, F_SMF_V, 0, 0, Velocity%smf(:,:,2), 0), 'smf')
    call check(mom5gpu_set_field(dom, F_BMF_U, 0, 0, Velocity%bmf(:,:,1), 0), 'bmf')
    call check(mom5gpu_set_field(dom, F_BMF_V, 0, 0, Velocity%bmf(:,:,2), 0), 'bmf')
    ! with udrho_lap / udrho_bih the friction acts on udrho(tau), which is on the
    ! device; lap_visc_* / bih_visc_* are set by the host after its friction modules
    ! form them (F_LAP_VISC_CEU ... F_BIH_VISC_CNU)
    call check(mom5gpu_ocean_barotropic_forcing_tau(dom, Time%tau), 'ocean_barotropic_forcing')
    call check(mom5gpu_get_field(dom, F_FORCING_BT_U, 0, 0, Ext_mode%forcing_bt(:,:,1), 0), 'forcing_bt')
    call check(mom5gpu_get_field(dom, F_FORCING_BT_V, 0, 0, Ext_mode%forcing_bt(:,:,2), 0), 'forcing_bt')
    call check(mom5gpu_get_field(dom, F_LAP_FRICTION_BT_U, 0, 0, Velocity%lap_friction_bt(:,:,1), 0), 'lap_friction_bt')
    call check(mom5gpu_get_field(dom, F_LAP_FRICTION_BT_V, 0, 0, Velocity%lap_friction_bt(:,:,2), 0), 'lap_friction_bt')
    call check(mom5gpu_get_field(dom, F_BIH_FRICTION_BT_U, 0, 0, Velocity%bih_friction_bt(:,:,1), 0), 'bih_friction_bt')
    call check(mom5gpu_get_field(dom, F_BIH_FRICTION_BT_V, 0, 0, Velocity%bih_friction_bt(:,:,2), 0), 'bih_friction_bt')
  end subroutine ocean_barotropic_forcing

  subroutine device_thickness_options(vert_coordinate, linear_free_surface, update_dzwu_k0)
    integer, intent(in) :: vert_coordinate
    logical, intent(in) :: linear_free_surface, update_dzwu_k0
    thk_vert_coordinate = vert_coordinate
    thk_linear_free_surface = merge(1, 0, linear_free_surface)
    thk_update_dzwu_k0 = merge(1, 0, update_dzwu_k0)
  end subroutine device_thickness_options

  ! ocean_thickness.F90:3507-3512, no blobs.  The T-cell thickness fields
  ! (F_DZT, F_DZWT, F_RHO_DZT, F_DEPTH_ZT, F_DEPTH_ZWT), Grd%umask (F_UMASK) and
  ! Grd%tmasken are on the device (copied by the host driver); eta_u(taup1) goes
  ! to the device and the U-cell and face thicknesses come back.
  subroutine update_ucell_thickness(Time, Grid, Ext_mode, Thickness)
    type(ocean_time_type),          intent(in)    :: Time
    type(ocean_grid_type),          intent(in)    :: Grid
    type(ocean_external_mode_type), intent(in)    :: Ext_mode
    type(ocean_thickness_type),     intent(inout) :: Thickness
    integer :: taup1
    taup1 = Time%taup1
    call check(mom5gpu_set_field(dom, F_ETA_U, 0, taup1, Ext_mode%eta_u(:,:,taup1), 0), 'eta_u')
    call check(mom5gpu_update_ucell_thickness(dom, taup1, thk_vert_coordinate, thk_linear_free_surface, &
         thk_update_dzwu_k0), 'update_ucell_thickness')
    call check(mom5gpu_get_field(dom, F_DZU, 0, 0, Thickness%dzu, 0), 'dzu')
    call check(mom5gpu_get_field(dom, F_DZWU, 0, 0, Thickness%dzwu, 0), 'dzwu')
    call check(mom5gpu_get_field(dom, F_RHO_DZU, 0, taup1, Thickness%rho_dzu(:,:,:,taup1), 0), 'rho_dzu')
    call check(mom5gpu_get_field(dom, F_RHO_DZUR, 0, 0, Thickness%rho_dzur, 0), 'rho_dzur')
    call check(mom5gpu_get_field(dom, F_DZTEN_E, 0, 0, Thickness%dzten(:,:,:,1), 0), 'dzten')
    call check(mom5gpu_get_field(dom, F_DZTEN_N, 0, 0, Thickness%dzten(:,:,:,2), 0), 'dzten')
    call check(mom5gpu_get_field(dom, F_RHO_DZTEN_E, 0, 0, Thickness%rho_dzten(:,:,:,1), 0), 'rho_dzten')
    call check(mom5gpu_get_field(dom, F_RHO_DZTEN_N, 0, 0, Thickness%rho_dzten(:,:,:,2), 0), 'rho_dzten')
    call check(mom5gpu_get_field(dom, F_DEPTH_ZU, 0, 0, Thickness%depth_zu, 0), 'depth_zu')
    call check(mom5gpu_get_field(dom, F_DEPTH_ZWU, 0, 0, Thickness%depth_zwu, 0), 'depth_zwu')
    call check(mom5gpu_get_field(dom, F_THICKU, 0, taup1, Thickness%thicku(:,:,taup1), 0), 'thicku')
    call check(mom5gpu_get_field(dom, F_THICKEN_E, 0, 0, Thickness%thicken(:,:,1), 0), 'thicken')
    call check(mom5gpu_get_field(dom, F_THICKEN_N, 0, 0, Thickness%thicken(:,:,2), 0), 'thicken')
    call check(mom5gpu_get_field(dom, F_MASS_U, 0, taup1, Thickness%mass_u(:,:,taup1), 0), 'mass_u')
    call check(mom5gpu_get_field(dom, F_MASS_EN_E, 0, 0, Thickness%mass_en(:,:,1), 0), 'mass_en')
    call check(mom5gpu_get_field(dom, F_MASS_EN_N, 0, 0, Thickness%mass_en(:,:,2), 0), 'mass_en')
  end subroutine update_ucell_thickness

  ! The restart files of the device-resident state at Time%taup1, in the layout
  ! save_restart writes (ocean_tracer_restart, ocean_tracer.F90:2658-2681, and the
  ! barotropic and PSOM files); directory is usually 'RESTART'.
  subroutine device_restart_write(Time, directory)
    type(ocean_time_type), intent(in) :: Time
    character(len=*),      intent(in) :: directory
    call check(mom5gpu_write_restart(dom, trim(directory)//c_null_char, int(Time%taup1, c_int)), 'write_restart')
  end subroutine device_restart_write

end module mom5gpu_mod
