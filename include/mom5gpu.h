/*
 * mom5gpu.h -- C ABI of the GB300 library for MOM5's tracer-advection and
 * split-explicit barotropic path.
 *
 * One mom5gpu_domain holds one ocean domain's grid, state and scratch in GPU
 * memory.  A Fortran host binds these entry points through ISO_C_BINDING
 * (mom5_gb300/fortran/mom5gpu_mod.F90); any C or Python host can do the same.
 *
 * Conventions
 *  - Every entry point returns an int status: MOM5GPU_OK (0) or a negative
 *    MOM5GPU_E* code.  Nothing aborts the caller.  mom5gpu_last_error() gives
 *    the message of the last failure on a domain.
 *  - Arrays crossing the boundary use the reference's memory layout: Fortran
 *    column-major over the data domain (isd:ied, jsd:jed) = (ni+2) x (nj+2)
 *    with a one-cell halo, then k = 1..nk (or 0..nk for wrho_bt).  A C caller
 *    sees a C array [nk][nj+2][ni+2].
 *  - Tracer numbers n and time levels (taum1, tau, taup1) are 1-based, exactly
 *    the values of ntracer and Time%taum1/tau/taup1 in the Fortran interfaces.
 *  - All work is queued on the domain's CUDA stream (mom5gpu_set_stream) and
 *    is asynchronous unless an entry point returns host data.
 *  - Domains are not thread-safe; distinct domains may be driven from
 *    different host threads concurrently.
 */
#ifndef MOM5GPU_H
#define MOM5GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define MOM5GPU_OK 0
#define MOM5GPU_EINVAL -1      /* bad argument (the reference aborts with mpp_error(FATAL)) */
#define MOM5GPU_ENOMEM -2      /* device allocation failed */
#define MOM5GPU_ECUDA -3       /* a CUDA runtime call failed */
#define MOM5GPU_ESTATE -4      /* called out of order (e.g. before the init routine) */
#define MOM5GPU_ECFL -5        /* barotropic gravity-wave CFL check failed */
#define MOM5GPU_ENUMERIC -6    /* non-finite value found in a checked field */
#define MOM5GPU_ETIMEDOUT -7   /* a bounded device wait gave up */
#define MOM5GPU_EUNSUPPORTED -8 /* option outside the implemented path */
#define MOM5GPU_EFULL -9       /* no free slot / HBM budget (serving admission) */

/* ---- enumerations shared with the reference ---------------------------- */
/* ocean_parameters.F90:141-142 */
#define MOM5GPU_BGRID 1
#define MOM5GPU_CGRID 2
/* tracer advection schemes, ocean_parameters.F90:148-162 (implemented subset) */
#define MOM5GPU_ADVECT_UPWIND 1
#define MOM5GPU_ADVECT_2ND_ORDER 2
#define MOM5GPU_ADVECT_4TH_ORDER 3
#define MOM5GPU_ADVECT_6TH_ORDER 4
#define MOM5GPU_ADVECT_QUICKER 5
#define MOM5GPU_ADVECT_QUICKMOM3 6 /* horizontal only (the vertical routine is undefined at k = nk) */
#define MOM5GPU_ADVECT_MDFL_SUP_B 7
#define MOM5GPU_ADVECT_MDPPM 8
#define MOM5GPU_ADVECT_MDFL_SWEBY 9
#define MOM5GPU_ADVECT_DST_LINEAR 10
#define MOM5GPU_ADVECT_PSOM 11

/* arithmetic of the advection kernels */
#define MOM5GPU_PRECISION_FP64 0  /* drop-in: IEEE FP64 in the reference's operation order */
#define MOM5GPU_PRECISION_MIXED 1 /* FP32 fluxes and limiters, FP64 tracer state */

/* ---- fields -------------------------------------------------------------- */
/* Shape classes: 2D = (ni+2)(nj+2); 3D = 2D*nk; 3DW = 2D*(nk+1);
 * "(n)" = per tracer, "(t)" = per time level 1..3. */
enum mom5gpu_field {
  /* grid metrics, 2D (ocean_types.F90:206-378) */
  MOM5GPU_DXT = 1, MOM5GPU_DYT, MOM5GPU_DXU, MOM5GPU_DYU, MOM5GPU_DXTE, MOM5GPU_DYTE, MOM5GPU_DXTN,
  MOM5GPU_DYTN, MOM5GPU_DAT, MOM5GPU_DATR, MOM5GPU_DXUR, MOM5GPU_DYUR, MOM5GPU_DXTER, MOM5GPU_DYTNR,
  MOM5GPU_DTE, MOM5GPU_DTW, MOM5GPU_DUS, MOM5GPU_DUN, MOM5GPU_DAUR, MOM5GPU_CORIOLIS_F,
  MOM5GPU_UMASK1,        /* Grd%umask(:,:,1) */
  MOM5GPU_TMASKEN_E1,    /* Grd%tmasken(:,:,1,1) */
  MOM5GPU_TMASKEN_N1,    /* Grd%tmasken(:,:,1,2) */
  MOM5GPU_DXT_DXTER,     /* C-grid face-area ratios (ocean_grids.F90), 2D */
  MOM5GPU_DYT_DYTER,
  MOM5GPU_DXT_DXTNR,
  MOM5GPU_DYT_DYTNR,
  /* 3D grid */
  MOM5GPU_TMASK = 40,    /* Grd%tmask, 3D */
  MOM5GPU_TMASKEN_E,     /* Grd%tmasken(:,:,:,1), 3D */
  MOM5GPU_TMASKEN_N,     /* Grd%tmasken(:,:,:,2), 3D */
  /* advection velocity (ocean_adv_vel_type, ocean_types.F90:408-417) */
  MOM5GPU_UHRHO_ET = 50, /* 3D */
  MOM5GPU_VHRHO_NT,      /* 3D */
  MOM5GPU_WRHO_BT,       /* 3DW, levels 0..nk */
  MOM5GPU_DIVERGE_T,     /* 3D, Adv_vel%diverge_t */
  /* thickness (ocean_thickness_type, ocean_types.F90:134-203) */
  MOM5GPU_RHO_DZT = 60,  /* 3D (t) */
  MOM5GPU_RHO_DZTR,      /* 3D */
  MOM5GPU_THICKU,        /* 2D (t) */
  MOM5GPU_THICKEN_E,     /* 2D, Thickness%thicken(:,:,1) */
  MOM5GPU_THICKEN_N,     /* 2D, Thickness%thicken(:,:,2) */
  MOM5GPU_RHO_DZU,       /* 3D (t), Thickness%rho_dzu (B grid) */
  MOM5GPU_RHO_DZTEN_E,   /* 3D, Thickness%rho_dzten(:,:,:,1) (C grid) */
  MOM5GPU_RHO_DZTEN_N,   /* 3D, Thickness%rho_dzten(:,:,:,2) */
  MOM5GPU_RHO_DZT_TENDENCY, /* 3D, Thickness%rho_dzt_tendency */
  MOM5GPU_MASS_SOURCE,   /* 3D, Thickness%mass_source */
  /* prognostic tracers (ocean_prog_tracer_type, ocean_types.F90:468-541) */
  MOM5GPU_TRACER = 70,   /* 3D (n)(t) */
  MOM5GPU_TH_TENDENCY,   /* 3D (n) */
  MOM5GPU_TMASK_LIMIT,   /* 3D (n) */
  MOM5GPU_TPME,          /* 2D (n), T_prog(n)%tpme */
  MOM5GPU_TRACER_ETA_SMOOTH, /* 2D (n), T_prog(n)%eta_smooth */
  MOM5GPU_PBOT_SMOOTH,   /* 2D (n), T_prog(n)%pbot_smooth */
  /* external mode (ocean_external_mode_type, ocean_types.F90:591-637) */
  MOM5GPU_ETA_T = 80,    /* 2D (t) */
  MOM5GPU_ETA_T_BAR,     /* 2D (t) */
  MOM5GPU_ETA_U,         /* 2D (t) */
  MOM5GPU_UDRHO_U,       /* 2D (t), Ext_mode%udrho(:,:,1,t) */
  MOM5GPU_UDRHO_V,       /* 2D (t), Ext_mode%udrho(:,:,2,t) */
  MOM5GPU_CONV_RHO_UD_T, /* 2D (t) */
  MOM5GPU_DETA_DT,       /* 2D */
  MOM5GPU_FORCING_BT_U,  /* 2D, Ext_mode%forcing_bt(:,:,1) */
  MOM5GPU_FORCING_BT_V,  /* 2D */
  MOM5GPU_SOURCE,        /* 2D, Ext_mode%source */
  MOM5GPU_ETA_SMOOTH,    /* 2D */
  MOM5GPU_PS,            /* 2D */
  MOM5GPU_GRAD_PS_X,     /* 2D */
  MOM5GPU_GRAD_PS_Y,     /* 2D */
  MOM5GPU_PATM = 100,    /* 2D, patm argument */
  MOM5GPU_PME,           /* 2D, pme argument */
  MOM5GPU_RIVER,         /* 2D, river argument */
  MOM5GPU_RHO_G,         /* 2D, module rho_g (grav*rho at k=1) */
  /* velocity (ocean_velocity_type, ocean_types.F90) */
  MOM5GPU_U_VEL = 110,   /* 3D (t), Velocity%u(:,:,:,1,t) */
  MOM5GPU_V_VEL,         /* 3D (t), Velocity%u(:,:,:,2,t) */
  MOM5GPU_ACCEL_U,       /* 3D, Velocity%accel(:,:,:,1) */
  MOM5GPU_ACCEL_V,       /* 3D, Velocity%accel(:,:,:,2) */
  MOM5GPU_SMF_U,         /* 2D, Velocity%smf(:,:,1) */
  MOM5GPU_SMF_V,
  MOM5GPU_BMF_U,         /* 2D, Velocity%bmf(:,:,1) */
  MOM5GPU_BMF_V,
  /* second-order moments of the PSOM scheme (ocean_types.F90 T_prog(n)%s0..syz,
   * allocated by psom_init, ocean_tracer_advect.F90:1798-1819); per tracer, 3D,
   * compute domain meaningful (the halo is not maintained) */
  MOM5GPU_PSOM_S0 = 120, /* 3D (n), mass-weighted tracer after the last sweep */
  MOM5GPU_PSOM_SX, MOM5GPU_PSOM_SXX, MOM5GPU_PSOM_SY, MOM5GPU_PSOM_SYY, MOM5GPU_PSOM_SZ, MOM5GPU_PSOM_SZZ,
  MOM5GPU_PSOM_SXY, MOM5GPU_PSOM_SXZ, MOM5GPU_PSOM_SYZ,
  /* thickness fields of update_ucell_thickness (ocean_thickness.F90:3507-3886),
   * ocean_thickness_type (ocean_types.F90:134-203) and Grd%umask */
  MOM5GPU_UMASK = 130,   /* 3D, Grd%umask (1 down to kmu, 0 below) */
  MOM5GPU_DZT,           /* 3D, Thickness%dzt */
  MOM5GPU_DZWT,          /* 3DW, Thickness%dzwt(:,:,0:nk) */
  MOM5GPU_DZU,           /* 3D, Thickness%dzu */
  MOM5GPU_DZWU,          /* 3DW, Thickness%dzwu(:,:,0:nk) */
  MOM5GPU_RHO_DZUR,      /* 3D, Thickness%rho_dzur */
  MOM5GPU_DZTEN_E,       /* 3D, Thickness%dzten(:,:,:,1) */
  MOM5GPU_DZTEN_N,       /* 3D, Thickness%dzten(:,:,:,2) */
  MOM5GPU_DEPTH_ZT,      /* 3D, Thickness%depth_zt */
  MOM5GPU_DEPTH_ZWT,     /* 3D, Thickness%depth_zwt */
  MOM5GPU_DEPTH_ZU,      /* 3D, Thickness%depth_zu */
  MOM5GPU_DEPTH_ZWU,     /* 3D, Thickness%depth_zwu */
  MOM5GPU_MASS_U,        /* 2D (t), Thickness%mass_u */
  MOM5GPU_MASS_EN_E,     /* 2D, Thickness%mass_en(:,:,1) */
  MOM5GPU_MASS_EN_N,     /* 2D, Thickness%mass_en(:,:,2) */
  /* barotropic friction of ocean_barotropic_forcing (udrho_lap / udrho_bih) */
  MOM5GPU_DYUE = 150,    /* 2D, Grd%dyue */
  MOM5GPU_DXUER,         /* 2D, Grd%dxuer */
  MOM5GPU_DXUN,          /* 2D, Grd%dxun */
  MOM5GPU_DYUNR,         /* 2D, Grd%dyunr */
  MOM5GPU_LAP_VISC_CEU,  /* 2D, lap_visc_ceu of ocean_lap_friction (zero unless set) */
  MOM5GPU_LAP_VISC_CNU,  /* 2D, lap_visc_cnu */
  MOM5GPU_BIH_VISC_CEU,  /* 2D, bih_visc_ceu of ocean_bih_friction (zero unless set) */
  MOM5GPU_BIH_VISC_CNU,  /* 2D, bih_visc_cnu */
  MOM5GPU_LAP_CEU_BACK,  /* 2D, background viscosities of ocean_barotropic_init */
  MOM5GPU_LAP_CNU_BACK,  /*     (ocean_barotropic.F90:1306-1341), formed from DXU, */
  MOM5GPU_BIH_CEU_BACK,  /*     DYU, UMASK1 and the udrho_*_vel_micom options by */
  MOM5GPU_BIH_CNU_BACK,  /*     mom5gpu_ocean_barotropic_forcing_tau */
  MOM5GPU_LAP_FRICTION_BT_U, /* 2D, Velocity%lap_friction_bt(:,:,1) */
  MOM5GPU_LAP_FRICTION_BT_V, /* 2D, Velocity%lap_friction_bt(:,:,2) */
  MOM5GPU_BIH_FRICTION_BT_U, /* 2D, Velocity%bih_friction_bt(:,:,1) */
  MOM5GPU_BIH_FRICTION_BT_V, /* 2D, Velocity%bih_friction_bt(:,:,2) */
  MOM5GPU_BIH_DEL2_VEL_U,    /* 2D, del2_vel(:,:,1) of ocean_bih_friction */
  MOM5GPU_BIH_DEL2_VEL_V,    /* 2D, del2_vel(:,:,2) */
  MOM5GPU_FIELD_END
};

/* ---- configuration ------------------------------------------------------- */
typedef struct mom5gpu_dims {
  int ni, nj, nk;          /* compute domain isc:iec = 1:ni, jsc:jec = 1:nj, 1:nk */
  int cyclic_x, cyclic_y;  /* periodic directions (mpp_domains cyclic flags) */
  int num_prog_tracers;
  int horz_grid;           /* MOM5GPU_BGRID or MOM5GPU_CGRID */
} mom5gpu_dims;

typedef struct mom5gpu_options {
  /* ocean_tracer_advect_nml, ocean_tracer_advect.F90:483-495 */
  int advect_sweby_all;          /* default 0 */
  int limit_with_upwind;         /* default 0 */
  int zero_tracer_advect_horz;   /* default 0 */
  int zero_tracer_advect_vert;   /* default 0 */
  /* ocean_barotropic_nml, ocean_barotropic.F90:607-614 */
  int barotropic_time_stepping_A; /* exactly one of A and B must be 1 */
  int barotropic_time_stepping_B;
  int initsum_with_bar;           /* default 1 */
  double pred_corr_gamma;         /* default 0.2 */
  /* ocean_parameters.F90:176, :194 */
  double rho0;                    /* 1035.0 */
  double grav;                    /* 9.80 */
  /* this library */
  int precision;                  /* MOM5GPU_PRECISION_FP64 (default) or _MIXED */
  /* ocean_barotropic_nml, ocean_barotropic.F90:528-529 */
  int zero_forcing_bt;            /* default 0 */
  int zero_nonlinear_forcing_bt;  /* default 0 */
  /* ocean_tracer_advect_nml psom_limit_prather, ocean_tracer_advect.F90:489 */
  int psom_limit_prather;         /* default 0: Merryfield-Holloway limiter */
  /* ocean_barotropic_nml, ocean_barotropic.F90:599-604: Laplacian / biharmonic
   * friction on udrho(tau) added to forcing_bt once per baroclinic step
   * (mom5gpu_ocean_barotropic_forcing_tau) */
  int udrho_lap;                  /* default 0 */
  int udrho_bih;                  /* default 0 */
  double udrho_lap_vel_micom;     /* default 0.05 m/s */
  double udrho_bih_vel_micom;     /* default 0.01 m/s */
} mom5gpu_options;

typedef struct mom5gpu_domain mom5gpu_domain;

/* Fill *opt with the reference's namelist defaults.  Neither barotropic time
 * stepping flag is set, as in the reference, whose init stops until one is. */
void mom5gpu_default_options(mom5gpu_options* opt);

/* Allocate one domain on the current CUDA device.  Replaces the allocations of
 * ocean_tracer_advect_init (ocean_tracer_advect.F90:507-756) and
 * ocean_barotropic_init (ocean_barotropic.F90:946-1780). */
int mom5gpu_create(const mom5gpu_dims* dims, const mom5gpu_options* opt, mom5gpu_domain** out);
void mom5gpu_destroy(mom5gpu_domain* d);
/* Message of the last failure on d; with d == NULL, of the last failed create. */
const char* mom5gpu_last_error(const mom5gpu_domain* d);
const char* mom5gpu_strerror(int status);
/* Queue subsequent work on `stream` (a cudaStream_t); NULL restores the domain's own stream. */
int mom5gpu_set_stream(mom5gpu_domain* d, void* stream);
int mom5gpu_synchronize(mom5gpu_domain* d);
/* Bytes of device memory held by d. */
size_t mom5gpu_device_bytes(const mom5gpu_domain* d);

/* ---- data movement ------------------------------------------------------ */
/* Number of doubles in field f (the size of one tracer / time level). */
size_t mom5gpu_field_count(const mom5gpu_domain* d, int field);
/* Copy a field in (out) from a host (on_device=0) or device (1) pointer.
 * n: tracer 1..num_prog_tracers or 0; level: time level 1..3 or 0. */
int mom5gpu_set_field(mom5gpu_domain* d, int field, int n, int level, const double* src, int on_device);
int mom5gpu_get_field(mom5gpu_domain* d, int field, int n, int level, double* dst, int on_device);
/* Queue a copy of field (n, level) between its device storage and host memory
 * on `stream` (a cudaStream_t; NULL = the domain's stream) and return without
 * waiting: to_device = 1 copies host -> device, 0 device -> host.  The host
 * buffer must stay valid until the stream has passed the copy, and must be
 * pinned for the copy to overlap other work.  Ordering against the domain's
 * stream is the caller's (events), as for any stream-ordered copy. */
int mom5gpu_copy_field_async(mom5gpu_domain* d, int field, int n, int level, double* host, int to_device,
                             void* stream);
/* Device address of a field (for aliasing by a caller that owns device code). */
int mom5gpu_field_device_ptr(mom5gpu_domain* d, int field, int n, int level, double** dptr);
/* Vertical grid for quicker_init and the barotropic CFL check: nominal dzt(nk),
 * zw(nk) and kmt (2D, int). */
int mom5gpu_set_vertical_grid(mom5gpu_domain* d, const double* dzt, const double* zw, const int* kmt);
/* Per-tracer field_table choices (ocean_tracer.F90:982-1066). */
int mom5gpu_set_tracer_scheme(mom5gpu_domain* d, int n, int horz_scheme, int vert_scheme,
                              double min_tracer_limit, double max_tracer_limit);
/* Edge limiter of the MDPPM scheme for tracer n (field_table ppm_hlimiter,
 * default 2): 1 Colella-Woodward 1984, 2 improved full constraint (Lin 2004),
 * 3 Suresh-Huynh 1997. */
int mom5gpu_set_ppm_limiter(mom5gpu_domain* d, int n, int ppm_hlimiter);
/* Moment limiter of the PSOM scheme for tracer n (field_table psom_limit,
 * ocean_tracer.F90:1013-1016; default 0, ocean_tpm_util.F90:86). */
int mom5gpu_set_psom_limit(mom5gpu_domain* d, int n, int psom_limit);
/* Time%itt0, the time-step counter whose value mod 6 orders the PSOM sweeps
 * (ocean_tracer_advect.F90:4592-4621); >= 0, default 0.  The library does not
 * advance it: the host sets it each step, as ocean_model does. */
int mom5gpu_set_itt0(mom5gpu_domain* d, long itt0);

/* Name and restart file of tracer n (T_prog(n)%name and %restart_file; default
 * "tracer<n>" in "ocean_tracer.res.nc", ocean_tpm_util.F90:76). */
int mom5gpu_set_tracer_name(mom5gpu_domain* d, int n, const char* name, const char* restart_file);

/* ---- restarts ------------------------------------------------------------ */
/* Write the prognostic state at time level `level` into directory dir as the
 * netCDF files fms_io save_restart writes (fms_io.F90:2996-3260, 64-bit offset
 * format): each tracer into its restart file (ocean_tracer.F90:2658-2681);
 * eta_t, conv_rho_ud_t, eta_t_bar, eta_u, patm_t, udrho, vdrho, forcing_u_bt,
 * forcing_v_bt into ocean_barotropic.res.nc (ocean_barotropic.F90:5240-5294,
 * two-level layout) when the barotropic state was set; the moments of PSOM
 * tracers into ocean_psom_moments.res.nc (ocean_tracer_advect.F90:1795-1843).
 * Compute-domain data, one time record, an fms checksum attribute per field. */
int mom5gpu_write_restart(mom5gpu_domain* d, const char* dir, int level);
/* Read those files back into time level `level` (restore_state): tracer files
 * are required; the barotropic file when the barotropic mode is initialised;
 * PSOM moments stay zero without their file (psom_init).  Dimensions must match
 * the domain; a checksum attribute that disagrees with the data is
 * MOM5GPU_ENUMERIC.  Halos are filled with the periodic images (0 elsewhere). */
int mom5gpu_read_restart(mom5gpu_domain* d, const char* dir, int level);

/* ---- initialisation (after the grid fields are set) ---------------------- */
/* ocean_tracer_advect_init's scheme set-up: quicker_init (:1442-1586) and
 * mdfl_init (:1644-1691). */
int mom5gpu_tracer_advect_init(mom5gpu_domain* d);
/* ocean_barotropic_init's time-step set-up (:1109-1115, :1195-1197,
 * :1283-1288, :1546-1662): nts = nint(2*dtuv/dtbt), cori1/cori2 and the
 * gravity-wave CFL check (MOM5GPU_ECFL when violated). */
int mom5gpu_barotropic_init(mom5gpu_domain* d, double dtuv, double dtbt);
int mom5gpu_barotropic_nts(const mom5gpu_domain* d);

/* ---- the hot path -------------------------------------------------------- */
/* horz_advect_tracer (ocean_tracer_advect.F90:1898-2083): add the horizontal
 * (or, for MDFL/DST, 3-D) advection tendency of tracer n to its th_tendency.
 * With advect_sweby_all and n == 1 it runs advect_tracer_sweby_all for every
 * tracer, as the reference does. */
int mom5gpu_horz_advect_tracer(mom5gpu_domain* d, int n, int taum1, int tau, double dtime);
/* vert_advect_tracer (ocean_tracer_advect.F90:2095-2226). */
int mom5gpu_vert_advect_tracer(mom5gpu_domain* d, int n, int taum1, int tau, double dtime);
/* advect_tracer_sweby_all (ocean_tracer_advect.F90:4104-4511). */
int mom5gpu_advect_tracer_sweby_all(mom5gpu_domain* d, int taum1, int tau, double dtime);
/* compute_tmask_limit (ocean_tracer.F90:2788-2892), tmask_limit_ts_same on
 * when index_temp/index_salt (1-based) are both > 0. */
int mom5gpu_compute_tmask_limit(mom5gpu_domain* d, int tau, int index_temp, int index_salt);
/* Set th_tendency of tracer n (0 = all) to zero. */
int mom5gpu_zero_th_tendency(mom5gpu_domain* d, int n);
/* Explicit update of tracer n (0 = all) (ocean_tracer.F90:2341-2350), then
 * the halo update of field(taup1) (ocean_model.F90:1903-1911). */
int mom5gpu_update_tracer(mom5gpu_domain* d, int n, int taum1, int taup1, double dtime);
/* update_advection_only (ocean_tracer.F90:2618-2649) for every tracer in one
 * call: zero th_tendency, horizontal + vertical advection, explicit update,
 * halo update. */
int mom5gpu_tracer_advection_step(mom5gpu_domain* d, int taum1, int tau, int taup1, double dtime);
/* Time the candidate launch shapes of mom5gpu_tracer_advection_step on this
 * domain (precision form: tile height 16, 24, 32 or 64 rows, plain, with a
 * cp.async tracer prefetch, or TMA-staged; FP64: y-pass rows per thread 2..16)
 * and keep the fastest.  The trials step taum1 = tau = 1 to
 * taup1 = 2: time level 2 of the tracers and th_tendency are overwritten.
 * A summary is written to report (may be NULL). */
int mom5gpu_autotune(mom5gpu_domain* d, double dtime, char* report, size_t report_len);
/* The launch shape autotune chose, or one to pin: precision-form tile height
 * (16, 24, 32 or 64 rows incl. halo); staging of the tile's operands: prefetch
 * 0 = plain loads, 1 = tracer levels prefetched by cp.async (height 16 only),
 * 2 = tiles staged by TMA with the tracer levels carried down the column in
 * registers (heights 16 and 24; domains of even ni, else the plain kernel),
 * 3 = the same with at most 5 tracers per block and two blocks per SM
 * (height 16);
 * FP64 y-pass rows per thread (0 = built-in choice, 2, 4, 8, 16).  Every shape
 * gives the same results bit for bit.  A TMA-staged launch whose bounded wait
 * gave up is reported by the next mom5gpu_synchronize as MOM5GPU_ETIMEDOUT. */
int mom5gpu_set_tuning(mom5gpu_domain* d, int rows, int prefetch, int tj);
/* Form of the exact B-grid barotropic subcycles (update_ocean_barotropic,
 * ocean_barotropic.F90:3344-3575): 0 (default) = momentum, and corrector with
 * the next subcycle's predictor, as two launches per subcycle (the predictor of
 * the first subcycle a third), replayed from a CUDA graph; 1 = one
 * launch per subcycle, each tile recomputing the ring of pressure and
 * transports it reads (about 11% more FP64 work); 2 = all subcycles of a step
 * in one cooperative launch, a bounded grid barrier between the phases (a wait
 * that gives up is reported by mom5gpu_synchronize as MOM5GPU_ETIMEDOUT; inside
 * a stream capture form 0 is used).  Forms 1 and 2 were slower
 * than 0 on every measured domain.  Every form gives the same results bit for
 * bit.  A domain in the precision form (MOM5GPU_PRECISION_MIXED) has forms 0
 * and 1 of its own subcycle (mode 2 runs form 0): form 1 was faster on a
 * 360x300 domain, where the launches set the time, and slower on 1440x1080;
 * both give the same bits. */
int mom5gpu_set_barotropic_fusion(mom5gpu_domain* d, int mode);
/* Self-test of the grid barrier of the cooperative subcycle launch: `rounds`
 * (1..100000) barriers over a full resident grid, after each of which every
 * block checks that every block arrived (MOM5GPU_ENUMERIC if one passed
 * early).  With unreachable != 0 each barrier waits for one block more than the
 * grid holds, so every wait runs out after about 8 ms of SM clocks and the
 * call returns MOM5GPU_ETIMEDOUT from the next mom5gpu_synchronize, the
 * context still usable.  MOM5GPU_EUNSUPPORTED without cooperative launch. */
int mom5gpu_grid_barrier_selftest(mom5gpu_domain* d, int rounds, int unreachable);
int mom5gpu_get_tuning(const mom5gpu_domain* d, int* rows, int* prefetch, int* tj);
/* eta_and_pbot_tendency (ocean_barotropic.F90:2668-2734), depth-based. */
int mom5gpu_eta_and_pbot_tendency(mom5gpu_domain* d, int tau);
/* eta_and_pbot_update (ocean_barotropic.F90:2290-2385), depth-based, no OBC. */
int mom5gpu_eta_and_pbot_update(mom5gpu_domain* d, int taum1, int taup1, double dtime);
/* update_ocean_barotropic (ocean_barotropic.F90:2763-3033), splitting branch,
 * depth-based, legacy halos, barotropic_halo = 1: pred_corr_tropic_depth_bgrid
 * (:3225-3579) or _cgrid (:3601-3965), then the time averages, conv_rho_ud_t,
 * eta_u, ps and grad_ps. */
int mom5gpu_update_ocean_barotropic(mom5gpu_domain* d, int tau, int taup1);
/* ocean_advection_velocity (ocean_advection_velocity.F90:568-672), T-cell
 * part: UHRHO_ET, VHRHO_NT (B grid: BAY/BAX of u*dyu*rho_dzu(tau) over dyte /
 * dxtn; C grid: u*rho_dzten*face-area ratios), DIVERGE_T and the continuity
 * WRHO_BT from PME, RIVER, RHO_DZT_TENDENCY and MASS_SOURCE (fields never set
 * read as zero).  The U-cell fluxes for momentum advection are not computed. */
int mom5gpu_ocean_advection_velocity(mom5gpu_domain* d, int tau);
/* Surface and bottom source terms of the explicit tracer step
 * (ocean_tracer.F90:2318-2336): th_tendency(k=1) += tmask*(pme*tpme + eta_smooth)
 * and th_tendency(kmt) += tmask*pbot_smooth on the compute domain, for tracer
 * n (0 = every tracer).  Reads PME and the per-tracer TPME, TRACER_ETA_SMOOTH
 * and PBOT_SMOOTH (zero until set); needs mom5gpu_set_vertical_grid (kmt). */
int mom5gpu_tracer_boundary_terms(mom5gpu_domain* d, int n);
/* Vertical coordinates (ocean_parameters.F90:107-112). */
#define MOM5GPU_GEOPOTENTIAL 1
#define MOM5GPU_ZSTAR 2
#define MOM5GPU_ZSIGMA 3
#define MOM5GPU_PRESSURE 4
#define MOM5GPU_PSTAR 5
#define MOM5GPU_PSIGMA 6
/* update_ucell_thickness (ocean_thickness.F90:3507-3886), without blobs: U-cell
 * and face thicknesses of time level taup1 from the T cells (geopotential: the
 * top U cell from eta_u(taup1) only; zsigma/psigma: copies; other coordinates:
 * the minimum of the neighbouring T cells, halos updated), rho_dzur, depth_zu,
 * depth_zwu, thicku(taup1), thicken, mass_u(taup1), mass_en.  kmu is the number
 * of wet levels of MOM5GPU_UMASK.  linear_free_surface and update_dzwu_k0 are
 * the ocean_thickness_nml switches (defaults 0 and 1).  The inputs of the
 * branch taken must have been set (MOM5GPU_ESTATE otherwise). */
int mom5gpu_update_ucell_thickness(mom5gpu_domain* d, int taup1, int vert_coordinate, int linear_free_surface,
                                   int update_dzwu_k0);
/* ocean_barotropic_forcing (ocean_barotropic.F90:3058-3141) without the
 * optional barotropic friction: FORCING_BT_U/V = sum_k tmasken*accel +
 * tmasken(k=1)*(smf - bmf) on the compute domain, zero halo then the single-PE
 * halo update; honours zero_forcing_bt and zero_nonlinear_forcing_bt. */
int mom5gpu_ocean_barotropic_forcing(mom5gpu_domain* d);
/* ocean_barotropic_forcing with Time%tau = tau: as mom5gpu_ocean_barotropic_forcing,
 * plus the barotropic friction on UDRHO_U/V(tau) (:3105-3120).  With udrho_lap:
 * lap_friction_barotropic (ocean_lap_friction.F90:423-446), BDX_EU(c_e*FDX_U(u))
 * + BDY_NU(c_n*FDY_U(u)) times umask with c = *_BACK + *_VISC
 * (ocean_operators.F90:917-930, :973-986, :1202-1215, :1258-1271); with udrho_bih:
 * bih_friction_barotropic (ocean_bih_friction.F90:416-454), the operator applied
 * twice and negated.  Each result has a zero halo and then the single-PE halo
 * update; it is written to LAP/BIH_FRICTION_BT_U/V (zero when its switch is off)
 * and forcing_bt = forcing_bt + friction_lap + friction_bih on the data domain,
 * before zero_forcing_bt.  The *_BACK viscosities are formed first, as
 * ocean_barotropic_init forms them.  mom5gpu_ocean_barotropic_forcing returns
 * MOM5GPU_EINVAL when either switch is set. */
int mom5gpu_ocean_barotropic_forcing_tau(mom5gpu_domain* d, int tau);

/* ---- diagnostics ---------------------------------------------------------- */
/* Global content of tracer n at a time level, sum of tmask*dat*rho_dzt(level)*T
 * (total_tracer, ocean_tracer_diag.F90:2380-2415) with a compensated,
 * fixed-order reduction (double-double), written to *out (host). */
int mom5gpu_global_tracer_content(mom5gpu_domain* d, int n, int level, double* out);
/* The same content as an exact fixed-point sum, for sums over decomposed
 * domains that must not depend on the decomposition (the reproducing global
 * sum of a 2-D block decomposition).  Each column's value (the reference's
 * k-sum) is truncated to a multiple of 2^-100 and added as an integer, split
 * into MOM5GPU_FIXED_CHUNKS 32-bit chunks (chunk i weighs 2^(32 i - 100)), each
 * summed in a signed 64-bit accumulator: acc[MOM5GPU_FIXED_CHUNKS] receives
 * the domain's accumulators (host).  Integer sums are exact and associative,
 * so the accumulators of the blocks of a decomposed domain, added element by
 * element in any order (an integer allreduce between ranks), equal those of
 * the whole domain.  Up to 2^31 columns per sum; MOM5GPU_ENUMERIC if a column
 * value is not finite or |value| >= 2^155. */
#define MOM5GPU_FIXED_CHUNKS 8
int mom5gpu_tracer_content_fixed(mom5gpu_domain* d, int n, int level, long long* acc);
/* The double nearest to the value of such accumulators (ties to even).
 * Needs no device. */
int mom5gpu_fixed_to_double(const long long* acc, double* out);
/* Sum of tmask1*dat*eta_t_bar(level), compensated, to *out (host). */
int mom5gpu_global_eta_integral(mom5gpu_domain* d, int field, int level, double* out);
/* 1 if any non-finite value is in tracer n (0 = all) at `level`, else 0, to *out. */
int mom5gpu_check_finite(mom5gpu_domain* d, int n, int level, int* out);

/* ---- profiling (the role of mpp_clock_begin/end, mpp_util.inc:797-904) ---- */
/* Record CUDA events around each section (advection passes, tracer update,
 * barotropic subcycle loop, ...) on the domain's stream. */
int mom5gpu_enable_timing(mom5gpu_domain* d, int on);
/* Total device milliseconds and number of calls of a named section since
 * timing was enabled; synchronises the stream.  Sections: "mdfl", "mdfl_mixed",
 * "tracer_update", "barotropic", "upwind", "quicker". */
int mom5gpu_timing_query(mom5gpu_domain* d, const char* section, double* total_ms, long* calls);
/* Number of kernels this domain has launched since creation. */
long mom5gpu_launch_count(const mom5gpu_domain* d);

/* ---- batching: many resident domains per launch ---------------------------
 * A batch groups resident domains so that one step of many domains costs a
 * handful of launches instead of a handful per domain: the FP64 advection
 * passes and each barotropic subcycle phase run as one launch over a work list
 * of (domain, block) items, and the precision form runs as one persistent
 * launch that drains a (domain, tile) queue.  Domains of a batch share the
 * precision, the tracer count (<= 10),
 * MDFL Sweby for every tracer, the B grid, and nts (mom5gpu_barotropic_init);
 * sizes may differ.  A batch borrows the domains: destroy it before them. */
typedef struct mom5gpu_batch mom5gpu_batch;
int mom5gpu_batch_create(mom5gpu_domain* const* domains, int ndomains, mom5gpu_batch** out);
void mom5gpu_batch_destroy(mom5gpu_batch* b);
const char* mom5gpu_batch_last_error(const mom5gpu_batch* b);
int mom5gpu_batch_set_stream(mom5gpu_batch* b, void* stream);
/* One baroclinic step -- MDFL advection of every tracer with the explicit
 * update, then update_ocean_barotropic -- of the domains index[0..count-1]
 * (positions in the batch), each at its own two-level time state: parity[i] = 0
 * steps tau = 1 -> taup1 = 2, 1 steps 2 -> 1 (taum1 = tau).  With count = -1
 * every domain is stepped with parity[0], from a CUDA graph captured on the
 * first such call for that parity and replayed afterwards. */
int mom5gpu_batch_step(mom5gpu_batch* b, const int* index, const int* parity, int count, double dtime);
/* Time the candidate launch shapes (precision-form tile height and resident
 * blocks per SM; FP64 y-pass rows per thread) on the whole batch and keep the
 * fastest.  Each trial is a parity-0 step: time level 1 is read, level 2 is
 * overwritten.  A summary is written to report (may be NULL). */
int mom5gpu_batch_autotune(mom5gpu_batch* b, double dtime, char* report, size_t report_len);
/* Read or set the launch shape directly (e.g. to reuse one autotune result on
 * several batches): rows = precision-form tile height (16 or 32; 24 = the
 * TMA-staged tiles, 24 rows or 32 for at most 4 tracers, one block per SM, for
 * every domain with an even ni, and the plain 32-row tiles for the others), tj
 * = FP64 y-pass rows per thread (0 = automatic, else 2, 4, 8 or 16),
 * blocks_per_sm = resident blocks per SM of the persistent launch of the plain
 * tiles (1..4).  A TMA-staged tile whose bounded
 * wait gave up is reported by the next mom5gpu_synchronize of its domain as
 * MOM5GPU_ETIMEDOUT. */
int mom5gpu_batch_get_tuning(const mom5gpu_batch* b, int* rows, int* tj, int* blocks_per_sm);
int mom5gpu_batch_set_tuning(mom5gpu_batch* b, int rows, int tj, int blocks_per_sm);
/* Device milliseconds of the last batch step (CUDA events on the batch stream). */
double mom5gpu_batch_last_ms(mom5gpu_batch* b);
/* Kernels launched by the batch since creation (graph replays count their kernels). */
long mom5gpu_batch_launch_count(const mom5gpu_batch* b);

/* ---- domain decomposition -------------------------------------------------
 * The reference runs one domain as a 2-D layout of blocks, one per processor
 * element, each with a one-cell halo kept current by mpp_update_domains
 * (set_ocean_domain, ocean_domains.F90:123-; halo updates of the MDFL
 * intermediates ocean_tracer_advect.F90:3912, :3970, of T(taup1)
 * ocean_model.F90:1903-1911, of the predicted eta ocean_barotropic.F90:3383
 * and of the barotropic outputs :2846-2901).  Here each block is its own
 * mom5gpu_domain, created NON-cyclic with the block's compute size (ni, nj >= 2)
 * and with its grid and inputs set on the whole data domain (halo included,
 * as after the reference's halo updates).  The entry points below split a step
 * into the phases between which the reference exchanges halos; the caller moves
 * each halo region from the neighbour that owns it (mom5gpu_copy_boxes on one
 * GPU; a send/receive between processes otherwise).  Decomposed stepping covers
 * the FP64 MDFL Sweby / DST-linear step with the explicit update (at most 10
 * tracers, advect_sweby_all or not) and the B-grid barotropic step. */

/* Sides of a block: halos of the four faces and the four corners. */
#define MOM5GPU_WEST 0
#define MOM5GPU_EAST 1
#define MOM5GPU_SOUTH 2
#define MOM5GPU_NORTH 3
#define MOM5GPU_SOUTHWEST 4
#define MOM5GPU_SOUTHEAST 5
#define MOM5GPU_NORTHWEST 6
#define MOM5GPU_NORTHEAST 7
/* What is exchanged (mom5gpu_halo_region / mom5gpu_halo_base). */
#define MOM5GPU_HALO_FIELD 1   /* one-cell halo of a field (all tracers when n = 0), faces and corners */
#define MOM5GPU_HALO_MDFL_Z 2  /* tracer_mdfl after the z pass: two columns, west and east */
#define MOM5GPU_HALO_MDFL_X 3  /* tracer_mdfl after the x pass: two rows, south and north */
#define MOM5GPU_HALO_BT_ETA 4  /* predicted eta of a subcycle (plane level = 0 or 1), faces and corners */
#define MOM5GPU_HALO_BT_PS 5   /* the surface pressure formed from it, faces and corners */
/* Roles: the region a block sends to its neighbour on `side`, or the region it
 * receives from that neighbour.  A block's SEND region for side s pairs with
 * its neighbour's RECV region for the opposite side. */
#define MOM5GPU_SEND 0
#define MOM5GPU_RECV 1

/* A strided 3-D box of doubles: n[0] x n[1] x n[2] elements, element (x,y,z) at
 * src + x*src_stride[0] + y*src_stride[1] + z*src_stride[2] (likewise dst). */
typedef struct mom5gpu_box {
  const double* src;
  double* dst;
  long src_stride[3];
  long dst_stride[3];
  int n[3];
} mom5gpu_box;

/* Declare which sides of d face a neighbouring block (1) or the edge of the
 * whole domain (0).  Allocates the MDFL halo strips.  A side facing a
 * neighbour takes its halo from the exchanges; a side at the edge keeps the
 * single-PE rule of a non-cyclic boundary (the halo holds zero). */
int mom5gpu_set_neighbours(mom5gpu_domain* d, int west, int east, int south, int north);
/* tmask_mdfl of a block with its two-cell halo from the neighbours, as
 * mdfl_init's halo update builds it (ocean_tracer_advect.F90:1660-1668): a host
 * array of (ni+4)*(nj+4)*nk values 0 or 1, i fastest, i = -1..ni+2.  Call
 * after mom5gpu_tracer_advect_init, which builds the single-PE mask. */
int mom5gpu_set_mask_halo2(mom5gpu_domain* d, const double* tmask_halo2);
/* Geometry of a halo region, relative to the base of its array
 * (mom5gpu_halo_base): offset of element (0,0,0), strides and extents.  Pure
 * host arithmetic on dims (no device call): level count nlev for
 * MOM5GPU_HALO_FIELD (nk, nk+1, 1, or ntr*nk for all tracers), ignored for the
 * other kinds.  MOM5GPU_EINVAL for a side the kind does not exchange. */
int mom5gpu_halo_region(const mom5gpu_dims* dims, int kind, int nlev, int side, int role, long* offset,
                        long stride[3], int n[3]);
/* Device base address of the array a halo region lives in: the field (field,
 * n, level) for MOM5GPU_HALO_FIELD; for the MDFL kinds the intermediate
 * (SEND) or its strip (RECV); for the barotropic kinds the scratch plane. */
int mom5gpu_halo_base(mom5gpu_domain* d, int kind, int field, int n, int level, int role, double** base);
/* Copy count boxes (device memory, same extents on both sides) in one launch on
 * `stream` (a cudaStream_t; NULL = the default stream). */
int mom5gpu_copy_boxes(const mom5gpu_box* boxes, int count, void* stream);
/* One pass of the FP64 MDFL step over every tracer (taum1 = tau, two-level):
 * pass 1 zeroes th_tendency's halo ring and runs the z pass, then exchange
 * MOM5GPU_HALO_MDFL_Z; pass 2 the x pass, then exchange MOM5GPU_HALO_MDFL_X;
 * pass 3 the y pass and th_tendency.  mom5gpu_update_tracer(d, 0, ...) then
 * updates every tracer; exchange MOM5GPU_HALO_FIELD of MOM5GPU_TRACER (n = 0)
 * at taup1 closes the step. */
int mom5gpu_mdfl_pass(mom5gpu_domain* d, int pass, int taum1, int tau, double dtime);
/* One phase of update_ocean_barotropic (B grid, FP64) for a decomposed block:
 *   0 start (time-average accumulators, subcycle state from tau),
 *   1 predictor of subcycle itime, then exchange MOM5GPU_HALO_BT_ETA with
 *     level = (itime + 1) % 2 (the plane the predictor wrote) and
 *     MOM5GPU_HALO_BT_PS,
 *   2 momentum and corrector of subcycle itime,
 *   3 time averages, then exchange MOM5GPU_HALO_FIELD of ETA_T_BAR, UDRHO_U,
 *     UDRHO_V at taup1,
 *   4 conv_rho_ud_t, eta_u, ps, then exchange CONV_RHO_UD_T and ETA_U at taup1,
 *   5 grad_ps.
 * Phases 1 and 2 run for itime = 1..nts in turn. */
int mom5gpu_barotropic_phase(mom5gpu_domain* d, int tau, int taup1, int phase, int itime);

/* ---- allocation-free variant ---------------------------------------------
 * No counterpart in the reference.  For callers that cannot let the library
 * allocate device memory (a model whose GPU memory is reserved by its own pool,
 * a process under a hard device-memory cap, or code that must not call
 * cudaMalloc/cudaFree because they synchronise the device): adds the MDFL Sweby
 * (scheme 9) or DST-linear (scheme 10) advection tendency of ONE tracer to
 * th_tendency, with the values mom5gpu_horz_advect_tracer gives under the
 * default options (FP64 precision, advect_sweby_all = 0,
 * zero_tracer_advect_horz = 0), without any device allocation.  Every pointer
 * is a caller-owned DEVICE array in the domain layout above: 2-D metrics (dat,
 * datr, dxte, dyte, dxtn, dytn), 3-D tmask (values 0.0 or 1.0 only: any other
 * value counts as wet here, where the domain API refuses it),
 * uhrho_et, vhrho_nt, rho_dzt(tau), T(taum1), th_tendency (read and written),
 * and wrho_bt with nk+1 levels.  Work is queued on `stream` (NULL = default).
 * Limit: (ni+2)*(nj+2)*nk <= 2097152 data-domain cells (and
 * (ni+4)*(nj+4)*nk <= 4194304); larger domains get MOM5GPU_EINVAL with a
 * message in mom5gpu_last_error(NULL).  The scratch is a 36 MB file-scope
 * device array held by every GPU that loads the library until exit; the first
 * call on each device looks up its address, so make that first call before any
 * stream capture.  The address is kept per device number for the process: it
 * belongs to the device's primary context, so the calls must run in that
 * context and not after a cudaDeviceReset.  Calls share the one array: calls
 * that overlap on the GPU race and must be serialised by the caller. */
int mom5gpu_mdfl_sweby_noalloc(const mom5gpu_dims* dims, int scheme, double dtime, const double* tmask,
                               const double* dat, const double* datr, const double* dxte, const double* dyte,
                               const double* dxtn, const double* dytn, const double* uhrho_et,
                               const double* vhrho_nt, const double* wrho_bt, const double* rho_dzt,
                               const double* T, double* th_tendency, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* MOM5GPU_H */
