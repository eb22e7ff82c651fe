! shark_gpu_mod.f90 -- ISO_C_BINDING interface of libshark_gpu (include/shark_gpu.h).
!
! Compiled with the unchanged SHARK sources (add to MODOBJ in bin/Makefile, link -lshark_gpu).
! The derived type mirrors struct shark_gpu_config field by field (bind(C) gives the C layout).
module shark_gpu
  use iso_c_binding
  implicit none

  integer(c_int32_t), parameter :: SHARK_GPU_ABI_VERSION = 2
  integer, parameter :: SHARK_MAX_DUST = 64
  integer(c_int32_t), parameter :: SHARK_OK = 0
  integer(c_int32_t), parameter :: SHARK_SETUP_SOD = 1, SHARK_SETUP_DUSTYWAVE = 2, SHARK_SETUP_SI = 3
  integer(c_int32_t), parameter :: SHARK_SETUP_DISK_POLAR = 4, SHARK_SETUP_DUSTYTURB = 5
  integer(c_int32_t), parameter :: SHARK_SETUP_KH = 6, SHARK_SETUP_SEDOV = 7
  integer(c_int32_t), parameter :: SHARK_SETUP_DISK_CART = 8
  integer(c_int32_t), parameter :: SHARK_FLAG_DRAG = 1, SHARK_FLAG_BACK_REACTION = 2
  integer(c_int32_t), parameter :: SHARK_FLAG_FORCE_KICK = 4, SHARK_FLAG_FARGO = 8
  integer(c_int32_t), parameter :: SHARK_FLAG_GROWTH = 16, SHARK_FLAG_CHARGING = 32
  integer(c_int32_t), parameter :: SHARK_FLAG_VISCOSITY = 64, SHARK_FLAG_STATIC = 128
  integer(c_int32_t), parameter :: SHARK_PREC_FP64 = 0, SHARK_PREC_MIXED = 1
  integer(c_int32_t), parameter :: SHARK_CHARGE_RESISTIVITIES = 1, SHARK_CHARGE_ANALYTICAL = 2
  integer(c_int32_t), parameter :: SHARK_CHARGE_MLP_SEED = 4
  integer(c_int32_t), parameter :: SHARK_GROWTH_FRAGMENTATION = 1, SHARK_GROWTH_DRIFT = 2
  integer(c_int32_t), parameter :: SHARK_GROWTH_TURB = 4, SHARK_GROWTH_BROWNIAN = 8
  integer(c_int32_t), parameter :: SHARK_GROWTH_AMBIPOLAR = 16

  type, bind(C) :: shark_gpu_config
    integer(c_int32_t) :: abi_version, nx, ny, nghost, ndust, geom, gridspace, solver, solverdust
    integer(c_int32_t) :: slope_type, iso_cs, precision, setup, flags, device, pad0
    real(c_double) :: gamma, cfl, smallr, smallc, smallp, box_l, box_l_y, inner_r, cs0
    real(c_double) :: dust_ratio_min, rhograin
    real(c_double) :: dust_size(SHARK_MAX_DUST), dust_K(SHARK_MAX_DUST), dust_tstop(SHARK_MAX_DUST)
    real(c_double) :: dust_eps(SHARK_MAX_DUST), dust_stokes(SHARK_MAX_DUST)
    real(c_double) :: sod_rho_l, sod_rho_r, sod_P_l, sod_P_r
    integer(c_int32_t) :: sod_direction, pad1
    real(c_double) :: dw_rho_0, dw_delta_rho, dw_vx_0, dw_kx_wave
    real(c_double) :: si_q_shear, si_omega, si_eta_stream, si_rad0, si_rho_init, si_hoverr
    real(c_double) :: disk_mstar, disk_hoverr, disk_sigma0, disk_r0, disk_rout
    real(c_double) :: disk_r_relax, disk_n_rel, disk_temp_slope
    real(c_double) :: unit_l, unit_d, unit_t, mu_gas, T_cloud
    real(c_double) :: chg_x, chg_sigma_att, chg_mu_ions, chg_stick_el, chg_eps, chg_B0
    integer(c_int32_t) :: chg_nitermax, chg_mode
    real(c_double) :: turb_rho0, turb_mach, turb_tcorr
    integer(c_int32_t) :: turb_kmin, turb_kmax, turb_seed, pad2
    real(c_double) :: grw_smin, grw_smax, grw_sticking, grw_clustered, grw_cfl, grw_eps_thr
    real(c_double) :: grw_eps_thr_frag, grw_dtcontrol, grw_delta_vambi, grw_alpha_turb, grw_size_mono
    real(c_double) :: grw_slope_mono, grw_Abr, grw_gamma_grains, grw_estar_grains
    integer(c_int32_t) :: grw_kernel, grw_mode
    real(c_double) :: disk_alpha_visc
    real(c_double) :: kh_rho_dense, kh_rho_diffuse, kh_T_dense, kh_mach, kh_vy0, kh_kx
    real(c_double) :: sedov_rho_ext, sedov_P_ext, sedov_P_cen, sedov_r_expl
    real(c_double) :: cdisk_smooth_r, cdisk_frac_r_disk, cdisk_buffer_in, cdisk_buffer_out
    type(c_ptr) :: dx, surf, vol, radii_c, position, cs
  end type shark_gpu_config

  interface
    integer(c_int32_t) function shark_gpu_config_defaults(cfg) bind(C, name="shark_gpu_config_defaults")
      import :: c_int32_t, shark_gpu_config
      type(shark_gpu_config), intent(out) :: cfg
    end function
    integer(c_int32_t) function shark_gpu_init(cfg, ctx) bind(C, name="shark_gpu_init")
      import :: c_int32_t, c_ptr, shark_gpu_config
      type(shark_gpu_config), intent(in) :: cfg
      type(c_ptr), intent(out) :: ctx
    end function
    integer(c_int32_t) function shark_gpu_upload(ctx, u_prim, ncells, nvar) bind(C, name="shark_gpu_upload")
      import :: c_int32_t, c_int64_t, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: u_prim(*)
      integer(c_int64_t), value :: ncells
      integer(c_int32_t), value :: nvar
    end function
    integer(c_int32_t) function shark_gpu_step(ctx, dt, status) bind(C, name="shark_gpu_step")
      import :: c_int32_t, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: dt
      integer(c_int32_t), intent(out) :: status
    end function
    integer(c_int32_t) function shark_gpu_download(ctx, u_prim, q) bind(C, name="shark_gpu_download")
      import :: c_int32_t, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: u_prim(*)
      type(c_ptr), value :: q
    end function
    integer(c_int32_t) function shark_gpu_ctoprim(ctx, q, cs) bind(C, name="shark_gpu_ctoprim")
      import :: c_int32_t, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: q(*), cs(*)
    end function
    integer(c_int32_t) function shark_gpu_totals(ctx, out) bind(C, name="shark_gpu_totals")
      import :: c_int32_t, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: out(*)
    end function
    ! output(iout) from the device (write_output.f90:2-300); prefix and dir are C strings
    ! (terminate them with c_null_char)
    integer(c_int32_t) function shark_gpu_output(ctx, iout, time, prefix) bind(C, name="shark_gpu_output")
      import :: c_int32_t, c_ptr, c_double, c_char
      type(c_ptr), value :: ctx
      integer(c_int32_t), value :: iout
      real(c_double), value :: time
      character(kind=c_char), intent(in) :: prefix(*)
    end function
    integer(c_int32_t) function shark_gpu_read_output(ctx, dir, time) bind(C, name="shark_gpu_read_output")
      import :: c_int32_t, c_ptr, c_double, c_char
      type(c_ptr), value :: ctx
      character(kind=c_char), intent(in) :: dir(*)
      real(c_double), intent(out) :: time
    end function
    ! last charging outputs (Fortran order): zd(ncells,N), ni, ne, psi_old (ncells),
    ! eta(ncells,3) = (eta_o, eta_H, eta_a), gamma_d(ncells,N), iterations; c_null_ptr skips one
    integer(c_int32_t) function shark_gpu_download_charge(ctx, zd, ni, ne, psi, eta, gamma_d, iters) &
        bind(C, name="shark_gpu_download_charge")
      import :: c_int32_t, c_ptr
      type(c_ptr), value :: ctx, zd, ni, ne, psi, eta, gamma_d, iters
    end function
    integer(c_int32_t) function shark_gpu_free(ctx) bind(C, name="shark_gpu_free")
      import :: c_int32_t, c_ptr
      type(c_ptr), value :: ctx
    end function
  end interface

  type(c_ptr), save :: gpu_ctx = c_null_ptr
  logical, save :: gpu_uploaded = .false.

contains

  ! Address of a contiguous real array for the config's grid pointers.  The library reads them
  ! only inside shark_gpu_init, so the address need not outlive that call.
  function shark_loc(a) result(p)
    real(c_double), target, intent(in) :: a(*)
    type(c_ptr) :: p
    p = c_loc(a(1))
  end function shark_loc
end module shark_gpu
