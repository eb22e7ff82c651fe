! solve_gpu.f90 -- drop-in replacement of src/solver/solve.f90 that runs each step on the GPU.
!
! Build: put this file (and shark_gpu_mod.f90) before src/solver on VPATH instead of solve.f90,
! add -DSHARK_GPU_SETUP=<1 SOD | 2 DUSTYWAVE | 3 SI | 4 disk_polar | 5 dustyTurb | 6 KH | 7 sedov |
! 8 disk (Cartesian)>
! and -DSHARK_GPU_PREC=<0 FP64 | 1 mixed>
! to DEFINES and link with -L<repo>/shark_gb300 -lshark_gpu.  The time loop (src/shark.f90),
! setups, namelists and output stay as they are.
!
! solve   : first call builds the configuration from the module parameters, creates the GPU
!           context and uploads u_prim; every call runs one step on the device and sets dt.
!           Before an iteration whose check_output will write (every freq_out steps) the state is
!           downloaded into u_prim and q so the unchanged output routines see it, and with
!           charging the charges and abundances it writes (zd, ni, ne, psi_old, the
!           resistivities and gamma_d).
!
! Setup 4 (disk_polar): the reference's disk has a constant H/R, i.e. T ~ 1/r (temperature
! slope -1); its dust bins all have the size the setup gave them (scut).  Setup 5 (dustyTurb):
! stopping times St_0 box_l rho_0/(cs rho) (dustyTurb/setup.f90:456); compiled with TURB>0, the
! turb_params namelist drives the device's 2D solenoidal Ornstein-Uhlenbeck forcing
! (Mach_x_target, k_min..k_max as wavenumbers 2 pi n/box_l, turnover_time as the correlation
! time, iseed) in place of the reference's 1D driving.
! ctoprim : primitive variables; from the device once the GPU owns the state, on the host before.
! primtoc : conservative from primitive variables (host; used by the setups).
subroutine solve(verbose,outputing)
  use parameters
  use commons
  use units
  use phys_const, only: pi
  use shark_gpu
#if NDUST>0
  use ionisation_commons
#endif
#if SHARK_GPU_SETUP==5 && TURB>0
  use turb_commons
#endif
  implicit none
  logical :: verbose, outputing
  type(shark_gpu_config) :: cfg
  integer(c_int32_t) :: rc, st
  integer, save :: nsolve = 0
  integer :: idust

  if (.not. gpu_uploaded) then
    rc = shark_gpu_config_defaults(cfg)
    cfg%nx = NX; cfg%ny = NY; cfg%nghost = NGHOST; cfg%ndust = NDUST
    cfg%geom = GEOM; cfg%gridspace = GRIDSPACE; cfg%solver = SOLVER; cfg%solverdust = SOLVERDUST
    cfg%slope_type = slope_type; cfg%iso_cs = iso_cs; cfg%precision = SHARK_GPU_PREC
    cfg%setup = SHARK_GPU_SETUP
    cfg%flags = 0
    if (force_kick) cfg%flags = ior(cfg%flags, SHARK_FLAG_FORCE_KICK)
    if (fargo)      cfg%flags = ior(cfg%flags, SHARK_FLAG_FARGO)
    if (viscosity)  cfg%flags = ior(cfg%flags, SHARK_FLAG_VISCOSITY)
    if (static)     cfg%flags = ior(cfg%flags, SHARK_FLAG_STATIC)
#if NDUST>0
    if (drag)               cfg%flags = ior(cfg%flags, SHARK_FLAG_DRAG)
    if (dust_back_reaction) cfg%flags = ior(cfg%flags, SHARK_FLAG_BACK_REACTION)
    if (growth)             cfg%flags = ior(cfg%flags, SHARK_FLAG_GROWTH)
    if (charging)           cfg%flags = ior(cfg%flags, SHARK_FLAG_CHARGING)
    cfg%dust_ratio_min = dust_ratio_min
    cfg%rhograin = rhograin
    do idust = 1, ndust
      cfg%dust_size(idust) = sdust(first_active + (first_active_y-1)*nx_max, idust)
      cfg%dust_tstop(idust) = tstop(first_active + (first_active_y-1)*nx_max, idust)
    end do
    if (growth) then            ! dust_commons.f90:6-63
      cfg%grw_smin = smin; cfg%grw_smax = smax
      cfg%grw_sticking = sticking_efficiency; cfg%grw_clustered = clustered_fraction
      cfg%grw_cfl = CFL_growth; cfg%grw_eps_thr = eps_threshold; cfg%grw_eps_thr_frag = eps_threshold_frag
      cfg%grw_dtcontrol = dtcontrol_growth; cfg%grw_delta_vambi = delta_vambi
      cfg%grw_alpha_turb = alpha_turb; cfg%grw_size_mono = size_mono; cfg%grw_slope_mono = slope_mono
      cfg%grw_Abr = Abr; cfg%grw_gamma_grains = gamma_grains; cfg%grw_estar_grains = estar_grains
      cfg%grw_kernel = kernel_type
      cfg%grw_mode = 0
      if (fragmentation)       cfg%grw_mode = ior(cfg%grw_mode, SHARK_GROWTH_FRAGMENTATION)
      if (drift_in_growth)     cfg%grw_mode = ior(cfg%grw_mode, SHARK_GROWTH_DRIFT)
      if (turb_in_growth)      cfg%grw_mode = ior(cfg%grw_mode, SHARK_GROWTH_TURB)
      if (brownian_in_growth)  cfg%grw_mode = ior(cfg%grw_mode, SHARK_GROWTH_BROWNIAN)
      if (ambipolar_in_growth) cfg%grw_mode = ior(cfg%grw_mode, SHARK_GROWTH_AMBIPOLAR)
    end if
    if (charging) then          ! ionisation_commons.f90:5-8,70-77
      cfg%chg_x = x; cfg%chg_mu_ions = mu_ions; cfg%chg_stick_el = stickeff_el
      cfg%chg_eps = epsilon_ionis; cfg%chg_nitermax = nitermax_ionis; cfg%chg_B0 = B_0_lee
      cfg%chg_mode = 0
      if (res_Marchand)        cfg%chg_mode = ior(cfg%chg_mode, SHARK_CHARGE_RESISTIVITIES)
      if (analytical_charging) cfg%chg_mode = ior(cfg%chg_mode, SHARK_CHARGE_ANALYTICAL)
    end if
#endif
    cfg%gamma = gamma; cfg%cfl = CFL
    cfg%smallr = smallr; cfg%smallc = smallc; cfg%smallp = smallp
    cfg%cs0 = cs(first_active + (first_active_y-1)*nx_max)
    ! the grid and sound speed the setup built, so both sides use the same numbers
    cfg%dx = shark_loc(dx); cfg%surf = shark_loc(surf); cfg%vol = shark_loc(vol)
    cfg%radii_c = shark_loc(radii_c); cfg%position = shark_loc(position); cfg%cs = shark_loc(cs)
#if SHARK_GPU_SETUP==1
    cfg%sod_rho_l = rho_l; cfg%sod_rho_r = rho_r; cfg%sod_P_l = P_l; cfg%sod_P_r = P_r
    cfg%sod_direction = direction_shock
#endif
#if SHARK_GPU_SETUP==2
    cfg%dust_K(1:NDUST) = K(1:NDUST)
#endif
#if SHARK_GPU_SETUP==3
    cfg%si_q_shear = q_shear; cfg%si_omega = Omega_shear; cfg%si_eta_stream = eta_stream
    cfg%si_rad0 = rad0; cfg%box_l = box_l; cfg%box_l_y = box_l_y
#endif
#if SHARK_GPU_SETUP==4
    ! disk_polar/setup_commons.f90, units.f90; setup.f90 has already put sigma_R0 in code units
    cfg%disk_mstar = Mstar; cfg%disk_hoverr = HoverR; cfg%disk_sigma0 = sigma_R0
    cfg%disk_r0 = R0_disk; cfg%disk_rout = R_out_disk
    cfg%disk_r_relax = r_relax; cfg%disk_n_rel = n_rel; cfg%disk_temp_slope = -1.0d0
    cfg%disk_alpha_visc = alpha_visc
    cfg%inner_r = rin; cfg%box_l = box_l; cfg%box_l_y = 2.0d0*pi
    cfg%unit_l = unit_l; cfg%unit_d = unit_d; cfg%unit_t = unit_t; cfg%mu_gas = mu_gas
#if NDUST>0
    cfg%rhograin = rhograin/unit_d   ! compute_tstop and the setup use rhograin/unit_d
#endif
#endif
#if SHARK_GPU_SETUP==5
    ! dustyTurb/setup_commons.f90, units.f90
    cfg%box_l = box_l; cfg%box_l_y = box_l
    cfg%turb_rho0 = rho_0; cfg%T_cloud = T_cloud; cfg%mu_gas = mu_gas
    cfg%unit_l = unit_l; cfg%unit_d = unit_d; cfg%unit_t = unit_t
#if NDUST>0
    cfg%dust_stokes(1:NDUST) = St_0(1:NDUST)
#endif
#if TURB>0
    cfg%turb_mach = Mach_x_target; cfg%turb_tcorr = turnover_time; cfg%turb_seed = iseed
    cfg%turb_kmin = nint(k_min*box_l/(2.0d0*pi)); cfg%turb_kmax = nint(k_max*box_l/(2.0d0*pi))
#endif
#endif
#if SHARK_GPU_SETUP==6
    ! KH/setup.f90 works in KH/units.f90's code units; its compute_tstop uses rhograin/unit_d
    cfg%unit_l = unit_l; cfg%unit_d = unit_d; cfg%unit_t = unit_t; cfg%mu_gas = mu_gas
    cfg%box_l = box_l; cfg%box_l_y = box_l_y
    cfg%kh_rho_dense = rho_dense; cfg%kh_rho_diffuse = rho_diffuse; cfg%kh_T_dense = T_dense
    cfg%kh_mach = Mach; cfg%kh_vy0 = vy0; cfg%kh_kx = kx
#if NDUST>0
    cfg%rhograin = rhograin/unit_d
#endif
#endif
#if SHARK_GPU_SETUP==8
    ! disk/setup_commons.f90, units.f90; setup.f90 has already put sigma_R0, R0_disk, smooth_r,
    ! Mstar and box_l in code units.  The library builds the Cartesian grid and the per-cell sound
    ! speed HoverR sqrt(Mstar/rr) itself from these (the same numbers as the setup's arrays).
    ! Every dust species starts at dust2gas, the inloop buffers' dust-to-gas ratio.
    cfg%dx = c_null_ptr; cfg%surf = c_null_ptr; cfg%vol = c_null_ptr
    cfg%radii_c = c_null_ptr; cfg%position = c_null_ptr; cfg%cs = c_null_ptr
    cfg%box_l = box_l; cfg%box_l_y = box_l_y
    cfg%disk_mstar = Mstar; cfg%disk_hoverr = HoverR; cfg%disk_sigma0 = sigma_R0; cfg%disk_r0 = R0_disk
    cfg%disk_alpha_visc = alpha_visc
    cfg%cdisk_smooth_r = smooth_r; cfg%cdisk_frac_r_disk = frac_R_disk
    cfg%cdisk_buffer_in = buffer_in; cfg%cdisk_buffer_out = buffer_out
    cfg%unit_l = unit_l; cfg%unit_d = unit_d; cfg%unit_t = unit_t; cfg%mu_gas = mu_gas
#if NDUST>0
    cfg%rhograin = rhograin/unit_d   ! compute_tstop uses rhograin/unit_d
    cfg%dust_eps(1:NDUST) = dust2gas
#endif
#endif
#if SHARK_GPU_SETUP==7
    cfg%box_l = box_l; cfg%box_l_y = box_l_y
    cfg%sedov_rho_ext = rho_ext; cfg%sedov_P_ext = P_ext; cfg%sedov_P_cen = P_cen
    cfg%sedov_r_expl = r_expl
#endif
    rc = shark_gpu_init(cfg, gpu_ctx)
    if (rc /= SHARK_OK) stop 'shark_gpu_init failed'
    rc = shark_gpu_upload(gpu_ctx, u_prim, int(ncells, c_int64_t), int(nvar, c_int32_t))
    if (rc /= SHARK_OK) stop 'shark_gpu_upload failed'
    gpu_uploaded = .true.
  end if

  rc = shark_gpu_step(gpu_ctx, dt, st)
  if (rc /= SHARK_OK) stop 'shark_gpu_step failed'
  if (st /= 0) print *, 'shark_gpu_step status word ', st
  nsolve = nsolve + 1
  ! check_output of the next iteration writes when its counter reaches freq_out
  if (mod(nsolve + 1, freq_out) == 0) then
    rc = shark_gpu_download(gpu_ctx, u_prim, c_null_ptr)
    if (rc /= SHARK_OK) stop 'shark_gpu_download failed'
    call ctoprim
#if NDUST>0
    if (charging) call download_charges
#endif
  end if
end subroutine solve

#if NDUST>0
! The charging outputs that output() writes (write_output.f90: zd, ni, ne, eta_o, eta_a, and the
! psi_old the next cold start would use), from the device's last charging call.
subroutine download_charges
  use parameters
  use commons
  use ionisation_commons
  use shark_gpu
  implicit none
  integer(c_int32_t) :: rc
  real(c_double), allocatable, target :: eta3(:,:)
  allocate(eta3(ncells,3))
  if (res_Marchand) then
    rc = shark_gpu_download_charge(gpu_ctx, c_loc(zd), c_loc(ni), c_loc(ne), c_loc(psi_old), c_loc(eta3), &
                                   c_loc(gamma_d), c_null_ptr)
  else
    rc = shark_gpu_download_charge(gpu_ctx, c_loc(zd), c_loc(ni), c_loc(ne), c_loc(psi_old), c_null_ptr, &
                                   c_null_ptr, c_null_ptr)
  end if
  if (rc /= SHARK_OK) stop 'shark_gpu_download_charge failed'
  if (res_Marchand) then
    eta_o(:) = eta3(:,1); eta_h(:) = eta3(:,2); eta_a(:) = eta3(:,3)
  end if
  deallocate(eta3)
end subroutine download_charges
#endif

subroutine ctoprim
  use parameters
  use commons
  use units
  use shark_gpu
  implicit none
  integer :: i, idust
  integer(c_int32_t) :: rc
  real(dp) :: ekin
  if (gpu_uploaded) then
    rc = shark_gpu_ctoprim(gpu_ctx, q, cs)
    if (rc /= SHARK_OK) stop 'shark_gpu_ctoprim failed'
    return
  end if
  do i = 1, ncells
    q(i,irho) = max(u_prim(i,irho), smallr)
    q(i,ivx) = u_prim(i,ivx)/u_prim(i,irho)
    q(i,ivy) = u_prim(i,ivy)/u_prim(i,irho)
    q(i,ivz) = u_prim(i,ivz)/u_prim(i,irho)
    ekin = half*(u_prim(i,ivx)**2 + u_prim(i,ivy)**2 + u_prim(i,ivz)**2)/u_prim(i,irho)
    q(i,iP) = max((gamma-1.0d0)*(u_prim(i,iP)-ekin), smallp)
    if (iso_cs < 1) cs(i) = sqrt(gamma*q(i,iP)/q(i,irho))
    if (iso_cs == 1) q(i,iP) = u_prim(i,irho)*cs(i)**2
#if NDUST>0
    do idust = 1, ndust
      q(i,irhod(idust)) = u_prim(i,irhod(idust))
      q(i,ivdx(idust)) = u_prim(i,ivdx(idust))/u_prim(i,irhod(idust))
      q(i,ivdy(idust)) = u_prim(i,ivdy(idust))/u_prim(i,irhod(idust))
      q(i,ivdz(idust)) = u_prim(i,ivdz(idust))/u_prim(i,irhod(idust))
    end do
#endif
  end do
end subroutine ctoprim

subroutine primtoc
  use parameters
  use commons
  use units
  implicit none
  integer :: i, idust
  do i = 1, ncells
    u_prim(i,irho) = q(i,irho)
    u_prim(i,ivx) = q(i,irho)*q(i,ivx)
    u_prim(i,ivy) = q(i,irho)*q(i,ivy)
    u_prim(i,ivz) = q(i,irho)*q(i,ivz)
    u_prim(i,iP) = q(i,iP)/(gamma-1.0d0) + half*q(i,irho)*(q(i,ivx)**2 + q(i,ivy)**2 + q(i,ivz)**2)
#if NDUST>0
    do idust = 1, ndust
      u_prim(i,irhod(idust)) = q(i,irhod(idust))
      u_prim(i,ivdx(idust)) = q(i,irhod(idust))*q(i,ivdx(idust))
      u_prim(i,ivdy(idust)) = q(i,irhod(idust))*q(i,ivdy(idust))
      u_prim(i,ivdz(idust)) = q(i,irhod(idust))*q(i,ivdz(idust))
    end do
#endif
  end do
end subroutine primtoc

! output_gpu : output(iout) written from the device state (shark_gpu_output) into
!              output_XXXXX/ of the working directory, the same files as write_output.f90's
!              output for MHD = NDUSTPSCAL = TURB = 0; call it where shark.f90 calls output once
!              the GPU owns the state.
subroutine output_gpu(iout)
  use commons
  use shark_gpu
  implicit none
  integer :: iout
  integer(c_int32_t) :: rc
  rc = shark_gpu_output(gpu_ctx, int(iout, c_int32_t), time, c_null_char)
  if (rc /= 0) then
    print *, 'shark_gpu_output failed: ', rc
    stop
  end if
end subroutine output_gpu
