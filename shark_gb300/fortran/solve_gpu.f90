! solve_gpu.f90 -- drop-in replacement of src/solver/solve.f90 that runs each step on the GPU.
!
! Build: put this file (and shark_gpu_mod.f90) before src/solver on VPATH instead of solve.f90,
! add -DSHARK_GPU_SETUP=<1 SOD | 2 DUSTYWAVE | 3 SI | 6 KH | 7 sedov> and
! -DSHARK_GPU_PREC=<0 FP64 | 1 mixed>
! to DEFINES and link with -L<repo>/shark_gb300 -lshark_gpu.  The time loop (src/shark.f90),
! setups, namelists and output stay as they are.
!
! solve   : first call builds the configuration from the module parameters, creates the GPU
!           context and uploads u_prim; every call runs one step on the device and sets dt.
!           Before an iteration whose check_output will write (every freq_out steps) the state is
!           downloaded into u_prim and q so the unchanged output routines see it.
! ctoprim : primitive variables; from the device once the GPU owns the state, on the host before.
! primtoc : conservative from primitive variables (host; used by the setups).
subroutine solve(verbose,outputing)
  use parameters
  use commons
  use units
  use shark_gpu
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
    call ctoprim
  end if
end subroutine solve

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
