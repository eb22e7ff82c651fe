/*
 * shark_gpu.h -- C ABI of the GB300 (sm_103a) per-step Godunov update for gas + N dust species.
 *
 * The reference (SHARK, Fortran 90) runs one time step as the argument-less subroutine
 * `solve(verbose,outputing)` (src/solver/solve.f90:10-181), called once per step from
 * `time_loop` (src/shark.f90:102).  `solve` talks to the rest of the code only through module
 * arrays: the conserved state `u_prim(1:ncells,1:nvar)` (src/commons/allocate_init.f90:82),
 * its primitive copy `q`, the sound speed `cs`, the stopping times `tstop` and the forces.
 * This header replaces that whole call with a device-resident context:
 *
 *   shark_gpu_init      <- allocate_init + gridinit + the per-setup parameter reads
 *   shark_gpu_upload    <- the state produced by `setup` (or by a restart)
 *   shark_gpu_step      <- solve(verbose,outputing)            src/solver/solve.f90:10-181
 *   shark_gpu_download  <- the host copy that `output`/`check_output` read
 *   shark_gpu_ctoprim   <- ctoprim                             src/solver/solve.f90:195-253
 *   shark_gpu_totals    <- the mass/momentum sums of check_output (e.g. src/setups/SI/setup.f90:271-285)
 *
 * Every function returns an int32 status (SHARK_OK == 0).  No function throws, aborts or
 * traps; device-side failures are reported through the step status word.
 *
 * Layout contract (identical to the reference): u_prim is variable-major with stride ncells
 * (Fortran u_prim(1:ncells,1:nvar), column-major), cells are x-fastest with ghost cells,
 * icell = ix + iy*nx_max (0-based), nx_max = nx + 2*nghost, ny_max = ny + 2*nghost (1 in 1D).
 * Variable order: rho, rho*vx, rho*vy, rho*vz, E, then rho_d(1..N), rho_d*vdx(1..N),
 * rho_d*vdy(1..N), rho_d*vdz(1..N)   (src/commons/allocate_init.f90:225-262).
 * nvar = 5 + 4*N (no MHD, no dust passive scalars: src/commons/parameters.f90:43).
 */
#ifndef SHARK_GPU_H
#define SHARK_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SHARK_GPU_ABI_VERSION 2
#define SHARK_MAX_DUST 64

/* ---- return codes ------------------------------------------------------------------------ */
#define SHARK_OK                   0
#define SHARK_ERR_INVALID_ARG     -1   /* bad pointer, size or config field                   */
#define SHARK_ERR_UNSUPPORTED     -2   /* valid reference option not built on the GPU path    */
#define SHARK_ERR_CUDA            -3   /* a CUDA runtime call failed (message: shark_gpu_last_error) */
#define SHARK_ERR_NO_DEVICE       -4   /* no sm_103 device visible                            */
#define SHARK_ERR_STATE           -5   /* call order violated (e.g. step before upload)       */
#define SHARK_ERR_NUMERICS        -6   /* the step status word reports a numerical failure    */

/* ---- step status word (bit mask written by the kernels, read back with the dt) ----------- */
#define SHARK_STATUS_NAN          0x1  /* a non-finite conserved value was produced            */
#define SHARK_STATUS_NEG_DENSITY  0x2  /* gas density <= 0 after the update                    */
#define SHARK_STATUS_DT_UNDERFLOW 0x4  /* CFL dt not positive/finite                           */
#define SHARK_STATUS_NEWTON       0x8  /* a charging Newton solve hit its iteration cap        */
#define SHARK_STATUS_GROWTH       0x10 /* growth sub-cycling hit its cap                        */
#define SHARK_STATUS_COPY_WAIT    0x20 /* a kernel gave up waiting for a shared-memory copy (TMA)
                                          and left its part of the step undone                  */

/* ---- setups whose per-step hooks exist on the device (src/setups/<NAME>/) ----------------- */
#define SHARK_SETUP_SOD         1   /* fixed left/right ghost states   SOD/boundaries.f90:49-77 */
#define SHARK_SETUP_DUSTYWAVE   2   /* periodic; tstop = rho_d/K        DUSTYWAVE/setup.f90:212-221 */
#define SHARK_SETUP_SI          3   /* shearing box                     SI/setup.f90, SI/boundaries.f90 */
#define SHARK_SETUP_DISK_POLAR  4   /* polar disk (FARGO)               disk_polar/                 */
#define SHARK_SETUP_DUSTYTURB   5   /* periodic driven turbulence       dustyTurb/                  */
#define SHARK_SETUP_KH          6   /* periodic shear layer, Epstein    KH/setup.f90, KH/units.f90  */
#define SHARK_SETUP_SEDOV       7   /* periodic blast wave, gas only    sedov/setup.f90             */
#define SHARK_SETUP_DISK_CART   8   /* Cartesian disk, softened star    disk/setup.f90, disk/boundaries.f90 */

/* ---- run-time switches (the reference's namelist logicals) -------------------------------- */
#define SHARK_FLAG_DRAG           0x1   /* drag               src/dust/dust_commons.f90:5        */
#define SHARK_FLAG_BACK_REACTION  0x2   /* dust_back_reaction src/dust/dust_commons.f90:15       */
#define SHARK_FLAG_FORCE_KICK     0x4   /* force_kick         src/commons/parameters.f90:49      */
#define SHARK_FLAG_FARGO          0x8   /* fargo              src/commons/parameters.f90:51      */
#define SHARK_FLAG_GROWTH         0x10  /* growth             src/dust/dust_commons.f90:6        */
#define SHARK_FLAG_CHARGING       0x20  /* charging           src/chemistry/ionisation_commons.f90 */
#define SHARK_FLAG_VISCOSITY      0x40  /* viscosity          src/commons/parameters.f90:50      */
#define SHARK_FLAG_STATIC         0x80  /* static             src/commons/parameters.f90:48      */

/* ---- precision of the device state and of the flux/update stage -------------------------- */
#define SHARK_CHARGE_HIST 64   /* bins of the Newton iteration histogram (last bin: >= 63) */
/* charging network: features per cell, trainable parameters, whole parameter blob */
#define SHARK_MLP_NFEAT  6
#define SHARK_MLP_NPARAM 5313  /* W1[64][16] b1[64] W2[64][64] b2[64] w3[64] b3[1]            */
#define SHARK_MLP_NBLOB  5327  /* + feature mean[6], sd[6], target mean, sd                   */

/* chg_mode bits */
#define SHARK_CHARGE_RESISTIVITIES 1   /* also eta_o, eta_H, eta_a, gamma_d (res_Marchand)       */
#define SHARK_CHARGE_ANALYTICAL    2   /* Fujii et al. per-species Newton (analytical_charge)    */
#define SHARK_CHARGE_MLP_SEED      4   /* start the Marchand Newton from the trained network     */

/* grw_mode bits (dust_commons.f90:9-13) */
#define SHARK_GROWTH_FRAGMENTATION 1
#define SHARK_GROWTH_DRIFT         2
#define SHARK_GROWTH_TURB          4
#define SHARK_GROWTH_BROWNIAN      8
#define SHARK_GROWTH_AMBIPOLAR     16

#define SHARK_PREC_FP64   0   /* everything FP64 (the FP64 GPU oracle run)                      */
#define SHARK_PREC_MIXED  1   /* FP32 state + FP32 flux/update; FP64 drag, FARGO split, totals  */

/*
 * Run configuration.  Plain old data: the Fortran shim fills it from the module parameters
 * (src/commons/parameters.f90, src/hydro/hydro_commons.f90, src/dust/dust_commons.f90) and
 * the setup_parameters module of the chosen setup.  Compile-time -D flags of the reference
 * (bin/Makefile:36) are run-time fields here.
 */
typedef struct shark_gpu_config {
    int32_t abi_version;      /* must be SHARK_GPU_ABI_VERSION                                  */
    int32_t nx, ny;           /* active cells (-DNX, -DNY); ny == 1 selects the 1D code path     */
    int32_t nghost;           /* must be 2 (-DNGHOST, bin/Makefile:8)                           */
    int32_t ndust;            /* -DNDUST, 0..SHARK_MAX_DUST                                      */
    int32_t geom;             /* -DGEOM: 0 Cartesian, 2 polar face-on                            */
    int32_t gridspace;        /* -DGRIDSPACE: 0 linear, 1 log-spaced radius (geom 2)             */
    int32_t solver;           /* -DSOLVER: 0 LLF, 1 HLL, 2 HLLC                                  */
    int32_t solverdust;       /* -DSOLVERDUST: 0 Huang & Bai, 1 LLF, 2 HLL, 3 HLLC (isothermal gas) */
    int32_t slope_type;       /* 1 minmod, 2 van Leer (harmonic), 3 MC(1.5)                      */
    int32_t iso_cs;           /* 1: isothermal (P = rho cs^2 with cs fixed by the setup)         */
    int32_t precision;        /* SHARK_PREC_*                                                    */
    int32_t setup;            /* SHARK_SETUP_*                                                   */
    int32_t flags;            /* SHARK_FLAG_*                                                    */
    int32_t device;           /* CUDA device ordinal                                             */
    int32_t pad0;

    double gamma, cfl;                 /* hydro_commons.f90:16, parameters.f90:55              */
    double smallr, smallc, smallp;     /* floors after allocate_init.f90:277-279 scaling       */
    double box_l, box_l_y;             /* domain extents handed to gridinit                    */
    double inner_r;                    /* inner radius for geom 2 (gridinit_disk_log inner_r)  */
    double cs0;                        /* isothermal sound speed scale (setup-defined profile) */
    double dust_ratio_min;             /* dust_commons.f90:29                                   */
    double rhograin;                   /* grain intrinsic density (code units)                  */

    /* per-species constants */
    double dust_size[SHARK_MAX_DUST];  /* sdust: grain radius (code units)                      */
    double dust_K[SHARK_MAX_DUST];     /* DUSTYWAVE drag constant K(idust)                      */
    double dust_tstop[SHARK_MAX_DUST]; /* SI: constant stopping time per species                */
    double dust_eps[SHARK_MAX_DUST];   /* initial dust-to-gas ratio per species (ICs only)      */
    double dust_stokes[SHARK_MAX_DUST];/* SI Stokes number per species (ICs only)               */

    /* SOD (src/setups/SOD/setup_commons.f90) */
    double sod_rho_l, sod_rho_r, sod_P_l, sod_P_r;
    int32_t sod_direction;             /* 0: shock along x, 1: along y                          */
    int32_t pad1;
    /* DUSTYWAVE (src/setups/DUSTYWAVE/setup_commons.f90; ICs only) */
    double dw_rho_0, dw_delta_rho, dw_vx_0, dw_kx_wave;
    /* SI shearing box (src/setups/SI/setup_commons.f90) */
    double si_q_shear, si_omega, si_eta_stream, si_rad0, si_rho_init, si_hoverr;
    /* polar disk (src/setups/disk_polar/setup_commons.f90); code units AU, Msun, 1/Omega(1 AU).
     * Sound speed cs(r) = h(r) sqrt(Mstar/r) with h(r) = disk_hoverr * r^((disk_temp_slope+1)/2),
     * i.e. T ~ r^disk_temp_slope (the reference's constant H/R is disk_temp_slope = -1).
     * Point-mass gravity -disk_mstar/r^2; stopping times Epstein on Sigma/(sqrt(2 pi) H);
     * setup_inloop relaxes the cells with r < disk_r_relax towards the initial state over
     * disk_n_rel orbits and resets the first active column; with SHARK_FLAG_FARGO the rings are
     * remapped by the orbital velocity -sqrt(disk_mstar/r) every step.  ICs: Sigma =
     * disk_sigma0 (disk_r0/r) exp(-r/disk_rout). */
    double disk_mstar, disk_hoverr, disk_sigma0, disk_r0, disk_rout;
    double disk_r_relax, disk_n_rel, disk_temp_slope;
    /* Code units in cgs (0 = 1): length, density, time.  unit_m = unit_l^3 unit_d,
     * unit_v = unit_l/unit_t, unit_nH = unit_d/(mu_gas mH) (dustyTurb/units.f90). */
    double unit_l, unit_d, unit_t;
    double mu_gas;                     /* mean molecular weight (setup_commons.f90: 2.31)        */
    double T_cloud;                    /* dustyTurb gas temperature (K) for charging and growth  */
    /* Charging (src/chemistry/ionisation_commons.f90): cosmic-ray ionisation rate x (s^-1),
     * for the polar disk attenuated by exp(-Sigma/chg_sigma_att) (g cm^-2, 0 = none); ion mass
     * (mH), electron sticking coefficient, Newton tolerance and iteration cap, B field
     * normalisation of the resistivities (G at nH = 1e4 cm^-3). */
    double chg_x, chg_sigma_att, chg_mu_ions, chg_stick_el, chg_eps, chg_B0;
    int32_t chg_nitermax;
    int32_t chg_mode;                  /* SHARK_CHARGE_* bits                                    */
    /* dustyTurb (src/setups/dustyTurb/setup_commons.f90): mean density rho_0; stopping times
     * t_k = dust_stokes[k] box_l rho_0 / cs / rho (setup.f90:456).  Ornstein-Uhlenbeck
     * solenoidal forcing: target RMS Mach number, correlation time, wavenumber band (in 2 pi/box_l)
     * and seed (turb_mach = 0: no forcing). */
    double turb_rho0, turb_mach, turb_tcorr;
    int32_t turb_kmin, turb_kmax;
    int32_t turb_seed, pad2;
    /* Dust growth (src/dust/dust_commons.f90): size grid smin..smax (cm, the bins' edges
     * smin zeta^(k-1), smin zeta^k with zeta = (smax/smin)^(1/N)), sticking efficiency,
     * clustered fraction, sub-cycle CFL, coagulation / fragmentation dust-to-gas thresholds, fixed
     * sub-step (years, <= 0: none), ambipolar drift factor, turbulence alpha, monomer size (cm)
     * and fragment slope, Blum & Wurm A, grain surface energy (erg cm^-2) and Young modulus. */
    double grw_smin, grw_smax, grw_sticking, grw_clustered, grw_cfl, grw_eps_thr, grw_eps_thr_frag;
    double grw_dtcontrol, grw_delta_vambi, grw_alpha_turb, grw_size_mono, grw_slope_mono, grw_Abr;
    double grw_gamma_grains, grw_estar_grains;
    int32_t grw_kernel;                /* 0 physical, 1 constant, 2 additive (kernel_type)     */
    int32_t grw_mode;                  /* SHARK_GROWTH_* bits                                   */
    /* viscosity (SHARK_FLAG_VISCOSITY, source_terms.f90:99-118): the polar disk's
     * eta_visc = disk_alpha_visc H cs (disk_polar/setup.f90:67) */
    double disk_alpha_visc;
    /* KH (KH/setup_commons.f90): dense and band densities (g cm^-3), temperature (K), Mach number
     * of the shear, amplitude vy0 and wavenumber kx of the vy seed; code units from unit_l/d/t */
    double kh_rho_dense, kh_rho_diffuse, kh_T_dense, kh_mach, kh_vy0, kh_kx;
    /* sedov (sedov/setup_commons.f90): ambient density and pressure, blast overpressure, radius */
    double sedov_rho_ext, sedov_P_ext, sedov_P_cen, sedov_r_expl;
    /* Cartesian disk (src/setups/disk/setup_commons.f90), in the disk units (AU, Msun, G = 1):
     * the star (disk_mstar) at the box centre with softening length cdisk_smooth_r, H/R =
     * disk_hoverr, Sigma = disk_sigma0 disk_r0 / r inside frac_R_disk box_l (1/100 of its edge
     * value outside), viscosity eta = disk_alpha_visc H cs; setup_inloop resets the cells with
     * r < buffer_in box_l or r > buffer_out box_l (r softened) every step.  No planet. */
    double cdisk_smooth_r, cdisk_frac_r_disk, cdisk_buffer_in, cdisk_buffer_out;

    /* Optional grid metrics from the caller (Fortran dx(ncells,ndim), surf(ncells,ndim),
     * vol(ncells), radii_c(ncells), position(ncells,ndim), cs(ncells)).  NULL: the library
     * builds them with the formulas of src/grid/grid.f90:104-173 (gridinit) and
     * gridinit_disk_log.  When given they must depend on ix only (true for every reference
     * grid); the library checks this and returns SHARK_ERR_UNSUPPORTED otherwise. */
    const double* dx;
    const double* surf;
    const double* vol;
    const double* radii_c;
    const double* position;
    const double* cs;
} shark_gpu_config;

typedef struct shark_gpu_ctx shark_gpu_ctx;

/* Library/ABI identification; never fails. */
int32_t shark_gpu_abi_version(void);

/* Fill *cfg with the reference defaults (hydro_commons.f90, dust_commons.f90, parameters.f90):
 * gamma 1.66667, CFL 0.5, smallr=smallc=1e-27, smallp=smallr*smallc^2, slope_type 1, HLLC,
 * Huang & Bai, nghost 2, drag + back reaction on, FP64. */
int32_t shark_gpu_config_defaults(shark_gpu_config* cfg);

/* Validate cfg, select the device, build the grid and allocate the device state.
 * Replaces allocate_init/gridinit (src/commons/allocate_init.f90:3-282, src/grid/grid.f90). */
int32_t shark_gpu_init(const shark_gpu_config* cfg, shark_gpu_ctx** ctx_out);

/* Copy the conserved state (ncells*nvar doubles, Fortran order) to the device.
 * ncells and nvar must match the context.  Also computes the first CFL dt.
 * SHARK_SETUP_DISK_POLAR: the first state uploaded to a context is also kept as the initial
 * state that setup_inloop relaxes towards (uprim_condinit, src/setups/disk_polar/setup.f90:79-83);
 * later uploads (a restart) replace the state only. */
int32_t shark_gpu_upload(shark_gpu_ctx* ctx, const double* u_prim, int64_t ncells, int32_t nvar);

/* One full `solve` on the device (src/solver/solve.f90:10-181): boundaries, ctoprim, forces,
 * stopping times, CFL dt, kick, MUSCL-Hancock predictor + Riemann fluxes + update, source
 * terms, FARGO, drag, setup_inloop.  *dt_out receives the dt used by this step (the value
 * `courant` sets, src/solver/courant.f90:11-124); *status_out the status word of the step
 * before this one (the kernels run asynchronously; the final word is returned by
 * shark_gpu_sync).  Either pointer may be NULL. */
int32_t shark_gpu_step(shark_gpu_ctx* ctx, double* dt_out, int32_t* status_out);

/* Run up to nsteps steps, stopping once time >= tend (src/shark.f90:71-110; dt is not clipped
 * to tend, exactly like the reference).  *time_io is advanced by the dts; *steps_done and
 * *status_out receive the count and the OR of all status words.  Pointers may be NULL except
 * time_io. */
int32_t shark_gpu_run(shark_gpu_ctx* ctx, int64_t nsteps, double tend, double* time_io,
                      int64_t* steps_done, int32_t* status_out);

/* Wait for all queued work; *status_out = OR of the status words so far (may be NULL). */
int32_t shark_gpu_sync(shark_gpu_ctx* ctx, int32_t* status_out);

/* Copy the conserved state back (ncells*nvar doubles, Fortran order), ghost cells included as
 * the last step left them.  q (nullable) receives the primitive variables of ctoprim. */
int32_t shark_gpu_download(shark_gpu_ctx* ctx, double* u_prim, double* q);

/* ctoprim on the device state (src/solver/solve.f90:195-253) into host q (ncells*nvar) and
 * cs (ncells, nullable). */
int32_t shark_gpu_ctoprim(shark_gpu_ctx* ctx, double* q, double* cs);

/* output(iout) -- replaces src/commons/write_output.f90:2-300 (called from shark.f90:114 and by
 * solve when outputing): writes the directory  prefix + "output_" + five digits of iout  with
 * info.dat (the reference's labels, I11 / E23.15) and one raw FP64 stream file per field, the
 * active cells in cell order, unit-scaled as the reference scales them: x, rho, v, y (2D), vy,
 * vz, P; with dust rhod_tot, rhod, sd, vd, vdy, vdz (species-major); with charging eta_a,
 * eta_o, eta_h, ni, ne, zd.  The primitives come from ctoprim of the current device state
 * (the final dump's `call ctoprim; call output(iout)`), packed on the device; `time` is the
 * run time to record.  prefix may be "" (current directory) or end in '/'.  Not written: the
 * MHD, NDUSTPSCAL and 1D-turbulence rms files (MHD = NDUSTPSCAL = TURB = 0 here). */
int32_t shark_gpu_output(shark_gpu_ctx* ctx, int32_t iout, double time, const char* prefix);

/* Restart from an output directory written by shark_gpu_output (or by the reference's output
 * for the same configuration) -- the reference's read_output (src/commons/read_output.f90) is an
 * empty stub, so this has no reference counterpart to replace.  Checks info.dat against the
 * context (nvar, ndust, NX, NY, GEOM), divides out the units, rebuilds the conserved state with
 * primtoc's operations (solve.f90:265-302) and uploads it (ghost cells from the boundaries, as
 * shark_gpu_upload does).  *time_out (nullable) receives the recorded time.  The energy of an
 * isothermal run is rebuilt from P = rho cs^2; it does not enter the isothermal update. */
int32_t shark_gpu_read_output(shark_gpu_ctx* ctx, const char* dir, double* time_out);

/* Compensated (Kahan) FP64 totals over the active cells, for each species s = 0..N (gas
 * first): out[4*s+0] = sum rho, out[4*s+1..3] = sum of the three momenta.  out has 4*(N+1)
 * doubles.  Deterministic: fixed reduction tree. */
int32_t shark_gpu_totals(shark_gpu_ctx* ctx, double* out);

/* Device time of the last `step` in milliseconds: ms_out[0] work before the flux kernel (the dt
 * slot reset), ms_out[1] flux/update kernels (K1), ms_out[2] drag + dt + ghost-fill kernel (K2)
 * (CUDA events on the context's stream; waits for the step). */
int32_t shark_gpu_last_step_ms(shark_gpu_ctx* ctx, float* ms_out);

/* Benchmark helper: synchronize, record a CUDA event on the context's stream, queue nsteps steps
 * back to back (the same kernels as shark_gpu_step, with each step's dt copied to pinned host
 * memory instead of waited on), record a second event, synchronize.  *ms_out = device time
 * between the events; *time_io is advanced by the dts.  No host wait sits inside the timed
 * region, so a stalled host thread cannot show up as GPU time. */
int32_t shark_gpu_timed_run(shark_gpu_ctx* ctx, int64_t nsteps, double* time_io, float* ms_out);

/* Benchmark helper: run nsteps steps with CUDA events around every kernel on the context's
 * stream and return the mean device time per launch in milliseconds: avg_ms[0] work before the
 * flux kernel, avg_ms[1] flux/update (K1), avg_ms[2] drag + dt + ghost fill (K2), avg_ms[3] whole
 * step. */
int32_t shark_gpu_kernel_times(shark_gpu_ctx* ctx, int64_t nsteps, float* avg_ms);

/* Totals without allocating: the same Kahan-compensated FP64 sums as shark_gpu_totals (layout
 * out[4*s + 0..3] = mass, three momenta of species s, gas first) of a conserved state that the
 * caller holds on the current device in the Fortran layout (u_dev: ncells*nvar doubles,
 * nvar = 5 + 4*ndust), written to the caller's device array out_dev (4*(ndust+1) doubles).
 * No counterpart in the reference: it exists for callers that cannot call cudaMalloc (a host
 * application whose own allocator owns every device allocation, or a time loop that cannot take
 * cudaMalloc's implicit synchronisation or a change of its device footprint), which rules out
 * shark_gpu_totals because its context allocates.  It needs no context and allocates nothing:
 * its partial sums live in a fixed device array of about 1 MiB compiled into the library.  The
 * array becomes resident when the library's CUDA module is loaded on the device: under CUDA's
 * default lazy module loading that happens in the first call on each device, which therefore
 * allocates the module's memory and may synchronise -- make one warm-up call at start-up, before
 * any stream capture (or run with CUDA_MODULE_LOADING=EAGER); afterwards the device holds it until
 * the process exits.  Limit: ndust <= 64 (SHARK_ERR_INVALID_ARG beyond).  The kernels are queued on
 * `stream` (a cudaStream_t, NULL = default stream) and the call returns without waiting.  Each call
 * whose stream is not capturing looks the array's device address up with the device current (so a
 * cudaDeviceReset between calls leaves no stale address); a call on a capturing stream reuses the
 * address of the previous call on that device and fails if there was none.  All calls share the
 * array: calls that overlap on the GPU race and give wrong results; order them on one stream. */
int32_t shark_gpu_totals_noalloc(const double* u_dev, int32_t nx, int32_t ny, int32_t nghost, int32_t ndust,
                                 double* out_dev, void* stream);

/* Human-readable message of the last error on this thread (static storage). */
const char* shark_gpu_last_error(void);

/* Release the device state and the context. */
/* ---- charging (SHARK_FLAG_CHARGING; src/chemistry/ionisation.f90:4-214) --------------------
 * Each step charges every cell (ghosts included) from the state at the start of the step, after
 * the stopping times (solve.f90:36-42), starting the Newton from the cell's previous psi
 * (psi_old) or, on a cold start, from the reference's psi0 or the trained network
 * (SHARK_CHARGE_MLP_SEED).  The charges do not feed back into the hydro state. */

/* Charge the current state now (outside a step); synchronous. */
int32_t shark_gpu_charge(shark_gpu_ctx* ctx);
/* psi_old = 0 everywhere: the next charging call starts cold (ionisation.f90:71-73). */
int32_t shark_gpu_charge_reset(shark_gpu_ctx* ctx);
/* Newton iteration histogram of the last charging call (SHARK_CHARGE_HIST bins, the last one
 * counting >= 63 iterations), the number of cells that hit chg_nitermax without reaching
 * chg_eps, and the total iteration count.  Any pointer may be NULL. */
int32_t shark_gpu_charge_stats(shark_gpu_ctx* ctx, int64_t* iters_hist, int64_t* nonconv, int64_t* total_iters);
/* Last charging outputs in Fortran order: zd(ncells,N), ni(ncells), ne(ncells), psi_old(ncells),
 * eta(ncells,3) = (eta_o, eta_H, eta_a), gamma_d(ncells,N) (the last two with
 * SHARK_CHARGE_RESISTIVITIES), Newton iterations per cell.  Any pointer may be NULL. */
int32_t shark_gpu_download_charge(shark_gpu_ctx* ctx, double* zd, double* ni, double* ne, double* psi,
                                  double* eta, double* gamma_d, int32_t* iters);

/* ---- charging network (SHARK_CHARGE_MLP_SEED) ----------------------------------------------
 * A 6 -> 64 -> 64 -> 1 tanh MLP (BF16 tensor-core GEMMs, FP32 accumulate) maps a cell's
 * log10 nH, log10 T, log10 zeta and grain moments log10(sum n_k pi a_k^2/nH), log10(sum n_k a_k/nH),
 * log10(sum n_k/nH) to t = psi/psi0 - 1, the start point of the charging Newton on a cold start.
 * Parameter blob (SHARK_MLP_NBLOB floats): W1[64][16] b1[64] W2[64][64] b2[64] w3[64] b3, then
 * the feature means[6], standard deviations[6], target mean, standard deviation. */

/* Charge the current state cold (psi_old = 0, the reference's start point) and append the
 * (features, t) pairs of every converged cell to the training set, allocated on the first call
 * with room for `capacity` pairs.  *count receives the fill level. */
int32_t shark_gpu_mlp_collect(shark_gpu_ctx* ctx, int64_t capacity, int64_t* count);
/* Adam on the mean squared error of the normalised target, `steps` mini-batches of `batch`
 * pairs drawn without replacement (shuffled with `seed`), on the GPU.  The normalisation comes
 * from the training set on the first training of a context without loaded weights.
 * loss_curve (steps floats, nullable) receives the mini-batch losses. */
int32_t shark_gpu_mlp_train(shark_gpu_ctx* ctx, int32_t steps, int32_t batch, float lr, uint64_t seed,
                            float* loss_curve);
int32_t shark_gpu_mlp_save(shark_gpu_ctx* ctx, float* blob, int64_t n);
int32_t shark_gpu_mlp_load(shark_gpu_ctx* ctx, const float* blob, int64_t n);
/* Network on host-given raw features (n x SHARK_MLP_NFEAT): out (n, nullable) receives t; with
 * target (n) and grad (SHARK_MLP_NPARAM) also the gradient of sum((y - y*)^2)/n over the
 * normalised outputs, without updating the weights (and *loss the sum of squares). */
int32_t shark_gpu_mlp_eval(shark_gpu_ctx* ctx, const float* feat, const float* target, int64_t n, float* out,
                           float* grad, float* loss);
/* Network features of every cell of the current state, (ncells x SHARK_MLP_NFEAT), cells in
 * Fortran order. */
int32_t shark_gpu_mlp_features(shark_gpu_ctx* ctx, float* feat);

int32_t shark_gpu_free(shark_gpu_ctx* ctx);

#ifdef __cplusplus
}
#endif

#endif /* SHARK_GPU_H */
