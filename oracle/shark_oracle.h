/*
 * shark_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU (FP64, OpenMP) restatement of SHARK's per-step `solve` (src/solver/solve.f90:10-181)
 * used as the parity oracle for the GPU library and as the timed CPU baseline.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline / reference legs may load it.  The
 * product (libshark_gpu) never links, loads or calls it.
 *
 * Parity status: pinned against the reference's own golden data (Sod exact solution
 * test/test-suite/Sod-tube/solution.dat, dusty-wave profiles
 * test/test-suite/DUSTYWAVE/dustywave-K{50,100,1000}.dat); every other path (multi-species
 * drag, SI box, FARGO, growth, charging, polar disk) is pinned only by this restatement,
 * because the Fortran reference cannot be compiled here (no Fortran compiler).
 */
#ifndef SHARK_ORACLE_H
#define SHARK_ORACLE_H

#include <stdint.h>
#include "shark_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_state oracle_state;

/* Builds grid + arrays like allocate_init/gridinit. NULL on invalid config. */
oracle_state* oracle_create(const shark_gpu_config* cfg);
void          oracle_destroy(oracle_state* s);

int64_t oracle_ncells(const oracle_state* s);
int32_t oracle_nvar(const oracle_state* s);

/* Initial conditions of the setup (SOD/DUSTYWAVE/SI as in src/setups/<NAME>/setup.f90).
 * `noise_amp`/`seed` only affect SI (white noise on dust velocities; 0 disables). */
int32_t oracle_setup_ic(oracle_state* s, double noise_amp, uint64_t seed);

int32_t oracle_get_u(const oracle_state* s, double* u);      /* ncells*nvar, Fortran order */
int32_t oracle_set_u(oracle_state* s, const double* u);
int32_t oracle_get_q(oracle_state* s, double* q, double* cs); /* runs ctoprim first          */
int32_t oracle_get_grid(const oracle_state* s, double* dx, double* surf, double* vol,
                        double* position, double* radii_c);  /* ncells*ndim etc. nullable   */
int32_t oracle_get_cs(const oracle_state* s, double* cs);
int32_t oracle_set_cs(oracle_state* s, const double* cs);

/* One `solve` (src/solver/solve.f90:10-181). *dt_out = the dt that courant set. */
int32_t oracle_solve(oracle_state* s, double* dt_out);

/* time_loop without output (src/shark.f90:71-110): up to nsteps solves until time >= tend. */
int32_t oracle_run(oracle_state* s, int64_t nsteps, double tend, double* time_io, int64_t* steps_done);

/* Kahan totals per species over the active cells, same layout as shark_gpu_totals. */
int32_t oracle_totals(const oracle_state* s, double* out);

/* Individual stages, for unit tests of one kernel at a time. */
int32_t oracle_apply_boundaries(oracle_state* s);
int32_t oracle_ctoprim(oracle_state* s);
int32_t oracle_courant(oracle_state* s, double* dt_out);
int32_t oracle_set_dt(oracle_state* s, double dt);
int32_t oracle_dust_drag(oracle_state* s, double coeffdt);
int32_t oracle_compute_tstop(oracle_state* s);
int32_t oracle_get_tstop(const oracle_state* s, double* tstop); /* ncells*ndust */
int32_t oracle_fargo(oracle_state* s);   /* fargo_scheme alone with the dt last set (needs FARGO) */
/* charge (ionisation.f90:4-214) on the current state; seed (ncells, nullable) overrides the start
 * point where nonzero; iters (ncells, nullable) receives the Newton iteration counts. */
int32_t oracle_charge(oracle_state* s, const double* seed, int32_t* iters);
int32_t oracle_get_charge(const oracle_state* s, double* zd, double* ni, double* ne, double* psi,
                          double* eta, double* gamma_d);
int32_t oracle_reset_charge(oracle_state* s);   /* psi_old = 0: the next call starts cold */
int32_t oracle_charge_psi0(const oracle_state* s, double* psi0);
/* dust_growth (dust_growth.f90:3-256) alone, with the dt last set, on the current state (ctoprim
 * and compute_tstop first); substeps (ncells, nullable) receives the sub-steps per cell. */
int32_t oracle_growth(oracle_state* s, int32_t* substeps);
int32_t oracle_growth_grid(const oracle_state* s, double* zeta_eta_massmin, double* mk, double* redis);
/* dustyTurb forcing: one Ornstein-Uhlenbeck update and gas kick with the dt last set; the
 * modes (3 nm: kx', ky', |k'|) and coefficients (2 nm) */
int32_t oracle_turb_kick(oracle_state* s);
int32_t oracle_turb_coef(const oracle_state* s, double* modes, double* coef, int32_t* nm);

/* output (src/commons/write_output.f90:2-300) of the current state after ctoprim: writes
 * prefix + "output_" + five digits (iout) with info.dat and the raw stream field files. */
int32_t oracle_output(oracle_state* s, int32_t iout, double time, const char* prefix);

int32_t oracle_set_threads(int32_t nthreads);

#ifdef __cplusplus
}
#endif
#endif
