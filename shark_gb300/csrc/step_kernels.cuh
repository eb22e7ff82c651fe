// step_kernels.cuh -- the device kernels of one `solve` step (src/solver/solve.f90:10-181).
//
//   k_boundaries   apply_boundaries of the setup (ghost fill), before anything reads the halo
//   k_flux         K1: per (tile, species): ctoprim on the halo tile, limited slopes, MUSCL-Hancock
//                  predictor, Riemann fluxes (HLLC/HLL/LLF gas, Huang-Bai/LLF/HLL dust), force
//                  kick, conservative update and the local source terms, in one pass through
//                  shared memory.  No qm/qp/flux array ever reaches HBM.
//   k_finalize     K2: per cell, all species: implicit multi-species drag (FP64 arithmetic),
//                  dust floor, setup_inloop, status checks, and the CFL dt of the NEXT step
//                  (courant on the final state: warp shuffle -> block -> one atomicMin).
//
// Device state layout: variable-major planes, each plane ny_max rows of `pitch` elements
// (pitch >= nx_max, rounded up to 32 elements so every row starts 128-byte aligned), ghost cells
// stored.  Element (v, iy, ix) lives at v*plane + iy*pitch + ix.
#pragma once

#include "physics.cuh"
#include "growth.cuh"
#include "../../include/shark_gpu.h"

namespace shark {

template <typename R>
struct KParams {
    // grid
    int nx, ny, ng, nx_max, ny_max, pitch;
    long long plane;
    int ndust, nvar, ndim, geom, solver, solverdust, slope_type, iso, setup, flags;
    int sod_dir;
    double gamma, cfl, smallr, smallp, dust_ratio_min, box_l, rhograin;
    double si_q, si_om, si_eta, si_r0;
    double sod_rho_l, sod_rho_r, sod_P_l, sod_P_r;
    // per-column metrics (length nx_max), compute precision
    const R *dx1, *dx2, *surf1, *surf2, *vol, *radc, *xpos, *cs;
    const R *sfx, *sfy, *irp, *rvol;   // division-free tables (mixed path)
    const R* fgrav;                    // polar disk: -Mstar/r^2 (0 for the other setups)
    const R* etav;                     // polar disk: kinematic viscosity alpha H cs
    int visc;                          // viscosity source term on
    // per-column metrics in FP64 (courant, drag)
    const double *dx1d, *dx2d, *radcd, *xposd, *csd;
    // polar disk per-column FP64 tables: gravity, relaxation time (0 = no relaxation),
    // sqrt(2 pi) H, FARGO orbital velocity
    const double *fgravd, *treld, *hsd, *vkd;
    const R* u_init;                   // polar disk relaxation reference state
    GrowthDev gw;                      // dust growth tables and constants
    int ou_nm;                         // dustyTurb forcing modes (0: no forcing)
    const double* ou;                  // [2 nm] this step's coefficients
    const double* ou_modes;            // [3 nm]
    double box_l_y;
    const R* chg_eta;                  // charging outputs: eta (3 planes), gamma_d (N planes)
    const R* chg_gamma_d;
    // per-species constants
    const double *dK, *dtstop, *dsize, *dstokes;
    const double* dinvts;             // 1/C_k, t_k = C_k / F_cell (dustyTurb, Epstein, polar disk)
    double turb_rho0;
    // time step bookkeeping
    const double* dt;                 // dt of the current step
    unsigned long long* dt_next;      // bit image of the next dt (positive doubles order as u64)
    unsigned int* status;             // SHARK_STATUS_* bits
    float* coef;                      // [2*SHARK_MAX_DUST] per-step drag coefficients 1/(1+a_k), a_k/(1+a_k)
    const float* dtf;                 // (float) dt of the current step, coef[2*SHARK_MAX_DUST]
    const float* dinvts_f;            // 1/C_k as float (mixed path)
    // FP32 copies of the scalar parameters for the mixed kernels, converted once on the host: a
    // double-to-float conversion issues on the FP64 pipe, which is narrow and variable-latency on
    // this GPU, so per-thread conversions stall the warps that do them
    float f_gamma, f_gm1, f_inv_g1, f_cfl, f_smallr, f_smallp, f_dust_ratio_min, f_box_l, f_half_box_l;
    float f_si_q, f_si_om, f_si_r0, f_si_eta;
    float f_rho_ref;                  // reference gas density of the mixed flux kernel (0: none)
    // Cartesian disk per-cell tables (null for the other setups), plane layout: sound speed,
    // force x, force y and viscosity in the kernel's precision; FP64 sound speed and sqrt(2 pi H);
    // the setup_inloop targets (7 FP64 planes, rho_ana = 0 outside the buffers); the ghost state
    // (2 nvar: the value every ghost takes, then the top ghosts' source of the first fill)
    const R *ccs, *cfx, *cfy, *ceta;
    const double *ccsd, *chsd, *ctgt;
    R* cgs;
    const R* u_cur;                   // state at the start of the step (read only)
    R* u_next;                        // state after the step
};

// A scalar parameter in the kernel's precision: the double itself, or its float copy.
template <typename R>
__device__ __forceinline__ R prm(double d, float f) {
    if constexpr (std::is_same<R, float>::value) return f;
    else return d;
}

// dt of the current step in the kernel's precision (the float copy k_prepare_step wrote).
template <typename R>
__device__ __forceinline__ R step_dt(const KParams<R>& p) {
    if constexpr (std::is_same<R, float>::value) return *p.dtf;
    else return *p.dt;
}

template <typename R>
__device__ __forceinline__ long long uidx(const KParams<R>& p, int v, int iy, int ix) {
    return (long long)v * p.plane + (long long)iy * p.pitch + ix;
}

// Global variable index of component c (0 rho, 1 vx, 2 vy, 3 vz) of species s (0 gas, k+1 dust k)
__device__ __forceinline__ int svar(int s, int c, int N) {
    return s == 0 ? c : 5 + c * N + (s - 1);
}

// ---------------------------------------------------------------------------------------------
// Boundaries: one thread per ghost cell.  Periodic and shear-periodic fills are done in a single
// pass with the source at (wrap(ix), wrap(iy)); this equals the reference's two passes (y rows for
// the active columns, then x columns over all rows, src/grid/boundary_types.f90:149-186 and
// src/setups/SI/boundaries.f90:1-81) because the x pass copies values that the y pass produced.
// ---------------------------------------------------------------------------------------------
template <typename R>
__global__ void k_boundaries(KParams<R> p, R* u) {
    const int ng = p.ng, nx = p.nx, ny = p.ny;
    const long long nghost_rows = (p.ndim == 2) ? 2LL * ng * p.nx_max : 0;  // y-ghost rows, full width
    const long long nghost_cols = 2LL * ng * (p.ndim == 2 ? ny : 1);          // x-ghost columns, active rows
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= nghost_rows + nghost_cols) return;
    int ix, iy;
    if (t < nghost_rows) {
        int r = (int)(t / p.nx_max);
        ix = (int)(t % p.nx_max);
        iy = r < ng ? r : ny + r;          // rows 0..ng-1 and ny+ng..ny+2ng-1
    } else {
        long long c = t - nghost_rows;
        int col = (int)(c % (2 * ng));
        iy = (p.ndim == 2) ? (int)(c / (2 * ng)) + ng : 0;
        ix = col < ng ? col : nx + col;
    }
    const bool xg = (ix < ng) || (ix >= ng + nx);
    const bool yg = (p.ndim == 2) && ((iy < ng) || (iy >= ng + ny));
    const int sx = ix < ng ? ix + nx : (ix >= ng + nx ? ix - nx : ix);
    const int sy = (p.ndim == 2) ? (iy < ng ? iy + ny : (iy >= ng + ny ? iy - ny : iy)) : 0;
    const int N = p.ndust;
    if (p.setup == SHARK_SETUP_SOD) {
        // fixed states along the shock direction (SOD/boundaries.f90:49-77), periodic otherwise
        const bool fixed = (p.sod_dir == 0) ? xg : yg;
        if (fixed) {
            const bool left = (p.sod_dir == 0) ? (ix < ng) : (iy < ng);
            const double g1 = p.gamma - 1.0;
            u[uidx(p, 0, iy, ix)] = R(left ? p.sod_rho_l : p.sod_rho_r);
            u[uidx(p, 1, iy, ix)] = R(0);
            u[uidx(p, 2, iy, ix)] = R(0);
            u[uidx(p, 3, iy, ix)] = R(0);
            u[uidx(p, 4, iy, ix)] = R((left ? p.sod_P_l : p.sod_P_r) / g1);
            return;
        }
    }
    if (p.setup == SHARK_SETUP_DISK_POLAR) {
        // disk_polar/boundaries.f90:1-70: periodic in phi; a radial ghost takes the first (last)
        // active cell of its row, phi image included, with the radial velocities clipped so that
        // nothing flows in (the reference's row-less u_prim(first_active) read as the row's cell)
        const int rx = ix < ng ? ng : (ix >= ng + nx ? ng + nx - 1 : ix);
        for (int v = 0; v < p.nvar; ++v) u[uidx(p, v, iy, ix)] = u[uidx(p, v, sy, rx)];
        if (xg) {
            for (int k = -1; k < N; ++k) {
                const long long i = uidx(p, k < 0 ? 1 : 5 + N + k, iy, ix);
                const R val = u[i];
                u[i] = ix < ng ? (val > R(0) ? val : R(0)) : (val < R(0) ? val : R(0));
            }
        }
        return;
    }
    for (int v = 0; v < p.nvar; ++v) u[uidx(p, v, iy, ix)] = u[uidx(p, v, sy, sx)];
    if (p.setup == SHARK_SETUP_SI && xg) {
        // shear: vz momentum -/+ rho * q * Omega * L (SI/boundaries.f90:60-74)
        const R sgn = ix < ng ? R(-1) : R(1);
        const R qsh = R(p.si_q), om = R(p.si_om), L = R(p.box_l);
        u[uidx(p, 3, iy, ix)] = u[uidx(p, 3, sy, sx)] + sgn * (u[uidx(p, 0, sy, sx)] * qsh * om * L);
        for (int k = 0; k < N; ++k)
            u[uidx(p, 5 + 3 * N + k, iy, ix)] =
                u[uidx(p, 5 + 3 * N + k, sy, sx)] + sgn * (u[uidx(p, 5 + k, sy, sx)] * qsh * om * L);
    }
    (void)yg;
}

}  // namespace shark

#include "flux_tile.cuh"
#include "flux_strip.cuh"
#include "flux_strip2.cuh"

namespace shark {

// ---------------------------------------------------------------------------------------------
// K2: drag + floor + inloop + status + next-step CFL dt, one thread per active cell.
// NS > 0: compile-time species count (register arrays); NS < 0: run-time count.
// MODE 0: full finalize; MODE 1: dt only (first step after an upload).
// ---------------------------------------------------------------------------------------------

// Producer-side boundary fill: an active cell within nghost of a periodic or shear-periodic edge
// writes its own ghost images (with the SI shear of the vz momenta for x images) from its final
// values.  This is apply_boundaries of the next step (SI/boundaries.f90, boundary_types.f90:149-186,
// SOD/boundaries.f90 periodic directions) done by the producer; fixed SOD ghosts never change after
// the upload and are skipped.  Reads back this thread's own just-written values.
template <typename R>
__device__ __forceinline__ void fill_ghost_images(const KParams<R>& p, R* u, int gx, int gy) {
    const int ng = p.ng, nx = p.nx, ny = p.ny;
    if (p.setup == SHARK_SETUP_DISK_CART) {
        // zero_gradients as written (boundary_types.f90:48-100) from the second call on: every
        // ghost takes the state of cell (first_active, 1), which no step changes (k_cdisk_ghosts
        // does the first call).  The active cells on the edge write the ghosts next to them.
        const bool l = gx == ng, r = gx == ng + nx - 1, b = gy == ng, t = gy == ng + ny - 1;
        if (!(l || r || b || t)) return;
        for (int v = 0; v < p.nvar; ++v) {
            const R val = p.cgs[v];
            for (int g = 0; g < ng; ++g) {
                if (b) u[uidx(p, v, g, gx)] = val;
                if (t) u[uidx(p, v, ng + ny + g, gx)] = val;
                if (l) u[uidx(p, v, gy, g)] = val;
                if (r) u[uidx(p, v, gy, ng + nx + g)] = val;
                for (int h = 0; h < ng; ++h) {   // corners, by the corner cells
                    if (l && b) u[uidx(p, v, g, h)] = val;
                    if (r && b) u[uidx(p, v, g, ng + nx + h)] = val;
                    if (l && t) u[uidx(p, v, ng + ny + g, h)] = val;
                    if (r && t) u[uidx(p, v, ng + ny + g, ng + nx + h)] = val;
                }
            }
        }
        return;
    }
    if (p.setup == SHARK_SETUP_DISK_POLAR) {
        // disk_polar/boundaries.f90:1-70 by the producer: phi images of the rows next to the
        // periodic seam; the first/last active column also writes its radial ghosts (and their
        // phi images) with the radial velocities clipped to outflow
        const int ty = gy < 2 * ng ? gy + ny : (gy >= ny ? gy - ny : -1);
        const bool left = gx == ng, right = gx == ng + nx - 1;
        if (ty < 0 && !left && !right) return;
        const int N = p.ndust;
        for (int v = 0; v < p.nvar; ++v) {
            const R val = u[uidx(p, v, gy, gx)];
            if (ty >= 0) u[uidx(p, v, ty, gx)] = val;
            if (left || right) {
                R xv = val;
                if (v == 1 || (v >= 5 + N && v < 5 + 2 * N))
                    xv = left ? (val > R(0) ? val : R(0)) : (val < R(0) ? val : R(0));
                for (int g = 0; g < ng; ++g) {
                    const int col = left ? g : ng + nx + g;
                    u[uidx(p, v, gy, col)] = xv;
                    if (ty >= 0) u[uidx(p, v, ty, col)] = xv;
                }
            }
        }
        return;
    }
    const bool xper = !(p.setup == SHARK_SETUP_SOD && p.sod_dir == 0);
    const bool yper = p.ndim == 2 && !(p.setup == SHARK_SETUP_SOD && p.sod_dir == 1);
    int tx = -1, ty = -1;
    if (xper) {
        if (gx < 2 * ng) tx = gx + nx;            // source of a right ghost
        else if (gx >= nx) tx = gx - nx;          // source of a left ghost
    }
    if (yper) {
        if (gy < 2 * ng) ty = gy + ny;
        else if (gy >= ny) ty = gy - ny;
    }
    if (tx < 0 && ty < 0) return;
    const bool shear = p.setup == SHARK_SETUP_SI;
    const R sgn = (tx >= 0 && tx > gx) ? R(1) : R(-1);   // right ghost: + rho q Omega L
    const R qoL = prm<R>(p.si_q, p.f_si_q), om = prm<R>(p.si_om, p.f_si_om), L = prm<R>(p.box_l, p.f_box_l);
    const int N = p.ndust;
    for (int v = 0; v < p.nvar; ++v) {
        R val = u[uidx(p, v, gy, gx)];
        if (ty >= 0) u[uidx(p, v, ty, gx)] = val;               // y image (no shear)
        if (tx >= 0) {
            R xv = val;
            if (shear) {
                int vr = -1;
                if (v == 3) vr = 0;
                else if (v >= 5 + 3 * N) vr = v - 3 * N;         // vz momentum of dust species -> its density
                if (vr >= 0) xv = val + sgn * (u[uidx(p, vr, gy, gx)] * qoL * om * L);
            }
            u[uidx(p, v, gy, tx)] = xv;                             // x image
            if (ty >= 0) u[uidx(p, v, ty, tx)] = xv;                // corner image
        }
    }
}

__device__ __forceinline__ void atomic_min_dt(unsigned long long* a, double v) {
    // positive finite doubles order like their bit patterns
    atomicMin(a, (unsigned long long)__double_as_longlong(v));
}

// Block-wide min of the CFL candidates and OR of the status bits, then one atomic per block.
// Every thread of the block must call it (no early return before it).
__device__ __forceinline__ void block_reduce_dt(double dtc, unsigned int st, unsigned long long* dt_next,
                                                unsigned int* status) {
    for (int o = 16; o > 0; o >>= 1) {
        const double other = __shfl_xor_sync(0xffffffffu, dtc, o);
        dtc = other < dtc ? other : dtc;
        st |= __shfl_xor_sync(0xffffffffu, st, o);
    }
    __shared__ double wmin[32];
    __shared__ unsigned int wst[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { wmin[wid] = dtc; wst[wid] = st; }
    __syncthreads();
    if (wid == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        dtc = lane < nw ? wmin[lane] : 2e44;
        st = lane < nw ? wst[lane] : 0u;
        for (int o = 16; o > 0; o >>= 1) {
            const double other = __shfl_xor_sync(0xffffffffu, dtc, o);
            dtc = other < dtc ? other : dtc;
            st |= __shfl_xor_sync(0xffffffffu, st, o);
        }
        if (lane == 0) {
            atomic_min_dt(dt_next, dtc);
            if (st) atomicOr(status, st);
        }
    }
}

// FP32 form for the mixed path, whose CFL candidates are FP32: the min runs in FP32 (the FP64
// pipe is narrow) and the block's result is widened once for the atomic.  No candidate: 2e38f.
__device__ __forceinline__ void block_reduce_dt_f(float dtc, unsigned int st, unsigned long long* dt_next,
                                                  unsigned int* status) {
    for (int o = 16; o > 0; o >>= 1) {
        dtc = fminf(dtc, __shfl_xor_sync(0xffffffffu, dtc, o));
        st |= __shfl_xor_sync(0xffffffffu, st, o);
    }
    __shared__ float wminf[32];
    __shared__ unsigned int wstf[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { wminf[wid] = dtc; wstf[wid] = st; }
    __syncthreads();
    if (wid == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        dtc = lane < nw ? wminf[lane] : 2e38f;
        st = lane < nw ? wstf[lane] : 0u;
        for (int o = 16; o > 0; o >>= 1) {
            dtc = fminf(dtc, __shfl_xor_sync(0xffffffffu, dtc, o));
            st |= __shfl_xor_sync(0xffffffffu, st, o);
        }
        if (lane == 0) {
            atomic_min_dt(dt_next, dtc >= 2e38f ? 2e44 : (double)dtc);
            if (st) atomicOr(status, st);
        }
    }
}

// Sound speed of the cell at the start of the step: the isothermal column value, or ctoprim's
// sqrt(gamma P / max(rho, smallr)) of the adiabatic state (solve.f90:205-233).
template <typename R>
__device__ __forceinline__ double cs_start(const KParams<R>& p, int gx, int gy) {
    if (p.iso == 1) return p.ccsd ? p.ccsd[(long long)gy * p.pitch + gx] : p.csd[gx];
    const double rho = (double)p.u_cur[uidx(p, 0, gy, gx)];
    const double vx = (double)p.u_cur[uidx(p, 1, gy, gx)] / rho, vy = (double)p.u_cur[uidx(p, 2, gy, gx)] / rho;
    const double vz = (double)p.u_cur[uidx(p, 3, gy, gx)] / rho;
    const double ekin = 0.5 * rho * (vx * vx) + 0.5 * rho * (vy * vy) + 0.5 * rho * (vz * vz);
    double P = (p.gamma - 1.0) * ((double)p.u_cur[uidx(p, 4, gy, gx)] - ekin - 0.0);
    P = P > p.smallp ? P : p.smallp;
    const double qr = rho > p.smallr ? rho : p.smallr;
    return sqrt(p.gamma * P / qr);
}

// Stopping time of species k at cell (gx, gy) from the state at the start of the step
// (compute_tstop runs before the update, solve.f90:34-35); qrho_old = max(rho_old, smallr).
template <typename R>
__device__ __forceinline__ double tstop_cell(const KParams<R>& p, int k, double qrho_old, int gx, int gy) {
    constexpr double pi = 3.141592653589793238462643383279;
    if (p.setup == SHARK_SETUP_SI) return p.dtstop[k];                       // SI/setup.f90:389-397
    if (p.setup == SHARK_SETUP_DUSTYWAVE) {                                  // DUSTYWAVE/setup.f90:217
        const double rd_old = (double)p.u_cur[uidx(p, 5 + k, gy, gx)];
        return rd_old * qrho_old / p.dK[k] / (qrho_old);
    }
    if (p.setup == SHARK_SETUP_DUSTYTURB)    // dustyTurb/setup.f90:456
        return p.dstokes[k] * p.box_l * p.turb_rho0 / p.csd[gx] / qrho_old;
    if (p.setup == SHARK_SETUP_DISK_POLAR)   // Epstein on the midplane density Sigma/(sqrt(2 pi) H)
        return sqrt(pi * p.gamma / 8.0) * (p.rhograin) * p.dsize[k] / (qrho_old / p.hsd[gx] * p.csd[gx]);
    if (p.setup == SHARK_SETUP_DISK_CART) {  // disk/setup.f90 compute_tstop: Sigma/sqrt(2 pi H)
        const long long e = (long long)gy * p.pitch + gx;
        return sqrt(pi * p.gamma / 8.0) * (p.rhograin) * p.dsize[k] / (qrho_old / p.chsd[e] * p.ccsd[e]);
    }
    // Epstein (SOD/setup.f90:179-185) with the cell's sound speed
    return sqrt(pi * p.gamma / 8.0) * (p.rhograin) * p.dsize[k] / (qrho_old * cs_start(p, gx, gy));
}

// Drag heating of an adiabatic gas with back reaction (source_terms.f90:88-97): the energy
// gains sum_k dt v.(v - v_k)/t_k with the velocities and stopping times at the start of the step.
template <typename R>
__device__ __forceinline__ double drag_heating(const KParams<R>& p, int gx, int gy, double dt) {
    const int N = p.ndust;
    const double rho = (double)p.u_cur[uidx(p, 0, gy, gx)];
    const double qrho = rho > p.smallr ? rho : p.smallr;
    const double vx = (double)p.u_cur[uidx(p, 1, gy, gx)] / rho, vy = (double)p.u_cur[uidx(p, 2, gy, gx)] / rho;
    const double vz = (double)p.u_cur[uidx(p, 3, gy, gx)] / rho;
    double S = 0.0;
    for (int k = 0; k < N; ++k) {
        const double ts = tstop_cell(p, k, qrho, gx, gy);
        const double rd = (double)p.u_cur[uidx(p, 5 + k, gy, gx)];
        const double vdx = (double)p.u_cur[uidx(p, 5 + N + k, gy, gx)] / rd;
        const double vdy = (double)p.u_cur[uidx(p, 5 + 2 * N + k, gy, gx)] / rd;
        const double vdz = (double)p.u_cur[uidx(p, 5 + 3 * N + k, gy, gx)] / rd;
        S = S + dt * (vx * (vx - vdx)) / ts + dt * (vy * (vy - vdy)) / ts + dt * (vz * (vz - vdz)) / ts;
    }
    return S;
}

// setup_inloop of the polar disk (disk_polar/setup.f90:206-284) for one active cell, FP64 or
// FP32 arithmetic: the first active column is reset to its initial state; inside r_relax the
// density and in-plane velocities of gas and dust relax towards the initial state with
// exp(-dt/t_rel).  Returns true when it changed the cell.
template <typename R, typename C>
__device__ __forceinline__ bool disk_inloop_cell(const KParams<R>& p, R* u, int gx, int gy, double dt) {
    const int N = p.ndust;
    if (gx == p.ng) {
        for (int v = 0; v < p.nvar; ++v) u[uidx(p, v, gy, gx)] = p.u_init[uidx(p, v, gy, gx)];
        return true;
    }
    const double trel = p.treld[gx];
    if (!(trel > 0.0)) return false;
    const C e = C(exp(-dt / trel));
    for (int s = 0; s <= N; ++s) {
        const int ir = svar(s, 0, N), ivx = svar(s, 1, N), ivy = svar(s, 2, N);
        const C rho_init = C(p.u_init[uidx(p, ir, gy, gx)]);
        const C vx_init = C(p.u_init[uidx(p, ivx, gy, gx)]) / rho_init;
        const C vy_init = C(p.u_init[uidx(p, ivy, gy, gx)]) / rho_init;
        const C rho_old = C(u[uidx(p, ir, gy, gx)]);
        const C vx_old = C(u[uidx(p, ivx, gy, gx)]) / rho_old;
        const C vy_old = C(u[uidx(p, ivy, gy, gx)]) / rho_old;
        const C rho_new = (rho_init) * (C(1) - e) + rho_old * e;
        const C vx_new = (vx_init) * (C(1) - e) + vx_old * e;
        const C vy_new = (vy_init) * (C(1) - e) + vy_old * e;
        u[uidx(p, ir, gy, gx)] = R(rho_new);
        u[uidx(p, ivx, gy, gx)] = R(rho_new * vx_new);
        u[uidx(p, ivy, gy, gx)] = R(rho_new * vy_new);
    }
    return true;
}

// setup_inloop of the Cartesian disk (disk/setup.f90) for one active cell: a buffer cell takes
// the state the host tabulated with the routine's operations (its relaxation rate is 0).
// Returns true when it changed the cell.
template <typename R>
__device__ __forceinline__ bool cdisk_inloop_cell(const KParams<R>& p, R* u, int gx, int gy) {
    const long long e = (long long)gy * p.pitch + gx, pl = p.plane;
    const double rho_ana = p.ctgt[e];
    if (!(rho_ana > 0.0)) return false;
    const int N = p.ndust;
    u[uidx(p, 0, gy, gx)] = R(rho_ana);
    u[uidx(p, 1, gy, gx)] = R(p.ctgt[pl + e]);
    u[uidx(p, 2, gy, gx)] = R(p.ctgt[2 * pl + e]);
    u[uidx(p, 4, gy, gx)] = R(p.ctgt[3 * pl + e]);
    const R rd = R(p.ctgt[4 * pl + e]), mx = R(p.ctgt[5 * pl + e]), my = R(p.ctgt[6 * pl + e]);
    for (int k = 0; k < N; ++k) {
        u[uidx(p, 5 + k, gy, gx)] = rd;
        u[uidx(p, 5 + N + k, gy, gx)] = mx;
        u[uidx(p, 5 + 2 * N + k, gy, gx)] = my;
    }
    return true;
}

// dust_growth of one active cell of K2 (growth.cuh); u holds the post-drag state.  Returns the
// status bits it raises.
template <typename R>
__device__ __noinline__ unsigned grow_in_finalize(const KParams<R>& p, R* u, int gx, int gy, double dt) {
    const int N = p.ndust;
    double rd[GROWTH_MAX_DUST], ts[GROWTH_MAX_DUST], vx[GROWTH_MAX_DUST], vy[GROWTH_MAX_DUST], vz[GROWTH_MAX_DUST];
    double gam[GROWTH_MAX_DUST];
    const double rho_old = (double)p.u_cur[uidx(p, 0, gy, gx)];
    const double qrho_old = rho_old > p.smallr ? rho_old : p.smallr;
    const bool ambi = (p.gw.mode & SHARK_GROWTH_AMBIPOLAR) && p.chg_gamma_d;
    const long long c = (long long)gy * p.pitch + gx;
    for (int k = 0; k < N; ++k) {
        rd[k] = (double)u[uidx(p, 5 + k, gy, gx)];
        ts[k] = tstop_cell(p, k, qrho_old, gx, gy);
        const double r0 = (double)p.u_cur[uidx(p, 5 + k, gy, gx)];
        vx[k] = (double)p.u_cur[uidx(p, 5 + N + k, gy, gx)] / r0;
        vy[k] = (double)p.u_cur[uidx(p, 5 + 2 * N + k, gy, gx)] / r0;
        vz[k] = (double)p.u_cur[uidx(p, 5 + 3 * N + k, gy, gx)] / r0;
        gam[k] = ambi ? (double)p.chg_gamma_d[(long long)k * p.plane + c] : 0.0;
    }
    const double eta_a = ambi ? (double)p.chg_eta[2 * p.plane + c] : 0.0;
    const double hs = p.setup == SHARK_SETUP_DISK_POLAR ? p.hsd[gx] : 1.0;
    const double rho_gas = (double)u[uidx(p, 0, gy, gx)];
    bool ok;
    if constexpr (sizeof(R) == 4)
        ok = growth_cell_f(p.gw, N, gx, dt, (float)rho_gas, (float)qrho_old, (float)hs, rd, ts, vx, vy, vz,
                           ambi ? gam : nullptr, (float)eta_a);
    else
        ok = growth_cell_d(p.gw, N, gx, dt, rho_gas, qrho_old, hs, rd, ts, vx, vy, vz, ambi ? gam : nullptr, eta_a);
    for (int k = 0; k < N; ++k) u[uidx(p, 5 + k, gy, gx)] = R(rd[k]);
    return ok ? 0u : (unsigned)SHARK_STATUS_GROWTH;
}

// Dust growth of the mixed path without fragmentation (dust_growth.f90:3-256), one warp per cell
// for the 256 cells of a K2 block (warp w takes cells 32 w .. 32 w + 31 in turn).  Lane b holds
// bin b's density.  Once per cell the lanes form the pair rates pK dv / hs of pairs
// q = lane, lane + 32, ... from the start-of-step stopping times and velocities (exchanged by
// shuffles).  Every sub-step each lane writes the collision rate w_q = rate_q rho_k rho_j (times
// the sticking efficiency) of its pairs to shared memory, and lane b gathers
// drho_b/dt = sum_t gc[t][b] w[gq[t][b]] from the host-built table of net transfers (staged in
// shared memory as four rows' coefficients per 128-bit entry and two rows' pair indices, 16 bits
// each, per 32-bit word, the four partial sums of rows t mod 4 as two packed FMAs); the sub-step is the warp minimum of CFL_growth rho_b/|drho_b/dt| (one redux.sync on the
// candidates' bit patterns), and the part of dt still to integrate is kept as an FP32 fraction
// (the last sub-step takes all of it).  The lanes of a warp take the same sub-steps, so a warp
// costs the sub-steps of its own cell rather than those of the slowest of 32 cells.  Called by
// every thread of the block.
constexpr int GROWTH_PAIR_SLOTS = (GROWTH_MAX_PAIRS + 31) / 32;
constexpr int GROWTH_SMEM_ROWS = 80;        // gather rows staged in shared memory (64 at 32 species)

static __device__ __noinline__ unsigned grow_block_warps(const KParams<float>& p, int gx_block, int gy, double dt) {
    __shared__ float sw[8][GROWTH_MAX_PAIRS];
    // gather table: coefficient of row t, lane l at sgc[128 (t >> 2) + 4 l + (t & 3)]; pair
    // indices of rows 4 u + 2 h, 4 u + 2 h + 1 (low, high 16 bits) at sgi[64 u + 2 l + h]
    __shared__ __align__(16) float sgc[GROWTH_SMEM_ROWS * 32];
    __shared__ __align__(8) unsigned sgi[GROWTH_SMEM_ROWS / 2 * 32];
    __shared__ int spair[GROWTH_PAIR_SLOTS * 32];   // pair (k << 8 | j) of slot i, lane l at [32 i + l]
    const GrowthDev& g = p.gw;
    const int N = p.ndust, P = g.npair, L = g.gL;
    const bool staged = L <= GROWTH_SMEM_ROWS;
    if (staged) {   // rows past L are zero (coefficient 0, pair 0)
        const int L4 = (L + 3) & ~3;
        for (int e = threadIdx.x; e < L4 * 32; e += blockDim.x) {
            const int t = e >> 5, l = e & 31;
            sgc[128 * (t >> 2) + 4 * l + (t & 3)] = t < L ? __ldg(g.gc + e) : 0.f;
        }
        for (int e = threadIdx.x; e < L4 / 2 * 32; e += blockDim.x) {
            const int r = e >> 5, l = e & 31, t0 = 2 * r;   // rows t0, t0 + 1 of lane l
            const unsigned i0 = t0 < L ? (unsigned)__ldg(g.gq + t0 * 32 + l) : 0u;
            const unsigned i1 = t0 + 1 < L ? (unsigned)__ldg(g.gq + (t0 + 1) * 32 + l) : 0u;
            sgi[64 * (t0 >> 2) + 2 * l + ((t0 >> 1) & 1)] = i0 | (i1 << 16);
        }
    }
    for (int e = threadIdx.x; e < GROWTH_PAIR_SLOTS * 32; e += blockDim.x) spair[e] = e < P ? __ldg(g.pair + e) : 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    float* w = sw[wid];
    float* u = p.u_next;
    const unsigned FULL = 0xffffffffu;
    const bool ambi = (g.mode & SHARK_GROWTH_AMBIPOLAR) && p.chg_gamma_d;
    const bool on = lane < N;
    const int b = on ? lane : 0;
    const bool thr_on = g.kernel == 0 && g.eps_thr > 0.0;
    const float dtf = (float)dt, idtf = 1.f / dtf;
    const float fctl = g.dtctl > 0.0 ? (float)(g.dtctl / dt) : 0.f, dtctl = (float)g.dtctl;
    const float stick = (float)g.sticking, cflg = (float)g.cfl;
    const float eps_thr = (float)g.eps_thr, rmin = (float)g.dust_ratio_min, smallr = (float)p.smallr;
    // stopping times for the pair velocities (FP32): t_k = C_k / F_cell with the tabulated 1/C_k
    // (dustyTurb F = c_s rho, polar disk F = rho/hs c_s); other setups through tstop_cell
    const bool ts_tab = p.setup == SHARK_SETUP_DUSTYTURB || p.setup == SHARK_SETUP_DISK_POLAR;
    const float invc = p.dinvts_f[b];
    const GrowthRunF rf = growth_run_consts_f(g);
    const float4 row0 = growth_row_f(g, 0);        // the one temperature row (dustyTurb)
    unsigned st = 0;
    for (int c = 0; c < 32; ++c) {
        const int gx = gx_block + wid * 32 + c;
        if (gx >= p.ng + p.nx) break;
        const float rho_old = p.u_cur[uidx(p, 0, gy, gx)];
        const float qrho_old = rho_old > smallr ? rho_old : smallr;
        float rd = u[uidx(p, 5 + b, gy, gx)];
        float ts;
        if (ts_tab) {
            const float F = p.setup == SHARK_SETUP_DUSTYTURB ? p.cs[gx] * qrho_old : qrho_old / (float)p.hsd[gx] * p.cs[gx];
            ts = 1.f / (invc * F);
        } else {
            ts = (float)tstop_cell(p, b, (double)qrho_old, gx, gy);
        }
        const float r0 = p.u_cur[uidx(p, 5 + b, gy, gx)];
        const float vx = p.u_cur[uidx(p, 5 + N + b, gy, gx)] / r0;
        const float vy = p.u_cur[uidx(p, 5 + 2 * N + b, gy, gx)] / r0;
        const float vz = p.u_cur[uidx(p, 5 + 3 * N + b, gy, gx)] / r0;
        const long long cidx = (long long)gy * p.pitch + gx;
        float gm = 0.f, eta_a = 0.f;
        if (ambi) {
            const float ga = p.chg_gamma_d[(long long)b * p.plane + cidx];
            gm = fabsf(ga) * rsqrtf(1.f + ga * ga);
            eta_a = p.chg_eta[2 * p.plane + cidx];
        }
        const float hs = p.setup == SHARK_SETUP_DISK_POLAR ? (float)p.hsd[gx] : 1.f;
        const float rho_gas = u[uidx(p, 0, gy, gx)];
        const GrowthCellF cc = growth_cell_consts_f(g, rf, g.t_per_col ? growth_row_f(g, gx) : row0, qrho_old, hs, eta_a);
        const float ihs = 1.f / hs;
        float kp[GROWTH_PAIR_SLOTS];
#pragma unroll
        for (int i = 0; i < GROWTH_PAIR_SLOTS; ++i) {
            kp[i] = 0.f;
            if (32 * i >= P) continue;                      // uniform over the warp
            const int q = lane + 32 * i;
            const bool has = q < P;
            const int pr = spair[q];
            const int k = pr >> 8, j = pr & 255;
            const float tk = __shfl_sync(FULL, ts, k), tj = __shfl_sync(FULL, ts, j);
            const float dx = __shfl_sync(FULL, vx, k) - __shfl_sync(FULL, vx, j);
            const float dy = __shfl_sync(FULL, vy, k) - __shfl_sync(FULL, vy, j);
            const float dz = __shfl_sync(FULL, vz, k) - __shfl_sync(FULL, vz, j);
            const float dg = __shfl_sync(FULL, gm, k) - __shfl_sync(FULL, gm, j);
            if (!has) continue;
            float dv = 1.f;
            if (g.kernel == 0) dv = growth_dv_f(g, rf, cc, tk, tj, cc.T * __ldg(g.pBf + q), dx, dy, dz, dg, ambi);
            kp[i] = __ldg(g.pKf + q) * dv * ihs * (k == j ? 0.5f : 1.f);
        }
        const float thr = eps_thr * rho_gas, fl = rho_gas * rmin;
        float rem = 1.f;                                    // part of dt still to integrate
        int niter = 0;
        while (rem > 0.f && niter < grw::MAX_SUB) {
            niter = niter + 1;
#pragma unroll
            for (int i = 0; i < GROWTH_PAIR_SLOTS; ++i) {
                if (32 * i >= P) continue;
                const int q = lane + 32 * i;
                const int pr = spair[q];
                const float rk = __shfl_sync(FULL, rd, pr >> 8), rj = __shfl_sync(FULL, rd, pr & 255);
                float pc = kp[i] * rk * rj;
                if (thr_on && (rk < thr || rj < thr)) pc = 0.f;
                if (q < P) w[q] = pc * stick;
            }
            __syncwarp();
            float d = 0.f;
            if (staged) {
                // four partial sums: the gather's products are independent, its FMA chain is not
                float2 a0 = make_float2(0.f, 0.f), a1 = make_float2(0.f, 0.f);
                int t = 0;
                for (; t + 4 <= L; t += 4) {
                    const float4 c = *reinterpret_cast<const float4*>(sgc + 32 * t + 4 * lane);
                    const uint2 ix = *reinterpret_cast<const uint2*>(sgi + 16 * t + 2 * lane);
                    a0 = __ffma2_rn(make_float2(c.x, c.y), make_float2(w[ix.x & 0xffffu], w[ix.x >> 16]), a0);
                    a1 = __ffma2_rn(make_float2(c.z, c.w), make_float2(w[ix.y & 0xffffu], w[ix.y >> 16]), a1);
                }
                d = a0.x;
                for (; t < L; ++t) {
                    const float c = sgc[128 * (t >> 2) + 4 * lane + (t & 3)];
                    const unsigned iw = sgi[64 * (t >> 2) + 2 * lane + ((t >> 1) & 1)];
                    d = fmaf(c, w[(t & 1) ? (iw >> 16) : (iw & 0xffffu)], d);
                }
                d = (d + a0.y) + (a1.x + a1.y);
            } else {
                for (int t = 0; t < L; ++t) d += __ldg(g.gc + t * 32 + lane) * w[__ldg(g.gq + t * 32 + lane)];
            }
            __syncwarp();
            // non-negative floats order like their bit patterns read as unsigned integers
            const float c0 = (on && d != 0.f) ? fmaxf(rd / fabsf(d) * cflg, 0.f) : 1e30f;
            const float cand = __uint_as_float(__reduce_min_sync(FULL, __float_as_uint(c0)));
            const float dtg0 = fctl > 0.f ? dtctl : cand;
            const float frac = fctl > 0.f ? fctl : cand * idtf;
            float dtg;
            if (frac >= rem) { dtg = rem * dtf; rem = 0.f; }
            else { dtg = dtg0; rem = rem - frac; }
            rd = fmaxf(rd + d * dtg, fl);
        }
        if (on) u[uidx(p, 5 + b, gy, gx)] = rd;
        if (rem > 0.f) st |= (unsigned)SHARK_STATUS_GROWTH;
    }
    return st;
}

// Driven-turbulence kick of the dustyTurb box (turb.f90:227-324 in 2D): the gas momentum gains
// rho a dt with the solenoidal Ornstein-Uhlenbeck acceleration of this step at the cell centre.
// C = double follows the oracle's operations; C = float is the mixed-precision form.
template <typename C, typename R>
__device__ __forceinline__ void turb_kick_cell(const KParams<R>& p, R* u, int gx, int gy, double dt) {
    const C x = C(p.xposd[gx]);
    const C y = C(((double)(float)(gy - p.ng) + 0.5) * p.box_l_y / (double)(float)p.ny);
    C ax = C(0), ay = C(0);
    for (int m = 0; m < p.ou_nm; ++m) {
        const C kxp = C(p.ou_modes[3 * m]), kyp = C(p.ou_modes[3 * m + 1]), kk = C(p.ou_modes[3 * m + 2]);
        const C ph = kxp * x + kyp * y;
        C sn, cs;
        if constexpr (sizeof(C) == 8) sincos(ph, &sn, &cs);
        else sincosf(ph, &sn, &cs);
        const C w = C(p.ou[2 * m]) * cs + C(p.ou[2 * m + 1]) * sn;
        ax = ax + kyp / kk * w;
        ay = ay - kxp / kk * w;
    }
    const C rho = C(u[uidx(p, 0, gy, gx)]);
    u[uidx(p, 1, gy, gx)] = R(C(u[uidx(p, 1, gy, gx)]) + rho * ax * C(dt));
    u[uidx(p, 2, gy, gx)] = R(C(u[uidx(p, 2, gy, gx)]) + rho * ay * C(dt));
}

template <typename R, int NS, int MODE, bool GROW = false>
__global__ void __launch_bounds__(256) k_finalize(KParams<R> p) {
    constexpr int NMAX = NS > 0 ? NS : 1;
    const int N = NS >= 0 ? NS : p.ndust;
    const int gx = blockIdx.x * blockDim.x + threadIdx.x + p.ng;
    const int gy = (p.ndim == 2) ? blockIdx.y + p.ng : 0;
    double dtc = 2e44;
    unsigned int st = 0;
    if (gx < p.ng + p.nx) {
        R* u = p.u_next;
        const double dt = *p.dt;
        double rho = (double)u[uidx(p, 0, gy, gx)];
        double px = (double)u[uidx(p, 1, gy, gx)], py = (double)u[uidx(p, 2, gy, gx)], pz = (double)u[uidx(p, 3, gy, gx)];
        const bool drag = MODE == 0 && N > 0 && (p.flags & SHARK_FLAG_DRAG);
        const bool br = (p.flags & SHARK_FLAG_BACK_REACTION) != 0;
        if (drag) {
            // dust_drag(1.0) (src/dust/dust_drag.f90:2-75), FP64 arithmetic
            double alpha[NMAX];
            double rhon = rho, pnx = px, pny = py, pnz = pz;
            // stopping time from the state at the start of the step (compute_tstop runs before
            // the update in solve.f90:34-35)
            const double rho_old = (double)p.u_cur[uidx(p, 0, gy, gx)];
            const double qrho_old = rho_old > p.smallr ? rho_old : p.smallr;
            for (int k = 0; k < N; ++k) {
                const double ts = tstop_cell(p, k, qrho_old, gx, gy);
                const double a = 1.0 * dt / ts;
                const double pdx = (double)u[uidx(p, 5 + N + k, gy, gx)];
                const double pdy = (double)u[uidx(p, 5 + 2 * N + k, gy, gx)];
                const double pdz = (double)u[uidx(p, 5 + 3 * N + k, gy, gx)];
                const double rd = (double)u[uidx(p, 5 + k, gy, gx)];
                pnx = pnx + a / (1.0 + a) * pdx;
                pny = pny + a / (1.0 + a) * pdy;
                pnz = pnz + a / (1.0 + a) * pdz;
                rhon = rhon + a / (1.0 + a) * rd;
                if (NS > 0) alpha[k < NMAX ? k : 0] = a;
            }
            for (int k = 0; k < N; ++k) {
                double a;
                if (NS > 0) a = alpha[k < NMAX ? k : 0];
                else a = 1.0 * dt / tstop_cell(p, k, qrho_old, gx, gy);   // run-time species count
                const long long ix_ = uidx(p, 5 + N + k, gy, gx), iy_ = uidx(p, 5 + 2 * N + k, gy, gx),
                                iz_ = uidx(p, 5 + 3 * N + k, gy, gx);
                const double rd = (double)u[uidx(p, 5 + k, gy, gx)];
                u[ix_] = R((double)u[ix_] / (1.0 + a) + (a / (1.0 + a)) * pnx / rhon * rd);
                u[iy_] = R((double)u[iy_] / (1.0 + a) + (a / (1.0 + a)) * pny / rhon * rd);
                u[iz_] = R((double)u[iz_] / (1.0 + a) + (a / (1.0 + a)) * pnz / rhon * rd);
            }
            if (br) {
                px = pnx / rhon * rho;
                py = pny / rhon * rho;
                pz = pnz / rhon * rho;
                u[uidx(p, 1, gy, gx)] = R(px);
                u[uidx(p, 2, gy, gx)] = R(py);
                u[uidx(p, 3, gy, gx)] = R(pz);
            }
            // re-read the stored (rounded) values so the dt below sees exactly the stored state
            px = (double)u[uidx(p, 1, gy, gx)];
            py = (double)u[uidx(p, 2, gy, gx)];
            pz = (double)u[uidx(p, 3, gy, gx)];
        }
        if (MODE == 0 && N > 0 && (p.flags & SHARK_FLAG_DRAG)) {
            // regularisation floor (dust_drag.f90:63-73)
            for (int k = 0; k < N; ++k) {
                const long long ir = uidx(p, 5 + k, gy, gx);
                const double rd = (double)u[ir];
                const double fl = rho * p.dust_ratio_min;
                if (fl > rd) u[ir] = R(fl);
            }
        }
        if (MODE == 0 && N > 0 && br && p.iso < 1) {   // drag heating, part of S_U (source_terms.f90:88-97)
            const long long ie = uidx(p, 4, gy, gx);
            u[ie] = R((double)u[ie] + drag_heating(p, gx, gy, dt));
        }
        if (GROW && MODE == 0) st |= grow_in_finalize(p, u, gx, gy, dt);   // dust_growth (solve.f90:113)
        if (MODE == 0 && p.ou_nm > 0) {                                    // turbulence kick (solve.f90:129-146)
            turb_kick_cell<double>(p, u, gx, gy, dt);
            px = (double)u[uidx(p, 1, gy, gx)];
            py = (double)u[uidx(p, 2, gy, gx)];
        }
        if (MODE == 0 && p.setup == SHARK_SETUP_SI && !(p.flags & SHARK_FLAG_FORCE_KICK)) {
            // setup_inloop: Crank-Nicolson rotation (SI/setup.f90:299-332)
            const double om = p.si_om, qsh = p.si_q;
            const double Ohmdt = om * dt;
            const double xc = p.xposd[gx] - 0.5 * p.box_l;
            double AA = 2.0 * qsh * om * xc - 2.0 * p.si_r0 * p.si_eta;
            {
                const double uz = pz / rho, vx = px / rho, d = rho;
                pz = d * (uz * (1. - Ohmdt * Ohmdt) + 2. * vx * Ohmdt + AA * (Ohmdt * Ohmdt)) / (1. + Ohmdt * Ohmdt);
                px = d * (vx * (1. - Ohmdt * Ohmdt) - 2. * uz * Ohmdt + AA * Ohmdt) / (1. + Ohmdt * Ohmdt);
                u[uidx(p, 3, gy, gx)] = R(pz);
                u[uidx(p, 1, gy, gx)] = R(px);
                pz = (double)u[uidx(p, 3, gy, gx)];
                px = (double)u[uidx(p, 1, gy, gx)];
            }
            AA = 2.0 * qsh * om * xc;
            for (int k = 0; k < N; ++k) {
                const long long iz = uidx(p, 5 + 3 * N + k, gy, gx), ixx = uidx(p, 5 + N + k, gy, gx);
                const double d = (double)u[uidx(p, 5 + k, gy, gx)];
                const double uz = (double)u[iz] / d, vx = (double)u[ixx] / d;
                u[iz] = R(d * (uz * (1. - Ohmdt * Ohmdt) + 2. * vx * Ohmdt + AA * (Ohmdt * Ohmdt)) / (1. + Ohmdt * Ohmdt));
                u[ixx] = R(d * (vx * (1. - Ohmdt * Ohmdt) - 2. * uz * Ohmdt + AA * Ohmdt) / (1. + Ohmdt * Ohmdt));
            }
        }
        if (MODE == 0 && ((p.setup == SHARK_SETUP_DISK_POLAR && disk_inloop_cell<R, double>(p, u, gx, gy, dt)) ||
                          (p.setup == SHARK_SETUP_DISK_CART && cdisk_inloop_cell<R>(p, u, gx, gy)))) {
            rho = (double)u[uidx(p, 0, gy, gx)];
            px = (double)u[uidx(p, 1, gy, gx)];
            py = (double)u[uidx(p, 2, gy, gx)];
            pz = (double)u[uidx(p, 3, gy, gx)];
        }
        // ---- courant on the final state (src/solver/courant.f90:11-124) -----------------------
        const double cfl = p.cfl;
        const double qrho = rho > p.smallr ? rho : p.smallr;
        const double vx = px / rho, vy = py / rho, vz = pz / rho;
        double cs;
        if (p.iso == 1) cs = p.ccsd ? p.ccsd[(long long)gy * p.pitch + gx] : p.csd[gx];
        else {
            const double E = (double)u[uidx(p, 4, gy, gx)];
            const double ekin = 0.5 * rho * (vx * vx) + 0.5 * rho * (vy * vy) + 0.5 * rho * (vz * vz);
            double P = (p.gamma - 1.0) * (E - ekin - 0.0);
            P = P > p.smallp ? P : p.smallp;
            cs = sqrt(p.gamma * P / qrho);
            if (!(E == E)) st |= SHARK_STATUS_NAN;
        }
        double dxx;
        if (p.ndim == 1) dxx = p.dx1d[gx];
        else if (p.geom == 2) { const double a = p.dx1d[gx], b = p.radcd[gx] * p.dx2d[gx]; dxx = a < b ? a : b; }
        else { const double a = p.dx1d[gx], b = p.dx2d[gx]; dxx = a < b ? a : b; }
        double vv = fabs(vx) + fabs(vy) + fabs(vz);
        double vmax = cs + vv;
        double fmax_d = 0.0;
        const bool fk = (p.flags & SHARK_FLAG_FORCE_KICK) != 0;
        if (fk && p.setup == SHARK_SETUP_SI) {
            const double xc = p.xposd[gx] - 0.5 * p.box_l, om = p.si_om, qsh = p.si_q;
            const double f1 = 2.0 * qsh * (om * om) * xc - 2.0 * om * vz - 2.0 * p.si_r0 * om * p.si_eta;
            const double f3 = 2.0 * om * vx;
            fmax_d = sqrt(f1 * f1 + 0.0 * 0.0 + f3 * f3);
        } else if (fk && p.setup == SHARK_SETUP_DISK_POLAR) {
            // the same point-mass force acts on gas and every dust species
            const double g = p.fgravd[gx];
            fmax_d = sqrt(g * g + 0.0 * 0.0 + 0.0 * 0.0);
        } else if (fk && p.setup == SHARK_SETUP_DISK_CART) {   // the star's softened force, gas and dust
            const long long e = (long long)gy * p.pitch + gx;
            const double fx = (double)p.cfx[e], fy = (double)p.cfy[e];
            fmax_d = sqrt(fx * fx + fy * fy + 0.0 * 0.0);
        }
        for (int k = 0; k < N; ++k) {
            const double rd = (double)u[uidx(p, 5 + k, gy, gx)];
            const double vdx = (double)u[uidx(p, 5 + N + k, gy, gx)] / rd;
            const double vdy = (double)u[uidx(p, 5 + 2 * N + k, gy, gx)] / rd;
            const double vdz = (double)u[uidx(p, 5 + 3 * N + k, gy, gx)] / rd;
            vv = fabs(vdx) + fabs(vdy) + fabs(vdz);
            vmax = vmax > (0.0 + vv) ? vmax : (0.0 + vv);
            if (fk && p.setup == SHARK_SETUP_SI) {
                const double xc = p.xposd[gx] - 0.5 * p.box_l, om = p.si_om, qsh = p.si_q;
                const double f1 = 2.0 * qsh * (om * om) * xc - 2.0 * om * vdz;
                const double f3 = 2.0 * om * vdx;
                const double fm = sqrt(f1 * f1 + 0.0 * 0.0 + f3 * f3);
                fmax_d = fmax_d > fm ? fmax_d : fm;
            }
            if (!(rd > 0.0)) st |= SHARK_STATUS_NEG_DENSITY;
            if (!isfinite(vdx) || !isfinite(vdy) || !isfinite(vdz)) st |= SHARK_STATUS_NAN;
        }
        const double c1 = cfl * dxx / fabs(vmax);
        dtc = dtc < c1 ? dtc : c1;
        if (fk && vv != 0.0) {
            double fratio = fmax_d * dxx / (vv * vv);
            fratio = fratio > 1e-3 ? fratio : 1e-3;
            const double c2 = cfl * dxx / vv * (sqrt(1.0 + 2.0 * cfl * fratio) - 1.0) / fratio;
            dtc = dtc < c2 ? dtc : c2;
        }
        if (!(rho > 0.0)) st |= SHARK_STATUS_NEG_DENSITY;
        if (!isfinite(vx) || !isfinite(vy) || !isfinite(vz) || !isfinite(rho)) st |= SHARK_STATUS_NAN;
        if (!(dtc > 0.0) || !isfinite(dtc)) { st |= SHARK_STATUS_DT_UNDERFLOW; dtc = 2e44; }
    }
    block_reduce_dt(dtc, st, p.dt_next, p.status);
    if (MODE == 0 && gx < p.ng + p.nx) fill_ghost_images(p, p.u_next, gx, gy);
}

// ---------------------------------------------------------------------------------------------
// K2, mixed precision (FP32 state).  The stiff part of the implicit drag -- the coefficients
// 1/(1+a_k) and a_k/(1+a_k) with a_k = dt/t_k, which carry the t_stop << dt limit -- is computed in
// FP64 (once per block when t_k is a per-species constant, as in the SI box; per cell otherwise).
// The per-cell barycentric combination (positive weights, no cancellation) and the CFL candidate
// run in FP32 like the rest of the mixed path.  Same algorithm as dust_drag.f90:29-73.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ void drag_coeffs(double a, float& r, float& w) {
    const double d = 1.0 + a;
    r = (float)(1.0 / d);
    w = (float)(a / d);
}

// a_k = dt/t_k of the mixed path where the per-cell stopping time factors as t_k = C_k / F_cell
// (dustyTurb C_k = St_0,k L rho_0, F = c_s rho; the disks' Epstein F = rho/hs c_s): dt F_cell times
// the tabulated 1/C_k, and the coefficients with a refined reciprocal (FP64 throughout; the
// divisions cost most of K2's FP64 work at 32 species).  Other setups divide directly.
__device__ __forceinline__ double drag_cell_factor(const KParams<float>& p, double dt, double qrho_old, int gx, int gy) {
    if (p.setup == SHARK_SETUP_DUSTYTURB) return dt * (p.csd[gx] * qrho_old);
    if (p.setup == SHARK_SETUP_DISK_CART) {
        const long long e = (long long)gy * p.pitch + gx;
        return dt * (qrho_old / p.chsd[e] * p.ccsd[e]);
    }
    return dt * (qrho_old / p.hsd[gx] * p.csd[gx]);
}

// The same coefficients in FP32 from a = dt F_cell / C_k formed in FP32 (dt F_cell once per cell
// in FP64, then per species one product): r = 1/(1+a) and w = a r are well conditioned for every
// a >= 0 (no cancellation; a = dt/t_k >> 1 gives r ~ 1/a, w ~ 1 to FP32 rounding), so the state's
// FP32 precision bounds them.  a is capped at 1e30 so that 1 + a stays finite.
__device__ __forceinline__ void drag_coeffs_f(float a, float& r, float& w) {
    a = fminf(a, 1e30f);
    r = 1.0f / (1.0f + a);
    w = a * r;
}

__device__ __forceinline__ void drag_coeffs_mix(double a, float& r, float& w) {
    const double d = 1.0 + a;
    if (d < 1e30) {
        const double q = rcp_refined(d);
        r = (float)q;
        w = (float)(a * q);
    } else {
        drag_coeffs(a, r, w);
    }
}

// Threads per block of the mixed K2 without growth: small blocks, so that the warps of a block
// waiting at the dt reduction's barrier and the last wave hold fewer idle slots (the growth
// variant keeps 256 threads: its block-cooperative phase is laid out for 8 warps).
constexpr int K2M_THREADS = 128;

// Blocks per SM: 8 species at 5 blocks of 128 threads (96 registers), measured best of 4-6.
template <int NS, int MODE, bool GROW = false>
__global__ void __launch_bounds__(GROW ? 256 : K2M_THREADS,
                                  GROW ? ((NS >= 8) ? 2 : 3) : (NS == 8 ? 5 : ((NS > 8) ? 2 : 3) * (256 / K2M_THREADS)))
k_finalize_mixed(KParams<float> p) {
    constexpr int NMAX = NS > 0 ? NS : 1;
    const int N = NS >= 0 ? NS : p.ndust;
    const bool drag = MODE == 0 && N > 0 && (p.flags & SHARK_FLAG_DRAG);
    // constant stopping times (SI): the FP64 coefficients of this step were computed once by
    // k_prepare_step; other setups compute them per cell below
    const bool const_ts = p.setup == SHARK_SETUP_SI;
    const float* __restrict__ cr = p.coef;
    const float* __restrict__ cw = p.coef + SHARK_MAX_DUST;
    const double dt = *p.dt;
    const int gx = blockIdx.x * blockDim.x + threadIdx.x + p.ng;
    const int gy = (p.ndim == 2) ? blockIdx.y + p.ng : 0;
    float dtc = 2e38f;
    unsigned int st = 0;
    const bool act = gx < p.ng + p.nx;
    float* u = p.u_next;
    // this cell's element of plane 0, variable v v planes further, as 32-bit offsets from the
    // state's (uniform) base pointer (the context guarantees nvar * plane < 2^31): an access is a
    // 32-bit offset on a uniform base, not a 64-bit address formed per thread
    const int cc = gy * p.pitch + gx;
    const float* __restrict__ ucur = p.u_cur;
    const int pl = (int)p.plane;
    float rho = 0.f, px = 0.f, py = 0.f, pz = 0.f;
    // compile-time species count: the cell's dust state is loaded once into registers (all loads
    // in flight together) and the CFL loop reads it there unless a setup hook rewrote it
    float dr[NMAX], dmx[NMAX], dmy[NMAX], dmz[NMAX];
    bool in_regs = false;
    // courant's dust terms taken in the drag update loop, right after each species' final values
    // (the species' registers then die one by one instead of living until the CFL): allowed when
    // no setup hook changes the dust between the drag and the CFL
    const bool fk_si = (p.flags & SHARK_FLAG_FORCE_KICK) != 0 && p.setup == SHARK_SETUP_SI;
    const bool cfl_in_drag = NS > 0 && NS <= 8 && drag && p.ou_nm == 0 && p.setup != SHARK_SETUP_DISK_POLAR &&
                             p.setup != SHARK_SETUP_DISK_CART &&
                             !(p.setup == SHARK_SETUP_SI && !(p.flags & SHARK_FLAG_FORCE_KICK));
    bool cfl_done = false;
    float vmax_d = 0.f, vv_last = 0.f, fmx2_d = 0.f;
    const float xc = act ? p.xpos[gx] - p.f_half_box_l : 0.f;
    // part 1: drag, floor, drag heating; part 2: kick, setup_inloop, CFL.  With growth in between
    // (a block-wide phase) the two parts are separate; otherwise they form one block of code.
    auto part1 = [&]() {
        // the loads take their offsets from an opaque copy of the cell offset, so that the
        // compiler forms the stores' offsets anew instead of keeping every load offset live
        int cl = cc;
        asm volatile("" : "+r"(cl));
        rho = u[cl + (0) * pl];
        px = u[cl + (1) * pl]; py = u[cl + (2) * pl]; pz = u[cl + (3) * pl];
        if constexpr (NS > 0) {
            if (drag) {
#pragma unroll
                for (int k = 0; k < NS; ++k) {
                    dr[k] = u[cl + (5 + k) * pl];
                    dmx[k] = u[cl + (5 + N + k) * pl];
                    dmy[k] = u[cl + (5 + 2 * N + k) * pl];
                    dmz[k] = u[cl + (5 + 3 * N + k) * pl];
                }
                float rk[NMAX], wk[NMAX];
                if (const_ts) {          // the step's coefficients (no FP64 work per cell)
#pragma unroll
                    for (int k = 0; k < NS; ++k) { rk[k] = cr[k]; wk[k] = cw[k]; }
                } else {
                    const float rho_old = ucur[cc + (0) * pl];
                    const double qrho_old = (double)fmaxf(rho_old, p.f_smallr);
                    const bool direct = p.setup != SHARK_SETUP_DUSTYTURB && p.setup != SHARK_SETUP_DISK_POLAR &&
                                          p.setup != SHARK_SETUP_DISK_CART;
                    const float Fcf = direct ? 0.f : (float)drag_cell_factor(p, dt, qrho_old, gx, gy);
#pragma unroll
                    for (int k = 0; k < NS; ++k) {
                        if (direct) drag_coeffs_mix(1.0 * dt / tstop_cell(p, k, qrho_old, gx, gy), rk[k], wk[k]);
                        else drag_coeffs_f(Fcf * p.dinvts_f[k], rk[k], wk[k]);
                    }
                }
                float rhon = rho, pnx = px, pny = py, pnz = pz;
#pragma unroll
                for (int k = 0; k < NS; ++k) {
                    pnx += wk[k] * dmx[k];
                    pny += wk[k] * dmy[k];
                    pnz += wk[k] * dmz[k];
                    rhon += wk[k] * dr[k];
                }
                const float irhon = 1.0f / rhon;
                const float vbx = pnx * irhon, vby = pny * irhon, vbz = pnz * irhon;
                const float fl = rho * p.f_dust_ratio_min;   // floor (dust_drag.f90:63-73)
                const float om = p.f_si_om, qsh = p.f_si_q;
#pragma unroll
                for (int k = 0; k < NS; ++k) {
                    const float wr = wk[k] * dr[k];
                    dmx[k] = dmx[k] * rk[k] + wr * vbx;
                    dmy[k] = dmy[k] * rk[k] + wr * vby;
                    dmz[k] = dmz[k] * rk[k] + wr * vbz;
                    u[cc + (5 + N + k) * pl] = dmx[k];
                    u[cc + (5 + 2 * N + k) * pl] = dmy[k];
                    u[cc + (5 + 3 * N + k) * pl] = dmz[k];
                    if (fl > dr[k]) { dr[k] = fl; u[cc + (5 + k) * pl] = fl; }
                    if (cfl_in_drag) {   // the dust loop of courant, see part 2
                        const float ird = 1.0f / dr[k];
                        const float vdx = dmx[k] * ird, vdy = dmy[k] * ird, vdz = dmz[k] * ird;
                        const float vv = fabsf(vdx) + fabsf(vdy) + fabsf(vdz);
                        vmax_d = fmaxf(vmax_d, vv);
                        vv_last = vv;
                        if (fk_si) {
                            const float f1 = 2.0f * qsh * (om * om) * xc - 2.0f * om * vdz;
                            const float f3 = 2.0f * om * vdx;
                            fmx2_d = fmaxf(fmx2_d, f1 * f1 + f3 * f3);
                        }
                        if (!(dr[k] > 0.f)) st |= SHARK_STATUS_NEG_DENSITY;
                        if (!isfinite(vv)) st |= SHARK_STATUS_NAN;
                    }
                }
                cfl_done = cfl_in_drag;
                if (p.flags & SHARK_FLAG_BACK_REACTION) {
                    px = vbx * rho; py = vby * rho; pz = vbz * rho;
                    u[cc + (1) * pl] = px;
                    u[cc + (2) * pl] = py;
                    u[cc + (3) * pl] = pz;
                }
                in_regs = true;
            }
        } else if (drag) {
            float rk[NMAX], wk[NMAX];
            float rhon = rho, pnx = px, pny = py, pnz = pz;
            const float rho_old = ucur[cc + (0) * pl];
            const double qrho_old = (double)fmaxf(rho_old, p.f_smallr);
            const bool direct = p.setup != SHARK_SETUP_DUSTYTURB && p.setup != SHARK_SETUP_DISK_POLAR &&
                                          p.setup != SHARK_SETUP_DISK_CART;
            const float Fcf = (const_ts || direct) ? 0.f : (float)drag_cell_factor(p, dt, qrho_old, gx, gy);
            // run-time species count: the cell's coefficients are kept (thread-local memory) for
            // the update loop instead of being formed a second time
            float2 rw_local[NS < 0 ? SHARK_MAX_DUST : 1];
            for (int k = 0; k < N; ++k) {
                float r, w;
                if (const_ts) { r = cr[k]; w = cw[k]; }
                else if (direct) drag_coeffs_mix(1.0 * dt / tstop_cell(p, k, qrho_old, gx, gy), r, w);
                else drag_coeffs_f(Fcf * p.dinvts_f[k], r, w);
                if (NS > 0) { rk[k < NMAX ? k : 0] = r; wk[k < NMAX ? k : 0] = w; }
                else if (!const_ts) rw_local[k] = make_float2(r, w);
                pnx += w * u[cc + (5 + N + k) * pl];
                pny += w * u[cc + (5 + 2 * N + k) * pl];
                pnz += w * u[cc + (5 + 3 * N + k) * pl];
                rhon += w * u[cc + (5 + k) * pl];
            }
            const float irhon = 1.0f / rhon;
            const float vbx = pnx * irhon, vby = pny * irhon, vbz = pnz * irhon;
            for (int k = 0; k < N; ++k) {
                float r, w;
                if (NS > 0) { r = rk[k < NMAX ? k : 0]; w = wk[k < NMAX ? k : 0]; }
                else if (const_ts) { r = cr[k]; w = cw[k]; }
                else { r = rw_local[k].x; w = rw_local[k].y; }
                const float rd = u[cc + (5 + k) * pl];
                const long long ixx = uidx(p, 5 + N + k, gy, gx), iyy = uidx(p, 5 + 2 * N + k, gy, gx),
                                izz = uidx(p, 5 + 3 * N + k, gy, gx);
                const float wr = w * rd;
                u[ixx] = u[ixx] * r + wr * vbx;
                u[iyy] = u[iyy] * r + wr * vby;
                u[izz] = u[izz] * r + wr * vbz;
            }
            if (p.flags & SHARK_FLAG_BACK_REACTION) {
                px = vbx * rho; py = vby * rho; pz = vbz * rho;
                u[cc + (1) * pl] = px;
                u[cc + (2) * pl] = py;
                u[cc + (3) * pl] = pz;
            }
            const float fl = rho * p.f_dust_ratio_min;   // floor (dust_drag.f90:63-73)
            for (int k = 0; k < N; ++k) {
                const long long ir = uidx(p, 5 + k, gy, gx);
                if (fl > u[ir]) u[ir] = fl;
            }
        }
        if (MODE == 0 && N > 0 && (p.flags & SHARK_FLAG_BACK_REACTION) && p.iso < 1) {   // drag heating
            const long long ie = uidx(p, 4, gy, gx);
            u[ie] = (float)((double)u[ie] + drag_heating(p, gx, gy, dt));
        }
    };
    auto part2 = [&]() {
        if (MODE == 0 && p.ou_nm > 0) {                                    // turbulence kick (solve.f90:129-146)
            turb_kick_cell<float>(p, u, gx, gy, dt);
            px = u[cc + (1) * pl];
            py = u[cc + (2) * pl];
        }
        if (MODE == 0 && p.setup == SHARK_SETUP_SI && !(p.flags & SHARK_FLAG_FORCE_KICK)) {
            // setup_inloop: Crank-Nicolson rotation (SI/setup.f90:299-332)
            in_regs = false;
            const float om = p.f_si_om, qsh = p.f_si_q;
            const float Ohmdt = (float)(p.si_om * dt), O2 = Ohmdt * Ohmdt, inv = 1.0f / (1.0f + O2);
            const float xc = p.xpos[gx] - p.f_half_box_l;
            float AA = 2.0f * qsh * om * xc - 2.0f * p.f_si_r0 * p.f_si_eta;
            {
                const float uz = pz / rho, vx = px / rho;
                pz = rho * (uz * (1.f - O2) + 2.f * vx * Ohmdt + AA * O2) * inv;
                px = rho * (vx * (1.f - O2) - 2.f * uz * Ohmdt + AA * Ohmdt) * inv;
                u[cc + (3) * pl] = pz;
                u[cc + (1) * pl] = px;
            }
            AA = 2.0f * qsh * om * xc;
            for (int k = 0; k < N; ++k) {
                const long long iz = uidx(p, 5 + 3 * N + k, gy, gx), ixx = uidx(p, 5 + N + k, gy, gx);
                const float d = u[cc + (5 + k) * pl];
                const float uz = u[iz] / d, vx = u[ixx] / d;
                u[iz] = d * (uz * (1.f - O2) + 2.f * vx * Ohmdt + AA * O2) * inv;
                u[ixx] = d * (vx * (1.f - O2) - 2.f * uz * Ohmdt + AA * Ohmdt) * inv;
            }
        }
        if (MODE == 0 && ((p.setup == SHARK_SETUP_DISK_POLAR && disk_inloop_cell<float, float>(p, u, gx, gy, dt)) ||
                          (p.setup == SHARK_SETUP_DISK_CART && cdisk_inloop_cell<float>(p, u, gx, gy)))) {
            in_regs = false;
            rho = u[cc + (0) * pl];
            px = u[cc + (1) * pl];
            py = u[cc + (2) * pl];
            pz = u[cc + (3) * pl];
        }
        // ---- courant on the final state (src/solver/courant.f90:11-124), FP32 ----------------------
        const float cfl = p.f_cfl;
        const float irho = 1.0f / rho;
        const float vx = px * irho, vy = py * irho, vz = pz * irho;
        float cs;
        if (p.iso == 1) cs = p.ccs ? p.ccs[cc] : p.cs[gx];
        else {
            const float E = u[cc + (4) * pl];
            const float ekin = 0.5f * rho * (vx * vx) + 0.5f * rho * (vy * vy) + 0.5f * rho * (vz * vz);
            const float P = fmaxf(p.f_gm1 * (E - ekin), p.f_smallp);
            cs = sqrtf(p.f_gamma * P / fmaxf(rho, p.f_smallr));
            if (!(E == E)) st |= SHARK_STATUS_NAN;
        }
        float dxx;
        if (p.ndim == 1) dxx = p.dx1[gx];
        else if (p.geom == 2) dxx = fminf(p.dx1[gx], p.radc[gx] * p.dx2[gx]);
        else dxx = fminf(p.dx1[gx], p.dx2[gx]);
        float vv = fabsf(vx) + fabsf(vy) + fabsf(vz);
        float vmax = cs + vv;
        float fmx = 0.f;
        const bool fk = fk_si || ((p.flags & SHARK_FLAG_FORCE_KICK) != 0 &&
                                  (p.setup == SHARK_SETUP_DISK_POLAR || p.setup == SHARK_SETUP_DISK_CART));
        const float om = p.f_si_om, qsh = p.f_si_q;
        float fmx2 = 0.f;                 // SI: the largest |f|^2, one square root after the loop
        if (fk_si) {
            const float f1 = 2.0f * qsh * (om * om) * xc - 2.0f * om * vz - 2.0f * p.f_si_r0 * om * p.f_si_eta;
            const float f3 = 2.0f * om * vx;
            fmx2 = f1 * f1 + f3 * f3;
        } else if (fk && p.setup == SHARK_SETUP_DISK_CART) {   // the star's softened force, gas and dust
            fmx = sqrtf(p.cfx[cc] * p.cfx[cc] + p.cfy[cc] * p.cfy[cc]);
        } else if (fk) {
            fmx = fabsf(p.fgrav[gx]);   // polar disk: the point-mass force, the same on gas and dust
        }
        if (cfl_done) {   // dust terms taken in the drag loop: the same maxima, the last species' vv
            vmax = fmaxf(vmax, vmax_d);
            fmx2 = fmaxf(fmx2, fmx2_d);
            vv = vv_last;
        } else {
#pragma unroll
        for (int k = 0; k < N; ++k) {
            float rd, mx, my, mz;
            if (NS > 0 && in_regs) {
                rd = dr[k < NMAX ? k : 0]; mx = dmx[k < NMAX ? k : 0]; my = dmy[k < NMAX ? k : 0]; mz = dmz[k < NMAX ? k : 0];
            } else {
                rd = u[cc + (5 + k) * pl];
                mx = u[cc + (5 + N + k) * pl];
                my = u[cc + (5 + 2 * N + k) * pl];
                mz = u[cc + (5 + 3 * N + k) * pl];
            }
            const float ird = 1.0f / rd;
            const float vdx = mx * ird;
            const float vdy = my * ird;
            const float vdz = mz * ird;
            vv = fabsf(vdx) + fabsf(vdy) + fabsf(vdz);
            vmax = fmaxf(vmax, vv);
            if (fk_si) {
                const float f1 = 2.0f * qsh * (om * om) * xc - 2.0f * om * vdz;
                const float f3 = 2.0f * om * vdx;
                fmx2 = fmaxf(fmx2, f1 * f1 + f3 * f3);
            }
            if (!(rd > 0.f)) st |= SHARK_STATUS_NEG_DENSITY;
            if (!isfinite(vv)) st |= SHARK_STATUS_NAN;
        }
        }
        if (fk_si) fmx = sqrtf(fmx2);
        dtc = cfl * dxx / fabsf(vmax);
        if (fk && vv != 0.f) {
            const float fratio = fmaxf(fmx * dxx / (vv * vv), 1e-3f);
            dtc = fminf(dtc, cfl * dxx / vv * (sqrtf(1.0f + 2.0f * cfl * fratio) - 1.0f) / fratio);
        }
        if (!(rho > 0.f)) st |= SHARK_STATUS_NEG_DENSITY;
        if (!isfinite(vx) || !isfinite(vy) || !isfinite(vz)) st |= SHARK_STATUS_NAN;
        if (!(dtc > 0.f) || !isfinite(dtc)) { st |= SHARK_STATUS_DT_UNDERFLOW; dtc = 2e38f; }
    };
    if constexpr (GROW && MODE == 0) {   // dust_growth (solve.f90:113) between the two parts
        if (act) part1();
        if (p.gw.mode & SHARK_GROWTH_FRAGMENTATION) {
            if (act) st |= grow_in_finalize(p, u, gx, gy, dt);
        } else {
            __syncthreads();             // the block's cells after the drag
            st |= grow_block_warps(p, blockIdx.x * blockDim.x + p.ng, gy, dt);
            __syncthreads();
        }
        if (act) part2();
    } else if (act) {
        part1();
        part2();
    }
    block_reduce_dt_f(dtc, st, p.dt_next, p.status);
    if (MODE == 0 && gx < p.ng + p.nx) fill_ghost_images(p, p.u_next, gx, gy);
}

// Per-step preparation, one small block before the flux kernels: reset the next-dt slot and,
// when the stopping times are per-species constants (SI box), compute the stiff drag
// coefficients 1/(1+a_k) and a_k/(1+a_k), a_k = dt/t_k, once in FP64 (dust_drag.f90:29-46).
__device__ __forceinline__ double hash_uniform_d(unsigned long long seed, unsigned long long counter) {
    unsigned long long z = seed * 0x9E3779B97F4A7C15ull + counter + 0x632BE59BD9B4E019ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z = z ^ (z >> 31);
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

// Ornstein-Uhlenbeck update of the forcing coefficients for step `step` (one thread each):
// c <- f c + sigma sqrt(1 - f^2) xi with f = exp(-dt/tcorr) and a Box-Muller normal deviate.
static __global__ void k_ou_update(double* ou, int nm, const double* dt, double sigma, double tcorr,
                                   unsigned long long seed, long long step) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= 2 * nm) return;
    const double f = exp(-(*dt) / tcorr);
    const double sg = sigma * sqrt(1.0 - f * f);
    const unsigned long long cnt = (unsigned long long)(step * nm + q / 2) * 2 + (q & 1);
    const double u1 = hash_uniform_d(seed, 2 * cnt), u2 = hash_uniform_d(seed, 2 * cnt + 1);
    const double xi = sqrt(-2.0 * log(1.0 - u1)) * cos(2.0 * 3.141592653589793238462643383279 * u2);
    ou[q] = f * ou[q] + sg * xi;
}

static __global__ void k_prepare_step(unsigned long long* dt_next, const double* dt, const double* dtstop, int ndust,
                                      int const_ts, float* coef, double* dt_log) {
    const int k = threadIdx.x;
    if (k == 0) {
        *dt_next = (unsigned long long)__double_as_longlong(2e44);
        coef[2 * SHARK_MAX_DUST] = (float)*dt;
        if (dt_log) *dt_log = *dt;
    }
    if (const_ts && k < ndust) {
        float r, w;
        drag_coeffs(1.0 * (*dt) / dtstop[k], r, w);
        coef[k] = r;
        coef[SHARK_MAX_DUST + k] = w;
    }
}

// ---------------------------------------------------------------------------------------------
// Layout conversion between the caller's Fortran-order FP64 array and the device state.
// ---------------------------------------------------------------------------------------------
template <typename R>
__global__ void k_from_fortran(const double* __restrict__ src, R* __restrict__ dst, int nx_max, int ny_max,
                               int pitch, long long plane, int nvar) {
    const long long ncells = (long long)nx_max * ny_max;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= ncells * nvar) return;
    const int v = (int)(t / ncells);
    const long long i = t - v * ncells;
    const int iy = (int)(i / nx_max), ix = (int)(i - (long long)iy * nx_max);
    dst[v * plane + (long long)iy * pitch + ix] = R(src[t]);
}

template <typename R>
__global__ void k_to_fortran(const R* __restrict__ src, double* __restrict__ dst, int nx_max, int ny_max,
                             int pitch, long long plane, int nvar) {
    const long long ncells = (long long)nx_max * ny_max;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= ncells * nvar) return;
    const int v = (int)(t / ncells);
    const long long i = t - v * ncells;
    const int iy = (int)(i / nx_max), ix = (int)(i - (long long)iy * nx_max);
    dst[t] = (double)src[v * plane + (long long)iy * pitch + ix];
}

// ctoprim of the whole device state into a Fortran-order FP64 q and cs (solve.f90:195-253).
template <typename R>
__global__ void k_ctoprim(KParams<R> p, const R* __restrict__ u, double* __restrict__ q, double* __restrict__ cs) {
    const long long ncells = (long long)p.nx_max * p.ny_max;
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= ncells) return;
    const int iy = (int)(i / p.nx_max), ix = (int)(i - (long long)iy * p.nx_max);
    const int N = p.ndust;
    const double rho = (double)u[uidx(p, 0, iy, ix)];
    const double px = (double)u[uidx(p, 1, iy, ix)], py = (double)u[uidx(p, 2, iy, ix)], pz = (double)u[uidx(p, 3, iy, ix)];
    q[0 * ncells + i] = rho > p.smallr ? rho : p.smallr;
    q[1 * ncells + i] = px / rho;
    q[2 * ncells + i] = py / rho;
    q[3 * ncells + i] = pz / rho;
    const double ekin = 0.5 * rho * ((px / rho) * (px / rho)) + 0.5 * rho * ((py / rho) * (py / rho)) +
                        0.5 * rho * ((pz / rho) * (pz / rho));
    double P = (p.gamma - 1.0) * ((double)u[uidx(p, 4, iy, ix)] - ekin - 0.0);
    P = P > p.smallp ? P : p.smallp;
    double c;
    if (p.iso == 1) { c = p.csd[ix]; P = rho * (c * c); }
    else c = sqrt(p.gamma * P / q[0 * ncells + i]);
    q[4 * ncells + i] = P;
    if (cs) cs[i] = c;
    for (int k = 0; k < N; ++k) {
        const double rd = (double)u[uidx(p, 5 + k, iy, ix)];
        q[(5 + k) * ncells + i] = rd;
        q[(5 + N + k) * ncells + i] = (double)u[uidx(p, 5 + N + k, iy, ix)] / rd;
        q[(5 + 2 * N + k) * ncells + i] = (double)u[uidx(p, 5 + 2 * N + k, iy, ix)] / rd;
        q[(5 + 3 * N + k) * ncells + i] = (double)u[uidx(p, 5 + 3 * N + k, iy, ix)] / rd;
    }
}

// ---------------------------------------------------------------------------------------------
// Kahan-compensated FP64 totals per species (deterministic two-level tree).
// Stage 1: each block Kahan-sums a contiguous range of active cells for all 4*(N+1) sums.
// Stage 2: one block combines the per-block (sum, compensation) pairs in a fixed order.
// ---------------------------------------------------------------------------------------------
template <typename R>
__global__ void k_totals_stage1(KParams<R> p, const R* __restrict__ u, double* __restrict__ part, long long per_block) {
    const int S = p.ndust + 1;
    const long long nact = (long long)p.nx * (p.ndim == 2 ? p.ny : 1);
    const long long b0 = blockIdx.x * per_block;
    const long long b1 = min(nact, b0 + per_block);
    // one quantity per thread group: threads stride over the 4*S quantities
    for (int qi = threadIdx.x; qi < 4 * S; qi += blockDim.x) {
        const int s = qi / 4, c = qi % 4;
        const int v = svar(s, c, p.ndust);
        double sum = 0.0, comp = 0.0;
        for (long long a = b0; a < b1; ++a) {
            const int iy = (p.ndim == 2) ? (int)(a / p.nx) + p.ng : 0;
            const int ix = (int)(a % p.nx) + p.ng;
            const double y = (double)u[uidx(p, v, iy, ix)] - comp;
            const double t = sum + y;
            comp = (t - sum) - y;
            sum = t;
        }
        part[(blockIdx.x * (long long)(4 * S) + qi) * 2 + 0] = sum;
        part[(blockIdx.x * (long long)(4 * S) + qi) * 2 + 1] = comp;
    }
}

static __global__ void k_totals_stage2(const double* __restrict__ part, int nblocks, int nq, double* __restrict__ out) {
    for (int qi = threadIdx.x; qi < nq; qi += blockDim.x) {
        double sum = 0.0, comp = 0.0;
        for (int b = 0; b < nblocks; ++b) {
            // add the block's sum minus its own compensation, compensated
            const double y = (part[((long long)b * nq + qi) * 2 + 0] - part[((long long)b * nq + qi) * 2 + 1]) - comp;
            const double t = sum + y;
            comp = (t - sum) - y;
            sum = t;
        }
        out[qi] = sum;
    }
}

}  // namespace shark
