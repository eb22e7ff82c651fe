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
    // per-column metrics in FP64 (courant, drag)
    const double *dx1d, *dx2d, *radcd, *xposd, *csd;
    // per-species constants
    const double *dK, *dtstop, *dsize;
    // time step bookkeeping
    const double* dt;                 // dt of the current step
    unsigned long long* dt_next;      // bit image of the next dt (positive doubles order as u64)
    unsigned int* status;             // SHARK_STATUS_* bits
    const R* u_cur;                   // state at the start of the step (read only)
    R* u_next;                        // state after the step
};

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

// ---------------------------------------------------------------------------------------------
// K1: fused MUSCL-Hancock flux/update, one CTA per (tile, species)
// ---------------------------------------------------------------------------------------------
template <int NDIM> struct Tile;
template <> struct Tile<2> {
    static constexpr int TX = 32, TY = 8;
    static constexpr int HX = TX + 4, HY = TY + 4, OX = 2, OY = 2;   // halo tile and origin offset
    static constexpr int RX = TX + 2, RY = TY + 2;                    // predicted ring region
    static constexpr int NT = TX * TY;
};
template <> struct Tile<1> {
    static constexpr int TX = 128, TY = 1;
    static constexpr int HX = TX + 4, HY = 1, OX = 2, OY = 0;
    static constexpr int RX = TX + 2, RY = 1;
    static constexpr int NT = TX;
};

template <typename R, int NDIM>
struct TileSmem {
    using T = Tile<NDIM>;
    static constexpr int NV = 5;   // sized for the gas (dust uses the first 4 slots)
    static constexpr size_t halo = (size_t)T::HX * T::HY;
    static constexpr size_t ring = (size_t)T::RX * T::RY;
    static constexpr size_t fxn = (size_t)(T::TX + 1) * T::TY;
    static constexpr size_t fyn = (NDIM == 2) ? (size_t)T::TX * (T::TY + 1) : 0;
    static constexpr size_t n_u = NV * halo, n_q = NV * halo, n_cs = halo;
    static constexpr size_t n_face = NV * ring;   // each of qm_x, qp_x, qm_y, qp_y
    static constexpr size_t n_fx = NV * fxn, n_fy = NV * fyn;
    static constexpr size_t elems = n_u + n_q + n_cs + (NDIM == 2 ? 4 : 2) * n_face + n_fx + n_fy;
    static constexpr size_t bytes = elems * sizeof(R);
};

// Force of the setup on a gas (s == 0) or dust (s > 0) element with primitive velocities
// (vx, vy, vz) at column ix: update_force_setup of SI (src/setups/SI/setup.f90:335-368).  The
// other in-scope setups have no force.  `drag` is on for every configuration that uses the force
// (the !drag extra terms are rejected at init).
template <typename R>
__device__ __forceinline__ void setup_force(const KParams<R>& p, int s, int ix, R vx, R vz, R& f1, R& f2, R& f3) {
    if (p.setup == SHARK_SETUP_SI) {
        const R qs = R(p.si_q), om = R(p.si_om);
        const R xc = p.xpos[ix] - R(0.5) * R(p.box_l);
        if (s == 0)
            f1 = R(2) * qs * sq(om) * xc - R(2) * om * vz - R(2) * R(p.si_r0) * om * R(p.si_eta);
        else
            f1 = R(2) * qs * sq(om) * xc - R(2) * om * vz;
        f2 = R(0);
        f3 = R(2) * om * vx;
    } else {
        f1 = f2 = f3 = R(0);
    }
}

// One species of one tile.  IS_GAS selects the 5-variable gas (solver per p.solver) or a
// 4-variable pressureless dust species (solver per p.solverdust).
template <typename R, int NDIM, bool IS_GAS>
__device__ void flux_tile(const KParams<R>& p, int s, R* sm) {
    using T = Tile<NDIM>;
    using S = TileSmem<R, NDIM>;
    constexpr int NV = IS_GAS ? 5 : 4;
    const int N = p.ndust;
    const int tid = threadIdx.x;
    const int ax0 = blockIdx.x * T::TX + p.ng;                     // first active column of tile
    const int ay0 = (NDIM == 2) ? blockIdx.y * T::TY + p.ng : 0;   // first active row of tile
    const int hx0 = ax0 - T::OX, hy0 = ay0 - T::OY;                 // halo origin (global)
    const R dt = R(*p.dt);
    const R half = R(0.5);
    const R gamma = R(p.gamma);
    const bool fk = (p.flags & SHARK_FLAG_FORCE_KICK) != 0;
    const bool polar = (p.geom == 2);
    const bool iso = (p.iso == 1);

    R* us = sm;                       // [NV][HY][HX] conserved
    R* qs = us + S::n_u;              // [NV][HY][HX] primitive
    R* css = qs + S::n_q;             // [HY][HX] sound speed (gas)
    R* qmx = css + S::n_cs;           // [NV][RY][RX] right-face state in x  (qm(:,:,1))
    R* qpx = qmx + S::n_face;         // [NV][RY][RX] left-face state in x   (qp(:,:,1))
    R* qmy = qpx + S::n_face;         // y faces (2D only)
    R* qpy = (NDIM == 2) ? qmy + S::n_face : qmy;
    R* fxs = (NDIM == 2) ? qpy + S::n_face : qmy;  // [NV][TY][TX+1]
    R* fys = fxs + S::n_fx;                        // [NV][TY+1][TX]

    // ---- stage the halo tile of this species (coalesced rows) ------------------------------
    for (int idx = tid; idx < NV * T::HY * T::HX; idx += T::NT) {
        const int c = idx / (T::HY * T::HX);
        const int r = idx - c * (T::HY * T::HX);
        const int hy = r / T::HX, hx = r - hy * T::HX;
        const int gx = hx0 + hx, gy = hy0 + hy;
        R val = R(0);
        if (gx < p.nx_max && gy < p.ny_max) val = p.u_cur[uidx(p, svar(s, c, N), gy, gx)];
        us[idx] = val;
    }
    __syncthreads();

    // ---- ctoprim on the halo tile (src/solver/solve.f90:195-253) ---------------------------
    for (int r = tid; r < T::HY * T::HX; r += T::NT) {
        const int hx = r % T::HX;
        const int gx = min(hx0 + hx, p.nx_max - 1);
        if (IS_GAS) {
            const R rho = us[0 * S::halo + r];
            const R px = us[1 * S::halo + r], py = us[2 * S::halo + r], pz = us[3 * S::halo + r];
            qs[0 * S::halo + r] = fmax2(rho, R(p.smallr));
            qs[1 * S::halo + r] = px / rho;
            qs[2 * S::halo + r] = py / rho;
            qs[3 * S::halo + r] = pz / rho;
            const R ekin = half * rho * sq(px / rho) + half * rho * sq(py / rho) + half * rho * sq(pz / rho);
            R P = fmax2((gamma - R(1)) * (us[4 * S::halo + r] - ekin - R(0)), R(p.smallp));
            R cs;
            if (!iso) cs = sqrt(gamma * P / qs[0 * S::halo + r]);
            else { cs = p.cs[gx]; P = rho * sq(cs); }
            qs[4 * S::halo + r] = P;
            css[r] = cs;
        } else {
            const R rd = us[0 * S::halo + r];
            qs[0 * S::halo + r] = rd;
            qs[1 * S::halo + r] = us[1 * S::halo + r] / rd;
            qs[2 * S::halo + r] = us[2 * S::halo + r] / rd;
            qs[3 * S::halo + r] = us[3 * S::halo + r] / rd;
        }
    }
    __syncthreads();

    // ---- predictor on the ring region (src/solver/godunov.f90:7-629) -----------------------
    for (int r = tid; r < T::RX * T::RY; r += T::NT) {
        const int ry = r / T::RX, rx = r - ry * T::RX;
        if (NDIM == 2 && (rx == 0 || rx == T::RX - 1) && (ry == 0 || ry == T::RY - 1)) continue;  // corners
        const int hx = rx + 1, hy = (NDIM == 2) ? ry + 1 : 0;
        const int gx = hx0 + hx;
        if (gx >= p.nx_max - 1 || (NDIM == 2 && hy0 + hy >= p.ny_max - 1)) continue;  // beyond a partial tile
        const int hc = hy * T::HX + hx;
        const R radius_polar = polar ? p.radc[gx] : R(1);
        R dqx[NV], dqy[NV];
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            const R* qc = qs + c * S::halo;
            dqx[c] = R(0);
            dqy[c] = R(0);
            if (p.slope_type > 0) {
                dqx[c] = slope_limit(p.slope_type, R(2) * (qc[hc] - qc[hc - 1]) / (p.dx1[gx] + p.dx1[gx - 1]),
                                     R(2) * (qc[hc + 1] - qc[hc]) / (p.dx1[gx + 1] + p.dx1[gx]));
                if (NDIM == 2)
                    dqy[c] = slope_limit(p.slope_type, R(2) * (qc[hc] - qc[hc - T::HX]) / (p.dx2[gx] + p.dx2[gx]),
                                         R(2) * (qc[hc + T::HX] - qc[hc]) / (p.dx2[gx] + p.dx2[gx])) /
                             radius_polar;
            }
        }
        R r_rho = qs[0 * S::halo + hc];
        R u = qs[1 * S::halo + hc], v = qs[2 * S::halo + hc], w = qs[3 * S::halo + hc];
        const R drx = dqx[0], dux = dqx[1], dvx = dqx[2], dwx = dqx[3];
        const R dry = dqy[0], duy = dqy[1], dvy = dqy[2], dwy = dqy[3];
        R f1, f2, f3;
        if (fk) {
            // update_force_setup only writes active cells; ghost cells keep force = 0
            // (src/setups/SI/setup.f90:339-340, the array is zeroed in allocate_init.f90:271)
            const int gy = hy0 + hy;
            const bool active = gx >= p.ng && gx < p.ng + p.nx && (NDIM == 1 || (gy >= p.ng && gy < p.ng + p.ny));
            if (active) setup_force(p, s, gx, u, w, f1, f2, f3);
            else f1 = f2 = f3 = R(0);
            u = u + f1 * half * dt;
            v = v + f2 * half * dt;
            w = w + f3 * half * dt;
        }
        R sr0 = -u * drx - v * dry - (dux + dvy) * r_rho;
        R su0, sv0, sw0;
        R face[NV][4];   // [c][qm_x, qp_x, qm_y, qp_y]
        const R dxl = p.dx1[gx];
        const R dyl = radius_polar * p.dx2[gx];
        if (IS_GAS) {
            const R csi = css[hc];
            R pp = qs[4 * S::halo + hc];
            R dpx = dqx[4], dpy = dqy[4];
            if (iso) {
                pp = qs[0 * S::halo + hc] * sq(csi);
                dpx = dqx[0] * sq(csi);
                if (NDIM == 2) dpy = dqy[0] * sq(csi);
            }
            R sp0 = -u * dpx - v * dpy - (dux + dvy) * gamma * pp;
            su0 = -u * dux - v * duy - (dpx) / r_rho;
            sv0 = -u * dvx - v * dvy - (dpy) / r_rho;
            sw0 = -u * dwx - v * dwy;
            if (polar) {
                sr0 = -u * drx - v * dry - (dux + dvy) * r_rho - r_rho * u / radius_polar;
                sp0 = -u * dpx - v * dpy - (dux + dvy) * gamma * pp - gamma * pp * u / radius_polar;
                su0 = -u * dux - v * duy - (dpx) / r_rho + (sq(v)) / radius_polar;
                sv0 = -u * dvx - v * dvy - (dpy) / r_rho - u * v / radius_polar;
                sw0 = -u * dwx - v * dwy;
            }
            const R smallP = R(p.smallp);
            face[0][0] = r_rho + half * dt * sr0 + half * drx * dxl;
            face[1][0] = u + half * dt * su0 + half * dux * dxl;
            face[4][0] = fmax2(pp + half * dt * sp0 + half * dpx * dxl, smallP);
            face[2][0] = v + half * dt * sv0 + half * dvx * dxl;
            face[3][0] = w + half * dt * sw0 + half * dwx * dxl;
            face[0][1] = r_rho + half * dt * sr0 - half * drx * dxl;
            face[1][1] = u + half * dt * su0 - half * dux * dxl;
            face[4][1] = fmax2(pp + half * dt * sp0 - half * dpx * dxl, smallP);
            face[2][1] = v + half * dt * sv0 - half * dvx * dxl;
            face[3][1] = w + half * dt * sw0 - half * dwx * dxl;
            if (NDIM == 2) {
                face[0][2] = r_rho + half * dt * sr0 + half * dry * dyl;
                face[1][2] = u + half * dt * su0 + half * duy * dyl;
                face[4][2] = fmax2(pp + half * dt * sp0 + half * dpy * dyl, smallP);
                face[2][2] = v + half * dt * sv0 + half * dvy * dyl;
                face[3][2] = w + half * dt * sw0 + half * dwy * dyl;
                face[0][3] = r_rho + half * dt * sr0 - half * dry * dyl;
                face[1][3] = u + half * dt * su0 - half * duy * dyl;
                face[4][3] = fmax2(pp + half * dt * sp0 - half * dpy * dyl, smallP);
                face[2][3] = v + half * dt * sv0 - half * dvy * dyl;
                face[3][3] = w + half * dt * sw0 - half * dwy * dyl;
            }
            if (iso) {   // godunov.f90:606-611
#pragma unroll
                for (int d = 0; d < (NDIM == 2 ? 4 : 2); ++d) face[4][d] = sq(csi) * face[0][d];
            }
        } else {
            su0 = -u * dux - v * duy;
            sv0 = -u * dvx - v * dvy;
            sw0 = -u * dwx - v * dwy;
            if (polar) {
                sr0 = sr0 - r_rho * u / radius_polar;
                su0 = su0 + sq(v) / radius_polar;
                sv0 = sv0 - u * v / radius_polar;
            }
            face[0][0] = r_rho + half * dt * sr0 + half * drx * dxl;
            face[1][0] = u + half * dt * su0 + half * dux * dxl;
            face[2][0] = v + half * dt * sv0 + half * dvx * dxl;
            face[3][0] = w + half * dt * sw0 + half * dwx * dxl;
            face[0][1] = r_rho + half * dt * sr0 - half * drx * dxl;
            face[1][1] = u + half * dt * su0 - half * dux * dxl;
            face[2][1] = v + half * dt * sv0 - half * dvx * dxl;
            face[3][1] = w + half * dt * sw0 - half * dwx * dxl;
            if (NDIM == 2) {
                face[0][2] = r_rho + half * dt * sr0 + half * dry * dyl;
                face[1][2] = u + half * dt * su0 + half * duy * dyl;
                face[2][2] = v + half * dt * sv0 + half * dvy * dyl;
                face[3][2] = w + half * dt * sw0 + half * dwy * dyl;
                face[0][3] = r_rho + half * dt * sr0 - half * dry * dyl;
                face[1][3] = u + half * dt * su0 - half * duy * dyl;
                face[2][3] = v + half * dt * sv0 - half * dvy * dyl;
                face[3][3] = w + half * dt * sw0 - half * dwy * dyl;
            }
        }
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            qmx[c * S::ring + r] = face[c][0];
            qpx[c * S::ring + r] = face[c][1];
            if (NDIM == 2) {
                qmy[c * S::ring + r] = face[c][2];
                qpy[c * S::ring + r] = face[c][3];
            }
        }
    }
    __syncthreads();

    // ---- Riemann fluxes (godunov.f90:659-722, solve_wrapper :768-833) ----------------------
    // x faces: face fx (0..TX) of tile row fy sits between ring cells (fx, ry) and (fx+1, ry).
    for (int f = tid; f < (T::TX + 1) * T::TY; f += T::NT) {
        const int fy = f / (T::TX + 1), fx = f - fy * (T::TX + 1);
        const int ry = (NDIM == 2) ? fy + 1 : 0;
        const int rl = ry * T::RX + fx, rr = rl + 1;
        const int gxl = hx0 + fx + 1;   // global column of the left cell
        if (gxl + 1 > p.nx_max - 2) continue;
        R fl[NV];
        if (IS_GAS) {
            R csl, csr;
            const R rl0 = qmx[0 * S::ring + rl], rr0 = qpx[0 * S::ring + rr];
            const R pl = qmx[4 * S::ring + rl], pr = qpx[4 * S::ring + rr];
            if (iso) {
                const int hy = (NDIM == 2) ? ry + 1 : 0;
                csl = css[hy * T::HX + fx + 1];
                csr = css[hy * T::HX + fx + 2];
            } else {
                csl = sqrt(gamma * pl / rl0);
                csr = sqrt(gamma * pr / rr0);
            }
            GasFlux<R> g;
            const R ul = qmx[1 * S::ring + rl], vl = qmx[2 * S::ring + rl], wl = qmx[3 * S::ring + rl];
            const R ur = qpx[1 * S::ring + rr], vr = qpx[2 * S::ring + rr], wr = qpx[3 * S::ring + rr];
            if (p.solver == 2) g = gas_hllc(gamma, rl0, ul, vl, wl, pl, rr0, ur, vr, wr, pr, csl, csr);
            else if (p.solver == 1) g = gas_hll(gamma, rl0, ul, vl, wl, pl, rr0, ur, vr, wr, pr, csl, csr);
            else g = gas_llf(gamma, rl0, ul, vl, wl, pl, rr0, ur, vr, wr, pr, csl, csr);
            fl[0] = g.rho; fl[1] = g.mn; fl[2] = g.mt; fl[3] = g.mz; fl[4] = g.e;
        } else {
            DustFlux<R> d;
            const R rl0 = qmx[0 * S::ring + rl], ul = qmx[1 * S::ring + rl], vl = qmx[2 * S::ring + rl], wl = qmx[3 * S::ring + rl];
            const R rr0 = qpx[0 * S::ring + rr], ur = qpx[1 * S::ring + rr], vr = qpx[2 * S::ring + rr], wr = qpx[3 * S::ring + rr];
            if (p.solverdust == 0) d = dust_hb(rl0, ul, vl, wl, rr0, ur, vr, wr);
            else if (p.solverdust == 1) d = dust_llf(rl0, ul, vl, wl, rr0, ur, vr, wr);
            else d = dust_hll(rl0, ul, vl, wl, rr0, ur, vr, wr);
            fl[0] = d.rho; fl[1] = d.mn; fl[2] = d.mt; fl[3] = d.mz;
        }
#pragma unroll
        for (int c = 0; c < NV; ++c) fxs[c * S::fxn + f] = fl[c];
    }
    if (NDIM == 2) {
        // y faces: face fy (0..TY) of tile column fx sits between ring cells (fx+1, fy), (fx+1, fy+1)
        for (int f = tid; f < T::TX * (T::TY + 1); f += T::NT) {
            const int fy = f / T::TX, fx = f - fy * T::TX;
            const int rl = fy * T::RX + fx + 1, rr = rl + T::RX;
            const int gx = hx0 + fx + 2;
            if (gx > p.nx_max - 3 || hy0 + fy + 2 > p.ny_max - 2) continue;
            R fl[NV];
            if (IS_GAS) {
                R csl, csr;
                const R rl0 = qmy[0 * S::ring + rl], rr0 = qpy[0 * S::ring + rr];
                const R pl = qmy[4 * S::ring + rl], pr = qpy[4 * S::ring + rr];
                if (iso) {
                    csl = css[(fy + 1) * T::HX + fx + 2];
                    csr = css[(fy + 2) * T::HX + fx + 2];
                } else {
                    csl = sqrt(gamma * pl / rl0);
                    csr = sqrt(gamma * pr / rr0);
                }
                // idim = 2: normal velocity vy, transverse vx (index_vn/vt, allocate_init.f90:249-252)
                const R ul = qmy[2 * S::ring + rl], vl = qmy[1 * S::ring + rl], wl = qmy[3 * S::ring + rl];
                const R ur = qpy[2 * S::ring + rr], vr = qpy[1 * S::ring + rr], wr = qpy[3 * S::ring + rr];
                GasFlux<R> g;
                if (p.solver == 2) g = gas_hllc(gamma, rl0, ul, vl, wl, pl, rr0, ur, vr, wr, pr, csl, csr);
                else if (p.solver == 1) g = gas_hll(gamma, rl0, ul, vl, wl, pl, rr0, ur, vr, wr, pr, csl, csr);
                else g = gas_llf(gamma, rl0, ul, vl, wl, pl, rr0, ur, vr, wr, pr, csl, csr);
                fl[0] = g.rho; fl[2] = g.mn; fl[1] = g.mt; fl[3] = g.mz; fl[4] = g.e;
            } else {
                const R rl0 = qmy[0 * S::ring + rl], ul = qmy[2 * S::ring + rl], vl = qmy[1 * S::ring + rl], wl = qmy[3 * S::ring + rl];
                const R rr0 = qpy[0 * S::ring + rr], ur = qpy[2 * S::ring + rr], vr = qpy[1 * S::ring + rr], wr = qpy[3 * S::ring + rr];
                DustFlux<R> d;
                if (p.solverdust == 0) d = dust_hb(rl0, ul, vl, wl, rr0, ur, vr, wr);
                else if (p.solverdust == 1) d = dust_llf(rl0, ul, vl, wl, rr0, ur, vr, wr);
                else d = dust_hll(rl0, ul, vl, wl, rr0, ur, vr, wr);
                fl[0] = d.rho; fl[2] = d.mn; fl[1] = d.mt; fl[3] = d.mz;
            }
#pragma unroll
            for (int c = 0; c < NV; ++c) fys[c * S::fyn + f] = fl[c];
        }
    }
    __syncthreads();

    // ---- kick + conservative update + local source terms, one thread per active cell ----------
    {
        const int cy = tid / T::TX, cx = tid - cy * T::TX;
        const int gx = ax0 + cx, gy = ay0 + cy;
        if (gx >= p.ng + p.nx || (NDIM == 2 && gy >= p.ng + p.ny)) return;
        const int hc = (cy + T::OY) * T::HX + cx + T::OX;
        R uu[NV];
#pragma unroll
        for (int c = 0; c < NV; ++c) uu[c] = us[c * S::halo + hc];
        if (fk) {   // kick(1.0) (src/solver/force_kicks.f90:2-41) before the flux update
            R f1, f2, f3;
            setup_force(p, s, gx, qs[1 * S::halo + hc], qs[3 * S::halo + hc], f1, f2, f3);
            const R rho = uu[0];
            if (IS_GAS) {
                const R eo = half * sq(uu[1]) / rho + half * sq(uu[2]) / rho + half * sq(uu[3]) / rho;
                uu[1] = uu[1] + rho * R(1) * dt * f1;
                uu[2] = uu[2] + rho * R(1) * dt * f2;
                uu[3] = uu[3] + rho * R(1) * dt * f3;
                const R en = half * sq(uu[1]) / rho + half * sq(uu[2]) / rho + half * sq(uu[3]) / rho;
                uu[4] = uu[4] + (en - eo);
            } else {
                uu[1] = uu[1] + rho * R(1) * dt * f1;
                uu[2] = uu[2] + rho * R(1) * dt * f2;
                uu[3] = uu[3] + rho * R(1) * dt * f3;
            }
        }
        const R s1l = p.surf1[gx], s1r = p.surf1[gx + 1], vol = p.vol[gx];
        const int fxl = cy * (T::TX + 1) + cx;
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            const R* F = fxs + c * S::fxn;
            if (NDIM == 1) {
                uu[c] = uu[c] + (F[fxl] * s1l - F[fxl + 1] * s1r) / vol * dt;
            } else {
                const R* G = fys + c * S::fyn;
                const R s2 = p.surf2[gx];
                uu[c] = uu[c] + (F[fxl] * s1l - F[fxl + 1] * s1r) / vol * dt +
                        (G[cy * T::TX + cx] * s2 - G[(cy + 1) * T::TX + cx] * s2) / vol * dt;
            }
        }
        if (polar) {   // Source_terms, GEOM==2 (src/solver/source_terms.f90:37-47), on the OLD q
            const R rc = p.radc[gx];
            const R qr = qs[0 * S::halo + hc], qvx = qs[1 * S::halo + hc], qvy = qs[2 * S::halo + hc];
            if (IS_GAS) {
                uu[1] = uu[1] + dt * (qr * sq(qvy) + qs[4 * S::halo + hc]) / rc;
                uu[2] = uu[2] + (R(0) - dt * (qr * qvy * qvx / rc));
            } else {
                uu[1] = uu[1] + dt * (qr * sq(qvy) / rc);
                uu[2] = uu[2] + (R(0) - dt * (qr * qvy * qvx / rc));
            }
        }
#pragma unroll
        for (int c = 0; c < NV; ++c) p.u_next[uidx(p, svar(s, c, N), gy, gx)] = uu[c];
    }
}

template <typename R, int NDIM>
__global__ void __launch_bounds__(Tile<NDIM>::NT) k_flux(KParams<R> p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* sm = reinterpret_cast<R*>(smem_raw);
    const int s = blockIdx.z;
    if (s == 0) flux_tile<R, NDIM, true>(p, 0, sm);
    else flux_tile<R, NDIM, false>(p, s, sm);
}

// ---------------------------------------------------------------------------------------------
// K2: drag + floor + inloop + status + next-step CFL dt, one thread per active cell.
// NS > 0: compile-time species count (register arrays); NS < 0: run-time count.
// MODE 0: full finalize; MODE 1: dt only (first step after an upload).
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ void atomic_min_dt(unsigned long long* a, double v) {
    // positive finite doubles order like their bit patterns
    atomicMin(a, (unsigned long long)__double_as_longlong(v));
}

template <typename R, int NS, int MODE>
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
                double ts;
                if (p.setup == SHARK_SETUP_SI) {
                    ts = p.dtstop[k];                                   // SI/setup.f90:389-397
                } else if (p.setup == SHARK_SETUP_DUSTYWAVE) {
                    const double rd_old = (double)p.u_cur[uidx(p, 5 + k, gy, gx)];
                    ts = rd_old * qrho_old / p.dK[k] / (qrho_old);   // DUSTYWAVE/setup.f90:217
                } else {
                    // Epstein (SOD/setup.f90:179-185); isothermal cs only (checked at init)
                    ts = sqrt(3.141592653589793238462643383279 * p.gamma / 8.0) * (p.rhograin) * p.dsize[k] /
                         (qrho_old * p.csd[gx]);
                }
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
                else {   // run-time species count: recompute alpha_k
                    double ts;
                    if (p.setup == SHARK_SETUP_SI) ts = p.dtstop[k];
                    else if (p.setup == SHARK_SETUP_DUSTYWAVE) {
                        const double rd_old = (double)p.u_cur[uidx(p, 5 + k, gy, gx)];
                        ts = rd_old * qrho_old / p.dK[k] / (qrho_old);
                    } else
                        ts = sqrt(3.141592653589793238462643383279 * p.gamma / 8.0) * (p.rhograin) * p.dsize[k] /
                             (qrho_old * p.csd[gx]);
                    a = 1.0 * dt / ts;
                }
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
        // ---- courant on the final state (src/solver/courant.f90:11-124) -----------------------
        const double cfl = p.cfl;
        const double qrho = rho > p.smallr ? rho : p.smallr;
        const double vx = px / rho, vy = py / rho, vz = pz / rho;
        double cs;
        if (p.iso == 1) cs = p.csd[gx];
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
    // block min of dtc and OR of status
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
            atomic_min_dt(p.dt_next, dtc);
            if (st) atomicOr(p.status, st);
        }
    }
}

// Reset the next-dt slot before k_finalize runs (single thread).
static __global__ void k_reset_dt(unsigned long long* dt_next) {
    *dt_next = (unsigned long long)__double_as_longlong(2e44);
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
