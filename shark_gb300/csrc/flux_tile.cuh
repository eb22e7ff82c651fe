// flux_tile.cuh -- K1: fused MUSCL-Hancock flux/update, one CTA per (tile, species).
//
// Included by step_kernels.cuh after KParams/uidx/svar/physics.  Per CTA, for one species of one
// tile of active cells:
//   1. stage the tile plus a 2-cell halo of the species' conserved planes (coalesced row loads)
//      and convert to primitives in shared memory                 (ctoprim, solve.f90:195-253)
//   2. limited slopes + half-step predictor on the tile plus a 1-cell ring; the four face
//      states of each ring cell go to shared memory                (predictor, godunov.f90:7-629)
//   3. one Riemann solve per face of the tile                      (add_delta_u, godunov.f90:659-722)
//   4. per active cell: force kick, conservative update, local geometric sources
//                                    (kick, force_kicks.f90:2-41; godunov.f90:728-750;
//                                     source_terms.f90:37-47)
// The FP64 instantiation (FAST = false) keeps the oracle's expressions literally (divisions
// included) so it rounds identically.  The FP32 instantiation (FAST = true) is the mixed path:
// the same algorithm without per-cell divisions -- slopes use the per-column factors
// sfx = 2/(dx_i+dx_{i-1}), sfy = 1/(dx2*r) (the limiters are positively homogeneous, so the
// polar 1/r folds into the arguments), the update uses dt/vol, ctoprim one reciprocal per cell
// and HLLC/HLL one or two per face.
#pragma once

#include <type_traits>

namespace shark {

template <typename R, int NDIM> struct Tile;
template <> struct Tile<double, 2> {
    static constexpr int TX = 32, TY = 8;
    static constexpr int HX = TX + 4, HY = TY + 4, OX = 2, OY = 2;   // halo tile and origin offset
    static constexpr int RX = TX + 2, RY = TY + 2;                    // predicted ring region
    static constexpr int NT = TX * TY;
};
template <> struct Tile<float, 2> {
    static constexpr int TX = 32, TY = 16;
    static constexpr int HX = TX + 4, HY = TY + 4, OX = 2, OY = 2;
    static constexpr int RX = TX + 2, RY = TY + 2;
    static constexpr int NT = TX * TY;
};
template <typename R> struct Tile<R, 1> {
    static constexpr int TX = 128, TY = 1;
    static constexpr int HX = TX + 4, HY = 1, OX = 2, OY = 0;
    static constexpr int RX = TX + 2, RY = 1;
    static constexpr int NT = TX;
};

template <typename R, int NDIM>
struct TileSmem {
    using T = Tile<R, NDIM>;
    static constexpr int NV = 5;   // sized for the gas (dust uses the first 4 slots)
    static constexpr size_t halo = (size_t)T::HX * T::HY;
    static constexpr size_t ring = (size_t)T::RX * T::RY;
    static constexpr size_t fxn = (size_t)(T::TX + 1) * T::TY;
    static constexpr size_t fyn = (NDIM == 2) ? (size_t)T::TX * (T::TY + 1) : 0;
    static constexpr size_t n_q = NV * halo, n_cs = halo;
    static constexpr size_t n_face = NV * ring;   // each of qm_x, qp_x, qm_y, qp_y
    static constexpr size_t n_fx = NV * fxn, n_fy = NV * fyn;
    static constexpr size_t elems = n_q + n_cs + (NDIM == 2 ? 4 : 2) * n_face + n_fx + n_fy;
    static constexpr size_t bytes = elems * sizeof(R);
};

// Force of the setup on a gas (s == 0) or dust (s > 0) element with primitive velocities
// (vx, vy, vz) at column ix: update_force_setup of SI (src/setups/SI/setup.f90:335-368) and of
// the polar disk (point-mass gravity -Mstar/r^2, disk_polar/setup.f90:358-366, no planet or
// self-gravity).  SOD and DUSTYWAVE have no force.  `drag` is on for every configuration that
// uses the force (the !drag extra terms are rejected at init).
template <typename R>
__device__ __forceinline__ void setup_force(const KParams<R>& p, int s, int ix, long long cell, R vx, R vz, R& f1,
                                            R& f2, R& f3) {
    if (p.setup == SHARK_SETUP_SI) {
        const R qs = prm<R>(p.si_q, p.f_si_q), om = prm<R>(p.si_om, p.f_si_om);
        const R xc = p.xpos[ix] - prm<R>(R(0.5) * R(p.box_l), p.f_half_box_l);
        if (s == 0)
            f1 = R(2) * qs * sq(om) * xc - R(2) * om * vz - R(2) * prm<R>(p.si_r0, p.f_si_r0) * om * prm<R>(p.si_eta, p.f_si_eta);
        else
            f1 = R(2) * qs * sq(om) * xc - R(2) * om * vz;
        f2 = R(0);
        f3 = R(2) * om * vx;
    } else if (p.setup == SHARK_SETUP_DISK_POLAR) {
        f1 = p.fgrav[ix];
        f2 = f3 = R(0);
    } else if (p.setup == SHARK_SETUP_DISK_CART) {   // the star's softened gravity (disk/setup.f90)
        f1 = p.cfx[cell];
        f2 = p.cfy[cell];
        f3 = R(0);
    } else {
        f1 = f2 = f3 = R(0);
    }
}

// HLLC with one reciprocal for the star state and one for the sampled star side (mixed path).
__device__ __forceinline__ GasFlux<float> gas_hllc_fast(float inv_g1, float rho_lft, float u_lft, float v_lft,
                                                        float w_lft, float P_lft, float rho_rgt, float u_rgt,
                                                        float v_rgt, float w_rgt, float P_rgt, float csl, float csr) {
    const float E_rgt = P_rgt * inv_g1 + 0.5f * rho_rgt * (u_rgt * u_rgt + v_rgt * v_rgt + w_rgt * w_rgt);
    const float E_lft = P_lft * inv_g1 + 0.5f * rho_lft * (u_lft * u_lft + v_lft * v_lft + w_lft * w_lft);
    const float cmax = fmaxf(csl, csr);
    const float S_lft = fminf(fminf(u_lft, u_rgt) - cmax, 0.f);
    const float S_rgt = fmaxf(fmaxf(u_lft, u_rgt) + cmax, 0.f);
    const float hllc_l = rho_lft * (u_lft - S_lft);
    const float hllc_r = rho_rgt * (S_rgt - u_rgt);
    const float inv = 1.0f / (hllc_r + hllc_l);
    const float ustar = (hllc_r * u_rgt + hllc_l * u_lft + (P_lft - P_rgt)) * inv;
    const float Pstar = (hllc_r * P_lft + hllc_l * P_rgt + hllc_l * hllc_r * (u_lft - u_rgt)) * inv;
    float r_o, u_o, P_o, e_o;
    if (S_lft > 0.f) {
        r_o = rho_lft; u_o = u_lft; P_o = P_lft; e_o = E_lft;
    } else if (S_rgt <= 0.f) {
        r_o = rho_rgt; u_o = u_rgt; P_o = P_rgt; e_o = E_rgt;
    } else {
        // star side chosen by the sign of u* (solvers.f90:469-481)
        const bool left = ustar > 0.f;
        const float S = left ? S_lft : S_rgt, rho = left ? rho_lft : rho_rgt, u = left ? u_lft : u_rgt;
        const float P = left ? P_lft : P_rgt, E = left ? E_lft : E_rgt;
        const float a = 1.0f / (S - ustar);
        r_o = rho * (S - u) * a;
        u_o = ustar;
        P_o = Pstar;
        e_o = ((S - u) * E - P * u + Pstar * ustar) * a;
    }
    GasFlux<float> f;
    f.rho = r_o * u_o;
    f.mn = r_o * u_o * u_o + P_o;
    f.e = (e_o + P_o) * u_o;
    if (ustar > 0.f) { f.mt = r_o * u_o * v_lft; f.mz = r_o * u_o * w_lft; }
    else { f.mt = r_o * u_o * v_rgt; f.mz = r_o * u_o * w_rgt; }
    return f;
}

// HLL with one reciprocal (mixed path).
__device__ __forceinline__ GasFlux<float> gas_hll_fast(float inv_g1, float rho_lft, float u_lft, float v_lft,
                                                       float w_lft, float P_lft, float rho_rgt, float u_rgt,
                                                       float v_rgt, float w_rgt, float P_rgt, float csl, float csr) {
    const float E_rgt = P_rgt * inv_g1 + 0.5f * rho_rgt * (u_rgt * u_rgt + v_rgt * v_rgt + w_rgt * w_rgt);
    const float E_lft = P_lft * inv_g1 + 0.5f * rho_lft * (u_lft * u_lft + v_lft * v_lft + w_lft * w_lft);
    const float cmax = fmaxf(csl, csr);
    const float S_lft = fminf(fminf(u_lft, u_rgt) - cmax, 0.f);
    const float S_rgt = fmaxf(fmaxf(u_lft, u_rgt) + cmax, 0.f);
    const float inv = 1.0f / (S_rgt - S_lft);
    const float ss = S_rgt * S_lft;
    const float ml = rho_lft * u_lft, mr = rho_rgt * u_rgt;
    GasFlux<float> f;
    f.rho = (S_rgt * ml - S_lft * mr + ss * (rho_rgt - rho_lft)) * inv;
    f.mn = (S_rgt * (ml * u_lft + P_lft) - S_lft * (mr * u_rgt + P_rgt) + ss * (mr - ml)) * inv;
    f.mt = (S_rgt * ml * v_lft - S_lft * mr * v_rgt + ss * (rho_rgt * v_rgt - rho_lft * v_lft)) * inv;
    f.mz = (S_rgt * ml * w_lft - S_lft * mr * w_rgt + ss * (rho_rgt * w_rgt - rho_lft * w_lft)) * inv;
    f.e = (S_rgt * (E_lft + P_lft) * u_lft - S_lft * (E_rgt + P_rgt) * u_rgt + ss * (E_rgt - E_lft)) * inv;
    return f;
}

template <typename R>
__device__ __forceinline__ GasFlux<R> gas_flux(const KParams<R>& p, R gamma, R inv_g1, R rl, R ul, R vl, R wl, R pl,
                                               R rr, R ur, R vr, R wr, R pr, R csl, R csr) {
    if constexpr (std::is_same<R, float>::value) {
        if (p.solver == 2) return gas_hllc_fast(inv_g1, rl, ul, vl, wl, pl, rr, ur, vr, wr, pr, csl, csr);
        if (p.solver == 1) return gas_hll_fast(inv_g1, rl, ul, vl, wl, pl, rr, ur, vr, wr, pr, csl, csr);
        return gas_llf(gamma, rl, ul, vl, wl, pl, rr, ur, vr, wr, pr, csl, csr);
    } else {
        if (p.solver == 2) return gas_hllc(gamma, rl, ul, vl, wl, pl, rr, ur, vr, wr, pr, csl, csr);
        if (p.solver == 1) return gas_hll(gamma, rl, ul, vl, wl, pl, rr, ur, vr, wr, pr, csl, csr);
        return gas_llf(gamma, rl, ul, vl, wl, pl, rr, ur, vr, wr, pr, csl, csr);
    }
}

// Compile-time solver choice (solve_wrapper, godunov.f90:768-833) for specialised kernels.
template <int SOLVER, typename R>
__device__ __forceinline__ GasFlux<R> gas_flux_t(R gamma, R inv_g1, R rl, R ul, R vl, R wl, R pl, R rr, R ur, R vr,
                                                 R wr, R pr, R csl, R csr) {
    if constexpr (std::is_same<R, float>::value) {
        if constexpr (SOLVER == 2) return gas_hllc_fast(inv_g1, rl, ul, vl, wl, pl, rr, ur, vr, wr, pr, csl, csr);
        else if constexpr (SOLVER == 1) return gas_hll_fast(inv_g1, rl, ul, vl, wl, pl, rr, ur, vr, wr, pr, csl, csr);
        else return gas_llf(gamma, rl, ul, vl, wl, pl, rr, ur, vr, wr, pr, csl, csr);
    } else {
        if constexpr (SOLVER == 2) return gas_hllc(gamma, rl, ul, vl, wl, pl, rr, ur, vr, wr, pr, csl, csr);
        else if constexpr (SOLVER == 1) return gas_hll(gamma, rl, ul, vl, wl, pl, rr, ur, vr, wr, pr, csl, csr);
        else return gas_llf(gamma, rl, ul, vl, wl, pl, rr, ur, vr, wr, pr, csl, csr);
    }
}

// csl, csr: the gas sound speeds of the face (used by the HLLC dust solver only).
template <int SOLVERDUST, typename R>
__device__ __forceinline__ DustFlux<R> dust_flux_t(R rl, R ul, R vl, R wl, R rr, R ur, R vr, R wr, R csl, R csr) {
    if constexpr (SOLVERDUST == 0 && std::is_same<R, float>::value) return dust_hb_f(rl, ul, vl, wl, rr, ur, vr, wr);
    else if constexpr (SOLVERDUST == 0) return dust_hb(rl, ul, vl, wl, rr, ur, vr, wr);
    else if constexpr (SOLVERDUST == 1) return dust_llf(rl, ul, vl, wl, rr, ur, vr, wr);
    else if constexpr (SOLVERDUST == 2) return dust_hll(rl, ul, vl, wl, rr, ur, vr, wr);
    else return dust_hllc(rl, ul, vl, wl, rr, ur, vr, wr, csl, csr);
}

template <typename R>
__device__ __forceinline__ DustFlux<R> dust_flux(int solverdust, R rl, R ul, R vl, R wl, R rr, R ur, R vr, R wr,
                                                 R csl, R csr) {
    if (solverdust == 0) return dust_hb(rl, ul, vl, wl, rr, ur, vr, wr);
    if (solverdust == 1) return dust_llf(rl, ul, vl, wl, rr, ur, vr, wr);
    if (solverdust == 2) return dust_hll(rl, ul, vl, wl, rr, ur, vr, wr);
    return dust_hllc(rl, ul, vl, wl, rr, ur, vr, wr, csl, csr);
}

// One species of one tile.  IS_GAS selects the 5-variable gas (solver per p.solver) or a
// 4-variable pressureless dust species (solver per p.solverdust).
template <typename R, int NDIM, bool IS_GAS>
__device__ void flux_tile(const KParams<R>& p, int s, R* sm) {
    using T = Tile<R, NDIM>;
    using S = TileSmem<R, NDIM>;
    constexpr bool FAST = std::is_same<R, float>::value;
    constexpr int NV = IS_GAS ? 5 : 4;
    const int N = p.ndust;
    const int tid = threadIdx.x;
    const int ax0 = blockIdx.x * T::TX + p.ng;                     // first active column of tile
    const int ay0 = (NDIM == 2) ? blockIdx.y * T::TY + p.ng : 0;   // first active row of tile
    const int hx0 = ax0 - T::OX, hy0 = ay0 - T::OY;                 // halo origin (global)
    const R dt = step_dt(p);
    const R half = R(0.5);
    const R gamma = prm<R>(p.gamma, p.f_gamma);
    const R smallR = prm<R>(p.smallr, p.f_smallr);
    const R inv_g1 = prm<R>(1.0 / (p.gamma - 1.0), p.f_inv_g1);
    const bool fk = (p.flags & SHARK_FLAG_FORCE_KICK) != 0;
    const bool polar = (p.geom == 2);
    const bool iso = (p.iso == 1);

    R* qs = sm;                       // [NV][HY][HX] primitive
    R* css = qs + S::n_q;             // [HY][HX] sound speed (gas)
    R* qmx = css + S::n_cs;           // [NV][RY][RX] right-face state in x  (qm(:,:,1))
    R* qpx = qmx + S::n_face;         // [NV][RY][RX] left-face state in x   (qp(:,:,1))
    R* qmy = qpx + S::n_face;         // y faces (2D only)
    R* qpy = (NDIM == 2) ? qmy + S::n_face : qmy;
    R* fxs = (NDIM == 2) ? qpy + S::n_face : qmy;  // [NV][TY][TX+1]
    R* fys = fxs + S::n_fx;                        // [NV][TY+1][TX]

    // ---- 1. stage the halo tile and run ctoprim on it (solve.f90:195-253) ----------------------
    // One thread per halo cell: coalesced row loads of the NV conserved planes, primitives to smem.
    for (int r = tid; r < T::HY * T::HX; r += T::NT) {
        const int hy = r / T::HX, hx = r - hy * T::HX;
        const int gx0 = hx0 + hx, gy0 = hy0 + hy;
        const bool inside = gx0 < p.nx_max && gy0 < p.ny_max;
        const int gx = min(gx0, p.nx_max - 1);
        R us[NV];
#pragma unroll
        for (int c = 0; c < NV; ++c) us[c] = inside ? p.u_cur[uidx(p, svar(s, c, N), gy0, gx0)] : R(1);
        if (IS_GAS) {
            const R rho = us[0];
            const R px = us[1], py = us[2], pz = us[3];
            R P, vx, vy, vz;
            if constexpr (FAST) {
                const R ir = R(1) / rho;
                vx = px * ir; vy = py * ir; vz = pz * ir;
                const R ekin = half * (px * vx + py * vy + pz * vz);
                P = fmax2((gamma - R(1)) * (us[4] - ekin), prm<R>(p.smallp, p.f_smallp));
            } else {
                vx = px / rho; vy = py / rho; vz = pz / rho;
                const R ekin = half * rho * sq(px / rho) + half * rho * sq(py / rho) + half * rho * sq(pz / rho);
                P = fmax2((gamma - R(1)) * (us[4] - ekin - R(0)), prm<R>(p.smallp, p.f_smallp));
            }
            const R qrho = fmax2(rho, smallR);
            R cs;
            if (!iso) cs = sqrt(gamma * P / qrho);
            else { cs = p.cs[gx]; P = rho * sq(cs); }
            qs[0 * S::halo + r] = qrho;
            qs[1 * S::halo + r] = vx;
            qs[2 * S::halo + r] = vy;
            qs[3 * S::halo + r] = vz;
            qs[4 * S::halo + r] = P;
            css[r] = cs;
        } else {
            const R rd = us[0];
            qs[0 * S::halo + r] = rd;
            if constexpr (FAST) {
                const R ir = R(1) / rd;
                qs[1 * S::halo + r] = us[1] * ir;
                qs[2 * S::halo + r] = us[2] * ir;
                qs[3 * S::halo + r] = us[3] * ir;
            } else {
                qs[1 * S::halo + r] = us[1] / rd;
                qs[2 * S::halo + r] = us[2] / rd;
                qs[3 * S::halo + r] = us[3] / rd;
            }
        }
    }
    __syncthreads();

    // ---- 2. slopes + predictor on the ring region (godunov.f90:7-629) ----------------------------
    for (int r = tid; r < T::RX * T::RY; r += T::NT) {
        const int ry = r / T::RX, rx = r - ry * T::RX;
        if (NDIM == 2 && (rx == 0 || rx == T::RX - 1) && (ry == 0 || ry == T::RY - 1)) continue;  // corners
        const int hx = rx + 1, hy = (NDIM == 2) ? ry + 1 : 0;
        const int gx = hx0 + hx;
        if (gx >= p.nx_max - 1 || (NDIM == 2 && hy0 + hy >= p.ny_max - 1)) continue;  // beyond a partial tile
        const int hc = hy * T::HX + hx;
        R dqx[NV], dqy[NV];
        if constexpr (FAST) {
            const R fl = p.sfx[gx], fr = p.sfx[gx + 1], fy = (NDIM == 2) ? p.sfy[gx] : R(0);
#pragma unroll
            for (int c = 0; c < NV; ++c) {
                const R* qc = qs + c * S::halo;
                dqx[c] = R(0);
                dqy[c] = R(0);
                if (p.slope_type > 0) {
                    dqx[c] = slope_limit(p.slope_type, (qc[hc] - qc[hc - 1]) * fl, (qc[hc + 1] - qc[hc]) * fr);
                    if (NDIM == 2)
                        dqy[c] = slope_limit(p.slope_type, (qc[hc] - qc[hc - T::HX]) * fy, (qc[hc + T::HX] - qc[hc]) * fy);
                }
            }
        } else {
            const R radius_polar = polar ? p.radc[gx] : R(1);
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
        }
        R r_rho = qs[0 * S::halo + hc];
        R u = qs[1 * S::halo + hc], v = qs[2 * S::halo + hc], w = qs[3 * S::halo + hc];
        const R drx = dqx[0], dux = dqx[1], dvx = dqx[2], dwx = dqx[3];
        const R dry = dqy[0], duy = dqy[1], dvy = dqy[2], dwy = dqy[3];
        if (fk) {
            // update_force_setup only writes active cells; ghost cells keep force = 0
            // (src/setups/SI/setup.f90:339-340, the array is zeroed in allocate_init.f90:271)
            R f1, f2, f3;
            const int gy = hy0 + hy;
            const bool active = gx >= p.ng && gx < p.ng + p.nx && (NDIM == 1 || (gy >= p.ng && gy < p.ng + p.ny));
            if (active) setup_force(p, s, gx, gx, u, w, f1, f2, f3);
            else f1 = f2 = f3 = R(0);
            u = u + f1 * half * dt;
            v = v + f2 * half * dt;
            w = w + f3 * half * dt;
        }
        // 1/r of the polar geometric terms (the FP64 path divides, the FP32 path multiplies)
        const R rp = polar ? (FAST ? p.irp[gx] : p.radc[gx]) : R(1);
        auto over_r = [&](R x) -> R { if constexpr (FAST) return x * rp; else return x / rp; };
        R sr0 = -u * drx - v * dry - (dux + dvy) * r_rho;
        R su0, sv0, sw0;
        R face[NV][4];   // [c][qm_x, qp_x, qm_y, qp_y]
        const R dxl = p.dx1[gx];
        const R dyl = (polar ? p.radc[gx] : R(1)) * p.dx2[gx];
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
            R dpx_r, dpy_r;
            if constexpr (FAST) { const R ir = R(1) / r_rho; dpx_r = dpx * ir; dpy_r = dpy * ir; }
            else { dpx_r = (dpx) / r_rho; dpy_r = (dpy) / r_rho; }
            su0 = -u * dux - v * duy - dpx_r;
            sv0 = -u * dvx - v * dvy - dpy_r;
            sw0 = -u * dwx - v * dwy;
            if (polar) {
                sr0 = -u * drx - v * dry - (dux + dvy) * r_rho - over_r(r_rho * u);
                sp0 = -u * dpx - v * dpy - (dux + dvy) * gamma * pp - over_r(gamma * pp * u);
                su0 = -u * dux - v * duy - dpx_r + over_r(sq(v));
                sv0 = -u * dvx - v * dvy - dpy_r - over_r(u * v);
                sw0 = -u * dwx - v * dwy;
            }
            const R smallP = prm<R>(p.smallp, p.f_smallp);
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
                sr0 = sr0 - over_r(r_rho * u);
                su0 = su0 + over_r(sq(v));
                sv0 = sv0 - over_r(u * v);
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

    // ---- 3. Riemann fluxes (godunov.f90:659-722, solve_wrapper :768-833) ----------------------
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
            const R ul = qmx[1 * S::ring + rl], vl = qmx[2 * S::ring + rl], wl = qmx[3 * S::ring + rl];
            const R ur = qpx[1 * S::ring + rr], vr = qpx[2 * S::ring + rr], wr = qpx[3 * S::ring + rr];
            const GasFlux<R> g = gas_flux(p, gamma, inv_g1, rl0, ul, vl, wl, pl, rr0, ur, vr, wr, pr, csl, csr);
            fl[0] = g.rho; fl[1] = g.mn; fl[2] = g.mt; fl[3] = g.mz; fl[4] = g.e;
        } else {
            const R rl0 = qmx[0 * S::ring + rl], ul = qmx[1 * S::ring + rl], vl = qmx[2 * S::ring + rl], wl = qmx[3 * S::ring + rl];
            const R rr0 = qpx[0 * S::ring + rr], ur = qpx[1 * S::ring + rr], vr = qpx[2 * S::ring + rr], wr = qpx[3 * S::ring + rr];
            // the HLLC dust solver's gas sound speeds (isothermal gas: per column, godunov.f90:675-677)
            const DustFlux<R> d = dust_flux(p.solverdust, rl0, ul, vl, wl, rr0, ur, vr, wr, p.cs[gxl], p.cs[gxl + 1]);
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
                const GasFlux<R> g = gas_flux(p, gamma, inv_g1, rl0, ul, vl, wl, pl, rr0, ur, vr, wr, pr, csl, csr);
                fl[0] = g.rho; fl[2] = g.mn; fl[1] = g.mt; fl[3] = g.mz; fl[4] = g.e;
            } else {
                const R rl0 = qmy[0 * S::ring + rl], ul = qmy[2 * S::ring + rl], vl = qmy[1 * S::ring + rl], wl = qmy[3 * S::ring + rl];
                const R rr0 = qpy[0 * S::ring + rr], ur = qpy[2 * S::ring + rr], vr = qpy[1 * S::ring + rr], wr = qpy[3 * S::ring + rr];
                const DustFlux<R> d = dust_flux(p.solverdust, rl0, ul, vl, wl, rr0, ur, vr, wr, p.cs[gx], p.cs[gx]);
                fl[0] = d.rho; fl[2] = d.mn; fl[1] = d.mt; fl[3] = d.mz;
            }
#pragma unroll
            for (int c = 0; c < NV; ++c) fys[c * S::fyn + f] = fl[c];
        }
    }
    __syncthreads();

    // ---- 4. kick + conservative update + local source terms, one thread per active cell ---------
    {
        const int cy = tid / T::TX, cx = tid - cy * T::TX;
        const int gx = ax0 + cx, gy = ay0 + cy;
        if (gx >= p.ng + p.nx || (NDIM == 2 && gy >= p.ng + p.ny)) return;
        const int hc = (cy + T::OY) * T::HX + cx + T::OX;
        R uu[NV];   // own conserved values, re-read from global memory (L2-resident after the stage)
#pragma unroll
        for (int c = 0; c < NV; ++c) uu[c] = p.u_cur[uidx(p, svar(s, c, N), gy, gx)];
        if (fk) {   // kick(1.0) (src/solver/force_kicks.f90:2-41) before the flux update
            R f1, f2, f3;
            setup_force(p, s, gx, gx, qs[1 * S::halo + hc], qs[3 * S::halo + hc], f1, f2, f3);
            const R rho = uu[0];
            if (IS_GAS) {
                R eo, en;
                if constexpr (FAST) {
                    const R ir = R(1) / rho;
                    eo = half * (sq(uu[1]) + sq(uu[2]) + sq(uu[3])) * ir;
                    uu[1] = uu[1] + rho * dt * f1;
                    uu[2] = uu[2] + rho * dt * f2;
                    uu[3] = uu[3] + rho * dt * f3;
                    en = half * (sq(uu[1]) + sq(uu[2]) + sq(uu[3])) * ir;
                } else {
                    eo = half * sq(uu[1]) / rho + half * sq(uu[2]) / rho + half * sq(uu[3]) / rho;
                    uu[1] = uu[1] + rho * R(1) * dt * f1;
                    uu[2] = uu[2] + rho * R(1) * dt * f2;
                    uu[3] = uu[3] + rho * R(1) * dt * f3;
                    en = half * sq(uu[1]) / rho + half * sq(uu[2]) / rho + half * sq(uu[3]) / rho;
                }
                uu[4] = uu[4] + (en - eo);
            } else {
                uu[1] = uu[1] + rho * R(1) * dt * f1;
                uu[2] = uu[2] + rho * R(1) * dt * f2;
                uu[3] = uu[3] + rho * R(1) * dt * f3;
            }
        }
        const R s1l = p.surf1[gx], s1r = p.surf1[gx + 1], vol = p.vol[gx];
        const int fxl = cy * (T::TX + 1) + cx;
        if constexpr (FAST) {
            const R dtv = dt * p.rvol[gx];
#pragma unroll
            for (int c = 0; c < NV; ++c) {
                const R* F = fxs + c * S::fxn;
                if (NDIM == 1) {
                    uu[c] = uu[c] + (F[fxl] * s1l - F[fxl + 1] * s1r) * dtv;
                } else {
                    const R* G = fys + c * S::fyn;
                    uu[c] = uu[c] + ((F[fxl] * s1l - F[fxl + 1] * s1r) + (G[cy * T::TX + cx] - G[(cy + 1) * T::TX + cx]) * p.surf2[gx]) * dtv;
                }
            }
        } else {
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
        }
        if (polar) {   // Source_terms, GEOM==2 (src/solver/source_terms.f90:37-47), on the OLD q
            const R qr = qs[0 * S::halo + hc], qvx = qs[1 * S::halo + hc], qvy = qs[2 * S::halo + hc];
            if constexpr (FAST) {
                const R dtr = dt * p.irp[gx];
                if (IS_GAS) uu[1] = uu[1] + (qr * sq(qvy) + qs[4 * S::halo + hc]) * dtr;
                else uu[1] = uu[1] + qr * sq(qvy) * dtr;
                uu[2] = uu[2] - qr * qvy * qvx * dtr;
            } else {
                const R rc = p.radc[gx];
                if (IS_GAS) uu[1] = uu[1] + dt * (qr * sq(qvy) + qs[4 * S::halo + hc]) / rc;
                else uu[1] = uu[1] + dt * (qr * sq(qvy) / rc);
                uu[2] = uu[2] + (R(0) - dt * (qr * qvy * qvx / rc));
            }
        }
#pragma unroll
        for (int c = 0; c < NV; ++c) p.u_next[uidx(p, svar(s, c, N), gy, gx)] = uu[c];
    }
}

template <typename R, int NDIM>
__global__ void __launch_bounds__(Tile<R, NDIM>::NT) k_flux(KParams<R> p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* sm = reinterpret_cast<R*>(smem_raw);
    const int s = blockIdx.z;
    if (s == 0) flux_tile<R, NDIM, true>(p, 0, sm);
    else flux_tile<R, NDIM, false>(p, s, sm);
}

}  // namespace shark
