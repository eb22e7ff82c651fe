// flux_strip.cuh -- K1 for 2D grids: barrier-free "column march" of one warp per strip.
//
// A warp owns 32 consecutive columns (lane = column) of one species and walks up a strip of
// STRIP_H rows.  Each iteration loads one new row of conserved values (one coalesced 128-byte
// access per variable), converts it to primitives and keeps a sliding window of three rows in
// registers.  The middle row is then predicted (limited slopes: y neighbours from the window,
// x neighbours by warp shuffle), its x-face fluxes are solved between neighbouring lanes
// (shuffle), the y-face flux below it is solved against the previous row's saved face state, and
// the row below is updated with the four fluxes now known.  No shared memory, no __syncthreads.
// Lanes 0,1,30,31 are the x halo: 28 columns per warp are updated.
//
// Same per-cell algorithm and expressions as flux_tile.cuh (ctoprim solve.f90:195-253, predictor
// godunov.f90:7-629, add_delta_u godunov.f90:659-750, kick force_kicks.f90:2-41, polar sources
// source_terms.f90:37-47); the FP64 instantiation keeps the oracle's operation order.
#pragma once

namespace shark {

constexpr int STRIP_UX = 28;     // columns updated per warp
constexpr int STRIP_H = 32;      // rows updated per warp
constexpr int STRIP_WARPS = 4;   // warps per CTA (along y)

template <typename R>
__device__ __forceinline__ R shfl_up1(R v) { return __shfl_up_sync(0xffffffffu, v, 1); }
template <typename R>
__device__ __forceinline__ R shfl_dn1(R v) { return __shfl_down_sync(0xffffffffu, v, 1); }

// ST: slope limiter (0..3), SOLV: gas solver (IS_GAS) or dust solver, both compile-time.
template <typename R, bool IS_GAS, int ST, int SOLV>
__device__ void flux_strip(const KParams<R>& p, int s, int bx, int by) {
    constexpr bool FAST = std::is_same<R, float>::value;
    constexpr int NV = IS_GAS ? 5 : 4;
    const int N = p.ndust;
    const int lane = threadIdx.x & 31;
    const int ax0 = p.ng + bx * STRIP_UX;      // first active column updated by this warp
    const int gx = ax0 - 2 + lane;             // this lane's column (>= 0)
    const int ay0 = p.ng + by * STRIP_H;       // first active row updated by this warp
    if (ay0 >= p.ng + p.ny) return;            // whole warp beyond the domain (uniform)
    const int ylast = min(ay0 + STRIP_H, p.ng + p.ny) - 1;
    const int gxc = min(gx, p.nx_max - 1);
    const bool col_in = gx < p.nx_max;
    const bool col_pred = lane >= 1 && lane <= 30 && gx <= p.nx_max - 2;                 // slopes defined
    const bool col_upd = lane >= 2 && lane <= 29 && gx < p.ng + p.nx;                    // cell updated
    const bool col_active = gx >= p.ng && gx < p.ng + p.nx;

    const R dt = step_dt(p);
    const R half = R(0.5);
    const R gamma = prm<R>(p.gamma, p.f_gamma);
    const R inv_g1 = prm<R>(1.0 / (p.gamma - 1.0), p.f_inv_g1);
    const R smallP = prm<R>(p.smallp, p.f_smallp), smallR = prm<R>(p.smallr, p.f_smallr);
    const bool fk = (p.flags & SHARK_FLAG_FORCE_KICK) != 0;
    const bool polar = (p.geom == 2);
    const bool iso = (p.iso == 1);
    // column metrics
    const R dx1 = p.dx1[gxc], dx1l = p.dx1[max(gxc - 1, 0)], dx1r = p.dx1[min(gxc + 1, p.nx_max - 1)];
    const R dx2 = p.dx2[gxc];
    const R radc = p.radc[gxc];
    const R sfl = p.sfx[gxc], sfr = p.sfx[min(gxc + 1, p.nx_max - 1)], sfy = p.sfy[gxc], irp = p.irp[gxc];
    const R s1l = p.surf1[gxc], s1r = p.surf1[min(gxc + 1, p.nx_max - 1)], s2 = p.surf2[gxc];
    const R vol = p.vol[gxc], rvol = p.rvol[gxc];
    const R cs_col = p.cs[gxc];
    const R dxl = dx1, dyl = (polar ? radc : R(1)) * dx2;
    const R hdt = half * dt, hdx = half * dxl, hdy = half * dyl, dtv = dt * rvol;   // mixed path

    R q0[NV], q1[NV], q2[NV];       // primitive rows P-1, P, P+1 (P = row being predicted)
    R c0 = R(0), c1 = R(0), c2 = R(0);
    R qmy_prev[NV];                 // qm_y of the previous predicted row
    R g_prev[NV];                   // y flux at the bottom face of the previous predicted row
    R t_prev[NV];                   // previous row after kick + x-flux part of the update
    R c_prev = R(0);                // cs of the previous predicted row (isothermal y faces)
    R vxm2 = R(0), vym2 = R(0);     // old vx, vy of row P-2 (Cartesian viscosity, y neighbour)

    // per-lane 32-bit element offsets of the species' planes (the context guarantees
    // nvar * plane < 2^31); row offsets are added per access
    int voff[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) voff[k] = svar(s, k, N) * (int)p.plane + gxc;
    const R* __restrict__ src = p.u_cur;
    R* __restrict__ dst = p.u_next;
    const int pitch = p.pitch;
    // raw conserved values of one row (issued one iteration ahead of their use)
    auto fetch_row = [&](int row, R* us) {
        const bool in = col_in && row < p.ny_max;
        const int ro = min(row, p.ny_max - 1) * pitch;
#pragma unroll
        for (int k = 0; k < NV; ++k) us[k] = in ? __ldg(src + (voff[k] + ro)) : R(1);
    };
    // isothermal sound speed of (row, column): per column, or per cell on the Cartesian disk
    auto cs_at = [&](int row) -> R { return p.ccs ? p.ccs[min(row, p.ny_max - 1) * pitch + gxc] : cs_col; };
    auto to_prim = [&](const R* us, R* q, R& c, int row) {
        if (IS_GAS) {
            const R rho = us[0], px = us[1], py = us[2], pz = us[3];
            R P, vx, vy, vz;
            if constexpr (FAST) {
                const R ir = R(1) / rho;
                vx = px * ir; vy = py * ir; vz = pz * ir;
                P = fmax2((gamma - R(1)) * (us[4] - half * (px * vx + py * vy + pz * vz)), smallP);
            } else {
                vx = px / rho; vy = py / rho; vz = pz / rho;
                const R ekin = half * rho * sq(px / rho) + half * rho * sq(py / rho) + half * rho * sq(pz / rho);
                P = fmax2((gamma - R(1)) * (us[4] - ekin - R(0)), smallP);
            }
            const R qrho = fmax2(rho, smallR);
            if (!iso) c = sqrt(gamma * P / qrho);
            else { c = cs_at(row); P = rho * sq(c); }
            q[0] = qrho; q[1] = vx; q[2] = vy; q[3] = vz; q[4] = P;
        } else {
            q[0] = us[0];
            if constexpr (FAST) {
                const R ir = R(1) / us[0];
                q[1] = us[1] * ir; q[2] = us[2] * ir; q[3] = us[3] * ir;
            } else {
                q[1] = us[1] / us[0]; q[2] = us[2] / us[0]; q[3] = us[3] / us[0];
            }
        }
    };

    // rows ay0-2 and ay0-1 prime the window; row ay0 is in flight
    R raw[NV];
    fetch_row(ay0 - 2, raw);
    to_prim(raw, q0, c0, ay0 - 2);
    fetch_row(ay0 - 1, raw);
    to_prim(raw, q1, c1, ay0 - 1);
    R nxt[NV];
    fetch_row(ay0, nxt);
    const int rend = ylast + 2;   // last row loaded
    for (int row = ay0; row <= rend; ++row) {
        to_prim(nxt, q2, c2, row);
        if (row < rend) fetch_row(row + 1, nxt);   // prefetch the next row (uniform branch)
        const int P = row - 1;    // predicted row, ay0-1 .. ylast+1
        // the update of row P starts in this iteration (kick + x fluxes) and ends in the next one
        // (y flux above it); load its own conserved values now (an L1/L2 hit)
        const bool start_upd = col_upd && P >= ay0 && P <= ylast;
        const bool finish_upd = col_upd && P - 1 >= ay0 && P - 1 <= ylast;
        R uu[NV];
        if (start_upd) {
#pragma unroll
            for (int k = 0; k < NV; ++k) uu[k] = __ldg(src + (voff[k] + P * pitch));
        }
        // ---- predictor of (P, gx) -------------------------------------------------------------
        R dqx[NV], dqy[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            dqx[k] = R(0);
            dqy[k] = R(0);
            if (IS_GAS && k == 4 && iso) continue;   // isothermal: the pressure slopes are rho's times cs^2
            const R ql = shfl_up1(q1[k]), qr = shfl_dn1(q1[k]);
            if constexpr (ST > 0) {
                if constexpr (FAST) {
                    dqx[k] = slope_limit_t<ST>((q1[k] - ql) * sfl, (qr - q1[k]) * sfr);
                    dqy[k] = slope_limit_t<ST>((q1[k] - q0[k]) * sfy, (q2[k] - q1[k]) * sfy);
                } else {
                    dqx[k] = slope_limit_t<ST>(R(2) * (q1[k] - ql) / (dx1 + dx1l), R(2) * (qr - q1[k]) / (dx1r + dx1));
                    dqy[k] = slope_limit_t<ST>(R(2) * (q1[k] - q0[k]) / (dx2 + dx2), R(2) * (q2[k] - q1[k]) / (dx2 + dx2)) /
                             (polar ? radc : R(1));
                }
            }
        }
        R r_rho = q1[0], u = q1[1], v = q1[2], w = q1[3];
        const R drx = dqx[0], dux = dqx[1], dvx = dqx[2], dwx = dqx[3];
        const R dry = dqy[0], duy = dqy[1], dvy = dqy[2], dwy = dqy[3];
        R f1 = R(0), f2 = R(0), f3 = R(0);   // force of row P; the kick of row P below reuses it
        if (fk) {
            const bool active = col_active && P >= p.ng && P < p.ng + p.ny;
            if (active) setup_force(p, s, gxc, (long long)P * pitch + gxc, u, w, f1, f2, f3);   // ghost cells keep force = 0 (SI/setup.f90:339)
            u = u + f1 * half * dt;
            v = v + f2 * half * dt;
            w = w + f3 * half * dt;
        }
        auto over_r = [&](R x) -> R { if constexpr (FAST) return x * irp; else return x / radc; };
        R qmx[NV], qpx[NV], qmy[NV], qpy[NV];
        R sr0 = -u * drx - v * dry - (dux + dvy) * r_rho;
        if (IS_GAS) {
            R pp = q1[4], dpx = dqx[4], dpy = dqy[4];
            if (iso) {
                pp = q1[0] * sq(c1);
                dpx = dqx[0] * sq(c1);
                dpy = dqy[0] * sq(c1);
            }
            R sp0 = -u * dpx - v * dpy - (dux + dvy) * gamma * pp;
            R dpx_r, dpy_r;
            if constexpr (FAST) { const R ir = R(1) / r_rho; dpx_r = dpx * ir; dpy_r = dpy * ir; }
            else { dpx_r = (dpx) / r_rho; dpy_r = (dpy) / r_rho; }
            R su0 = -u * dux - v * duy - dpx_r;
            R sv0 = -u * dvx - v * dvy - dpy_r;
            R sw0 = -u * dwx - v * dwy;
            if (polar) {
                sr0 = -u * drx - v * dry - (dux + dvy) * r_rho - over_r(r_rho * u);
                sp0 = -u * dpx - v * dpy - (dux + dvy) * gamma * pp - over_r(gamma * pp * u);
                su0 = -u * dux - v * duy - dpx_r + over_r(sq(v));
                sv0 = -u * dvx - v * dvy - dpy_r - over_r(u * v);
            }
            if constexpr (FAST) {
                const R b0 = r_rho + hdt * sr0, b1 = u + hdt * su0, b2 = v + hdt * sv0, b3 = w + hdt * sw0, b4 = pp + hdt * sp0;
                qmx[0] = b0 + hdx * drx; qpx[0] = b0 - hdx * drx;
                qmx[1] = b1 + hdx * dux; qpx[1] = b1 - hdx * dux;
                qmx[2] = b2 + hdx * dvx; qpx[2] = b2 - hdx * dvx;
                qmx[3] = b3 + hdx * dwx; qpx[3] = b3 - hdx * dwx;
                qmx[4] = fmaxf(b4 + hdx * dpx, smallP); qpx[4] = fmaxf(b4 - hdx * dpx, smallP);
                qmy[0] = b0 + hdy * dry; qpy[0] = b0 - hdy * dry;
                qmy[1] = b1 + hdy * duy; qpy[1] = b1 - hdy * duy;
                qmy[2] = b2 + hdy * dvy; qpy[2] = b2 - hdy * dvy;
                qmy[3] = b3 + hdy * dwy; qpy[3] = b3 - hdy * dwy;
                qmy[4] = fmaxf(b4 + hdy * dpy, smallP); qpy[4] = fmaxf(b4 - hdy * dpy, smallP);
            } else {
                qmx[0] = r_rho + half * dt * sr0 + half * drx * dxl;
                qmx[1] = u + half * dt * su0 + half * dux * dxl;
                qmx[4] = fmax2(pp + half * dt * sp0 + half * dpx * dxl, smallP);
                qmx[2] = v + half * dt * sv0 + half * dvx * dxl;
                qmx[3] = w + half * dt * sw0 + half * dwx * dxl;
                qpx[0] = r_rho + half * dt * sr0 - half * drx * dxl;
                qpx[1] = u + half * dt * su0 - half * dux * dxl;
                qpx[4] = fmax2(pp + half * dt * sp0 - half * dpx * dxl, smallP);
                qpx[2] = v + half * dt * sv0 - half * dvx * dxl;
                qpx[3] = w + half * dt * sw0 - half * dwx * dxl;
                qmy[0] = r_rho + half * dt * sr0 + half * dry * dyl;
                qmy[1] = u + half * dt * su0 + half * duy * dyl;
                qmy[4] = fmax2(pp + half * dt * sp0 + half * dpy * dyl, smallP);
                qmy[2] = v + half * dt * sv0 + half * dvy * dyl;
                qmy[3] = w + half * dt * sw0 + half * dwy * dyl;
                qpy[0] = r_rho + half * dt * sr0 - half * dry * dyl;
                qpy[1] = u + half * dt * su0 - half * duy * dyl;
                qpy[4] = fmax2(pp + half * dt * sp0 - half * dpy * dyl, smallP);
                qpy[2] = v + half * dt * sv0 - half * dvy * dyl;
                qpy[3] = w + half * dt * sw0 - half * dwy * dyl;
            }
            if (iso) {   // godunov.f90:606-611
                qmx[4] = sq(c1) * qmx[0];
                qpx[4] = sq(c1) * qpx[0];
                qmy[4] = sq(c1) * qmy[0];
                qpy[4] = sq(c1) * qpy[0];
            }
        } else {
            R su0 = -u * dux - v * duy;
            R sv0 = -u * dvx - v * dvy;
            R sw0 = -u * dwx - v * dwy;
            if (polar) {
                sr0 = sr0 - over_r(r_rho * u);
                su0 = su0 + over_r(sq(v));
                sv0 = sv0 - over_r(u * v);
            }
            if constexpr (FAST) {
                const R b0 = r_rho + hdt * sr0, b1 = u + hdt * su0, b2 = v + hdt * sv0, b3 = w + hdt * sw0;
                qmx[0] = b0 + hdx * drx; qpx[0] = b0 - hdx * drx;
                qmx[1] = b1 + hdx * dux; qpx[1] = b1 - hdx * dux;
                qmx[2] = b2 + hdx * dvx; qpx[2] = b2 - hdx * dvx;
                qmx[3] = b3 + hdx * dwx; qpx[3] = b3 - hdx * dwx;
                qmy[0] = b0 + hdy * dry; qpy[0] = b0 - hdy * dry;
                qmy[1] = b1 + hdy * duy; qpy[1] = b1 - hdy * duy;
                qmy[2] = b2 + hdy * dvy; qpy[2] = b2 - hdy * dvy;
                qmy[3] = b3 + hdy * dwy; qpy[3] = b3 - hdy * dwy;
            } else {
                qmx[0] = r_rho + half * dt * sr0 + half * drx * dxl;
                qmx[1] = u + half * dt * su0 + half * dux * dxl;
                qmx[2] = v + half * dt * sv0 + half * dvx * dxl;
                qmx[3] = w + half * dt * sw0 + half * dwx * dxl;
                qpx[0] = r_rho + half * dt * sr0 - half * drx * dxl;
                qpx[1] = u + half * dt * su0 - half * dux * dxl;
                qpx[2] = v + half * dt * sv0 - half * dvx * dxl;
                qpx[3] = w + half * dt * sw0 - half * dwx * dxl;
                qmy[0] = r_rho + half * dt * sr0 + half * dry * dyl;
                qmy[1] = u + half * dt * su0 + half * duy * dyl;
                qmy[2] = v + half * dt * sv0 + half * dvy * dyl;
                qmy[3] = w + half * dt * sw0 + half * dwy * dyl;
                qpy[0] = r_rho + half * dt * sr0 - half * dry * dyl;
                qpy[1] = u + half * dt * su0 - half * duy * dyl;
                qpy[2] = v + half * dt * sv0 - half * dvy * dyl;
                qpy[3] = w + half * dt * sw0 - half * dwy * dyl;
            }
        }
        (void)col_pred;

        // ---- x faces of row P: left face of this lane = (qm_x of lane-1, qp_x of this lane) --------
        R fxl[NV];
        {
            R ql[NV];
#pragma unroll
            for (int k = 0; k < NV; ++k) ql[k] = shfl_up1(qmx[k]);
            if (IS_GAS) {
                R csl, csr;
                if (iso) { csl = shfl_up1(c1); csr = c1; }
                else { csl = sqrt(gamma * ql[4] / ql[0]); csr = sqrt(gamma * qpx[4] / qpx[0]); }
                const GasFlux<R> g = gas_flux_t<SOLV>(gamma, inv_g1, ql[0], ql[1], ql[2], ql[3], ql[4],
                                              qpx[0], qpx[1], qpx[2], qpx[3], qpx[4], csl, csr);
                fxl[0] = g.rho; fxl[1] = g.mn; fxl[2] = g.mt; fxl[3] = g.mz; fxl[4] = g.e;
            } else {
                // gas sound speeds of the face for the HLLC dust solver (isothermal: per column)
                const DustFlux<R> d = dust_flux_t<SOLV>(ql[0], ql[1], ql[2], ql[3], qpx[0], qpx[1], qpx[2], qpx[3],
                                                        shfl_up1(cs_col), cs_col);
                fxl[0] = d.rho; fxl[1] = d.mn; fxl[2] = d.mt; fxl[3] = d.mz;
            }
        }
        R fxr[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) fxr[k] = shfl_dn1(fxl[k]);

        // ---- y face below row P: (qm_y of row P-1, qp_y of row P) -------------------------------------
        R gb[NV];
        if (row > ay0) {
            if (IS_GAS) {
                R csl, csr;
                if (iso) { csl = c_prev; csr = c1; }
                else { csl = sqrt(gamma * qmy_prev[4] / qmy_prev[0]); csr = sqrt(gamma * qpy[4] / qpy[0]); }
                // idim = 2: normal velocity vy, transverse vx (allocate_init.f90:249-252)
                const GasFlux<R> g = gas_flux_t<SOLV>(gamma, inv_g1, qmy_prev[0], qmy_prev[2], qmy_prev[1], qmy_prev[3], qmy_prev[4],
                                              qpy[0], qpy[2], qpy[1], qpy[3], qpy[4], csl, csr);
                gb[0] = g.rho; gb[2] = g.mn; gb[1] = g.mt; gb[3] = g.mz; gb[4] = g.e;
            } else {
                const DustFlux<R> d = dust_flux_t<SOLV>(qmy_prev[0], qmy_prev[2], qmy_prev[1], qmy_prev[3],
                                                qpy[0], qpy[2], qpy[1], qpy[3], cs_col, cs_col);
                gb[0] = d.rho; gb[2] = d.mn; gb[1] = d.mt; gb[3] = d.mz;
            }
        }
        // radial neighbours of row P-1's old velocities for the viscous term (all lanes shuffle)
        R vxl = R(0), vxr = R(0), vyl = R(0), vyr = R(0);
        if (IS_GAS && p.visc) {
            vxl = shfl_up1(q0[1]); vxr = shfl_dn1(q0[1]);
            vyl = shfl_up1(q0[2]); vyr = shfl_dn1(q0[2]);
        }
        // ---- finish row P-1: y-flux part, then the polar sources on its OLD q (= q0) ---------------
        if (row > ay0 && finish_upd) {
            R un[NV];
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                if constexpr (FAST) un[k] = t_prev[k] + (g_prev[k] - gb[k]) * s2 * (dt * rvol);
                else un[k] = t_prev[k] + (g_prev[k] * s2 - gb[k] * s2) / vol * dt;
            }
            if (polar && IS_GAS && p.visc) {
                // Source_terms GEOM==2 (source_terms.f90:37-47) plus the viscous term
                // (source_terms.f90:110-115), accumulated in S_U before the update as there
                const R qr = q0[0], qvx = q0[1], qvy = q0[2];
                const R eta = p.etav[gxc];
                R S1, S2;
                if constexpr (FAST) {
                    const R dtr = dt * irp, idx2 = R(1) / (dx1 * dx1);
                    S1 = (qr * sq(qvy) + q0[4]) * dtr;
                    S2 = -(qr * qvy * qvx * dtr);
                    const R lu = (vxr + vxl - R(2) * qvx) * idx2 + (vxr + vxl) * irp / dx1 * half - qvx * irp * irp;
                    const R lv = (vyr + vyl - R(2) * qvy) * idx2 - qvy * irp * irp + (vyr + vyl) * irp / dx1 * half;
                    S1 = S1 + qr * dt * eta * lu;
                    S2 = S2 + qr * dt * eta * lv;
                } else {
                    S1 = dt * (qr * sq(qvy) + q0[4]) / radc;
                    S2 = R(0) - dt * (qr * qvy * qvx / radc);
                    const R lu = (vxr + vxl - R(2) * qvx) / (dx1 * dx1) + (vxr + vxl) / radc / dx1 / R(2) - qvx / radc / radc;
                    S1 = S1 + qr * dt * eta * lu;
                    const R lv = (vyr + vyl - R(2) * qvy) / (dx1 * dx1) - qvy / (radc * radc) + (vyr + vyl) / radc / dx1 / R(2);
                    S2 = S2 + qr * dt * eta * lv;
                }
                un[1] = un[1] + S1;
                un[2] = un[2] + S2;
            } else if (IS_GAS && p.visc) {
                // Cartesian viscosity (source_terms.f90:99-109) on the old velocities of row P-1,
                // its x neighbours and rows P-2 and P, accumulated in S_U before the update
                const R qr = q0[0], qvx = q0[1], qvy = q0[2];
                const R eta = p.ceta[(P - 1) * pitch + gxc];
                const R dy = p.dx2[gxc];
                const R lap_x_u = (vxr + vxl - R(2) * qvx) / (dx1 * dx1);
                R S1 = qr * dt * eta * lap_x_u;
                const R lap_y_u = (q1[1] + vxm2 - R(2) * qvx) / (dy * dy);
                S1 = S1 + qr * dt * eta * lap_y_u;
                const R lap_x_v = (vyr + vyl - R(2) * qvy) / (dx1 * dx1);
                const R lap_y_v = (q1[2] + vym2 - R(2) * qvy) / (dy * dy);
                const R S2 = qr * dt * eta * (lap_x_v + lap_y_v);
                un[1] = un[1] + S1;
                un[2] = un[2] + S2;
            } else if (polar) {   // Source_terms GEOM==2 (source_terms.f90:37-47)
                const R qr = q0[0], qvx = q0[1], qvy = q0[2];
                if constexpr (FAST) {
                    const R dtr = dt * irp;
                    if (IS_GAS) un[1] = un[1] + (qr * sq(qvy) + q0[4]) * dtr;
                    else un[1] = un[1] + qr * sq(qvy) * dtr;
                    un[2] = un[2] - qr * qvy * qvx * dtr;
                } else {
                    if (IS_GAS) un[1] = un[1] + dt * (qr * sq(qvy) + q0[4]) / radc;
                    else un[1] = un[1] + dt * (qr * sq(qvy) / radc);
                    un[2] = un[2] + (R(0) - dt * (qr * qvy * qvx / radc));
                }
            }
#pragma unroll
            for (int k = 0; k < NV; ++k) dst[voff[k] + (P - 1) * pitch] = un[k];
        }
        // ---- start row P: kick(1.0) with the force of its OLD q (= q1), then the x-flux part ------
        if (start_upd) {
            if (fk) {   // force_kicks.f90:2-41, before the flux update (force of this row's OLD q)
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
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                if constexpr (FAST) uu[k] = uu[k] + (fxl[k] * s1l - fxr[k] * s1r) * (dt * rvol);
                else uu[k] = uu[k] + (fxl[k] * s1l - fxr[k] * s1r) / vol * dt;
            }
        }
            // ---- slide the window ---------------------------------------------------------------
        vxm2 = q0[1];
        vym2 = q0[2];
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            qmy_prev[k] = qmy[k];
            g_prev[k] = gb[k];
            t_prev[k] = uu[k];
            q0[k] = q1[k];
            q1[k] = q2[k];
        }
        c_prev = c1;
        c0 = c1;
        c1 = c2;
    }
    (void)c0;
}

// Gas and dust run as separate kernels so the dust warps (N of every N+1) are not held to the
// register footprint of the 5-variable gas path with its HLLC solver.
template <typename R, bool IS_GAS, int ST, int SOLV>
__global__ void __launch_bounds__(32 * STRIP_WARPS, (IS_GAS || !std::is_same<R, float>::value) ? 1 : 5)
k_flux_strip(KParams<R> p) {
    const int warp = threadIdx.x >> 5;
    const int bx = blockIdx.x;
    const int by = blockIdx.y * STRIP_WARPS + warp;
    const int s = IS_GAS ? 0 : blockIdx.z + 1;
    flux_strip<R, IS_GAS, ST, SOLV>(p, s, bx, by);
}

}  // namespace shark
