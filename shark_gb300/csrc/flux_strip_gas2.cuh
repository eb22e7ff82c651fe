// flux_strip_gas2.cuh -- K1 for the gas of the mixed path on 2D Cartesian grids, two adjacent
// columns per lane (the layout of flux_strip_dust2: lane l owns columns c0 + 2l, c0 + 2l + 1,
// lanes 0 and 31 are the x halo, 60 columns per warp).  Every FP32 operation that acts on both
// columns the same way is one packed FP32x2 instruction; comparisons, min/max, selects and the
// reciprocals stay per column.
//
// Algorithm: the FP32 gas path of flux_strip.cuh (ctoprim solve.f90:195-253, predictor
// godunov.f90:7-629, HLLC / HLL / LLF solvers.f90:4-500, add_delta_u godunov.f90:659-750, kick
// force_kicks.f90:2-41, SI force SI/setup.f90:335-350).  The limited slopes are carried doubled
// (2 dq) as in flux_strip_dust2, and the half-step factors halved to match.
#pragma once

namespace shark {

__device__ __forceinline__ float2 rcp2(float2 a) { return make_float2(1.f / a.x, 1.f / a.y); }
__device__ __forceinline__ float2 sel2(bool cx, bool cy, float2 a, float2 b) {
    return make_float2(cx ? a.x : b.x, cy ? a.y : b.y);
}

// The three gas solvers of gas_flux_t (flux_tile.cuh) on two faces.  f = (mass, normal momentum,
// transverse momentum, second transverse momentum, energy).  The face pressures L[4], R[4] are
// given as P - p0 for a constant p0: the momentum flux carries P - p0 (a constant added to it
// cancels in the flux difference of a cell whose opposite faces have the same area) and the
// energy flux the absolute pressure, so that with p0 near the typical pressure the momentum flux
// keeps the pressure's small variations at full FP32 precision.  p0 = 0 gives the solvers as
// written in the reference.
template <int GSOLV>
__device__ __forceinline__ void gas_flux2(float gamma, float inv_g1, const float2* L, const float2* R, float2 csl,
                                          float2 csr, float2* f, float p0) {
    const float2 rl = L[0], ul = L[1], vl = L[2], wl = L[3], pl = L[4];
    const float2 rr = R[0], ur = R[1], vr = R[2], wr = R[3], pr = R[4];
    const float2 h = bc2(0.5f), P0 = bc2(p0);
    const float2 pla = add2(pl, P0), pra = add2(pr, P0);   // absolute pressures (energy only)
    // E = P/(gamma-1) + rho (u^2 + v^2 + w^2)/2
    const float2 El = fma2(pla, bc2(inv_g1), mul2(mul2(h, rl), fma2(ul, ul, fma2(vl, vl, mul2(wl, wl)))));
    const float2 Er = fma2(pra, bc2(inv_g1), mul2(mul2(h, rr), fma2(ur, ur, fma2(vr, vr, mul2(wr, wr)))));
    if constexpr (GSOLV == 2) {   // HLLC (gas_hllc_fast)
        const float2 cmax = make_float2(fmaxf(csl.x, csr.x), fmaxf(csl.y, csr.y));
        const float2 Sl = make_float2(fminf(fminf(ul.x, ur.x) - cmax.x, 0.f), fminf(fminf(ul.y, ur.y) - cmax.y, 0.f));
        const float2 Sr = make_float2(fmaxf(fmaxf(ul.x, ur.x) + cmax.x, 0.f), fmaxf(fmaxf(ul.y, ur.y) + cmax.y, 0.f));
        const float2 hl = mul2(rl, sub2(ul, Sl)), hr = mul2(rr, sub2(Sr, ur));
        const float2 inv = rcp2(add2(hr, hl));
        const float2 ustar = mul2(fma2(hr, ur, fma2(hl, ul, sub2(pl, pr))), inv);
        const float2 pstar = mul2(fma2(hr, pl, fma2(hl, pr, mul2(mul2(hl, hr), sub2(ul, ur)))), inv);
        // star side by the sign of u* (solvers.f90:469-481); S_l <= 0 <= S_r by construction, so
        // the sampled state is a star state unless S_r = 0 (then the right state)
        const bool lx = ustar.x > 0.f, ly = ustar.y > 0.f;
        const float2 S = sel2(lx, ly, Sl, Sr), rho = sel2(lx, ly, rl, rr), u = sel2(lx, ly, ul, ur);
        const float2 P = sel2(lx, ly, pl, pr), E = sel2(lx, ly, El, Er);
        const float2 Su = sub2(S, u);
        const float2 a = rcp2(sub2(S, ustar));
        float2 ro = mul2(mul2(rho, Su), a);
        // ((pstar + p0) ustar + Su E - (P + p0) u) / (S - ustar)
        float2 eo = mul2(fma2(P0, sub2(ustar, u), fma2(pstar, ustar, fma2(Su, E, mul2(bc2(-1.f), mul2(P, u))))), a);
        float2 uo = ustar, po = pstar;
        const bool rx = Sr.x <= 0.f, ry = Sr.y <= 0.f;
        ro = sel2(rx, ry, rr, ro);
        uo = sel2(rx, ry, ur, uo);
        po = sel2(rx, ry, pr, po);
        eo = sel2(rx, ry, Er, eo);
        const float2 m = mul2(ro, uo);
        f[0] = m;
        f[1] = fma2(m, uo, po);
        f[4] = mul2(add2(eo, add2(po, P0)), uo);
        f[2] = mul2(m, sel2(lx, ly, vl, vr));
        f[3] = mul2(m, sel2(lx, ly, wl, wr));
    } else if constexpr (GSOLV == 1) {   // HLL (gas_hll_fast)
        const float2 cmax = make_float2(fmaxf(csl.x, csr.x), fmaxf(csl.y, csr.y));
        const float2 Sl = make_float2(fminf(fminf(ul.x, ur.x) - cmax.x, 0.f), fminf(fminf(ul.y, ur.y) - cmax.y, 0.f));
        const float2 Sr = make_float2(fmaxf(fmaxf(ul.x, ur.x) + cmax.x, 0.f), fmaxf(fmaxf(ul.y, ur.y) + cmax.y, 0.f));
        const float2 inv = rcp2(sub2(Sr, Sl));
        const float2 ss = mul2(Sr, Sl);
        const float2 ml = mul2(rl, ul), mr = mul2(rr, ur);
        // (S_r F_l - S_l F_r + S_r S_l (U_r - U_l)) / (S_r - S_l)
        auto hll = [&](float2 Fl, float2 Fr, float2 Ul, float2 Ur) {
            return mul2(fma2(Sr, Fl, fma2(mul2(bc2(-1.f), Sl), Fr, mul2(ss, sub2(Ur, Ul)))), inv);
        };
        f[0] = hll(ml, mr, rl, rr);
        f[1] = hll(fma2(ml, ul, pl), fma2(mr, ur, pr), ml, mr);
        f[2] = hll(mul2(ml, vl), mul2(mr, vr), mul2(rl, vl), mul2(rr, vr));
        f[3] = hll(mul2(ml, wl), mul2(mr, wr), mul2(rl, wl), mul2(rr, wr));
        f[4] = hll(mul2(add2(El, pla), ul), mul2(add2(Er, pra), ur), El, Er);
    } else {   // LLF (gas_llf)
        const float2 lam = make_float2(fmaxf(fabsf(ul.x) + csl.x, fabsf(ur.x) + csr.x),
                                       fmaxf(fabsf(ul.y) + csl.y, fabsf(ur.y) + csr.y));
        const float2 hlam = mul2(h, lam);
        const float2 ml = mul2(rl, ul), mr = mul2(rr, ur);
        auto llf = [&](float2 Fl, float2 Fr, float2 Ul, float2 Ur) {
            return fma2(h, add2(Fl, Fr), mul2(bc2(-1.f), mul2(hlam, sub2(Ur, Ul))));
        };
        f[0] = llf(ml, mr, rl, rr);
        f[1] = llf(fma2(ml, ul, pl), fma2(mr, ur, pr), ml, mr);
        f[2] = llf(mul2(ml, vl), mul2(mr, vr), mul2(rl, vl), mul2(rr, vr));
        f[3] = llf(mul2(ml, wl), mul2(mr, wr), mul2(rl, wl), mul2(rr, wr));
        f[4] = llf(mul2(add2(El, pla), ul), mul2(add2(Er, pra), ur), El, Er);
    }
}

// K1 of the gas on a uniform Cartesian grid (UniformGrid, flux_strip2.cuh), two columns per lane,
// rows ay0 .. ylast from `Rows` (rows.cuh).  ISO: isothermal (the pressure is rho cs^2
// everywhere, so it is not carried in the row window).  Same row structure as flux_strip_dust2:
// x differences of the row, the y difference to the next row carried to the next iteration.
template <int ST, int GSOLV, bool ISO, class Rows>
__device__ __forceinline__ void flux_strip_gas2(const KParams<float>& p, RingArgs& ra, int bx, int ay0, int ylast) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int ax0 = p.ng + bx * STRIP2_UX;
    const int ga = ax0 - 2 + 2 * lane;         // this lane's columns ga, ga + 1 (ga even)
    const bool col_in = ga < p.nx_max;         // ga + 1 is then inside the row's pitch padding
    const int ca = min(ga, p.nx_max - 1), cb = min(ga + 1, p.nx_max - 1);
    const bool halo = lane == 0 || lane == 31;
    const bool upd_a = !halo && ga < p.ng + p.nx, upd_b = !halo && ga + 1 < p.ng + p.nx;
    const bool upd_1 = upd_a && !upd_b;        // only the first of the pair is updated
    const bool act_a = ga >= p.ng && ga < p.ng + p.nx, act_b = ga + 1 >= p.ng && ga + 1 < p.ng + p.nx;

    const float dt = *p.dtf;
    const UniformGrid G = uniform_grid(p, dt);
    const float2 cxf = bc2(G.cxf), ncxf = bc2(-G.cxf), cyf = bc2(G.cyf), ncyf = bc2(-G.cyf);
    const float2 q4 = bc2(0.25f), nq4 = bc2(-0.25f);
    const float gamma = p.f_gamma, inv_g1 = p.f_inv_g1, smallp = p.f_smallp, smallr = p.f_smallr;
    constexpr bool iso = ISO;
    const float2 c = iso ? make_float2(p.cs[ca], p.cs[cb]) : make_float2(0.f, 0.f);
    const float2 c2 = mul2(c, c);
    // isothermal gas: the density is carried as rho - rho0 through the predictor and the face
    // states, the face pressures as c^2 (rho - rho0) = P - p0 (gas_flux2); rho0 (the mean density
    // of the first uploaded state, 0 where the sound speed varies between columns or the gas is
    // adiabatic) makes the small density and pressure variations of a near-uniform box exact to
    // FP32 rounding of the variations instead of the mean
    const float rho0 = iso ? p.f_rho_ref : 0.f;
    const float p0 = rho0 * c2.x;
    const float2 R0 = bc2(rho0);
    // SI force on the gas (setup_force, species 0): f1 = 2 q om^2 xc - 2 om vz - 2 r0 om eta, f3 = 2 om vx
    const bool fk = (p.flags & SHARK_FLAG_FORCE_KICK) != 0 && p.setup == SHARK_SETUP_SI;
    const float om = p.f_si_om, qs = p.f_si_q;
    const float f1x = 2.f * qs * (om * om) * (p.xpos[ca] - p.f_half_box_l) - 2.f * p.f_si_r0 * om * p.f_si_eta;
    const float f1y = 2.f * qs * (om * om) * (p.xpos[cb] - p.f_half_box_l) - 2.f * p.f_si_r0 * om * p.f_si_eta;
    const float2 f1c = make_float2(f1x, f1y);
    const float2 m2om = bc2(-2.f * om), p2om = bc2(2.f * om);
    const float2 fsel = make_float2(act_a ? 1.f : 0.f, act_b ? 1.f : 0.f);   // ghost columns: force 0

    constexpr int NV = 5;
    float2 q1[NV];                      // primitive row P (rho, vx, vy, vz, P)
    float2 dyl[NV];                     // y difference q(P) - q(P-1)
    float2 qmy_prev[NV], t_prev[NV];   // t_prev: row P-1 after its kick, x fluxes and lower y flux
    // element offset of variable k of this lane's first column: ca + k * plane
    const int vpl = (int)p.plane;
    auto voff = [&](int k) { return ca + k * vpl; };
    float* __restrict__ dst = p.u_next;
    const int pitch = p.pitch;
    Rows rows = make_rows<Rows>(p, ra, ca, vpl, col_in, ax0 - 2, ay0 - 2, -1, ylast - ay0 + 5);
    auto to_prim = [&](const float2* us, float2* q) {
        const float2 ir = rcp2(us[0]);
        q[1] = mul2(us[1], ir);
        q[2] = mul2(us[2], ir);
        q[3] = mul2(us[3], ir);
        q[0] = sub2(make_float2(fmaxf(us[0].x, smallr), fmaxf(us[0].y, smallr)), R0);
        if (iso) {
            q[4] = mul2(q[0], c2);
        } else {
            // P = max((gamma - 1) (E - (m . v)/2), smallp)
            const float2 e = fma2(bc2(-0.5f), fma2(us[1], q[1], fma2(us[2], q[2], mul2(us[3], q[3]))), us[4]);
            const float2 pp = mul2(bc2(gamma - 1.f), e);
            q[4] = make_float2(fmaxf(pp.x, smallp), fmaxf(pp.y, smallp));
        }
    };

    rows.begin();
    {
        float2 raw[NV], q0[NV];
        rows.fetch(ay0 - 2, raw);
        to_prim(raw, q0);
        rows.fetch(ay0 - 1, raw);
        to_prim(raw, q1);
#pragma unroll
        for (int k = 0; k < NV; ++k) dyl[k] = sub2(q1[k], q0[k]);
    }
    const int rend = ylast + 2;
#pragma unroll 1
    for (int row = ay0; row <= rend; ++row) {
        float2 q2[NV];               // primitive row P+1, straight from the staged row
        {
            float2 raw[NV];
            rows.fetch(row, raw);
            if (!rows.ok()) break;
            to_prim(raw, q2);
        }
        const int P = row - 1;
        const bool in_p = P >= ay0 && P <= ylast, in_pm = P - 1 >= ay0 && P - 1 <= ylast;   // warp-uniform
        // ---- doubled limited slopes of row P (isothermal: the pressure's are rho's times cs^2) ------
        float2 Lx[NV], Ly[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            if (k == 4 && iso) {
                Lx[4] = mul2(Lx[0], c2);
                Ly[4] = mul2(Ly[0], c2);
                continue;
            }
            const float qL = __shfl_up_sync(FULL, q1[k].y, 1), qR = __shfl_down_sync(FULL, q1[k].x, 1);
            const float mid = q1[k].y - q1[k].x;
            Lx[k] = limit2<ST>(make_float2(q1[k].x - qL, mid), make_float2(mid, qR - q1[k].y));
            const float2 dyr = sub2(q2[k], q1[k]);
            Ly[k] = limit2<ST>(dyl[k], dyr);
            dyl[k] = dyr;
        }
        // ---- predictor ------------------------------------------------------------------------
        const float2 dr = q1[0], r = add2(dr, R0), pp = iso ? mul2(r, c2) : q1[4];
        float2 u = q1[1], v = q1[2], w = q1[3];
        float2 f1 = make_float2(0.f, 0.f), f3 = make_float2(0.f, 0.f);
        if (fk) {
            const bool in_rows = P >= p.ng && P < p.ng + p.ny;   // ghost cells keep force = 0
            const float2 g1 = fma2(w, m2om, f1c), g3 = mul2(u, p2om);
            const float2 fs = in_rows ? fsel : bc2(0.f);
            f1 = mul2(g1, fs);
            f3 = mul2(g3, fs);
            const float2 hd = bc2(0.5f * dt);
            u = fma2(f1, hd, u);
            w = fma2(f3, hd, w);
        }
        // half-step sources, the half-step factors dt/(4 dx), dt/(4 dy) on the velocities
        const float2 ir = rcp2(r);
        const float2 ux = mul2(u, bc2(G.cxq)), vy = mul2(v, bc2(G.cyq));
        const float2 irx = mul2(ir, bc2(G.cxq)), iry = mul2(ir, bc2(G.cyq));
        const float2 divq = fma2(Lx[1], bc2(G.cxq), mul2(Ly[2], bc2(G.cyq)));
        float2 b[NV];
        b[0] = sub2(dr, fma2(divq, r, fma2(vy, Ly[0], mul2(ux, Lx[0]))));
        b[1] = sub2(u, fma2(Lx[4], irx, fma2(vy, Ly[1], mul2(ux, Lx[1]))));
        b[2] = sub2(v, fma2(Ly[4], iry, fma2(vy, Ly[2], mul2(ux, Lx[2]))));
        b[3] = sub2(w, fma2(vy, Ly[3], mul2(ux, Lx[3])));
        b[4] = sub2(pp, fma2(mul2(divq, bc2(gamma)), pp, fma2(vy, Ly[4], mul2(ux, Lx[4]))));
        // ---- y face below row P: (qm_y of row P-1, qp_y of row P); normal velocity vy ----------
        float2 qpy[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) qpy[k] = fma2(Ly[k], nq4, b[k]);
        if constexpr (iso) qpy[4] = mul2(c2, qpy[0]);   // godunov.f90:606-611
        else qpy[4] = make_float2(fmaxf(qpy[4].x, smallp), fmaxf(qpy[4].y, smallp));
        float2 gb[NV];
        if (row > ay0) {
            const float2 L[NV] = {add2(qmy_prev[0], R0), qmy_prev[2], qmy_prev[1], qmy_prev[3],
                                  iso ? mul2(c2, qmy_prev[0]) : qmy_prev[4]};
            const float2 R[NV] = {add2(qpy[0], R0), qpy[2], qpy[1], qpy[3], qpy[4]};
            float2 csl, csr;
            if (iso) {
                csl = c;
                csr = c;
            } else {
                csl = make_float2(sqrtf(gamma * L[4].x / L[0].x), sqrtf(gamma * L[4].y / L[0].y));
                csr = make_float2(sqrtf(gamma * R[4].x / R[0].x), sqrtf(gamma * R[4].y / R[0].y));
            }
            float2 f[NV];
            gas_flux2<GSOLV>(gamma, inv_g1, L, R, csl, csr, f, p0);
            gb[0] = f[0]; gb[2] = f[1]; gb[1] = f[2]; gb[3] = f[3]; gb[4] = f[4];
        }
#pragma unroll
        for (int k = 0; k < NV; ++k) qmy_prev[k] = fma2(Ly[k], q4, b[k]);   // qm_y of row P
        if constexpr (!iso) qmy_prev[4] = make_float2(fmaxf(qmy_prev[4].x, smallp), fmaxf(qmy_prev[4].y, smallp));
        // ---- x faces left of a and b: (qm_x of the column to the left, qp_x of the column) -------
        float2 fxl[NV];
        {
            float2 ql[NV], qpx[NV];
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                float2 qmx = fma2(Lx[k], q4, b[k]);
                qpx[k] = fma2(Lx[k], nq4, b[k]);
                if (k == 4) {
                    if constexpr (iso) {
                        qmx = mul2(c2, fma2(Lx[0], q4, b[0]));
                        qpx[4] = mul2(c2, qpx[0]);
                    } else {
                        qmx = make_float2(fmaxf(qmx.x, smallp), fmaxf(qmx.y, smallp));
                        qpx[4] = make_float2(fmaxf(qpx[4].x, smallp), fmaxf(qpx[4].y, smallp));
                    }
                }
                ql[k] = make_float2(__shfl_up_sync(FULL, qmx.y, 1), qmx.x);
            }
            ql[0] = add2(ql[0], R0);     // absolute face densities
            qpx[0] = add2(qpx[0], R0);
            float2 csl, csr;
            if (iso) {
                csl = make_float2(__shfl_up_sync(FULL, c.y, 1), c.x);
                csr = c;
            } else {
                csl = make_float2(sqrtf(gamma * ql[4].x / ql[0].x), sqrtf(gamma * ql[4].y / ql[0].y));
                csr = make_float2(sqrtf(gamma * qpx[4].x / qpx[0].x), sqrtf(gamma * qpx[4].y / qpx[0].y));
            }
            gas_flux2<GSOLV>(gamma, inv_g1, ql, qpx, csl, csr, fxl, p0);
        }
        float2 fxr[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) fxr[k] = make_float2(fxl[k].y, __shfl_down_sync(FULL, fxl[k].x, 1));
        // ---- finish row P-1 with the flux above it (every lane computes, updated columns store) --
        if (row > ay0 && in_pm) {
            const int ro = (P - 1) * pitch;
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                store_cols(dst + (voff(k) + ro), fma2(gb[k], ncyf, t_prev[k]), upd_b, upd_1);
            }
        }
        // ---- start row P: kick with the force of its old q, then the x fluxes ------------------
        if (in_p) {
#pragma unroll
            for (int k = 0; k < NV; ++k) t_prev[k] = rows.get(P, k);
            if (fk) {   // force_kicks.f90:2-41: momenta += rho dt f, energy += the kinetic change
                float2* uu = t_prev;
                const float2 iru = rcp2(uu[0]);
                const float2 eo = mul2(mul2(bc2(0.5f), fma2(uu[1], uu[1], fma2(uu[2], uu[2], mul2(uu[3], uu[3])))), iru);
                const float2 rdt = mul2(uu[0], bc2(dt));
                uu[1] = fma2(rdt, f1, uu[1]);
                uu[3] = fma2(rdt, f3, uu[3]);
                const float2 en = mul2(mul2(bc2(0.5f), fma2(uu[1], uu[1], fma2(uu[2], uu[2], mul2(uu[3], uu[3])))), iru);
                uu[4] = add2(uu[4], sub2(en, eo));
            }
#pragma unroll
            for (int k = 0; k < NV; ++k)
                t_prev[k] = fma2(gb[k], cyf, fma2(fxr[k], ncxf, fma2(fxl[k], cxf, t_prev[k])));
        }
        // ---- slide the window -----------------------------------------------------------------
#pragma unroll
        for (int k = 0; k < NV; ++k) q1[k] = q2[k];
        rows.done(row);
    }
    if (!rows.ok()) {
        if (lane == 0) atomicOr(p.status, SHARK_STATUS_COPY_WAIT);
        rows.finish();
    }
    keep_ring(rows, ra);
}

}  // namespace shark
