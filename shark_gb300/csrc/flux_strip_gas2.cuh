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
// transverse momentum, second transverse momentum, energy).
template <int GSOLV>
__device__ __forceinline__ void gas_flux2(float gamma, float inv_g1, const float2* L, const float2* R, float2 csl,
                                          float2 csr, float2* f) {
    const float2 rl = L[0], ul = L[1], vl = L[2], wl = L[3], pl = L[4];
    const float2 rr = R[0], ur = R[1], vr = R[2], wr = R[3], pr = R[4];
    const float2 h = bc2(0.5f);
    // E = P/(gamma-1) + rho (u^2 + v^2 + w^2)/2
    const float2 El = fma2(pl, bc2(inv_g1), mul2(mul2(h, rl), fma2(ul, ul, fma2(vl, vl, mul2(wl, wl)))));
    const float2 Er = fma2(pr, bc2(inv_g1), mul2(mul2(h, rr), fma2(ur, ur, fma2(vr, vr, mul2(wr, wr)))));
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
        float2 eo = mul2(fma2(pstar, ustar, fma2(Su, E, mul2(bc2(-1.f), mul2(P, u)))), a);
        float2 uo = ustar, po = pstar;
        const bool rx = Sr.x <= 0.f, ry = Sr.y <= 0.f;
        ro = sel2(rx, ry, rr, ro);
        uo = sel2(rx, ry, ur, uo);
        po = sel2(rx, ry, pr, po);
        eo = sel2(rx, ry, Er, eo);
        const float2 m = mul2(ro, uo);
        f[0] = m;
        f[1] = fma2(m, uo, po);
        f[4] = mul2(add2(eo, po), uo);
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
        f[4] = hll(mul2(add2(El, pl), ul), mul2(add2(Er, pr), ur), El, Er);
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
        f[4] = llf(mul2(add2(El, pl), ul), mul2(add2(Er, pr), ur), El, Er);
    }
}

// ISO: isothermal (the pressure is rho cs^2 everywhere, so it is not carried in the row window)
template <int ST, int GSOLV, bool ISO>
__device__ void flux_strip_gas2(const KParams<float>& p, int bx, int by) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int ax0 = p.ng + bx * STRIP2_UX;
    const int ga = ax0 - 2 + 2 * lane;         // this lane's columns ga, ga + 1 (ga even)
    const int ay0 = p.ng + by * STRIP_H;
    if (ay0 >= p.ng + p.ny) return;            // uniform over the warp
    const int ylast = min(ay0 + STRIP_H, p.ng + p.ny) - 1;
    const bool col_in = ga < p.nx_max;         // ga + 1 is then inside the row's pitch padding
    const int ca = min(ga, p.nx_max - 1), cb = min(ga + 1, p.nx_max - 1), cc = min(ga + 2, p.nx_max - 1);
    const bool halo = lane == 0 || lane == 31;
    const bool upd_a = !halo && ga < p.ng + p.nx, upd_b = !halo && ga + 1 < p.ng + p.nx;
    const bool act_a = ga >= p.ng && ga < p.ng + p.nx, act_b = ga + 1 >= p.ng && ga + 1 < p.ng + p.nx;

    const float dt = *p.dtf;
    const float qdt = 0.25f * dt;
    const float gamma = p.f_gamma, inv_g1 = p.f_inv_g1, smallp = p.f_smallp, smallr = p.f_smallr;
    constexpr bool iso = ISO;
    const float2 c = iso ? make_float2(p.cs[ca], p.cs[cb]) : make_float2(0.f, 0.f);
    const float2 c2 = mul2(c, c);
    const float sfa = p.sfx[ca], sfb = p.sfx[cb], sfc = p.sfx[cc];
    const float2 sfy = make_float2(p.sfy[ca], p.sfy[cb]);
    const float2 dtv = make_float2(dt * p.rvol[ca], dt * p.rvol[cb]);
    const float2 cl = mul2(make_float2(p.surf1[ca], p.surf1[cb]), dtv);
    const float2 ncr = mul2(make_float2(-p.surf1[cb], -p.surf1[cc]), dtv);
    const float2 cy = mul2(make_float2(p.surf2[ca], p.surf2[cb]), dtv), ncy = make_float2(-cy.x, -cy.y);
    const float2 hx = make_float2(0.25f * p.dx1[ca], 0.25f * p.dx1[cb]), nhx = make_float2(-hx.x, -hx.y);
    const float2 hy = make_float2(0.25f * p.dx2[ca], 0.25f * p.dx2[cb]), nhy = make_float2(-hy.x, -hy.y);
    // SI force on the gas (setup_force, species 0): f1 = 2 q om^2 xc - 2 om vz - 2 r0 om eta, f3 = 2 om vx
    const bool fk = (p.flags & SHARK_FLAG_FORCE_KICK) != 0 && p.setup == SHARK_SETUP_SI;
    const float om = p.f_si_om, qs = p.f_si_q;
    const float f1x = 2.f * qs * (om * om) * (p.xpos[ca] - p.f_half_box_l) - 2.f * p.f_si_r0 * om * p.f_si_eta;
    const float f1y = 2.f * qs * (om * om) * (p.xpos[cb] - p.f_half_box_l) - 2.f * p.f_si_r0 * om * p.f_si_eta;
    const float2 f1c = make_float2(f1x, f1y);
    const float2 m2om = bc2(-2.f * om), p2om = bc2(2.f * om);

    constexpr int NV = 5;
    float2 q0[NV], q1[NV], q2[NV];      // primitive rows P-1, P, P+1 (rho, vx, vy, vz, P)
    float2 qmy_prev[NV], t_prev[NV];   // t_prev: row P-1 after its kick, x fluxes and lower y flux
    // element offset of variable k of this lane's first column: ca + k * plane (computed per
    // access from two registers instead of holding five offsets)
    const int vpl = (int)p.plane;
    auto voff = [&](int k) { return ca + k * vpl; };
    const float* __restrict__ src = p.u_cur;
    float* __restrict__ dst = p.u_next;
    const int pitch = p.pitch;
    auto fetch_row = [&](int row, float2* us) {
        const bool in = col_in && row < p.ny_max;
        const int ro = min(row, p.ny_max - 1) * pitch;
#pragma unroll
        for (int k = 0; k < NV; ++k)
            us[k] = in ? __ldg(reinterpret_cast<const float2*>(src + (voff(k) + ro))) : make_float2(1.f, 1.f);
    };
    auto to_prim = [&](const float2* us, float2* q) {
        const float2 ir = rcp2(us[0]);
        q[1] = mul2(us[1], ir);
        q[2] = mul2(us[2], ir);
        q[3] = mul2(us[3], ir);
        if (iso) {
            q[4] = mul2(us[0], c2);
        } else {
            // P = max((gamma - 1) (E - (m . v)/2), smallp)
            const float2 e = fma2(bc2(-0.5f), fma2(us[1], q[1], fma2(us[2], q[2], mul2(us[3], q[3]))), us[4]);
            const float2 pp = mul2(bc2(gamma - 1.f), e);
            q[4] = make_float2(fmaxf(pp.x, smallp), fmaxf(pp.y, smallp));
        }
        q[0] = make_float2(fmaxf(us[0].x, smallr), fmaxf(us[0].y, smallr));
    };

    float2 raw[NV];
    fetch_row(ay0 - 2, raw);
    to_prim(raw, q0);
    fetch_row(ay0 - 1, raw);
    to_prim(raw, q1);
    float2 nxt[NV];
    fetch_row(ay0, nxt);
    const int rend = ylast + 2;
    for (int row = ay0; row <= rend; ++row) {
        to_prim(nxt, q2);
        if (row < rend) fetch_row(row + 1, nxt);
        const int P = row - 1;
        const bool in_p = P >= ay0 && P <= ylast, in_pm = P - 1 >= ay0 && P - 1 <= ylast;
        const bool start_upd = upd_a && in_p, finish_upd = upd_a && in_pm;
        float2 uu[NV];
        if (start_upd) {
#pragma unroll
            for (int k = 0; k < NV; ++k) uu[k] = __ldg(reinterpret_cast<const float2*>(src + (voff(k) + P * pitch)));
        }
        // ---- doubled limited slopes of row P (isothermal: the pressure's are rho's times cs^2) ------
        float2 Dx[NV], Dy[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            if (k == 4 && iso) {
                Dx[4] = mul2(Dx[0], c2);
                Dy[4] = mul2(Dy[0], c2);
                continue;
            }
            const float qL = __shfl_up_sync(FULL, q1[k].y, 1), qR = __shfl_down_sync(FULL, q1[k].x, 1);
            const float mid = (q1[k].y - q1[k].x) * sfb;
            Dx[k] = limit2<ST>(make_float2((q1[k].x - qL) * sfa, mid), make_float2(mid, (qR - q1[k].y) * sfc));
            Dy[k] = limit2<ST>(mul2(sub2(q1[k], q0[k]), sfy), mul2(sub2(q2[k], q1[k]), sfy));
        }
        // ---- predictor ------------------------------------------------------------------------
        const float2 r = q1[0], pp = iso ? mul2(q1[0], c2) : q1[4];
        float2 u = q1[1], v = q1[2], w = q1[3];
        float2 f1 = make_float2(0.f, 0.f), f3 = make_float2(0.f, 0.f);
        if (fk) {
            const bool in_rows = P >= p.ng && P < p.ng + p.ny;   // ghost cells keep force = 0
            const float2 g1 = fma2(w, m2om, f1c), g3 = mul2(u, p2om);
            f1 = make_float2(in_rows && act_a ? g1.x : 0.f, in_rows && act_b ? g1.y : 0.f);
            f3 = make_float2(in_rows && act_a ? g3.x : 0.f, in_rows && act_b ? g3.y : 0.f);
            const float2 hd = bc2(0.5f * dt);
            u = fma2(f1, hd, u);
            w = fma2(f3, hd, w);
        }
        // doubled sources s = -(...), as t = -2 s
        const float2 ir = rcp2(r);
        const float2 div = add2(Dx[1], Dy[2]);
        float2 t[NV];
        t[0] = fma2(div, r, fma2(v, Dy[0], mul2(u, Dx[0])));
        t[1] = fma2(Dx[4], ir, fma2(v, Dy[1], mul2(u, Dx[1])));
        t[2] = fma2(Dy[4], ir, fma2(v, Dy[2], mul2(u, Dx[2])));
        t[3] = fma2(v, Dy[3], mul2(u, Dx[3]));
        t[4] = fma2(mul2(div, bc2(gamma)), pp, fma2(v, Dy[4], mul2(u, Dx[4])));
        const float2 nq = bc2(-qdt);
        const float2 b[NV] = {fma2(t[0], nq, r), fma2(t[1], nq, u), fma2(t[2], nq, v), fma2(t[3], nq, w),
                              fma2(t[4], nq, pp)};
        float2 qmx[NV], qpx[NV], qmy[NV], qpy[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            qmx[k] = fma2(Dx[k], hx, b[k]);
            qpx[k] = fma2(Dx[k], nhx, b[k]);
            qmy[k] = fma2(Dy[k], hy, b[k]);
            qpy[k] = fma2(Dy[k], nhy, b[k]);
        }
        if constexpr (iso) {   // godunov.f90:606-611 (qm_y's is formed where it is used)
            qmx[4] = mul2(c2, qmx[0]); qpx[4] = mul2(c2, qpx[0]);
            qpy[4] = mul2(c2, qpy[0]);
        } else {
            qmx[4] = make_float2(fmaxf(qmx[4].x, smallp), fmaxf(qmx[4].y, smallp));
            qpx[4] = make_float2(fmaxf(qpx[4].x, smallp), fmaxf(qpx[4].y, smallp));
            qmy[4] = make_float2(fmaxf(qmy[4].x, smallp), fmaxf(qmy[4].y, smallp));
            qpy[4] = make_float2(fmaxf(qpy[4].x, smallp), fmaxf(qpy[4].y, smallp));
        }
        // ---- x faces left of a and b: (qm_x of the column to the left, qp_x of the column) -------
        float2 fxl[NV];
        {
            float2 ql[NV];
#pragma unroll
            for (int k = 0; k < NV; ++k) ql[k] = make_float2(__shfl_up_sync(FULL, qmx[k].y, 1), qmx[k].x);
            float2 csl, csr;
            if (iso) {
                csl = make_float2(__shfl_up_sync(FULL, c.y, 1), c.x);
                csr = c;
            } else {
                csl = make_float2(sqrtf(gamma * ql[4].x / ql[0].x), sqrtf(gamma * ql[4].y / ql[0].y));
                csr = make_float2(sqrtf(gamma * qpx[4].x / qpx[0].x), sqrtf(gamma * qpx[4].y / qpx[0].y));
            }
            gas_flux2<GSOLV>(gamma, inv_g1, ql, qpx, csl, csr, fxl);
        }
        float2 fxr[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) fxr[k] = make_float2(fxl[k].y, __shfl_down_sync(FULL, fxl[k].x, 1));
        // ---- y faces below row P: (qm_y of row P-1, qp_y of row P); normal velocity vy ----------
        float2 gb[NV];
        if (row > ay0) {
            const float2 L[NV] = {qmy_prev[0], qmy_prev[2], qmy_prev[1], qmy_prev[3],
                                  iso ? mul2(c2, qmy_prev[0]) : qmy_prev[4]};
            const float2 R[NV] = {qpy[0], qpy[2], qpy[1], qpy[3], qpy[4]};
            float2 csl, csr;
            if (iso) {
                csl = c;
                csr = c;
            } else {
                csl = make_float2(sqrtf(gamma * L[4].x / L[0].x), sqrtf(gamma * L[4].y / L[0].y));
                csr = make_float2(sqrtf(gamma * R[4].x / R[0].x), sqrtf(gamma * R[4].y / R[0].y));
            }
            float2 f[NV];
            gas_flux2<GSOLV>(gamma, inv_g1, L, R, csl, csr, f);
            gb[0] = f[0]; gb[2] = f[1]; gb[1] = f[2]; gb[3] = f[3]; gb[4] = f[4];
        }
        // ---- finish row P-1 with the flux above it -------------------------------------------
        if (row > ay0 && finish_upd) {
            const int ro = (P - 1) * pitch;
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                const float2 un = fma2(gb[k], ncy, t_prev[k]);
                if (upd_b) *reinterpret_cast<float2*>(dst + (voff(k) + ro)) = un;
                else dst[voff(k) + ro] = un.x;
            }
        }
        // ---- start row P: kick with the force of its old q, then the x fluxes ------------------
        if (start_upd) {
            if (fk) {   // force_kicks.f90:2-41: momenta += rho dt f, energy += the kinetic change
                const float2 iru = rcp2(uu[0]);
                const float2 eo = mul2(mul2(bc2(0.5f), fma2(uu[1], uu[1], fma2(uu[2], uu[2], mul2(uu[3], uu[3])))), iru);
                const float2 rdt = mul2(uu[0], bc2(dt));
                uu[1] = fma2(rdt, f1, uu[1]);
                uu[3] = fma2(rdt, f3, uu[3]);
                const float2 en = mul2(mul2(bc2(0.5f), fma2(uu[1], uu[1], fma2(uu[2], uu[2], mul2(uu[3], uu[3])))), iru);
                uu[4] = add2(uu[4], sub2(en, eo));
            }
#pragma unroll
            for (int k = 0; k < NV; ++k) uu[k] = fma2(gb[k], cy, fma2(fxr[k], ncr, fma2(fxl[k], cl, uu[k])));
        }
        // ---- slide the window -----------------------------------------------------------------
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            qmy_prev[k] = qmy[k];
            t_prev[k] = uu[k];
            q0[k] = q1[k];
            q1[k] = q2[k];
        }
    }
}

}  // namespace shark
