// flux_strip2.cuh -- K1 for the dust species of the mixed path on 2D Cartesian grids: the column
// march of flux_strip.cuh with TWO adjacent columns per lane.
//
// Lane l owns columns (a, b) = (c0 + 2l, c0 + 2l + 1) of one species, c0 even; lanes 0 and 31
// are the x halo, so 60 columns per warp are updated.  Every FP32 operation of the cell
// algorithm is issued once for both columns as a packed FP32x2 instruction (__fadd2_rn,
// __fmul2_rn, __ffma2_rn); loads and stores move both columns in one 64-bit access; the x
// neighbours across lanes need one shuffle per variable and direction for the pair.  Comparisons,
// min/max and selects stay per column.
//
// Algorithm: as flux_strip.cuh's FP32 path (ctoprim solve.f90:195-253, predictor
// godunov.f90:7-629, Huang & Bai dust fluxes solvers.f90:506-698, add_delta_u
// godunov.f90:659-750, kick force_kicks.f90:2-41).  The limited slopes are carried doubled
// (2 dq) and the half-step factors halved to match, which saves a multiply per slope; the
// limiters are the FP32 forms of physics.cuh on the doubled slopes.
#pragma once

namespace shark {

constexpr int STRIP2_UX = 60;    // columns updated per warp

__device__ __forceinline__ float2 bc2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// a - b
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }

// Doubled limited slope 2 dq of the FP32 limiters (physics.cuh) for two columns.
template <int ST>
__device__ __forceinline__ float2 limit2(float2 l, float2 r) {
    if constexpr (ST == 0) {
        return make_float2(0.f, 0.f);
    } else if constexpr (ST == 1) {   // minmod
        const float2 pr = mul2(l, r);
        const float mx = fabsf(r.x) < fabsf(l.x) ? r.x : l.x, my = fabsf(r.y) < fabsf(l.y) ? r.y : l.y;
        const float2 m = make_float2(pr.x < 0.f ? 0.f : mx, pr.y < 0.f ? 0.f : my);
        return add2(m, m);
    } else if constexpr (ST == 2) {   // van Leer: 2 (2 l r / (l + r))
        const float2 pr = mul2(l, r), s = add2(l, r);
        const float2 q = mul2(pr, make_float2(4.f / s.x, 4.f / s.y));
        return make_float2(pr.x <= 0.f ? 0.f : q.x, pr.y <= 0.f ? 0.f : q.y);
    } else {                          // MC: 2 sign(s) min(1.5 min(|l|,|r|), |s|/2) = sign(s) min(3 min, |s|)
        const float2 pr = mul2(l, r), s = add2(l, r);
        const float2 t = mul2(make_float2(fminf(fabsf(l.x), fabsf(r.x)), fminf(fabsf(l.y), fabsf(r.y))), bc2(3.f));
        const float mx = copysignf(fminf(t.x, fabsf(s.x)), s.x), my = copysignf(fminf(t.y, fabsf(s.y)), s.y);
        return make_float2(pr.x <= 0.f ? 0.f : mx, pr.y <= 0.f ? 0.f : my);
    }
}

// Huang & Bai dust flux (dust_hb_f) of two faces: f = (mass, normal momentum, transverse 1, 2).
__device__ __forceinline__ void hb2(float2 rL, float2 uL, float2 vL, float2 wL, float2 rR, float2 uR, float2 vR,
                                    float2 wR, float2* f) {
    const float2 mlf = mul2(rL, uL), mrf = mul2(rR, uR);
    const float2 ml = make_float2((uL.x > 0.f && uR.x != 0.f) ? mlf.x : 0.f, (uL.y > 0.f && uR.y != 0.f) ? mlf.y : 0.f);
    const float2 mr = make_float2((uR.x < 0.f && uL.x != 0.f) ? mrf.x : 0.f, (uR.y < 0.f && uL.y != 0.f) ? mrf.y : 0.f);
    f[0] = add2(ml, mr);
    f[1] = fma2(mr, uR, mul2(ml, uL));
    f[2] = fma2(mr, vR, mul2(ml, vL));
    f[3] = fma2(mr, wR, mul2(ml, wL));
}

template <int ST>
__device__ void flux_strip_dust2(const KParams<float>& p, int s, int bx, int by) {
    const unsigned FULL = 0xffffffffu;
    const int N = p.ndust;
    const int lane = threadIdx.x & 31;
    const int ax0 = p.ng + bx * STRIP2_UX;     // first active column updated by this warp
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
    // column tables: x-face factors of the faces left of a, between a and b, right of b
    const float sfa = p.sfx[ca], sfb = p.sfx[cb], sfc = p.sfx[cc];
    const float2 sfy = make_float2(p.sfy[ca], p.sfy[cb]);
    const float2 dtv = make_float2(dt * p.rvol[ca], dt * p.rvol[cb]);
    const float2 cl = mul2(make_float2(p.surf1[ca], p.surf1[cb]), dtv);           // left x faces
    const float2 ncr = mul2(make_float2(-p.surf1[cb], -p.surf1[cc]), dtv);        // right x faces, negated
    const float2 cy = mul2(make_float2(p.surf2[ca], p.surf2[cb]), dtv), ncy = make_float2(-cy.x, -cy.y);
    const float2 hx = make_float2(0.25f * p.dx1[ca], 0.25f * p.dx1[cb]), nhx = make_float2(-hx.x, -hx.y);
    const float2 hy = make_float2(0.25f * p.dx2[ca], 0.25f * p.dx2[cb]), nhy = make_float2(-hy.x, -hy.y);
    // SI force kick on the dust (setup_force, species s >= 1): f1 = 2 q om^2 xc - 2 om vz, f3 = 2 om vx
    const bool fk = (p.flags & SHARK_FLAG_FORCE_KICK) != 0 && p.setup == SHARK_SETUP_SI;
    const float om = p.f_si_om, qs = p.f_si_q;
    const float2 f1c = make_float2(2.f * qs * (om * om) * (p.xpos[ca] - p.f_half_box_l),
                                   2.f * qs * (om * om) * (p.xpos[cb] - p.f_half_box_l));
    const float2 m2om = bc2(-2.f * om), p2om = bc2(2.f * om);

    float2 q0[4], q1[4], q2[4];      // primitive rows P-1, P, P+1
    float2 qmy_prev[4], t_prev[4];   // t_prev: row P-1 after its kick, x fluxes and lower y flux
    // element offset of component k of this lane's first column, svar(s, k, N) * plane + ca,
    // from a base and a stride (two registers instead of four offsets)
    const int vbase = svar(s, 0, N) * (int)p.plane + ca, vstride = N * (int)p.plane;
    auto voff = [&](int k) { return vbase + k * vstride; };
    const float* __restrict__ src = p.u_cur;
    float* __restrict__ dst = p.u_next;
    const int pitch = p.pitch;
    auto fetch_row = [&](int row, float2* us) {
        const bool in = col_in && row < p.ny_max;
        const int ro = min(row, p.ny_max - 1) * pitch;
#pragma unroll
        for (int k = 0; k < 4; ++k)
            us[k] = in ? __ldg(reinterpret_cast<const float2*>(src + (voff(k) + ro))) : make_float2(1.f, 1.f);
    };
    auto to_prim = [&](const float2* us, float2* q) {
        const float2 ir = make_float2(1.f / us[0].x, 1.f / us[0].y);
        q[0] = us[0];
        q[1] = mul2(us[1], ir);
        q[2] = mul2(us[2], ir);
        q[3] = mul2(us[3], ir);
    };

    float2 raw[4];
    fetch_row(ay0 - 2, raw);
    to_prim(raw, q0);
    fetch_row(ay0 - 1, raw);
    to_prim(raw, q1);
    float2 nxt[4];
    fetch_row(ay0, nxt);
    const int rend = ylast + 2;
    for (int row = ay0; row <= rend; ++row) {
        to_prim(nxt, q2);
        if (row < rend) fetch_row(row + 1, nxt);
        const int P = row - 1;
        const bool in_p = P >= ay0 && P <= ylast, in_pm = P - 1 >= ay0 && P - 1 <= ylast;
        const bool start_upd = upd_a && in_p, finish_upd = upd_a && in_pm;
        float2 uu[4];
        if (start_upd) {
#pragma unroll
            for (int k = 0; k < 4; ++k) uu[k] = __ldg(reinterpret_cast<const float2*>(src + (voff(k) + P * pitch)));
        }
        // ---- doubled limited slopes of row P -----------------------------------------------------
        float2 Dx[4], Dy[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float qL = __shfl_up_sync(FULL, q1[k].y, 1), qR = __shfl_down_sync(FULL, q1[k].x, 1);
            const float mid = (q1[k].y - q1[k].x) * sfb;
            Dx[k] = limit2<ST>(make_float2((q1[k].x - qL) * sfa, mid), make_float2(mid, (qR - q1[k].y) * sfc));
            Dy[k] = limit2<ST>(mul2(sub2(q1[k], q0[k]), sfy), mul2(sub2(q2[k], q1[k]), sfy));
        }
        // ---- predictor ------------------------------------------------------------------------
        const float2 r = q1[0];
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
        // doubled sources: s = -(u dq/dx + v dq/dy) (- rho (du/dx + dv/dy) for the density)
        const float2 tr = fma2(add2(Dx[1], Dy[2]), r, fma2(v, Dy[0], mul2(u, Dx[0])));
        const float2 tu = fma2(v, Dy[1], mul2(u, Dx[1]));
        const float2 tv = fma2(v, Dy[2], mul2(u, Dx[2]));
        const float2 tw = fma2(v, Dy[3], mul2(u, Dx[3]));
        const float2 nq = bc2(-qdt);
        float2 b[4];
        b[0] = fma2(tr, nq, r);
        b[1] = fma2(tu, nq, u);
        b[2] = fma2(tv, nq, v);
        b[3] = fma2(tw, nq, w);
        float2 qmx[4], qpx[4], qmy[4], qpy[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            qmx[k] = fma2(Dx[k], hx, b[k]);
            qpx[k] = fma2(Dx[k], nhx, b[k]);
            qmy[k] = fma2(Dy[k], hy, b[k]);
            qpy[k] = fma2(Dy[k], nhy, b[k]);
        }
        // ---- x faces left of a and b: (qm_x of the column to the left, qp_x of the column) -------
        float2 ql[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) ql[k] = make_float2(__shfl_up_sync(FULL, qmx[k].y, 1), qmx[k].x);
        float2 fxl[4];
        hb2(ql[0], ql[1], ql[2], ql[3], qpx[0], qpx[1], qpx[2], qpx[3], fxl);
        float2 fxr[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) fxr[k] = make_float2(fxl[k].y, __shfl_down_sync(FULL, fxl[k].x, 1));
        // ---- y faces below row P: (qm_y of row P-1, qp_y of row P); normal velocity vy ----------
        float2 gb[4];
        if (row > ay0) {
            float2 f[4];
            hb2(qmy_prev[0], qmy_prev[2], qmy_prev[1], qmy_prev[3], qpy[0], qpy[2], qpy[1], qpy[3], f);
            gb[0] = f[0]; gb[2] = f[1]; gb[1] = f[2]; gb[3] = f[3];
        }
        // ---- finish row P-1 with the flux above it -------------------------------------------
        if (row > ay0 && finish_upd) {
            const int ro = (P - 1) * pitch;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float2 un = fma2(gb[k], ncy, t_prev[k]);
                if (upd_b) *reinterpret_cast<float2*>(dst + (voff(k) + ro)) = un;
                else dst[voff(k) + ro] = un.x;
            }
        }
        // ---- start row P: kick with the force of its old q, then the x fluxes ------------------
        if (start_upd) {
            if (fk) {
                const float2 rdt = mul2(uu[0], bc2(dt));
                uu[1] = fma2(rdt, f1, uu[1]);
                uu[3] = fma2(rdt, f3, uu[3]);
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) uu[k] = fma2(gb[k], cy, fma2(fxr[k], ncr, fma2(fxl[k], cl, uu[k])));
        }
        // ---- slide the window -----------------------------------------------------------------
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            qmy_prev[k] = qmy[k];
            t_prev[k] = uu[k];
            q0[k] = q1[k];
            q1[k] = q2[k];
        }
    }
}

}  // namespace shark

#include "flux_strip_gas2.cuh"

namespace shark {

// Gas and dust of the mixed path's K1 in one launch: blocks 0 .. ng-1 take the gas strips, the
// rest the dust strips of every species, both 60 columns per warp.  The gas blocks come first in
// the launch order, so the gas grid runs beside the dust instead of after it.
template <int ST, int GSOLV>
__global__ void __launch_bounds__(32 * STRIP_WARPS, 4) k_flux_strip_mixed(KParams<float> p, int nbx_g, int nbx_d, int nby) {
    const int warp = threadIdx.x >> 5;
    const int id = blockIdx.x, ngas = nbx_g * nby;
    if (id < ngas) {
        if (p.iso == 1) flux_strip_gas2<ST, GSOLV, true>(p, id % nbx_g, (id / nbx_g) * STRIP_WARPS + warp);
        else flux_strip_gas2<ST, GSOLV, false>(p, id % nbx_g, (id / nbx_g) * STRIP_WARPS + warp);
    } else {
        const int d = id - ngas, bx = d % nbx_d, rest = d / nbx_d;
        flux_strip_dust2<ST>(p, rest / nby + 1, bx, (rest % nby) * STRIP_WARPS + warp);
    }
}

}  // namespace shark
