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

#include <algorithm>

#include "k1_schedule.h"
#include "rows.cuh"

namespace shark {

constexpr int STRIP2_UX = K1_STRIP_UX;   // columns updated per warp

__device__ __forceinline__ float2 bc2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// a - b
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }

// Doubled limited slope 2 dq of the FP32 limiters (physics.cuh) for two columns.  minmod and MC
// start from m = max(min.xorsign.abs(l, r), 0) (min_xorsign_abs_f, physics.cuh), which is
// min(|l|, |r|) when l and r have the same sign and 0 otherwise (the l r <= 0 case of the
// reference limiters); the max is taken as (mx + |mx|) / 2, folded into the factor that follows.
template <int ST>
__device__ __forceinline__ float2 limit2(float2 l, float2 r) {
    if constexpr (ST == 0) {
        return make_float2(0.f, 0.f);
    } else if constexpr (ST == 1) {   // minmod: 2 sign(l) min(|l|, |r|)
        const float2 mx = make_float2(min_xorsign_abs_f(l.x, r.x), min_xorsign_abs_f(l.y, r.y));
        // 2 max(mx, 0) = mx + |mx| exactly: a packed add (the |.| an operand modifier) instead of two
        // scalar max on the ALU pipe
        const float2 m2 = add2(mx, make_float2(fabsf(mx.x), fabsf(mx.y)));
        return make_float2(copysignf(m2.x, l.x), copysignf(m2.y, l.y));
    } else if constexpr (ST == 2) {   // van Leer: 2 (2 l r / (l + r))
        const float2 pr = mul2(l, r), s = add2(l, r);
        const float2 q = mul2(pr, make_float2(4.f / s.x, 4.f / s.y));
        return make_float2(pr.x <= 0.f ? 0.f : q.x, pr.y <= 0.f ? 0.f : q.y);
    } else {                          // MC: 2 sign(s) min(1.5 min(|l|,|r|), |s|/2) = sign(s) min(3 min, |s|)
        const float2 s = add2(l, r);
        const float2 mx = make_float2(min_xorsign_abs_f(l.x, r.x), min_xorsign_abs_f(l.y, r.y));
        // 3 max(mx, 0) = 1.5 (mx + |mx|) exactly (the same single rounding of 3 mx, or 0), packed on
        // the FMA pipe instead of two scalar max on the ALU pipe (FMNMX 8.6 -> 5.9 M per launch)
        const float2 a = mul2(add2(mx, make_float2(fabsf(mx.x), fabsf(mx.y))), bc2(1.5f));
        // sign(s) min(|s|, a) for a >= +0 is min.xorsign.abs(a, s): one instruction per column
        return make_float2(min_xorsign_abs_f(a.x, s.x), min_xorsign_abs_f(a.y, s.y));
    }
}

// Store of a lane's two updated columns of one variable: both (st2), the first alone (st1: the
// last active column when it is the first of its pair), or neither, as predicated stores with no
// branch around them.  K1 never reads the buffer it writes, so no memory ordering is asked for.
__device__ __forceinline__ void store_cols(float* ptr, float2 v, bool st2, bool st1) {
    asm volatile(
        "{\n\t.reg .pred p2, p1;\n\t"
        "setp.ne.b32 p2, %3, 0;\n\t"
        "setp.ne.b32 p1, %4, 0;\n\t"
        "@p2 st.global.v2.f32 [%0], {%1, %2};\n\t"
        "@p1 st.global.f32 [%0], %1;\n\t}" ::"l"(ptr),
        "f"(v.x), "f"(v.y), "r"((int)st2), "r"((int)st1));
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

// Arguments of a strip's row source: the tensor map of this launch's current state, the warp's
// shared-memory ring, and the ring's barrier state carried from one strip of the warp to the
// next (TmaRows: phase bits, whether the barriers are initialised, whether every wait so far
// completed).
struct RingArgs {
    const CUtensorMap* map;
    float* ring;
    uint64_t* bar;
    uint32_t phase = 0;
    bool fresh = true;
    bool good = true;
};

// The row source of a strip (overloads chosen by the type of the null first argument).
template <int NV, int R, int NST>
__device__ __forceinline__ TmaRows<NV, R, NST> make_rows_impl(TmaRows<NV, R, NST>*, const KParams<float>&,
                                                              const RingArgs& ra, int, int, bool, int x0, int r0,
                                                              int sp, int nrows) {
    TmaRows<NV, R, NST> t;
    t.map = ra.map;
    t.ring = ra.ring;
    t.bar = ra.bar;
    t.x0 = x0;
    t.r0 = r0;
    t.sp = sp;
    t.lane = threadIdx.x & 31;
    t.phase = ra.phase;
    t.fresh = ra.fresh;
    t.setup(nrows);
    return t;
}
// The ring's state after a strip, for the warp's next strip.
template <int NV, int R, int NST>
__device__ __forceinline__ void keep_ring(const TmaRows<NV, R, NST>& t, RingArgs& ra) {
    ra.phase = t.phase;
    ra.fresh = false;
    ra.good = t.good;
}
template <class Rows>
__device__ __forceinline__ Rows make_rows(const KParams<float>& p, const RingArgs& ra, int vb, int vs, bool col_in,
                                          int x0, int r0, int sp, int nrows) {
    return make_rows_impl(static_cast<Rows*>(nullptr), p, ra, vb, vs, col_in, x0, r0, sp, nrows);
}

// Scalars of a uniform Cartesian grid (every column has the same dx1, dx2, surf1, surf2, vol, as
// gridinit builds them, grid.f90:104-160): the limited slopes are formed from the raw differences
// (the limiters are homogeneous of degree one, so limit(d_l/dx, d_r/dx) dx = limit(d_l, d_r)),
// the half-step factors dt/(4 dx), dt/(4 dy) multiply the velocities once per row, and the
// update factors surf dt/vol are the same for every cell.
struct UniformGrid {
    float cxq, cyq;   // dt / (4 dx1), dt / (4 dx2): doubled slopes -> half-step source
    float cxf, cyf;   // surf1 dt / vol, surf2 dt / vol: face fluxes -> cell update
};

__device__ __forceinline__ UniformGrid uniform_grid(const KParams<float>& p, float dt) {
    const int c = p.ng;
    UniformGrid g;
    g.cxq = 0.25f * dt * p.sfx[c];          // sfx = 1/dx1 on a uniform grid
    g.cyq = 0.25f * dt * p.sfy[c];          // sfy = 1/dx2
    g.cxf = p.surf1[c] * (dt * p.rvol[c]);
    g.cyf = p.surf2[c] * (dt * p.rvol[c]);
    return g;
}

// K1 of one dust species (4 variables) on a uniform Cartesian grid, two columns per lane, rows
// ay0 .. ylast (active rows, warp-uniform).  Per row: the x differences of the row, the y
// difference to the next row (the y difference below the row is the one the previous row
// computed), the limited doubled slopes, the predictor, the four face states, the Huang & Bai
// fluxes of the x faces and of the y face below, then the row below is finished and this row
// started.  The row loop is unrolled by two, so that the row window and the other state carried
// from one row to the next alternate between two sets of registers instead of being moved
// (IMAD/MOV 12.8 -> 8.2 M per launch on the SI box, K1 0.102 -> 0.097 ms).
template <int ST, class Rows>
__device__ __forceinline__ void flux_strip_dust2(const KParams<float>& p, RingArgs& ra, int s, int bx, int ay0,
                                                 int ylast) {
    const unsigned FULL = 0xffffffffu;
    const int N = p.ndust;
    const int lane = threadIdx.x & 31;
    const int ax0 = p.ng + bx * STRIP2_UX;     // first active column updated by this warp
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
    // SI force kick on the dust (setup_force, species s >= 1): f1 = 2 q om^2 xc - 2 om vz, f3 = 2 om vx
    const bool fk = (p.flags & SHARK_FLAG_FORCE_KICK) != 0 && p.setup == SHARK_SETUP_SI;
    const float om = p.f_si_om, qs = p.f_si_q;
    const float2 f1c = make_float2(2.f * qs * (om * om) * (p.xpos[ca] - p.f_half_box_l),
                                   2.f * qs * (om * om) * (p.xpos[cb] - p.f_half_box_l));
    const float2 m2om = bc2(-2.f * om), p2om = bc2(2.f * om);
    const float2 fsel = make_float2(act_a ? 1.f : 0.f, act_b ? 1.f : 0.f);   // ghost columns: force 0

    // element offset of component k of this lane's first column: svar(s, k, N) * plane + ca
    // = vb + k * vs (species planes from a base and a stride)
    const int vb = svar(s, 0, N) * (int)p.plane + ca, vs = N * (int)p.plane;
    float* __restrict__ dst = p.u_next;
    const int pitch = p.pitch;
    Rows rows = make_rows<Rows>(p, ra, vb, vs, col_in, ax0 - 2, ay0 - 2, s - 1, ylast - ay0 + 5);
    auto to_prim = [&](const float2* us, float2* q) {
        const float2 ir = make_float2(1.f / us[0].x, 1.f / us[0].y);
        q[0] = us[0];
        q[1] = mul2(us[1], ir);
        q[2] = mul2(us[2], ir);
        q[3] = mul2(us[3], ir);
    };

    float2 q1[4];                    // primitive row P
    float2 dyl[4];                   // y difference q(P) - q(P-1)
    float2 qmy_prev[4], t_prev[4];   // t_prev: row P-1 after its kick, x fluxes and lower y flux
    rows.begin();
    {
        float2 raw[4], q0[4];
        rows.fetch(ay0 - 2, raw);
        to_prim(raw, q0);
        rows.fetch(ay0 - 1, raw);
        to_prim(raw, q1);
#pragma unroll
        for (int k = 0; k < 4; ++k) dyl[k] = sub2(q1[k], q0[k]);
    }
    const int rend = ylast + 2;
#pragma unroll 2
    for (int row = ay0; row <= rend; ++row) {
        float2 q2[4];                // primitive row P+1, straight from the staged row
        {
            float2 raw[4];
            rows.fetch(row, raw);
            if (!rows.ok()) break;
            to_prim(raw, q2);
        }
        const int P = row - 1;
        const bool in_p = P >= ay0 && P <= ylast, in_pm = P - 1 >= ay0 && P - 1 <= ylast;   // warp-uniform
        // ---- doubled limited slopes of row P (raw differences, uniform grid) ---------------------
        float2 Lx[4], Ly[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float qL = __shfl_up_sync(FULL, q1[k].y, 1), qR = __shfl_down_sync(FULL, q1[k].x, 1);
            const float mid = q1[k].y - q1[k].x;
            Lx[k] = limit2<ST>(make_float2(q1[k].x - qL, mid), make_float2(mid, qR - q1[k].y));
            const float2 dyr = sub2(q2[k], q1[k]);
            Ly[k] = limit2<ST>(dyl[k], dyr);
            dyl[k] = dyr;
        }
        // ---- predictor ------------------------------------------------------------------------
        const float2 r = q1[0];
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
        // half-step sources: -(u dq/dx + v dq/dy) dt/2 (- rho (du/dx + dv/dy) dt/2 for the density)
        const float2 ux = mul2(u, bc2(G.cxq)), vy = mul2(v, bc2(G.cyq));
        const float2 div = fma2(Lx[1], bc2(G.cxq), mul2(Ly[2], bc2(G.cyq)));
        float2 b[4];
        b[0] = sub2(r, fma2(div, r, fma2(vy, Ly[0], mul2(ux, Lx[0]))));
        b[1] = sub2(u, fma2(vy, Ly[1], mul2(ux, Lx[1])));
        b[2] = sub2(v, fma2(vy, Ly[2], mul2(ux, Lx[2])));
        b[3] = sub2(w, fma2(vy, Ly[3], mul2(ux, Lx[3])));
        // ---- y face below row P: (qm_y of row P-1, qp_y of row P); normal velocity vy ----------
        float2 qpy[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) qpy[k] = fma2(Ly[k], nq4, b[k]);
        float2 gb[4];
        if (row > ay0) {
            float2 f[4];
            hb2(qmy_prev[0], qmy_prev[2], qmy_prev[1], qmy_prev[3], qpy[0], qpy[2], qpy[1], qpy[3], f);
            gb[0] = f[0]; gb[2] = f[1]; gb[1] = f[2]; gb[3] = f[3];
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) qmy_prev[k] = fma2(Ly[k], q4, b[k]);   // qm_y of row P
        // ---- x faces left of a and b: (qm_x of the column to the left, qp_x of the column) -------
        float2 fxl[4];
        {
            float2 ql[4], qpx[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float2 qmx = fma2(Lx[k], q4, b[k]);
                qpx[k] = fma2(Lx[k], nq4, b[k]);
                ql[k] = make_float2(__shfl_up_sync(FULL, qmx.y, 1), qmx.x);
            }
            hb2(ql[0], ql[1], ql[2], ql[3], qpx[0], qpx[1], qpx[2], qpx[3], fxl);
        }
        float2 fxr[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) fxr[k] = make_float2(fxl[k].y, __shfl_down_sync(FULL, fxl[k].x, 1));
        // ---- finish row P-1 with the flux above it (every lane computes, updated columns store) --
        if (row > ay0 && in_pm) {
            const int ro = (P - 1) * pitch;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                store_cols(dst + (vb + k * vs + ro), fma2(gb[k], ncyf, t_prev[k]), upd_b, upd_1);
            }
        }
        // ---- start row P: kick with the force of its old q, then the x fluxes ------------------
        if (in_p) {
#pragma unroll
            for (int k = 0; k < 4; ++k) t_prev[k] = rows.get(P, k);
            if (fk) {
                const float2 rdt = mul2(t_prev[0], bc2(dt));
                t_prev[1] = fma2(rdt, f1, t_prev[1]);
                t_prev[3] = fma2(rdt, f3, t_prev[3]);
            }
#pragma unroll
            for (int k = 0; k < 4; ++k)
                t_prev[k] = fma2(gb[k], cyf, fma2(fxr[k], ncxf, fma2(fxl[k], cxf, t_prev[k])));
        }
        // ---- slide the window -----------------------------------------------------------------
#pragma unroll
        for (int k = 0; k < 4; ++k) q1[k] = q2[k];
        rows.done(row);
    }
    if (!rows.ok()) {
        if (lane == 0) atomicOr(p.status, SHARK_STATUS_COPY_WAIT);
        rows.finish();
    }
    keep_ring(rows, ra);
}

}  // namespace shark

#include "flux_strip_gas2.cuh"

namespace shark {

// Gas and dust of the mixed path's K1 in one launch, scheduled by k1_work (k1_schedule.h).
struct K1Maps {
    CUtensorMap gas, dust;
};

constexpr int K1_R = K1_TMA_ROWS, K1_NST = K1_TMA_STAGES;
using K1Ring = RingSize<K1_R, K1_NST, 5>;
constexpr int K1_SMEM = STRIP_WARPS * (K1Ring::ring_bytes + K1Ring::bar_bytes);

// The pieces of warp i of a class (K1Class): k1_piece (k1_schedule.h) for every phase with such a
// block; calls strip(block, first row, last row) (active-row numbering from 0) until one fails.
template <class Strip>
__device__ __forceinline__ void k1_pieces(const K1Class& c, int ny, int i, RingArgs& ra, Strip&& strip) {
    int t, r0, r1;
#pragma unroll 1
    for (int ph = 0; ra.good && k1_piece(c, ny, i, ph, t, r0, r1); ++ph) strip(t, r0, r1);
}

// blocks per SM the kernel is compiled for (4 blocks of 128 threads: 128 registers per thread)
#ifndef SHARK_K1_MINBLOCKS
#define SHARK_K1_MINBLOCKS 4
#endif
template <int NV> using K1Rows = TmaRows<NV, K1_R, K1_NST>;
// ISO: the gas is isothermal (p.iso == 1); compiled apart so that each instance inlines one gas
// strip (both in one kernel spill registers).
template <int ST, int GSOLV, bool ISO>
__global__ void __launch_bounds__(32 * STRIP_WARPS, SHARK_K1_MINBLOCKS)
    k_flux_strip_mixed(const __grid_constant__ K1Maps maps, const __grid_constant__ KParams<float> p, K1Work wk) {
    extern __shared__ __align__(128) unsigned char k1_smem[];
    const int warp = threadIdx.x >> 5;
    const int w = blockIdx.x * STRIP_WARPS + warp;
    if (w >= wk.g.n + wk.d.n) return;   // whole warps; the kernel has no block-wide barrier
    RingArgs ra;
    ra.ring = reinterpret_cast<float*>(k1_smem + warp * K1Ring::ring_bytes);
    ra.bar = reinterpret_cast<uint64_t*>(k1_smem + STRIP_WARPS * K1Ring::ring_bytes + warp * K1Ring::bar_bytes);
    const int ng = p.ng;
    if (w < wk.g.n) {
        ra.map = &maps.gas;
        using GR = K1Rows<5>;
        k1_pieces(wk.g, p.ny, w, ra, [&](int t, int r0, int r1) {
            flux_strip_gas2<ST, GSOLV, ISO, GR>(p, ra, t, ng + r0, ng + r1);
        });
    } else {
        ra.map = &maps.dust;
        const int nbx = wk.nbx;
        k1_pieces(wk.d, p.ny, w - wk.g.n, ra, [&](int t, int r0, int r1) {
            flux_strip_dust2<ST, K1Rows<4>>(p, ra, t / nbx + 1, t % nbx, ng + r0, ng + r1);
        });
    }
}

}  // namespace shark
