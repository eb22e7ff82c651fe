// growth.cuh -- dust growth (src/dust/dust_growth.f90:3-256) of one cell inside K2, after the
// drag and its floor and before setup_inloop and the CFL dt (solve.f90:112-113).
//
// Smoluchowski coagulation (and fragmentation) on the mass grid of dust_init.f90:11-45,
// sub-cycled per cell with dt_growth = CFL_growth rho_k/|drho_k/dt|.  The pair relative velocity
// (turbulent, Brownian, drift, ambipolar) is formed from the state at the start of the step
// (q velocities, stopping times) exactly as the CPU oracle (oracle/shark_oracle.cpp, growth_*)
// forms it; per-pair constants that involve no state -- the collision cross-section factor, the
// Brownian mass factor, and without fragmentation the target bins and their mass split -- are
// tabulated on the host with the oracle's operations.  The FP64 path follows the oracle's
// operations; the mixed path integrates in FP32 (growth_dv_f, growth_cell_f and the warp-per-cell
// form in the mixed K2).  A cell needing more than 100000 sub-steps stops there and raises
// SHARK_STATUS_GROWTH.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/shark_gpu.h"

namespace shark {

// largest species count of the growth kernels: one bin per lane of a warp in the mixed path, and
// per-cell pair tables in local memory in the FP64 path
constexpr int GROWTH_MAX_DUST = 32;
constexpr int GROWTH_MAX_PAIRS = GROWTH_MAX_DUST * (GROWTH_MAX_DUST + 1) / 2;

struct GrowthDev {
    int on, kernel, mode, t_per_col;
    const double* pA;        // [N*N] (clustered^2 pi)(s_k + s_j)^2
    // FP32 path.  Pairs are numbered q = k (k + 1) / 2 + j, j <= k.
    const int32_t* pair;     // [npair] k << 8 | j
    const float* pKf;        // [npair] pair rate factor pA/m_k/m_j (constant kernel 1/m_k/m_j, additive
                             // (m_k+m_j)/m_k/m_j) times mref, formed in FP64 on the host
    const float* pBf;        // [npair] (8 kB / pi) (m_k + m_j) / (m_k m_j) / uv^2, masses in g: Brownian dv^2 / T
    const int32_t* gq;       // [gL * 32] without fragmentation, entry t of bin b at t * 32 + b: a pair
    const float* gc;         //           and the net mass it moves into bin b per collision, in units of
                             //           mref (formed in FP64; 0 pads the short rows)
    int npair, gL;
    const double* pS;        // [N*N] m_k unit_m + m_j unit_m
    const double* pD;        // [N*N] m_k m_j unit_m^2
    const int32_t* pic;      // [N*N*2] target bins ic1, ic2 (1-based) without fragmentation
    const double* peps;      // [N*N] mass share of ic1 without fragmentation
    const double* mk;        // [N] grain masses (code)
    const double* sk;        // [N] grain sizes (code)
    const double* redis;     // [N*N] fragment shares: redis[ifrag * N + k]
    const double* col;       // [rows][4]: T, cs_T (cgs), cs_v (code), t_L (disk; 0 otherwise)
    double massmin, eta, m_mono, Ebr_mono, uv, uv2, ud, ut, mu_gas, dtctl, cfl, sticking, eps_thr, eps_thr_frag;
    double mref;             // mass unit of the FP32 path (the smallest grain mass): pKf is pre-multiplied
                             // and gc pre-divided by it, so code-unit masses (1e-45 in AU/Msun) stay in range
    double delta_vambi, alpha_turb, dust_ratio_min;
};

namespace grw {
constexpr double pi = 3.141592653589793238462643383279;
constexpr double kB = 1.38e-16, mH = 1.67e-24, grav = 6.67e-8, clight = 3e10;
constexpr int MAX_SUB = 100000;
}

__device__ __forceinline__ double growth_f_stokes_d(double x) {
    return (double)3.2f - 1.0 - x + 2.0 / (1. + x) * ((double)(1.0f / 2.6f) + (x * x * x) / ((double)1.6f + x));
}

__device__ __forceinline__ int growth_bin_d(double mc, double massmin, double eta, int add, int cap) {
    const int b = (int)floor(log(mc / massmin) / log(eta) + 1) + add;
    return max(min(b, cap), 1);
}

// Relative velocity of species k and j <= k (dust_growth.f90:88-114).
__device__ __forceinline__ double growth_dv_d(const GrowthDev& g, int N, int k, int j, double T, double cs_v,
                                              double t_L, double t_eta, double rm, double vambi, const double* ts,
                                              const double* vx, const double* vy, const double* vz,
                                              const double* gam) {
    const double x_stokes = ts[j] / ts[k];
    const double f_Stokes = growth_f_stokes_d(x_stokes);
    const double St1 = ts[k] / t_L, St2 = ts[j] / t_L;
    const double a = g.alpha_turb;
    double dv = 0.0;
    if (g.mode & SHARK_GROWTH_TURB) {
        double vturb = a * cs_v * sqrt(f_Stokes * St1);
        if (ts[k] < t_eta)
            vturb = a * cs_v * sqrt((St1 - St2) / (St1 + St2)) * sqrt(St1 * St1 / (St1 + rm) - St2 * St2 / (St2 + rm));
        if (ts[k] > t_L) vturb = a * cs_v * sqrt(1.0 / (1.0 + St1) + 1.0 / (1.0 + St2));
        dv = vturb;
    }
    if (g.mode & SHARK_GROWTH_BROWNIAN) {
        const double X = (8.0 * grw::kB * T / grw::pi) * g.pS[k * N + j] / g.pD[k * N + j] / g.uv2;
        const double sX = sqrt(X);
        const double vbrow = sqrt(sX * sX);
        dv = sqrt(dv * dv + vbrow * vbrow);
    }
    if (g.mode & SHARK_GROWTH_DRIFT) {
        const double dxv = vx[k] - vx[j], dyv = vy[k] - vy[j], dzv = vz[k] - vz[j];
        const double vh = sqrt(dxv * dxv + dyv * dyv + dzv * dzv);
        dv = sqrt(dv * dv + vh * vh);
    }
    if ((g.mode & SHARK_GROWTH_AMBIPOLAR) && gam) {
        const double d = vambi / g.uv * (fabs(gam[k]) / sqrt(1.0 + gam[k] * gam[k]) -
                                                fabs(gam[j]) / sqrt(1.0 + gam[j] * gam[j]));
        const double vad = sqrt(d * d);
        dv = sqrt(dv * dv + vad * vad);
    }
    return dv;
}

// FP32 constants of the pair relative velocity (dust_growth.f90:60-87): those of the run, formed
// once per thread (each is a conversion on the narrow FP64 pipe), and those of one cell.
struct GrowthRunF {
    float ud, mu_mH, ut, dvambi, alpha, inv_uv;
};
__device__ __forceinline__ GrowthRunF growth_run_consts_f(const GrowthDev& g) {
    GrowthRunF r;
    r.ud = (float)g.ud;
    r.mu_mH = (float)g.mu_gas * (float)grw::mH;
    r.ut = (float)g.ut;
    r.dvambi = (float)g.delta_vambi;
    r.alpha = (float)g.alpha_turb;
    r.inv_uv = 1.f / (float)g.uv;
    return r;
}
struct GrowthCellF {
    float T, cs_v, t_L, t_eta, rm, vambi;
};
// the temperature row's T, cs_T (cgs), cs_v (code), t_L (disk) in FP32
__device__ __forceinline__ float4 growth_row_f(const GrowthDev& g, int ix) {
    const double* cc = g.col + (size_t)(g.t_per_col ? ix : 0) * 4;
    return make_float4((float)cc[0], (float)cc[1], (float)cc[2], (float)cc[3]);
}

__device__ __forceinline__ GrowthCellF growth_cell_consts_f(const GrowthDev& g, const GrowthRunF& r, float4 row,
                                                            float rho_q, float hs, float eta_a) {
    GrowthCellF c;
    c.T = row.x;
    const float cs_T = row.y;
    c.cs_v = row.z;
    const float pi = (float)grw::pi;
    const float rho_cgs = rho_q / hs * r.ud;
    const float tff = sqrtf(3.f * pi / (32.f * (float)grw::grav * rho_cgs));
    const float lambJ = tff * cs_T;
    c.vambi = r.dvambi * (float)(grw::clight * grw::clight) * eta_a / lambJ / (4.f * pi) * r.inv_uv;
    const float Re = 6.2e7f * sqrtf(rho_cgs / r.mu_mH / 1e5f) * sqrtf(c.T / 10.f);
    c.t_L = g.t_per_col ? row.w : tff / r.ut;
    c.t_eta = c.t_L / sqrtf(Re);
    c.rm = rsqrtf(Re);
    return c;
}

// FP32 relative velocity of a pair k >= j (dust_growth.f90:88-114): stopping times tk, tj, the
// Brownian term X = T pBf, the drift (dx, dy, dz) = v_k - v_j and dg = |G_k| - |G_j| of the
// ambipolar term, G = gamma / sqrt(1 + gamma^2).
__device__ __forceinline__ float growth_dv_f(const GrowthDev& g, const GrowthRunF& r, const GrowthCellF& c, float tk,
                                             float tj, float X, float dx, float dy, float dz, float dg, bool ambi) {
    float dv = 0.f;
    if (g.mode & SHARK_GROWTH_TURB) {
        const float a = r.alpha;
        const float x = tj / tk;
        const float fS = 3.2f - 1.f - x + 2.f / (1.f + x) * (1.f / 2.6f + x * x * x / (1.6f + x));
        const float St1 = tk / c.t_L, St2 = tj / c.t_L;
        float vt = a * c.cs_v * sqrtf(fS * St1);
        if (tk < c.t_eta) {
            // both radicands are >= 0 in exact arithmetic and 0 for k == j; with contracted,
            // reciprocal-based division the second can round to -1 ulp, whose square root (NaN)
            // would floor every bin the pair touches
            const float r1 = fmaxf((St1 - St2) / (St1 + St2), 0.f);
            const float r2 = fmaxf(St1 * St1 / (St1 + c.rm) - St2 * St2 / (St2 + c.rm), 0.f);
            vt = a * c.cs_v * sqrtf(r1) * sqrtf(r2);
        }
        if (tk > c.t_L) vt = a * c.cs_v * sqrtf(1.f / (1.f + St1) + 1.f / (1.f + St2));
        dv = vt;
    }
    if (g.mode & SHARK_GROWTH_BROWNIAN) dv = sqrtf(dv * dv + X);
    if (g.mode & SHARK_GROWTH_DRIFT) dv = sqrtf(dv * dv + dx * dx + dy * dy + dz * dz);
    if ((g.mode & SHARK_GROWTH_AMBIPOLAR) && ambi) {
        const float d = c.vambi * dg;                 // vambi carries 1/unit_v
        dv = sqrtf(dv * dv + d * d);
    }
    return dv;
}

// Mixed-precision form of the cell update with fragmentation, one thread per cell (without
// fragmentation the warp-per-cell form in the mixed K2 runs instead): the same algorithm with the
// relative velocities, rates, mass bookkeeping and sub-steps in FP32 (the state is FP32 on this
// path), the elapsed growth time in FP64.  Masses are counted in units of the smallest grain mass
// and rates in grains of that mass, so the bookkeeping stays in FP32 range whatever the code units.
static __device__ __noinline__ bool growth_cell_f(const GrowthDev& g, int N, int ix, double dt, float rho_gas, float rho_q,
                                           float hs, double* rdd, const double* tsd, const double* vxd,
                                           const double* vyd, const double* vzd, const double* gamd, float eta_a) {
    const GrowthRunF rf = growth_run_consts_f(g);
    const GrowthCellF cc = growth_cell_consts_f(g, rf, growth_row_f(g, ix), rho_q, hs, eta_a);
    const bool frag = (g.mode & SHARK_GROWTH_FRAGMENTATION) != 0;
    float rd[GROWTH_MAX_DUST], ts[GROWTH_MAX_DUST], gm[GROWTH_MAX_DUST];
    for (int k = 0; k < N; ++k) {
        rd[k] = (float)rdd[k];
        ts[k] = (float)tsd[k];
        gm[k] = gamd ? fabsf((float)gamd[k]) * rsqrtf(1.f + (float)gamd[k] * (float)gamd[k]) : 0.f;
    }
    // pair rate constants pK dv / hs (and the fragmented fraction), once per cell
    float kp[GROWTH_MAX_DUST * (GROWTH_MAX_DUST + 1) / 2], fp[GROWTH_MAX_DUST * (GROWTH_MAX_DUST + 1) / 2];
    const float ihs = 1.f / hs;
    for (int k = 0, q = 0; k < N; ++k)
        for (int j = 0; j <= k; ++j, ++q) {
            float dv = 1.f;
            if (g.kernel == 0)
                dv = growth_dv_f(g, rf, cc, ts[k], ts[j], cc.T * g.pBf[q], (float)(vxd[k] - vxd[j]), (float)(vyd[k] - vyd[j]),
                                 (float)(vzd[k] - vzd[j]), gm[k] - gm[j], gamd != nullptr);
            float ff = 0.f;
            if (frag) {
                const double Ecol = 0.5 * (g.mk[k] * g.mk[j]) / (g.mk[k] + g.mk[j]) * ((double)dv * dv);
                const double Ebr = (g.mk[k] + g.mk[j]) / g.m_mono * g.Ebr_mono;
                ff = (float)fmin(fmax((Ecol - 0.1 * Ebr) / (4.9 * Ebr), 0.0), 1.0);
            }
            kp[q] = g.pKf[q] * dv * ihs * (k == j ? 0.5f : 1.f);
            fp[q] = ff;
        }
    float drhodt[GROWTH_MAX_DUST];
    double time_growth = 0.0;
    int niter = 0;
    const float st = (float)g.sticking;
    while (time_growth < dt && niter < grw::MAX_SUB) {
        for (int k = 0; k < N; ++k) drhodt[k] = 0.f;
        niter = niter + 1;
        for (int k = 0, q = 0; k < N; ++k) {
            const float m1 = (float)(g.mk[k] / g.mref);
            for (int j = 0; j <= k; ++j, ++q) {
                const float m2 = (float)(g.mk[j] / g.mref);
                float f_frag = fp[q], p_coag = 1.f;
                const float dndt = kp[q] * rd[k] * rd[j];
                if (g.kernel == 0) {
                    if (g.eps_thr > 0.0 && (rd[k] < (float)g.eps_thr * rho_gas)) p_coag = 0.f;
                    if (g.eps_thr > 0.0 && (rd[j] < (float)g.eps_thr * rho_gas)) p_coag = 0.f;
                    if (g.eps_thr_frag > 0.0 && (rd[k] < (float)g.eps_thr_frag * rho_gas)) f_frag = 0.f;
                    if (g.eps_thr_frag > 0.0 && (rd[j] < (float)g.eps_thr_frag * rho_gas)) f_frag = 0.f;
                }
                int ic1, ic2;
                float eps_m;
                if (f_frag == 0.f) {
                    ic1 = g.pic[(k * N + j) * 2];
                    ic2 = g.pic[(k * N + j) * 2 + 1];
                    eps_m = (float)g.peps[k * N + j];
                } else {
                    const double mc = (1.0 - f_frag) * (g.mk[k] + g.mk[j]);
                    ic1 = growth_bin_d(mc, g.massmin, g.eta, 0, N);
                    ic2 = growth_bin_d(mc, g.massmin, g.eta, 1, N);
                    eps_m = 1.f;
                    if (ic1 < ic2) eps_m = fminf((float)((g.mk[ic2 - 1] - mc) / (g.mk[ic2 - 1] - g.mk[ic1 - 1])), 1.f);
                }
                const float pc = p_coag * dndt, one_f = 1.f - f_frag;
                drhodt[k] -= pc * m1 * (one_f * st + f_frag);
                drhodt[j] -= pc * m2 * (one_f * st + f_frag);
                if (f_frag < 1.f) {
                    const float add = pc * one_f * (m1 + m2) * st;
                    drhodt[ic1 - 1] += eps_m * add;
                    drhodt[ic2 - 1] += (1.f - eps_m) * add;
                }
                if (frag && f_frag > 0.f && p_coag > 0.f) {
                    const int b = (int)floor(log(0.1 * f_frag * (g.mk[k] + g.mk[j]) / g.massmin) / log(g.eta) + 1);
                    const int ifrag2 = max(min(b, ic1), 1);
                    const float add = pc * f_frag * (m1 + m2);
                    for (int kd = 0; kd < ifrag2; ++kd) drhodt[kd] += add * (float)g.redis[(ifrag2 - 1) * N + kd];
                }
            }
        }
        float dtg = 1e30f;
        for (int k = 0; k < N; ++k)
            if (drhodt[k] != 0.f) dtg = fminf(dtg, rd[k] / fabsf(drhodt[k]) * (float)g.cfl);
        double dtgd = (double)dtg;
        const double rest = dt - time_growth;
        dtgd = dtgd < rest ? dtgd : rest;
        if (g.dtctl > 0.0) dtgd = g.dtctl < rest ? g.dtctl : rest;
        const float dtf = (float)dtgd, fl = rho_gas * (float)g.dust_ratio_min;
        for (int k = 0; k < N; ++k) rd[k] = fmaxf(rd[k] + drhodt[k] * dtf, fl);
        time_growth = time_growth + dtgd;
    }
    for (int k = 0; k < N; ++k) rdd[k] = (double)rd[k];
    return time_growth >= dt;
}

// Sub-cycled growth of one cell: rd[N] in/out (dust densities after the drag), rho_gas the
// conserved gas density, rho_q the floored gas density at the start of the step (q(irho)).
// The pair velocities depend only on the start of the step, so they are formed once per cell
// (the values the oracle re-forms every sub-step).  Returns false if the sub-step cap was reached.
static __device__ bool growth_cell_d(const GrowthDev& g, int N, int ix, double dt, double rho_gas, double rho_q, double hs,
                              double* rd, const double* ts, const double* vx, const double* vy, const double* vz,
                              const double* gam, double eta_a) {
    const int row = g.t_per_col ? ix : 0;
    const double* cc = g.col + (size_t)row * 4;
    const double T = cc[0], cs_T = cc[1], cs_v = cc[2];
    const double rho = rho_q / hs;
    const double rho_cgs = rho * g.ud;
    const double lambJ = sqrt(3. * grw::pi / (32. * grw::grav * rho_cgs)) * cs_T;
    const double vambi = g.delta_vambi * (grw::clight * grw::clight) * eta_a / lambJ / (4.0 * grw::pi);
    const double Re = 6.2e7 * sqrt(rho_cgs / (g.mu_gas * grw::mH) / 1e5) * sqrt(T / 10.0);
    const double t_L = g.t_per_col ? cc[3] : sqrt(3. * grw::pi / (32. * grw::grav * rho_cgs)) / g.ut;
    const double t_eta = t_L / sqrt(Re);
    const double rm = pow(Re, -0.5);
    const bool frag = (g.mode & SHARK_GROWTH_FRAGMENTATION) != 0;
    double dvp[GROWTH_MAX_DUST * (GROWTH_MAX_DUST + 1) / 2];
    for (int k = 0, q = 0; k < N; ++k)
        for (int j = 0; j <= k; ++j, ++q)
            dvp[q] = g.kernel == 0 ? growth_dv_d(g, N, k, j, T, cs_v, t_L, t_eta, rm, vambi, ts, vx, vy, vz, gam) : 0.0;
    double drhodt[GROWTH_MAX_DUST];
    double time_growth = 0.0;
    int niter = 0;
    while (time_growth < dt && niter < grw::MAX_SUB) {
        for (int k = 0; k < N; ++k) drhodt[k] = 0.0;
        niter = niter + 1;
        for (int k = 0, q = 0; k < N; ++k) {
            const double m1 = g.mk[k];
            for (int j = 0; j <= k; ++j, ++q) {
                const double m2 = g.mk[j];
                const double dv = dvp[q];
                double f_frag = 0.0, p_coag = 1.0;
                if (frag) {
                    const double Ecol = 0.5 * (m1 * m2) / (m1 + m2) * (dv * dv);
                    const double Ebr = (m1 + m2) / g.m_mono * g.Ebr_mono;
                    const double fr = (Ecol - 0.1 * Ebr) / (4.9 * Ebr);
                    const double lo = fr < 1.0 ? fr : 1.0;
                    f_frag = lo > 0.0 ? lo : 0.0;
                }
                double dndt;
                if (g.kernel == 1) dndt = rd[k] * rd[j] / m1 / m2;
                else if (g.kernel == 2) dndt = (m1 + m2) * rd[k] * rd[j] / m1 / m2;
                else dndt = g.pA[k * N + j] * dv * rd[k] * rd[j] / m1 / m2;
                dndt = dndt / hs;
                if (k == j) dndt = dndt / 2.0;
                if (g.kernel == 0) {
                    if (g.eps_thr > 0.0 && (rd[k] < g.eps_thr * rho_gas)) p_coag = 0.0;
                    if (g.eps_thr > 0.0 && (rd[j] < g.eps_thr * rho_gas)) p_coag = 0.0;
                    if (g.eps_thr_frag > 0.0 && (rd[k] < g.eps_thr_frag * rho_gas)) f_frag = 0.0;
                    if (g.eps_thr_frag > 0.0 && (rd[j] < g.eps_thr_frag * rho_gas)) f_frag = 0.0;
                }
                int ic1, ic2;
                double eps_m;
                if (f_frag == 0.0) {
                    ic1 = g.pic[(k * N + j) * 2];
                    ic2 = g.pic[(k * N + j) * 2 + 1];
                    eps_m = g.peps[k * N + j];
                } else {
                    const double mc = (1.0 - f_frag) * (m1 + m2);
                    ic1 = growth_bin_d(mc, g.massmin, g.eta, 0, N);
                    ic2 = growth_bin_d(mc, g.massmin, g.eta, 1, N);
                    eps_m = 1.0;
                    if (ic1 < ic2) {
                        const double e = (g.mk[ic2 - 1] - (1.0 - f_frag) * (m1 + m2)) / (g.mk[ic2 - 1] - g.mk[ic1 - 1]);
                        eps_m = e < 1.0 ? e : 1.0;
                    }
                }
                if (p_coag >= 0.0) {
                    const double st = g.sticking;
                    drhodt[k] = drhodt[k] - p_coag * (1.0 - f_frag) * m1 * dndt * st - p_coag * f_frag * m1 * dndt;
                    drhodt[j] = drhodt[j] - p_coag * (1.0 - f_frag) * m2 * dndt * st - p_coag * f_frag * m2 * dndt;
                    if (f_frag < 1.0) {
                        drhodt[ic1 - 1] = drhodt[ic1 - 1] + eps_m * p_coag * (1.0 - f_frag) * (m1 + m2) * dndt * st;
                        drhodt[ic2 - 1] = drhodt[ic2 - 1] + (1. - eps_m) * p_coag * (1.0 - f_frag) * (m1 + m2) * dndt * st;
                    }
                }
                if ((frag && f_frag > 0.0) && p_coag > 0.) {
                    const int b = (int)floor(log(0.1 * f_frag * (m1 + m2) / g.massmin) / log(g.eta) + 1);
                    const int ifrag2 = max(min(b, ic1), 1);
                    for (int kd = 0; kd < ifrag2; ++kd)
                        drhodt[kd] = drhodt[kd] + p_coag * f_frag * (m1 + m2) * dndt * g.redis[(ifrag2 - 1) * N + kd];
                }
            }
        }
        double dtg = 1e32;
        for (int k = 0; k < N; ++k)
            if (fabs(drhodt[k]) != 0.0) {
                const double c = rd[k] / fabs(drhodt[k]) * g.cfl;
                dtg = dtg < c ? dtg : c;
            }
        {
            const double rest = dt - time_growth;
            dtg = dtg < rest ? dtg : rest;
            if (g.dtctl > 0.0) dtg = g.dtctl < rest ? g.dtctl : rest;
        }
        for (int k = 0; k < N; ++k) {
            const double a = rd[k] + drhodt[k] * dtg, fl = rho_gas * g.dust_ratio_min;
            rd[k] = a > fl ? a : fl;
        }
        time_growth = time_growth + dtg;
    }
    return time_growth >= dt;
}

}  // namespace shark
