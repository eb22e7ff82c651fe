// charge.cuh -- K5: grain charging, Marchand et al. (2021) Newton on the reduced grain potential
// psi per cell (src/chemistry/ionisation.f90:4-214), optionally seeded by the charging network.
//
// One thread per cell over every cell of the grid, ghosts included (the reference's active-cell
// test is commented out).  The cell's inputs come from the conserved state at the start of the
// step through the setup's map (host-built tables):
//   nH   = rho/hs * unit_nH                  hs = sqrt(2 pi) H for the 2D polar disk, else 1
//   n_k  = rho_k/hs * unit_d / (m_k unit_m)  m_k = 4/3 pi rhograin s_k^3
//   T    = per temperature row (one row, or one per column for the disk), with the T-only
//          constants sigmav_ie, vi, tau_k, alpha_k tabulated on the host
//   zeta = chg_x, attenuated by exp(-Sigma unit_d unit_l/chg_sigma_att) for the disk.
// R = double follows the CPU oracle operation by operation (nvcc --fmad=false); R = float
// (mixed precision) runs the cold part of the iteration in FP32 and finishes it in FP64.  Outputs: psi_old (FP64, the warm start of the
// next call), zd (N planes), ni, ne, and with SHARK_CHARGE_RESISTIVITIES eta_o/H/a and gamma_d,
// plus the per-call histogram of Newton iteration counts.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/shark_gpu.h"
#include "physics.cuh"

namespace shark {

constexpr int CHARGE_HIST = SHARK_CHARGE_HIST;   // histogram bins: iterations 0..62, the last >= 63

template <typename R>
struct ChargeParams {
    const R* u;                  // state (variable planes, pitch layout)
    long long plane;
    int pitch, nx_max, ny_max, ndust, nvar;
    int t_per_col;               // 1: temperature tables per column (disk), 0: one row
    int res;                     // compute the resistivities
    int use_seed;                // 0 none, 1 seed where psi_old == 0, 2 seed always
    const double* hs;            // [nx_max] column-to-midplane factor (nullptr: 1)
    const double* trow;          // [rows][8]: T, sigmav_ie, vi, cs_T, c_el, c_ions, sigmav_el, sigmav_ions
    const double* tau;           // [rows][N]
    const double* alpha;         // [rows][N]
    const double* l2;            // [N] grain radius^2 (cm^2)
    const double* mkum;          // [N] grain mass (g)
    const double* ak;            // [N] sqrt(pi gamma/8) rhograin_cgs l_k (stopping-time numerator)
    const double* rtau;          // [rows][N] 1/tau_k        (mixed path)
    const double* nfac;          // [N] unit_d / m_k (g)     (mixed path: n_k = rho_k / hs * nfac_k)
    const double* rmk;           // [N] 1/m_k (g)            (mixed path)
    const double* pl2;           // [N] pi l_k^2             (mixed path)
    const float4* tf;            // [rows][N][2] (alpha, 1/tau, pi l^2/tau, tau), (unit_d/m, pi l^2, 1/m,
                                 // sqrt(pi gamma/8) rhograin l) in FP32 (mixed path)
    double unH, ud, ul, x0, sig_att;
    double thetai, th2, th3, psi0, eps, B0, mu_ions;
    int nitermax;
    double* psi_old;             // [plane] FP64
    R* zd;                       // [N][plane]
    R* ni;                       // [plane]
    R* ne;
    R* eta;                      // [3][plane] (o, H, a)
    R* gamma_d;                  // [N][plane]
    const float* seed;           // [plane] network start points (nullptr: none)
    int32_t* iters;              // [plane] Newton iterations of the last call
    unsigned long long* hist;    // [CHARGE_HIST + 2]: histogram, non-converged cells, total iterations
    unsigned int* status;        // the step's status word: SHARK_STATUS_NEWTON if a cell did not converge
};

namespace chg {
constexpr double pi = 3.141592653589793238462643383279;
constexpr double e_el = 4.8e-10, m_el = 9.109e-28, clight = 3e10, mH = 1.67e-24;
}

template <typename R>
__device__ __forceinline__ R dexp(R x);
template <> __device__ __forceinline__ double dexp<double>(double x) { return exp(x); }
template <> __device__ __forceinline__ float dexp<float>(float x) { return expf(x); }
template <typename R>
__device__ __forceinline__ R dsqrt_(R x);
template <> __device__ __forceinline__ double dsqrt_<double>(double x) { return sqrt(x); }
template <> __device__ __forceinline__ float dsqrt_<float>(float x) { return sqrtf(x); }

// One Newton iteration loop of ionisation.f90:79-135 in arithmetic C: iterates while
// |f(psi)| > tol and niter < nitermax, updating psi, niter, lowT and conv (|f| of the last
// evaluation).  `nk(k)` gives the grain number density of species k in C.  With stall = true the
// loop also stops when an update leaves psi unchanged (no further progress in C).
template <typename C, typename R, typename NK>
__device__ __forceinline__ void charge_newton(const ChargeParams<R>& p, const double* tau, const double* alp, NK nk,
                                              C nH, C x, C sigmav_ie, C vi, C tol, bool stall, C& psi, int& niter,
                                              int& lowT, C& conv) {
    const int N = p.ndust;
    const C pi = C(chg::pi);
    const C thetai = C(p.thetai), th2 = C(p.th2), th3 = C(p.th3), psi0 = C(p.psi0);
    const C one = C(1), two = C(2);
    const C xnH = x * nH;
    while (conv > tol && niter < p.nitermax) {
        const C eps_psi = (one - psi) / thetai * dexp<C>(-psi);
        const C et = eps_psi * thetai;
        const C et2 = et * et;
        const C om = one - eps_psi;
        const C D = (-eps_psi * (two - psi) / (one - psi));
        C S1 = C(0), S2 = C(0), S3 = C(0), S4 = C(0), S5 = C(0), S6 = C(0);
        C n_i = C(0);
        for (int k = 0; k < N; ++k) {
            const C n = nk(k), tk = C(tau[k]), ak = C(alp[k]), l2 = C(p.l2[k]);
            const C den = one + et * ak + et2;
            n_i = n_i + (-(psi * tk + (one - et2) / den) * n / om);
            const C npl = n * pi * l2;
            S1 = S1 + npl * ((one - psi) + (two / tk) * (et2 + et) / den);
            S2 = S2 + n * (-(et2 * et2) + (C(4) * th2 - th3 * ak) * (eps_psi * eps_psi) +
                           (two * thetai * ak - C(4) * th2) * eps_psi + one - thetai * ak) / (den * den);
            S3 = S3 + n * tk;
            S4 = S4 + npl / (tk * den);
            S5 = S5 + npl * (two * eps_psi * th2 + thetai * ak) / (tk * (den * den));
            S6 = S6 + npl;
        }
        const C fpsi = sigmav_ie * eps_psi * (n_i * n_i) / (xnH) + n_i * vi / (xnH) * (S1) - one;
        const C dni = -one / (om * om) * (D) * (S2) - (psi / om * (D) + one) * S3 / om;
        const C dfdpsi = sigmav_ie * n_i / (xnH) * (n_i * (D) + two * eps_psi * dni) +
                         two * n_i * vi / (xnH) * (et2 + et) *
                             ((dni / n_i + (D) * (two * et + one) / (eps_psi * (one + et))) * (S4) + ((D) * S5)) +
                         n_i * vi / (xnH) * (dni / n_i * (one - psi) - one) * (S6);
        const C prev = psi;
        psi = psi - fpsi / dfdpsi;
        if (psi < psi0) {
            psi = psi0 * C(0.9999999);
            lowT = 1;
        } else if (psi > C(0)) {
            psi = C(-1e-5);
        }
        conv = fabs(fpsi);
        niter = niter + 1;
        if (psi == prev) {
            if (stall) break;   // FP32 phase: no further progress in FP32
            // an unchanged psi with the residual above the tolerance repeats itself until
            // nitermax (e.g. the psi0 clamp): go there directly, same final state
            if (conv > tol) niter = p.nitermax;
        }
    }
}

// Compensated FP32 sum (Kahan): s + c carries the sum of the added terms to ~1 ulp.
__device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
}

// FP64 phase of the mixed path: the iteration of charge_newton with the residual f accurate to
// ~1e-8.  Its species sums split into psi-independent parts, formed once per cell in FP64,
//   T1 = sum n_k tau_k,  T3 = sum n_k pi l_k^2,
// and psi-dependent corrections of a few per cent, formed per iteration in compensated FP32,
//   T2 = sum n_k r_k,  T4 = sum n_k pi l_k^2 r_k / tau_k,   r_k = 1/(1 + et alpha_k + et^2):
//   n_i = -(psi T1 + (1 - et^2) T2)/(1 - eps),   S1 = (1 - psi) T3 + 2 (et^2 + et) T4.
// The derivative's species sums are FP32 (Newton needs f' to a few digits).  n_k = rho_k/hs
// unit_d/m_k; the FP32 sums run on rho_k unit_d/m_k and take 1/hs afterwards.  The stopping test
// |f| < chg_eps is the reference's.  `uk` points at species 0 of the cell, `tf` at the cell's row.
template <typename R>
__device__ __forceinline__ void charge_newton_mix(const ChargeParams<R>& p, const float4* tf, const R* uk,
                                                  double T1, double T3, double ihs, double nH, double x,
                                                  double sigmav_ie, double vi, double& psi, int& niter, int& lowT,
                                                  double& conv) {
    const int N = p.ndust;
    const double thetai = p.thetai, psi0 = p.psi0;
    const float thf = (float)p.thetai, th2f = (float)p.th2, th3f = (float)p.th3;
    const double rxnH = 1.0 / (x * nH);
    while (conv > p.eps && niter < p.nitermax) {
        const double eps_psi = (1.0 - psi) / thetai * exp(-psi);
        const double et = eps_psi * thetai;
        const double et2 = et * et, et21 = et2 + et, om = 1.0 - eps_psi, rom = 1.0 / om;
        const double D = (-eps_psi * (2.0 - psi) / (1.0 - psi));
        const float ef = (float)eps_psi, etf = (float)et, et2f = (float)et2;
        const float c2a = -(et2f * et2f), c2b = ef * ef, c5 = 2.f * ef * th2f;
        float T2 = 0.f, k2 = 0.f, T4 = 0.f, k4 = 0.f, S2 = 0.f, S5 = 0.f;
        for (int k = 0; k < N; ++k) {
            const float4 a = tf[2 * k], b = tf[2 * k + 1];   // (alpha, 1/tau, pi l^2/tau, tau), (unit_d/m, ...)
            const float nf = (float)uk[(long long)k * p.plane] * b.x;
            const float r = 1.f / (1.f + etf * a.x + et2f);
            const float nr = nf * r;
            kahan_add(T2, k2, nr);
            kahan_add(T4, k4, nr * a.z);
            const float f2 = (c2a + (4.f * th2f - th3f * a.x) * c2b + (2.f * thf * a.x - 4.f * th2f) * ef + 1.f - thf * a.x) * r;
            S2 = S2 + nr * f2;
            S5 = S5 + nr * a.z * (c5 + thf * a.x) * r;
        }
        const double T2d = ihs * (double)T2, T4d = ihs * (double)T4;
        const double n_i = -(psi * T1 + (1.0 - et2) * T2d) * rom;
        const double S1 = (1.0 - psi) * T3 + 2.0 * et21 * T4d;
        const double fpsi = sigmav_ie * eps_psi * (n_i * n_i) * rxnH + n_i * vi * rxnH * S1 - 1.0;
        const double S2d = ihs * (double)S2, S4d = T4d, S5d = ihs * (double)S5;
        const double dni = -(rom * rom) * D * S2d - (psi * rom * D + 1.0) * T1 * rom;
        const double dfdpsi = sigmav_ie * n_i * rxnH * (n_i * D + 2.0 * eps_psi * dni) +
                              2.0 * n_i * vi * rxnH * et21 *
                                  ((dni / n_i + D * (2.0 * et + 1.0) / (eps_psi * (1.0 + et))) * S4d + D * S5d) +
                              n_i * vi * rxnH * (dni / n_i * (1.0 - psi) - 1.0) * T3;
        const double prev = psi;
        psi = psi - fpsi / dfdpsi;
        if (psi < psi0) {
            psi = psi0 * 0.9999999;
            lowT = 1;
        } else if (psi > 0.0) {
            psi = -1e-5;
        }
        conv = fabs(fpsi);
        niter = niter + 1;
        if (psi == prev && conv > p.eps) niter = p.nitermax;
    }
}

// Outputs of the mixed path (ionisation.f90:137-206): Z_k, n_i, n_e, psi_old and, with the
// resistivities, eta_o/H/a and gamma_d.  The per-species terms are FP32 (the outputs are stored
// in FP32) with compensated sums; the cell-level electron and ion terms are FP64.
template <typename R>
__device__ __forceinline__ void charge_outputs_mix(const ChargeParams<R>& p, const float4* tf, long long c, double ihs,
                                                   double rho, double nH, double x, double sigmav_ie, const double* tr,
                                                   double psi, double eps_psi, int lowT) {
    const int N = p.ndust;
    const R* uk = p.u + 5 * p.plane + c;
    const float psif = (float)psi, e2t = (float)((eps_psi * eps_psi) * p.th2), et1 = (float)(eps_psi * p.thetai);
    float zs = 0.f, kz = 0.f;
    for (int k = 0; k < N; ++k) {
        const float4 a = tf[2 * k], b = tf[2 * k + 1];
        const float z = psif * a.w + (1.f - e2t) / (1.f + et1 * a.x + e2t);
        p.zd[(long long)k * p.plane + c] = R(z);
        kahan_add(zs, kz, z * ((float)uk[(long long)k * p.plane] * b.x));
    }
    double nsum = -(ihs * (double)zs) / (1.0 - eps_psi);
    if (lowT > 0 && N > 0) nsum = sqrt(eps_psi * x * nH / sigmav_ie);
    p.ni[c] = R(nsum);
    p.ne[c] = R(eps_psi * nsum);
    p.psi_old[c] = lowT > 0 ? p.psi0 : psi;
    if (!p.res) return;
    const double e = chg::e_el, cl = chg::clight, mel = chg::m_el, mi = p.mu_ions * chg::mH;
    const double B = p.B0 * sqrt(nH / 1e4);
    const double rnH = 1.0 / nH;
    const double t_sel = tr[4] * rnH, t_sions = tr[5] * rnH;
    const double irc = 1.0 / (rho * p.ud * tr[3]);      // t_sd = sqrt(pi gamma/8) rhograin l / (rho_cgs cs_T)
    const double sig_el = (eps_psi * nsum) * (e * e) * t_sel / mel;
    const double sig_i = (nsum) * (e * e) * t_sions / mi;
    const double om_el = -e * B / cl / mel;
    const double om_i = e * B / cl / mi;
    const float ircf = (float)irc, eBc = (float)(e * B / cl), ef = (float)e;
    float so = 0.f, ko = 0.f, sp = 0.f, kp = 0.f, sh = 0.f, kh = 0.f;
    for (int k = 0; k < N; ++k) {
        const float4 a = tf[2 * k], b = tf[2 * k + 1];
        const float z = psif * a.w + (1.f - e2t) / (1.f + et1 * a.x + e2t);
        const float t_sd = b.w * ircf;
        const float ze = z * ef;
        const float sd = ((float)uk[(long long)k * p.plane] * b.x) * b.z * (ze * ze) * t_sd;   // times 1/hs below
        const float omd = z * eBc * b.z;
        const float wt = omd * t_sd;
        const float q = 1.f / (1.f + wt * wt);
        const float h = fabsf(wt) > 1e18f ? 1.f / wt : wt * q;   // wt / (1 + wt^2) without overflow
        kahan_add(so, ko, sd);
        kahan_add(sp, kp, sd * q);
        kahan_add(sh, kh, sd * h);
        p.gamma_d[(long long)k * p.plane + c] = R(wt);
    }
    const double wi = om_i * t_sions, we = om_el * t_sel;
    const double sigma_o = ihs * (double)so + sig_i + sig_el;
    const double sigma_p = sig_i / (1.0 + wi * wi) + sig_el / (1.0 + we * we) + ihs * (double)sp;
    const double sigma_h = -sig_i * (wi) / (1.0 + wi * wi) - sig_el * (we) / (1.0 + we * we) - ihs * (double)sh;
    p.eta[c] = R(1.0 / sigma_o);
    p.eta[p.plane + c] = R(sigma_h / (sigma_p * 2.0 + sigma_h * sigma_h));
    p.eta[2 * p.plane + c] = R(sigma_p / (sigma_p * sigma_p + sigma_h * sigma_h) - 1.0 / sigma_o);
}

// K5.  R = double: the reference loop in FP64 (parity path).  R = float (mixed precision): from a
// cold or network start, FP32 Newton steps until |f| < 1e-3 or psi stops moving in FP32, then FP64
// steps to the reference tolerance chg_eps; a warm start (psi_old, FP64) goes to FP64 directly.
// The residual is steep (|df/dpsi| ~ 1e2-1e3 at the root), so an FP32 psi pins f only to ~1e-4:
// the last digits need FP64.  The iteration count is the sum of both phases.
template <typename R>
__global__ void __launch_bounds__(128) k_charge(ChargeParams<R> p) {
    const int N = p.ndust;
    const long long ncell = (long long)p.nx_max * p.ny_max;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    __shared__ unsigned int s_hist[CHARGE_HIST + 1];
    __shared__ unsigned long long s_iter;
    for (int b = threadIdx.x; b <= CHARGE_HIST; b += blockDim.x) s_hist[b] = 0u;
    if (threadIdx.x == 0) s_iter = 0ull;
    __syncthreads();
    if (t < ncell) {
        const int iy = (int)(t / p.nx_max), ix = (int)(t - (long long)iy * p.nx_max);
        const long long c = (long long)iy * p.pitch + ix;
        const int row = p.t_per_col ? ix : 0;
        const double* tr = p.trow + (size_t)row * 8;
        const double* tau = p.tau + (size_t)row * N;
        const double* alp = p.alpha + (size_t)row * N;
        // cell inputs in FP64 (the FP64 path reproduces the oracle's operation order)
        const double hs = p.hs ? p.hs[ix] : 1.0;
        const double u0 = (double)p.u[c];
        const double rho = u0 / hs;
        const double nH = rho * p.unH;
        double x = p.x0;
        if (p.sig_att > 0.0) x = p.x0 * exp(-(u0 * p.ud * p.ul) / p.sig_att);
        auto nk64 = [&](int k) -> double { return ((double)p.u[(long long)(5 + k) * p.plane + c] / hs) * p.ud / p.mkum[k]; };
        const double sigmav_ie = tr[1], vi = tr[2];
        const double thetai = p.thetai, th2 = p.th2, psi0 = p.psi0;
        double psi = psi0, conv = 1e4;
        int niter = 0, lowT = 0;
        const double pold = p.psi_old[c];
        bool cold = true;
        if (pold != 0.0) { psi = pold; cold = false; }
        if (p.seed && (p.use_seed == 2 || (p.use_seed == 1 && pold == 0.0))) {
            const float sd = p.seed[c];
            if (sd < 0.0f) { psi = (double)sd; cold = true; }
        }
        const double ihs = 1.0 / hs;
        if (sizeof(R) == 4 && cold) {
            float psif = (float)psi, convf = 1e4f;
            auto nk32 = [&](int k) -> float { return (float)((double)p.u[(long long)(5 + k) * p.plane + c] * ihs * p.nfac[k]); };
            charge_newton<float>(p, tau, alp, nk32, (float)nH, (float)x, (float)sigmav_ie, (float)vi,
                                 fmaxf((float)p.eps, 1e-3f), true, psif, niter, lowT, convf);
            psi = (double)psif;
            conv = 1e4;   // the FP64 phase re-evaluates the residual
        }
        if constexpr (sizeof(R) == 4) {
            double T1 = 0.0, T3 = 0.0;                 // psi-independent sums of the mixed iteration
            for (int k = 0; k < N; ++k) {
                const double n = (double)p.u[(long long)(5 + k) * p.plane + c] * ihs * p.nfac[k];
                T1 = T1 + n * tau[k];
                T3 = T3 + n * p.pl2[k];
            }
            charge_newton_mix(p, p.tf + (size_t)row * N * 2, p.u + 5 * p.plane + c, T1, T3, ihs, nH, x, sigmav_ie, vi,
                              psi, niter, lowT, conv);
        } else
            charge_newton<double>(p, tau, alp, nk64, nH, x, sigmav_ie, vi, p.eps, false, psi, niter, lowT, conv);
        double eps_psi = (1.0 - psi) / thetai * exp(-psi);
        if (lowT > 0) eps_psi = 0.99999;
        if constexpr (sizeof(R) == 4)
            charge_outputs_mix(p, p.tf + (size_t)row * N * 2, c, ihs, rho, nH, x, sigmav_ie, tr, psi, eps_psi, lowT);
        else {
            double nsum = 0.0;
            for (int k = 0; k < N; ++k) {
                const double tk = tau[k], ak = alp[k];
                const double z = psi * tk + (1.0 - (eps_psi * eps_psi) * th2) / (1.0 + eps_psi * thetai * ak + (eps_psi * eps_psi) * th2);
                p.zd[(long long)k * p.plane + c] = R(z);
                nsum = nsum - z * nk64(k) / (1.0 - eps_psi);
            }
            if (lowT > 0 && N > 0) nsum = sqrt(eps_psi * x * nH / sigmav_ie);
            p.ni[c] = R(nsum);
            p.ne[c] = R(eps_psi * nsum);
            p.psi_old[c] = lowT > 0 ? p.psi0 : psi;
            if (p.res) {
                // resistivities (ionisation.f90:163-206)
                const double e = chg::e_el, cl = chg::clight, mel = chg::m_el, mi = p.mu_ions * chg::mH;
                const double B = p.B0 * sqrt(nH / 1e4);
                const double cs_T = tr[3];
                const double t_sel = tr[4] / nH, t_sions = tr[5] / nH;
                const double rho_cgs = rho * p.ud;
                const double sig_el = (eps_psi * nsum) * (e * e) * t_sel / mel;
                const double sig_i = (nsum) * (e * e) * t_sions / mi;
                const double om_el = -e * B / cl / mel;
                const double om_i = e * B / cl / mi;
                double so = 0.0, sp = 0.0, sh = 0.0;
                for (int k = 0; k < N; ++k) {
                    const double tk = tau[k], ak = alp[k];
                    const double z = psi * tk + (1.0 - (eps_psi * eps_psi) * th2) / (1.0 + eps_psi * thetai * ak + (eps_psi * eps_psi) * th2);
                    const double t_sd = p.ak[k] / (rho_cgs * cs_T);
                    const double sd = nk64(k) * ((z * e) * (z * e)) * t_sd / p.mkum[k];
                    const double omd = z * e * B / cl / p.mkum[k];
                    const double wt = omd * t_sd;
                    so = so + sd;
                    sp = sp + sd / (1.0 + wt * wt);
                    sh = sh + sd * wt / (1.0 + wt * wt);
                    p.gamma_d[(long long)k * p.plane + c] = R(t_sd * omd);
                }
                const double wi = om_i * t_sions, we = om_el * t_sel;
                const double sigma_o = so + sig_i + sig_el;
                const double sigma_p = sig_i / (1.0 + wi * wi) + sig_el / (1.0 + we * we) + sp;
                const double sigma_h = -sig_i * (wi) / (1.0 + wi * wi) - sig_el * (we) / (1.0 + we * we) - sh;
                p.eta[c] = R(1.0 / sigma_o);
                p.eta[p.plane + c] = R(sigma_h / (sigma_p * 2.0 + sigma_h * sigma_h));
                p.eta[2 * p.plane + c] = R(sigma_p / (sigma_p * sigma_p + sigma_h * sigma_h) - 1.0 / sigma_o);
            }
        }
        p.iters[c] = niter;
        atomicAdd(&s_hist[niter < CHARGE_HIST - 1 ? niter : CHARGE_HIST - 1], 1u);
        if (conv > p.eps) atomicAdd(&s_hist[CHARGE_HIST], 1u);
        atomicAdd(&s_iter, (unsigned long long)niter);
    }
    __syncthreads();
    for (int b = threadIdx.x; b <= CHARGE_HIST; b += blockDim.x)
        if (s_hist[b]) atomicAdd(&p.hist[b], (unsigned long long)s_hist[b]);
    if (threadIdx.x == 0 && s_iter) atomicAdd(&p.hist[CHARGE_HIST + 1], s_iter);
    if (threadIdx.x == 0 && s_hist[CHARGE_HIST] && p.status) atomicOr(p.status, (unsigned)SHARK_STATUS_NEWTON);
}

// Fujii et al. (2011) analytical charging (ionisation.f90:809-922, functions_NR.f90:15-128,
// newton_raphson.f90:7-97): per cell and species, Newton on the grain charge Z from -1 until
// |f| < 1e-14 or 1e5 iterations, FP64 in both precisions.  f is the small difference of two
// large, nearly equal terms, so its rounding stays above 1e-14 and the reference's loop runs its
// full 1e5 iterations; restated as written.  n_i, n_e are those of the last species (the
// reference overwrites them in its species loop).
__device__ __forceinline__ double fujii_f_d(double y, double zeta, double rho, double m_d, double rho_d, double s_d,
                                            double T, double mu_gas, double mu_ions, double* fp) {
    const double mH = chg::mH, kB = 1.38e-16, e = chg::e_el, pi = chg::pi;
    const double m_i = mu_ions * mH, m_e = chg::m_el;
    const double k_e = pi * (s_d * s_d) * sqrt(8 * kB * T / (pi * m_e)) * exp((e * e) * y / (s_d * kB * T));
    const double k_i = pi * (s_d * s_d) * sqrt(8 * kB * T / (pi * m_i)) * (1 - (e * e) * y / (s_d * kB * T));
    const double a = m_d * rho / (rho_d * mu_gas * mH);
    const double f = mu_gas * mH * zeta / rho * (a * a) * ((1 / k_i) - (1 / k_e)) - y;
    if (fp) {
        const double kp_e = pi * s_d * sqrt(8 * kB * T / pi / m_e) * (e * e) / kB / T * exp((e * e) * (y) / s_d / kB / T);
        const double kp_i = -pi * s_d * sqrt(8 * kB * T / pi / m_i) * (e * e) / kB / T;
        const double b = m_d * rho / rho_d / mu_gas / mH;
        *fp = mu_gas * mH * zeta / rho * (b * b) * (kp_e / (k_e * k_e) - kp_i / (k_i * k_i)) - 1;
    }
    return f;
}

template <typename R>
__global__ void __launch_bounds__(128) k_charge_fujii(ChargeParams<R> p, double smallr, double mu_gas, double ul) {
    const int N = p.ndust;
    const long long ncell = (long long)p.nx_max * p.ny_max;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    __shared__ unsigned int s_hist[CHARGE_HIST + 1];
    __shared__ unsigned long long s_iter;
    for (int b = threadIdx.x; b <= CHARGE_HIST; b += blockDim.x) s_hist[b] = 0u;
    if (threadIdx.x == 0) s_iter = 0ull;
    __syncthreads();
    if (t < ncell) {
        const int iy = (int)(t / p.nx_max), ix = (int)(t - (long long)iy * p.nx_max);
        const long long c = (long long)iy * p.pitch + ix;
        const int row = p.t_per_col ? ix : 0;
        const double T = p.trow[(size_t)row * 8];
        const double hs = p.hs ? p.hs[ix] : 1.0;
        const double u0 = (double)p.u[c];
        double x = p.x0;
        if (p.sig_att > 0.0) x = p.x0 * exp(-(u0 * p.ud * p.ul) / p.sig_att);
        const double rho = (u0 > smallr ? u0 : smallr) / hs * p.ud;
        int total = 0;
        unsigned int nconv = 0;
        double ni = 0.0, ne = 0.0;
        for (int k = 0; k < N; ++k) {
            const double m_d = p.mkum[k];
            const double rho_d = (double)p.u[(long long)(5 + k) * p.plane + c] / hs * p.ud;
            const double s_d = sqrt(p.l2[k]);
            double y = -1.0;
            int it;
            bool conv = false;
            for (it = 1; it <= 100000; ++it) {
                double fp;
                const double fy = fujii_f_d(y, x, rho, m_d, rho_d, s_d, T, mu_gas, p.mu_ions, &fp);
                if (fabs(fy) < 1.e-14) { conv = true; break; }
                y = y - fy / fp;
            }
            if (!conv) conv = fabs(fujii_f_d(y, x, rho, m_d, rho_d, s_d, T, mu_gas, p.mu_ions, nullptr)) <= 1.e-14;
            if (!conv) ++nconv;
            total += it - 1;
            p.zd[(long long)k * p.plane + c] = R(y);
            const double mH = chg::mH, kB = 1.38e-16, e = chg::e_el, pi = chg::pi;
            const double k_e = pi * (s_d * s_d) * sqrt(8 * kB * T / (pi * chg::m_el)) * exp((e * e) * y / (s_d * kB * T));
            const double k_i = pi * (s_d * s_d) * sqrt(8 * kB * T / (pi * (p.mu_ions * mH))) * (1 - (e * e) * y / (s_d * kB * T));
            ni = x * rho * m_d / (k_i * mu_gas * mH * rho_d);
            ne = x * rho * m_d / (k_e * mu_gas * mH * rho_d);
        }
        p.ni[c] = R(ni);
        p.ne[c] = R(ne);
        p.iters[c] = total;
        atomicAdd(&s_hist[total < CHARGE_HIST - 1 ? total : CHARGE_HIST - 1], 1u);
        if (nconv) atomicAdd(&s_hist[CHARGE_HIST], nconv);
        atomicAdd(&s_iter, (unsigned long long)total);
    }
    __syncthreads();
    for (int b = threadIdx.x; b <= CHARGE_HIST; b += blockDim.x)
        if (s_hist[b]) atomicAdd(&p.hist[b], (unsigned long long)s_hist[b]);
    if (threadIdx.x == 0 && s_iter) atomicAdd(&p.hist[CHARGE_HIST + 1], s_iter);
    if (threadIdx.x == 0 && s_hist[CHARGE_HIST] && p.status) atomicOr(p.status, (unsigned)SHARK_STATUS_NEWTON);
}

// Network features of the cells (SHARK_MLP_NFEAT floats per cell, plane layout [plane][F]):
// log10 nH, log10 T, log10 zeta, log10 of the grain cross-section, radius and number per H
// (sum_k n_k pi a_k^2 / nH, sum_k n_k a_k / nH, sum_k n_k / nH).  The same state -> input map as
// k_charge.  Pad columns of the plane get zeros.
template <typename R>
__global__ void __launch_bounds__(128) k_charge_features(ChargeParams<R> p, float* __restrict__ feat) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= p.plane) return;
    const int iy = (int)(t / p.pitch), ix = (int)(t - (long long)iy * p.pitch);
    float* f = feat + t * SHARK_MLP_NFEAT;
    if (ix >= p.nx_max) {
        for (int i = 0; i < SHARK_MLP_NFEAT; ++i) f[i] = 0.0f;
        return;
    }
    const int N = p.ndust;
    const int row = p.t_per_col ? ix : 0;
    const double T = p.trow[(size_t)row * 8];
    const double hs = p.hs ? p.hs[ix] : 1.0;
    const double rho = (double)p.u[t] / hs;
    const double nH = rho * p.unH;
    double x = p.x0;
    if (p.sig_att > 0.0) x = p.x0 * exp(-((double)p.u[t] * p.ud * p.ul) / p.sig_att);
    double s2 = 0.0, s1 = 0.0, s0 = 0.0;
    for (int k = 0; k < N; ++k) {
        const double n = ((double)p.u[(long long)(5 + k) * p.plane + t] / hs) * p.ud / p.mkum[k];
        s2 += n * chg::pi * p.l2[k];
        s1 += n * sqrt(p.l2[k]);
        s0 += n;
    }
    f[0] = (float)log10(nH);
    f[1] = (float)log10(T);
    f[2] = (float)log10(x);
    f[3] = (float)log10(s2 / nH);
    f[4] = (float)log10(s1 / nH);
    f[5] = (float)log10(s0 / nH);
}

// Append (features, t = psi/psi0 - 1) of every cell the last charging call converged to the
// network's training set (cap rows of SHARK_MLP_NFEAT + 1 floats; `count` is the fill level).
template <typename R>
__global__ void k_charge_collect(ChargeParams<R> p, const float* __restrict__ feat, float* __restrict__ out,
                                 unsigned long long* count, long long cap) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= p.plane) return;
    const int iy = (int)(t / p.pitch), ix = (int)(t - (long long)iy * p.pitch);
    if (ix >= p.nx_max || iy >= p.ny_max) return;
    if (p.iters[t] >= p.nitermax) return;
    const unsigned long long slot = atomicAdd(count, 1ull);
    if ((long long)slot >= cap) return;
    float* o = out + slot * (SHARK_MLP_NFEAT + 1);
    for (int i = 0; i < SHARK_MLP_NFEAT; ++i) o[i] = feat[t * SHARK_MLP_NFEAT + i];
    o[SHARK_MLP_NFEAT] = (float)(p.psi_old[t] / p.psi0 - 1.0);
}

}  // namespace shark
