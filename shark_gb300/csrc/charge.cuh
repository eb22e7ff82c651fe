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
// R = double follows the CPU oracle operation by operation (nvcc --fmad=false); R = float is
// the mixed-precision form of the same iteration.  Outputs: psi_old (FP64, the warm start of the
// next call), zd (N planes), ni, ne, and with SHARK_CHARGE_RESISTIVITIES eta_o/H/a and gamma_d,
// plus the per-call histogram of Newton iteration counts.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/shark_gpu.h"

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
        const R pi = R(chg::pi);
        const R hs = p.hs ? R(p.hs[ix]) : R(1);
        const R rho = p.u[c] / hs;
        const R nH = rho * R(p.unH);
        R x = R(p.x0);
        if (p.sig_att > 0.0) x = R(p.x0) * dexp<R>(-(p.u[c] * R(p.ud) * R(p.ul)) / R(p.sig_att));
        const R sigmav_ie = R(tr[1]), vi = R(tr[2]);
        const R thetai = R(p.thetai), th2 = R(p.th2), th3 = R(p.th3), psi0 = R(p.psi0);
        const R one = R(1), two = R(2);
        const R xnH = x * nH;
        // n_k of this cell
        auto nk = [&](int k) -> R { return (p.u[(long long)(5 + k) * p.plane + c] / hs) * R(p.ud) / R(p.mkum[k]); };
        R conv = R(1e4);
        R psi = psi0;
        int niter = 0;
        const double pold = p.psi_old[c];
        if (pold != 0.0) psi = R(pold);
        if (p.seed && (p.use_seed == 2 || (p.use_seed == 1 && pold == 0.0))) {
            const float sd = p.seed[c];
            if (sd < 0.0f) psi = R(sd);
        }
        int lowT = 0;
        R eps_psi, n_i = R(0);
        while (conv > R(p.eps) && niter < p.nitermax) {
            eps_psi = (one - psi) / thetai * dexp<R>(-psi);
            const R et = eps_psi * thetai;
            const R et2 = et * et;
            const R om = one - eps_psi;
            const R D = (-eps_psi * (two - psi) / (one - psi));
            R S1 = R(0), S2 = R(0), S3 = R(0), S4 = R(0), S5 = R(0), S6 = R(0);
            n_i = R(0);
            for (int k = 0; k < N; ++k) {
                const R n = nk(k), tk = R(tau[k]), ak = R(alp[k]), l2 = R(p.l2[k]);
                const R den = one + et * ak + et2;
                n_i = n_i + (-(psi * tk + (one - et2) / den) * n / om);
                const R npl = n * pi * l2;
                S1 = S1 + npl * ((one - psi) + (two / tk) * (et2 + et) / den);
                S2 = S2 + n * (-(et2 * et2) + (R(4) * th2 - th3 * ak) * (eps_psi * eps_psi) +
                               (two * thetai * ak - R(4) * th2) * eps_psi + one - thetai * ak) / (den * den);
                S3 = S3 + n * tk;
                S4 = S4 + npl / (tk * den);
                S5 = S5 + npl * (two * eps_psi * th2 + thetai * ak) / (tk * (den * den));
                S6 = S6 + npl;
            }
            const R fpsi = sigmav_ie * eps_psi * (n_i * n_i) / (xnH) + n_i * vi / (xnH) * (S1) - one;
            const R dni = -one / (om * om) * (D) * (S2) - (psi / om * (D) + one) * S3 / om;
            const R dfdpsi = sigmav_ie * n_i / (xnH) * (n_i * (D) + two * eps_psi * dni) +
                             two * n_i * vi / (xnH) * (et2 + et) *
                                 ((dni / n_i + (D) * (two * et + one) / (eps_psi * (one + et))) * (S4) + ((D) * S5)) +
                             n_i * vi / (xnH) * (dni / n_i * (one - psi) - one) * (S6);
            psi = psi - fpsi / dfdpsi;
            if (psi < psi0) {
                psi = psi0 * R(0.9999999);
                lowT = 1;
            } else if (psi > R(0)) {
                psi = R(-1e-5);
            }
            conv = fabs(fpsi);
            niter = niter + 1;
        }
        eps_psi = (one - psi) / thetai * dexp<R>(-psi);
        if (lowT > 0) eps_psi = R(0.99999);
        R nsum = R(0);
        for (int k = 0; k < N; ++k) {
            const R tk = R(tau[k]), ak = R(alp[k]);
            const R z = psi * tk + (one - (eps_psi * eps_psi) * th2) / (one + eps_psi * thetai * ak + (eps_psi * eps_psi) * th2);
            p.zd[(long long)k * p.plane + c] = z;
            nsum = nsum - z * nk(k) / (one - eps_psi);
        }
        if (lowT > 0 && N > 0) nsum = dsqrt_<R>(eps_psi * x * nH / sigmav_ie);
        p.ni[c] = nsum;
        p.ne[c] = eps_psi * nsum;
        p.psi_old[c] = lowT > 0 ? p.psi0 : (double)psi;
        if (p.res) {
            // resistivities (ionisation.f90:163-206)
            const R e = R(chg::e_el), cl = R(chg::clight), mel = R(chg::m_el), mi = R(p.mu_ions * chg::mH);
            const R B = R(p.B0) * dsqrt_<R>(nH / R(1e4));
            const R cs_T = R(tr[3]);
            const R t_sel = R(tr[4]) / nH, t_sions = R(tr[5]) / nH;
            const R rho_cgs = rho * R(p.ud);
            const R sig_el = (eps_psi * nsum) * (e * e) * t_sel / mel;
            const R sig_i = (nsum) * (e * e) * t_sions / mi;
            const R om_el = -e * B / cl / mel;
            const R om_i = e * B / cl / mi;
            R so = R(0), sp = R(0), sh = R(0);
            for (int k = 0; k < N; ++k) {
                const R z = p.zd[(long long)k * p.plane + c];
                const R t_sd = R(p.ak[k]) / (rho_cgs * cs_T);
                const R sd = nk(k) * ((z * e) * (z * e)) * t_sd / R(p.mkum[k]);
                const R omd = z * e * B / cl / R(p.mkum[k]);
                const R wt = omd * t_sd;
                so = so + sd;
                sp = sp + sd / (one + wt * wt);
                sh = sh + sd * wt / (one + wt * wt);
                p.gamma_d[(long long)k * p.plane + c] = t_sd * omd;
            }
            const R wi = om_i * t_sions, we = om_el * t_sel;
            const R sigma_o = so + sig_i + sig_el;
            const R sigma_p = sig_i / (one + wi * wi) + sig_el / (one + we * we) + sp;
            const R sigma_h = -sig_i * (wi) / (one + wi * wi) - sig_el * (we) / (one + we * we) - sh;
            p.eta[c] = one / sigma_o;
            p.eta[p.plane + c] = sigma_h / (sigma_p * two + sigma_h * sigma_h);
            p.eta[2 * p.plane + c] = sigma_p / (sigma_p * sigma_p + sigma_h * sigma_h) - one / sigma_o;
        }
        p.iters[c] = niter;
        atomicAdd(&s_hist[niter < CHARGE_HIST - 1 ? niter : CHARGE_HIST - 1], 1u);
        if (conv > R(p.eps)) atomicAdd(&s_hist[CHARGE_HIST], 1u);
        atomicAdd(&s_iter, (unsigned long long)niter);
    }
    __syncthreads();
    for (int b = threadIdx.x; b <= CHARGE_HIST; b += blockDim.x)
        if (s_hist[b]) atomicAdd(&p.hist[b], (unsigned long long)s_hist[b]);
    if (threadIdx.x == 0 && s_iter) atomicAdd(&p.hist[CHARGE_HIST + 1], s_iter);
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
