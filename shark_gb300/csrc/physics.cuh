// physics.cuh -- device-side pointwise physics of the per-step Godunov update.
//
// Every function follows the Fortran routine it cites with the same operation order (Fortran
// evaluates `a*b*c` as (a*b)*c and `a/b*c` as (a/b)*c), so the FP64 build compiled without FMA
// contraction reproduces the CPU oracle bit for bit.  The mixed-precision build instantiates
// the same templates with float.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace shark {

template <typename R> __device__ __forceinline__ R sq(R x) { return x * x; }
// gfortran MAX/MIN on non-NaN operands
template <typename R> __device__ __forceinline__ R fmax2(R a, R b) { return a > b ? a : b; }
template <typename R> __device__ __forceinline__ R fmin2(R a, R b) { return a < b ? a : b; }
__device__ __forceinline__ float fsign1(float x) { return signbit(x) ? -1.0f : 1.0f; }
__device__ __forceinline__ double fsign1(double x) { return signbit(x) ? -1.0 : 1.0; }

// slope_limit (src/solver/slope_limiters.f90:5-37)
template <typename R>
__device__ __forceinline__ R slope_limit(int slope_type, R l, R r) {
    R s;
    if (slope_type == 1) {
        s = l;
        if (fabs(r) < fabs(l)) s = r;
        if (r * l < R(0)) s = R(0);
    } else if (slope_type == 2) {
        s = R(2) * l * r / (l + r);
        if (r * l <= R(0)) s = R(0);
    } else {
        R dcen = R(0.5) * (l + r);
        R dsgn = fsign1(dcen);
        R slop = fmin2(R(1.5) * R(fabs(l)), R(1.5) * R(fabs(r)));
        R dlim = slop;
        if ((l * r) <= R(0)) dlim = R(0);
        s = dsgn * fmin2(dlim, R(fabs(dcen)));
    }
    return s;
}

// Compile-time limiter choice (0 = first order) for kernels specialised per configuration.
template <int ST, typename R>
__device__ __forceinline__ R slope_limit_t(R l, R r) {
    if constexpr (ST == 0) return R(0);
    else return slope_limit(ST, l, r);
}

template <typename R> struct GasFlux { R rho, mn, mt, mz, e; };
template <typename R> struct DustFlux { R rho, mn, mt, mz; };

// solver_llf (src/solver/solvers.f90:4-155), non-MHD
template <typename R>
__device__ __forceinline__ GasFlux<R> gas_llf(R gamma, R rho_lft, R u_lft, R v_lft, R w_lft, R P_lft,
                                              R rho_rgt, R u_rgt, R v_rgt, R w_rgt, R P_rgt, R csl, R csr) {
    const R half = R(0.5);
    R mom_u_rgt = rho_rgt * u_rgt, mom_u_lft = rho_lft * u_lft;
    R E_rgt = P_rgt / (gamma - R(1)) + half * rho_rgt * sq(u_rgt);
    R E_lft = P_lft / (gamma - R(1)) + half * rho_lft * sq(u_lft);
    R mom_v_rgt = rho_rgt * v_rgt, mom_v_lft = rho_lft * v_lft;
    E_rgt = E_rgt + half * rho_rgt * sq(v_rgt);
    E_lft = E_lft + half * rho_lft * sq(v_lft);
    R mom_w_rgt = rho_rgt * w_rgt, mom_w_lft = rho_lft * w_lft;
    E_rgt = E_rgt + half * rho_rgt * sq(w_rgt);
    E_lft = E_lft + half * rho_lft * sq(w_lft);
    R flx_rho_rgt = rho_rgt * u_rgt, flx_rho_lft = rho_lft * u_lft;
    R flx_mom_u_rgt = (rho_rgt * sq(u_rgt) + P_rgt), flx_mom_u_lft = (rho_lft * sq(u_lft) + P_lft);
    R flx_mom_v_rgt = rho_rgt * u_rgt * v_rgt, flx_mom_v_lft = rho_lft * u_lft * v_lft;
    R flx_mom_w_rgt = rho_rgt * u_rgt * w_rgt, flx_mom_w_lft = rho_lft * u_lft * w_lft;
    R flx_P_rgt = (E_rgt + P_rgt) * u_rgt, flx_P_lft = (E_lft + P_lft) * u_lft;
    R lam = fmax2(R(fabs(u_lft)) + csl, R(fabs(u_rgt)) + csr);
    GasFlux<R> f;
    f.rho = half * (flx_rho_lft + flx_rho_rgt) - half * lam * (rho_rgt - rho_lft);
    f.mn = half * (flx_mom_u_lft + flx_mom_u_rgt) - half * lam * (mom_u_rgt - mom_u_lft);
    f.mt = half * (flx_mom_v_lft + flx_mom_v_rgt) - half * lam * (mom_v_rgt - mom_v_lft);
    f.mz = half * (flx_mom_w_lft + flx_mom_w_rgt) - half * lam * (mom_w_rgt - mom_w_lft);
    f.e = half * (flx_P_lft + flx_P_rgt) - half * lam * (E_rgt - E_lft);
    return f;
}

// solver_hll (src/solver/solvers.f90:157-306), non-MHD
template <typename R>
__device__ __forceinline__ GasFlux<R> gas_hll(R gamma, R rho_lft, R u_lft, R v_lft, R w_lft, R P_lft,
                                              R rho_rgt, R u_rgt, R v_rgt, R w_rgt, R P_rgt, R csl, R csr) {
    const R half = R(0.5);
    R mom_u_rgt = rho_rgt * u_rgt, mom_u_lft = rho_lft * u_lft;
    R E_rgt = P_rgt / (gamma - R(1)) + half * rho_rgt * sq(u_rgt);
    R E_lft = P_lft / (gamma - R(1)) + half * rho_lft * sq(u_lft);
    R mom_v_rgt = rho_rgt * v_rgt, mom_v_lft = rho_lft * v_lft;
    E_rgt = E_rgt + half * rho_rgt * sq(v_rgt);
    E_lft = E_lft + half * rho_lft * sq(v_lft);
    R mom_w_rgt = rho_rgt * w_rgt, mom_w_lft = rho_lft * w_lft;
    E_rgt = E_rgt + half * rho_rgt * sq(w_rgt);
    E_lft = E_lft + half * rho_lft * sq(w_lft);
    R flx_rho_rgt = rho_rgt * u_rgt, flx_rho_lft = rho_lft * u_lft;
    R flx_mom_u_rgt = (rho_rgt * sq(u_rgt) + P_rgt), flx_mom_u_lft = (rho_lft * sq(u_lft) + P_lft);
    R flx_mom_v_rgt = rho_rgt * u_rgt * v_rgt, flx_mom_v_lft = rho_lft * u_lft * v_lft;
    R flx_mom_w_rgt = rho_rgt * u_rgt * w_rgt, flx_mom_w_lft = rho_lft * u_lft * w_lft;
    R flx_P_rgt = (E_rgt + P_rgt) * u_rgt, flx_P_lft = (E_lft + P_lft) * u_lft;
    R S_lft = fmin2(fmin2(u_lft, u_rgt) - fmax2(csl, csr), R(0));
    R S_rgt = fmax2(fmax2(u_lft, u_rgt) + fmax2(csl, csr), R(0));
    GasFlux<R> f;
    f.rho = (S_rgt * flx_rho_lft - S_lft * flx_rho_rgt + S_rgt * S_lft * (rho_rgt - rho_lft)) / (S_rgt - S_lft);
    f.mn = (S_rgt * flx_mom_u_lft - S_lft * flx_mom_u_rgt + S_rgt * S_lft * (mom_u_rgt - mom_u_lft)) / (S_rgt - S_lft);
    f.mt = (S_rgt * flx_mom_v_lft - S_lft * flx_mom_v_rgt + S_rgt * S_lft * (mom_v_rgt - mom_v_lft)) / (S_rgt - S_lft);
    f.mz = (S_rgt * flx_mom_w_lft - S_lft * flx_mom_w_rgt + S_rgt * S_lft * (mom_w_rgt - mom_w_lft)) / (S_rgt - S_lft);
    f.e = (S_rgt * flx_P_lft - S_lft * flx_P_rgt + S_rgt * S_lft * (E_rgt - E_lft)) / (S_rgt - S_lft);
    return f;
}

// solver_hllc (src/solver/solvers.f90:308-500): RAMSES-style HLLC with the wave speeds clipped to
// include 0 (:435-436), Lagrangian star state (:450-463), sampling at x/t = 0 (:466-486) and the
// passive transverse momenta upwinded on the sign of u* (:491-497).
template <typename R>
__device__ __forceinline__ GasFlux<R> gas_hllc(R gamma, R rho_lft, R u_lft, R v_lft, R w_lft, R P_lft,
                                               R rho_rgt, R u_rgt, R v_rgt, R w_rgt, R P_rgt, R csl, R csr) {
    const R half = R(0.5);
    R E_rgt = P_rgt / (gamma - R(1)) + half * rho_rgt * sq(u_rgt) + half * rho_rgt * sq(v_rgt) + half * rho_rgt * sq(w_rgt);
    R E_lft = P_lft / (gamma - R(1)) + half * rho_lft * sq(u_lft) + half * rho_lft * sq(v_lft) + half * rho_lft * sq(w_lft);
    R S_lft = fmin2(fmin2(u_lft, u_rgt) - fmax2(csl, csr), R(0));
    R S_rgt = fmax2(fmax2(u_lft, u_rgt) + fmax2(csl, csr), R(0));
    R hllc_l = rho_lft * (u_lft - S_lft);
    R hllc_r = rho_rgt * (S_rgt - u_rgt);
    R ustar = (hllc_r * u_rgt + hllc_l * u_lft + (P_lft - P_rgt)) / (hllc_r + hllc_l);
    R Pstar = (hllc_r * P_lft + hllc_l * P_rgt + hllc_l * hllc_r * (u_lft - u_rgt)) / (hllc_r + hllc_l);
    R r_o, u_o, P_o, e_o;
    if (S_lft > R(0)) {
        r_o = rho_lft; u_o = u_lft; P_o = P_lft; e_o = E_lft;
    } else if (ustar > R(0)) {
        r_o = rho_lft * (S_lft - u_lft) / (S_lft - ustar);
        u_o = ustar; P_o = Pstar;
        e_o = ((S_lft - u_lft) * E_lft - P_lft * u_lft + Pstar * ustar) / (S_lft - ustar);
    } else if (S_rgt > R(0)) {
        r_o = rho_rgt * (S_rgt - u_rgt) / (S_rgt - ustar);
        u_o = ustar; P_o = Pstar;
        e_o = ((S_rgt - u_rgt) * E_rgt - P_rgt * u_rgt + Pstar * ustar) / (S_rgt - ustar);
    } else {
        r_o = rho_rgt; u_o = u_rgt; P_o = P_rgt; e_o = E_rgt;
    }
    GasFlux<R> f;
    f.rho = r_o * u_o;
    f.mn = r_o * u_o * u_o + P_o;
    f.e = (e_o + P_o) * u_o;
    if (ustar > R(0)) { f.mt = r_o * u_o * v_lft; f.mz = r_o * u_o * w_lft; }
    else { f.mt = r_o * u_o * v_rgt; f.mz = r_o * u_o * w_rgt; }
    return f;
}

// solver_dust_Huang_Bai (src/solver/solvers.f90:506-698): pressureless upwind, 4 cases (:654-694)
template <typename R>
__device__ __forceinline__ DustFlux<R> dust_hb(R rho_lft, R u_lft, R v_lft, R w_lft,
                                               R rho_rgt, R u_rgt, R v_rgt, R w_rgt) {
    DustFlux<R> f{R(0), R(0), R(0), R(0)};
    const bool lp = u_lft > R(0), ln = u_lft < R(0), rp = u_rgt > R(0), rn = u_rgt < R(0);
    if (rp && lp) {
        f.rho = rho_lft * u_lft; f.mn = rho_lft * sq(u_lft);
        f.mt = rho_lft * u_lft * v_lft; f.mz = rho_lft * u_lft * w_lft;
    } else if (ln && rn) {
        f.rho = rho_rgt * u_rgt; f.mn = rho_rgt * sq(u_rgt);
        f.mt = rho_rgt * u_rgt * v_rgt; f.mz = rho_rgt * u_rgt * w_rgt;
    } else if (lp && rn) {
        f.rho = rho_lft * u_lft + rho_rgt * u_rgt;
        f.mn = rho_lft * sq(u_lft) + rho_rgt * sq(u_rgt);
        f.mt = rho_lft * u_lft * v_lft + rho_rgt * u_rgt * v_rgt;
        f.mz = rho_lft * u_lft * w_lft + rho_rgt * u_rgt * w_rgt;
    }
    return f;   // diverging (ln && rp) or any zero velocity: zero flux
}

// solver_dust_llf (src/solver/solvers.f90:840-1001), non-MHD
template <typename R>
__device__ __forceinline__ DustFlux<R> dust_llf(R rho_lft, R u_lft, R v_lft, R w_lft,
                                                R rho_rgt, R u_rgt, R v_rgt, R w_rgt) {
    const R half = R(0.5);
    R lam = fmax2(R(fabs(u_lft)), R(fabs(u_rgt)));
    DustFlux<R> f;
    f.rho = half * (rho_lft * u_lft + rho_rgt * u_rgt) - half * lam * (rho_rgt - rho_lft);
    f.mn = half * (rho_lft * sq(u_lft) + rho_rgt * sq(u_rgt)) - half * lam * (rho_rgt * u_rgt - rho_lft * u_lft);
    f.mt = half * (rho_lft * u_lft * v_lft + rho_rgt * u_rgt * v_rgt) - half * lam * (rho_rgt * v_rgt - rho_lft * v_lft);
    f.mz = half * (rho_lft * u_lft * w_lft + rho_rgt * u_rgt * w_rgt) - half * lam * (rho_rgt * w_rgt - rho_lft * w_lft);
    return f;
}

// solver_dust_hll (src/solver/solvers.f90:1010-1194), non-MHD
template <typename R>
__device__ __forceinline__ DustFlux<R> dust_hll(R rho_lft, R u_lft, R v_lft, R w_lft,
                                                R rho_rgt, R u_rgt, R v_rgt, R w_rgt) {
    R S_lft = fmin2(fmin2(u_lft, u_rgt), R(0));
    R S_rgt = fmax2(fmax2(u_lft, u_rgt), R(0));
    DustFlux<R> f{R(0), R(0), R(0), R(0)};
    if (S_rgt - S_lft != R(0)) {
        f.rho = (S_rgt * (rho_lft * u_lft) - S_lft * (rho_rgt * u_rgt) + S_rgt * S_lft * (rho_rgt - rho_lft)) / (S_rgt - S_lft);
        f.mn = (S_rgt * (rho_lft * sq(u_lft)) - S_lft * (rho_rgt * sq(u_rgt)) + S_rgt * S_lft * (rho_rgt * u_rgt - rho_lft * u_lft)) / (S_rgt - S_lft);
        f.mt = (S_rgt * (rho_lft * u_lft * v_lft) - S_lft * (rho_rgt * u_rgt * v_rgt) + S_rgt * S_lft * (rho_rgt * v_rgt - rho_lft * v_lft)) / (S_rgt - S_lft);
        f.mz = (S_rgt * (rho_lft * u_lft * w_lft) - S_lft * (rho_rgt * u_rgt * w_rgt) + S_rgt * S_lft * (rho_rgt * w_rgt - rho_lft * w_lft)) / (S_rgt - S_lft);
    }
    return f;
}

}  // namespace shark
