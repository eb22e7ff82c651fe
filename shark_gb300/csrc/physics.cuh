// physics.cuh -- device-side pointwise physics of the per-step Godunov update.
//
// Every function follows the Fortran routine it cites with the same operation order (Fortran
// evaluates `a*b*c` as (a*b)*c and `a/b*c` as (a/b)*c), so the FP64 build compiled without FMA
// contraction reproduces the CPU oracle bit for bit.  The mixed-precision build instantiates
// the same templates with float.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

namespace shark {

// 1/x for the mixed path: the FP32 reciprocal refined by one FP64 Newton step, relative error
// ~1e-14, for x within FP32 range (a handful of FP64 operations instead of a division).
__device__ __forceinline__ double rcp_refined(double x) {
    const double r = (double)(1.0f / (float)x);
    return r * (2.0 - x * r);
}

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

// FP32 forms of the three limiters for the mixed path, equal to slope_limit in exact
// arithmetic with fewer operations (single FMNMX min/max, copysign instead of a sign multiply):
//   minmod: 0 if l*r < 0, else the argument of smaller modulus (the right one on ties)
//   van Leer (harmonic): 0 if l*r <= 0, else 2 l r / (l + r)
//   MC(1.5): 0 if l*r <= 0, else sign(l+r) min(1.5 min(|l|,|r|), |l+r|/2)
__device__ __forceinline__ float limit_minmod_f(float l, float r) {
    const float m = fabsf(r) < fabsf(l) ? r : l;
    return l * r < 0.f ? 0.f : m;
}
__device__ __forceinline__ float limit_vl_f(float l, float r) {
    const float p = l * r;
    return p <= 0.f ? 0.f : 2.f * p / (l + r);
}
// min(|a|, |b|) carrying the sign sign(a) xor sign(b): >= 0 exactly when a and b have the same
// sign (or one is zero)
__device__ __forceinline__ float min_xorsign_abs_f(float a, float b) {
    float d;
    asm("min.xorsign.abs.f32 %0, %1, %2;" : "=f"(d) : "f"(a), "f"(b));
    return d;
}
// MC: sign(s) min(1.5 min(|l|, |r|), |s|/2) when l r > 0, else 0; with m = max(min.xorsign.abs(l, r), 0)
// (0 unless l and r have the same sign) it is min.xorsign.abs(1.5 m, s/2)
__device__ __forceinline__ float limit_mc_f(float l, float r) {
    // 1.5 max(mx, 0) = 0.75 (mx + |mx|) exactly (one rounding of 1.5 mx, or 0): an add with an
    // operand modifier in place of a max
    const float mx = min_xorsign_abs_f(l, r);
    return min_xorsign_abs_f(0.75f * (mx + fabsf(mx)), 0.5f * (l + r));
}

// Compile-time limiter choice (0 = first order) for kernels specialised per configuration.
template <int ST, typename R>
__device__ __forceinline__ R slope_limit_t(R l, R r) {
    if constexpr (ST == 0) return R(0);
    else if constexpr (std::is_same<R, float>::value) {
        if constexpr (ST == 1) return limit_minmod_f(l, r);
        else if constexpr (ST == 2) return limit_vl_f(l, r);
        else return limit_mc_f(l, r);
    } else return slope_limit(ST, l, r);
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

// solver_dust_Huang_Bai (src/solver/solvers.f90:506-698): pressureless upwind, 4 cases (:654-694):
// both velocities > 0 -> left flux; both < 0 -> right flux; converging (u_l > 0 > u_r) -> sum;
// diverging or any exactly-zero velocity -> 0.  Written branch-free: the left flux enters when
// u_l > 0 and u_r != 0, the right flux when u_r < 0 and u_l != 0 (same cases, same sums).
template <typename R>
__device__ __forceinline__ DustFlux<R> dust_hb(R rho_lft, R u_lft, R v_lft, R w_lft,
                                               R rho_rgt, R u_rgt, R v_rgt, R w_rgt) {
    const bool takeL = (u_lft > R(0)) && (u_rgt != R(0));
    const bool takeR = (u_rgt < R(0)) && (u_lft != R(0));
    const R ml = takeL ? rho_lft * u_lft : R(0);
    const R mr = takeR ? rho_rgt * u_rgt : R(0);
    DustFlux<R> f;
    if (takeL && takeR) {   // converging: flx_lft + flx_rgt (solvers.f90:687-691)
        f.rho = ml + mr;
        f.mn = rho_lft * sq(u_lft) + rho_rgt * sq(u_rgt);
        f.mt = ml * v_lft + mr * v_rgt;
        f.mz = ml * w_lft + mr * w_rgt;
    } else {
        const R m = takeL ? ml : mr;
        const R un = takeL ? u_lft : u_rgt, vt = takeL ? v_lft : v_rgt, wt = takeL ? w_lft : w_rgt;
        const R rh = takeL ? rho_lft : rho_rgt;
        f.rho = m;
        f.mn = (takeL || takeR) ? rh * sq(un) : R(0);
        f.mt = m * vt;
        f.mz = m * wt;
    }
    return f;
}

// FP32 Huang & Bai with selects only (mixed path); same cases as dust_hb.
__device__ __forceinline__ DustFlux<float> dust_hb_f(float rho_lft, float u_lft, float v_lft, float w_lft,
                                                     float rho_rgt, float u_rgt, float v_rgt, float w_rgt) {
    const bool takeL = (u_lft > 0.f) && (u_rgt != 0.f);
    const bool takeR = (u_rgt < 0.f) && (u_lft != 0.f);
    const float ml = takeL ? rho_lft * u_lft : 0.f;
    const float mr = takeR ? rho_rgt * u_rgt : 0.f;
    DustFlux<float> f;
    f.rho = ml + mr;
    f.mn = ml * u_lft + mr * u_rgt;
    f.mt = ml * v_lft + mr * v_rgt;
    f.mz = ml * w_lft + mr * w_rgt;
    return f;
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

// solver_hllc_dust (src/solver/solvers.f90:704-836): the gas HLLC with zero pressure on one
// pressureless species, signal speeds bounded by the gas sound speeds csl, csr of the face (the
// reference's operation order; the energies it forms do not enter the flux).
template <typename R>
__device__ __forceinline__ DustFlux<R> dust_hllc(R rho_lft, R u_lft, R v_lft, R w_lft, R rho_rgt, R u_rgt, R v_rgt,
                                                 R w_rgt, R csl, R csr) {
    const R P_rgt = R(0), P_lft = R(0);
    const R cm = fmax2(csl, csr);
    const R S_lft = fmin2(fmin2(u_lft, u_rgt) - cm, R(0));
    const R S_rgt = fmax2(fmax2(u_lft, u_rgt) + cm, R(0));
    const R hllc_l = rho_lft * (u_lft - S_lft);
    const R hllc_r = rho_rgt * (S_rgt - u_rgt);
    const R ustar = (hllc_r * u_rgt + hllc_l * u_lft + (P_lft - P_rgt)) / (hllc_r + hllc_l);
    const R Pstar = (hllc_r * P_lft + hllc_l * P_rgt + hllc_l * hllc_r * (u_lft - u_rgt)) / (hllc_r + hllc_l);
    R r_o, u_o, P_o;
    if (S_lft > R(0)) { r_o = rho_lft; u_o = u_lft; P_o = P_lft; }
    else if (ustar > R(0)) { r_o = rho_lft * (S_lft - u_lft) / (S_lft - ustar); u_o = ustar; P_o = Pstar; }
    else if (S_rgt > R(0)) { r_o = rho_rgt * (S_rgt - u_rgt) / (S_rgt - ustar); u_o = ustar; P_o = Pstar; }
    else { r_o = rho_rgt; u_o = u_rgt; P_o = P_rgt; }
    DustFlux<R> f;
    f.rho = r_o * u_o;
    f.mn = r_o * u_o * u_o + P_o;
    const bool lft = ustar > R(0);
    f.mt = r_o * u_o * (lft ? v_lft : v_rgt);
    f.mz = r_o * u_o * (lft ? w_lft : w_rgt);
    return f;
}

}  // namespace shark
