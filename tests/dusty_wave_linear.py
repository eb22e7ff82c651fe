"""Linear theory of the multi-species dusty wave (test helper).

The reference's dusty-wave problem (src/setups/DUSTYWAVE/setup.f90:12-79) is an isothermal gas of
sound speed c_s and N pressureless dust fluids coupled by drag with constant coefficients K_k
(stopping time t_k = rho_k / K_k, setup.f90:217).  Linearised about rho_g0, rho_k0 = eps_k rho_g0
and zero velocities, a perturbation ~ exp(i k x) obeys

    d(drho_g)/dt = -i k rho_g0 dv_g
    d(dv_g)/dt   = -i k c_s^2 drho_g / rho_g0 + sum_k K_k (dv_k - dv_g) / rho_g0
    d(drho_k)/dt = -i k rho_k0 dv_k
    d(dv_k)/dt   = -K_k (dv_k - dv_g) / rho_k0

i.e. y' = A y with y = (drho_g, dv_g, drho_1..N, dv_1..N).  The exact linear solution is
y(t) = expm(A t) y(0); the eigenvalues of A are the modes' growth (damping) rates and
frequencies.  A field f(x, t) = Im(y_f(t) exp(i k x)) = Re(y_f) sin kx + Im(y_f) cos kx, so the
setup's sin(k x) perturbations give y(0) real.
"""
import math

import numpy as np
import scipy.linalg as sl


def matrix(cs, rho_g, eps, K, k):
    eps, K = np.asarray(eps, float), np.asarray(K, float)
    N = eps.size
    rd = eps * rho_g
    A = np.zeros((2 + 2 * N, 2 + 2 * N), complex)
    A[0, 1] = -1j * k * rho_g
    A[1, 0] = -1j * k * cs ** 2 / rho_g
    A[1, 1] = -K.sum() / rho_g
    for i in range(N):
        A[1, 2 + N + i] = K[i] / rho_g
        A[2 + i, 2 + N + i] = -1j * k * rd[i]
        A[2 + N + i, 2 + N + i] = -K[i] / rd[i]
        A[2 + N + i, 1] = K[i] / rd[i]
    return A


def from_config(cfg):
    """(A, y0, k) for the dusty wave of ``cfg`` (setups.dustywave)."""
    N = cfg.ndust
    eps = np.array([cfg.dust_eps[i] for i in range(N)])
    K = np.array([cfg.dust_K[i] for i in range(N)])
    k = 2.0 * math.pi * cfg.dw_kx_wave / cfg.box_l
    rho0, d, v0 = cfg.dw_rho_0, cfg.dw_delta_rho, cfg.dw_vx_0
    A = matrix(cfg.cs0, rho0, eps, K, k)
    y0 = np.array([rho0 * d, v0] + list(eps * rho0 * d) + [v0] * N, complex)
    return A, y0, k


def solution(cfg, t):
    """Complex mode amplitudes of (drho_g, dv_g, drho_k, dv_k) at time t."""
    A, y0, _ = from_config(cfg)
    return sl.expm(A * t) @ y0


def rates(cfg):
    """Eigenvalues of A (damping rate = -real part, angular frequency = imaginary part)."""
    A, _, _ = from_config(cfg)
    return np.linalg.eigvals(A)


def measured_modes(cfg, u, x):
    """Complex mode amplitudes of a 1D state ``u`` (nvar, ncells, active cells only) at cell
    positions ``x``: the sin(kx) and cos(kx) projections of drho_g, v_g, drho_k, v_k."""
    _, _, k = from_config(cfg)
    N = cfg.ndust
    s, c = np.sin(k * x), np.cos(k * x)

    def mode(f):
        return 2.0 * np.mean(f * s) + 2.0j * np.mean(f * c)

    rho = u[0]
    out = [mode(rho - cfg.dw_rho_0), mode(u[1] / rho)]
    out += [mode(u[5 + i] - cfg.dust_eps[i] * cfg.dw_rho_0) for i in range(N)]
    out += [mode(u[5 + N + i] / u[5 + i]) for i in range(N)]
    return np.array(out)


def mode_errors(cfg, u_active, x, t):
    """Relative error |measured - linear| / |linear| of every mode amplitude at time t."""
    got = measured_modes(cfg, u_active, x)
    ref = solution(cfg, t)
    return np.abs(got - ref) / np.abs(ref)
