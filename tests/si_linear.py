"""Linear theory of the streaming instability in the reference's SI box (test helper).

The SI setup (src/setups/SI/setup.f90) is a 2D axisymmetric shearing box: x radial (ivx), y
vertical (ivy, the grid's second axis), z azimuthal (ivz, out of the plane), with the shear
velocity q Omega x carried in the z momenta and the forces of setup_force
(SI/setup.f90:335-350): gas a_x = 2 q Omega^2 x - 2 Omega v_z - 2 r0 Omega eta, a_z = 2 Omega v_x;
dust the same without the pressure-gradient term; drag (rho_d/rho_g)(v_d - v_g)/t_k on the gas
and (v_g - v_d)/t_k on species k; isothermal gas of sound speed c_s.

With the velocities measured from the shear flow (v_z = q Omega x + w), the equilibrium is the
multi-species Nakagawa-Sekiya-Hayashi drift (uniform densities, constant velocities; solved here
as the linear system it is), and a perturbation ~ exp(i (k_x x + k_y y) + s t) obeys y' = A y with
y = (drho_g, dv_gx, dv_gy, dw_g, then per species drho_k, dv_kx, dv_ky, dw_k):

    s drho   = -i k_x U drho - i rho (k_x dv_x + k_y dv_y)            (U: the fluid's radial drift)
    s dv_x   = -i k_x U dv_x - 2 Omega dw + [gas: - i k_x c_s^2 drho_g/rho_g] + drag_x
    s dv_y   = -i k_x U dv_y + [gas: - i k_y c_s^2 drho_g/rho_g] + drag_y
    s dw     = -i k_x U dw + (2 - q) Omega dv_x + drag_z

where the gas drag perturbation also carries the change of rho_k/rho_g times the equilibrium
relative velocity.  The largest real part of the eigenvalues of A is the growth rate; in the
incompressible limit it reproduces the published linA and linB rates (Youdin & Johansen 2007).
"""
import numpy as np


def equilibrium(eps, ts, eta, vk=1.0, omega=1.0, q=1.5):
    """Radial drift U and azimuthal velocity w (relative to the shear) of the gas and of every
    species in the drag-force equilibrium of the SI box's equations (uniform densities)."""
    eps, ts = np.asarray(eps, float), np.asarray(ts, float)
    N = eps.size
    n = 2 + 2 * N
    M = np.zeros((n, n))
    b = np.zeros(n)
    # gas x: 0 = -2 Omega w_g - 2 eta vk Omega + sum eps_k (U_k - U_g)/t_k
    M[0, 1] = -2.0 * omega
    b[0] = 2.0 * eta * vk * omega
    # gas z: 0 = (2 - q) Omega U_g + sum eps_k (w_k - w_g)/t_k
    M[1, 0] = (2.0 - q) * omega
    for i in range(N):
        M[0, 2 + i] += eps[i] / ts[i]
        M[0, 0] -= eps[i] / ts[i]
        M[1, 2 + N + i] += eps[i] / ts[i]
        M[1, 1] -= eps[i] / ts[i]
        # dust x: 0 = -2 Omega w_k + (U_g - U_k)/t_k ; z: 0 = (2 - q) Omega U_k + (w_g - w_k)/t_k
        r = 2 + 2 * i                   # species i: x and z equations
        M[r, 2 + N + i] = -2.0 * omega
        M[r, 0] = 1.0 / ts[i]
        M[r, 2 + i] = -1.0 / ts[i]
        M[r + 1, 2 + i] = (2.0 - q) * omega
        M[r + 1, 1] = 1.0 / ts[i]
        M[r + 1, 2 + N + i] = -1.0 / ts[i]
    sol = np.linalg.solve(M, b)
    return sol[0], sol[1], sol[2:2 + N], sol[2 + N:2 + 2 * N]


def matrix(kx, ky, cs, rho_g, eps, ts, eta, vk=1.0, omega=1.0, q=1.5):
    eps, ts = np.asarray(eps, float), np.asarray(ts, float)
    N = eps.size
    Ug, wg, Ud, wd = equilibrium(eps, ts, eta, vk, omega, q)
    rd = eps * rho_g
    n = 4 + 4 * N
    A = np.zeros((n, n), complex)
    # gas
    A[0, 0] = -1j * kx * Ug
    A[0, 1] = -1j * rho_g * kx
    A[0, 2] = -1j * rho_g * ky
    A[1, 1] = -1j * kx * Ug
    A[1, 0] = -1j * kx * cs ** 2 / rho_g
    A[1, 3] = -2.0 * omega
    A[2, 2] = -1j * kx * Ug
    A[2, 0] = -1j * ky * cs ** 2 / rho_g
    A[3, 3] = -1j * kx * Ug
    A[3, 1] = (2.0 - q) * omega
    for i in range(N):
        d = 4 + 4 * i
        t = ts[i]
        # gas drag: (rho_k/rho_g)(v_k - v_g)/t_k, perturbed
        for c, dc in ((1, 1), (2, 2), (3, 3)):
            A[c, d + dc] += eps[i] / t
            A[c, c] -= eps[i] / t
        dU, dW = Ud[i] - Ug, wd[i] - wg      # equilibrium relative velocity (x, z)
        A[1, d] += dU / t / rho_g
        A[1, 0] -= rd[i] * dU / t / rho_g ** 2
        A[3, d] += dW / t / rho_g
        A[3, 0] -= rd[i] * dW / t / rho_g ** 2
        # dust
        A[d, d] = -1j * kx * Ud[i]
        A[d, d + 1] = -1j * rd[i] * kx
        A[d, d + 2] = -1j * rd[i] * ky
        A[d + 1, d + 1] = -1j * kx * Ud[i] - 1.0 / t
        A[d + 1, d + 3] = -2.0 * omega
        A[d + 1, 1] = 1.0 / t
        A[d + 2, d + 2] = -1j * kx * Ud[i] - 1.0 / t
        A[d + 2, 2] = 1.0 / t
        A[d + 3, d + 3] = -1j * kx * Ud[i] - 1.0 / t
        A[d + 3, d + 1] = (2.0 - q) * omega
        A[d + 3, 3] = 1.0 / t
    return A


def fastest_mode(kx, ky, cs, rho_g, eps, ts, eta, vk=1.0, omega=1.0, q=1.5):
    """(growth rate, frequency, eigenvector) of the fastest-growing mode."""
    A = matrix(kx, ky, cs, rho_g, eps, ts, eta, vk, omega, q)
    lam, V = np.linalg.eig(A)
    i = int(np.argmax(lam.real))
    return lam[i].real, lam[i].imag, V[:, i]


def mode_amplitude(field, x, y, kx, ky):
    """Complex amplitude a of a real field f = Re(a exp(i (k_x x + k_y y))) + background, from
    the cell values over whole wavelengths."""
    ph = np.exp(-1j * (kx * x + ky * y))
    return 2.0 * np.mean((field - field.mean()) * ph)


def eigenmode_box(n, stokes=0.1, eps=3.0, K=30.0, eta=0.05, amp=1e-5, precision=0):
    """The SI setup (one dust species, force kick, drag with back-reaction) on an n x n box of one
    wavelength 2 pi eta r0 / K in each direction, in the drag equilibrium plus the fastest linear
    mode with |drho_d| = amp rho_d.  The reference's own initial drift (NSH with A/(A + B) where
    the drag equilibrium has A/(A^2 + B^2)) is not an equilibrium, so the background is the
    solution of `equilibrium`.  eta = 0.05 with the setup's c_s = 0.1 v_K keeps the sound
    crossing (and so the step count) moderate; the theory is the compressible one.

    Returns (cfg, u0, growth rate, k, x, y) with x, y the cell centres."""
    import math
    from shark_gb300 import setups
    cfg, _ = setups.si(n=16, ndust=1, precision=precision, noise=0.0)
    cfg.nx = cfg.ny = n
    om, qs, cs = cfg.si_omega, cfg.si_q_shear, cfg.cs0
    vk = cfg.si_rad0 * om
    cfg.si_eta_stream = eta
    cfg.dust_tstop[0] = stokes / om
    cfg.dust_eps[0] = eps
    cfg.dust_stokes[0] = stokes
    k = K / (eta * cfg.si_rad0)
    cfg.box_l = cfg.box_l_y = 2.0 * math.pi / k
    s, _, V = fastest_mode(k, k, cs, cfg.si_rho_init, [eps], [stokes / om], eta, vk=vk, omega=om, q=qs)
    V = V / V[4] * (amp * eps * cfg.si_rho_init)
    Ug, wg, Ud, wd = equilibrium([eps], [stokes / om], eta, vk=vk, omega=om, q=qs)
    pos = setups.positions(cfg)
    x, y = pos[:, 0], pos[:, 1]
    xx = x - 0.5 * cfg.box_l
    ph = np.exp(1j * (k * x + k * y))
    f = lambda c: (c * ph).real
    q = np.zeros((cfg.nvar, cfg.ncells))
    q[0] = cfg.si_rho_init + f(V[0])
    q[1] = Ug + f(V[1])
    q[2] = f(V[2])
    q[3] = qs * om * xx + wg + f(V[3])
    q[4] = q[0] * cs ** 2
    q[5] = eps * cfg.si_rho_init + f(V[4])
    q[6] = Ud[0] + f(V[5])
    q[7] = f(V[6])
    q[8] = qs * om * xx + wd[0] + f(V[7])
    u = setups.primtoc(cfg, q).reshape(-1)
    setups.si_boundaries(cfg, u)
    return cfg, u, s, k, x, y


def dust_mode(cfg, u, x, y, k):
    """|complex amplitude| of the dust density's mode over the active cells."""
    ng = cfg.nghost
    act = np.zeros((cfg.ny_max, cfg.nx_max), bool)
    act[ng:ng + cfg.ny, ng:ng + cfg.nx] = True
    act = act.reshape(-1)
    g = u.reshape(cfg.nvar, -1)
    return abs(mode_amplitude(g[5][act], x[act], y[act], k, k))
