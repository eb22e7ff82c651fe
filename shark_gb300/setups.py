"""Host-side setup builders: the run configuration and the initial conserved state of the
in-scope problems, written with numpy the way the reference's ``setup`` routines build them.

Each builder returns ``(cfg, u0)`` where ``cfg`` is a :class:`SharkConfig` and ``u0`` is the
conserved state ``u_prim(1:ncells,1:nvar)`` in Fortran order flattened to a 1-D float64 array
(variable-major, ``u0[v*ncells + i]``).  These are the inputs the Fortran driver would hand to
the GPU library after its own ``setup``; they are not part of the per-step hot path.

References: src/setups/SOD/setup.f90:1-46, src/setups/DUSTYWAVE/setup.f90:12-79,
src/setups/SI/setup.f90:1-117, src/dust/dust_init.f90:11-103,164-197 (MRN bins),
src/grid/grid.f90:104-173 (positions), src/solver/solve.f90:265-302 (primtoc).
"""
import numpy as np

import math

from .config import (SharkConfig, default_config, SETUP_SOD, SETUP_DUSTYWAVE, SETUP_SI, SETUP_DISK_POLAR,
                     SETUP_DUSTYTURB, SETUP_KH, SETUP_SEDOV, SETUP_DISK_CART, FLAG_DRAG, FLAG_VISCOSITY, FLAG_BACK_REACTION, FLAG_FORCE_KICK, FLAG_FARGO,
                     FLAG_CHARGING, FLAG_GROWTH, GROWTH_TURB, GROWTH_BROWNIAN, GROWTH_DRIFT, PREC_FP64)

GROWTH_DEFAULT = GROWTH_TURB | GROWTH_BROWNIAN | GROWTH_DRIFT

MH = 1.67e-24        # src/commons/phys_const.f90:8
KB = 1.38e-16        # src/commons/phys_const.f90:9
PC = 3e18            # src/commons/phys_const.f90:12

PI = 3.141592653589793238462643383279          # src/commons/phys_const.f90:14
F43 = float(np.float32(4.0) / np.float32(3.0))  # Fortran `4./3.` is a default-REAL quotient


def _powi(x, n):
    """x**n for integer n exactly as gfortran's __builtin_powi (square-and-multiply)."""
    r = 1.0
    a = float(x)
    b = abs(int(n))
    while True:
        if b & 1:
            r *= a
        b //= 2
        if b == 0:
            break
        a *= a
    return 1.0 / r if n < 0 else r


def positions(cfg):
    """Cell positions (ncells, ndim) as gridinit builds them (grid.f90:104-173).

    1D Cartesian: right cell edges accumulated over the active cells, ghosts at 0.
    2D Cartesian: cell centres ((ix-first_active)+1/2)*L/nx.
    """
    nxm, nym, ng = cfg.nx_max, cfg.ny_max, cfg.nghost
    if cfg.ny == 1:
        pos = np.zeros((nxm, 1))
        dx = cfg.box_l / float(np.float32(cfg.nx))
        acc = 0.0
        for ix in range(nxm):
            if ng <= ix < ng + cfg.nx:
                acc = acc + dx
                pos[ix, 0] = acc
        return pos
    ix = np.arange(nxm)
    iy = np.arange(nym)
    px = ((ix - ng).astype(np.float64) + 0.5) * cfg.box_l / float(np.float32(cfg.nx))
    py = ((iy - ng).astype(np.float64) + 0.5) * cfg.box_l_y / float(np.float32(cfg.ny))
    pos = np.zeros((nym, nxm, 2))
    pos[:, :, 0] = px[None, :]
    pos[:, :, 1] = py[:, None]
    return pos.reshape(-1, 2)


def primtoc(cfg, q):
    """Conservative from primitive variables (solve.f90:265-302); q has shape (nvar, ncells)."""
    N = cfg.ndust
    u = np.zeros_like(q)
    r = q[0]
    u[0] = r
    u[1] = r * q[1]
    u[2] = r * q[2]
    u[3] = r * q[3]
    u[4] = q[4] / (cfg.gamma - 1.0) + 0.5 * r * q[1] ** 2 + 0.5 * r * q[2] ** 2 + 0.5 * r * q[3] ** 2
    for k in range(N):
        rd = q[5 + k]
        u[5 + k] = rd
        u[5 + N + k] = rd * q[5 + N + k]
        u[5 + 2 * N + k] = rd * q[5 + 2 * N + k]
        u[5 + 3 * N + k] = rd * q[5 + 3 * N + k]
    return u


def _grid_view(cfg, u):
    """(nvar, ny_max, nx_max) view of a flat state."""
    return u.reshape(cfg.nvar, cfg.ny_max, cfg.nx_max)


def periodic_boundaries(cfg, u):
    """periodic_boundaries (src/grid/boundary_types.f90:149-186) on a flat state, in place."""
    g = _grid_view(cfg, u)
    ng = cfg.nghost
    if cfg.ny > 1:
        g[:, :ng, ng:ng + cfg.nx] = g[:, cfg.ny:cfg.ny + ng, ng:ng + cfg.nx]
        g[:, ng + cfg.ny:, ng:ng + cfg.nx] = g[:, ng:2 * ng, ng:ng + cfg.nx]
    g[:, :, :ng] = g[:, :, cfg.nx:cfg.nx + ng]
    g[:, :, ng + cfg.nx:] = g[:, :, ng:2 * ng]
    return u


def si_boundaries(cfg, u):
    """SI apply_boundaries (src/setups/SI/boundaries.f90): periodic + shear in the vz momenta."""
    periodic_boundaries(cfg, u)
    g = _grid_view(cfg, u)
    ng, N = cfg.nghost, cfg.ndust
    nx = cfg.nx
    # left ghosts take the right edge's values with vz momentum - rho q Omega L, and vice versa
    g[3, :, :ng] = g[3, :, nx:nx + ng] - g[0, :, nx:nx + ng] * cfg.si_q_shear * cfg.si_omega * cfg.box_l
    g[3, :, ng + nx:] = g[3, :, ng:2 * ng] + g[0, :, ng:2 * ng] * cfg.si_q_shear * cfg.si_omega * cfg.box_l
    for k in range(N):
        iz, ir = 5 + 3 * N + k, 5 + k
        g[iz, :, :ng] = g[iz, :, nx:nx + ng] - g[ir, :, nx:nx + ng] * cfg.si_q_shear * cfg.si_omega * cfg.box_l
        g[iz, :, ng + nx:] = g[iz, :, ng:2 * ng] + g[ir, :, ng:2 * ng] * cfg.si_q_shear * cfg.si_omega * cfg.box_l
    return u


# ---------------------------------------------------------------------------------------------
# SOD
# ---------------------------------------------------------------------------------------------
def sod(nx=1000, ny=1, gamma=1.4, cfl=0.5, slope_type=1, solver=2, precision=PREC_FP64,
        rho_l=1.0, rho_r=0.125, P_l=1.0, P_r=0.1, ndust=0, dust2gas=1.0, sizes=(1e-3, 1e-1),
        rhograin=1.0):
    """1D Sod shock tube (src/setups/SOD/setup.f90:1-46, boundaries.f90:49-77).  With ndust > 0 a
    dusty shock tube: each species carries dust2gas/ndust of the gas density, at rest, with grain
    radii log-spaced over `sizes` (Epstein drag on the adiabatic sound speed, back reaction and
    drag heating, SOD/setup.f90:179-185 and source_terms.f90:88-97)."""
    cfg = default_config()
    cfg.nx, cfg.ny, cfg.ndust = nx, ny, ndust
    cfg.gamma, cfg.cfl, cfg.slope_type, cfg.solver = gamma, cfl, slope_type, solver
    cfg.precision = precision
    cfg.setup = SETUP_SOD
    cfg.flags = (FLAG_DRAG | FLAG_BACK_REACTION) if ndust > 0 else 0
    cfg.rhograin = rhograin
    for k in range(ndust):
        cfg.dust_size[k] = sizes[0] * (sizes[1] / sizes[0]) ** (k / max(ndust - 1, 1))
        cfg.dust_eps[k] = dust2gas / ndust
    cfg.sod_rho_l, cfg.sod_rho_r, cfg.sod_P_l, cfg.sod_P_r = rho_l, rho_r, P_l, P_r
    cfg.sod_direction = 0
    pos = positions(cfg)
    q = np.zeros((cfg.nvar, cfg.ncells))
    right = pos[:, 0] > 0.5
    q[0] = np.where(right, rho_r, rho_l)
    q[4] = np.where(right, P_r, P_l)
    for k in range(ndust):
        q[5 + k] = cfg.dust_eps[k] * q[0]
    u = primtoc(cfg, q).reshape(-1)
    return cfg, u


# ---------------------------------------------------------------------------------------------
# DUSTYWAVE
# ---------------------------------------------------------------------------------------------
def dustywave(nx=2048, ndust=4, eps=None, tstop=None, K=None, cs0=1.0, rho_0=1.0,
              delta=1e-4, vx_0=1e-4, kx_wave=1.0, cfl=0.8, slope_type=2, gamma=1.6666667,
              precision=PREC_FP64):
    """1D periodic dusty wave (src/setups/DUSTYWAVE/setup.f90:12-79).

    Either ``K`` (the namelist drag constants) or ``tstop`` (stopping times, converted with
    ts = rho_d/K, DUSTYWAVE/setup.f90:217) may be given.
    """
    cfg = default_config()
    cfg.nx, cfg.ny, cfg.ndust = nx, 1, ndust
    cfg.gamma, cfg.cfl, cfg.slope_type = gamma, cfl, slope_type
    cfg.iso_cs = 1
    cfg.precision = precision
    cfg.setup = SETUP_DUSTYWAVE
    cfg.flags = FLAG_DRAG | FLAG_BACK_REACTION
    cfg.cs0 = cs0
    cfg.dw_rho_0, cfg.dw_delta_rho, cfg.dw_vx_0, cfg.dw_kx_wave = rho_0, delta, vx_0, kx_wave
    eps = np.full(ndust, 0.25) if eps is None else np.asarray(eps, dtype=np.float64)
    if K is None:
        tstop = np.logspace(-3, 0, ndust) if tstop is None else np.asarray(tstop, dtype=np.float64)
        K = eps * rho_0 / tstop
    for k in range(ndust):
        cfg.dust_eps[k] = eps[k]
        cfg.dust_K[k] = K[k]
    pos = positions(cfg)
    ph = np.sin(2.0 * PI * pos[:, 0] / cfg.box_l * kx_wave)
    q = np.zeros((cfg.nvar, cfg.ncells))
    q[0] = rho_0 * (1 + delta * ph)
    q[1] = vx_0 * ph
    q[4] = cs0 ** 2 * q[0]
    N = ndust
    for k in range(N):
        q[5 + k] = eps[k] * q[0]
        q[5 + N + k] = vx_0 * ph
    # the reference calls apply_boundaries before primtoc, so the ghost cells keep the values of
    # q at the ghosts' (zero) positions until the first solve refills them
    u = primtoc(cfg, q).reshape(-1)
    return cfg, u


# ---------------------------------------------------------------------------------------------
# SI shearing box
# ---------------------------------------------------------------------------------------------
def mrn_bins(ndust, smin, smax, scutmin, scut, dust2gas, mrn=3.5, rhograin=1.0,
             dust_ratio_min=1e-11, unit_l=1.0, unit_m=1.0):
    """distribution_dust(.true.) + mrn_distri (src/dust/dust_init.f90:11-103,164-197).

    Returns (sdust, eps) per species (ice mantle excluded), radii in code units (/unit_l)."""
    zeta = (smax / smin) ** (1.0 / ndust)
    eta = zeta ** 3.0
    m_min = F43 * PI * rhograin * smin ** 3.0 / unit_m
    aminus = np.array([smin * _powi(zeta, k) / unit_l for k in range(ndust)])
    aplus = np.array([smin * _powi(zeta, k + 1) / unit_l for k in range(ndust)])
    sdust = np.sqrt(aminus * aplus)
    massmin = m_min
    mono1 = F43 * PI * rhograin * scutmin ** 3.0 / unit_m
    mono2 = F43 * PI * rhograin * scut ** 3.0 / unit_m
    icutmin = max(1, int(np.floor(np.log(mono1 / massmin) / np.log(eta) + 1)))
    icutmax = min(int(np.floor(np.log(mono2 / massmin) / np.log(eta) + 1)), ndust)
    eps = np.zeros(ndust)
    norm = 0.0
    for k in range(icutmin - 1, icutmax):
        w = aplus[k] ** (4.0 - mrn) - aminus[k] ** (4.0 - mrn)
        norm = norm + w
        eps[k] = w
    eps = dust2gas * eps / norm
    eps = np.maximum(eps, dust_ratio_min)
    return sdust, eps


def si(n=1024, ndust=8, stokes_min=1e-3, stokes_max=1.0, stokes_cut=1.0, dust2gas=0.02,
       hoverr=0.1, box_l=4.0, omega=1.0, q_shear=1.5, rho_init=1.0, rad0=1.0, theta_dust=1e-11,
       noise=1e-3, seed=1, cfl=0.5, slope_type=3, gamma=1.666667, precision=PREC_FP64,
       force_kick=True):
    """2D streaming-instability shearing box (src/setups/SI/setup.f90:1-117, stokes_distrib).

    Dust velocities get uniform white noise of amplitude ``noise*cs0`` from a counter-based hash
    (seed ``seed``); the gas gets none.
    """
    cfg = default_config()
    cfg.nx, cfg.ny, cfg.ndust = n, n, ndust
    cfg.gamma, cfg.cfl, cfg.slope_type = gamma, cfl, slope_type
    cfg.iso_cs = 1
    cfg.precision = precision
    cfg.setup = SETUP_SI
    cfg.flags = FLAG_DRAG | FLAG_BACK_REACTION | (FLAG_FORCE_KICK if force_kick else 0)
    eta_stream = float(np.float32(0.05)) * hoverr          # SI/setup.f90:24 (0.05 is REAL*4)
    L = box_l * eta_stream * rad0
    cfg.box_l = cfg.box_l_y = L
    vkep = rad0 * omega
    cs0 = hoverr * vkep
    cfg.cs0 = cs0
    rhograin = rho_init / theta_dust
    cfg.rhograin = rhograin
    cfg.si_q_shear, cfg.si_omega, cfg.si_eta_stream, cfg.si_rad0 = q_shear, omega, eta_stream, rad0
    cfg.si_rho_init, cfg.si_hoverr = rho_init, hoverr
    unit_s = rho_init * cs0 / rhograin / omega
    smin = stokes_min * rho_init * cs0 / rhograin / omega
    smax = stokes_max * rho_init * cs0 / rhograin / omega
    scut = stokes_cut * rho_init * cs0 / rhograin / omega
    scutmin = stokes_min * rho_init * cs0 / rhograin / omega
    sdust, eps = mrn_bins(ndust, smin, smax, scutmin, scut, dust2gas, rhograin=rhograin,
                          dust_ratio_min=cfg.dust_ratio_min)
    stokes = sdust / unit_s
    for k in range(ndust):
        cfg.dust_size[k] = sdust[k]
        cfg.dust_eps[k] = eps[k]
        cfg.dust_stokes[k] = stokes[k]
        cfg.dust_tstop[k] = rhograin * sdust[k] / rho_init / (rad0 * omega * hoverr)  # SI/setup.f90:394
    u = si_ic(cfg, noise * cs0, seed)
    return cfg, u


def hash_uniform(seed, counter):
    """Counter-based uniform deviate in [0,1): splitmix64 of (seed, counter) (vectorised)."""
    with np.errstate(over="ignore"):
        z = (np.uint64(seed) * np.uint64(0x9E3779B97F4A7C15) + counter.astype(np.uint64)
             + np.uint64(0x632BE59BD9B4E019))
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def si_ic(cfg, noise_amp, seed):
    """SI initial state: NSH equilibrium (SI/setup.f90:52-70) + noise on dust velocities."""
    N = cfg.ndust
    qs, om, eta, r0 = cfg.si_q_shear, cfg.si_omega, cfg.si_eta_stream, cfg.si_rad0
    rho_init, cs0 = cfg.si_rho_init, cfg.cs0
    vkep = r0 * om
    A = 0.0
    B = 1.0
    for k in range(N):
        e, St = cfg.dust_eps[k], cfg.dust_stokes[k]
        A = A + e * St / (1.0 + St ** 2)
        B = B + e / (1.0 + St ** 2)
    vx_nak = 2.0 * eta * vkep * A / (A + B)
    vy_nak = -eta * vkep * B / (A + B)
    pos = positions(cfg)
    xx = pos[:, 0] - 0.5 * cfg.box_l
    nc = cfg.ncells
    q = np.zeros((cfg.nvar, nc))
    q[0] = rho_init
    q[1] = vx_nak
    q[2] = 0.0
    q[3] = qs * om * xx + vy_nak
    q[4] = q[0] * cs0 ** 2
    cells = np.arange(nc, dtype=np.uint64)
    for k in range(N):
        St = cfg.dust_stokes[k]
        ux = (vx_nak + 2.0 * St * vy_nak) / (1.0 + St ** 2)
        uy = (vy_nak - 0.5 * St * vx_nak) / (1.0 + St ** 2)
        q[5 + k] = cfg.dust_eps[k] * rho_init
        if noise_amp > 0:
            base = np.uint64(k * 3) * np.uint64(nc) + cells
            nx_ = (2.0 * hash_uniform(seed, base) - 1.0) * noise_amp
            ny_ = (2.0 * hash_uniform(seed, base + np.uint64(nc)) - 1.0) * noise_amp
            nz_ = (2.0 * hash_uniform(seed, base + np.uint64(2 * nc)) - 1.0) * noise_amp
        else:
            nx_ = ny_ = nz_ = 0.0
        q[5 + N + k] = nx_ + ux
        q[5 + 2 * N + k] = ny_
        q[5 + 3 * N + k] = nz_ + qs * om * xx + uy
    u = primtoc(cfg, q).reshape(-1)
    si_boundaries(cfg, u)
    return u


# ---------------------------------------------------------------------------------------------
# Polar disk
# ---------------------------------------------------------------------------------------------
def disk_radii(cfg):
    """Cell-centre radius per column of gridinit_disk_log (src/grid/grid.f90:180-240): a log grid
    from inner_r to box_l, ghost columns at inner_r/2 and box_l + dr_last/2."""
    nx, ng = cfg.nx, cfg.nghost
    zeta = math.pow(cfg.box_l / cfg.inner_r, 1.0 / float(nx - 1))
    r = np.empty(cfg.nx_max)
    dr = np.empty(cfg.nx_max)
    for ix in range(cfg.nx_max):
        k = ix - ng
        r[ix] = cfg.inner_r * 0.5 * (_powi(zeta, k) + _powi(zeta, k + 1))
        dr[ix] = cfg.inner_r * (_powi(zeta, k + 1) - _powi(zeta, k))
    for g in range(ng):
        r[g] = cfg.inner_r * 0.5
        r[cfg.nx_max - 1 - g] = cfg.box_l + 0.5 * dr[ng + nx - 1]
    return r


AU = 1.5e13          # src/commons/phys_const.f90:11
MSUN = 2e33          # src/commons/phys_const.f90:13
GRAV = 6.67e-8       # src/commons/phys_const.f90:10


def disk_polar(nr=128, nphi=128, ndust=4, stokes_min=1e-3, stokes_max=0.3, dust2gas=0.01, mstar=1.0,
               hoverr=0.05, temp_slope=-1.0, sigma0=1e-3, r0=1.0, rout=40.0, rin=1.0, rmax=40.0,
               r_relax=3.0, n_rel=8.0, rhograin=1.0, noise=0.0, seed=1, cfl=0.8, slope_type=1,
               gamma=1.666666666666667, fargo=False, precision=PREC_FP64, sizes=None, charging=False):
    """Face-on polar disk around a point mass (src/setups/disk_polar/setup.f90:1-84) on the log
    grid, in code units G = Mstar = 1 (r in AU, t in 1/Omega(1 AU)).

    Sigma = sigma0 (r0/r) exp(-r/rout) with optional relative white noise ``noise``; isothermal
    cs = h(r) sqrt(Mstar/r), h = hoverr r^((temp_slope+1)/2); gas rotation
    Omega r sqrt(1 - h^2 (1 - temp_slope + r/rout)); dust in MRN bins between the grain sizes of
    Stokes numbers ``stokes_min``/``stokes_max`` at r0, each bin with its own size, drifting
    inwards at eta Omega r/(St + 1/St) with the full Keplerian azimuthal velocity.  The ghost
    cells hold the initial state of their own radii, like the reference's setup.
    """
    cfg = default_config()
    cfg.nx, cfg.ny, cfg.ndust = nr, nphi, ndust
    cfg.geom, cfg.gridspace = 2, 1
    cfg.gamma, cfg.cfl, cfg.slope_type = gamma, cfl, slope_type
    cfg.iso_cs = 1
    cfg.precision = precision
    cfg.setup = SETUP_DISK_POLAR
    cfg.flags = FLAG_DRAG | FLAG_BACK_REACTION | FLAG_FORCE_KICK | (FLAG_FARGO if fargo else 0)
    cfg.box_l, cfg.inner_r = rmax, rin
    cfg.box_l_y = 2.0 * PI
    cfg.rhograin = rhograin
    cfg.disk_mstar, cfg.disk_hoverr, cfg.disk_sigma0 = mstar, hoverr, sigma0
    cfg.disk_r0, cfg.disk_rout = r0, rout
    cfg.disk_r_relax, cfg.disk_n_rel, cfg.disk_temp_slope = r_relax, n_rel, temp_slope
    cfg.flags |= FLAG_CHARGING if charging else 0
    sig0 = sigma0 * math.exp(-r0 / rout)
    unit_s = sig0 / (math.sqrt(PI * gamma / 8.0) * math.sqrt(2.0 * PI) * rhograin)   # St = 1 at r0
    if ndust > 0:
        smin, smax = sizes if sizes is not None else (stokes_min * unit_s, stokes_max * unit_s)
        sdust, eps = mrn_bins(ndust, smin, smax, smin, smax, dust2gas, rhograin=rhograin,
                              dust_ratio_min=cfg.dust_ratio_min)
        for k in range(ndust):
            cfg.dust_size[k] = sdust[k]
            cfg.dust_eps[k] = eps[k]
            cfg.dust_stokes[k] = sdust[k] / unit_s
    cfg.cs0 = hoverr * math.sqrt(mstar / r0)
    return cfg, disk_ic(cfg, noise, seed)


def disk_polar_au(nr=512, nphi=1024, ndust=16, smin_cm=1e-4, smax_cm=1.0, sigma0_cgs=1700.0,
                  rhograin_cgs=2.7, rin=1.0, rmax=100.0, hoverr=0.05, temp_slope=-0.5, dust2gas=0.01,
                  zeta=1e-17, sigma_att=96.0, noise=1e-3, seed=2, fargo=True, charging=True,
                  growth=False, growth_mode=GROWTH_DEFAULT, precision=PREC_FP64, **kw):
    """The polar disk in the reference's disk units (disk_polar/units.f90: AU, Msun, G = 1):
    Sigma = sigma0_cgs (1 AU/r) g cm^-2 without outer taper, T ~ r^temp_slope, grains from
    smin_cm to smax_cm, cosmic-ray ionisation zeta exp(-Sigma/sigma_att)."""
    unit_l = AU
    unit_d = MSUN / AU ** 3
    unit_t = 1.0 / math.sqrt(GRAV * MSUN / AU ** 3)
    cfg, _ = disk_polar(nr=nr, nphi=nphi, ndust=ndust, dust2gas=dust2gas, hoverr=hoverr, temp_slope=temp_slope,
                        sigma0=sigma0_cgs / (unit_d * unit_l), r0=1.0, rout=float("inf"), rin=rin, rmax=rmax,
                        rhograin=rhograin_cgs / unit_d, fargo=fargo, precision=precision,
                        sizes=(smin_cm / unit_l, smax_cm / unit_l), charging=charging, **kw)
    cfg.unit_l, cfg.unit_d, cfg.unit_t = unit_l, unit_d, unit_t
    cfg.chg_x = zeta
    cfg.chg_sigma_att = sigma_att
    if growth:
        cfg.flags |= FLAG_GROWTH
    cfg.grw_smin, cfg.grw_smax, cfg.grw_mode = smin_cm, smax_cm, growth_mode
    return cfg, disk_ic(cfg, noise, seed)


def disk_ic(cfg, noise_amp, seed):
    """Initial conserved state of the polar disk (disk_polar/setup.f90:27-74); see disk_polar."""
    N = cfg.ndust
    nxm, nym = cfg.nx_max, cfg.ny_max
    r = disk_radii(cfg)
    q = np.zeros((cfg.nvar, nym, nxm))
    cells = np.arange(cfg.ncells, dtype=np.uint64).reshape(nym, nxm)
    M, slope = cfg.disk_mstar, cfg.disk_temp_slope
    for ix in range(nxm):
        rr = float(r[ix])
        h = cfg.disk_hoverr * math.pow(rr, 0.5 * (slope + 1.0))
        H = h * rr
        omega = math.sqrt(M / _powi(rr, 3))
        cs0 = omega * H
        sig = cfg.disk_sigma0 * (cfg.disk_r0 / rr) * math.exp(-rr / cfg.disk_rout)
        if noise_amp > 0:
            sig = sig * (1.0 + noise_amp * (2.0 * hash_uniform(seed, cells[:, ix]) - 1.0))
        else:
            sig = np.full(nym, sig)
        rot = math.sqrt(1.0 - (h * h) * (1.0 - slope + rr / cfg.disk_rout))
        q[0, :, ix] = sig
        q[2, :, ix] = omega * rr * rot
        q[4, :, ix] = sig * (cs0 * cs0)
        hs = math.sqrt(2.0 * PI) * H
        for k in range(N):
            q[5 + k, :, ix] = cfg.dust_eps[k] * sig
            ts = math.sqrt(PI * cfg.gamma / 8.0) * cfg.rhograin * cfg.dust_size[k] / (sig / hs * cs0)
            St = ts * omega
            q[5 + N + k, :, ix] = (rot - 1.0) * omega * rr / (St + 1.0 / St)
            q[5 + 2 * N + k, :, ix] = omega * rr
    return primtoc(cfg, q.reshape(cfg.nvar, -1)).reshape(-1)


# ---------------------------------------------------------------------------------------------
# Cartesian disk
# ---------------------------------------------------------------------------------------------
ICE_MANTLE_CM = 8.7e-7   # src/dust/dust_commons.f90:47
# test/CARTESIAN_disk/disk.nml (SETUP_PARAMS and GRID_PARAMS)
CARTESIAN_DISK_NML = dict(box_l=320.0, buffer_in=0.0, buffer_out=0.375, alpha_visc=1e-2, frac_r_disk=0.125,
                          smooth_r=0.1, sigma_r0=300.0, cfl=0.8, gamma=1.666667, slope_type=3)


def disk_cart(n=256, ndust=4, box_l=320.0, sigma_r0=300.0, r0_disk=1.0, mstar=1.0, hoverr=0.05, smooth_r=0.1,
              alpha_visc=1e-2, frac_r_disk=0.125, buffer_in=0.0, buffer_out=0.375, dust2gas=0.01,
              smin_cm=1e-7, smax_cm=1e-2, rhograin_cgs=2.7, cfl=0.8, gamma=1.666667, slope_type=3,
              viscosity=True, force_kick=True, precision=PREC_FP64):
    """The Cartesian disk (src/setups/disk/setup.f90, units.f90) on an n x n box of box_l AU: a
    star of mstar Msun at the centre with softening smooth_r, Sigma = sigma_r0 (g cm^-2)
    r0_disk/rr (1/100 of the value at R_out = frac_r_disk box_l beyond it), isothermal
    cs = hoverr sqrt(Mstar/rr), Keplerian rotation Omega = sqrt(Mstar/rr^3) on the softened
    offsets, viscosity alpha_visc H cs, every dust species at dust2gas with the gas velocity,
    grains in MRN bins between smin_cm and smax_cm (the dust_commons defaults) plus the ice mantle.
    The defaults are those of test/CARTESIAN_disk/disk.nml.  Every cell, ghosts included, gets
    the profile at its own position, as the setup loop does; the boundaries are applied by the
    step."""
    unit_l = AU
    unit_d = MSUN / AU ** 3
    unit_t = 1.0 / math.sqrt(GRAV * unit_d)
    unit_dcol = MSUN / AU ** 2
    cfg = default_config()
    cfg.nx, cfg.ny, cfg.ndust = n, n, ndust
    cfg.geom = 0
    cfg.gamma, cfg.cfl, cfg.slope_type = gamma, cfl, slope_type
    cfg.iso_cs = 1
    cfg.precision = precision
    cfg.setup = SETUP_DISK_CART
    cfg.flags = (FLAG_DRAG | FLAG_BACK_REACTION | (FLAG_FORCE_KICK if force_kick else 0)
                 | (FLAG_VISCOSITY if viscosity else 0))
    cfg.box_l = cfg.box_l_y = box_l * AU / unit_l
    cfg.disk_mstar = mstar * MSUN / MSUN
    cfg.disk_hoverr = hoverr
    cfg.disk_sigma0 = sigma_r0 / unit_dcol
    cfg.disk_r0 = r0_disk * AU / unit_l
    cfg.disk_alpha_visc = alpha_visc
    cfg.cdisk_smooth_r = smooth_r * AU / unit_l
    cfg.cdisk_frac_r_disk, cfg.cdisk_buffer_in, cfg.cdisk_buffer_out = frac_r_disk, buffer_in, buffer_out
    cfg.unit_l, cfg.unit_d, cfg.unit_t = unit_l, unit_d, unit_t
    cfg.rhograin = rhograin_cgs / unit_d
    if ndust > 0:
        sdust, _ = mrn_bins(ndust, smin_cm, smax_cm, smin_cm, smax_cm, dust2gas, rhograin=rhograin_cgs,
                            unit_l=unit_l, unit_m=MSUN)
        for k in range(ndust):
            cfg.dust_size[k] = sdust[k] + ICE_MANTLE_CM / unit_l
            cfg.dust_eps[k] = dust2gas
    cfg.cs0 = hoverr * math.sqrt(cfg.disk_mstar / cfg.disk_r0)
    return cfg, disk_cart_ic(cfg)


def disk_cart_geometry(cfg):
    """Per cell (all cells): offsets xx, yy from the box centre, r_cyl, the softened radius rr and
    the softened offsets x_soft, y_soft of disk/setup.f90."""
    pos = positions(cfg)
    xx = pos[:, 0] - 0.5 * cfg.box_l
    yy = pos[:, 1] - 0.5 * cfg.box_l_y
    r_cyl = np.sqrt(xx * xx + yy * yy)
    rr = np.sqrt(xx * xx + yy * yy + cfg.cdisk_smooth_r * cfg.cdisk_smooth_r)
    with np.errstate(invalid="ignore", divide="ignore"):
        x_soft = xx * rr / r_cyl
        y_soft = yy * rr / r_cyl
    return xx, yy, r_cyl, rr, x_soft, y_soft


def disk_cart_ic(cfg):
    """Initial conserved state of the Cartesian disk (disk/setup.f90 setup loop, then primtoc)."""
    N = cfg.ndust
    xx, yy, r_cyl, rr, x_soft, y_soft = disk_cart_geometry(cfg)
    M = cfg.disk_mstar
    cs0 = cfg.disk_hoverr * np.sqrt(M / rr)
    omega = np.sqrt(M / (rr * (rr * rr)))
    r_out = cfg.cdisk_frac_r_disk * cfg.box_l
    rho = cfg.disk_sigma0 * (cfg.disk_r0 / rr)
    rho = np.where(rr > r_out, cfg.disk_sigma0 * (cfg.disk_r0 / r_out) / 100.0, rho)
    q = np.zeros((cfg.nvar, cfg.ncells))
    q[0] = rho
    q[1] = -omega * y_soft
    q[2] = omega * x_soft
    q[4] = rho * (cs0 * cs0)
    for k in range(N):
        q[5 + k] = cfg.dust_eps[k] * rho
        q[5 + N + k] = -omega * y_soft
        q[5 + 2 * N + k] = omega * x_soft
    return primtoc(cfg, q).reshape(-1)


# ---------------------------------------------------------------------------------------------
# Dusty turbulence
# ---------------------------------------------------------------------------------------------
def dusty_turb(n=256, ndust=32, smin=1e-6, smax=0.1, dust2gas=0.01, nH=1e9, T=10.0, box_pc=0.1,
               mach=1.0, kmin=1, kmax=3, seed=3, tcorr=None, rhograin=2.7, gamma=1.66667, cfl=0.5,
               slope_type=1, charging=False, forcing=False, growth=False, growth_mode=GROWTH_DEFAULT,
               precision=PREC_FP64):
    """2D periodic isothermal dusty box in cgs units (src/setups/dustyTurb/setup.f90, units.f90).

    Gas of number density ``nH`` (cm^-3, mu_gas = 2.31) at ``T`` K; grains in ``ndust`` MRN bins
    between radii ``smin`` and ``smax`` (cm), total dust-to-gas ratio ``dust2gas``.  The stopping
    time law of the reference, t_k = St_0,k box_l rho_0/cs/rho, takes St_0,k from the Epstein
    time of grain k at rho_0.  Gas and dust start with the same solenoidal velocity field: a sum
    of Fourier modes of the stream function with wavenumbers kmin <= |k| L/(2 pi) <= kmax,
    seeded amplitudes and phases, scaled to RMS Mach ``mach``.  ``forcing`` enables the
    Ornstein-Uhlenbeck driving of the same band with correlation time ``tcorr`` (default one
    sound crossing time of the box).
    """
    cfg = default_config()
    cfg.nx = cfg.ny = n
    cfg.ndust = ndust
    cfg.gamma, cfg.cfl, cfg.slope_type = gamma, cfl, slope_type
    cfg.iso_cs = 1
    cfg.precision = precision
    cfg.setup = SETUP_DUSTYTURB
    cfg.flags = FLAG_DRAG | FLAG_BACK_REACTION | (FLAG_CHARGING if charging else 0) | (FLAG_GROWTH if growth else 0)
    cfg.grw_smin, cfg.grw_smax, cfg.grw_mode = smin, smax, growth_mode
    L = box_pc * PC
    cfg.box_l = cfg.box_l_y = L
    cfg.mu_gas = 2.31
    cfg.T_cloud = T
    rho0 = nH * cfg.mu_gas * MH
    cfg.turb_rho0 = rho0
    cs = math.sqrt(KB * T / (cfg.mu_gas * MH))
    cfg.cs0 = cs
    cfg.rhograin = rhograin
    if ndust > 0:
        sdust, eps = mrn_bins(ndust, smin, smax, smin, smax, dust2gas, rhograin=rhograin,
                              dust_ratio_min=cfg.dust_ratio_min)
        for k in range(ndust):
            cfg.dust_size[k] = sdust[k]
            cfg.dust_eps[k] = eps[k]
            cfg.dust_stokes[k] = math.sqrt(PI * gamma / 8.0) * rhograin * sdust[k] / (rho0 * L)
    cfg.turb_mach = mach if forcing else 0.0
    cfg.turb_tcorr = tcorr if tcorr is not None else L / cs
    cfg.turb_kmin, cfg.turb_kmax, cfg.turb_seed = kmin, kmax, seed
    return cfg, turb_ic(cfg, mach, seed, kmin, kmax)


def solenoidal_modes(kmin, kmax):
    """Integer wave vectors (kx, ky), one per +-k pair, with kmin <= |k| <= kmax."""
    modes = []
    for kx in range(0, kmax + 1):
        for ky in range(-kmax, kmax + 1):
            if kx == 0 and ky <= 0:
                continue
            kk = math.hypot(kx, ky)
            if kmin <= kk <= kmax:
                modes.append((kx, ky))
    return modes


def turb_ic(cfg, mach, seed, kmin, kmax):
    """Initial conserved state of the dusty box (see dusty_turb)."""
    N = cfg.ndust
    pos = positions(cfg)
    L = cfg.box_l
    x, y = pos[:, 0], pos[:, 1]
    vx = np.zeros(cfg.ncells)
    vy = np.zeros(cfg.ncells)
    modes = solenoidal_modes(kmin, kmax)
    cnt = np.arange(2 * len(modes), dtype=np.uint64)
    u = hash_uniform(seed, cnt)
    for m, (kx, ky) in enumerate(modes):
        amp = u[2 * m] + 0.5
        ph = 2.0 * PI * u[2 * m + 1]
        kxp, kyp = 2.0 * PI * kx / L, 2.0 * PI * ky / L
        c = np.cos(kxp * x + kyp * y + ph)
        # stream function amp sin(k.x + ph)/|k|: v = (d/dy, -d/dx)
        kk = math.hypot(kxp, kyp)
        vx += amp * kyp / kk * c
        vy -= amp * kxp / kk * c
    ng = cfg.nghost
    act = np.zeros((cfg.ny_max, cfg.nx_max), bool)
    act[ng:ng + cfg.ny, ng:ng + cfg.nx] = True
    act = act.reshape(-1)
    rms = math.sqrt(float(np.mean(vx[act] ** 2 + vy[act] ** 2)))
    scale = mach * cfg.cs0 / rms if rms > 0 else 0.0
    vx *= scale
    vy *= scale
    q = np.zeros((cfg.nvar, cfg.ncells))
    q[0] = cfg.turb_rho0
    q[1], q[2] = vx, vy
    q[4] = q[0] * cfg.cs0 ** 2
    for k in range(N):
        q[5 + k] = cfg.dust_eps[k] * cfg.turb_rho0
        q[5 + N + k] = vx
        q[5 + 2 * N + k] = vy
    u0 = primtoc(cfg, q).reshape(-1)
    periodic_boundaries(cfg, u0)
    return u0


# ---------------------------------------------------------------------------------------------
# Kelvin-Helmholtz shear layer
# ---------------------------------------------------------------------------------------------
GRAV = 6.67e-8       # src/commons/phys_const.f90:10

# test/KH/kh.nml of the reference: a 1 au box of 1e-18 g cm^-3 gas at 10 K, Mach 0.25 shear,
# MRN grains from 5e-7 to 0.1 cm (initial 1e-7 .. 2.5e-5 cm) of density 2.3, MC limiter, CFL 0.1
KH_NML = dict(box_pc=4.8481e-6, rho_dense=1.0e-18, rho_diffuse=1.0e-18, T_dense=10.0, mach=0.25, vy0=0.1,
              kx=2.0, smin=5e-7, scutmin=1e-7, scut=250e-7, smax=0.10, rhograin=2.3, dust2gas=0.01,
              mrn=3.5, gamma=1.666667, slope_type=3, cfl=0.1)


def kh_units(mu_gas=2.31):
    """(unit_l, unit_d, unit_t) of KH/units.f90: parsec, mu_gas mH, 1/sqrt(G unit_d)."""
    unit_d = mu_gas * MH
    return PC, unit_d, 1.0 / math.sqrt(GRAV * unit_d)


def kh(n=256, ny=None, ndust=4, box_pc=1.0, rho_dense=1.0, rho_diffuse=0.8, T_dense=10.0, mach=0.5,
       vy0=0.1, kx=10.0, smin=1e-7, smax=1e-2, scutmin=5e-7, scut=250e-7, mrn=3.5, rhograin=2.7,
       dust2gas=0.01, gamma=1.66667, cfl=0.5, slope_type=1, solver=2, drag=True, precision=PREC_FP64):
    """Kelvin-Helmholtz shear layer (src/setups/KH/setup.f90:1-51, setup_commons.f90, units.f90).

    Inputs are cgs and Kelvin as in the reference's namelist (box in parsec); the run is in the
    setup's code units (unit_l = pc, unit_d = mu_gas mH, unit_t = 1/sqrt(G unit_d)).  Periodic,
    adiabatic; grains in ``ndust`` MRN bins (distribution_dust), or one species of radius
    ``scut`` at dust-to-gas ratio 0.01 for ``ndust == 1``, at rest, with Epstein drag on the
    adiabatic sound speed (KH/setup.f90:218-239) and back reaction.  Defaults are the reference's
    (KH/setup_commons.f90, dust_commons.f90); ``KH_NML`` holds its test/KH/kh.nml values.
    """
    cfg = default_config()
    cfg.nx = n
    cfg.ny = n if ny is None else ny
    cfg.ndust = ndust
    cfg.gamma, cfg.cfl, cfg.slope_type, cfg.solver = gamma, cfl, slope_type, solver
    cfg.precision = precision
    cfg.setup = SETUP_KH
    cfg.flags = (FLAG_DRAG | FLAG_BACK_REACTION) if (ndust > 0 and drag) else 0
    cfg.mu_gas = 2.31
    ul, ud, ut = kh_units(cfg.mu_gas)
    cfg.unit_l, cfg.unit_d, cfg.unit_t = ul, ud, ut
    cfg.box_l = cfg.box_l_y = box_pc
    cfg.kh_rho_dense, cfg.kh_rho_diffuse, cfg.kh_T_dense = rho_dense, rho_diffuse, T_dense
    cfg.kh_mach, cfg.kh_vy0, cfg.kh_kx = mach, vy0, kx
    cfg.rhograin = rhograin / ud                    # (rhograin/unit_d) of compute_tstop
    if ndust == 1:
        cfg.dust_size[0] = scut / ul                # KH/setup.f90:41
        cfg.dust_eps[0] = float(np.float32(0.01))   # `epsilondust = 0.01`: a default-REAL literal
    elif ndust > 1:
        sdust, eps = mrn_bins(ndust, smin, smax, scutmin, scut, dust2gas, mrn=mrn, rhograin=rhograin,
                              dust_ratio_min=cfg.dust_ratio_min, unit_l=ul, unit_m=ul ** 3 * ud)
        for k in range(ndust):
            cfg.dust_size[k] = sdust[k]
            cfg.dust_eps[k] = eps[k]
    return cfg, kh_ic(cfg)


def kh_ic(cfg):
    """Initial conserved state of the shear layer (KH/setup.f90:17-51), over all cells and then
    periodic ghosts."""
    uv = cfg.unit_l / cfg.unit_t
    uP = cfg.unit_d * (uv * uv)
    cs = math.sqrt(cfg.gamma * KB * cfg.kh_T_dense / (cfg.mu_gas * MH))     # KH/eos.f90 cs_eos
    pos = positions(cfg)
    xx = pos[:, 0] - 0.5 * cfg.box_l
    yy = pos[:, 1] - 0.5 * cfg.box_l_y
    band = np.abs(yy / cfg.box_l_y) < 0.25
    q = np.zeros((cfg.nvar, cfg.ncells))
    q[0] = np.where(band, cfg.kh_rho_diffuse / cfg.unit_d, cfg.kh_rho_dense / cfg.unit_d)
    q[1] = np.where(band, -(cs * cfg.kh_mach / uv / 2.0), cs * cfg.kh_mach / uv * 0.5)
    # libm's cos per grid column (numpy's vectorised cos may differ in the last bit)
    cosx = {v: math.cos(v * 2.0 * cfg.kh_kx * PI / cfg.box_l) for v in np.unique(xx).tolist()}
    q[2] = (cfg.kh_vy0 * cs * cfg.kh_mach * np.array([cosx[v] for v in xx.tolist()])) / uv
    q[4] = cfg.kh_rho_dense * (cs * cs) / uP
    for k in range(cfg.ndust):
        q[5 + k] = cfg.dust_eps[k] * q[0]
    u0 = primtoc(cfg, q).reshape(-1)
    periodic_boundaries(cfg, u0)
    return u0


# ---------------------------------------------------------------------------------------------
# Sedov blast wave
# ---------------------------------------------------------------------------------------------
def sedov(n=256, box_l=1.0, rho_ext=1.0, P_ext=1e-5, P_cen=1.0, r_expl=None, gamma=1.66667, cfl=0.5,
          slope_type=1, solver=2, precision=PREC_FP64):
    """2D Sedov blast wave in a periodic square (src/setups/sedov/setup.f90:1-34,
    setup_commons.f90): gas at rest of density ``rho_ext`` and pressure ``P_ext``, raised by
    ``P_cen`` inside radius ``r_expl`` of the box centre.  Unit-free, gas only.  The default
    radius is the reference's `r_expl=0.1`, a default-REAL literal (0.1 rounded to float)."""
    cfg = default_config()
    cfg.nx = cfg.ny = n
    cfg.ndust = 0
    cfg.gamma, cfg.cfl, cfg.slope_type, cfg.solver = gamma, cfl, slope_type, solver
    cfg.precision = precision
    cfg.setup = SETUP_SEDOV
    cfg.flags = 0
    cfg.box_l = cfg.box_l_y = box_l
    cfg.sedov_rho_ext, cfg.sedov_P_ext, cfg.sedov_P_cen = rho_ext, P_ext, P_cen
    if r_expl is not None:
        cfg.sedov_r_expl = r_expl
    return cfg, sedov_ic(cfg)


def sedov_ic(cfg):
    """Initial conserved state of the blast (sedov/setup.f90:15-33): active cells set, ghosts
    from the periodic images."""
    pos = positions(cfg)
    xn = np.abs(pos[:, 0] - 0.5 * cfg.box_l)
    yn = np.abs(pos[:, 1] - 0.5 * cfg.box_l_y)
    q = np.zeros((cfg.nvar, cfg.ncells))
    q[0] = cfg.sedov_rho_ext
    q[4] = np.where(xn * xn + yn * yn < cfg.sedov_r_expl * cfg.sedov_r_expl,
                    cfg.sedov_P_ext + cfg.sedov_P_cen, cfg.sedov_P_ext)
    u0 = primtoc(cfg, q).reshape(-1)
    periodic_boundaries(cfg, u0)
    return u0


def build(name, **kw):
    """Dispatch by setup name ('sod', 'dustywave', 'si', 'disk_polar', 'disk_cart', 'dusty_turb',
    'kh', 'sedov')."""
    return {"sod": sod, "dustywave": dustywave, "si": si, "disk_polar": disk_polar, "disk_cart": disk_cart,
            "dusty_turb": dusty_turb, "kh": kh, "sedov": sedov}[name](**kw)
