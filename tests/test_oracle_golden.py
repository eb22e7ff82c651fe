"""The CPU oracle against the reference's own golden data and against analytic known answers.

Golden data (tests/golden/, copied by tests/golden/make_golden.py from the reference test suite):
  * Sod exact solution, t = 0.245, 1024 cells (test/test-suite/Sod-tube/solution.dat with
    sod.nml: CFL 0.8, gamma 1.4, slope_type 3).
  * Single-species dusty-wave profiles for K = 50, 100, 1000 (test/test-suite/DUSTYWAVE/ with
    wave{50,100,1000}.nml: CFL 0.8, tend 4.5, slope_type 2, eps 1, amplitude 1e-4).
"""
import os

import numpy as np
import pytest

from shark_gb300 import setups
from oracle.oracle import Oracle
from tests.exact_riemann import sample as riemann_sample

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _gas_prims(o, cfg):
    q, cs = o.get_q()
    nc = cfg.ncells
    act = slice(cfg.nghost, cfg.nghost + cfg.nx)
    return q[0:nc][act], q[nc:2 * nc][act], q[4 * nc:5 * nc][act]


def test_sod_golden_exact_solution():
    cfg, u0 = setups.sod(nx=1024, gamma=1.4, cfl=0.8, slope_type=3)
    o = Oracle(cfg)
    o.setup_ic()
    assert np.array_equal(o.get_u(), u0), "host-side SOD ICs differ from the oracle's"
    o.run(10 ** 6, 0.245)
    assert 0.245 <= o.time < 0.2460   # dt is not clipped at tend
    rho, u, P = _gas_prims(o, cfg)
    g = np.loadtxt(os.path.join(GOLDEN, "sod_exact_t0.245_n1024.dat"))
    # second-order MUSCL at 1024 cells: L1 errors a few 1e-4 (mostly at the shock and contact)
    assert np.mean(np.abs(rho - g[:, 3])) < 1.0e-3
    assert np.mean(np.abs(u - g[:, 2])) < 1.5e-3
    assert np.mean(np.abs(P - g[:, 4])) < 1.0e-3
    # pointwise agreement away from the discontinuities
    smooth = (np.abs(g[:, 1] - 0.93) > 0.01) & (np.abs(g[:, 1] - 0.728) > 0.02) & (np.abs(g[:, 1] - 0.26) > 0.01) \
        & (np.abs(g[:, 1] - 0.49) > 0.01)
    assert np.max(np.abs(rho - g[:, 3])[smooth]) < 2e-2


@pytest.mark.parametrize("K", [50, 100, 1000])
def test_dustywave_golden(K):
    g = np.loadtxt(os.path.join(GOLDEN, f"dustywave_K{K}.dat"))
    NX = 512
    cfg, u0 = setups.dustywave(nx=NX, ndust=1, eps=[1.0], K=[float(K)], delta=1e-4, vx_0=1e-4,
                               cfl=0.8, slope_type=2, gamma=1.6666667)
    o = Oracle(cfg)
    o.setup_ic()
    assert np.array_equal(o.get_u(), u0), "host-side DUSTYWAVE ICs differ from the oracle's"
    o.run(10 ** 6, 4.5)
    q, cs = o.get_q()
    nc = cfg.ncells
    act = slice(2, 2 + NX)
    j = np.arange(128)
    k = (j * NX // 128 - 1) % NX   # the cell whose (right-edge) position is x = j/128
    amp = 1e-4
    cols = {"vgas": (q[nc:2 * nc][act], 1), "vdust": (q[6 * nc:7 * nc][act], 2),
            "rhogas": (q[0:nc][act], 3), "rhodust": (q[5 * nc:6 * nc][act], 4)}
    for name, (arr, c) in cols.items():
        l1 = np.mean(np.abs(arr[k] - g[:, c])) / amp
        assert l1 < (0.03 if name.startswith("v") else 0.1), (name, l1)


def test_sod_1000_cells_minmod_hllc_vs_exact_riemann():
    """1000 cells, minmod, HLLC, CFL 0.5, to t = 0.2, against the exact solution at the final
    time actually reached (the last step overshoots tend)."""
    cfg, u0 = setups.sod(nx=1000, gamma=1.4, cfl=0.5, slope_type=1)
    o = Oracle(cfg)
    o.set_u(u0)
    o.run(10 ** 6, 0.2)
    rho, u, P = _gas_prims(o, cfg)
    x = (np.arange(1000) + 0.5) / 1000.0
    ex = riemann_sample(x, o.time, 0.5, 1.0, 0.0, 1.0, 0.125, 0.0, 0.1, 1.4)
    assert np.mean(np.abs(rho - ex[0])) < 2.5e-3
    assert np.mean(np.abs(u - ex[1])) < 4e-3
    assert np.mean(np.abs(P - ex[2])) < 2.5e-3


def _uniform_two_fluid(eps, ts, vd0, nx=16):
    cfg, _ = setups.dustywave(nx=nx, ndust=len(eps), eps=eps, tstop=ts, delta=0.0, vx_0=0.0)
    # dustywave builds K from eps/ts with rho_0 = 1: ts = rho_d/K holds exactly
    nc = cfg.ncells
    N = cfg.ndust
    u = np.zeros(cfg.nvar * nc)
    u[0:nc] = 1.0
    u[4 * nc:5 * nc] = 1.0 / (cfg.gamma - 1.0)
    for k in range(N):
        u[(5 + k) * nc:(6 + k) * nc] = eps[k]
        u[(5 + N + k) * nc:(6 + N + k) * nc] = eps[k] * vd0[k]
    return cfg, u


def test_drag_single_species_recurrence():
    """Uniform gas at rest + one dust species drifting: fluxes cancel, and the implicit drag makes
    dv_{n+1} = dv_n / (1 + a_n (1 + eps)) with a_n = dt_n / ts (dust_drag.f90:29-54)."""
    eps, ts = 0.5, 0.05
    cfg, u = _uniform_two_fluid([eps], [ts], [1e-3])
    o = Oracle(cfg)
    o.set_u(u)
    nc = cfg.ncells
    dv = 1e-3
    for _ in range(20):
        dt = o.solve()
        dv = dv / (1.0 + dt / ts * (1.0 + eps))
        uu = o.get_u()
        i = 5
        vg = uu[nc + i] / uu[i]
        vd = uu[6 * nc + i] / uu[5 * nc + i]
        assert abs((vd - vg) - dv) <= 1e-12 * 1e-3
        # momentum is conserved exactly by the scheme (up to round-off)
        assert abs(uu[nc + i] + uu[6 * nc + i] - eps * 1e-3) < 1e-17


def test_drag_stiff_limit_multispecies():
    """t_s << dt: every species ends at the barycentric velocity in one step, total momentum kept."""
    eps = [0.25, 0.25, 0.25, 0.25]
    ts = [1e-9, 2e-9, 5e-9, 1e-8]
    vd0 = [1e-3, -2e-3, 3e-3, 4e-3]
    cfg, u = _uniform_two_fluid(eps, ts, vd0)
    o = Oracle(cfg)
    o.set_u(u)
    o.solve()
    uu = o.get_u()
    nc, N, i = cfg.ncells, 4, 5
    ptot0 = sum(e * v for e, v in zip(eps, vd0))
    vbar = ptot0 / (1.0 + sum(eps))
    assert abs(uu[nc + i] / uu[i] - vbar) < 1e-6 * abs(vbar)   # O(ts/dt) ~ 1e-7 off
    for k in range(N):
        vk = uu[(5 + N + k) * nc + i] / uu[(5 + k) * nc + i]
        assert abs(vk - vbar) < 1e-6 * abs(vbar)
    ptot = uu[nc + i] + sum(uu[(5 + N + k) * nc + i] for k in range(N))
    assert abs(ptot - ptot0) < 1e-16


def test_si_ic_matches_oracle():
    """Host-side SI ICs (NSH equilibrium + seeded dust-velocity noise) equal the oracle's.

    Mass is NOT a conserved quantity of the reference's SI box: update_force_setup writes the
    force on active cells only (src/setups/SI/setup.f90:339), so the ghost cells' predicted face
    states differ from their periodic images and the two x-boundary fluxes do not cancel."""
    cfg, u0 = setups.si(n=16, ndust=4, noise=1e-3, seed=7)
    o = Oracle(cfg)
    o.setup_ic(noise_amp=1e-3 * cfg.cs0, seed=7)
    assert np.max(np.abs(o.get_u() - u0)) == 0.0


def test_dustywave_conserves_mass_and_momentum():
    """Periodic box without forces: every species' mass and the total x momentum are conserved
    to round-off (fluxes telescope; the implicit drag conserves total momentum)."""
    cfg, u0 = setups.dustywave(nx=256, ndust=4, delta=1e-2, vx_0=1e-2)
    o = Oracle(cfg)
    o.set_u(u0)
    t0 = o.totals().reshape(-1, 4)
    o.run(200)
    t1 = o.totals().reshape(-1, 4)
    assert np.all(np.abs(t1[:, 0] - t0[:, 0]) <= 1e-13 * t0[:, 0])
    assert abs(t1[:, 1].sum() - t0[:, 1].sum()) <= 1e-15
