"""Grain charging (src/chemistry/ionisation.f90:4-214) in the CPU oracle, checked against an
independent numpy evaluation of the balance the Newton iteration zeroes, and against the
known structure of the iteration (cold start from psi0, one-iteration warm start)."""
import math

import numpy as np
import pytest

from shark_gb300 import setups
from oracle.oracle import Oracle

MH, KB, E_EL, M_EL = 1.67e-24, 1.38e-16, 4.8e-10, 9.109e-28


def _noisy_turb(n=16, ndust=8, seed=5, amp=0.6, nH=1e9):
    cfg, u0 = setups.dusty_turb(n=n, ndust=ndust, nH=nH, charging=True)
    rng = np.random.default_rng(seed)
    g = u0.reshape(cfg.nvar, -1)
    f = np.exp(amp * rng.standard_normal(cfg.ncells))          # gas density factor
    fd = np.exp(amp * rng.standard_normal((ndust, cfg.ncells)))  # dust abundance factors
    for v in range(5):
        g[v] *= f
    for k in range(ndust):
        for c in range(4):
            g[5 + c * ndust + k] *= f * fd[k]
    setups.periodic_boundaries(cfg, u0)
    return cfg, u0


def balance(cfg, u, psi):
    """The charge balance f(psi) of ionisation.f90:88-96 for dustyTurb cells (cgs)."""
    N = cfg.ndust
    g = u.reshape(cfg.nvar, -1)
    T, mu = cfg.T_cloud, cfg.chg_mu_ions
    thetai = cfg.chg_stick_el * math.sqrt(mu * MH / M_EL)
    nH = g[0] / (cfg.mu_gas * MH)
    a = np.array(cfg.dust_size[:N])
    m = float(np.float32(4.0) / np.float32(3.0)) * math.pi * cfg.rhograin * a ** 3
    nk = g[5:5 + N] / m[:, None]
    tau = a * KB * T / E_EL ** 2
    alpha = np.sqrt(8.0 / (math.pi * tau))
    sig = 2e-7 / math.sqrt(T / 300.0)
    vi = math.sqrt(8.0 * KB * T / (math.pi * mu * MH))
    eps = (1.0 - psi) / thetai * np.exp(-psi)
    et = eps * thetai
    den = 1.0 + et * alpha[:, None] + et ** 2
    ni = np.sum(-(psi * tau[:, None] + (1.0 - et ** 2) / den) * nk / (1.0 - eps), axis=0)
    s1 = np.sum(nk * math.pi * (a ** 2)[:, None] * ((1.0 - psi) + (2.0 / tau[:, None]) * (et ** 2 + et) / den), axis=0)
    xn = cfg.chg_x * nH
    return sig * eps * ni ** 2 / xn + ni * vi / xn * s1 - 1.0


def test_psi0_solves_the_dust_free_balance():
    cfg, u0 = setups.dusty_turb(n=8, ndust=4, charging=True)
    o = Oracle(cfg)
    psi0 = o.charge_psi0()
    thetai = cfg.chg_stick_el * math.sqrt(cfg.chg_mu_ions * MH / M_EL)
    f = (1.0 - psi0) / (0.99999 * thetai) * math.exp(-psi0) - 1.0
    assert abs(f) < 1e-6
    assert -4.0 < psi0 < -2.5


def test_converged_cells_zero_the_balance():
    cfg, u0 = _noisy_turb()
    o = Oracle(cfg)
    o.set_u(u0)
    it = o.charge()
    c = o.get_charge()
    ok = it < cfg.chg_nitermax
    assert ok.mean() > 0.9
    f = balance(cfg, u0, c["psi"])
    # the last update is one Newton step past a residual below chg_eps
    assert np.all(np.abs(f[ok]) < 10 * cfg.chg_eps)
    # charge neutrality of the outputs: n_i - n_e + sum_k Z_k n_k = 0
    N = cfg.ndust
    g = u0.reshape(cfg.nvar, -1)
    a = np.array(cfg.dust_size[:N])
    m = float(np.float32(4.0) / np.float32(3.0)) * math.pi * cfg.rhograin * a ** 3
    nk = g[5:5 + N] / m[:, None]
    q = c["ni"] - c["ne"] + np.sum(c["zd"] * nk, axis=0)
    assert np.all(np.abs(q[ok]) <= 1e-10 * c["ni"][ok])


def test_warm_start_takes_one_iteration_on_an_unchanged_state():
    cfg, u0 = _noisy_turb(n=8)
    o = Oracle(cfg)
    o.set_u(u0)
    cold = o.charge()
    warm = o.charge()
    conv = cold < cfg.chg_nitermax
    assert np.all(warm[conv] <= 2)
    assert cold[conv].mean() > 5 * warm[conv].mean()
    o.reset_charge()
    assert np.array_equal(o.charge(), cold)


def test_seed_at_the_solution_converges_at_once():
    cfg, u0 = _noisy_turb(n=8)
    o = Oracle(cfg)
    o.set_u(u0)
    cold = o.charge()
    psi = o.get_charge()["psi"].copy()
    o.reset_charge()
    seeded = o.charge(seed=psi)
    conv = cold < cfg.chg_nitermax
    assert np.all(seeded[conv] <= 2)


def test_charging_in_the_step_leaves_the_hydro_state_unchanged():
    cfg, u0 = _noisy_turb(n=12, ndust=4)
    a, b = Oracle(cfg), Oracle(cfg)
    a.set_u(u0)
    b.set_u(u0)
    cfg2 = cfg.copy()
    cfg2.flags &= ~setups.FLAG_CHARGING
    c = Oracle(cfg2)
    c.set_u(u0)
    for _ in range(3):
        a.solve(); c.solve()
    assert np.array_equal(a.get_u(), c.get_u())
