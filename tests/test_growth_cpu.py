"""Dust growth (src/dust/dust_growth.f90:3-256) in the CPU oracle against what the mathematics
of the Smoluchowski equation fixes independently of the restatement: mass conservation, and the
total number density of the constant kernel, N(t) = N0/(1 + K N0 t/2), and of the additive kernel,
N(t) = N0 exp(-M t), from a monodisperse start (the mass grid with eta = 2 resolves them to a few
per cent)."""
import math

import numpy as np
import pytest

from shark_gb300 import setups, config as K
from oracle.oracle import Oracle


def _kernel_box(kernel, N=24):
    cfg, u0 = setups.dusty_turb(n=4, ndust=N)
    cfg.flags |= K.FLAG_GROWTH
    cfg.grw_kernel = kernel
    cfg.grw_smin, cfg.grw_smax = 1.0, 2.0 ** (N / 3.0)      # eta = 2
    zeta = (cfg.grw_smax / cfg.grw_smin) ** (1.0 / N)
    for k in range(N):
        cfg.dust_size[k] = math.sqrt(zeta ** k * zeta ** (k + 1))
    m = np.array([cfg.dust_size[k] ** 3 for k in range(N)])
    g = u0.reshape(cfg.nvar, -1)
    g[5:5 + N] = 1e-30 * g[0]
    g[5] = m[0]                                              # n0 = 1 in the first bin
    g[5 + N:] = 0.0
    return cfg, u0, m


def _cell(cfg, u):
    return u.reshape(cfg.nvar, -1)[:, 2 * cfg.nx_max + 2]


@pytest.mark.parametrize("kernel", [1, 2])
def test_analytic_kernels(kernel):
    cfg, u0, m = _kernel_box(kernel)
    N = cfg.ndust
    o = Oracle(cfg)
    o.set_u(u0)
    M0 = _cell(cfg, u0)[5:5 + N].sum()
    t = 0.0
    for _ in range(16):
        o.set_dt(0.25)
        o.growth()
        t += 0.25
        rk = _cell(cfg, o.get_u())[5:5 + N]
        n = np.sum(rk / m)
        exact = 1.0 / (1.0 + t / 2.0) if kernel == 1 else math.exp(-M0 * t)
        assert abs(n / exact - 1.0) < 0.08, (t, n, exact)
        assert abs(rk.sum() / M0 - 1.0) < 1e-13


@pytest.mark.parametrize("mode", [K.GROWTH_TURB | K.GROWTH_BROWNIAN | K.GROWTH_DRIFT,
                                  K.GROWTH_TURB | K.GROWTH_BROWNIAN | K.GROWTH_FRAGMENTATION])
def test_physical_kernel_conserves_mass_and_grows(mode):
    cfg, u0 = setups.dusty_turb(n=8, ndust=12, nH=1e12, smin=1e-5, smax=1e-2)
    cfg.flags |= K.FLAG_GROWTH
    cfg.grw_mode = mode
    cfg.grw_smin, cfg.grw_smax = 1e-5, 1e-2
    cfg.grw_eps_thr = cfg.grw_eps_thr_frag = 0.0
    o = Oracle(cfg)
    o.set_u(u0)
    N = cfg.ndust
    r0 = _cell(cfg, u0)[5:5 + N].copy()
    o.set_dt(3e8)                 # short enough that no bin reaches the dust floor
    it = o.growth()
    r1 = _cell(cfg, o.get_u())[5:5 + N]
    assert r1.min() > 1e3 * cfg.dust_ratio_min * _cell(cfg, u0)[0]
    # each bin's net rate is a difference of pair terms up to ~1e5 times larger: rounding level
    assert abs(r1.sum() / r0.sum() - 1.0) < 1e-9
    assert it.max() > 1
    s = np.array(cfg.dust_size[:N])
    assert np.sum(r1 * s) > np.sum(r0 * s) or (mode & K.GROWTH_FRAGMENTATION)


def test_growth_inside_the_step():
    cfg, u0 = setups.dusty_turb(n=12, ndust=6, nH=1e12, smin=1e-5, smax=1e-2)
    cfg.flags |= K.FLAG_GROWTH
    cfg.grw_mode = K.GROWTH_TURB | K.GROWTH_BROWNIAN | K.GROWTH_DRIFT
    cfg.grw_smin, cfg.grw_smax = 1e-5, 1e-2
    o = Oracle(cfg)
    o.set_u(u0)
    for _ in range(3):
        o.solve()
    assert np.isfinite(o.get_u()).all()
