"""The 2D Ornstein-Uhlenbeck solenoidal forcing of the dustyTurb box (the reference drives 1D
modes only, src/turb/turb.f90:227-324) in the CPU oracle: the kick field is divergence-free and
confined to the forced band, and the coefficients have the stationary variance and the
exp(-dt/tcorr) memory of the process."""
import math

import numpy as np

from shark_gb300 import setups
from oracle.oracle import Oracle


def _box(n=32):
    cfg, u0 = setups.dusty_turb(n=n, ndust=2, forcing=True, mach=1.0)
    return cfg, u0


def test_modes_are_the_band():
    cfg, _ = _box()
    m, c = Oracle(cfg).turb_coef()
    kk = m[:, 2] * cfg.box_l / (2 * math.pi)
    assert len(m) == len(setups.solenoidal_modes(cfg.turb_kmin, cfg.turb_kmax))
    assert np.all((kk >= cfg.turb_kmin - 1e-12) & (kk <= cfg.turb_kmax + 1e-12))


def test_kick_is_solenoidal_and_band_limited():
    cfg, u0 = _box(n=48)
    o = Oracle(cfg)
    o.set_u(u0)
    o.set_dt(1e9)
    o.turb_kick()
    ng, n = cfg.nghost, cfg.nx
    du = (o.get_u() - u0).reshape(cfg.nvar, cfg.ny_max, cfg.nx_max)[:, ng:ng + n, ng:ng + n]
    rho = u0.reshape(cfg.nvar, cfg.ny_max, cfg.nx_max)[0, ng:ng + n, ng:ng + n]
    ax, ay = du[1] / rho, du[2] / rho
    fx, fy = np.fft.fft2(ax), np.fft.fft2(ay)
    k = np.fft.fftfreq(n, d=1.0 / n)
    KY, KX = np.meshgrid(k, k, indexing="ij")
    div = np.abs(KX * fx + KY * fy)
    power = np.abs(fx) ** 2 + np.abs(fy) ** 2
    assert div.max() <= 1e-9 * np.sqrt(power.max())
    kmag = np.sqrt(KX ** 2 + KY ** 2)
    outside = (kmag < cfg.turb_kmin - 1e-9) | (kmag > cfg.turb_kmax + 1e-9)
    assert power[outside].sum() <= 1e-18 * power.sum()
    assert np.all(du[3] == 0) and np.all(du[5:] == 0)


def test_ou_statistics():
    cfg, u0 = _box(n=8)
    cfg.turb_kmax = 6                              # many coefficients for the statistics
    o = Oracle(cfg)
    o.set_u(u0)
    _, c0 = o.turb_coef()
    nm = len(c0)
    sigma = cfg.turb_mach ** 1.5 * cfg.cs0 ** 2 / cfg.box_l / math.sqrt(nm)
    dt = 0.05 * cfg.turb_tcorr
    series = [c0.ravel().copy()]
    o.set_dt(dt)
    for _ in range(400):
        o.turb_kick()
        series.append(o.turb_coef()[1].ravel().copy())
    x = np.array(series) / sigma
    assert abs(x.var() - 1.0) < 0.25
    lag = 5
    r = np.mean(x[:-lag] * x[lag:]) / np.mean(x * x)
    assert abs(r - math.exp(-lag * 0.05)) < 0.1
