"""Polar disk and FARGO on the CPU: the host-side setup builder against the oracle, and
properties of the oracle's orbital remap (src/solver/fargo_scheme.f90:2-81) that do not depend
on the restatement being right (conservation per ring, the first-order remap as an explicit
linear interpolation between shifted rings)."""
import math

import numpy as np
import pytest

from shark_gb300 import setups
from oracle.oracle import Oracle


@pytest.mark.parametrize("noise,fargo", [(0.0, False), (1e-2, True)])
def test_disk_ic_matches_oracle(noise, fargo):
    cfg, u0 = setups.disk_polar(nr=40, nphi=48, ndust=4, noise=noise, seed=7, fargo=fargo)
    o = Oracle(cfg)
    o.setup_ic(noise, 7)
    assert np.array_equal(o.get_u(), u0)


def test_disk_log_grid_matches_oracle():
    cfg, _ = setups.disk_polar(nr=40, nphi=48, ndust=2)
    g = Oracle(cfg).grid()
    r = np.asarray(g["radii_c"]).reshape(cfg.ny_max, cfg.nx_max)
    for iy in range(cfg.ny_max):
        assert np.array_equal(r[iy], setups.disk_radii(cfg))
    # log spacing: constant ratio of consecutive active radii
    ra = setups.disk_radii(cfg)[cfg.nghost:cfg.nghost + cfg.nx]
    ratio = ra[1:] / ra[:-1]
    assert np.ptp(ratio) < 1e-12


def _ring_shift_state(cfg, slope_type, noise=0.05):
    cfg.slope_type = slope_type
    u0 = setups.disk_ic(cfg, noise, 11)
    o = Oracle(cfg)
    o.set_u(u0)
    # a dt that moves the inner rings by ~1.7 cells: whole-cell shifts plus a fraction
    r = setups.disk_radii(cfg)
    dphi = 2.0 * math.pi / cfg.ny
    ri = r[cfg.nghost]
    dt = 1.7 * ri * dphi / math.sqrt(cfg.disk_mstar / ri)
    o.set_dt(dt)
    return o, u0, dt


@pytest.mark.parametrize("slope_type", [0, 1, 2, 3])
def test_fargo_conserves_every_ring(slope_type):
    cfg, _ = setups.disk_polar(nr=24, nphi=40, ndust=2, fargo=True)
    o, u0, _ = _ring_shift_state(cfg, slope_type)
    o.fargo()
    u1 = o.get_u()
    ng = cfg.nghost
    a0 = u0.reshape(cfg.nvar, cfg.ny_max, cfg.nx_max)[:, ng:ng + cfg.ny, ng:ng + cfg.nx]
    a1 = u1.reshape(cfg.nvar, cfg.ny_max, cfg.nx_max)[:, ng:ng + cfg.ny, ng:ng + cfg.nx]
    s0, s1 = a0.sum(axis=1), a1.sum(axis=1)          # (nvar, nx): one sum per ring
    scale = np.abs(a0).sum(axis=1)
    assert np.all(np.abs(s1 - s0) <= 1e-13 * scale)
    assert not np.array_equal(a0, a1)


def test_fargo_first_order_is_interpolation_between_shifted_rings():
    cfg, _ = setups.disk_polar(nr=24, nphi=40, ndust=1, fargo=True)
    o, u0, dt = _ring_shift_state(cfg, 0)
    o.fargo()
    u1 = o.get_u().reshape(cfg.nvar, cfg.ny_max, cfg.nx_max)
    g0 = u0.reshape(cfg.nvar, cfg.ny_max, cfg.nx_max)
    ng, ny = cfg.nghost, cfg.ny
    r = setups.disk_radii(cfg)
    dphi = 2.0 * math.pi / ny
    for ix in range(ng, ng + cfg.nx):
        vk = -math.sqrt(cfg.disk_mstar / r[ix] ** 3) * r[ix]
        cells = abs(vk * dt) / (r[ix] * dphi)
        n, eps = int(cells), cells - int(cells)
        ring = g0[:, ng:ng + ny, ix]
        # vk < 0: the value at phi_a comes from a + n and a + n + 1
        want = (1.0 - eps) * np.roll(ring, -n, axis=1) + eps * np.roll(ring, -n - 1, axis=1)
        np.testing.assert_allclose(u1[:, ng:ng + ny, ix], want, rtol=1e-12, atol=0)


def test_disk_relaxation_reference_is_the_first_state():
    """setup_inloop relaxes towards the first state given (uprim_condinit), not a later one."""
    cfg, u0 = setups.disk_polar(nr=24, nphi=16, ndust=1)
    a = Oracle(cfg)
    a.set_u(u0)
    u1 = u0 * 1.01
    a.set_u(u1)
    b = Oracle(cfg)
    b.set_u(u0)
    b.set_u(u1)
    c = Oracle(cfg)
    c.set_u(u1)
    a.solve(); b.solve(); c.solve()
    assert np.array_equal(a.get_u(), b.get_u())
    assert not np.array_equal(a.get_u(), c.get_u())


def test_disk_run_stays_finite_and_first_column_frozen():
    cfg, u0 = setups.disk_polar(nr=32, nphi=32, ndust=3, noise=1e-2, fargo=True)
    o = Oracle(cfg)
    o.set_u(u0)
    o.run(40)
    u = o.get_u().reshape(cfg.nvar, cfg.ny_max, cfg.nx_max)
    assert np.isfinite(u).all()
    g0 = u0.reshape(cfg.nvar, cfg.ny_max, cfg.nx_max)
    ng = cfg.nghost
    # the first active column is reset to its initial state every step
    assert np.array_equal(u[:, ng:ng + cfg.ny, ng], g0[:, ng:ng + cfg.ny, ng])
