"""The Cartesian disk (src/setups/disk: setup.f90, boundaries.f90 -> zero_gradients) on the oracle
and the library's validation of its configuration (no GPU).

* Initial state: the setup loop's profile at every cell, ghosts included.
* Boundaries: zero_gradients as written (boundary_types.f90:48-100) takes the cells numbered
  first_active_y, last_active_y, first_active, last_active -- cells of the first ghost row -- as
  sources.  After its first call the ghosts hold cell (2, 0)'s state (0-based), except the top
  ghosts of the active columns left of column ny + 1, which hold cell (ny + 1, 0)'s first state;
  from the second call on every ghost holds cell (2, 0)'s state.
* setup_inloop with its relaxation rate 0: the buffer cells (softened radius < buffer_in box_l
  or > buffer_out box_l) hold the tabulated profile after every step, momenta -+ Omega rho_ana
  (y_soft, x_soft), i.e. turning the other way round from the initial rotation.
"""
import ctypes as C

import numpy as np
import pytest

from shark_gb300 import config as K, setups
from shark_gb300.solver import load_library
from oracle.oracle import Oracle


def _grid(cfg, u):
    return u.reshape(cfg.nvar, cfg.ny_max, cfg.nx_max)


def test_initial_state_is_the_setup_profile():
    cfg, u0 = setups.disk_cart(n=32, ndust=2)
    g = _grid(cfg, u0)
    xx, yy, r_cyl, rr, xs, ys = (a.reshape(cfg.ny_max, cfg.nx_max) for a in setups.disk_cart_geometry(cfg))
    om = np.sqrt(cfg.disk_mstar / rr ** 3)
    r_out = cfg.cdisk_frac_r_disk * cfg.box_l
    sig = np.where(rr > r_out, cfg.disk_sigma0 * cfg.disk_r0 / r_out / 100.0, cfg.disk_sigma0 * cfg.disk_r0 / rr)
    np.testing.assert_allclose(g[0], sig, rtol=1e-14)
    np.testing.assert_allclose(g[1] / g[0], -om * ys, rtol=1e-13)
    np.testing.assert_allclose(g[2] / g[0], om * xs, rtol=1e-13)
    N = cfg.ndust
    for k in range(N):
        np.testing.assert_allclose(g[5 + k], 0.01 * sig, rtol=1e-14)
        np.testing.assert_allclose(g[5 + N + k] / g[5 + k], -om * ys, rtol=1e-13)


@pytest.mark.parametrize("nx,ny", [(32, 32), (40, 24)])
def test_oracle_ghosts_follow_zero_gradients_as_written(nx, ny):
    cfg, _ = setups.disk_cart(n=nx, ndust=2)
    cfg.ny = ny
    u0 = setups.disk_cart_ic(cfg)
    g0 = _grid(cfg, u0).copy()
    o = Oracle(cfg)
    o.set_u(u0)
    o.solve()
    g1 = _grid(cfg, o.get_u())
    ng = cfg.nghost
    ghost = np.ones((cfg.ny_max, cfg.nx_max), bool)
    ghost[ng:ng + ny, ng:ng + nx] = False
    s3, sT = g0[:, 0, 2], g0[:, 0, ny + 1]
    expect = np.repeat(s3[:, None], ghost.sum(), axis=1)
    iy, ix = np.nonzero(ghost)
    top = (iy >= ng + ny) & (ix >= ng) & (ix < ng + nx) & (ix < ny + 1)
    expect[:, top] = sT[:, None]
    np.testing.assert_array_equal(g1[:, iy, ix], expect)
    o.solve()
    g2 = _grid(cfg, o.get_u())
    np.testing.assert_array_equal(g2[:, iy, ix], np.repeat(s3[:, None], ghost.sum(), axis=1))


def test_oracle_buffers_are_reset_every_step():
    cfg, u0 = setups.disk_cart(n=48, ndust=2)
    o = Oracle(cfg)
    o.set_u(u0)
    for _ in range(3):
        o.solve()
    g = _grid(cfg, o.get_u())
    xx, yy, r_cyl, rr, xs, ys = (a.reshape(cfg.ny_max, cfg.nx_max) for a in setups.disk_cart_geometry(cfg))
    ng = cfg.nghost
    act = np.zeros_like(rr, bool)
    act[ng:ng + cfg.ny, ng:ng + cfg.nx] = True
    buf = act & ((rr < cfg.cdisk_buffer_in * cfg.box_l) | (rr > cfg.cdisk_buffer_out * cfg.box_l))
    assert buf.sum() > 0 and (act & ~buf).sum() > 0
    om = np.sqrt(cfg.disk_mstar / rr ** 3)
    r_out = cfg.cdisk_frac_r_disk * cfg.box_l
    rho_ana = np.where(rr > r_out, cfg.disk_sigma0 * cfg.disk_r0 / r_out / 100.0, cfg.disk_sigma0 * cfg.disk_r0 / rr)
    np.testing.assert_allclose(g[0][buf], rho_ana[buf], rtol=1e-14)
    # v_ana = -Omega rho_ana: m_x = -y_soft v_ana = +Omega rho_ana y_soft (the initial state has -)
    np.testing.assert_allclose(g[1][buf], (om * rho_ana * ys)[buf], rtol=1e-13)
    np.testing.assert_allclose(g[2][buf], (-om * rho_ana * xs)[buf], rtol=1e-13)
    N = cfg.ndust
    np.testing.assert_allclose(g[5 + N][buf], (om * rho_ana * yy * 0.01)[buf], rtol=1e-13)
    # the interior evolves
    assert np.abs(g[0][act & ~buf] / _grid(cfg, u0)[0][act & ~buf] - 1.0).max() > 1e-6


@pytest.fixture(scope="module")
def lib():
    try:
        return load_library()
    except OSError as e:
        pytest.skip(f"library not built: {e}")


def test_cartesian_disk_configs_are_checked_before_touching_a_device(lib):
    h = C.c_void_p()
    cd, _ = setups.disk_cart(n=16, ndust=2)
    cases = []
    bad = cd.copy(); bad.ny = 1; cases.append((bad, K.ERR_UNSUPPORTED, b"2D Cartesian"))
    bad = cd.copy(); bad.ny = 20; cases.append((bad, K.ERR_UNSUPPORTED, b"ny <= nx"))
    bad = cd.copy(); bad.iso_cs = -1; cases.append((bad, K.ERR_UNSUPPORTED, b"isothermal"))
    bad = cd.copy(); bad.solverdust = 3; cases.append((bad, K.ERR_UNSUPPORTED, b"HLLC dust"))
    bad = cd.copy(); bad.flags |= K.FLAG_GROWTH; bad.grw_smin = 1e-5; bad.grw_smax = 1.0; bad.grw_cfl = 0.5
    bad.mu_gas = 2.31; cases.append((bad, K.ERR_UNSUPPORTED, b"growth"))
    bad = cd.copy(); bad.cdisk_smooth_r = 0.0; cases.append((bad, K.ERR_INVALID_ARG, b"cdisk_smooth_r"))
    bad = cd.copy(); bad.dust_size[1] = 0.0; cases.append((bad, K.ERR_INVALID_ARG, b"dust_size"))
    cs = (C.c_double * cd.ncells)()
    bad = cd.copy(); bad.cs = C.cast(cs, K._P); cases.append((bad, K.ERR_UNSUPPORTED, b"own grid"))
    for cfg, code, msg in cases:
        assert lib.shark_gpu_init(C.byref(cfg), C.byref(h)) == code, msg
        assert msg in lib.shark_gpu_last_error(), (msg, lib.shark_gpu_last_error())
