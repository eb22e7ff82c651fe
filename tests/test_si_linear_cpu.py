"""The streaming instability's linear growth (tests/si_linear.py) as a pin of the SI box's
equations on the oracle: the theory helper against the published linA and linB growth rates
(Youdin & Johansen 2007: 0.4190 and 0.0154 Omega, tau_s = 0.1, eps = 3 and 0.2, K = 30 and 6),
the drag equilibrium kept by the oracle away from the x edges (at the edges the reference's
force-free ghost cells raise an x-only ramp), and the oracle's growth of the fastest mode on a
box of one wavelength within 3 % of the theory at 32 cells per wavelength (measured -2.2 %; 64
cells: -1.4 %)."""
import math

import numpy as np
import pytest

from oracle.oracle import Oracle
from tests import si_linear as S


@pytest.mark.parametrize("name,eps,K,rate", [("linA", 3.0, 30.0, 0.4190), ("linB", 0.2, 6.0, 0.0154)])
def test_theory_reproduces_published_growth_rates(name, eps, K, rate):
    eta = 0.005
    s, _, _ = S.fastest_mode(K / eta, K / eta, 1e3 * eta, 1.0, [eps], [0.1], eta)
    assert abs(s - rate) <= 5e-5 if name == "linA" else abs(s - rate) <= 1e-4, (s, rate)


def _run(cfg, u0, nsteps):
    o = Oracle(cfg)
    o.set_u(u0)
    o.run(nsteps, 1e9)
    ng = cfg.nghost
    a = o.get_u().reshape(cfg.nvar, cfg.ny_max, cfg.nx_max)[:, ng:-ng, ng:-ng]
    b = u0.reshape(cfg.nvar, cfg.ny_max, cfg.nx_max)[:, ng:-ng, ng:-ng]
    return a, b


@pytest.mark.parametrize("eps", [1e-8, 3.0])
def test_drag_equilibrium_is_stationary_in_the_interior(eps):
    """The equilibrium solved from the box's equations is the oracle's: after one step the cells
    two or more from the x edges keep their densities and in-plane momenta (to 1e-10 of each
    field); the azimuthal momenta move by the operator splitting's O(dt) offset (kick before the
    flux update, implicit drag after it) only."""
    cfg, u0, _, k, x, y = S.eigenmode_box(32, amp=0.0, eps=eps)
    a, b = _run(cfg, u0, 1)
    n = cfg.nx
    for v in (0, 1, 2, 5, 6, 7):
        d = np.abs(a[v][:, 2:n - 2] - b[v][:, 2:n - 2]).max()
        assert d <= 1e-10 * max(np.abs(b[v]).max(), 1e-300), (v, d)
    for v in (3, 8):
        assert np.abs(a[v][:, 2:n - 2] - b[v][:, 2:n - 2]).max() <= 1e-4 * np.abs(b[v]).max(), v


def test_heavy_dust_equilibrium_stays_axisymmetric():
    """With rho_d/rho_g = 3 the uniform equilibrium develops a radial (x) density ramp at the
    shear-periodic edges: the ghost cells carry no force (update_force_setup fills the active
    cells only, SI/setup.f90:335-368), so the predictor does not half-kick them and the edge
    faces' fluxes differ from the interior's, where gas and dust forces are each balanced by the
    drag.  The ramp depends on x only, so the k_y != 0 mode the growth test measures does not see
    it.  The force-free ghost rows act on the y faces too, but there the normal velocity is zero
    and the y dependence stays a thousand times below the ramp."""
    cfg, u0, _, k, x, y = S.eigenmode_box(32, amp=0.0)
    a, b = _run(cfg, u0, 200)
    ramp = np.abs(a[0] - b[0]).max()
    assert ramp > 1e-5
    for v in (0, 5):
        assert np.abs(a[v] - a[v][:1, :]).max() <= 1e-3 * ramp * np.abs(b[v]).max(), v


def test_oracle_linear_growth_matches_theory():
    cfg, u0, s, k, x, y = S.eigenmode_box(32)
    o = Oracle(cfg)
    o.set_u(u0)
    amps = []
    for tend in (1.0, 5.0):
        o.run(10 ** 7, tend)
        amps.append((o.time, S.dust_mode(cfg, o.get_u(), x, y, k)))
    (t1, a1), (t2, a2) = amps
    rate = math.log(a2 / a1) / (t2 - t1)
    assert abs(rate / s - 1.0) <= 0.03, (rate, s)
