"""Polar disk (geom 2, log grid, point-mass gravity, Epstein drag on Sigma/(sqrt(2 pi) H),
inner relaxation, outflow radial boundaries) and the FARGO orbital remap: the GPU path through
the C ABI against the CPU oracle on the same inputs.

Tolerances as for the other setups: FP64 within 1e-10 relative L1 per conserved field (the
relaxation factor exp(-dt/t_rel) is the one transcendental of the step whose device and host
results may differ in the last bit), mixed precision within 1e-5.
"""
import numpy as np
import pytest

from shark_gb300 import config as K, setups
from shark_gb300.solver import Shark
from oracle.oracle import Oracle
from tests.test_gpu_parity import FP64_TOL, MIXED_TOL, rel_l1, run_pair

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fargo", [False, True])
@pytest.mark.parametrize("ndust,slope_type", [(4, 1), (3, 3), (0, 2)])
def test_disk_fp64(fargo, ndust, slope_type):
    cfg, u0 = setups.disk_polar(nr=40, nphi=48, ndust=ndust, noise=1e-2, seed=5, fargo=fargo,
                                slope_type=slope_type)
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 25)
    assert st == 0
    np.testing.assert_allclose(dtg, dto, rtol=1e-13, atol=0)
    assert rel_l1(cfg, ug, uo).max() <= FP64_TOL


def test_disk_fargo_whole_cell_shifts_fp64():
    """CFL 2.6: the inner rings move by more than one cell per step (nshft > 0)."""
    cfg, u0 = setups.disk_polar(nr=40, nphi=48, ndust=3, noise=1e-2, seed=3, fargo=True, cfl=2.6,
                                slope_type=3)
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 6)
    np.testing.assert_allclose(dtg, dto, rtol=1e-13, atol=0)
    assert rel_l1(cfg, ug, uo).max() <= FP64_TOL


def test_disk_ragged_columns_fp64():
    """nr not a multiple of the flux strip width nor of the FARGO column block."""
    cfg, u0 = setups.disk_polar(nr=57, nphi=36, ndust=2, noise=1e-2, seed=9, fargo=True)
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 15)
    np.testing.assert_allclose(dtg, dto, rtol=1e-13, atol=0)
    assert rel_l1(cfg, ug, uo).max() <= FP64_TOL


@pytest.mark.parametrize("fargo", [False, True])
def test_disk_mixed(fargo):
    cfg, u0 = setups.disk_polar(nr=96, nphi=128, ndust=4, noise=1e-2, seed=2, fargo=fargo,
                                precision=K.PREC_MIXED)
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 20)
    assert st == 0
    np.testing.assert_allclose(dtg, dto, rtol=1e-5)
    assert rel_l1(cfg, ug, uo).max() <= MIXED_TOL


def test_disk_relaxation_reference_is_first_upload():
    cfg, u0 = setups.disk_polar(nr=40, nphi=32, ndust=2, noise=1e-2, seed=4)
    u1 = setups.disk_ic(cfg, 2e-2, 8)
    o = Oracle(cfg)
    o.set_u(u0)
    o.set_u(u1)
    with Shark(cfg) as g:
        g.upload(u0)
        g.solve()
        g.upload(u1)
        for _ in range(10):
            o.solve()
            g.solve()
        assert rel_l1(cfg, g.download(), o.get_u()).max() <= FP64_TOL
