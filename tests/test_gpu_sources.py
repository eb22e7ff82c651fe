"""Source_terms beyond the polar geometric terms (src/solver/source_terms.f90:88-118) on the GPU
against the CPU oracle: the drag heating of an adiabatic gas with dust back reaction (a dusty
shock tube, Epstein stopping times on the adiabatic sound speed) and the viscosity of the polar
disk (eta = alpha H cs).  FP64 within 1e-10, mixed within 1e-5 relative L1."""
import numpy as np
import pytest

from shark_gb300 import config as K, setups
from tests.test_gpu_parity import FP64_TOL, MIXED_TOL, rel_l1, run_pair

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ndust", [2, 3])
def test_dusty_shock_tube_fp64(ndust):
    cfg, u0 = setups.sod(nx=800, ndust=ndust, dust2gas=1.0, sizes=(1e-2, 3e-1))
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 150)
    assert st == 0
    np.testing.assert_allclose(dtg, dto, rtol=1e-13, atol=0)
    assert rel_l1(cfg, ug, uo).max() <= FP64_TOL


def test_dusty_shock_tube_mixed():
    cfg, u0 = setups.sod(nx=800, ndust=2, precision=K.PREC_MIXED, sizes=(1e-2, 3e-1))
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 60)
    assert rel_l1(cfg, ug, uo).max() <= 1e-4


@pytest.mark.parametrize("precision,tol", [(K.PREC_FP64, FP64_TOL), (K.PREC_MIXED, MIXED_TOL)])
def test_viscous_disk(precision, tol):
    cfg, u0 = setups.disk_polar(nr=48, nphi=40, ndust=2, noise=1e-2, seed=6, precision=precision)
    cfg.flags |= K.FLAG_VISCOSITY
    cfg.disk_alpha_visc = 0.05
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 20)
    assert st == 0
    assert rel_l1(cfg, ug, uo).max() <= tol
