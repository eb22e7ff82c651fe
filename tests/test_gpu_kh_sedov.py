"""The KH shear layer and the Sedov blast (src/setups/KH, src/setups/sedov) through the C ABI
against the CPU oracle on the same inputs.

Tolerances as for the other setups' parity tests: FP64 within 1e-10 relative L1 per conserved
field and dt within 1e-14; mixed within 1e-4 (the band edges of KH and the blast's shock front are
discontinuities that amplify FP32 round-off locally, as the Sod tube's mixed test allows)."""
import numpy as np
import pytest

from shark_gb300 import config as K, setups
from tests.test_gpu_parity import FP64_TOL, MIXED_TOL, rel_l1, run_pair

pytestmark = pytest.mark.gpu


def _kh(precision, ndust=4):
    # every MRN bin populated (scut = smax): no species sits at the dust_ratio_min floor
    kw = dict(setups.KH_NML)
    kw.update(scut=kw["smax"])
    return setups.kh(n=96, ny=64, ndust=ndust, precision=precision, **kw)


@pytest.mark.parametrize("ndust", [0, 1, 4])
def test_kh_fp64(ndust):
    cfg, u0 = _kh(K.PREC_FP64, ndust)
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 40)
    assert st == 0
    np.testing.assert_allclose(dtg, dto, rtol=1e-14, atol=0)
    assert rel_l1(cfg, ug, uo).max() <= FP64_TOL


def test_kh_default_parameters_fp64():
    cfg, u0 = setups.kh(n=64, ndust=3)
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 30)
    assert st == 0
    np.testing.assert_allclose(dtg, dto, rtol=1e-14, atol=0)
    assert rel_l1(cfg, ug, uo).max() <= FP64_TOL


@pytest.mark.parametrize("solver", [2, 1, 0])
def test_kh_mixed(solver):
    """The adiabatic two-column gas strips with each gas solver."""
    cfg, u0 = _kh(K.PREC_MIXED)
    cfg.solver = solver
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 30)
    assert st == 0
    np.testing.assert_allclose(dtg, dto, rtol=1e-5, atol=0)
    err = rel_l1(cfg, ug, uo)
    assert err.max() <= MIXED_TOL * 10, err


@pytest.mark.parametrize("slope_type", [1, 3])
def test_sedov_fp64(slope_type):
    cfg, u0 = setups.sedov(n=80, slope_type=slope_type)
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 60)
    assert st == 0
    np.testing.assert_allclose(dtg, dto, rtol=1e-14, atol=0)
    assert rel_l1(cfg, ug, uo).max() <= FP64_TOL


def test_sedov_mixed():
    cfg, u0 = setups.sedov(n=80, precision=K.PREC_MIXED)
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 60)
    assert st == 0
    np.testing.assert_allclose(dtg, dto, rtol=1e-5, atol=0)
    err = rel_l1(cfg, ug, uo)
    assert err.max() <= MIXED_TOL * 10, err


def test_sedov_blast_on_gpu_is_symmetric_and_matches_oracle():
    """200 FP64 steps of the blast: the GPU state equals the oracle's and keeps the blast's
    x <-> y and mirror symmetries (to rounding)."""
    cfg, u0 = setups.sedov(n=64)
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 200)
    assert st == 0
    assert rel_l1(cfg, ug, uo).max() <= FP64_TOL
    g = ug.reshape(cfg.nvar, cfg.ny_max, cfg.nx_max)
    ng = cfg.nghost
    rho = g[0, ng:ng + cfg.ny, ng:ng + cfg.nx]
    assert rho.max() > 1.2 * cfg.sedov_rho_ext                     # the shell has formed
    np.testing.assert_allclose(rho, rho.T, rtol=1e-9, atol=0)
    np.testing.assert_allclose(rho, rho[::-1, :], rtol=1e-9, atol=0)
    np.testing.assert_allclose(rho, rho[:, ::-1], rtol=1e-9, atol=0)


def test_kh_long_run_fp64():
    """300 FP64 steps of the namelist's shear layer with dust: the band's edges roll up the same
    way on the GPU as in the oracle."""
    cfg, u0 = setups.kh(n=64, ndust=4, **setups.KH_NML)
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 300)
    assert st == 0
    np.testing.assert_allclose(dtg, dto, rtol=1e-12, atol=0)
    assert rel_l1(cfg, ug, uo).max() <= FP64_TOL
