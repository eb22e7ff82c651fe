"""The driven dusty box (config 5 of the benchmark set: 2D Ornstein-Uhlenbeck solenoidal
forcing, charging and growth every step) on the GPU against the CPU oracle.  The forcing
coefficients are advanced on the device from the step's dt; cos/sin/exp/log may differ from the
host's in the last bit, so FP64 is held to 1e-10 relative L1 like the rest.  The box starts at
RMS Mach 1 and shocks within a few steps; where the limiters switch branch on last-bit
differences the FP32 path departs from FP64 faster than in the smooth SI box, so the mixed path is
held to 2e-4 here (measured 8.3e-5 after 12 steps)."""
import numpy as np
import pytest

from shark_gb300 import config as K, setups
from tests.test_gpu_parity import FP64_TOL, MIXED_TOL, rel_l1, run_pair

pytestmark = pytest.mark.gpu


def test_forced_box_fp64():
    cfg, u0 = setups.dusty_turb(n=40, ndust=4, forcing=True, mach=1.0)
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 12)
    assert st == 0
    np.testing.assert_allclose(dtg, dto, rtol=1e-12, atol=0)
    assert rel_l1(cfg, ug, uo).max() <= FP64_TOL


def test_forced_box_mixed():
    cfg, u0 = setups.dusty_turb(n=64, ndust=4, forcing=True, mach=1.0, precision=K.PREC_MIXED)
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 12)
    np.testing.assert_allclose(dtg, dto, rtol=1e-5)
    err = rel_l1(cfg, ug, uo)
    assert err.max() <= 2e-4, err


def test_forced_charged_growing_box_fp64():
    cfg, u0 = setups.dusty_turb(n=24, ndust=6, nH=1e12, smin=1e-5, smax=1e-2, forcing=True, charging=True,
                                growth=True)
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 4)
    np.testing.assert_allclose(dtg, dto, rtol=1e-12, atol=0)
    assert rel_l1(cfg, ug, uo).max() <= FP64_TOL
