"""The streaming instability's linear growth on the GPU (tests/si_linear.py): the SI box of one
wavelength (tau_s = 0.1, eps = 3, K = 30, c_s = 2 eta v_K) seeded with the fastest linear mode.

* FP64, 64 cells per wavelength: the mode's amplitude equals the oracle's on the same input, and
  its growth rate from t = 1 to 5 / Omega is within 2 % of the theory (measured -1.4 %).
* Mixed precision, 64 cells: within 2 % of the theory and within 5e-3 of the FP64 rate (measured
  -1.12 % and 1e-4), seeded at |drho_d| = 1e-3 rho_d: the mode's gas density perturbation is 1e-3
  of the dust's, so at the FP64 tests' 1e-4 it is 3e-7 of rho_g ~ 1, two FP32 units in the last
  place, and the FP32 state does not carry it (the mixed growth then falls 22 % short at 128
  cells); at 1e-3 the mode is still linear over the run (growth x5).
* FP64, 128 cells: within 1 % (the error falls with resolution: -1.4 %, -0.4 %)."""
import math

import numpy as np
import pytest

from shark_gb300 import config as K
from shark_gb300.solver import Shark
from oracle.oracle import Oracle
from tests import si_linear as S

pytestmark = pytest.mark.gpu


def _growth(n, precision, amp=1e-4, with_oracle=False):
    cfg, u0, s, k, x, y = S.eigenmode_box(n, amp=amp, precision=precision)
    out = {"theory": s, "gpu": [], "oracle": []}
    with Shark(cfg) as g:
        g.upload(u0)
        for tend in (1.0, 5.0):
            g.time_loop(tend)
            out["gpu"].append((g.time, S.dust_mode(cfg, g.download(), x, y, k)))
        assert g.sync() == 0
    if with_oracle:
        o = Oracle(cfg)
        o.set_u(u0)
        for tend in (1.0, 5.0):
            o.run(10 ** 7, tend)
            out["oracle"].append((o.time, S.dust_mode(cfg, o.get_u(), x, y, k)))
    for key in ("gpu", "oracle"):
        if out[key]:
            (t1, a1), (t2, a2) = out[key]
            out[key + "_rate"] = math.log(a2 / a1) / (t2 - t1)
    return out


def test_fp64_growth_matches_theory_and_oracle():
    r = _growth(64, K.PREC_FP64, with_oracle=True)
    for (tg, ag), (to, ao) in zip(r["gpu"], r["oracle"]):
        assert abs(tg - to) <= 1e-12 * to and abs(ag / ao - 1.0) <= 1e-8, (tg, to, ag, ao)
    assert abs(r["gpu_rate"] / r["theory"] - 1.0) <= 0.02, (r["gpu_rate"], r["theory"])


def test_mixed_growth_matches_theory_and_fp64():
    m = _growth(64, K.PREC_MIXED, amp=1e-3)
    d = _growth(64, K.PREC_FP64, amp=1e-3)
    assert abs(m["gpu_rate"] / m["theory"] - 1.0) <= 0.02, (m["gpu_rate"], m["theory"])
    assert abs(m["gpu_rate"] / d["gpu_rate"] - 1.0) <= 5e-3, (m["gpu_rate"], d["gpu_rate"])


def test_fp64_growth_converges_with_resolution():
    r = _growth(128, K.PREC_FP64)
    assert abs(r["gpu_rate"] / r["theory"] - 1.0) <= 0.01, (r["gpu_rate"], r["theory"])
