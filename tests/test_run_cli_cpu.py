"""The setup runner (python -m shark_gb300.run): its arguments build the same setups the tests
and the benchmark build (no GPU call)."""
import argparse

import numpy as np
import pytest

from shark_gb300 import config as K, run, setups


def _args(setup, **kw):
    d = dict(setup=setup, n=32, nr=16, nphi=32, ndust=4, steps=1, precision="mixed",
             forcing=False, charging=False, growth=False)
    d.update(kw)
    return argparse.Namespace(**d)


@pytest.mark.parametrize("setup", ["si", "turb", "disk", "dustywave", "sod"])
def test_runner_builds_the_named_setup(setup):
    cfg, u0 = run.build_setup(_args(setup))
    assert cfg.precision == K.PREC_MIXED
    assert np.isfinite(u0).all()


def test_runner_si_matches_the_benchmark_setup():
    cfg, u0 = run.build_setup(_args("si", precision="fp64"))
    ref_cfg, ref_u0 = setups.si(n=32, ndust=4, noise=1e-3, seed=1)
    assert cfg.ndust == ref_cfg.ndust and cfg.nx == ref_cfg.nx
    np.testing.assert_array_equal(u0, ref_u0)


def test_runner_turb_flags():
    cfg, _ = run.build_setup(_args("turb", forcing=True, charging=True, growth=True))
    assert cfg.flags & K.FLAG_CHARGING and cfg.flags & K.FLAG_GROWTH
