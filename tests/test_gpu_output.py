"""The device output writer (src/commons/write_output.f90:2-300) against the oracle's restatement
after the same steps, and the restart reader (the reference's read_output is a stub).

Files: the same set, info.dat text identical, every field stream within the path's parity
tolerance, as relative L1 with velocities scaled by the species' velocity magnitude (FP64: 1e-10,
set by the last bit of exp() in the charging and the disk relaxation; mixed: 1e-5, and 2e-4 for
the Mach-1 forced box and the KH shear layer, whose band edges amplify FP32 round-off).  Restart: the state read back
equals the written one to rounding (unit scaling and ctoprim/primtoc round trip, 1e-13 relative),
and the next step's dt agrees to 1e-12."""
import os

import numpy as np
import pytest

from shark_gb300 import config as K, setups
from shark_gb300.solver import Shark, SharkError
from oracle.oracle import Oracle
from tests.test_gpu_parity import active

pytestmark = pytest.mark.gpu


def _case(make, precision=K.PREC_FP64):
    if make == "si":
        return setups.si(n=32, ndust=3, precision=precision)
    if make == "disk":
        return setups.disk_polar_au(nr=24, nphi=32, ndust=3, noise=1e-2, precision=precision)
    if make == "kh":
        return setups.kh(n=32, ndust=3, precision=precision, **setups.KH_NML)
    return setups.dusty_turb(n=64, ndust=4, charging=True, forcing=True, precision=precision)


def _files(d):
    return sorted(os.listdir(d))


@pytest.mark.parametrize("make", ["si", "disk", "turb", "kh"])
@pytest.mark.parametrize("prec", [K.PREC_FP64, K.PREC_MIXED])
def test_output_matches_oracle(tmp_path, make, prec):
    cfg, u0 = _case(make, prec)
    o = Oracle(cfg)
    o.set_u(u0)
    t = 0.0
    with Shark(cfg) as g:
        g.upload(u0)
        for _ in range(3):
            t += o.solve()
            g.solve()
        os.makedirs(tmp_path / "gpu", exist_ok=True)
        g.output(3, t, str(tmp_path / "gpu") + "/")
    os.makedirs(tmp_path / "cpu", exist_ok=True)
    o.output(3, t, str(tmp_path / "cpu") + "/")
    dg, dc = tmp_path / "gpu" / "output_00003", tmp_path / "cpu" / "output_00003"
    assert _files(dg) == _files(dc)
    assert open(dg / "info.dat").read() == open(dc / "info.dat").read()
    R = lambda d, n: np.fromfile(d / n, dtype="<f8")
    tol = 1e-10 if prec == K.PREC_FP64 else (2e-4 if make in ("turb", "kh") else 1e-5)
    for name in _files(dc):
        if name == "info.dat":
            continue
        a, b = R(dg, name), R(dc, name)
        assert a.size == b.size, name
        if name in ("x", "y", "sd"):
            assert np.array_equal(a, b), name
            continue
        if name in ("v", "vy", "vz"):
            scale = np.sqrt(R(dc, "v") ** 2 + R(dc, "vy") ** 2 + R(dc, "vz") ** 2).sum()
        elif name in ("vd", "vdy", "vdz"):
            scale = np.sqrt(R(dc, "vd") ** 2 + R(dc, "vdy") ** 2 + R(dc, "vdz") ** 2).sum()
        else:
            scale = np.abs(b).sum()
        err = np.abs(a - b).sum() / max(scale, 1e-300)
        assert err <= tol, (name, err)


@pytest.mark.parametrize("make", ["si", "disk", "turb", "kh"])
def test_restart_round_trip(tmp_path, make):
    cfg, u0 = _case(make)
    with Shark(cfg) as a, Shark(cfg) as b:
        a.upload(u0)
        for _ in range(3):
            a.solve()
        ua = a.download()
        d = a.output(12, 0.5, str(tmp_path) + "/")
        assert b.read_output(d) == 0.5
        ub = b.download()
        A, B = active(cfg, ua), active(cfg, ub)
        keep = [v for v in range(cfg.nvar) if v != 4]           # isothermal boxes: E is not evolved
        for v in keep:
            scale = np.abs(A[v]).max()
            assert np.abs(B[v] - A[v]).max() <= 1e-13 * max(scale, 1e-300), v
        dta, dtb = a.solve(), b.solve()
        assert dtb == pytest.approx(dta, rel=1e-12)


def test_restart_rejects_another_configuration(tmp_path):
    cfg, u0 = _case("si")
    with Shark(cfg) as a:
        a.upload(u0)
        d = a.output(1, 0.0, str(tmp_path) + "/")
    cfg2, _ = setups.si(n=32, ndust=4)
    with Shark(cfg2) as b:
        with pytest.raises(SharkError):
            b.read_output(d)
