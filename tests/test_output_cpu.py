"""The output writer (src/commons/write_output.f90:2-300) in the CPU oracle: the file set, the
raw stream layout (active cells in cell order, species-major dust fields, unit scaling) against
the oracle's own primitives, and info.dat's Fortran edit descriptors (I11, E23.15)."""
import math
import os

import numpy as np
import pytest

from shark_gb300 import config as K, setups
from oracle.oracle import Oracle, lib


def _active(cfg, a):
    g = np.asarray(a).reshape(-1, cfg.ny_max, cfg.nx_max)
    ng = cfg.nghost
    if cfg.ny == 1:
        return g[:, :, ng:ng + cfg.nx].reshape(g.shape[0], -1)
    return g[:, ng:ng + cfg.ny, ng:ng + cfg.nx].reshape(g.shape[0], -1)


def _read(d, name):
    return np.fromfile(os.path.join(d, name), dtype="<f8")


def _info(d):
    out = {}
    for line in open(os.path.join(d, "info.dat")):
        k, v = line.rstrip("\n").split("=")
        out[k.strip()] = v
    return out


def fortran_e23_15(x):
    """Ew.d of a Fortran processor: [-]0.d1..d15 with a two-digit exponent after E, or a signed
    three-digit exponent without the E, right-justified in 23 characters."""
    if x == 0.0:
        body = "0.000000000000000E+00"
    else:
        m, e = f"{abs(x):.14E}".split("E")
        e = int(e) + 1
        digits = m.replace(".", "")
        ex = f"E{'+' if e >= 0 else '-'}{abs(e):02d}" if abs(e) <= 99 else f"{'+' if e >= 0 else '-'}{abs(e):03d}"
        body = ("-" if x < 0 else "") + "0." + digits + ex
    return body.rjust(23)


def test_e23_15_examples():
    assert fortran_e23_15(1.0) == "  0.100000000000000E+01"
    assert fortran_e23_15(-2.5e-3) == " -0.250000000000000E-02"
    assert fortran_e23_15(1.0e100) == "  0.100000000000000+101"
    assert fortran_e23_15(0.0) == "  0.000000000000000E+00"


@pytest.mark.parametrize("make", ["si", "sod", "disk", "turb", "kh"])
def test_oracle_output_layout(tmp_path, make):
    if make == "si":
        cfg, u0 = setups.si(n=16, ndust=3)
    elif make == "sod":
        cfg, u0 = setups.sod(nx=64, ndust=2)
    elif make == "disk":
        cfg, u0 = setups.disk_polar_au(nr=12, nphi=16, ndust=2, noise=1e-2)
    elif make == "kh":
        cfg, u0 = setups.kh(n=12, ndust=2, **setups.KH_NML)
    else:
        cfg, u0 = setups.dusty_turb(n=8, ndust=3, charging=True)
    o = Oracle(cfg)
    o.set_u(u0)
    if make == "turb":
        o.apply_boundaries()
        o.charge()
    o.solve()
    o.output(7, 0.125, str(tmp_path) + "/")
    d = os.path.join(str(tmp_path), "output_00007")
    info = _info(d)
    N = cfg.ndust
    assert int(info["nvar"]) == cfg.nvar and int(info["ndust"]) == N
    assert int(info["NX"]) == cfg.nx and int(info["NY"]) == cfg.ny and int(info["GEOM"]) == cfg.geom
    assert info["time"] == fortran_e23_15(0.125)
    ul = cfg.unit_l or 1.0
    ud = cfg.unit_d or 1.0
    ut = cfg.unit_t or 1.0
    uv = ul / ut
    uP = ud * (uv * uv) if cfg.setup == K.SETUP_KH else uv * uv     # KH/units.f90: unit_d unit_v**2
    assert info["unit_v"] == fortran_e23_15(uv) and info["unit_p"] == fortran_e23_15(uP)
    for line in open(os.path.join(d, "info.dat")):
        assert len(line.rstrip("\n").split("=")[1]) in (11, 23)
    q, _ = o.get_q()
    qa = _active(cfg, q.reshape(cfg.nvar, -1))
    nact = qa.shape[1]
    polar = cfg.geom == 2
    urho = ud * ul if polar else ud
    np.testing.assert_array_equal(_read(d, "rho"), qa[0] * urho)
    np.testing.assert_array_equal(_read(d, "v"), qa[1] * uv)
    np.testing.assert_array_equal(_read(d, "vy"), qa[2] * uv)
    np.testing.assert_array_equal(_read(d, "vz"), qa[3] * uv)
    np.testing.assert_array_equal(_read(d, "P"), qa[4] * uP * ul if polar else qa[4] * uP)
    grid = o.grid()
    xs = grid["radii_c"] if polar else grid["position"][0]
    np.testing.assert_array_equal(_read(d, "x"), _active(cfg, xs)[0])
    if cfg.ny > 1:
        np.testing.assert_array_equal(_read(d, "y"), _active(cfg, grid["position"][1])[0])
    else:
        assert not os.path.exists(os.path.join(d, "y"))
    if N:
        rhod = _read(d, "rhod").reshape(N, nact)
        np.testing.assert_array_equal(rhod, qa[5:5 + N] * urho)
        tot = np.zeros(nact)
        for k in range(N):
            tot = tot + qa[5 + k] * urho
        np.testing.assert_array_equal(_read(d, "rhod_tot"), tot)
        np.testing.assert_array_equal(_read(d, "vd").reshape(N, nact), qa[5 + N:5 + 2 * N] * uv)
        np.testing.assert_array_equal(_read(d, "vdz").reshape(N, nact), qa[5 + 3 * N:5 + 4 * N] * uv)
        sd = _read(d, "sd").reshape(N, nact)
        for k in range(N):
            assert np.all(sd[k] == cfg.dust_size[k] * ul)
    files = set(os.listdir(d))
    assert ({"eta_a", "eta_o", "eta_h", "ni", "ne"} <= files) == bool(cfg.flags & K.FLAG_CHARGING)
    if cfg.flags & K.FLAG_CHARGING:
        ch = o.get_charge()
        np.testing.assert_array_equal(_read(d, "ni"), _active(cfg, ch["ni"])[0])
        np.testing.assert_array_equal(_read(d, "eta_a"), _active(cfg, ch["eta"][2])[0])
        np.testing.assert_array_equal(_read(d, "zd").reshape(N, nact), _active(cfg, ch["zd"]))
