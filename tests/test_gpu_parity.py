"""GPU path (through the C ABI) against the CPU oracle on the same inputs.

Tolerances: the FP64 path must match the oracle within 1e-10 relative L1 on every conserved field
(it is built without FMA contraction and follows the oracle's operation order, so it is usually
bit-identical); the mixed path (FP32 state and flux/update, FP64 drag/dt) within 1e-5.
"""
import numpy as np
import pytest

from shark_gb300 import config as K, setups
from shark_gb300.solver import Shark, SharkError
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
MIXED_TOL = 1e-5


def active(cfg, u):
    g = u.reshape(cfg.nvar, cfg.ny_max, cfg.nx_max)
    if cfg.ny == 1:
        return g[:, :, cfg.nghost:cfg.nghost + cfg.nx]
    return g[:, cfg.nghost:cfg.nghost + cfg.ny, cfg.nghost:cfg.nghost + cfg.nx]


def field_scales(cfg, B):
    """L1 scale of every conserved field: densities and energy by their own L1 norm, each
    momentum component by the L1 norm of its species' momentum magnitude (a component whose
    mean is zero, e.g. the gas vertical momentum of the SI box, has no meaningful own scale)."""
    N = cfg.ndust
    sc = np.array([np.sum(np.abs(B[v])) for v in range(cfg.nvar)])
    comps = [(1, 2, 3)] + [(5 + N + k, 5 + 2 * N + k, 5 + 3 * N + k) for k in range(N)]
    for c in comps:
        mag = np.sum(np.sqrt(B[c[0]] ** 2 + B[c[1]] ** 2 + B[c[2]] ** 2))
        for v in c:
            sc[v] = mag
    return sc


def rel_l1(cfg, a, b):
    """Relative L1 error of a against b per conserved field over the active cells."""
    A, B = active(cfg, a), active(cfg, b)
    sc = field_scales(cfg, B)
    num = np.array([np.sum(np.abs(A[v] - B[v])) for v in range(cfg.nvar)])
    return np.where(sc > 0, num / np.where(sc > 0, sc, 1.0), num)


def run_pair(cfg, u0, nsteps):
    o = Oracle(cfg)
    o.set_u(u0)
    g = Shark(cfg)
    g.upload(u0)
    dts_o, dts_g = [], []
    for _ in range(nsteps):
        dts_o.append(o.solve())
        dts_g.append(g.solve())
    ug = g.download()
    st = g.sync()
    uo = o.get_u()
    g.close()
    return np.array(dts_o), np.array(dts_g), uo, ug, st


@pytest.mark.parametrize("solver", [0, 1, 2])
@pytest.mark.parametrize("slope_type", [1, 2, 3])
def test_sod_fp64(solver, slope_type):
    cfg, u0 = setups.sod(nx=1000, gamma=1.4, cfl=0.5, slope_type=slope_type, solver=solver)
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 120)
    assert st == 0
    np.testing.assert_allclose(dtg, dto, rtol=1e-14, atol=0)
    assert rel_l1(cfg, ug, uo).max() <= FP64_TOL


def test_sod_full_run_to_tend():
    cfg, u0 = setups.sod(nx=1000, gamma=1.4, cfl=0.5, slope_type=1)
    o = Oracle(cfg)
    o.set_u(u0)
    n_o = o.run(10 ** 6, 0.2)
    with Shark(cfg) as g:
        g.upload(u0)
        n_g = g.time_loop(0.2)
        assert n_g == n_o
        assert abs(g.time - o.time) <= 1e-14
        assert rel_l1(cfg, g.download(), o.get_u()).max() <= FP64_TOL


@pytest.mark.parametrize("solverdust", [0, 1, 2, 3])
def test_dustywave_fp64(solverdust):
    cfg, u0 = setups.dustywave(nx=2048, ndust=4)
    cfg.solverdust = solverdust
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 200)
    assert st == 0
    np.testing.assert_allclose(dtg, dto, rtol=1e-14, atol=0)
    assert rel_l1(cfg, ug, uo).max() <= FP64_TOL


@pytest.mark.parametrize("ndust", [1, 3, 8])
def test_si_fp64_ragged_tiles(ndust):
    """SI box of 70 x 45 active cells: partial tiles in both directions."""
    cfg, u0 = _ragged_si(70, 45, ndust)
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 25)
    assert st == 0
    np.testing.assert_allclose(dtg, dto, rtol=1e-14, atol=0)
    assert rel_l1(cfg, ug, uo).max() <= FP64_TOL


def _ragged_si(nx, ny, ndust, precision=K.PREC_FP64):
    cfg, _ = setups.si(n=16, ndust=ndust, precision=precision)
    cfg.nx, cfg.ny = nx, ny
    u0 = setups.si_ic(cfg, 1e-3 * cfg.cs0, 5)
    return cfg, u0


@pytest.mark.parametrize("precision,tol", [(K.PREC_FP64, FP64_TOL), (K.PREC_MIXED, MIXED_TOL)])
def test_si_hllc_dust(precision, tol):
    """solver_hllc_dust (solvers.f90:704-836, SOLVERDUST=3) on the SI box: ragged tiles in FP64,
    the generic FP32 strips in mixed precision."""
    cfg, u0 = _ragged_si(70, 45, 4, precision=precision)
    cfg.solverdust = 3
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 25)
    assert st == 0
    np.testing.assert_allclose(dtg, dto, rtol=1e-14 if precision == K.PREC_FP64 else 1e-5, atol=0)
    assert rel_l1(cfg, ug, uo).max() <= tol


def test_si_without_force_kick_uses_inloop_rotation():
    cfg, u0 = setups.si(n=64, ndust=4, force_kick=False)
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 20)
    np.testing.assert_allclose(dtg, dto, rtol=1e-14, atol=0)
    assert rel_l1(cfg, ug, uo).max() <= FP64_TOL


@pytest.mark.parametrize("solver,slope_type", [(2, 3), (1, 3), (0, 3), (2, 1), (2, 2)])
def test_si_mixed_precision(solver, slope_type):
    """Every gas solver and limiter of the two-column strips on the isothermal box."""
    cfg, u0 = setups.si(n=128, ndust=8, precision=K.PREC_MIXED, slope_type=slope_type)
    cfg.solver = solver
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 30)
    assert st == 0
    np.testing.assert_allclose(dtg, dto, rtol=1e-5, atol=0)
    err = rel_l1(cfg, ug, uo)
    assert err.max() <= MIXED_TOL, err


def test_sod_mixed_precision():
    cfg, u0 = setups.sod(nx=1000, gamma=1.4, precision=K.PREC_MIXED)
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 100)
    assert rel_l1(cfg, ug, uo).max() <= MIXED_TOL * 10   # shocks amplify FP32 round-off locally


def test_totals_and_ctoprim_match_oracle():
    cfg, u0 = setups.si(n=64, ndust=4)
    o = Oracle(cfg)
    o.set_u(u0)
    with Shark(cfg) as g:
        g.upload(u0)
        for _ in range(5):
            o.solve()
            g.solve()
        tg = g.totals().reshape(-1)
        to = o.totals()
        np.testing.assert_allclose(tg, to, rtol=1e-12, atol=1e-18)
        qg, csg = g.ctoprim()
        qo, cso = o.get_q()
        ag, ao = active(cfg, qg), active(cfg, qo)
        np.testing.assert_allclose(ag, ao, rtol=1e-12, atol=1e-300)


def test_sod_2d_both_directions():
    cfg, u0 = setups.sod(nx=64, ny=40, gamma=1.4)
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 40)
    assert rel_l1(cfg, ug, uo).max() <= FP64_TOL


def test_bad_state_sets_status_and_context_recovers():
    """A state with a negative density is a host-side fault injection: the kernels flag it in the
    status word, the GPU context stays usable and a good state runs normally afterwards."""
    cfg, u0 = setups.dustywave(nx=256, ndust=2)
    bad = u0.copy()
    nc = cfg.ncells
    bad[10] = -1.0            # gas density of one active cell
    with Shark(cfg) as g:
        g.upload(bad)
        for _ in range(3):
            g.solve()
        st = g.sync()
        assert st & (K.STATUS_NEG_DENSITY | K.STATUS_NAN)
        g.upload(u0)
        for _ in range(3):
            g.solve()
        assert g.sync() == 0


def test_static_flag_leaves_state_untouched():
    cfg, u0 = setups.sod(nx=128)
    cfg.flags |= K.FLAG_STATIC
    with Shark(cfg) as g:
        g.upload(u0)
        g.solve()
        g.solve()
        assert np.array_equal(active(cfg, g.download()), active(cfg, u0))


def test_timed_run_matches_stepping():
    """The benchmark helper queues its steps without host waits: the same states and times as
    stepping one solve() at a time, and ordinary steps carry on after it."""
    cfg, u0 = setups.si(n=64, ndust=4)
    with Shark(cfg) as a, Shark(cfg) as b:
        a.upload(u0)
        b.upload(u0)
        a.solve()
        b.solve()
        t = 0.0
        for _ in range(7):
            t = t + a.solve()
        t0 = b.time
        ms = b.timed_run(7)
        assert ms > 0.0
        assert b.time - t0 == pytest.approx(t, rel=1e-15)
        assert np.array_equal(a.download(), b.download())
        assert a.solve() == b.solve()
        assert np.array_equal(a.download(), b.download())
        assert a.sync() == b.sync() == 0


@pytest.mark.parametrize("make", ["si_mixed", "si_fp64", "disk_mixed"])
def test_pinned_host_buffers_match_pageable(make):
    """Pinned host buffers are read and written by the conversion kernels directly; pageable ones go
    through the staging copy.  Both give the same states, the polar disk's relaxation reference
    (the first upload) included."""
    torch = pytest.importorskip("torch")
    if make == "disk_mixed":
        cfg, u0 = setups.disk_polar(nr=40, nphi=32, ndust=2, noise=1e-2, seed=3, fargo=True, precision=K.PREC_MIXED)
    else:
        cfg, u0 = setups.si(n=64, ndust=4, precision=K.PREC_MIXED if make == "si_mixed" else K.PREC_FP64)
    pin = torch.empty(u0.size, dtype=torch.float64).pin_memory()
    pin.numpy()[:] = u0
    with Shark(cfg) as a, Shark(cfg) as b:
        a.upload(u0)
        b.upload_ptr(pin.data_ptr())
        for _ in range(4):
            assert a.solve() == b.solve()
        ua = a.download()
        pin.numpy()[:] = 0.0
        b.download_ptr(pin.data_ptr())
        assert np.array_equal(ua, pin.numpy())
        a.upload(ua)
        b.upload_ptr(pin.data_ptr())
        for _ in range(2):
            assert a.solve() == b.solve()
        assert np.array_equal(a.download(), b.download())


def test_unsupported_options_fail_loudly():
    cfg, _ = setups.si(n=32, ndust=2)
    cfg.flags |= K.FLAG_GROWTH
    with pytest.raises(SharkError) as e:
        Shark(cfg)
    assert e.value.code == K.ERR_UNSUPPORTED
