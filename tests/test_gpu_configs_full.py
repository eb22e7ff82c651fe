"""The benchmark configurations at their own sizes and species counts, GPU (through the C ABI)
against the CPU oracle on the same inputs, every feature of the configuration switched on.

* SI box, 1024^2 active cells, 8 species (config 3, the bench workload), FP64 and mixed.
* Polar disk with FARGO, growth and charging at 128 x 256 cells (a coarser grid of the
  512 x 1024 case: the oracle's charging and growth are the slow part), 16 species.
* Driven dusty box with OU forcing, charging and growth at 128^2 cells, 32 species.  32 species
  take the run-time species path of K2; 8 and 16 the compile-time register paths.
* The 4-species dusty wave to t = 2 (config 2) in FP64 and mixed precision, against the oracle
  and against the linear multi-species solution (tests/dusty_wave_linear.py).

Tolerances: FP64 within 1e-10 relative L1 per conserved field; mixed within 1e-5, except where
growth is on (the reference's explicit growth sub-cycling moves with the sub-step count: 1e-2 on
the dust fields, 1e-4 on the gas fields, 1e-5 on the total dust mass, as in test_gpu_growth.py)
and on the driven Mach-1 box (2e-4, as in test_gpu_turb.py).

FP64 with growth on the driven boxes: the reference's explicit growth sub-cycle (sub-steps of
CFL_growth rho_k/|drho_k/dt|, dust_growth.f90:117-249) is ill-conditioned on these grain
distributions: the oracle run from its own initial state perturbed by 1e-15 relative moves the
dust densities by ~5e-7 after five steps.  The last-bit differences of exp/log/pow between the
device and the host are of that size, so there the dust fields are held to the oracle's own
sensitivity (the oracle against itself from an input perturbed by 1e-14 relative), the gas fields
to 1e-10.

Config 2 in mixed precision: the wave's perturbation is 1e-4 of an O(1) background, and an FP32
state resolves rho ~ 1 only to 6e-8, i.e. 6e-4 of the perturbation.  After the 5,121 steps the
densities and the energy (whose L1 scale is the background) stay within 5e-5 (measured: gas
9e-8, energy 2.9e-6, dust up to 2.8e-5 for the least coupled species); the momenta, whose L1
scale is the perturbation itself, within 5e-3 (measured 2.2e-3 for the gas).  Against the linear
solution the gas modes and every velocity mode are within 1e-2 (measured 3.8e-3), the dust
density modes within 6e-2 (measured up to 4.4e-2): their amplitude is 2.5e-5 on a background of
0.25, and the FP32 state's rounding noise after 5,121 steps, ~sqrt(5121) ulp(0.25)/2 = 1e-6, is a
few per cent of it."""
import numpy as np
import pytest

from shark_gb300 import config as K, setups
from shark_gb300.solver import Shark
from oracle.oracle import Oracle
from tests import dusty_wave_linear as DW
from tests.test_gpu_parity import FP64_TOL, MIXED_TOL, active, rel_l1, run_pair

pytestmark = pytest.mark.gpu

GROWTH_DUST_TOL = 1e-2
GROWTH_GAS_TOL = 1e-4
ALLOWED = K.STATUS_NEWTON     # the disk's outer cells stall at psi0 in the reference's loop too


def _perturbed_oracle_spread(cfg, u0, nsteps, rel=1e-14, seed=0):
    """Relative L1 per field between two oracle runs, one from u0 and one from u0 perturbed by
    `rel` relative (the conditioning of the reference algorithm on this input)."""
    rng = np.random.default_rng(seed)
    runs = []
    for u in (u0, u0 * (1.0 + rel * rng.standard_normal(u0.size))):
        o = Oracle(cfg)
        o.set_u(u)
        for _ in range(nsteps):
            o.solve()
        runs.append(o.get_u())
    return rel_l1(cfg, runs[1], runs[0])


def _fp64_growth_parity(cfg, u0, nsteps):
    dto, dtg, uo, ug, st = run_pair(cfg, u0, nsteps)
    assert st & ~ALLOWED == 0
    np.testing.assert_allclose(dtg, dto, rtol=1e-12, atol=0)
    err = rel_l1(cfg, ug, uo)
    assert err[:5].max() <= FP64_TOL, err[:5]
    spread = _perturbed_oracle_spread(cfg, u0, nsteps)
    assert spread[5:].max() > FP64_TOL                       # the case is ill-conditioned
    assert err[5:].max() <= max(FP64_TOL, spread[5:].max()), (err[5:].max(), spread[5:].max())


def _dust_mass_ratio(cfg, ug, uo):
    N = cfg.ndust
    return active(cfg, ug)[5:5 + N].sum() / active(cfg, uo)[5:5 + N].sum()


@pytest.mark.parametrize("precision,tol,nsteps", [(K.PREC_FP64, FP64_TOL, 4), (K.PREC_MIXED, MIXED_TOL, 6)])
def test_si_1024_8_species(precision, tol, nsteps):
    cfg, u0 = setups.si(n=1024, ndust=8, precision=precision, noise=1e-3, seed=1)
    dto, dtg, uo, ug, st = run_pair(cfg, u0, nsteps)
    assert st == 0
    np.testing.assert_allclose(dtg, dto, rtol=1e-14 if precision == K.PREC_FP64 else 1e-5, atol=0)
    err = rel_l1(cfg, ug, uo)
    assert err.max() <= tol, err.max()


def test_polar_disk_16_species_fargo_growth_charging_fp64():
    cfg, u0 = setups.disk_polar_au(nr=128, nphi=256, ndust=16, growth=True)
    assert cfg.flags & K.FLAG_FARGO and cfg.flags & K.FLAG_CHARGING and cfg.flags & K.FLAG_GROWTH
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 6)
    assert st & ~ALLOWED == 0
    np.testing.assert_allclose(dtg, dto, rtol=1e-13, atol=0)
    assert rel_l1(cfg, ug, uo).max() <= FP64_TOL


def test_polar_disk_16_species_fargo_growth_charging_mixed():
    cfg, u0 = setups.disk_polar_au(nr=128, nphi=256, ndust=16, growth=True, precision=K.PREC_MIXED)
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 4)
    assert st & ~ALLOWED == 0
    np.testing.assert_allclose(dtg, dto, rtol=1e-4)
    err = rel_l1(cfg, ug, uo)
    assert err[:5].max() <= GROWTH_GAS_TOL, err[:5]
    assert err.max() <= GROWTH_DUST_TOL, err.max()
    assert abs(_dust_mass_ratio(cfg, ug, uo) - 1.0) <= 1e-5


def test_driven_box_32_species_forcing_growth_charging_fp64():
    cfg, u0 = setups.dusty_turb(n=128, ndust=32, forcing=True, charging=True, growth=True)
    _fp64_growth_parity(cfg, u0, 6)


def test_driven_box_32_species_forcing_charging_no_growth_fp64():
    """The same box without growth: every field within 1e-10."""
    cfg, u0 = setups.dusty_turb(n=128, ndust=32, forcing=True, charging=True)
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 6)
    assert st & ~ALLOWED == 0
    np.testing.assert_allclose(dtg, dto, rtol=1e-12, atol=0)
    assert rel_l1(cfg, ug, uo).max() <= FP64_TOL


@pytest.mark.parametrize("n", [1024, 1088])
def test_driven_box_32_species_mixed_flux_schedules(n):
    """The mixed K1 at the driven box's species count on the two schedules of its launch (for a
    GPU of 152 SMs): 1024^2 is one persistent wave of warps with the dust swept in two phases of
    128-row pieces; 1088^2 fills more than eight waves of 32-row pieces and runs one piece per
    warp.  Pieces of either schedule recompute their halo rows, so the result does not depend on
    the schedule and the mixed tolerance of the driven box holds against the oracle."""
    cfg, u0 = setups.dusty_turb(n=n, ndust=32, precision=K.PREC_MIXED)
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 3)
    assert st == 0
    np.testing.assert_allclose(dtg, dto, rtol=1e-5)
    err = rel_l1(cfg, ug, uo)
    assert err.max() <= 2e-4, err


def test_driven_box_32_species_forcing_growth_charging_mixed():
    cfg, u0 = setups.dusty_turb(n=128, ndust=32, forcing=True, charging=True, growth=True,
                                precision=K.PREC_MIXED)
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 4)
    assert st & ~ALLOWED == 0
    np.testing.assert_allclose(dtg, dto, rtol=1e-4)
    err = rel_l1(cfg, ug, uo)
    assert err[:5].max() <= 2e-4, err[:5]
    assert err.max() <= GROWTH_DUST_TOL, err.max()
    assert abs(_dust_mass_ratio(cfg, ug, uo) - 1.0) <= 1e-5


def test_driven_box_16_species_register_path_fp64():
    """16 species without growth: the largest compile-time species count of K2 (growth runs the
    run-time species path), with forcing and charging; every field within 1e-10."""
    cfg, u0 = setups.dusty_turb(n=96, ndust=16, forcing=True, charging=True)
    dto, dtg, uo, ug, st = run_pair(cfg, u0, 5)
    assert st & ~ALLOWED == 0
    np.testing.assert_allclose(dtg, dto, rtol=1e-12, atol=0)
    assert rel_l1(cfg, ug, uo).max() <= FP64_TOL


def test_driven_box_16_species_growth_fp64():
    cfg, u0 = setups.dusty_turb(n=96, ndust=16, forcing=True, charging=True, growth=True)
    _fp64_growth_parity(cfg, u0, 5)


# ---- config 2: the 4-species dusty wave to t = 2 ---------------------------------------------
DW_TEND = 2.0
DW_LINEAR_TOL = 1e-2         # the oracle's own distance to the linear solution: 6.4e-3 at 2048 cells
# mixed: the dust density modes carry the FP32 state's rounding noise, ~sqrt(5121) x ulp(0.25)/2
# = 1e-6 after the run, i.e. a few per cent of their 2.5e-5 amplitude (measured up to 4.4e-2)
DW_MIXED_DUST_DENSITY_LINEAR_TOL = 6e-2
DW_MIXED_MOMENTUM_TOL = 5e-3  # FP32 resolves the 1e-4 perturbation of rho ~ 1 to 6e-4 of itself
DW_MIXED_DENSITY_TOL = 5e-5   # 5,121 FP32 steps on the perturbed densities


def _dusty_wave_run(precision):
    cfg, u0 = setups.dustywave(nx=2048, ndust=4, precision=precision)
    o = Oracle(cfg)
    o.set_u(u0)
    n_o = o.run(10 ** 7, DW_TEND)
    with Shark(cfg) as g:
        g.upload(u0)
        n_g = g.time_loop(DW_TEND)
        ug, tg, st = g.download(), g.time, g.sync()
    g_ = cfg.nghost
    x = setups.positions(cfg)[g_:g_ + cfg.nx, 0]
    return cfg, (n_o, o.time, o.get_u()), (n_g, tg, ug, st), x


@pytest.mark.parametrize("precision", [K.PREC_FP64, K.PREC_MIXED])
def test_dusty_wave_4_species_to_t2(precision):
    cfg, (n_o, t_o, uo), (n_g, t_g, ug, st), x = _dusty_wave_run(precision)
    assert st == 0
    if precision == K.PREC_FP64:
        assert n_g == n_o and abs(t_g - t_o) <= 1e-13
        assert rel_l1(cfg, ug, uo).max() <= FP64_TOL
    else:
        # FP32 dt candidates may move the last step across t = 2 (one step changes the fields
        # by ~1e-7 of their L1 norm)
        assert abs(n_g - n_o) <= 1
        err = rel_l1(cfg, ug, uo)
        N = cfg.ndust
        mom = [1, 2, 3] + list(range(5 + N, 5 + 4 * N))
        dens = [v for v in range(cfg.nvar) if v not in mom]
        assert err[dens].max() <= DW_MIXED_DENSITY_TOL, err[dens]
        assert err[mom].max() <= DW_MIXED_MOMENTUM_TOL, err[mom]
    # mode damping and phase of every species against the linear solution at the time reached
    ua = active(cfg, ug)[:, 0, :]
    err = DW.mode_errors(cfg, ua, x, t_g)
    if precision == K.PREC_FP64:
        assert err.max() <= DW_LINEAR_TOL, err
    else:   # modes: gas density, gas velocity, N dust densities, N dust velocities
        N = cfg.ndust
        rd = list(range(2, 2 + N))
        rest = [i for i in range(err.size) if i not in rd]
        assert err[rest].max() <= DW_LINEAR_TOL, err
        assert err[rd].max() <= DW_MIXED_DUST_DENSITY_LINEAR_TOL, err
    ref = DW.mode_errors(cfg, active(cfg, uo)[:, 0, :], x, t_o)
    if precision == K.PREC_FP64:   # the FP64 run is as close to the linear solution as the oracle's
        assert err.max() <= ref.max() * (1.0 + 1e-6), (err.max(), ref.max())
