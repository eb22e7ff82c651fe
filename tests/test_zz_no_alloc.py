"""shark_gpu_totals_noalloc, the entry point for callers that cannot allocate device memory (their
own allocator owns every device allocation, or their time loop cannot take cudaMalloc's implicit
synchronisation): it must return the same totals as shark_gpu_totals for the same state, on
consecutive calls that share its fixed scratch array.  Covered: a 2D box of 4 stage-1 blocks,
the 1024^2 box (more active cells than 256 blocks x 1024, so the block count is capped), a 1D
state (ny = 1) and the largest species count (64).  Collected last on purpose."""
import numpy as np
import pytest

from shark_gb300 import setups
from shark_gb300.solver import Shark, totals_noalloc

pytestmark = pytest.mark.gpu

TOL = 1e-12   # the totals tolerance of the other GPU tests


def _check_two_calls(cfg, u0, steps_between=2):
    torch = pytest.importorskip("torch")
    nq = 4 * (cfg.ndust + 1)
    out = torch.zeros(nq, dtype=torch.float64, device="cuda")
    with Shark(cfg) as g:
        g.upload(u0)
        for call in range(2):
            for _ in range(steps_between):
                g.solve()
            ref = g.totals().reshape(-1)
            u = torch.from_numpy(g.download()).to("cuda")
            out.fill_(float("nan"))
            torch.cuda.synchronize()
            totals_noalloc(u.data_ptr(), cfg.nx, cfg.ny, cfg.nghost, cfg.ndust, out.data_ptr(), None)
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            np.testing.assert_allclose(got, ref, rtol=TOL, atol=1e-18, err_msg=f"call {call}")


def test_totals_noalloc_matches_context_totals_on_two_calls():
    cfg, u0 = setups.si(n=64, ndust=4)
    _check_two_calls(cfg, u0)


def test_totals_noalloc_capped_block_count_1024():
    cfg, u0 = setups.si(n=1024, ndust=8, noise=1e-3, seed=1)
    assert cfg.nx * cfg.ny > 256 * 1024
    _check_two_calls(cfg, u0, steps_between=1)


def test_totals_noalloc_one_dimensional_state():
    cfg, u0 = setups.dustywave(nx=2048, ndust=4)
    assert cfg.ny == 1
    _check_two_calls(cfg, u0)


def test_totals_noalloc_64_species():
    cfg, u0 = setups.dusty_turb(n=24, ndust=64)
    _check_two_calls(cfg, u0, steps_between=1)


def test_totals_noalloc_leaves_device_memory_unchanged_after_warm_up():
    torch = pytest.importorskip("torch")
    cfg, u0 = setups.si(n=128, ndust=4)
    u = torch.from_numpy(u0).to("cuda")
    out = torch.zeros(4 * (cfg.ndust + 1), dtype=torch.float64, device="cuda")
    totals_noalloc(u.data_ptr(), cfg.nx, cfg.ny, cfg.nghost, cfg.ndust, out.data_ptr(), None)   # warm-up
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        totals_noalloc(u.data_ptr(), cfg.nx, cfg.ny, cfg.nghost, cfg.ndust, out.data_ptr(), None)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_totals_noalloc_rejects_too_many_species():
    torch = pytest.importorskip("torch")
    from shark_gb300.solver import SharkError
    u = torch.zeros(16, dtype=torch.float64, device="cuda")
    with pytest.raises(SharkError):
        totals_noalloc(u.data_ptr(), 4, 1, 2, 65, u.data_ptr(), None)
