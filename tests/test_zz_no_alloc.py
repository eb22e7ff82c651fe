"""shark_gpu_totals_noalloc, the entry point for callers that cannot allocate device memory (their
own allocator owns every device allocation, or their time loop cannot take cudaMalloc's implicit
synchronisation): it must return the same totals as shark_gpu_totals for the same state, on
consecutive calls that share its fixed scratch array.  Collected last on purpose."""
import numpy as np
import pytest

from shark_gb300 import setups
from shark_gb300.solver import Shark, totals_noalloc

pytestmark = pytest.mark.gpu

TOL = 1e-12   # the totals tolerance of the other GPU tests


def test_totals_noalloc_matches_context_totals_on_two_calls():
    torch = pytest.importorskip("torch")
    cfg, u0 = setups.si(n=64, ndust=4)
    nq = 4 * (cfg.ndust + 1)
    out = torch.zeros(nq, dtype=torch.float64, device="cuda")
    with Shark(cfg) as g:
        g.upload(u0)
        for call in range(2):
            g.solve()
            g.solve()
            ref = g.totals().reshape(-1)
            u = torch.from_numpy(g.download()).to("cuda")
            out.fill_(float("nan"))
            torch.cuda.synchronize()
            totals_noalloc(u.data_ptr(), cfg.nx, cfg.ny, cfg.nghost, cfg.ndust, out.data_ptr(), None)
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            np.testing.assert_allclose(got, ref, rtol=TOL, atol=1e-18, err_msg=f"call {call}")


def test_totals_noalloc_rejects_too_many_species():
    torch = pytest.importorskip("torch")
    from shark_gb300.solver import SharkError
    u = torch.zeros(16, dtype=torch.float64, device="cuda")
    with pytest.raises(SharkError):
        totals_noalloc(u.data_ptr(), 4, 1, 2, 65, u.data_ptr(), None)
