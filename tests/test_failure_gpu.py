"""Failure detection without a GPU fault: the split GEMM's bounded mbarrier
wait, run on a barrier that nothing arrives at, gives up after its poll limit
and the host reads SU2G_ETIMEOUT; the context stays usable (an H_eff
application right after it matches the oracle).  The library's own plans
report such an event through su2g_heff_plan_status, and su2g_lanczos refuses
its result."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_context_survives(su2lib, oracle):
    import torch

    from su2dmrg_gb300 import capi
    from su2dmrg_gb300.su2 import HeffPlan
    from su2dmrg_gb300.workloads import synthetic_heff

    assert torch.cuda.is_available()
    L = capi.lib()
    t0 = time.perf_counter()
    rc = L.su2g_selftest_bounded_wait(1 << 10, None)
    assert rc == capi.SU2G_ETIMEOUT, rc
    assert time.perf_counter() - t0 < 10.0
    assert b"gave up" in L.su2g_last_error()
    assert L.su2g_selftest_bounded_wait(0, None) == capi.SU2G_EINVAL

    w = synthetic_heff(D=60, nspin1=3, seed=7)
    psi, t, hl, hr = w.to_device()
    plan = HeffPlan(w.psi, t, hl, hr, mode=1)
    y = torch.empty_like(psi)
    plan.apply(psi, y)
    assert plan.status() == 0
    want = oracle.heff_apply(oracle.HeffProblem(w.psi, w.terms, w.hl, w.hr), w.psi_data)
    assert np.linalg.norm(y.cpu().numpy() - want) <= 1e-12 * np.linalg.norm(want)  # split mode's bound
