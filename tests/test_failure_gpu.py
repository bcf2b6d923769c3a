"""Failure detection without a GPU fault: the split GEMM's bounded mbarrier
wait, run on a barrier that nothing arrives at, gives up after its poll limit
and the host reads SU2G_ETIMEOUT; the context stays usable (an H_eff
application right after it matches the oracle).  The library's own plans
report such an event through su2g_heff_plan_status, and su2g_lanczos refuses
its result."""
import ctypes
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


@pytest.mark.parametrize("mode", [0, 1])
def test_lanczos_refuses_result_on_every_exit(su2lib, mode):
    """A Lanczos solve whose plan recorded a bounded wait that gave up
    returns SU2G_ETIMEOUT on each of its exits: the eigenvector check every
    four steps (lanczos_su2.cpp:178-188) and the final step (:189-194).  The
    error word is set from the host (su2g_heff_plan_mark_failed), so no device
    wait has to give up; an unmarked run from the same start vector shows
    which exit the solve takes (5 matvecs = the check at step 4 ends the
    solve; 7 = that check fails, then the final step and its check)."""
    import torch

    from su2dmrg_gb300 import capi
    from su2dmrg_gb300.su2 import HeffPlan
    from su2dmrg_gb300.workloads import synthetic_heff

    L = capi.lib()
    w = synthetic_heff(D=60, nspin1=3, seed=11)
    psi, t, hl, hr = w.to_device()
    plan = HeffPlan(w.psi, t, hl, hr, mode=mode)
    fresh = psi.clone()
    # restarted Lanczos until the start vector is converged enough for the
    # check at step 4 to end the solve
    conv = psi.clone()
    for _ in range(40):
        _, nmv = plan.lanczos(conv, mlanc=5)
        if nmv == 5:
            break
    assert nmv == 5
    for start, want_nmv in ((conv, 5), (fresh, 7)):
        v = start.clone()
        e, nmv = plan.lanczos(v, mlanc=5)
        assert nmv == want_nmv
        assert np.isfinite(e)
        v = start.clone()
        capi.check(L.su2g_heff_plan_mark_failed(plan.handle, 7))
        rc = L.su2g_lanczos(plan.handle, capi.ptr(v), 5, ctypes.addressof(ctypes.c_double()),
                            ctypes.addressof(ctypes.c_int()), None)
        assert rc == capi.SU2G_ETIMEOUT
        assert b"gave up" in L.su2g_last_error()
        # the status read cleared the word: the plan works again
        v = start.clone()
        e2, nmv2 = plan.lanczos(v, mlanc=5)
        assert nmv2 == want_nmv and e2 == e
    assert L.su2g_heff_plan_mark_failed(plan.handle, 0) == capi.SU2G_EINVAL
    torch.cuda.synchronize()
