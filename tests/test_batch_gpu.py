"""Several H_eff plans in shared launches (su2g_heff_batch_*), through the C
ABI: every plan's product and every Lanczos solve of the lockstep batch must
equal the plan's own su2g_heff_apply / su2g_lanczos bit for bit (same tiles,
same kernels, same order per plan), in FP64 and split precision, for plans of
different sizes, with an excited-state projector on one of them, and for
subsets of a batch whose solves exit at different steps."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _plans(torch, mode, specs):
    from su2dmrg_gb300.su2 import HeffPlan
    from su2dmrg_gb300.workloads import synthetic_heff

    out = []
    for D, nspin1, seed in specs:
        w = synthetic_heff(D=D, nspin1=nspin1, seed=seed)
        psi, terms, hl, hr = w.to_device()
        out.append((HeffPlan(w.psi, terms, hl, hr, mode=mode), psi, (terms, hl, hr)))
    return out


SPECS = [(60, 3, 1), (120, 4, 2), (40, 2, 3), (200, 2, 4)]


@pytest.mark.parametrize("mode", [0, 1])
def test_batch_apply_equals_each_plan(su2lib, mode):
    import torch

    from su2dmrg_gb300.su2 import HeffBatch

    ps = _plans(torch, mode, SPECS)
    # an excited-state projector on one plan
    o = torch.randn_like(ps[1][1])
    o /= o.norm()
    ps[1][0].add_projector(o, 0.7)
    B = HeffBatch([p for p, _, _ in ps])
    off = B.offsets()
    x = torch.empty(B.total, dtype=torch.float64, device="cuda")
    for (p, psi, _), a in zip(ps, off):
        x[a: a + psi.numel()] = psi
    y = torch.full_like(x, np.nan)
    for _ in range(2):  # the batch's lists are reused on the second call
        B.apply(x, y)
        torch.cuda.synchronize()
        for (p, psi, _), a in zip(ps, off):
            want = torch.empty_like(psi)
            p.apply(psi, want)
            torch.cuda.synchronize()
            assert torch.equal(y[a: a + psi.numel()], want)
    B.status()


@pytest.mark.parametrize("mode", [0, 1])
def test_batch_lanczos_equals_solo(su2lib, mode):
    import torch

    from su2dmrg_gb300.su2 import HeffBatch

    ps = _plans(torch, mode, SPECS)
    starts = [psi.clone() for _, psi, _ in ps]
    # one start vector nearly converged, so that its solve leaves at the
    # eigenvector check of step 4 while the others take the final step
    for _ in range(12):
        ps[2][0].lanczos(starts[2], mlanc=5)
    solo = []
    for (p, _, _), s in zip(ps, starts):
        v = s.clone()
        e, nmv = p.lanczos(v, mlanc=5)
        solo.append((e, nmv, v))
    assert solo[2][1] == 5 and solo[0][1] == 7
    B = HeffBatch([p for p, _, _ in ps])
    for _ in range(2):
        vs = [s.clone() for s in starts]
        res = B.lanczos(vs, mlanc=5)
        torch.cuda.synchronize()
        for (e, nmv), v, (e0, nmv0, v0) in zip(res, vs, solo):
            assert e == e0 and nmv == nmv0
            assert torch.equal(v, v0)
    # a batch of one and a short Lanczos (mlanc 3)
    B1 = HeffBatch([ps[1][0]])
    v = starts[1].clone()
    (e, nmv), = B1.lanczos([v], mlanc=3)
    w = starts[1].clone()
    e0, nmv0 = ps[1][0].lanczos(w, mlanc=3)
    assert e == e0 and nmv == nmv0 and torch.equal(v, w)
