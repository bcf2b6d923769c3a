"""Tile classes of the FP64 engine (the block-size autotuner's choices): a
work list tiled 64x64, 64x32, 32x64 or 32x32 must give the same result bit
for bit (every output element sums its products in the same order whatever
the tile shape), for H_eff applications and environment updates; the
autotuner's measurement entry point runs every class."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture
def tables(su2lib):
    from su2dmrg_gb300 import autotune as A

    yield A
    A.load()


@pytest.mark.parametrize("cls", [1, 2, 3])
def test_heff_tile_classes_bit_identical(tables, oracle, cls):
    import torch

    from su2dmrg_gb300.su2 import HeffPlan
    from su2dmrg_gb300.workloads import synthetic_heff

    A = tables
    w = synthetic_heff(D=150, nspin1=3, seed=5)
    psi, terms, hl, hr = w.to_device()
    A.reset()
    p0 = HeffPlan(w.psi, terms, hl, hr, mode=0)
    y0 = torch.empty_like(psi)
    p0.apply(psi, y0)
    # every block in class cls, then a mixed table
    A.install({"m_edges": [], "n_edges": [], "cls": [cls]})
    p1 = HeffPlan(w.psi, terms, hl, hr, mode=0)
    y1 = torch.empty_like(psi)
    p1.apply(psi, y1)
    A.install({"m_edges": [24, 48], "n_edges": [32], "cls": [3, 2, 1, 3, 0, cls]})
    p2 = HeffPlan(w.psi, terms, hl, hr, mode=0)
    y2 = torch.empty_like(psi)
    p2.apply(psi, y2)
    torch.cuda.synchronize()
    assert torch.equal(y0, y1) and torch.equal(y0, y2)
    ref = oracle.heff_apply(oracle.HeffProblem(w.psi, w.terms, w.hl, w.hr), w.psi_data)
    assert np.linalg.norm(y1.cpu().numpy() - ref) <= 1e-12 * np.linalg.norm(ref)


def test_env_tile_classes_bit_identical(tables):
    import torch

    from su2dmrg_gb300 import su2 as S
    from su2dmrg_gb300.workloads import synthetic_site_step

    A = tables
    w = synthetic_site_step(D=120, nops=3)
    su, xu = w.uu
    du = torch.from_numpy(xu).cuda()
    jobs = [{"kind": "transform", "slot": i, "coef": 1.0, "x": (s_, torch.from_numpy(x_).cuda())}
            for i, (s_, x_) in enumerate(w.ops)]
    outs = []
    for table in (None, {"m_edges": [], "n_edges": [], "cls": [3]}):
        if table is None:
            A.reset()
        else:
            A.install(table)
        res = S.env_batch(su, du, su, du, 0, jobs, mode=0)
        torch.cuda.synchronize()
        outs.append([y.clone() for _, y in res])
    for a, b in zip(*outs):
        assert torch.equal(a, b)


def test_tile_bench_runs_every_class(tables):
    A = tables
    for c in range(4):
        assert A.bench_class(40, 24, 64, c, reps=2) > 0
