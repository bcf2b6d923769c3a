"""Host planning over many seeded random shapes (no GPU): for H_eff plans and
environment batches, the FP64 work lists (blocks, products and tiles) and the
split work lists (blocks, products, pack jobs, 128x64 tiles, partial sums)
both pass the host-side check of every access, and count the same FLOPs."""
import numpy as np
import pytest


@pytest.mark.parametrize("seed", range(12))
def test_heff_plans_validate_in_both_modes(su2lib, seed):
    from su2dmrg_gb300.su2 import HeffPlan
    from su2dmrg_gb300.workloads import synthetic_heff

    rng = np.random.default_rng(seed)
    D = int(rng.integers(8, 160))
    w = synthetic_heff(D=D, nspin1=int(rng.integers(0, 5)), seed=seed, max2j=int(rng.integers(1, 9)),
                       spin0=bool(rng.integers(0, 2)))
    f64 = HeffPlan.validate(w.psi, w.terms, w.hl, w.hr, mode=0)
    for mode in (1, 2):
        got = HeffPlan.validate(w.psi, w.terms, w.hl, w.hr, mode=mode)
        assert got["flops"] == f64["flops"]
        assert got["scratch_bytes"] >= f64["scratch_bytes"]


@pytest.mark.parametrize("seed", range(8))
def test_env_batches_validate_in_both_modes(su2lib, seed):
    from su2dmrg_gb300 import su2 as S
    from su2dmrg_gb300.workloads import synthetic_site_step

    rng = np.random.default_rng(100 + seed)
    w = synthetic_site_step(D=int(rng.integers(8, 160)), nops=int(rng.integers(1, 6)), seed=seed,
                            max2j=int(rng.integers(1, 9)))
    su, du = w.uu
    jobs = [{"kind": "transform", "slot": i, "coef": float(rng.normal()), "x": op} for i, op in enumerate(w.ops)]
    jobs.append({"kind": "overlap", "slot": len(w.ops), "coef": 1.0, "x": w.hh})
    f64 = S.env_validate(su, du, su, du, 0, jobs, mode=0)
    got = S.env_validate(su, du, su, du, 0, jobs, mode=1)
    assert got["flops"] == f64["flops"] and got["scratch_bytes"] >= f64["scratch_bytes"]
