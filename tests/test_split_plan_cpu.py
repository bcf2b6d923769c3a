"""Host side of the split-precision planner: an output block fed by more
products (or contracted values) than one tile's exact group combination holds
is planned as partial tiles summed in a fixed order, and its work lists pass
the host-side bounds check of every access (su2g_heff_plan_validate)."""


def test_block_fed_by_more_than_1024_products_is_planned(su2lib):
    from su2dmrg_gb300.su2 import HeffPlan
    from su2dmrg_gb300.workloads import synthetic_heff

    # every one of the 1100 terms feeds every output block: 1100 products per block
    w = synthetic_heff(D=8, nspin1=1100, seed=3, max2j=2)
    f64 = HeffPlan.validate(w.psi, w.terms, w.hl, w.hr, mode=0)
    for mode in (1, 2):
        got = HeffPlan.validate(w.psi, w.terms, w.hl, w.hr, mode=mode)
        assert got["flops"] == f64["flops"]
        assert got["scratch_bytes"] > f64["scratch_bytes"]
