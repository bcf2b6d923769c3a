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


def test_block_fed_by_more_than_2_17_contracted_values_is_planned(su2lib):
    """Four products of K = 34000 into one 34000 x 34000 block (136,000
    contracted values per output element): two runs of products, each output
    tile computed as two partial tiles (64 KiB of scratch each) and summed."""
    import numpy as np

    from su2dmrg_gb300.su2 import HeffPlan, Su2Bond, Su2Struct

    K = 34000
    enl = Su2Bond(-1, [1], [K])
    psi = Su2Struct([enl, enl], 0).with_legal_flags()
    op = Su2Struct([enl.inverted(), Su2Bond(1, [2], [1]), enl], 0).with_legal_flags()
    dummy = np.zeros(1)  # validation reads structures only
    terms = [(op, dummy, op, dummy, 1.0)] * 4
    got = HeffPlan.validate(psi, terms, None, None, mode=1)
    assert got["flops"] == 4 * 2.0 * 2 * K * K * K  # both phases, four terms
    tiles = -(-K // 128) * -(-K // 64)
    assert got["scratch_bytes"] >= 2 * tiles * 128 * 64 * 8
