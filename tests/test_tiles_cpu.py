"""Host side of the FP64 engine's tile classes: the table is checked when it
is installed, and work lists built under any table pass the host-side bounds
check of every access (su2g_heff_plan_validate) with the same FLOP count."""
import pytest


def test_tile_table_rejects_bad_tables(su2lib):
    from su2dmrg_gb300 import autotune as A

    with pytest.raises(Exception):
        A.install({"m_edges": [32, 16], "n_edges": [], "cls": [0, 0, 0]})  # edges must increase
    with pytest.raises(Exception):
        A.install({"m_edges": [], "n_edges": [], "cls": [4]})  # classes 0..3
    with pytest.raises(ValueError):
        A.install({"m_edges": [16], "n_edges": [], "cls": [0]})  # 2 x 1 buckets need 2 classes
    A.load()


@pytest.mark.parametrize("cls", [0, 1, 2, 3])
def test_tiled_work_lists_validate(su2lib, cls):
    from su2dmrg_gb300 import autotune as A
    from su2dmrg_gb300.su2 import HeffPlan
    from su2dmrg_gb300.workloads import synthetic_heff

    w = synthetic_heff(D=300, nspin1=2, seed=9)
    A.reset()
    ref = HeffPlan.validate(w.psi, w.terms, w.hl, w.hr, mode=0)
    A.install({"m_edges": [20, 40], "n_edges": [30], "cls": [cls, 3 - cls, 0, cls, 1, 2]})
    got = HeffPlan.validate(w.psi, w.terms, w.hl, w.hr, mode=0)
    A.load()
    assert got["flops"] == ref["flops"]
