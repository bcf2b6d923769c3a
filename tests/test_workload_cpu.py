"""The benchmark's synthetic H_eff workload built two ways: by the library's
generator (su2dmrg_gb300.workloads, which the GPU arm uses) and by the oracle
alone (oracle.synthetic_heff, which the CPU reference arm uses so that it
loads nothing of the GPU library).  Both must hold the same structures and
the same numbers, bit for bit, or the two arms would time different work."""
import numpy as np
import pytest


@pytest.mark.parametrize("D,nspin1,seed", [(60, 3, 5), (300, 2, 1234), (2000, 1, 1234)])
def test_oracle_workload_equals_library_workload(su2lib, oracle, D, nspin1, seed):
    from su2dmrg_gb300.workloads import synthetic_heff

    w = synthetic_heff(D=D, nspin1=nspin1, seed=seed)
    prob, x = oracle.synthetic_heff(D=D, nspin1=nspin1, seed=seed)
    assert np.array_equal(prob.psi.desc(), w.psi.desc())
    assert np.array_equal(prob.psi.flag, w.psi.flag)
    assert np.array_equal(x, w.psi_data)
    assert len(prob.terms) == len(w.terms)
    for (a1, ax1, a2, ax2, ac), (b1, bx1, b2, bx2, bc) in zip(prob.terms, w.terms):
        assert np.array_equal(a1.desc(), b1.desc()) and np.array_equal(a1.flag, b1.flag)
        assert np.array_equal(a2.desc(), b2.desc()) and np.array_equal(a2.flag, b2.flag)
        assert np.array_equal(ax1, bx1) and np.array_equal(ax2, bx2) and ac == bc
    for a, b in ((prob.hl, w.hl), (prob.hr, w.hr)):
        assert np.array_equal(a[0].desc(), b[0].desc()) and np.array_equal(a[1], b[1])
