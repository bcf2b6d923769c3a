"""Synthetic workload shapes (no GPU)."""
import numpy as np

from su2dmrg_gb300.workloads import gaussian_sector_counts, synthetic_heff


def test_d2000_sector_counts():
    assert gaussian_sector_counts(2000) == [117, 173, 229, 270, 285, 270, 229, 173, 117, 71, 39, 19, 8]
    assert sum(gaussian_sector_counts(4000)) == 4000


def test_enlarged_legs_and_term_count(su2lib):
    w = synthetic_heff(D=2000, nspin1=2, spin0=True)
    enl = w.psi.bonds[0]
    assert enl.angm == list(range(14))
    assert enl.dim == [173, 346, 443, 514, 540, 514, 443, 346, 244, 156, 90, 47, 19, 8]
    assert sum(d * d for d in enl.dim) == w.psi_data.size == 1576457
    assert abs(np.linalg.norm(w.psi_data) - 1) < 1e-12
    assert len(w.terms) == 2


def test_synthetic_heff_is_symmetric(su2lib, oracle):
    """<z, H x> == <x, H z> for the construction used by the benchmarks."""
    w = synthetic_heff(D=60, nspin1=3, seed=7)
    prob = oracle.HeffProblem(w.psi, w.terms, w.hl, w.hr)
    rng = np.random.default_rng(0)
    x = rng.standard_normal(w.psi_data.size)
    z = rng.standard_normal(w.psi_data.size)
    a = z @ oracle.heff_apply(prob, x)
    b = x @ oracle.heff_apply(prob, z)
    assert abs(a - b) <= 1e-12 * abs(a)
