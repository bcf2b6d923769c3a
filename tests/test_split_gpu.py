"""Split-precision (BF16 digit slices on tcgen05) H_eff parity.

Tolerances (relative Frobenius error of y = H_eff psi against the FP64
oracle): 7 slices 1e-12, 6 slices 1e-10.  Lanczos energies in the 7-slice
mode agree with the FP64 oracle to 1e-10 relative."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {1: 1e-12, 2: 1e-10}


@pytest.fixture(scope="module")
def torch_cuda(su2lib):
    import torch

    assert torch.cuda.is_available()
    return torch


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("D,nspin1,spin0", [(40, 1, False), (60, 4, True), (300, 3, True), (777, 2, True)])
def test_split_matches_oracle(torch_cuda, oracle, mode, D, nspin1, spin0):
    from su2dmrg_gb300.su2 import HeffPlan
    from su2dmrg_gb300.workloads import synthetic_heff

    torch = torch_cuda
    w = synthetic_heff(D=D, nspin1=nspin1, seed=D + 11, spin0=spin0)
    psi, terms, hl, hr = w.to_device()
    plan = HeffPlan(w.psi, terms, hl, hr, mode=mode)
    y = torch.empty_like(psi)
    plan.apply(psi, y)
    torch.cuda.synchronize()
    assert plan.status() == 0
    prob = oracle.HeffProblem(w.psi, w.terms, w.hl, w.hr)
    ref = oracle.heff_apply(prob, w.psi_data)
    assert _rel(y.cpu().numpy(), ref) <= TOL[mode]


def test_split_block_fed_by_many_products(torch_cuda, oracle):
    """1100 terms, each feeding every output block: more products than one
    tile's exact combination holds, so each block is summed from partial
    tiles in a fixed order; same tolerance as any 7-slice result."""
    from su2dmrg_gb300.su2 import HeffPlan
    from su2dmrg_gb300.workloads import synthetic_heff

    torch = torch_cuda
    w = synthetic_heff(D=8, nspin1=1100, seed=3, max2j=2)
    psi, terms, hl, hr = w.to_device()
    plan = HeffPlan(w.psi, terms, hl, hr, mode=1)
    y = torch.empty_like(psi)
    plan.apply(psi, y)
    torch.cuda.synchronize()
    assert plan.status() == 0
    ref = oracle.heff_apply(oracle.HeffProblem(w.psi, w.terms, w.hl, w.hr), w.psi_data)
    assert _rel(y.cpu().numpy(), ref) <= TOL[1]
    y2 = torch.empty_like(psi)
    plan.apply(psi, y2)
    torch.cuda.synchronize()
    assert torch.equal(y, y2)


def test_split_scaled_terms_and_zero_blocks(torch_cuda, oracle):
    """Coefficients folded into the operator slices, an all-zero psi block and
    an operator with no stored block."""
    from su2dmrg_gb300.su2 import HeffPlan
    from su2dmrg_gb300.workloads import synthetic_heff

    torch = torch_cuda
    w = synthetic_heff(D=150, nspin1=3, seed=9)
    s1, x1, s2, x2, _ = w.terms[2]
    empty = type(s1)(s1.bonds, s1.locspin, np.zeros_like(s1.flag))
    w.terms = [w.terms[0][:4] + (0.3,), w.terms[1][:4] + (-2.5,), (empty, np.zeros(0), s2, x2, 1.0)]
    w.hl = (w.hl[0], w.hl[1], -0.5)
    off, _ = w.psi.offsets()
    k = int(np.flatnonzero(w.psi.flag)[3])
    a, b = w.psi.block_shape(k)
    w.psi_data[off[k]: off[k] + a * b] = 0.0
    psi, terms, hl, hr = w.to_device()
    plan = HeffPlan(w.psi, terms, hl, hr, mode=1)
    y = torch.empty_like(psi)
    plan.apply(psi, y)
    torch.cuda.synchronize()
    assert plan.status() == 0
    ref = oracle.heff_apply(oracle.HeffProblem(w.psi, w.terms, w.hl, w.hr), w.psi_data)
    assert _rel(y.cpu().numpy(), ref) <= TOL[1]


def test_split_d2000_against_fp64_path(torch_cuda):
    """Full benchmark shape: the 7-slice result against the FP64 GPU path
    (itself held to 1e-12 of the oracle), plus determinism."""
    from su2dmrg_gb300.su2 import HeffPlan
    from su2dmrg_gb300.workloads import synthetic_heff

    torch = torch_cuda
    w = synthetic_heff(D=2000, nspin1=18, seed=1234)
    psi, terms, hl, hr = w.to_device()
    p64 = HeffPlan(w.psi, terms, hl, hr, mode=0)
    psp = HeffPlan(w.psi, terms, hl, hr, mode=1)
    y64, ysp, ysp2 = (torch.empty_like(psi) for _ in range(3))
    p64.apply(psi, y64)
    psp.apply(psi, ysp)
    psp.apply(psi, ysp2)
    torch.cuda.synchronize()
    assert psp.status() == 0
    assert torch.equal(ysp, ysp2)
    rel = float((ysp - y64).norm() / y64.norm())
    assert rel <= TOL[1], rel


@pytest.mark.parametrize("D,nspin1", [(60, 4), (200, 6)])
def test_split_lanczos_energy(torch_cuda, oracle, D, nspin1):
    from su2dmrg_gb300.su2 import HeffPlan
    from su2dmrg_gb300.workloads import synthetic_heff

    torch = torch_cuda
    w = synthetic_heff(D=D, nspin1=nspin1, seed=D + 5)
    psi, terms, hl, hr = w.to_device()
    plan = HeffPlan(w.psi, terms, hl, hr, mode=1)
    e, nmv = plan.lanczos(psi, mlanc=5)
    assert plan.status() == 0
    prob = oracle.HeffProblem(w.psi, w.terms, w.hl, w.hr)
    e_or, _, nmv_or = oracle.lanczos1(lambda v: oracle.heff_apply(prob, v), w.psi_data.copy(), 5)
    assert abs(e - e_or) <= 1e-10 * abs(e_or)
    assert nmv == nmv_or
