"""GPU parity of the block-sparse H_eff engine through the C ABI.

Bar: <= 1e-12 relative (Frobenius) against the reference's own outputs
(tests/golden) and against the oracle at sizes it finishes in seconds; at the
full D=2000 shape, size-independent properties (linearity, symmetry,
determinism) plus a block-subset comparison with the oracle."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture(scope="module")
def torch_cuda(su2lib):
    import torch

    assert torch.cuda.is_available()
    return torch


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float64)).cuda()


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "heff_term_*.npz"))))
def test_one_shot_term_matches_reference(torch_cuda, oracle, path):
    """su2g_hamiltonian_vector_multiplication vs the reference's
    tensor_su2::hamiltonian_vector_multiplication on the same inputs."""
    from su2dmrg_gb300.su2 import hamiltonian_vector_multiplication

    torch = torch_cuda
    g = np.load(path)
    vs = oracle.struct_from_desc(g["vdesc"], g["vflag"])
    s1 = oracle.struct_from_desc(g["d1"], g["f1"])
    s2 = oracle.struct_from_desc(g["d2"], g["f2"])
    y = torch.zeros(g["vx"].size, dtype=torch.float64, device="cuda")
    hamiltonian_vector_multiplication(vs, _dev(torch, g["vx"]), s1, _dev(torch, g["x1"]), s2, _dev(torch, g["x2"]), y)
    torch.cuda.synchronize()
    rs = oracle.struct_from_desc(g["vdesc"], g["rflag"])
    ref = oracle.to_layout(rs, g["rx"], vs)
    assert _rel(y.cpu().numpy(), ref) <= TOL


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "spin0_*.npz"))))
def test_spin0_plan_matches_reference(torch_cuda, oracle, path):
    from su2dmrg_gb300.su2 import HeffPlan

    torch = torch_cuda
    g = np.load(path)
    vs = oracle.struct_from_desc(g["vdesc"], g["vflag"])
    hs = oracle.struct_from_desc(g["hdesc"], g["hflag"])
    hx = _dev(torch, g["hx"])
    side = int(g["side"])
    plan = HeffPlan(vs, [], hl=(hs, hx, 1.0) if side == 0 else None, hr=(hs, hx, 1.0) if side == 1 else None)
    y = torch.zeros(g["vx"].size, dtype=torch.float64, device="cuda")
    plan.apply(_dev(torch, g["vx"]), y)
    torch.cuda.synchronize()
    rs = oracle.struct_from_desc(g["vdesc"], g["rflag"])
    ref = oracle.to_layout(rs, g["rx"], vs)
    assert _rel(y.cpu().numpy(), ref) <= TOL


def _plan_and_oracle(torch, oracle, w):
    from su2dmrg_gb300.su2 import HeffPlan

    psi, terms, hl, hr = w.to_device()
    plan = HeffPlan(w.psi, terms, hl, hr)
    prob = oracle.HeffProblem(w.psi, w.terms, w.hl, w.hr)
    return plan, prob, psi


@pytest.mark.parametrize("D,nspin1,spin0", [(40, 1, False), (60, 4, True), (150, 6, True), (333, 3, True)])
def test_full_plan_matches_oracle(torch_cuda, oracle, D, nspin1, spin0):
    from su2dmrg_gb300.workloads import synthetic_heff

    torch = torch_cuda
    w = synthetic_heff(D=D, nspin1=nspin1, seed=D, spin0=spin0)
    plan, prob, psi = _plan_and_oracle(torch, oracle, w)
    y = torch.empty_like(psi)
    plan.apply(psi, y)
    torch.cuda.synchronize()
    ref = oracle.heff_apply(prob, w.psi_data)
    assert _rel(y.cpu().numpy(), ref) <= TOL
    # flops bookkeeping agrees with the oracle's count
    assert abs(plan.info()["flops"] - oracle.heff_flops(prob)) <= 1e-9 * oracle.heff_flops(prob)


def test_term_coefficients_and_missing_blocks(torch_cuda, oracle):
    """Coefficients scale terms; operators with dropped blocks; an operator
    with no stored block contributes nothing."""
    from su2dmrg_gb300.workloads import synthetic_heff

    torch = torch_cuda
    w = synthetic_heff(D=90, nspin1=3, seed=3)
    rng = np.random.default_rng(5)
    terms = []
    for n, (s1, x1, s2, x2, _c) in enumerate(w.terms):
        s1 = type(s1)(s1.bonds, s1.locspin, s1.flag.copy())
        s2 = type(s2)(s2.bonds, s2.locspin, s2.flag.copy())
        o1, _ = s1.offsets()
        drop = (rng.random(s1.nten) < 0.3) if n < 2 else np.ones(s1.nten, bool)
        keep = s1.flag.astype(bool) & ~drop
        new1 = type(s1)(s1.bonds, s1.locspin, keep.astype(np.int32))
        x1n = oracle.to_layout(s1, x1, new1)
        terms.append((new1, x1n, s2, x2, [0.5, -1.25, 3.0][n]))
    w.terms = terms
    w.hl = (w.hl[0], w.hl[1], 0.75)
    w.hr = (w.hr[0], w.hr[1], -2.0)
    plan, prob, psi = _plan_and_oracle(torch, oracle, w)
    y = torch.empty_like(psi)
    plan.apply(psi, y)
    torch.cuda.synchronize()
    ref = oracle.heff_apply(prob, w.psi_data)
    assert _rel(y.cpu().numpy(), ref) <= TOL


@pytest.mark.parametrize("mode", [0, 1])
def test_empty_plan_writes_zeros(torch_cuda, oracle, mode):
    """Output blocks no product reaches are written as zeros (FP64 tiles and
    split tiles without segments alike)."""
    from su2dmrg_gb300.su2 import HeffPlan
    from su2dmrg_gb300.workloads import synthetic_heff

    torch = torch_cuda
    w = synthetic_heff(D=30, nspin1=0, seed=1, spin0=False)
    plan = HeffPlan(w.psi, [], mode=mode)
    psi = _dev(torch, w.psi_data)
    y = torch.full_like(psi, 7.0)
    plan.apply(psi, y)
    torch.cuda.synchronize()
    assert float(y.abs().max()) == 0.0


def test_aliasing_rejected(torch_cuda):
    from su2dmrg_gb300 import capi
    from su2dmrg_gb300.su2 import HeffPlan
    from su2dmrg_gb300.workloads import synthetic_heff

    torch = torch_cuda
    w = synthetic_heff(D=30, nspin1=1, seed=1)
    psi, terms, hl, hr = w.to_device()
    plan = HeffPlan(w.psi, terms, hl, hr)
    with pytest.raises(capi.Su2gError) as ei:
        plan.apply(psi, psi)
    assert ei.value.code == capi.SU2G_EINVAL


@pytest.fixture(scope="module")
def d2000(torch_cuda):
    from su2dmrg_gb300.su2 import HeffPlan
    from su2dmrg_gb300.workloads import synthetic_heff

    w = synthetic_heff(D=2000, nspin1=18, seed=1234)
    psi, terms, hl, hr = w.to_device()
    plan = HeffPlan(w.psi, terms, hl, hr)
    return w, plan, psi, (terms, hl, hr)


def test_d2000_linearity_symmetry_determinism(torch_cuda, d2000):
    torch = torch_cuda
    w, plan, psi, _keep = d2000
    n = psi.numel()
    g = torch.Generator(device="cuda").manual_seed(11)
    x = torch.randn(n, dtype=torch.float64, device="cuda", generator=g)
    z = torch.randn(n, dtype=torch.float64, device="cuda", generator=g)
    hx, hz, hxz, hx2 = (torch.empty_like(x) for _ in range(4))
    plan.apply(x, hx)
    plan.apply(z, hz)
    plan.apply(2.0 * x - 3.0 * z, hxz)
    plan.apply(x, hx2)
    torch.cuda.synchronize()
    assert torch.equal(hx, hx2)  # deterministic, bit for bit
    lin = (hxz - (2.0 * hx - 3.0 * hz)).norm() / hxz.norm()
    assert float(lin) <= TOL
    a = float(torch.dot(z, hx))
    b = float(torch.dot(x, hz))
    assert abs(a - b) <= 1e-11 * abs(a)


def test_d2000_matches_oracle_on_reduced_width(torch_cuda, oracle):
    """Full D=2000 block shapes (blocks up to 540x540) with two spin-1 terms
    and the spin-0 terms, compared element-wise with the oracle."""
    from su2dmrg_gb300.workloads import synthetic_heff

    torch = torch_cuda
    w = synthetic_heff(D=2000, nspin1=2, seed=77)
    plan, prob, psi = _plan_and_oracle(torch, oracle, w)
    y = torch.empty_like(psi)
    plan.apply(psi, y)
    torch.cuda.synchronize()
    oracle.set_blas_threads(os.cpu_count() or 1)
    ref = oracle.heff_apply(prob, w.psi_data)
    assert _rel(y.cpu().numpy(), ref) <= TOL


@pytest.mark.parametrize("D,nspin1", [(50, 3), (120, 5)])
def test_lanczos_matches_oracle(torch_cuda, oracle, D, nspin1):
    """su2g_lanczos vs the restated lanczos_su2::lanczos1 on the same H_eff
    and start vector: same eigenvalue (1e-10 relative), same number of
    matvecs, same ground state up to sign."""
    from su2dmrg_gb300.workloads import synthetic_heff

    torch = torch_cuda
    w = synthetic_heff(D=D, nspin1=nspin1, seed=D + 1)
    plan, prob, psi = _plan_and_oracle(torch, oracle, w)
    e_gpu, nmv = plan.lanczos(psi, mlanc=5)
    torch.cuda.synchronize()
    e_or, v_or, nmv_or = oracle.lanczos1(lambda v: oracle.heff_apply(prob, v), w.psi_data.copy(), 5)
    assert abs(e_gpu - e_or) <= 1e-10 * abs(e_or)
    assert nmv == nmv_or
    v = psi.cpu().numpy()
    assert abs(abs(v @ v_or) / (np.linalg.norm(v) * np.linalg.norm(v_or)) - 1) < 1e-10
