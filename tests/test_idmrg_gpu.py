"""GPU parity of a whole two-site H_eff as the engine assembles it
(hamiltonian_vector_multiplication_idmrg, dmrg_su2.cpp:543-664), on the
environments of real runs (tests/golden/idmrg_*.npz: J1-J2 and J-Q with
plaquette terms): partner operators combined on the device once
(su2g_operator_combine), one plan, one application against the engine's own
output (1e-12 relative, FP64 and 7-slice split); Lanczos from the engine's
converged vector reproduces its Rayleigh quotient (1e-10 relative); the
excited-state projector term matches y - w (o.psi) o."""
import glob
import os

import numpy as np
import pytest

import idmrg_case
from conftest import GOLDEN

pytestmark = pytest.mark.gpu
PATHS = sorted(glob.glob(os.path.join(GOLDEN, "idmrg_*.npz")))


@pytest.fixture(scope="module")
def torch_cuda(su2lib):
    import torch

    assert torch.cuda.is_available()
    return torch


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float64)).cuda()


def _plan(oracle, torch, g, mode):
    from su2dmrg_gb300.su2 import HeffPlan, operator_combine

    vs, vx, yref, _, T, terms, hl, hr = idmrg_case.load(oracle, g)
    dev = {i: (t[0], _dev(torch, t[1])) for i, t in T.items() if t is not None}
    keep = []

    def side(lst):
        if len(lst) == 1 and lst[0][1] == 1.0:
            return dev[lst[0][0]]
        r = operator_combine([dev[i] for i, _ in lst], [c for _, c in lst])
        keep.append(r)
        return r

    tl = []
    for coef, left, right in terms:
        L, R = side(left), side(right)
        tl.append((L[0], L[1], R[0], R[1], coef))
    hlt = (dev[2][0], dev[2][1], 1.0) if hl is not None else None
    hrt = (dev[3][0], dev[3][1], 1.0) if hr is not None else None
    plan = HeffPlan(vs, tl, hlt, hrt, mode=mode)
    plan._keep = keep
    return plan, vs, vx, yref


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("path", PATHS)
def test_idmrg_heff_matches_reference(oracle, torch_cuda, path, mode):
    g = np.load(path)
    plan, vs, vx, yref = _plan(oracle, torch_cuda, g, mode)
    psi = _dev(torch_cuda, vx)
    y = torch_cuda.zeros_like(psi)
    plan.apply(psi, y)
    torch_cuda.cuda.synchronize()
    assert plan.status() == 0
    assert np.linalg.norm(y.cpu().numpy() - yref) <= 1e-12 * np.linalg.norm(yref)


@pytest.mark.parametrize("path", PATHS)
def test_idmrg_lanczos_energy(oracle, torch_cuda, path):
    """From the engine's vector (converged only to its own Lanczos tolerance)
    the device Lanczos gives the energy of the oracle's lanczos1 on the
    oracle's H_eff to 1e-10 relative, at or below the vector's Rayleigh
    quotient."""
    g = np.load(path)
    plan, vs, vx, yref = _plan(oracle, torch_cuda, g, 0)
    e_rq = float(np.dot(vx, yref) / np.dot(vx, vx))
    _, _, _, _, T, terms, hl, hr = idmrg_case.load(oracle, g)
    tl = []
    for coef, left, right in terms:
        L, R = idmrg_case.combine_host(oracle, T, left), idmrg_case.combine_host(oracle, T, right)
        tl.append((L[0], L[1], R[0], R[1], coef))
    prob = oracle.HeffProblem(vs, tl, hl, hr)
    e_or, _, _ = oracle.lanczos1(lambda v: oracle.heff_apply(prob, v), vx.copy(), 5)
    psi = _dev(torch_cuda, vx)
    e, nmv = plan.lanczos(psi, mlanc=5)
    assert nmv >= 1
    assert abs(e - e_or) <= 1e-10 * abs(e_or)
    assert e <= e_rq + 1e-10 * abs(e_rq)


@pytest.mark.parametrize("path", PATHS[:1])
def test_idmrg_projector(oracle, torch_cuda, path):
    g = np.load(path)
    plan, vs, vx, yref = _plan(oracle, torch_cuda, g, 0)
    rng = np.random.default_rng(5)
    o = rng.standard_normal(vx.size)
    o /= np.linalg.norm(o)
    w = -3.25
    od = _dev(torch_cuda, o)
    plan.add_projector(od, w)
    psi = _dev(torch_cuda, vx)
    y = torch_cuda.zeros_like(psi)
    plan.apply(psi, y)
    want = yref - w * np.dot(o, vx) * o
    assert np.linalg.norm(y.cpu().numpy() - want) <= 1e-12 * np.linalg.norm(want)


@pytest.mark.parametrize("path", PATHS[:1])
def test_lanczos_graph_replay_and_projector(oracle, torch_cuda, path):
    """su2g_lanczos runs each Lanczos step as a captured CUDA graph: a second
    solve on the same plan replays the graphs and is bit-identical; a
    projector added afterwards invalidates them, and the new solve matches
    the oracle's lanczos1 on H - w |o><o| (1e-10 relative)."""
    g = np.load(path)
    plan, vs, vx, yref = _plan(oracle, torch_cuda, g, 0)
    rng = np.random.default_rng(11)
    start = rng.standard_normal(vx.size)
    runs = []
    for _ in range(2):
        psi = _dev(torch_cuda, start)
        e, nmv = plan.lanczos(psi, mlanc=5)
        runs.append((e, nmv, psi.cpu().numpy()))
    assert runs[0][0] == runs[1][0] and runs[0][1] == runs[1][1]
    assert np.array_equal(runs[0][2], runs[1][2])

    o = vx / np.linalg.norm(vx)
    w = 7.5
    plan.add_projector(_dev(torch_cuda, o), w)
    psi = _dev(torch_cuda, start)
    e, _ = plan.lanczos(psi, mlanc=5)
    _, _, _, _, T, terms, hl, hr = idmrg_case.load(oracle, g)
    tl = []
    for coef, left, right in terms:
        L, R = idmrg_case.combine_host(oracle, T, left), idmrg_case.combine_host(oracle, T, right)
        tl.append((L[0], L[1], R[0], R[1], coef))
    prob = oracle.HeffProblem(vs, tl, hl, hr)
    e_or, _, _ = oracle.lanczos1(lambda v: oracle.heff_apply(prob, v) - w * np.dot(o, v) * o, start.copy(), 5)
    assert abs(e - e_or) <= 1e-10 * abs(e_or)
