"""GPU parity of the site updates through the C ABI (su2g_env_run):
operator_initial (with and without endt), operator_pairup and permutation
against the reference's own outputs (tests/golden/site_*.npz), a whole site
step batched into one call (shared output slots summed, as hh[i] = overlap +
pairups) against the oracle, and larger seeded cases against the oracle.
Tolerance: 1e-12 relative (Frobenius) for FP64 and the 7-slice split mode."""
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


def _case(oracle, g):
    su = oracle.struct_from_desc(g["du"], g["fu"])
    x = (oracle.struct_from_desc(g["dx"], g["fx"]), g["xx"]) if "dx" in g.files else None
    sites = [(oracle.struct_from_desc(g[f"ds{i}"], g[f"fs{i}"]), g[f"xs{i}"]) for i in range(2) if f"ds{i}" in g.files]
    kind = str(g["kind"])
    kind = "init" if kind.startswith("init") else ("pair" if kind == "pair" else "perm")
    return kind, int(g["flag"]), su, x, sites


def _job(torch, kind, x, sites, slot=0, coef=1.0):
    j = {"kind": kind, "slot": slot, "coef": coef}
    if x is not None:
        j["x"] = (x[0], _dev(torch, x[1]))
    for i, s in enumerate(sites):
        j[f"site{i + 1}"] = s
    return j


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "site_*.npz"))))
def test_site_update_matches_reference(oracle, torch_cuda, path, mode):
    from su2dmrg_gb300.su2 import env_batch

    g = np.load(path)
    kind, flag, su, x, sites = _case(oracle, g)
    xu, xv = _dev(torch_cuda, g["xu"]), _dev(torch_cuda, g["xv"])
    (st, y), = env_batch(su, xu, su, xv, flag, [_job(torch_cuda, kind, x, sites)], mode=mode)
    assert st.flag.tolist() == g["rflag"].tolist()
    got = y[: st.size()].cpu().numpy()
    assert np.linalg.norm(got - g["rx"]) <= TOL * np.linalg.norm(g["rx"])


def _rand_tensor(oracle, rng, bonds, drop=0.0):
    s = oracle.Struct(bonds, 0).with_legal_flags()
    s.flag = (s.flag * (rng.random(s.nten) >= drop)).astype(np.int32)
    _, tot = s.offsets()
    return s, rng.standard_normal(tot)


def _site_ops(oracle, flag):
    """The engine's site operators from the fixtures (sigma, qterm)."""
    out = {}
    for path in sorted(glob.glob(os.path.join(GOLDEN, f"site_*_0_{flag}.npz"))):
        g = np.load(path)
        kind = str(g["kind"])
        out[kind] = [(oracle.struct_from_desc(g[f"ds{i}"], g[f"fs{i}"]), g[f"xs{i}"]) for i in range(2)
                     if f"ds{i}" in g.files]
    return out


def site_step_case(oracle, flag):
    """A whole site step as one batch (host data): slot 0 = overlap(hh) +
    pairup(op_a, sigma) - 0.7 pairup(op_b, sigma) (summed in place); slots
    1, 2 = transformations (spin multiplicities 1 and 1+2); slot 3 =
    operator_initial; slot 4 = a plaquette permutation; slot 5 =
    operator_initial with endt.  Bond dims 20-60 per sector.  Returns
    (su, xu, xv, jobs, expected [(Struct, data)] per slot)."""
    rng = np.random.default_rng(77 + flag)
    sa, sc = [0, 2, 4, 6], [1, 3, 5, 7]
    da = [int(v) for v in rng.integers(20, 61, len(sa))]
    dc = [int(v) for v in rng.integers(20, 61, len(sc))]
    B = oracle.Bond
    phys = B(1, [1], [1])
    ub = [B(-1, sa, da), phys, B(1, sc, dc)] if flag == 0 else [phys, B(-1, sa, da), B(1, sc, dc)]
    su, xu = _rand_tensor(oracle, rng, ub)
    _, xv = _rand_tensor(oracle, rng, ub)
    hh = _rand_tensor(oracle, rng, [B(1, sa, da), B(-1, sa, da)])
    op_a = _rand_tensor(oracle, rng, [B(1, sa, da), B(-1, [2], [1]), B(-1, sa, da)])
    op_b = _rand_tensor(oracle, rng, [B(1, sa, da), B(-1, [2], [1]), B(-1, sa, da)], drop=0.2)
    op_c = _rand_tensor(oracle, rng, [B(1, sa, da), B(-1, [0, 2], [1, 2]), B(-1, sa, da)])
    vec = _rand_tensor(oracle, rng, [B(1, sa, da), B(-1, [2], [1]), B(-1, sa, da)])
    endt = _rand_tensor(oracle, rng, [B(1, sa, da), B(-1, sa, da)])
    sites = _site_ops(oracle, flag)
    sig_init, sig_pair, perm = sites["init"], sites["pair"], sites["perm1"]
    jobs = [
        ("overlap", hh, [], 0, 1.0),
        ("pair", op_a, sig_pair, 0, 1.0),
        ("pair", op_b, sig_pair, 0, -0.7),
        ("transform", op_a, [], 1, 1.0),
        ("transform", op_c, [], 2, 1.0),
        ("init", None, sig_init, 3, 1.0),
        ("perm", vec, perm, 4, 1.0),
        ("init", endt, sig_init, 5, 1.0),
    ]

    def ref_env(kind, x):
        return oracle.env_transform(kind, su, xu, su, xv, x[0], x[1], flag)

    def add(a, b, cb=1.0):  # union-layout sum of two (Struct, data)
        (sa_, xa), (sb_, xb) = a, b
        out = oracle.Struct(sa_.bonds, sa_.locspin)
        out.flag = np.maximum(sa_.flag, sb_.flag).astype(np.int32)
        return out, oracle.to_layout(sa_, xa, out) + cb * oracle.to_layout(sb_, xb, out)

    def want():
        return [
            add(add(ref_env(0, hh), oracle.site_update("pair", flag, su, xu, su, xv, op_a, sig_pair)),
                oracle.site_update("pair", flag, su, xu, su, xv, op_b, sig_pair), -0.7),
            ref_env(1, op_a),
            ref_env(1, op_c),
            oracle.site_update("init", flag, su, xu, su, xv, None, sig_init),
            oracle.site_update("perm", flag, su, xu, su, xv, vec, perm),
            oracle.site_update("init", flag, su, xu, su, xv, endt, sig_init),
        ]

    return su, xu, xv, jobs, want


def job_dicts(jobs, dev=lambda a: a):
    return [{"kind": k, "slot": s, "coef": c, "x": None if x is None else (x[0], dev(x[1])),
             **{f"site{i + 1}": st for i, st in enumerate(sites)}} for k, x, sites, s, c in jobs]


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("flag", [0, 1])
def test_site_step_batch_matches_oracle(oracle, torch_cuda, flag, mode):
    """One call for a whole site step (site_step_case) against the oracle."""
    from su2dmrg_gb300.su2 import env_batch

    su, xu, xv, jobs, want = site_step_case(oracle, flag)
    res = env_batch(su, _dev(torch_cuda, xu), su, _dev(torch_cuda, xv), flag,
                    job_dicts(jobs, lambda a: _dev(torch_cuda, a)), mode=mode)
    for slot, ((st, y), (ws, wx)) in enumerate(zip(res, want())):
        assert st.flag.tolist() == ws.flag.tolist(), slot
        got = y[: st.size()].cpu().numpy()
        assert np.linalg.norm(got - wx) <= TOL * np.linalg.norm(wx), slot
