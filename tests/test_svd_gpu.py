"""GPU parity of the truncation step (su2g_svd = tensor_su2::svd) through the
C ABI: against the reference's own outputs (tests/golden/svd_*.npz) and
against the oracle on larger seeded cases, including degenerate spectra
across sectors (the tie order of the reference's Shell sort decides which
multiplets survive) and the max_dcut extremes.

Kept multiplets per sector must match exactly; singular values within
1e-12*s_max + 1e-15*s_max^2/s (the Gram method's own accuracy); the new MPS
tensors gauge-free (U_c V_c^T and column norms within 1e-10 relative)."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN
from svd_checks import check_mps, check_truncation_values

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda(su2lib):
    import torch

    assert torch.cuda.is_available()
    return torch


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float64)).cuda()


def _su2(struct):
    from su2dmrg_gb300 import su2

    s = su2.Su2Struct([su2.Su2Bond(b.dir, list(b.angm), list(b.dim)) for b in struct.bonds], struct.locspin)
    s.flag = np.asarray(struct.flag, np.int32)
    return s


def _as_oracle(oracle, s, x):
    return oracle.struct_from_desc(s.desc(), s.flag), x.cpu().numpy()


def _run(oracle, torch, vs, x, su, sv, p1, p2, dcut):
    from su2dmrg_gb300 import su2

    tus, tux, tvs, tvx, wout = su2.svd(_su2(vs), _dev(torch, x), _su2(su), p1, _su2(sv), p2, dcut)
    torch.cuda.synchronize()
    return _as_oracle(oracle, tus, tux), _as_oracle(oracle, tvs, tvx), wout


def _kept(tu):
    S = tu[0]
    return {a: d for a, d in zip(S.bonds[2].angm, S.bonds[2].dim)}


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "svd_*.npz"))))
def test_svd_matches_reference(oracle, torch_cuda, path):
    g = np.load(path)
    vs = oracle.struct_from_desc(g["dvec"], g["fvec"])
    su, sv = oracle.struct_from_desc(g["du"]), oracle.struct_from_desc(g["dv"])
    tu, tv, wout = _run(oracle, torch_cuda, vs, g["xvec"], su, sv, float(g["p1"]), float(g["p2"]), int(g["dcut"]))
    ref_kept = {a: int(d) for a, d in enumerate(g["kept"]) if d}
    assert _kept(tu) == ref_kept
    check_truncation_values(wout, g["wout"], int(g["kept"].sum()))
    rtu = (oracle.struct_from_desc(g["tu_desc"], g["tu_flag"]), g["tu_x"])
    rtv = (oracle.struct_from_desc(g["tv_desc"], g["tv_flag"]), g["tv_x"])
    check_mps(oracle, tu, tv, rtu, rtv)


def _case(oracle, rng, la, lda, ra, rda, decay, tie=False):
    """psi on fuse(bond, spin-1/2) x fuse(bond, spin-1/2); blocks with spectra
    s_k = exp(-decay k)(1 + u_k).  tie=True gives every sector of equal shape
    the same block, so equal singular values appear across sectors."""
    ph = oracle.Bond(-1, [1], [1])
    Lb, Rb = oracle.Bond(-1, la, lda), oracle.Bond(-1, ra, rda)
    vs = oracle.Struct([oracle.fuse(Lb, ph), oracle.fuse(Rb, ph)], 0).with_legal_flags()
    off, tot = vs.offsets()
    x = np.zeros(tot)
    shared = {}
    for b in range(vs.nten):
        if not vs.flag[b]:
            continue
        m, n = vs.block_shape(b)
        if tie and (m, n) in shared:
            blk = shared[(m, n)]
        else:
            q1, _ = np.linalg.qr(rng.standard_normal((m, min(m, n))))
            q2, _ = np.linalg.qr(rng.standard_normal((n, min(m, n))))
            sv = np.exp(-decay * np.arange(min(m, n))) * (1 + rng.random(min(m, n)))
            blk = (q1 * sv) @ q2.T
            shared[(m, n)] = blk
        x[off[b]: off[b] + m * n] = blk.ravel(order="F")
    su = oracle.Struct([Lb, ph, oracle.Bond(1, [0], [1])], 0).with_legal_flags()
    sv = oracle.Struct([Rb, ph, oracle.Bond(1, [0], [1])], 0).with_legal_flags()
    return vs, x, su, sv


CASES = [  # (left sectors, dims, right sectors, dims, p1, p2, max_dcut, decay, tie)
    ([0, 2, 4, 6, 8], [40, 70, 60, 30, 10], [0, 2, 4, 6, 8], [50, 60, 60, 25, 12], 1.0, 0.0, 120, 0.05, False),
    ([1, 3, 5, 7], [90, 110, 70, 20], [1, 3, 5, 7], [80, 120, 60, 30], 0.0, 1.0, 200, 0.02, False),
    ([0, 1, 2, 3, 4, 5], [20, 35, 40, 35, 20, 8], [0, 1, 2, 3, 4, 5], [20, 35, 40, 35, 20, 8], 1.0, 0.0, 90, 0.1,
     False),
    # two 30 x 30 sectors (2j = 0, 2) holding the same block: every value is a
    # pair across sectors, and an odd max_dcut splits one pair
    ([1], [30], [1], [30], 1.0, 0.0, 21, 0.2, True),
    # keep everything; keep one multiplet
    ([0, 2, 4], [12, 20, 9], [0, 2, 4], [15, 18, 9], 1.0, 0.0, 100000, 0.3, False),
    ([0, 2, 4], [12, 20, 9], [0, 2, 4], [15, 18, 9], 0.0, 1.0, 1, 0.3, False),
]


@pytest.mark.parametrize("ci", range(len(CASES)))
def test_svd_matches_oracle(oracle, torch_cuda, ci):
    la, lda, ra, rda, p1, p2, dcut, decay, tie = CASES[ci]
    rng = np.random.default_rng(1000 + ci)
    vs, x, su, sv = _case(oracle, rng, la, lda, ra, rda, decay, tie)
    tu, tv, wout = _run(oracle, torch_cuda, vs, x, su, sv, p1, p2, dcut)
    dims, rw, uv = oracle.svd_truncate(vs, x, p1, p2, dcut)
    rtu, rtv = oracle.svd_mps(vs, dims, uv, su.bonds[:2], sv.bonds[:2])
    ref_kept = {vs.bonds[0].angm[i]: int(d) for i, d in enumerate(dims) if d}
    assert _kept(tu) == ref_kept
    check_truncation_values(wout, rw, int(np.sum(dims)))
    check_mps(oracle, tu, tv, rtu, rtv)
    if tie:  # the tie really is exercised: a degenerate value straddles the cut
        kept_min = min(wout[: int(np.sum(dims))])
        assert np.any(np.abs(wout[int(np.sum(dims)):] - kept_min) <= 1e-12 * kept_min)
