"""GPU parity of the environment updates (operator_transformation,
overlap_transformation) through the C ABI: against the reference's own outputs
(tests/golden/env_*.npz) and against the oracle on batched synthetic inputs.
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


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "env_*.npz"))))
def test_env_matches_reference(torch_cuda, oracle, path, mode):
    from su2dmrg_gb300 import su2

    torch = torch_cuda
    g = np.load(path)
    ovl = "env_ovl" in path
    su = oracle.struct_from_desc(g["du"], g["fu"])
    so = oracle.struct_from_desc(g["dop"], g["fop"])
    flag = int(g["flag"])
    layout = (su2.overlap_transformation_layout if ovl else su2.operator_transformation_layout)(
        su, g["xu"], su, g["xv"], so, g["xop"], flag)
    y = torch.full((layout.size(),), np.nan, dtype=torch.float64, device="cuda")
    run = su2.overlap_transformation if ovl else su2.operator_transformation
    run(su, _dev(torch, g["xu"]), su, _dev(torch, g["xv"]), [(so, _dev(torch, g["xop"]))], [y], flag, mode=mode)
    got = y.cpu().numpy()
    ref = g["rx"]
    assert np.all(np.isfinite(got))
    assert np.linalg.norm(got - ref) <= TOL * np.linalg.norm(ref)


def _random_env(rng, D=200, nops=5):
    """A left-canonical-shaped MPS tensor (bond A x spin-1/2 -> bond C) and
    spin-1 operators on bond A."""
    from su2dmrg_gb300.su2 import Su2Bond, Su2Struct
    from su2dmrg_gb300.workloads import gaussian_sector_counts

    ca = gaussian_sector_counts(D, 10)
    cc = gaussian_sector_counts(D, 11)
    A = Su2Bond(-1, [k for k in range(11) if ca[k]], [c for c in ca if c])
    C = Su2Bond(1, [k for k in range(12) if cc[k]], [c for c in cc if c])
    uu = Su2Struct([A, Su2Bond(-1, [1], [1]), C], 0).with_legal_flags()
    xu = rng.standard_normal(uu.size())
    xv = rng.standard_normal(uu.size())
    ops = []
    for t in range(nops):
        spin = Su2Bond(1, [2], [1]) if t % 2 == 0 else Su2Bond(1, [0, 2], [1, 1])
        op = Su2Struct([A.inverted(), spin, A], 0).with_legal_flags()
        op.flag = (op.flag * (rng.random(op.nten) > 0.1)).astype(np.int32)
        ops.append((op, rng.standard_normal(op.size())))
    return uu, xu, xv, ops


@pytest.mark.parametrize("mode", [0, 1])
def test_batched_operator_transformation_matches_oracle(torch_cuda, oracle, mode):
    from su2dmrg_gb300 import su2

    torch = torch_cuda
    rng = np.random.default_rng(17)
    uu, xu, xv, ops = _random_env(rng, D=60, nops=5)
    layouts = [su2.operator_transformation_layout(uu, xu, uu, xv, op, xo, 0) for op, xo in ops]
    outs = [torch.full((l.size(),), np.nan, dtype=torch.float64, device="cuda") for l in layouts]
    su2.operator_transformation(uu, _dev(torch, xu), uu, _dev(torch, xv), [(op, _dev(torch, xo)) for op, xo in ops],
                                outs, 0, mode=mode)
    for (op, xo), lay, y in zip(ops, layouts, outs):
        ref_s, ref = oracle.env_transform(1, uu, xu, uu, xv, op, xo, 0)
        assert ref_s.flag.tolist() == lay.flag.tolist()
        got = y.cpu().numpy()
        assert np.linalg.norm(got - ref) <= TOL * np.linalg.norm(ref)


def test_overlap_transformation_d200_fp64_vs_split(torch_cuda):
    """Larger blocks (D = 200 bonds): split mode against the FP64 mode."""
    from su2dmrg_gb300 import su2
    from su2dmrg_gb300.su2 import Su2Struct

    torch = torch_cuda
    rng = np.random.default_rng(5)
    uu, xu, xv, _ = _random_env(rng, D=200, nops=1)
    A = uu.bonds[0]
    hh = Su2Struct([A.inverted(), A], 0).with_legal_flags()
    xh = rng.standard_normal(hh.size())
    lay = su2.overlap_transformation_layout(uu, xu, uu, xv, hh, xh, 0)
    ys = []
    for mode in (0, 1):
        y = torch.empty(lay.size(), dtype=torch.float64, device="cuda")
        su2.overlap_transformation(uu, _dev(torch, xu), uu, _dev(torch, xv), [(hh, _dev(torch, xh))], [y], 0,
                                   mode=mode)
        ys.append(y.cpu().numpy())
    assert np.linalg.norm(ys[1] - ys[0]) <= TOL * np.linalg.norm(ys[0])
