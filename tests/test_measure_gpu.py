"""GPU parity of the centre-bond energy (dmrg_su2::mea_enr,
dmrg_su2_omp_mea_enr.cpp:194-242) and its reductions through the C ABI:
take_trace and ss_inner_prod against the engine's own values (1e-13
relative), multiply_singular_value bit-exact, and su2g_mea_enr against the
value the engine's measurement variant returned on its own checkpoints
(tests/golden/mea_*.npz, 1e-12 relative), then against the oracle on
D=2000-sized centre tensors."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN
from test_oracle_golden import mea_case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda(su2lib):
    import torch

    assert torch.cuda.is_available()
    return torch


def _lib(oracle_struct):
    from su2dmrg_gb300.su2 import _parse_desc

    s = _parse_desc(oracle_struct.desc())
    s.flag = np.ascontiguousarray(oracle_struct.flag, np.int32)
    return s


def _dev(torch, t):
    if t is None:
        return None
    return _lib(t[0]), torch.from_numpy(np.ascontiguousarray(t[1], np.float64)).cuda()


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "meaop_*.npz"))))
def test_reductions_match_engine(oracle, torch_cuda, path):
    from su2dmrg_gb300 import su2 as S

    g = np.load(path)
    sh, xh = _dev(torch_cuda, (oracle.struct_from_desc(g["dh"], g["fh"]), g["xh"]))
    assert abs(S.take_trace(sh, xh) - g["trace"]) <= 1e-13 * max(1.0, abs(g["trace"]))
    for leg in (0, 1):
        y = xh.clone()
        S.multiply_singular_value(sh, y, leg, g["w"])
        assert np.array_equal(y.cpu().numpy(), g[f"msv{leg}"])
    a = _dev(torch_cuda, (oracle.struct_from_desc(g["do"], g["fa"]), g["xa"]))
    b = _dev(torch_cuda, (oracle.struct_from_desc(g["do"], g["fb"]), g["xb"]))
    assert abs(S.ss_inner_prod(a, b) - g["inner"]) <= 1e-13 * max(1.0, abs(g["inner"]))


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "mea_*.npz"))))
def test_mea_enr_matches_engine(oracle, torch_cuda, path):
    from su2dmrg_gb300 import su2 as S

    g = np.load(path)
    hl, hr, ww, pairs = mea_case(oracle, g)
    e, parts = S.mea_enr(_dev(torch_cuda, hl), _dev(torch_cuda, hr), ww,
                         [(_dev(torch_cuda, l), _dev(torch_cuda, r), c) for l, r, c in pairs])
    assert abs(e - g["parts"][4]) <= 1e-12 * abs(g["parts"][4])
    assert np.allclose(parts, g["parts"][:4], rtol=1e-12, atol=1e-14)


def test_mea_enr_d2000_matches_oracle(oracle, torch_cuda):
    """Centre tensors at D=2000 (sector counts of the benchmark workload):
    block Hamiltonians, 18 spin-1 operator pairs, two never-built plaquette
    pairs, random weights."""
    from su2dmrg_gb300 import su2 as S
    from su2dmrg_gb300.workloads import gaussian_sector_counts

    rng = np.random.default_rng(2000)
    counts = gaussian_sector_counts(2000)
    angm = [k for k in range(13) if counts[k] > 0]
    dims = [counts[k] for k in angm]
    B = oracle.Bond

    def mk(bonds):
        s = oracle.Struct(bonds, 0).with_legal_flags()
        _, tot = s.offsets()
        return s, rng.standard_normal(tot)

    hl = mk([B(1, angm, dims), B(-1, angm, dims)])
    hr = mk([B(1, angm, dims), B(-1, angm, dims)])
    ww = rng.random(2000)
    ops = [(mk([B(1, angm, dims), B(-1, [2], [1]), B(-1, angm, dims)]),
            mk([B(1, angm, dims), B(-1, [2], [1]), B(-1, angm, dims)]), float(c)) for c in rng.standard_normal(18)]
    pairs = ops + [(None, None, -1.0), (None, None, -1.0)]
    want = oracle.mea_enr(hl, hr, ww, pairs)
    e, _ = S.mea_enr(_dev(torch_cuda, hl), _dev(torch_cuda, hr), ww,
                     [(_dev(torch_cuda, l), _dev(torch_cuda, r), c) for l, r, c in pairs])
    assert abs(e - want) <= 1e-12 * abs(want)
