"""GPU parity of the moves between two steps through the C ABI:
su2g_vectran (wavefunc_transformation: right2left / left2right_vectran) and
su2g_prepare_input_vector (dmrg_su2::prepare_input_vector), against the
reference's own outputs (tests/golden/inputvec_*.npz, vectran_*.npz) and
against the oracle on larger seeded MPS tensors.  vectran moves numbers only:
bit-exact.  The input vector is a sum of products: 1e-12 relative
(Frobenius) for FP64 and the 7-slice split mode, 1e-10 for the 6-slice mode."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
TOL = {0: 1e-12, 1: 1e-12, 2: 1e-10}


@pytest.fixture(scope="module")
def torch_cuda(su2lib):
    import torch

    assert torch.cuda.is_available()
    return torch


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float64)).cuda()


def _lib_struct(oracle_struct):
    from su2dmrg_gb300.su2 import _parse_desc

    s = _parse_desc(oracle_struct.desc())
    s.flag = np.ascontiguousarray(oracle_struct.flag, np.int32)
    return s


def _from_desc(desc, flag):
    from su2dmrg_gb300.su2 import _parse_desc

    s = _parse_desc(desc)
    s.flag = np.ascontiguousarray(flag, np.int32)
    return s


@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "inputvec_*.npz"))))
def test_input_vector_matches_reference(torch_cuda, path, mode):
    from su2dmrg_gb300.su2 import prepare_input_vector

    g = np.load(path)
    s, y = prepare_input_vector(_from_desc(g["dl"], g["fl"]), _dev(torch_cuda, g["xl"]),
                                _from_desc(g["dr"], g["fr"]), _dev(torch_cuda, g["xr"]), mode=mode)
    assert s.desc().tolist() == g["rdesc"].tolist()
    assert s.flag.tolist() == g["rflag"].tolist()
    got = y[: s.size()].cpu().numpy()
    assert np.linalg.norm(got - g["rx"]) <= TOL[mode] * np.linalg.norm(g["rx"])


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "vectran_*.npz"))))
def test_vectran_matches_reference(torch_cuda, path):
    from su2dmrg_gb300.su2 import vectran

    g = np.load(path)
    s, y = vectran(_from_desc(g["du"], g["fu"]), _dev(torch_cuda, g["xu"]), int(g["dir"]))
    assert s.desc().tolist() == g["rdesc"].tolist()
    assert s.flag.tolist() == g["rflag"].tolist()
    assert np.array_equal(y[: s.size()].cpu().numpy(), g["rx"])


def mps_pair(oracle, seed, lo, hi, drop=0.0):
    """uu[il] (bond, spin, centre) and uu[ir] (spin, bond, centre) with
    spin-1/2 physical legs, multiplet counts in [lo, hi], and a fraction
    `drop` of their legal blocks absent."""
    rng = np.random.default_rng(seed)
    B = oracle.Bond
    sa, sc, sb = [0, 2, 4, 6, 8], [1, 3, 5, 7], [0, 2, 4, 6, 8]
    dims = lambda sec: [int(v) for v in rng.integers(lo, hi + 1, len(sec))]
    da, dc, db = dims(sa), dims(sc), dims(sb)
    ph = B(1, [1], [1])

    def mk(bonds):
        s = oracle.Struct(bonds, 0).with_legal_flags()
        s.flag = (s.flag * (rng.random(s.nten) >= drop)).astype(np.int32)
        _, tot = s.offsets()
        return s, rng.standard_normal(tot)

    return mk([B(1, sa, da), ph, B(-1, sc, dc)]), mk([ph, B(1, sb, db), B(-1, sc, dc)])


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("drop", [0.0, 0.25])
def test_input_vector_matches_oracle(oracle, torch_cuda, mode, drop):
    """Multiplet counts 60-250 per sector (products with K up to 250 in
    every split tile shape), with and without absent blocks."""
    from su2dmrg_gb300.su2 import prepare_input_vector

    (sl, xl), (sr, xr) = mps_pair(oracle, 11 + int(drop * 100), 60, 250, drop)
    want_s, want = oracle.prepare_input_vector(sl, xl, sr, xr)
    s, y = prepare_input_vector(_lib_struct(sl), _dev(torch_cuda, xl), _lib_struct(sr), _dev(torch_cuda, xr),
                                mode=mode)
    assert s.desc().tolist() == want_s.desc().tolist()
    assert s.flag.tolist() == want_s.flag.tolist()
    got = y[: s.size()].cpu().numpy()
    assert np.linalg.norm(got - want) <= TOL[mode] * np.linalg.norm(want)


@pytest.mark.parametrize("direction", [0, 1])
def test_vectran_matches_oracle_and_round_trips(oracle, torch_cuda, direction):
    """Larger blocks (multiplets 100-700, partial 32x32 tiles everywhere):
    bit-exact against the oracle, in place as well, and the opposite
    rotation restores the tensor bit for bit."""
    from su2dmrg_gb300.su2 import vectran

    (sl, xl), _ = mps_pair(oracle, 5, 100, 700, 0.2)
    want_s, want = oracle.vectran(sl, xl, direction)
    x = _dev(torch_cuda, xl)
    s, y = vectran(_lib_struct(sl), x, direction)
    assert s.flag.tolist() == want_s.flag.tolist()
    assert np.array_equal(y[: s.size()].cpu().numpy(), want)
    s2, z = vectran(s, y, 1 - direction)
    assert s2.desc().tolist() == sl.desc().tolist()
    assert np.array_equal(z[: s2.size()].cpu().numpy(), xl)
    x2 = _dev(torch_cuda, xl)
    vectran(_lib_struct(sl), x2, direction, out=x2)  # in place, as the reference rotates uu[i]
    assert np.array_equal(x2.cpu().numpy(), want)


def test_step_move_chain(oracle, torch_cuda):
    """A tensor rotated by left2right_vectran and back by right2left_vectran
    (the rotations successive steps apply to one MPS tensor) comes back bit
    for bit and feeds prepare_input_vector: the vector equals the oracle's."""
    from su2dmrg_gb300.su2 import prepare_input_vector, vectran

    (sl, xl), (sr, xr) = mps_pair(oracle, 23, 30, 90, 0.1)
    pre_s, pre_x = oracle.vectran(sr, xr, 1)
    s_rot, x_rot = vectran(_lib_struct(pre_s), _dev(torch_cuda, pre_x), 0)
    assert np.array_equal(x_rot[: s_rot.size()].cpu().numpy(), xr)
    want_s, want = oracle.prepare_input_vector(sl, xl, sr, xr)
    s, y = prepare_input_vector(_lib_struct(sl), _dev(torch_cuda, xl), s_rot, x_rot)
    got = y[: s.size()].cpu().numpy()
    assert np.linalg.norm(got - want) <= 1e-12 * np.linalg.norm(want)


def test_input_vector_product_refuses_different_centre_bonds(torch_cuda):
    """U_L U_R^T contracts the two tensors' leg 2: bonds that differ are
    refused before any device work (the structure alone accepts them)."""
    from su2dmrg_gb300.capi import Su2gError
    from su2dmrg_gb300.su2 import prepare_input_vector

    g = np.load(os.path.join(GOLDEN, "inputvec_0.npz"))
    ur = _from_desc(g["dr"], g["fr"])
    b2 = ur.bonds[2]
    ur.bonds[2] = type(b2)(b2.dir, list(b2.angm), [d + 1 for d in b2.dim])
    ur.flag = np.asarray(ur.flag, np.int32)
    xr = _dev(torch_cuda, np.zeros(ur.size() + 1))
    with pytest.raises(Su2gError, match="leg 2"):
        prepare_input_vector(_from_desc(g["dl"], g["fl"]), _dev(torch_cuda, g["xl"]), ur, xr)
