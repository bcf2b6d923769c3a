"""Checkpoint files read into and written from device buffers: the reduced
blocks of every site the reference engine wrote (tests/golden/ckpt/) load
bit-exactly equal to the engine's own tensors, writing them back reproduces
the engine's files byte for byte, a CG part scaled by 2 loads as half the
blocks, and a D=2000 MPS tensor round-trips bit-exactly."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
CK = os.path.join(GOLDEN, "ckpt")


@pytest.fixture(scope="module")
def engine(su2lib):
    import torch

    assert torch.cuda.is_available()
    return np.load(os.path.join(GOLDEN, "ckpt_engine.npz"))


def _site(S, ns, i):
    return (os.path.join(CK, S.checkpoint_name(S.CKPT_MPS_DAT, ns, 16, pos=i)),
            os.path.join(CK, S.checkpoint_name(S.CKPT_MPS_BIN, ns, 16, pos=i)))


def test_load_matches_engine_and_save_reproduces_files(engine, tmp_path):
    from su2dmrg_gb300 import su2 as S

    ns = int(engine["ns"])
    for i in range(ns):
        dat, bin_ = _site(S, ns, i)
        s, x = S.mps_load(dat, bin_)
        assert np.array_equal(x[: s.size()].cpu().numpy(), engine[f"x{i}"]), i
        S.mps_save(tmp_path / "a.dat", tmp_path / "a.bin", s, x)
        assert (tmp_path / "a.dat").read_bytes() == open(dat, "rb").read(), i
        assert (tmp_path / "a.bin").read_bytes() == open(bin_, "rb").read(), i


def test_scaled_cg_part_rescales_blocks(engine, tmp_path):
    from su2dmrg_gb300 import su2 as S

    ns = int(engine["ns"])
    dat, bin_ = _site(S, ns, ns // 2)
    raw = open(bin_, "rb").read()
    s = S.mps_load_layout(dat, bin_)
    ncg = (len(raw) - 4 * s.nten - 8 * s.size()) // 8
    cg = np.frombuffer(raw[len(raw) - 8 * ncg:], np.float64) * 2.0
    (tmp_path / "s.bin").write_bytes(raw[: len(raw) - 8 * ncg] + cg.tobytes())
    _, x = S.mps_load(dat, tmp_path / "s.bin")
    assert np.array_equal(x[: s.size()].cpu().numpy(), 2.0 * engine[f"x{ns // 2}"])


def test_d2000_round_trip(tmp_path):
    import torch

    from su2dmrg_gb300 import su2 as S
    from su2dmrg_gb300.workloads import synthetic_site_step

    w = synthetic_site_step(D=2000, nops=0)
    s, xh = w.ul
    x = torch.from_numpy(xh).cuda()
    S.mps_save(tmp_path / "u.dat", tmp_path / "u.bin", s, x)
    s2, y = S.mps_load(tmp_path / "u.dat", tmp_path / "u.bin")
    assert s2.desc().tolist() == s.desc().tolist() and s2.flag.tolist() == s.flag.tolist()
    assert torch.equal(y[: s.size()], x)
