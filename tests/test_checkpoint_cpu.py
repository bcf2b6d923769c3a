"""Checkpoint files (dmrg_su2::save_mps2 / read_mps, save_enr / read_enr,
save_ww / read_ww, dmrg_su2_omp.cpp:864-1242), host side: names, structures,
flags, energies and weights against files the reference engine wrote itself
(tests/golden/ckpt/, after do_idmrg and one sweep of a 4x2 lattice at D=16)
and against what its own readers returned (tests/golden/ckpt_engine.npz).
The reduced data travels to and from device buffers: tests/test_checkpoint_gpu.py."""
import os
import shutil

import numpy as np
import pytest

from conftest import GOLDEN

CK = os.path.join(GOLDEN, "ckpt")


@pytest.fixture(scope="module")
def engine(su2lib):
    return np.load(os.path.join(GOLDEN, "ckpt_engine.npz"))


def _site(S, ns, i):
    return (os.path.join(CK, S.checkpoint_name(S.CKPT_MPS_DAT, ns, 16, pos=i)),
            os.path.join(CK, S.checkpoint_name(S.CKPT_MPS_BIN, ns, 16, pos=i)))


def test_names_are_the_engines(engine):
    from su2dmrg_gb300 import su2 as S

    ns = int(engine["ns"])
    want = set(str(f) for f in engine["files"])
    got = {S.checkpoint_name(k, ns, 16, pos=i) for k in (S.CKPT_MPS_DAT, S.CKPT_MPS_BIN) for i in range(ns)}
    got |= {S.checkpoint_name(S.CKPT_ENR, ns, 16), S.checkpoint_name(S.CKPT_WW, ns, 16, pos=ns // 2)}
    assert got == want


def test_mps_layouts_match_the_engine(engine):
    from su2dmrg_gb300 import su2 as S

    ns = int(engine["ns"])
    for i in range(ns):
        s = S.mps_load_layout(*_site(S, ns, i))
        assert s.desc().tolist() == engine[f"desc{i}"].tolist(), i
        assert s.flag.tolist() == engine[f"flag{i}"].tolist(), i
        assert s.size() == len(engine[f"x{i}"]), i


def test_energies_match_the_engine(engine, tmp_path):
    from su2dmrg_gb300 import su2 as S

    path = os.path.join(CK, S.checkpoint_name(S.CKPT_ENR, int(engine["ns"]), 16))
    vals = S.enr_read(path)
    assert vals[-1] + 1000.0 == float(engine["enr_read"])  # read_enr keeps the last value, shifted back
    out = tmp_path / "enr.dat"
    for v in vals:
        S.enr_append(out, v)
    assert out.read_bytes() == open(path, "rb").read()
    S.enr_append(tmp_path / "one.dat", float(engine["enr_written"]))
    assert (tmp_path / "one.dat").read_bytes() == open(path, "rb").read().splitlines(True)[-1]


def test_weights_match_the_engine(engine, tmp_path):
    from su2dmrg_gb300 import su2 as S

    ns = int(engine["ns"])
    path = os.path.join(CK, S.checkpoint_name(S.CKPT_WW, ns, 16, pos=ns // 2))
    ww = S.ww_load(path, 64)
    assert len(ww) == 32  # save_ww writes max_dcut * phdim doubles
    assert np.array_equal(ww[:16], engine["ww_read"])  # read_ww reads max_dcut of them
    S.ww_save(tmp_path / "ww.bin", ww)
    assert (tmp_path / "ww.bin").read_bytes() == open(path, "rb").read()


def test_malformed_files_are_refused(engine, tmp_path):
    from su2dmrg_gb300 import capi
    from su2dmrg_gb300 import su2 as S

    ns = int(engine["ns"])
    dat, bin_ = _site(S, ns, ns // 2)
    with pytest.raises(capi.Su2gError) as e:
        S.mps_load_layout(dat, tmp_path / "missing.bin")
    assert e.value.code == capi.SU2G_EIO
    raw = open(bin_, "rb").read()
    (tmp_path / "short.bin").write_bytes(raw[:-8])
    with pytest.raises(capi.Su2gError) as e:
        S.mps_load_layout(dat, tmp_path / "short.bin")
    assert e.value.code == capi.SU2G_EIO
    (tmp_path / "long.bin").write_bytes(raw + b"\0" * 8)
    with pytest.raises(capi.Su2gError) as e:
        S.mps_load_layout(dat, tmp_path / "long.bin")
    assert e.value.code == capi.SU2G_EIO
    # a CG part that is not proportional to the canonical one
    s = S.mps_load_layout(dat, bin_)
    ncg = (len(raw) - 4 * s.nten - 8 * s.size()) // 8
    cg = np.frombuffer(raw[len(raw) - 8 * ncg:], np.float64).copy()
    cg[::2] *= -1.0
    (tmp_path / "cg.bin").write_bytes(raw[: len(raw) - 8 * ncg] + cg.tobytes())
    with pytest.raises(capi.Su2gError) as e:
        S.mps_load_layout(dat, tmp_path / "cg.bin")
    assert e.value.code == capi.SU2G_EUNSUPPORTED
    (tmp_path / "bad.dat").write_text("3 0\n1 2\n0\n")
    with pytest.raises(capi.Su2gError) as e:
        S.mps_load_layout(tmp_path / "bad.dat", bin_)
    assert e.value.code == capi.SU2G_EIO
