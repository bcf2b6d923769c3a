"""The lattice tables built here (su2dmrg_gb300.warmup.cylinder_tables, the
dmrg_su2 constructor restated) equal the reference engine's own tables, bit
for bit, on every lattice the fixtures hold (J1 4x2 and J-Q 4x4, J1-J2 6x2,
4x2, 3x4 and 6x4, J-Q 3x4 with boundary 2; six more with boundaries 0, 1 and
3, tests/golden/lattice_tables.npz); the packaged spin-1/2 site operators
equal the engine's."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN

CASES = sorted(glob.glob(os.path.join(GOLDEN, "warmup_*.npz")) + glob.glob(os.path.join(GOLDEN, "sweep_*.npz")))


@pytest.mark.parametrize("path", CASES)
def test_cylinder_tables_match_engine(path):
    from su2dmrg_gb300.warmup import Lattice, cylinder_tables

    g = np.load(path)
    lx, ly = int(g["lx"]), int(g["ly"])
    hmap, coup, fll, frr, plqflg, plqpos = cylinder_tables(lx, ly, float(g["jcoup"]), float(g["qcoup"]))
    sites = [(g[f"site{i}_desc"], g[f"site{i}_flag"], g[f"site{i}_x"]) for i in range(10)]
    ref = Lattice.from_tables(g["tables"], g["coup"], sites, float(g["qcoup"]), int(g["d"]))
    assert ref.ns == lx * ly
    for a, b in ((hmap, ref.hmap), (fll, ref.fll), (frr, ref.frr), (plqflg, ref.plqflg), (plqpos, ref.plqpos)):
        assert np.array_equal(a, b)
    used = sorted({int(v) for v in np.unique(ref.hmap) if v > 0})
    assert np.array_equal(coup[used], ref.coup[used])


def test_packaged_site_operators_are_the_engines():
    from su2dmrg_gb300.warmup import Lattice

    g = np.load(CASES[0])
    lat = Lattice.cylinder(int(g["lx"]), int(g["ly"]), float(g["jcoup"]), float(g["qcoup"]), int(g["d"]))
    mine = lat.sigma + lat.qterm
    for i in range(10):
        st, x = mine[i]
        assert st.desc().tolist() == g[f"site{i}_desc"].tolist()
        assert st.flag.tolist() == g[f"site{i}_flag"].tolist()
        assert np.array_equal(x, g[f"site{i}_x"])


def _parse_tables(ints):
    """[ns, physpn, totspin, hmap, fll, frr, plqflg (ns x ns each), plqpos (ns x 4)]"""
    ns, q = int(ints[0]), 3
    mats = []
    for _ in range(4):
        mats.append(np.asarray(ints[q: q + ns * ns]).reshape(ns, ns))
        q += ns * ns
    return ns, mats, np.asarray(ints[q: q + 4 * ns]).reshape(ns, 4)


LT = np.load(os.path.join(GOLDEN, "lattice_tables.npz"))


@pytest.mark.parametrize("c", sorted({int(k.split("_")[0][1:]) for k in LT.files}))
def test_other_boundaries_match_engine(c):
    """Boundary 0 (square, periodic), 1 (J1-J3) and 3 (Shastry-Sutherland), with
    and without plaquette couplings."""
    from su2dmrg_gb300.warmup import cylinder_tables

    g = {k.split("_", 1)[1]: LT[k] for k in LT.files if k.startswith(f"c{c}_")}
    lx, ly = int(g["lx"]), int(g["ly"])
    ns, (hmap_r, fll_r, frr_r, plqflg_r), plqpos_r = _parse_tables(g["tables"])
    hmap, coup, fll, frr, plqflg, plqpos = cylinder_tables(lx, ly, float(g["jcoup"]), float(g["qcoup"]),
                                                           int(g["boundary"]))
    assert ns == lx * ly
    for a, b in ((hmap, hmap_r), (fll, fll_r), (frr, frr_r), (plqflg, plqflg_r), (plqpos, plqpos_r)):
        assert np.array_equal(a, b)
    used = sorted({int(v) for v in np.unique(hmap_r) if v > 0})
    assert np.array_equal(coup[used], np.asarray(g["coup"])[used])
