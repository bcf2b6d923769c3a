"""DMRG sweeps with every tensor on the device (su2dmrg_gb300.sweep: the
warm-up, then dmrg_su2::sweep until a sweep changes the energy by less than
1e-6, as main_omp does) against whole runs of the reference engine
(tests/golden/dmrg_energies.json: J1-J2 4x2 and 3x4 and J-Q 3x4 at D=64, J1-J2
6x4 with nearest-neighbour coupling 2 and diagonal 1 at D=200; lattice tables in tests/golden/sweep_*.npz).

The warm-up's path follows rounding noise (tests/test_warmup_gpu.py), but
the sweeps converge to the same state: the converged energy in FP64 and in
split precision is the reference's to 1e-10 relative, and the final FP64 MPS
has the reference's retained multiplets, sector by sector, at every bond."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
RUNS = json.load(open(os.path.join(GOLDEN, "dmrg_energies.json")))


@pytest.fixture(scope="module")
def torch_cuda(su2lib):
    import torch

    assert torch.cuda.is_available()
    return torch


def _lattice(c):
    from su2dmrg_gb300.warmup import Lattice

    g = np.load(os.path.join(GOLDEN, f"sweep_{c}.npz"))
    sites = [(g[f"site{i}_desc"], g[f"site{i}_flag"], g[f"site{i}_x"]) for i in range(10)]
    return Lattice.from_tables(g["tables"], g["coup"], sites, float(g["qcoup"]), int(g["d"]))


_CACHE = {}


def _run(c, mode):
    from su2dmrg_gb300.sweep import Dmrg
    from su2dmrg_gb300.warmup import discarded_weight

    if (c, mode) not in _CACHE:
        d = Dmrg(_lattice(c), mode=mode)
        e, _ = d.run_dmrg(RUNS[c]["niter"])
        dw = {}  # site -> discarded weight of the last truncation that set its bond
        for il, ir, kept, w in d.truncations:
            dw[il] = dw[ir] = discarded_weight(kept, w)
        _CACHE[(c, mode)] = (e, [d.uu[i][0].desc().tolist() for i in range(d.lat.ns)], dw)
    return _CACHE[(c, mode)]


def _legs(desc):
    """[(dir, spins, dims)] per leg of a structure descriptor."""
    out, p = [], 2
    for _ in range(desc[0]):
        n = desc[p + 1]
        out.append((desc[p], desc[p + 2: p + 2 + n], desc[p + 2 + n: p + 2 + 2 * n]))
        p += 2 + 2 * n
    return out

@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("c", range(len(RUNS)))
def test_sweep_energy_matches_reference(torch_cuda, c, mode):
    e, _, _ = _run(c, mode)
    ref = RUNS[c]["energies_minus_1000"][-1] + 1000.0
    assert abs(e[-1] - ref) <= 1e-10 * abs(ref), (e, ref)


@pytest.mark.parametrize("c", range(len(RUNS)))
def test_sweep_retained_multiplets_match_reference(torch_cuda, c):
    _, descs, _ = _run(c, 0)
    ref = RUNS[c]["mps_desc"]
    assert len(descs) == len(ref)
    for i, (a, b) in enumerate(zip(descs, ref)):
        assert a == b, i


@pytest.mark.parametrize("c", range(len(RUNS)))
def test_split_sweep_matches_fp64(torch_cuda, c):
    """Split-precision contractions against the FP64 path: converged energies
    to 1e-10 relative, and per bond the same retained multiplets, sector by
    sector, or, where the two runs settled on different truncations of the
    same quality, the same total with discarded weights within 1e-10 (at
    D = 200 on 6x4 a 1e-16 change of the arithmetic moves one multiplet
    between sectors at one bond)."""
    e0, d0, w0 = _run(c, 0)
    e1, d1, w1 = _run(c, 1)
    assert abs(e1[-1] - e0[-1]) <= 1e-10 * abs(e0[-1])
    assert len(d0) == len(d1)
    for i, (a, b) in enumerate(zip(d0, d1)):
        if a == b:
            continue
        la, lb = _legs(a), _legs(b)
        assert [x[:2] for x in la] == [x[:2] for x in lb], i  # directions and sector spins
        for x, y in zip(la, lb):  # a bond whose multiplets differ (it is a leg of both its sites)
            if x[2] != y[2]:
                assert sum(x[2]) == sum(y[2]), i
                assert abs(w0[i] - w1[i]) <= 1e-10, (i, w0[i], w1[i])


@pytest.mark.parametrize("c", [1, 2])
def test_host_resident_blocks_change_nothing(torch_cuda, c):
    """Block tensors moved to host memory once the sweep has passed their
    position (the reference's memory_flag mode, with host memory for its
    files) and brought back when read: the same run, bit for bit, as with
    every tensor on the device, on a J1-J2 and a J-Q lattice (plaquette
    operators included)."""
    from su2dmrg_gb300.sweep import Dmrg

    lat = _lattice(c)
    res = []
    for offload in (False, True):
        d = Dmrg(lat, mode=1, seed=7)
        d.offload = offload
        d.run()
        moved = 0
        for _ in range(2):
            d.sweep()
            moved = max(moved, getattr(d, "host_bytes", 0))
        res.append((d, [e for _, _, e in d.energies], moved))
    (d0, e0, _), (d1, e1, moved) = res
    assert moved > 0
    assert e0 == e1
    for i in range(lat.ns):
        assert torch_cuda.equal(d0.uu[i][1], d1.uu[i][1])
