"""DMRG sweeps with every tensor on the device (su2dmrg_gb300.sweep: the
warm-up, then dmrg_su2::sweep until a sweep changes the energy by less than
1e-6, as main_omp does) against whole runs of the reference engine
(tests/golden/dmrg_energies.json: J1-J2 4x2 and 3x4 and J-Q 3x4 at D=64, J1-J2
6x4 with J2/J1 = 2 at D=200; lattice tables in tests/golden/sweep_*.npz).

The warm-up's path follows rounding noise (tests/test_warmup_gpu.py), but
the sweeps converge to the same state: the converged energy in FP64 and in
split precision is the reference's to 1e-10 relative, and the final MPS has
the reference's retained multiplets, sector by sector, at every bond."""
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

    if (c, mode) not in _CACHE:
        d = Dmrg(_lattice(c), mode=mode)
        e, _ = d.run_dmrg(RUNS[c]["niter"])
        _CACHE[(c, mode)] = (e, [d.uu[i][0].desc().tolist() for i in range(d.lat.ns)])
    return _CACHE[(c, mode)]


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("c", range(len(RUNS)))
def test_sweep_energy_matches_reference(torch_cuda, c, mode):
    e, _ = _run(c, mode)
    ref = RUNS[c]["energies_minus_1000"][-1] + 1000.0
    assert abs(e[-1] - ref) <= 1e-10 * abs(ref), (e, ref)


@pytest.mark.parametrize("c", range(len(RUNS)))
def test_sweep_retained_multiplets_match_reference(torch_cuda, c):
    _, descs = _run(c, 0)
    ref = RUNS[c]["mps_desc"]
    assert len(descs) == len(ref)
    for i, (a, b) in enumerate(zip(descs, ref)):
        assert a == b, i


@pytest.mark.parametrize("c", range(len(RUNS)))
def test_split_sweep_matches_fp64(torch_cuda, c):
    """Split-precision contractions against the FP64 path: converged energies
    to 1e-10 relative and the same retained multiplets."""
    e0, d0 = _run(c, 0)
    e1, d1 = _run(c, 1)
    assert abs(e1[-1] - e0[-1]) <= 1e-10 * abs(e0[-1])
    assert d1 == d0
