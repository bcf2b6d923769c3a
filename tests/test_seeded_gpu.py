"""The seeded random start (the -seed option added on both sides: the
warm-up's two-site steps start from tensor_su2::random_initialize_tensor
with the ran() generator seeded once, tensor_su2.cpp:2375-2393, ran.f90).
su2g_random_vector must draw the reference generator's numbers (the state
after n draws equal, values equal to the oracle's to rounding of the norm),
and whole device runs from the same seed must reach the reference's seeded
runs (tests/golden/dmrg_seeded.json, among them the 6x4 J1-J2 D=200 run of 4
sweeps): converged energy within 1e-10 relative in FP64 and split precision,
and the reference's retained multiplets at every bond (FP64)."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
SEEDED = json.load(open(os.path.join(GOLDEN, "dmrg_seeded.json")))


@pytest.mark.parametrize("n", [1, 37, 1000, 300001])
def test_random_vector_draws_the_reference_generator(su2lib, oracle, n):
    import torch

    from su2dmrg_gb300 import su2 as S

    x = torch.empty(n, dtype=torch.float64, device="cuda")
    st = S.random_vector(x, 1234)
    if n <= 1000:
        want, raw, st_or = oracle.random_vector(1234, n)
        assert st == st_or
        assert np.max(np.abs(x.cpu().numpy() - want)) <= 1e-15 * np.max(np.abs(want))
    # continuing the stream: two calls equal one call of the summed length
    y = torch.empty(n + 5, dtype=torch.float64, device="cuda")
    st2 = S.random_vector(y, 1234)
    z = torch.empty(5, dtype=torch.float64, device="cuda")
    assert S.random_vector(z, st) == st2


_CACHE = {}


def _run(c, mode):
    from su2dmrg_gb300.sweep import Dmrg
    from su2dmrg_gb300.warmup import Lattice

    if (c, mode) not in _CACHE:
        r = SEEDED["runs"][c]
        lat = Lattice.cylinder(r["lx"], r["ly"], r["jcoup"], r["qcoup"], r["d"], r["boundary"], totspin=r["sec"])
        d = Dmrg(lat, mode=mode, seed=r["seed"])
        e, _ = d.run_dmrg(r["niter"])
        _CACHE[(c, mode)] = (e, [d.uu[i][0].desc().tolist() for i in range(lat.ns)])
    return _CACHE[(c, mode)]


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("c", range(len(SEEDED["runs"])))
def test_seeded_run_energy_matches_reference(su2lib, c, mode):
    e, _ = _run(c, mode)
    ref = SEEDED["runs"][c]["energies_minus_1000"][-1] + 1000.0
    assert abs(e[-1] - ref) <= 1e-10 * abs(ref), (e, ref)


@pytest.mark.parametrize("c", range(len(SEEDED["runs"])))
def test_seeded_run_retained_multiplets_match_reference(su2lib, c):
    _, descs = _run(c, 0)
    ref = SEEDED["runs"][c]["mps_desc"]
    assert descs == ref
