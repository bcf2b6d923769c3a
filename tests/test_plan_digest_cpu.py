"""The host planner pinned by digests of its work lists (FP64 and split
precision) for seeded synthetic H_eff plans and environment batches
(tests/golden/plan_digests.json, written by tests/golden/gen_plan_digests.py).
The lists fix the order of every sum the kernels form: a planner change that
moves any of them changes results bit for bit and fails here."""
import json
import os
import sys

import pytest

from conftest import GOLDEN

sys.path.insert(0, GOLDEN)
import gen_plan_digests as G  # noqa: E402

REF = json.load(open(os.path.join(GOLDEN, "plan_digests.json")))


@pytest.fixture
def default_tiles(su2lib):
    from su2dmrg_gb300 import autotune as A

    A.reset()
    yield
    A.load()


@pytest.mark.parametrize("case", G.HEFF, ids=lambda c: ",".join(map(str, c)))
def test_heff_plan_digests(default_tiles, case):
    want = REF["heff"][",".join(map(str, case))]
    for mode in (0, 1, 2):
        assert f"{G.heff_digest(case, mode):016x}" == want[str(mode)], mode


@pytest.mark.parametrize("case", G.ENV, ids=lambda c: ",".join(map(str, c)))
def test_env_batch_digests(default_tiles, case):
    want = REF["env"][",".join(map(str, case))]
    for mode in (0, 1, 2):
        assert f"{G.env_digest(case, mode):016x}" == want[str(mode)], mode


def test_digest_sees_addresses_and_tile_table(default_tiles):
    """A different operand address or FP64 tile class changes the digest; the
    split lists do not depend on the FP64 tile table."""
    from su2dmrg_gb300 import autotune as A
    from su2dmrg_gb300.su2 import HeffPlan
    from su2dmrg_gb300.workloads import synthetic_heff

    w = synthetic_heff(D=60, nspin1=2, seed=5)
    terms = [(s1, G.Addr(1 << 40), s2, G.Addr(2 << 40), c) for (s1, _a, s2, _b, c) in w.terms]
    moved = [(s1, G.Addr(1 << 40), s2, G.Addr(3 << 40), c) for (s1, _a, s2, _b, c) in w.terms]
    base = {m: HeffPlan.digest(w.psi, terms, mode=m) for m in (0, 1)}
    assert HeffPlan.digest(w.psi, moved, mode=0) != base[0]
    A.install({"m_edges": [], "n_edges": [], "cls": [3]})  # 32 x 32 tiles everywhere
    assert HeffPlan.digest(w.psi, terms, mode=0) != base[0]
    assert HeffPlan.digest(w.psi, terms, mode=1) == base[1]
