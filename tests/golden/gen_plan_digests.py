"""Digests of the work lists the library's host planner builds (FP64 and
split precision) for seeded synthetic H_eff plans and environment batches:
tests/golden/plan_digests.json.

The lists fix the order of every sum the kernels form, so a planner change
that alters any of them changes results bit for bit; tests/test_plan_digest_cpu.py
recomputes these digests.  They pin the planner against itself (the
reference has no such lists), not against the reference.  Operand addresses
enter a digest, so every tensor gets a fixed stand-in address here (the host
planner never dereferences device data).  The FP64 tile table is reset to
its default (64 x 64 everywhere) while digesting.

    python tests/golden/gen_plan_digests.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


class Addr:
    """A stand-in device address (the planner reads addresses, never data)."""

    def __init__(self, a):
        self.a = a

    def data_ptr(self):
        return self.a


def _addresses():
    state = {"n": 0}

    def nxt():
        state["n"] += 1
        return Addr((1 << 40) + state["n"] * (1 << 34))

    return nxt


HEFF = [  # (D, nspin1, seed, max2j, spin0)
    (8, 0, 1, 2, False), (30, 0, 1, 12, False), (40, 1, 51, 12, False), (60, 4, 71, 12, True),
    (150, 3, 9, 12, True), (300, 3, 311, 12, True), (777, 2, 788, 12, True), (2000, 18, 1234, 12, True),
    (8, 1100, 3, 2, False),
]
ENV = [  # (D, nops, seed, max2j)
    (40, 2, 3, 6), (120, 5, 3, 12), (500, 4, 7, 12), (2000, 18, 4321, 12),
]


def heff_digest(case, mode):
    from su2dmrg_gb300.su2 import HeffPlan
    from su2dmrg_gb300.workloads import synthetic_heff

    D, n, seed, m2j, spin0 = case
    w = synthetic_heff(D=D, nspin1=n, seed=seed, max2j=m2j, spin0=spin0)
    nxt = _addresses()
    terms = [(s1, nxt(), s2, nxt(), c) for (s1, _x1, s2, _x2, c) in w.terms]
    hl = (w.hl[0], nxt(), w.hl[2]) if w.hl is not None else None
    hr = (w.hr[0], nxt(), w.hr[2]) if w.hr is not None else None
    return HeffPlan.digest(w.psi, terms, hl, hr, mode=mode)


def env_digest(case, mode):
    from su2dmrg_gb300 import su2 as S
    from su2dmrg_gb300.workloads import synthetic_site_step

    D, nops, seed, m2j = case
    w = synthetic_site_step(D=D, nops=nops, seed=seed, max2j=m2j)
    nxt = _addresses()
    u = nxt()
    jobs = [{"kind": "transform", "slot": i, "coef": 1.0 + 0.25 * i, "x": (s, nxt())} for i, (s, _x) in enumerate(w.ops)]
    jobs.append({"kind": "overlap", "slot": len(w.ops), "coef": 1.0, "x": (w.hh[0], nxt())})
    jobs.append({"kind": "transform", "slot": 0, "coef": -0.5, "x": (w.ops[0][0], nxt())})  # a shared slot
    outs = [nxt() for _ in range(len(w.ops) + 1)]
    return S.env_digest(w.uu[0], u, w.uu[0], u, 0, jobs, outs, mode=mode)


def compute():
    from su2dmrg_gb300 import autotune as A

    A.reset()
    try:
        out = {"heff": {}, "env": {}}
        for case in HEFF:
            out["heff"][",".join(map(str, case))] = {str(m): f"{heff_digest(case, m):016x}" for m in (0, 1, 2)}
        for case in ENV:
            out["env"][",".join(map(str, case))] = {str(m): f"{env_digest(case, m):016x}" for m in (0, 1, 2)}
        return out
    finally:
        A.load()


if __name__ == "__main__":
    with open(os.path.join(HERE, "plan_digests.json"), "w") as f:
        json.dump(compute(), f, indent=1, sort_keys=True)
        f.write("\n")
