"""Output structures of an environment batch (su2g_env_layout, host only):
the batched form used per site update equals one call per slot."""


def test_batched_layouts_equal_per_slot_layouts(su2lib):
    from su2dmrg_gb300 import su2 as S
    from su2dmrg_gb300.workloads import synthetic_site_step

    w = synthetic_site_step(D=120, nops=5, seed=3)
    su, du = w.uu
    jobs = [{"kind": "transform", "slot": i, "coef": 1.0, "x": (s_, x_)} for i, (s_, x_) in enumerate(w.ops)]
    jobs.append({"kind": "overlap", "slot": len(w.ops), "coef": 1.0, "x": (w.hh[0], w.hh[1])})
    jobs.append({"kind": "transform", "slot": 0, "coef": -0.5, "x": w.ops[0]})  # a shared slot
    n = len(w.ops) + 1
    batched = S.env_layouts(su, du, su, du, 0, jobs, range(n))
    assert len(batched) == n
    for s in range(n):
        one = S.env_layout(su, du, su, du, 0, jobs, s)
        assert one.desc().tolist() == batched[s].desc().tolist()
        assert one.flag.tolist() == batched[s].flag.tolist()
        assert one.size() > 0
