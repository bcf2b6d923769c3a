"""The serving loop (su2dmrg_gb300.serve): independent DMRG solves admitted by
device footprint, run concurrently on their own streams, with their Lanczos
solves batched into shared launches.  Every solve's result must be the same
in the mix as alone: energies after the warm-up and after every sweep within
1e-10 relative, and the retained multiplets at every bond identical.  (Run
one after another, batched or not, the solves are bit-identical: the
batched Lanczos returns per solve what su2g_lanczos returns.  When other
solves share the GPU at the same time, the truncation's library GEMMs and
eigensolvers may sum in another order; the energies then move by about
1e-13 relative.)  Admission must respect the HBM budget."""
import pytest

pytestmark = pytest.mark.gpu


def _requests():
    from su2dmrg_gb300.serve import Request, couplings
    from su2dmrg_gb300.warmup import Lattice

    specs = [  # lx, ly, J2/J1, Q/J1, 2S, D
        (4, 2, 0.5, 0.0, 0, 16),
        (3, 4, 0.0, 1.0, 0, 32),
        (6, 2, 0.5, 0.3, 0, 24),
        (4, 4, 0.2, 0.0, 2, 32),
        (6, 4, 0.5, 0.0, 0, 48),
    ]
    out = []
    for k, (lx, ly, r, q, s2, d) in enumerate(specs):
        delta, qd = couplings(r, q)
        out.append(Request(k, Lattice.cylinder(lx, ly, delta, qd, d, totspin=s2), niter=3, arrival=0.0,
                           meta={"lattice": f"{lx}x{ly}"}))
    return out


@pytest.fixture(scope="module")
def alone(su2lib):
    """Each request solved on its own, through the plain per-solve path."""
    import torch

    from su2dmrg_gb300.sweep import Dmrg

    out = {}
    for r in _requests():
        d = Dmrg(r.lattice, mode=1)
        e, _ = d.run_dmrg(r.niter)
        torch.cuda.synchronize()
        out[r.rid] = (e, [d.uu[i][0].desc().tolist() for i in range(d.lat.ns)])
    return out


def test_mix_equals_alone(alone):
    from su2dmrg_gb300.serve import Server

    srv = Server(slots=5, mode=1, batch=True, window_s=0.01)
    res = srv.run(_requests())
    assert srv.max_inflight >= 2  # the solves did overlap
    assert max(srv.batch_sizes) >= 2  # and shared Lanczos launches
    for r in res:
        e, descs = alone[r.rid]
        assert len(r.energies) == len(e)
        assert all(abs(a - b) <= 1e-10 * abs(b) for a, b in zip(r.energies, e)), (r.rid, r.energies, e)
        assert r.mps_desc == descs, r.rid


def test_admission_respects_the_budget(alone):
    from su2dmrg_gb300.serve import Server, footprint_bytes

    reqs = _requests()
    fps = sorted(footprint_bytes(r.lattice) for r in reqs)
    budget = fps[-1] + fps[-2] - 1  # the two largest never run together
    srv = Server(slots=5, hbm_budget=budget, mode=1, batch=True, window_s=0.002)
    res = srv.run(reqs)
    assert srv.max_reserved <= budget
    for r in res:
        e = alone[r.rid][0]
        assert all(abs(a - b) <= 1e-10 * abs(b) for a, b in zip(r.energies, e))
        assert r.t_admit >= r.t_arrive
