"""Host side of the serving loop: the seeded request stream and the footprint
estimate that admission uses."""
import numpy as np


def test_request_stream_is_seeded():
    from su2dmrg_gb300.serve import request_stream

    a = request_stream(16, 0.5, seed=42)
    b = request_stream(16, 0.5, seed=42)
    assert [r.meta for r in a] == [r.meta for r in b]
    assert [r.arrival for r in a] == [r.arrival for r in b]
    assert a[0].arrival == 0.0 and all(np.diff([r.arrival for r in a]) >= 0)
    for r in a:
        assert r.meta["D"] in (128, 256, 512) and r.meta["spin"] in (0, 1)
        assert r.lattice.totspin == 2 * r.meta["spin"]


def test_footprint_grows_with_d_and_lattice():
    from su2dmrg_gb300.serve import footprint_bytes
    from su2dmrg_gb300.warmup import Lattice

    f = lambda lx, ly, d: footprint_bytes(Lattice.cylinder(lx, ly, 2.0, 0.0, d))
    assert f(6, 4, 256) > f(6, 4, 128) > 0
    assert f(12, 6, 256) > f(6, 4, 256)
    assert f(12, 6, 512) < 2e9  # a serving request stays far below one GPU's HBM
