"""Host-resident block tensors of the warm-up and sweep driver (Warmup.offload,
the reference's memory_flag mode with host memory for its files), on the host
alone: which slots of a position move, the cap on the bytes held by the host,
and the guard that keeps a host tensor from reaching the library."""
import os

import numpy as np
import pytest

from conftest import GOLDEN


class _FakeDeviceTensor:
    """Stands in for a device tensor: moves between 'cuda' and 'cpu' by .to()."""

    def __init__(self, n, where="cuda"):
        self.n, self.where = n, where

    @property
    def is_cuda(self):
        return self.where == "cuda"

    @property
    def device(self):
        return "cuda"

    def numel(self):
        return self.n

    def element_size(self):
        return 8

    def to(self, where):
        return _FakeDeviceTensor(self.n, "cpu" if str(where) == "cpu" else "cuda")

    def clone(self):
        return _FakeDeviceTensor(self.n, self.where)


def _warmup():
    from su2dmrg_gb300.warmup import Lattice, Warmup

    g = np.load(os.path.join(GOLDEN, "sweep_2.npz"))
    sites = [(g[f"site{i}_desc"], g[f"site{i}_flag"], g[f"site{i}_x"]) for i in range(10)]
    lat = Lattice.from_tables(g["tables"], g["coup"], sites, float(g["qcoup"]), int(g["d"]))
    return Warmup(lat)


def test_position_moves_out_and_back():
    w = _warmup()
    w.offload = True
    p = 5
    w.opr[p][3] = ("s", _FakeDeviceTensor(100))
    w.plq[p][w.lat.ns + 1] = ("s", _FakeDeviceTensor(50))
    w.hh[p] = ("s", _FakeDeviceTensor(20))
    w.opr[p + 1][3] = ("s", _FakeDeviceTensor(7))  # another position: untouched
    w._evict(p)
    assert not w.opr[p][3][1].is_cuda and not w.plq[p][w.lat.ns + 1][1].is_cuda and not w.hh[p][1].is_cuda
    assert w.opr[p + 1][3][1].is_cuda
    assert w.host_bytes == 8 * 170
    w._fetch(p)
    assert w.opr[p][3][1].is_cuda and w.plq[p][w.lat.ns + 1][1].is_cuda and w.hh[p][1].is_cuda
    assert w.host_bytes == 0


def test_host_cap_keeps_tensors_on_the_device():
    w = _warmup()
    w.offload = True
    w.host_fraction = 0.0
    w.opr[2][1] = ("s", _FakeDeviceTensor(10))
    w._evict(2)
    assert w.opr[2][1][1].is_cuda and w.host_bytes == 0


def test_off_by_default_and_out_of_range_positions():
    w = _warmup()
    w.opr[2][1] = ("s", _FakeDeviceTensor(10))
    w._evict(2)
    assert w.opr[2][1][1].is_cuda
    w.offload = True
    w._evict(-1)
    w._evict(w.lat.ns)
    w._fetch(w.lat.ns + 3)


def test_host_tensor_never_reaches_the_library():
    import torch

    from su2dmrg_gb300 import su2 as S

    st = S.Su2Struct([S.Su2Bond(1, [0], [1]), S.Su2Bond(-1, [0], [1])], 0).with_legal_flags()
    with pytest.raises(ValueError):
        S._tensor(st, torch.zeros(1, dtype=torch.float64), [])
    S._tensor(st, np.zeros(1), [])  # one-site operators travel as numpy host data


def test_refused_allocation_is_retried_once_after_freeing_the_cache():
    from su2dmrg_gb300 import capi
    from su2dmrg_gb300.warmup import Warmup

    calls = []

    def refused_once(x):
        calls.append(x)
        if len(calls) == 1:
            raise capi.Su2gError(capi.SU2G_ENOMEM, "pool allocation refused")
        return x + 1

    assert Warmup._freeing(refused_once, 4) == 5 and calls == [4, 4]

    def invalid(x):
        raise capi.Su2gError(capi.SU2G_EINVAL, "bad arguments")

    with pytest.raises(capi.Su2gError):
        Warmup._freeing(invalid, 1)

    def always_refused(x):
        raise capi.Su2gError(capi.SU2G_ENOMEM, "pool allocation refused")

    with pytest.raises(capi.Su2gError):
        Warmup._freeing(always_refused, 1)


def test_released_host_tensors_leave_the_host_count():
    w = _warmup()
    w.offload = True
    L = w.lat
    p = 4
    ks = [k for k in range(L.ns) if L.fll[p][k] == 1]
    assert ks
    for k in ks:
        w.opr[p][k] = ("s", _FakeDeviceTensor(10))
    w.hh[p] = ("s", _FakeDeviceTensor(5))
    w._evict(p)
    assert w.host_bytes == 8 * (10 * len(ks) + 5)
    w._release(p, 0)
    assert w.host_bytes == 0 and w.hh[p] is None and all(w.opr[p][k] is None for k in ks)


def test_replaced_host_tensors_leave_the_host_count():
    w = _warmup()
    w.offload = True
    w.opr[3][1] = ("s", _FakeDeviceTensor(10))
    w._evict(3)
    assert w.host_bytes == 80
    w._put(w.opr[3], 1, ("s", _FakeDeviceTensor(4)))  # a site update's new result
    assert w.host_bytes == 0 and w.opr[3][1][1].is_cuda


def test_clone_shares_the_host_budget():
    from su2dmrg_gb300.sweep import Dmrg

    w = _warmup()
    d = Dmrg(w.lat)
    d.offload = True
    d.opr[2][1] = ("s", _FakeDeviceTensor(10))
    d._evict(2)
    c = d.clone()
    assert not c.opr[2][1][1].is_cuda and c.offload
    assert d.host_bytes == c.host_bytes == 160  # the original's tensor and the clone's copy
    c._fetch(2)
    assert d.host_bytes == 80
