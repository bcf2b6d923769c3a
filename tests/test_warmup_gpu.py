"""The warm-up of a run (dmrg_su2::do_idmrg) with every tensor on the device
(su2dmrg_gb300.warmup over the C ABI), against the reference engine's own
warm-up on the same lattices (tests/golden/warmup_*.npz: J1 4x2 at D=16,
J1-J2 6x2 and J-Q 4x4 at D=24), and the fuse tensors (tensor_su2::fuse)
bit-exact.

Each warm-up Lanczos starts from the uniform vector in the current MPS basis,
so the path depends on the signs of the singular vectors of every earlier
truncation and of the Lanczos eigenvector, which LAPACK leaves free.  The
fixtures come from the reference built with the eigenvector sign rule of the
device engine (the first entry above 1e-4 of a column's largest is positive,
applied in the reference build's dsyev/dstev), which removes that freedom."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda(su2lib):
    import torch

    assert torch.cuda.is_available()
    return torch


def lattice(g):
    from su2dmrg_gb300.warmup import Lattice

    sites = [(g[f"site{i}_desc"], g[f"site{i}_flag"], g[f"site{i}_x"]) for i in range(10)]
    return Lattice.from_tables(g["tables"], g["coup"], sites, float(g["qcoup"]), int(g["d"]))


def test_fuse_tensor_matches_reference(torch_cuda):
    from su2dmrg_gb300 import su2 as S

    g = np.load(os.path.join(GOLDEN, "fuse_tensor.npz"))
    for i in range(2):
        b = S._parse_desc(g[f"bonds{i}"]).bonds
        s, x = S.fuse_tensor(b[0], b[1])
        assert s.desc().tolist() == g[f"desc{i}"].tolist() and s.flag.tolist() == g[f"flag{i}"].tolist()
        assert np.array_equal(x[: s.size()].cpu().numpy(), g[f"x{i}"])


def _ed_ground(sites, bonds):
    """Lowest eigenvalue of sum_b J_b S_i.S_k (spin 1/2) on the given sites."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla

    idx = {s: q for q, s in enumerate(sites)}
    N = 1 << len(sites)
    st = np.arange(N)
    diag = np.zeros(N)
    rows, cols, vals = [st], [st], []
    for (a, b), c in bonds.items():
        if a in idx and b in idx:
            sa, sb = (st >> idx[a]) & 1, (st >> idx[b]) & 1
            diag += c * np.where(sa == sb, 0.25, -0.25)
            m = sa != sb
            rows.append(st[m] ^ ((1 << idx[a]) | (1 << idx[b])))
            cols.append(st[m])
            vals.append(np.full(m.sum(), 0.5 * c))
    H = sp.csr_matrix((np.concatenate([diag] + vals), (np.concatenate(rows), np.concatenate(cols))), shape=(N, N))
    return float(sla.eigsh(H, k=1, which="SA")[0][0])


def _steps(w):
    return np.array([ev for _, _, ev in w.energies])


@pytest.mark.parametrize("mode", [0, 1])
def test_warmup_matches_reference_4x2(torch_cuda, mode):
    """J1 4x2 at D=16 with the engine's five Lanczos vectors: the eigenvalue
    of every step to 1e-10 relative and the last truncation's singular values
    above 1e-6 of the largest to 1e-8.  D does not bind here, so the
    truncation keeps every positive Gram eigenvalue above 1e-100 of the
    largest, rounding-noise ones included (around 1e-9 as singular values):
    how many of those there are depends on the GEMM's summation order, so
    they are not compared."""
    from su2dmrg_gb300.warmup import Warmup

    g = np.load(os.path.join(GOLDEN, "warmup_0.npz"))
    w = Warmup(lattice(g), mode=mode, mlanc=int(g["mlanc"]))
    e = w.run()
    assert abs(e - g["energy"]) <= 1e-10 * abs(g["energy"])
    assert np.allclose(_steps(w), g["step_energies"], rtol=1e-10, atol=0)
    big = lambda v: np.sort(v[v > 1e-6 * np.max(v)])
    assert np.allclose(big(np.asarray(w.ww)), big(g["ww"]), rtol=0, atol=1e-8)


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("case,exact_steps", [(1, 2), (2, 3)])
def test_warmup_larger_lattices(torch_cuda, case, exact_steps, mode):
    """J1-J2 6x2 and J-Q 4x4 at D=24, both engines with 40 Lanczos vectors.
    The steps before the first truncation to a rank-deficient Schmidt basis
    match the reference's eigenvalues to 1e-7 relative (the Lanczos overlap
    test stops at |ov - 1| < 1e-8, so converged eigenvalues agree to about
    that).  After it the reference's basis holds every Schmidt vector above
    1e-100 of the largest (tensor.cpp:1533), rounding-noise directions
    included, and the H_eff of later steps is a compression onto a
    noise-chosen subspace (the FP64 and split engines differ there as much as
    either differs from the reference); each step is then checked against the
    exact ground energy of its sites' Hamiltonian, the variational bound
    every compression satisfies (6x2, whose Hamiltonian is the table's
    Heisenberg bonds), and to be finite."""
    from su2dmrg_gb300.warmup import Warmup

    g = np.load(os.path.join(GOLDEN, f"warmup_{case}.npz"))
    lat = lattice(g)
    w = Warmup(lat, mode=mode, mlanc=int(g["mlanc"]))
    w.run()
    steps, ref = _steps(w), g["step_energies"]
    assert len(steps) == len(ref) and np.all(np.isfinite(steps))
    assert np.allclose(steps[:exact_steps], ref[:exact_steps], rtol=1e-7, atol=0)
    ww = np.asarray(w.ww)
    assert np.all(ww >= 0) and np.sum(ww**2) <= 1 + 1e-10  # kept weight of a unit vector
    if float(g["qcoup"]) == 0:
        ns = lat.ns
        bonds = {(a, b): float(lat.coup[lat.hmap[a][b]]) for a in range(ns) for b in range(a + 1, ns)
                 if lat.hmap[a][b] > 0}
        for il, ir, ev in w.energies:
            e0 = _ed_ground(list(range(il + 1)) + list(range(ir, ns)), bonds)
            assert ev >= e0 - 1e-9 * abs(e0), (il, ev, e0)
