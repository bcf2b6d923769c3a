"""Seeded synthetic H_eff workloads of the named benchmark shapes.

The reference publishes no benchmark inputs, so the microbenchmark is a
synthetic two-site effective Hamiltonian with the shapes of a D-multiplet
SU(2) DMRG step on a spin-1/2 lattice:

* bond sectors 2j = 0..12 with multiplet counts from a discretised Gaussian in
  j (mean 2, sd 1.5), rounded by largest remainder to exactly D multiplets
  (D = 2000 gives 117,173,229,270,285,270,229,173,117,71,39,19,8);
* the enlarged legs are bond (x) spin-1/2 (su2bond::fuse);
* psi is a 2-leg singlet (blocks (j,j)), i.i.d. N(0,1) entries, normalised;
* `nspin1` spin-1 operator pairs (L_t, R_t) (3 legs: in, operator spin 2j=2
  with multiplicity 1, out) plus the two spin-0 block Hamiltonians H_L, H_R:
  width = nspin1 + 2 (18 + 2 = 20 for the headline shape);
* operator entries are N(0,1) scaled by 1/sqrt(rows).  The operator blocks are
  tied so that H_eff is symmetric (L_t(j'->j) = L_t(j->j')^T and R_t's
  counterpart carries the recoupling ratio), which the Lanczos solver needs.

Random numbers come from numpy's PCG64 seeded generator; the same seed gives
the same workload on every host.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .su2 import Su2Bond, Su2Struct, fac_hamilt_vec


def gaussian_sector_counts(total: int, max2j: int = 12, mean_j: float = 2.0, sd_j: float = 1.5):
    """Multiplet counts per 2j in 0..max2j, largest-remainder rounding."""
    j = np.arange(max2j + 1) / 2.0
    w = np.exp(-0.5 * ((j - mean_j) / sd_j) ** 2)
    raw = w / w.sum() * total
    base = np.floor(raw).astype(int)
    rem = total - base.sum()
    order = np.argsort(-(raw - base), kind="stable")
    base[order[:rem]] += 1
    return base.tolist()


@dataclass
class HeffWorkload:
    psi: Su2Struct
    psi_data: np.ndarray
    terms: list  # [(Su2Struct, np.ndarray, Su2Struct, np.ndarray, coef)]
    hl: tuple    # (Su2Struct, np.ndarray, coef)
    hr: tuple
    D: int

    def to_device(self, device="cuda"):
        import torch

        t = lambda a: torch.from_numpy(a).to(device)
        terms = [(s1, t(x1), s2, t(x2), c) for (s1, x1, s2, x2, c) in self.terms]
        hl = (self.hl[0], t(self.hl[1]), self.hl[2]) if self.hl is not None else None
        hr = (self.hr[0], t(self.hr[1]), self.hr[2]) if self.hr is not None else None
        return t(self.psi_data), terms, hl, hr


def _spin_half():
    return Su2Bond(1, [1], [1])


def _fill_operator(struct: Su2Struct, rng, fac, ratio_side: bool):
    """Operator data with the symmetry that makes H_eff symmetric.

    For blocks (j, s, j') and (j', s, j): the first is drawn, the second is its
    transpose; on the right-hand operator the transpose is scaled by
    fac[j][s][j'] / fac[j'][s][j].  Diagonal blocks are symmetrised."""
    off, total = struct.offsets()
    data = np.zeros(total)
    idx = {}
    for i in range(struct.nten):
        if struct.flag[i]:
            idx[struct.block_angm(i)] = i
    for key, i in idx.items():
        ja, s, jc = key
        a, ms, c = struct.block_shape(i)
        if ja > jc:
            continue
        blk = rng.standard_normal((a, c)) / np.sqrt(a)
        if ja == jc:
            blk = 0.5 * (blk + blk.T)
        data[off[i]: off[i] + a * c] = blk.ravel(order="F")
        if ja != jc and (jc, s, ja) in idx:
            i2 = idx[(jc, s, ja)]
            t = blk.T.copy()
            if ratio_side:
                t *= fac[ja, s, jc] / fac[jc, s, ja]
            data[off[i2]: off[i2] + a * c] = t.ravel(order="F")
    return data


def synthetic_heff(D: int = 2000, nspin1: int = 18, seed: int = 1234, max2j: int = 12,
                   spin0: bool = True) -> HeffWorkload:
    rng = np.random.Generator(np.random.PCG64(seed))
    counts = gaussian_sector_counts(D, max2j)
    angm = [k for k in range(max2j + 1) if counts[k] > 0]
    bond = Su2Bond(1, angm, [counts[k] for k in angm])
    enl = bond.fuse(_spin_half())  # direction -1
    enl.dir = -1
    psi = Su2Struct([enl, enl], 0).with_legal_flags()
    off, total = psi.offsets()
    x = np.zeros(total)
    for i in range(psi.nten):
        if psi.flag[i]:
            a, b = psi.block_shape(i)
            x[off[i]: off[i] + a * b] = rng.standard_normal(a * b)
    x /= np.linalg.norm(x)

    fac = fac_hamilt_vec(25)
    spin = Su2Bond(1, [2], [1])
    inb = enl.inverted()
    terms = []
    for t in range(nspin1):
        s1 = Su2Struct([inb, spin, enl], 0).with_legal_flags()
        s2 = Su2Struct([inb, spin, enl], 0).with_legal_flags()
        x1 = _fill_operator(s1, rng, fac, ratio_side=False)
        x2 = _fill_operator(s2, rng, fac, ratio_side=True)
        terms.append((s1, x1, s2, x2, 1.0))
    hl = hr = None
    if spin0:
        hs = Su2Struct([inb, enl], 0).with_legal_flags()
        hoff, htot = hs.offsets()
        hx = [np.zeros(htot), np.zeros(htot)]
        for side in range(2):
            for i in range(hs.nten):
                if hs.flag[i]:
                    a, c = hs.block_shape(i)
                    blk = rng.standard_normal((a, c)) / np.sqrt(a)
                    blk = 0.5 * (blk + blk.T)
                    hx[side][hoff[i]: hoff[i] + a * c] = blk.ravel(order="F")
        hl = (hs, hx[0], 1.0)
        hr = (hs, hx[1], 1.0)
    return HeffWorkload(psi, x, terms, hl, hr, D)


@dataclass
class SiteStepWorkload:
    """The tensors around one two-site step at bond dimension D (same sector
    counts as synthetic_heff): the MPS pair (ul, ur) whose product is the
    step's initial vector, and an environment batch (uu = vv, operators,
    block Hamiltonian) of the site update that follows."""
    ul: tuple   # (Su2Struct, data): (bond +1, spin-1/2, centre bond -1)
    ur: tuple   # (spin-1/2, bond +1, centre bond -1)
    uu: tuple   # (bond -1, spin-1/2, new bond +1)
    ops: list   # [(Su2Struct, data)]: (bond +1, spin 1 (-1), bond -1)
    hh: tuple   # (bond +1, bond -1) block Hamiltonian
    D: int


def synthetic_site_step(D: int = 2000, nops: int = 18, seed: int = 4321, max2j: int = 12) -> SiteStepWorkload:
    rng = np.random.Generator(np.random.PCG64(seed))
    counts = gaussian_sector_counts(D, max2j)
    angm = [k for k in range(max2j + 1) if counts[k] > 0]
    dims = [counts[k] for k in angm]
    b = lambda d: Su2Bond(d, list(angm), list(dims))
    ph = _spin_half()

    def fill(struct):
        s = struct.with_legal_flags()
        off, tot = s.offsets()
        x = np.zeros(tot)
        for i in range(s.nten):
            if s.flag[i]:
                shape = s.block_shape(i)
                n = int(np.prod(shape))
                x[off[i]: off[i] + n] = rng.standard_normal(n) / np.sqrt(max(1, shape[0]))
        return s, x

    ul = fill(Su2Struct([b(1), ph, b(-1)], 0))
    ur = fill(Su2Struct([ph, b(1), b(-1)], 0))
    uu = fill(Su2Struct([b(-1), ph, b(1)], 0))
    spin = Su2Bond(-1, [2], [1])
    ops = [fill(Su2Struct([b(1), spin, b(-1)], 0)) for _ in range(nops)]
    hh = fill(Su2Struct([b(1), b(-1)], 0))
    return SiteStepWorkload(ul, ur, uu, ops, hh, D)
