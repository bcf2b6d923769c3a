"""Warm-up of a DMRG run with every tensor on the device.

dmrg_su2::do_idmrg (dmrg_su2_omp.cpp:20-95) grows the MPS from both ends to
the centre: at each step the site operators of the two new sites are built
(prepare_site_operator_from_left / _right, :319-603 and :604-827), the two
new sites start as fuse tensors (tensor_su2::fuse), and once the block is
large enough the two-site ground state is found (Lanczos from the uniform
start vector, lanczos_solve_eigenvector_idmrg dmrg_su2.cpp:527-540) and
truncated (tensor_su2::svd).  This module drives that sequence over the C ABI
of libsu2g: MPS tensors, block Hamiltonians, site operators, plaquette
operators and the two-site vector stay in device memory from the first step
to the last; only structures, the engine's lattice tables and its one-site
operators (a few doubles) live on the host.

The lattice (hmap, coup, fll, frr, plqflg, plqpos) and the one-site
operators (sigma, qterm) are the engine's own tables (built by its
constructor and initialize_local_operators, dmrg_su2.cpp:31-300); they are
inputs here.  Only the ground state (exci = 0) is covered: the excited-state
overlaps (ovlp, orth) are not built.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np

from . import capi
from . import su2 as S


@dataclass
class Lattice:
    """The engine tables the warm-up reads (dmrg_su2.cpp:31-300)."""
    ns: int
    physpn: int
    totspin: int
    hmap: np.ndarray    # (ns, ns): index into coup of the coupling of sites (i, k), 0 = none
    coup: np.ndarray    # (ns,)
    fll: np.ndarray     # (ns, ns): opr[i][k] is carried to the left block at site i
    frr: np.ndarray     # (ns, ns): ... to the right block
    plqflg: np.ndarray  # (ns, ns): plaquette j passes site i
    plqpos: np.ndarray  # (ns, 4): the four sites of plaquette j
    qdelta: float
    sigma: list         # [(Su2Struct, host data)] x 2: the one-site spin operators
    qterm: list         # [(Su2Struct, host data)] x 8: the plaquette permutation operators
    max_dcut: int

    @classmethod
    def cylinder(cls, lx: int, ly: int, delta: float, qdelta: float, max_dcut: int, boundary: int = 2,
                 totspin: int = 0) -> "Lattice":
        """An lx x ly spin-1/2 cylinder built here (cylinder_tables), with the
        engine's spin-1/2 one-site operators (site_ops_spin_half.npz)."""
        hmap, coup, fll, frr, plqflg, plqpos = cylinder_tables(lx, ly, delta, qdelta, boundary)
        g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "site_ops_spin_half.npz"))
        ops = []
        for i in range(10):
            st = S._parse_desc(g[f"site{i}_desc"])
            st.flag = np.ascontiguousarray(g[f"site{i}_flag"], np.int32)
            ops.append((st, np.ascontiguousarray(g[f"site{i}_x"], np.float64)))
        return cls(lx * ly, 1, int(totspin), hmap, coup, fll, frr, plqflg, plqpos, float(qdelta), ops[:2], ops[2:10],
                   int(max_dcut))

    @classmethod
    def from_tables(cls, ints, coup, sites, qdelta: float, max_dcut: int) -> "Lattice":
        """From the flat layout [ns, physpn, totspin, hmap, fll, frr, plqflg
        (each ns x ns, row-major), plqpos (ns x 4)], coup[0..ns) and the ten
        one-site operators [sigma[0], sigma[1], qterm[0..8)] as (desc, flag,
        host data) (desc of length <= 2: never built)."""
        ints = np.asarray(ints)
        ns, q = int(ints[0]), 3
        mats = []
        for _ in range(4):
            mats.append(ints[q: q + ns * ns].reshape(ns, ns).copy())
            q += ns * ns
        plqpos = ints[q: q + 4 * ns].reshape(ns, 4).copy()
        ops = []
        for desc, flag, x in sites:
            if len(desc) <= 2:
                ops.append(None)
                continue
            st = S._parse_desc(desc)
            st.flag = np.ascontiguousarray(flag, np.int32)
            ops.append((st, np.ascontiguousarray(x, np.float64)))
        return cls(ns, int(ints[1]), int(ints[2]), mats[0], np.asarray(coup, np.float64), mats[1], mats[2], mats[3],
                   plqpos, float(qdelta), ops[:2], ops[2:10], int(max_dcut))


def _snake(x: int, y: int, ly: int) -> int:
    """Site index of column x, row y: columns in order, rows reversed in odd
    columns (dmrg_su2.cpp:174-177)."""
    return x * ly + (y if x % 2 == 0 else ly - 1 - y)


def cylinder_tables(lx: int, ly: int, delta: float, qdelta: float, boundary: int = 2):
    """The engine's lattice tables for an lx x ly cylinder (open in x, periodic
    in y), restated from the dmrg_su2 constructor (dmrg_su2.cpp:93-300):

      hmap[i][k]  coupling class of sites i, k (0 none, 1 nearest neighbour,
                  2 diagonal / next-nearest, 3 vertical bond on the open ends of
                  the boundary-2 lattice), for boundary 0 (square, periodic),
                  1 (J1-J3), 2 (J1-J2) and 3 (Shastry-Sutherland);
      coup[c]     delta + qdelta/2, 1 - |qdelta|, delta + qdelta/4 for c = 1, 2, 3;
      plqpos[m]   the four sites of the plaquette at column m/ly, row m%ly
                  (periodic in both directions), ascending;
      plqflg[i][m]  plaquette m spans site i (|qdelta| > 1e-5, not the last column);
      fll / frr   operators site i must carry for bonds and plaquettes that
                  cross it towards the right / left.

    Returns (hmap, coup, fll, frr, plqflg, plqpos) as numpy arrays."""
    ns = lx * ly
    hmap = np.zeros((ns, ns), np.int32)
    for k in range(5):
        for i in range(ns):
            x1 = i // ly
            y1 = i % ly if x1 % 2 == 0 else ly - 1 - (i % ly)
            nb = None
            if boundary == 0:
                if k == 0:
                    nb = ((x1 + 1) % lx, y1)
                elif k == 1:
                    nb = (x1, (y1 + 1) % ly)
            elif boundary == 2:
                nb = {0: (x1 + 1, y1), 1: (x1, (y1 + 1) % ly), 2: (x1 + 1, (y1 + 1) % ly),
                      3: (x1 - 1, (y1 + 1) % ly)}.get(k)
            elif boundary == 1:
                nb = {0: (x1 + 1, y1), 1: (x1, (y1 + 1) % ly), 2: (x1 + 2, y1), 3: (x1, (y1 + 2) % ly)}.get(k)
            elif boundary == 3:
                if k == 0:
                    nb = (x1 + 1, y1)
                elif k == 1:
                    nb = (x1, (y1 + 1) % ly)
                elif k == 2 and x1 % 2 == 0 and y1 % 2 == 0:
                    nb = (x1 + 1, (y1 + 1) % ly)
                elif k == 3 and x1 % 2 == 1 and y1 % 2 == 0:
                    nb = (x1 + 1, (y1 + ly - 1) % ly)
                elif k == 4 and (x1 == 0 or x1 == lx - 1):
                    nb = (x1 + 1, (y1 + 2) % ly)
            if nb is None:
                continue
            x2, y2 = nb
            if not (0 <= x2 < lx and 0 <= y2 < ly):
                continue
            j = _snake(x2, y2, ly)
            if boundary == 2 and k == 1 and (x1 == 0 or x1 == lx - 1):
                c = 3
            elif (boundary == 3 and k < 2) or (boundary in (1, 2) and 2 <= k < 4):
                c = 2
            elif (boundary == 3 and 2 <= k < 4) or (boundary in (0, 1, 2) and k < 2):
                c = 1
            else:
                continue
            hmap[i][j] = hmap[j][i] = c
    plqpos = np.zeros((ns, 4), np.int32)
    for m in range(ns):
        x1, y1 = m // ly, m % ly
        corners = [(x1, y1), (x1 % lx, (y1 + 1) % ly), ((x1 + 1) % lx, (y1 + 1) % ly), ((x1 + 1) % lx, y1)]
        plqpos[m] = sorted(_snake(x, y, ly) for x, y in corners)
    coup = np.zeros(max(ns, 4))
    coup[1] = delta + qdelta / 2.0
    coup[2] = 1.0 - abs(qdelta)
    coup[3] = delta + qdelta / 4.0
    plqflg = np.zeros((ns, ns), np.int32)
    if abs(qdelta) > 1e-5:
        for i in range(ns):
            for j in range(ns - ly):
                if plqpos[j][0] <= i <= plqpos[j][3]:
                    plqflg[i][j] = 1
    fll = np.zeros((ns, ns), np.int32)
    frr = np.zeros((ns, ns), np.int32)
    for i in range(ns):
        for j in range(i):
            if np.any(hmap[j, i + 1:] != 0):
                fll[i][j] = 1
        for j in range(ns):
            if plqflg[i][j] and plqpos[j][0] < i < plqpos[j][1]:
                fll[i][plqpos[j][0]] = 1
        for j in range(i + 1, ns):
            if np.any(hmap[j, :i] != 0):
                frr[i][j] = 1
        for j in range(ns):
            if plqflg[i][j] and plqpos[j][2] < i < plqpos[j][3]:
                frr[i][plqpos[j][3]] = 1
    return hmap, coup, fll, frr, plqflg, plqpos


@dataclass
class _Jobs:
    """One environment batch: jobs and their named output slots."""
    jobs: list = field(default_factory=list)
    names: list = field(default_factory=list)

    def add(self, name, kind, x=None, site1=None, site2=None, coef=1.0):
        if name not in self.names:
            self.names.append(name)
        j = {"kind": kind, "slot": self.names.index(name), "coef": coef, "x": x}
        if site1 is not None:
            j["site1"] = site1
        if site2 is not None:
            j["site2"] = site2
        self.jobs.append(j)


def discarded_weight(kept: int, w) -> float:
    """Discarded fraction of the squared singular values of one truncation
    (w: kept then discarded, as the svd returns them)."""
    w = np.asarray(w, np.float64)
    tot = float(np.sum(w * w))
    return float(np.sum(w[kept:] ** 2)) / tot if tot > 0 else 0.0


def host_available_bytes() -> int:
    """MemAvailable of the host (bytes), 0 when it cannot be read."""
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) * 1024
    except OSError:
        pass
    return 0


class Warmup:
    """do_idmrg on the device.  mode: capi.MODE_* for every contraction."""

    def __init__(self, lat: Lattice, mode: int = capi.MODE_F64, mlanc: int = 5, seed: int = None):
        self.lat, self.mode, self.mlanc = lat, mode, mlanc
        # seed: start every two-site step of the warm-up from a random vector
        # of the ran() generator (initran(seed), random_initialize_tensor)
        # instead of the uniform one; the stream continues across steps
        self.ran_state = None if seed is None else int(seed)
        ns = lat.ns
        self.uu = [None] * ns
        self.hh = [None] * ns
        self.opr = [[None] * ns for _ in range(ns)]
        self.plq = [[None] * (2 * ns) for _ in range(ns)]
        self.energies = []   # (il, ir, eigenvalue) per Lanczos step
        self.ww = None       # singular values of the last truncation
        self.truncations = []  # (il, ir, kept multiplets, singular values kept then discarded) per step
        self._keep = []

    # ---------------------------------------------------------- helpers
    @staticmethod
    def _freeing(f, *a, **k):
        """f(*a, **k); when the library's device pool is refused memory, the
        blocks torch keeps cached are returned to the device and f runs once
        more (the two allocators share the HBM; every call retried here
        leaves its inputs unchanged when it fails)."""
        try:
            return f(*a, **k)
        except capi.Su2gError as e:
            if e.code != capi.SU2G_ENOMEM:
                raise
            import torch

            torch.cuda.empty_cache()
            return f(*a, **k)

    def _run(self, u, flag, b: _Jobs):
        if not b.jobs:
            return {}
        res = self._freeing(S.env_batch, u[0], u[1], u[0], u[1], flag, b.jobs, mode=self.mode)
        return {name: (st, x[: st.size()]) for name, (st, x) in zip(b.names, res)}

    def _combine(self, lst):
        """sum c * op over [(op, c)], None when empty (tensor_su2 += of scaled copies)."""
        lst = [(t, c) for t, c in lst if t is not None]
        if not lst:
            return None
        if len(lst) == 1 and lst[0][1] == 1.0:
            return lst[0][0]
        r = S.operator_combine([t for t, _ in lst], [c for _, c in lst])
        return r[0], r[1][: r[0].size()]

    @staticmethod
    def _legs01(u):
        return u[0].bonds[0], u[0].bonds[1]

    # ------------------------------------------ host-resident block tensors
    # offload: the block tensors stored at a position (its site operators,
    # plaquette operators and block Hamiltonian) move to host memory once the
    # sweep has passed it and come back when a site update or an H_eff reads
    # them: the reference's memory_flag mode, which writes a position to disk
    # after the update next to it (save_memory + release_memory_all,
    # dmrg_su2_omp.cpp:449-450 and :591-592) and reads the one three sites
    # ahead before each update (read_memory, :341 and :482), with host memory
    # in place of files.  The bytes held on the host stay below host_fraction
    # of the memory the host had available at the first move; past that,
    # tensors stay on the device.
    offload = False
    host_fraction = 0.5

    @property
    def host_bytes(self) -> int:
        """Bytes of block tensors this run (and its clones) hold in host memory."""
        return self._host["used"] if hasattr(self, "_host") else 0

    def _position_slots(self, p: int):
        """(list, index) of every block tensor slot of position p."""
        ns = self.lat.ns
        return [(self.opr[p], k) for k in range(ns)] + [(self.plq[p], m) for m in range(2 * ns)] + [(self.hh, p)]

    def _fetch(self, p: int) -> None:
        """Brings the block tensors of position p to the device."""
        if not self.offload or p < 0 or p >= self.lat.ns:
            return
        for lst, k in self._position_slots(p):
            t = lst[k]
            if t is not None and not t[1].is_cuda:
                self._host["used"] -= t[1].numel() * t[1].element_size()
                lst[k] = (t[0], t[1].to(self._device))

    def _evict(self, p: int) -> None:
        """Moves the block tensors of position p to host memory (within the cap)."""
        if not self.offload or p < 0 or p >= self.lat.ns:
            return
        import torch

        if not hasattr(self, "_host"):  # shared with clones: one cap for all of them
            self._host = {"cap": int(self.host_fraction * host_available_bytes()), "used": 0}
        moved = 0
        for lst, k in self._position_slots(p):
            t = lst[k]
            if t is None or not t[1].is_cuda:
                continue
            nb = t[1].numel() * t[1].element_size()
            if self._host["used"] + nb > self._host["cap"]:
                continue
            self._device = t[1].device
            lst[k] = (t[0], t[1].to("cpu"))
            self._host["used"] += nb
            moved += nb
        if moved:
            torch.cuda.empty_cache()  # the freed blocks return to the device for the library's own pool

    def _release(self, p: int, lr: int) -> None:
        """release_memory2(p, lr) (dmrg_su2_omp.cpp:1804-1824), which the
        two-argument site updates call even without disk swap: the operators
        carried at site p towards the left (lr 0) or right (lr 1) end, its block
        Hamiltonian and its plaquette operators are emptied."""
        L = self.lat
        if p < 0 or p >= L.ns:
            return
        carry = L.fll if lr == 0 else L.frr
        for k in range(L.ns):
            if carry[p][k] == 1:
                self._drop(self.opr[p], k)
        self._drop(self.hh, p)
        for j in range(L.ns):
            if L.plqflg[p][j]:
                self._drop(self.plq[p], j)
                self._drop(self.plq[p], j + L.ns)

    def _put(self, lst, k: int, t) -> None:
        """Stores a block tensor in a slot (a host-resident one it replaces leaves the host count)."""
        self._drop(lst, k)
        lst[k] = t

    def _drop(self, lst, k: int) -> None:
        """Empties a block tensor slot (a host-resident tensor leaves the host count)."""
        t = lst[k]
        if t is not None and not t[1].is_cuda:
            self._host["used"] -= t[1].numel() * t[1].element_size()
        lst[k] = None

    # ---------------------------------------------------- site updates
    def site_left(self, i: int, u, release: bool = False):
        """prepare_site_operator_from_left(i[, flag]) with MPS tensor u at site
        i; release: the two-argument form, which first empties sites i+1 and
        i+2 (dmrg_su2_omp.cpp:338-339)."""
        L, p = self.lat, self.lat.plqpos
        if i == 0:
            b = _Jobs()
            b.add(("opr", 0), "init", site1=L.sigma[0])
            self._put(self.opr[0], 0, self._run(u, 0, b)[("opr", 0)])
            self._drop(self.hh, 0)
            return
        if release:
            self._release(i + 1, 1)
            self._release(i + 2, 1)
            self._fetch(i + 3)
        self._fetch(i - 1)
        b = _Jobs()
        if self.hh[i - 1] is not None:
            b.add("hh", "overlap", x=self.hh[i - 1])
        for k in range(i):
            if L.fll[i][k] == 1:
                b.add(("opr", k), "transform", x=self.opr[i - 1][k])
        op = self._combine([(self.opr[i - 1][k], float(L.coup[L.hmap[i][k]])) for k in range(i) if L.hmap[i][k] > 0])
        if op is not None:
            b.add("hh", "pair", x=op, site1=L.sigma[1])
        b.add(("opr", i), "init", site1=L.sigma[0])
        for m in range(2 * L.ns):
            j, k = m % L.ns, m // L.ns
            if L.plqflg[i][j] == 0 or i < p[j][1]:
                continue
            prev = self.plq[i - 1][m]
            if k == 0:
                if i == p[j][1]:
                    b.add(("plq", m), "pair", x=self.opr[i - 1][p[j][0]], site1=L.sigma[1])
                elif i == p[j][2]:
                    b.add(("plq", m), "init", x=prev, site1=L.sigma[0])
                elif i == p[j][3]:
                    b.add(("plq", m), "pair", x=prev, site1=L.sigma[1], coef=-L.qdelta)
                    b.add("hh", "pair", x=prev, site1=L.sigma[1], coef=-L.qdelta)
                elif p[j][1] < i < p[j][2]:
                    b.add(("plq", m), "overlap", x=prev)
                elif p[j][2] < i < p[j][3]:
                    b.add(("plq", m), "transform", x=prev)
            else:
                if i == p[j][1]:
                    b.add(("plq", m), "perm", x=self.opr[i - 1][p[j][0]], site1=L.qterm[0], site2=L.qterm[1])
                elif i == p[j][2]:
                    b.add(("plq", m), "perm", x=prev, site1=L.qterm[2], site2=L.qterm[3])
                elif i == p[j][3]:
                    b.add(("plq", m), "pair", x=prev, site1=L.sigma[1], coef=-L.qdelta)
                    b.add("hh", "pair", x=prev, site1=L.sigma[1], coef=-L.qdelta)
                elif p[j][1] < i < p[j][2] or p[j][2] < i < p[j][3]:
                    b.add(("plq", m), "transform", x=prev)
        out = self._run(u, 0, b)
        self._put(self.hh, i, out.get("hh"))
        for name, t in out.items():
            if isinstance(name, tuple) and name[0] == "opr":
                self._put(self.opr[i], name[1], t)
            elif isinstance(name, tuple):
                self._put(self.plq[i], name[1], t)
        if release:
            self._evict(i - 1)

    def site_right(self, i: int, u, release: bool = False):
        """prepare_site_operator_from_right(i[, flag]) with MPS tensor u at site
        i; release: the two-argument form, which first empties sites i-1 and
        i-2 (dmrg_su2_omp.cpp:480-481)."""
        L, p, ns = self.lat, self.lat.plqpos, self.lat.ns
        if i == ns - 1:
            b = _Jobs()
            b.add(("opr", i), "init", site1=L.sigma[1])
            self._put(self.opr[i], i, self._run(u, 1, b)[("opr", i)])
            self._drop(self.hh, i)
            return
        if release:
            self._release(i - 1, 0)
            self._release(i - 2, 0)
            self._fetch(i - 3)
        self._fetch(i + 1)
        b = _Jobs()
        if self.hh[i + 1] is not None:
            b.add("hh", "overlap", x=self.hh[i + 1])
        for k in range(i + 1, ns):
            if L.frr[i][k] == 1:
                b.add(("opr", k), "transform", x=self.opr[i + 1][k])
        op = self._combine([(self.opr[i + 1][k], float(L.coup[L.hmap[i][k]])) for k in range(i + 1, ns)
                            if L.hmap[i][k] > 0])
        if op is not None:
            b.add("hh", "pair", x=op, site1=L.sigma[0])
        b.add(("opr", i), "init", site1=L.sigma[1])
        for m in range(2 * ns):
            j, k = m % ns, m // ns
            if L.plqflg[i][j] == 0 or i > p[j][2]:
                continue
            prev = self.plq[i + 1][m]
            if k == 0:
                if i == p[j][2]:
                    b.add(("plq", m), "pair", x=self.opr[i + 1][p[j][3]], site1=L.sigma[0])
                elif i == p[j][1]:
                    b.add(("plq", m), "init", x=prev, site1=L.sigma[1])
                elif i == p[j][0]:
                    b.add(("plq", m), "pair", x=prev, site1=L.sigma[0], coef=-L.qdelta)
                    b.add("hh", "pair", x=prev, site1=L.sigma[0], coef=-L.qdelta)
                elif p[j][1] < i < p[j][2]:
                    b.add(("plq", m), "overlap", x=prev)
                elif p[j][0] < i < p[j][1]:
                    b.add(("plq", m), "transform", x=prev)
            else:
                if i == p[j][2]:
                    b.add(("plq", m), "perm", x=self.opr[i + 1][p[j][3]], site1=L.qterm[6], site2=L.qterm[7])
                elif i == p[j][1]:
                    b.add(("plq", m), "perm", x=prev, site1=L.qterm[4], site2=L.qterm[5])
                elif i == p[j][0]:
                    b.add(("plq", m), "pair", x=prev, site1=L.sigma[0], coef=-L.qdelta)
                    b.add("hh", "pair", x=prev, site1=L.sigma[0], coef=-L.qdelta)
                elif p[j][1] < i < p[j][2] or p[j][0] < i < p[j][1]:
                    b.add(("plq", m), "transform", x=prev)
        out = self._run(u, 1, b)
        self._put(self.hh, i, out.get("hh"))
        for name, t in out.items():
            if isinstance(name, tuple) and name[0] == "opr":
                self._put(self.opr[i], name[1], t)
            elif isinstance(name, tuple):
                self._put(self.plq[i], name[1], t)
        if release:
            self._evict(i + 1)

    # ------------------------------------------------------- two-site step
    # the Lanczos solve of a two-site step; a serving loop replaces it with
    # one that shares launches with other solves (same results, bit for bit)
    lanczos_hook = None

    def eigensolve(self, plan, vx, mlanc: int):
        if self.lanczos_hook is not None:
            return self.lanczos_hook(plan, vx, mlanc)
        return self._freeing(plan.lanczos, vx, mlanc=mlanc)

    def heff_plan(self, il: int, ir: int, vs):
        """The terms of hamiltonian_vector_multiplication_idmrg (dmrg_su2.cpp:543-664)."""
        L, ns = self.lat, self.lat.ns
        self._fetch(il)
        self._fetch(ir)
        terms = []

        def term(a, b, coef):
            if a is not None and b is not None:
                terms.append((a[0], a[1], b[0], b[1], coef))

        if il < ns // 2:
            for j in range(il + 1):
                r = self._combine([(self.opr[ir][k], float(L.coup[L.hmap[j][k]])) for k in range(ir, ns)
                                   if L.hmap[j][k] > 0])
                if r is not None:
                    self._keep.append(r)
                    term(self.opr[il][j], r, 1.0)
        else:
            for k in range(ir, ns):
                l = self._combine([(self.opr[il][j], float(L.coup[L.hmap[j][k]])) for j in range(il + 1)
                                   if L.hmap[j][k] > 0])
                if l is not None:
                    self._keep.append(l)
                    term(l, self.opr[ir][k], 1.0)
        if il == ir - 1:
            for m in range(2 * ns):
                j = m % ns
                if L.plqflg[il][j] != 1 or L.plqflg[ir][j] != 1:
                    continue
                q = L.plqpos[j]
                if il >= q[0] and ir <= q[1]:
                    term(self.opr[il][q[0]], self.plq[ir][m], -L.qdelta)
                elif il >= q[1] and ir <= q[2]:
                    term(self.plq[il][m], self.plq[ir][m], -L.qdelta)
                elif il >= q[2] and ir <= q[3]:
                    term(self.plq[il][m], self.opr[ir][q[3]], -L.qdelta)
        hl = (self.hh[il][0], self.hh[il][1], 1.0) if self.hh[il] is not None else None
        hr = (self.hh[ir][0], self.hh[ir][1], 1.0) if self.hh[ir] is not None else None
        return self._freeing(S.HeffPlan, vs, terms, hl, hr, mode=self.mode)

    def run(self):
        """do_idmrg: returns the eigenvalue of the last two-site step."""
        L, ns = self.lat, self.lat.ns
        B = S.Su2Bond
        self.uu[0] = S.fuse_tensor(B(1, [0], [1]), B(1, [L.physpn], [1]))
        self.uu[ns - 1] = S.fuse_tensor(B(1, [L.physpn], [1]), B(1, [L.totspin], [1]))
        phys = B(1, [L.physpn], [1])
        for i in range(ns // 2 - 1):
            self.site_left(i, self.uu[i], release=True)
            self.site_right(ns - 1 - i, self.uu[ns - 1 - i], release=True)
            bl = self.uu[i][0].bonds[2].inverted()
            br = self.uu[ns - 1 - i][0].bonds[2].inverted()
            self.uu[i + 1] = S.fuse_tensor(bl, phys)
            self.uu[ns - 2 - i] = S.fuse_tensor(phys, br)
            if (i + 2) * 2 * L.physpn >= L.totspin and i >= 1 or i == ns // 2 - 2:
                il, ir = i + 1, ns - 2 - i
                ul, ur = self.uu[il], self.uu[ir]
                vs, vx = S.initial_vector(ul[0], ul[1], ur[0], ur[1])
                vx = vx[: vs.size()]
                if self.ran_state is not None:
                    self.ran_state = S.random_vector(vx, self.ran_state)
                self.site_left(il, S.fuse_tensor(*self._legs01(ul)))
                self.site_right(ir, S.fuse_tensor(*self._legs01(ur)))
                plan = self.heff_plan(il, ir, vs)
                n = vs.size()
                e, _ = self.eigensolve(plan, vx, self.mlanc if self.mlanc <= n else n + 1)
                plan.close()
                self._keep.clear()
                self.energies.append((il, ir, e))
                p1, p2 = (1.0, 0.0) if i == ns // 2 - 2 else (0.0, 0.0)
                tu, xu, tv, xv, w = self._freeing(S.svd, vs, vx, ul[0], p1, ur[0], p2, L.max_dcut)
                self.uu[il], self.uu[ir] = (tu, xu), (tv, xv)
                self.ww = w
                self.truncations.append((il, ir, int(sum(tu.bonds[2].dim)), np.asarray(w)))
        return self.energies[-1][2] if self.energies else None
