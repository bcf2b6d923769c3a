"""DMRG sweeps with every tensor on the device.

dmrg_su2::sweep (dmrg_su2_omp.cpp:97-145) moves the two-site centre from the
middle to the left end, across to the right end and back to the middle.  At
each step the centre tensor is rotated to the side it moves to
(wavefunc_transformation, :1864-1877), the site just left behind is
updated (the two-argument prepare_site_operator_from_left / _right), the
two-site vector is predicted from the MPS pair (prepare_input_vector,
:229-254), the new centre's operators are built (the one-argument forms),
the Lanczos ground state is found (lanczos_solve_eigenvector_idmrg,
dmrg_su2.cpp:527-540, five vectors from the predicted state) and truncated
(tensor_su2::svd, with the singular values on the side the centre moves to).
main_omp.cpp:183-201 repeats sweeps after the warm-up until the energy
changes by less than 1e-6.  This module drives that sequence over the C ABI
of libsu2g, continuing from the device state the warm-up leaves
(su2dmrg_gb300.warmup); nothing but structures and the engine's tables lives
on the host.  Ground state only (exci = 0).
"""
from __future__ import annotations

import time

import numpy as np

from . import su2 as S
from .warmup import Warmup, host_available_bytes


class Dmrg(Warmup):
    """do_idmrg followed by sweeps.  nfree: the sites at each end the sweep
    does not reach (dmrg_su2.cpp:54 sets 2)."""

    nfree = 2
    step_hook = None  # called as step_hook(il, ir, energy) after each two-site step

    def clone(self, mode: int = None) -> "Dmrg":
        """A copy of the whole device state (MPS, block Hamiltonians, site and
        plaquette operators) that continues independently, in `mode` (default:
        this one's)."""
        def cp(t):
            return None if t is None else (t[0], t[1].clone())

        host = sum(t[1].numel() * t[1].element_size() for row in self.opr + self.plq + [self.hh] for t in row
                   if t is not None and not t[1].is_cuda)
        if host and host > self.host_fraction * host_available_bytes():
            raise MemoryError(f"clone: {host / 1e9:.1f} GB of host-resident block tensors do not fit the host")
        d = Dmrg(self.lat, mode=self.mode if mode is None else mode, mlanc=self.mlanc)
        d.offload, d.host_fraction = self.offload, self.host_fraction
        if hasattr(self, "_host"):  # the copies count against the same cap
            self._host["used"] += host
            d._host, d._device = self._host, getattr(self, "_device", None)
        d.ran_state = self.ran_state
        d.uu = [cp(t) for t in self.uu]
        d.hh = [cp(t) for t in self.hh]
        d.opr = [[cp(t) for t in row] for row in self.opr]
        d.plq = [[cp(t) for t in row] for row in self.plq]
        d.energies = list(self.energies)
        d.truncations = list(self.truncations)
        d.ww = self.ww
        return d

    def _timed(self, phase: str, t0: float) -> float:
        """Adds the wall time since t0 to phase_seconds[phase] (every library
        call blocks, so this is the phase's device and host time)."""
        t1 = time.perf_counter()
        self.phase_seconds[phase] = self.phase_seconds.get(phase, 0.0) + (t1 - t0)
        return t1

    @property
    def phase_seconds(self) -> dict:
        if not hasattr(self, "_phase_seconds"):
            self._phase_seconds = {}
        return self._phase_seconds

    def _vectran(self, i: int, flag: int) -> None:
        """wavefunc_transformation(i, flag): right2left_vectran (0) or
        left2right_vectran (1) of uu[i]."""
        t0 = time.perf_counter()
        s, y = S.vectran(*self.uu[i], flag)
        self.uu[i] = (s, y[: s.size()])
        self._timed("vectran", t0)

    def _step(self, il: int, ir: int, p1: float, p2: float) -> float:
        L = self.lat
        t = time.perf_counter()
        vs, vx = S.prepare_input_vector(*self.uu[il], *self.uu[ir], mode=self.mode)
        vx = vx[: vs.size()]
        t = self._timed("input_vector", t)
        self.site_left(il, S.fuse_tensor(*self._legs01(self.uu[il])))
        self.site_right(ir, S.fuse_tensor(*self._legs01(self.uu[ir])))
        t = self._timed("site_update_centre", t)
        plan = self.heff_plan(il, ir, vs)
        t = self._timed("heff_plan", t)
        n = vs.size()
        e, _ = self.eigensolve(plan, vx, self.mlanc if self.mlanc <= n else n + 1)
        plan.close()
        self._keep.clear()
        t = self._timed("lanczos", t)
        self.energies.append((il, ir, e))
        tu, xu, tv, xv, w = self._freeing(S.svd, vs, vx, self.uu[il][0], p1, self.uu[ir][0], p2, L.max_dcut)
        self.uu[il], self.uu[ir] = (tu, xu), (tv, xv)
        self._timed("truncation", t)
        self.ww = w
        self.truncations.append((il, ir, int(sum(tu.bonds[2].dim)), np.asarray(w)))
        if self.step_hook is not None:
            self.step_hook(il, ir, e)
        return e

    def sweep(self) -> float:
        """One sweep; returns the eigenvalue of its last step (the centre)."""
        ns, nf = self.lat.ns, self.nfree
        for i in range(ns // 2, nf + 1, -1):        # centre -> left end
            self._vectran(i - 1, 1)
            t = time.perf_counter()
            self.site_right(i, self.uu[i], release=True)
            self._timed("site_update", t)
            self._step(i - 2, i - 1, *((1.0, 0.0) if i > nf + 2 else (0.0, 1.0)))
        for i in range(nf, ns - nf - 2):             # left end -> right end
            self._vectran(i + 1, 0)
            t = time.perf_counter()
            self.site_left(i, self.uu[i], release=True)
            self._timed("site_update", t)
            self._step(i + 1, i + 2, *((0.0, 1.0) if i < ns - nf - 3 else (1.0, 0.0)))
        for i in range(ns - nf - 1, ns // 2, -1):   # right end -> centre
            self._vectran(i - 1, 1)
            t = time.perf_counter()
            self.site_right(i, self.uu[i], release=True)
            self._timed("site_update", t)
            self._step(i - 2, i - 1, 1.0, 0.0)
        return self.energies[-1][2]

    def run_dmrg(self, niter: int, tol: float = 1e-6):
        """main_omp's loop: the warm-up, then up to niter sweeps, stopping when
        a sweep changes the energy by less than tol.  Returns the energies
        (eigenvalues) after the warm-up and after each sweep, and the seconds
        each sweep took (device work included: every call blocks)."""
        e1 = self.run()
        energies, seconds = [e1], []
        for _ in range(niter):
            t0 = time.perf_counter()
            e2 = self.sweep()
            seconds.append(time.perf_counter() - t0)
            energies.append(e2)
            if abs(e1 - e2) < tol:
                break
            e1 = e2
        return energies, seconds
