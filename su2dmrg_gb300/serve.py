"""Serving loop: independent DMRG solves as requests, continuously batched.

The reference runs one solve per process (main_omp.cpp:158-202: the warm-up,
then sweeps until the energy changes by less than 1e-6).  Here a server keeps
several solves in flight on one GPU:

* admission: a request that has arrived is admitted when a slot is free and
  its estimated device footprint (footprint_bytes) fits in the HBM budget
  beside the solves already running; otherwise it waits, in arrival order;
* every admitted solve runs on its own host thread and CUDA stream with all
  of its tensors (MPS, environments, block Hamiltonians) resident on the
  device, so its environment updates, truncations and planning overlap those
  of the other solves;
* the Lanczos solves of the two-site steps are the hot path: a batcher
  collects the solves that reach one (waiting up to `window_s` for the other
  running solves to get there) and runs them in lockstep as one batch
  (su2g_heff_batch_lanczos), every matvec of every solve at a step in one set
  of shared launches.

A solve's result does not depend on the others in the mix: the batched
Lanczos returns, per solve, what su2g_lanczos returns bit for bit, and every
other operation of a solve runs on its own data.  Requests that arrive while
others run join the next batch as soon as they reach a Lanczos solve.
"""
from __future__ import annotations

import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import su2 as S
from .sweep import Dmrg
from .warmup import Lattice, discarded_weight


@dataclass
class Request:
    rid: int
    lattice: Lattice
    niter: int = 4           # sweeps after the warm-up at most (main_omp's -niter)
    arrival: float = 0.0     # seconds after the server starts
    meta: dict = field(default_factory=dict)


@dataclass
class Result:
    rid: int
    energies: list           # after the warm-up and after each sweep
    sweep_seconds: list
    mps_desc: list           # per site, the structure of its MPS tensor (retained multiplets)
    discarded: dict          # site -> discarded weight of the last truncation that set its bond
    t_arrive: float
    t_admit: float
    t_done: float
    footprint: int
    meta: dict

    @property
    def latency(self) -> float:
        return self.t_done - self.t_arrive

    @property
    def service(self) -> float:
        return self.t_done - self.t_admit


def footprint_bytes(lat: Lattice) -> int:
    """Estimated device bytes of one solve.  Per site its MPS tensor, block
    Hamiltonian and the spin-1 operators carried across it (the widest cut of
    the coupling map, half again with plaquette terms), each a D x D reduced
    matrix over the sectors (about a quarter of D^2 FP64 values); plus the
    transient work of one two-site step (operators packed as 7 BF16 digit
    slices, intermediates), four times one site's operators."""
    hm = np.asarray(lat.hmap) > 0
    ns = lat.ns
    width = 0
    for c in range(ns - 1):
        width = max(width, int(np.count_nonzero(hm[: c + 1, c + 1:].any(axis=1))))
    nops = (width + 2) * (1.5 if lat.qdelta != 0 else 1.0)
    per_op = 0.25 * float(lat.max_dcut) ** 2 * 8
    return int((ns + 4) * nops * per_op)


class LanczosBatcher:
    """Runs the Lanczos solves that running requests submit as lockstep
    batches of shared launches, on its own thread and CUDA stream."""

    def __init__(self, running, window_s: float = 0.005, device: int = 0):
        self.running = running  # callable: solves currently in flight
        self.window = window_s
        self.device = device
        self.cv = threading.Condition()
        self.pending = []
        self.stopping = False
        self.sizes = []
        self.thread = threading.Thread(target=self._loop, daemon=True)
        self.thread.start()

    def submit(self, plan, vx, mlanc: int):
        """Called from a solve's thread in place of plan.lanczos: blocks until
        the batch holding this solve is done; returns (energy, nmatvec)."""
        box = {}
        with self.cv:
            self.pending.append((plan, vx, mlanc, box))
            self.cv.notify_all()
            while "done" not in box:
                self.cv.wait()
        if "error" in box:
            raise box["error"]
        return box["result"]

    def stop(self):
        with self.cv:
            self.stopping = True
            self.cv.notify_all()
        self.thread.join()

    def _loop(self):
        import torch

        torch.cuda.set_device(self.device)
        stream = torch.cuda.Stream()
        with torch.cuda.stream(stream):
            while True:
                with self.cv:
                    while not self.pending and not self.stopping:
                        self.cv.wait()
                    if not self.pending:
                        return
                    t0 = time.monotonic()
                    # the other running solves may be about to reach their solves
                    while len(self.pending) < self.running() and time.monotonic() - t0 < self.window:
                        self.cv.wait(timeout=max(0.0, self.window - (time.monotonic() - t0)))
                    batch, self.pending = self.pending, []
                groups = {}
                for item in batch:
                    groups.setdefault((item[0].mode, item[2]), []).append(item)
                for (_mode, mlanc), items in groups.items():
                    try:
                        b = S.HeffBatch([it[0] for it in items])
                        res = b.lanczos([it[1] for it in items], mlanc=mlanc)
                        b.close()
                        for it, r in zip(items, res):
                            it[3]["result"] = r
                    except Exception as ex:  # every solve of the batch sees the error
                        for it in items:
                            it[3]["error"] = ex
                    self.sizes.append(len(items))
                with self.cv:
                    for it in batch:
                        it[3]["done"] = True
                    self.cv.notify_all()


class Server:
    """Continuous batching of independent solves on one GPU (see the module
    docstring).  slots: solves in flight at most; hbm_budget: device bytes the
    admitted solves' footprints may add up to (default: 80 % of the free
    memory at start); batch: share the Lanczos launches (False: every solve
    runs its own su2g_lanczos)."""

    def __init__(self, slots: int = 8, hbm_budget: int = None, mode: int = 1, batch: bool = True,
                 window_s: float = 0.005, device: int = 0):
        import torch

        S.lib()  # loaded once, before the worker threads start
        self.slots, self.mode, self.device = int(slots), int(mode), int(device)
        if hbm_budget is None:
            free, _ = torch.cuda.mem_get_info(device)
            hbm_budget = int(0.8 * free)
        self.budget = int(hbm_budget)
        self.batch = batch
        self.window = window_s
        self.max_inflight = 0
        self.max_reserved = 0

    def run(self, requests):
        """Serves the requests (arrival times in seconds after the start) and
        returns their results in request order."""
        import torch

        reqs = sorted(requests, key=lambda r: (r.arrival, r.rid))
        for r in reqs:
            if footprint_bytes(r.lattice) > self.budget:
                raise ValueError(f"request {r.rid}: footprint {footprint_bytes(r.lattice)} exceeds the budget")
        lock = threading.Condition()
        state = {"next": 0, "inflight": 0, "reserved": 0}
        results = {}
        errors = []
        t_start = time.perf_counter()
        batcher = LanczosBatcher(lambda: state["inflight"], self.window, self.device) if self.batch else None

        def admit():
            """The next request once it has arrived and fits; None when none are left."""
            with lock:
                while True:
                    if state["next"] >= len(reqs):
                        return None
                    r = reqs[state["next"]]
                    now = time.perf_counter() - t_start
                    fp = footprint_bytes(r.lattice)
                    if r.arrival <= now and state["reserved"] + fp <= self.budget:
                        state["next"] += 1
                        state["inflight"] += 1
                        state["reserved"] += fp
                        self.max_inflight = max(self.max_inflight, state["inflight"])
                        self.max_reserved = max(self.max_reserved, state["reserved"])
                        return r, fp, now
                    lock.wait(timeout=max(1e-3, r.arrival - now) if r.arrival > now else 0.05)

        def worker():
            torch.cuda.set_device(self.device)
            stream = torch.cuda.Stream()
            with torch.cuda.stream(stream):
                while True:
                    got = admit()
                    if got is None:
                        return
                    r, fp, t_admit = got
                    try:
                        d = Dmrg(r.lattice, mode=self.mode)
                        if batcher is not None:
                            d.lanczos_hook = batcher.submit
                        energies, secs = d.run_dmrg(r.niter)
                        stream.synchronize()
                        dw = {}
                        for il, ir, kept, w in d.truncations:
                            dw[il] = dw[ir] = discarded_weight(kept, w)
                        res = Result(r.rid, list(energies), list(secs),
                                     [d.uu[i][0].desc().tolist() for i in range(d.lat.ns)], dw, r.arrival, t_admit,
                                     time.perf_counter() - t_start, fp, dict(r.meta))
                        del d
                        with lock:
                            results[r.rid] = res
                    except Exception as ex:
                        errors.append((r.rid, ex))
                    finally:
                        with lock:
                            state["inflight"] -= 1
                            state["reserved"] -= fp
                            lock.notify_all()
                        if batcher is not None:
                            with batcher.cv:  # a solve left: the batcher may stop waiting for it
                                batcher.cv.notify_all()

        threads = [threading.Thread(target=worker, daemon=True) for _ in range(self.slots)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        if batcher is not None:
            batcher.stop()
            self.batch_sizes = list(batcher.sizes)
        if errors:
            raise RuntimeError(f"{len(errors)} solves failed: {errors[0][1]!r}") from errors[0][1]
        return [results[r.rid] for r in sorted(requests, key=lambda r: r.rid)]


def request_stream(n: int, rate: float, seed: int = 42, lx=(6, 8, 10, 12), ly=(4, 6), dcut=(128, 256, 512),
                   niter: int = 4):
    """The serving stream of the benchmark: seeded Poisson arrivals at `rate`
    per second; per request lx and ly uniform over the given choices, J2/J1
    uniform in [0, 1], Q/J1 uniform in [0, 2], total spin 0 or 1, D uniform
    over `dcut`."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n)) if rate > 0 else np.zeros(n)
    out = []
    for k in range(n):
        x, y = int(rng.choice(lx)), int(rng.choice(ly))
        r, q = rng.uniform(0.0, 1.0), rng.uniform(0.0, 2.0)
        spin, d = int(rng.integers(0, 2)), int(rng.choice(dcut))
        delta, qd = couplings(r, q)
        lat = Lattice.cylinder(x, y, delta, qd, d, totspin=2 * spin)
        out.append(Request(k, lat, niter, float(t[k] - t[0]) if n else 0.0,
                           {"lattice": f"{x}x{y}", "j2_over_j1": round(float(r), 4), "q_over_j1": round(float(q), 4),
                            "spin": spin, "D": d}))
    return out


def couplings(j2_over_j1, q_over_j1):
    """The engine's (delta, qdelta) for a J1-J2-Q cylinder given as ratios: its
    nearest-neighbour bond is delta + qdelta/2, its diagonal bond 1 - |qdelta|
    and its plaquette term qdelta (up to the overall scale, which the ratios
    do not fix)."""
    r, q = float(j2_over_j1), float(q_over_j1)
    qd = q / (r + q)
    delta = (1.0 - qd) / r - qd / 2.0 if r > 0 else 1.0 / q - 0.5
    return delta, qd
