"""Benchmark of the SU(2) block-sparse H_eff*psi hot path on GB300.

Workload (the reference's microbenchmark shape): one two-site effective
Hamiltonian with D=2000 SU(2) multiplets per bond (sectors 2j=0..12, Gaussian
counts), spin-1/2 sites (enlarged legs 2j=0..13, psi = 1,576,457 doubles), 18
spin-1 operator pairs plus the two spin-0 block Hamiltonians (width 20),
seeded synthetic data (workloads.synthetic_heff, seed 1234).  One "step" is
one application y = H_eff psi.

Printed JSON (rank 0, one line):
  value  algorithmic FLOPs per application / device time, operators and psi
         resident in HBM (the operators, ~1.3 GB, exceed the 129 MB L2, so no
         flush is needed between iterations);
  e2e    the same metric through the C ABI with host buffers: pinned-host psi
         copied in, applied, y copied back, every step;
  roofline  the two split GEMM launches against the measured BF16 burst peak
         of MEASURED_PEAKS.json (28 BF16 products per FP64 product), with
         their DRAM traffic per launch;
  cpu_baseline  the oracle port on the host cores (a bounded sample);
  clocks  nvidia-smi SM clocks and throttle reasons during the timed region;
  gpu_launches  the library's kernel launches in the timed region.
Default steps: 250 applications (about 1 s, so that the clock record holds
several samples under load); 10 calls for the other rows.
--impl reference times the CPU restatement of the reference's hot path (the
reference itself is not built on the GPU host) on all host cores.

--row input_vector | vectran | env | svd times one other operation of a site
step instead, on workloads.synthetic_site_step at the same D, through its C
ABI call with arguments prepared once (each call blocks; its host planning is
inside the timed region), with L2 flushed before every call; same JSON keys,
its own metric.

--row sweep runs whole DMRG sweeps of an lx x ly cylinder (--lattice, --D,
--delta, --qdelta, --seed; --converge or --sweeps-before), then the next sweep
in split and in FP64 precision from the same state (--skip-fp64: split only);
--offload keeps the block tensors of passed positions in host memory and
--step-log prints one stderr line per two-site step.  --row serve runs the
serving stream (--requests, --rate, --slots, --no-batch, --seq-requests);
--row tune measures the FP64 engine's tile table (--table-out).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "H_eff*psi TFLOP/s (FP64-equivalent), SU(2) D=2000 two-site step, width 20"
UNIT = "TFLOP/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="su2g", choices=["su2g", "reference"])
    ap.add_argument("--mode", default="split", choices=["f64", "split", "split-fast"])
    ap.add_argument("--D", type=int, default=2000)
    ap.add_argument("--nspin1", type=int, default=18)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--row", default="heff",
                    choices=["heff", "input_vector", "vectran", "env", "svd", "sweep", "serve", "tune"],
                    help="heff (the headline) or another operation of the site step, timed on the "
                         "D-multiplet site-step workload (workloads.synthetic_site_step); sweep: one whole "
                         "DMRG sweep of a J1-J2 cylinder after the device warm-up, split and FP64 contractions "
                         "from the same state")
    ap.add_argument("--lattice", default="16x8", help="sweep row: LXxLY cylinder")
    ap.add_argument("--delta", type=float, default=2.0,
                    help="sweep row: nearest-neighbour coupling (diagonal 1 - |qdelta|; 2.0 = J2/J1 0.5)")
    ap.add_argument("--qdelta", type=float, default=0.0, help="sweep row: plaquette coupling Q")
    ap.add_argument("--skip-fp64", action="store_true", help="sweep row: time the split sweep only")
    ap.add_argument("--step-log", action="store_true", help="sweep row: one stderr line per two-site step")
    ap.add_argument("--offload", action="store_true",
                    help="sweep row: block tensors of positions the sweep has passed live in host memory")
    ap.add_argument("--requests", type=int, default=32, help="serve row: requests of the stream served")
    ap.add_argument("--rate", type=float, default=2.0, help="serve row: Poisson arrival rate (solves per second)")
    ap.add_argument("--slots", type=int, default=8, help="serve row: solves in flight at most")
    ap.add_argument("--no-batch", action="store_true",
                    help="serve row: every solve runs its own Lanczos (no shared launches)")
    ap.add_argument("--seq-requests", type=int, default=8,
                    help="serve row: the first requests of the stream also run one after another")
    ap.add_argument("--sweeps-before", type=int, default=1,
                    help="sweep row: untimed split sweeps between the warm-up and the timed sweep")
    ap.add_argument("--converge", action="store_true",
                    help="sweep row: split sweeps until one changes the energy by less than 1e-6 before the "
                         "timed split and FP64 sweeps")
    ap.add_argument("--max-sweeps", type=int, default=8, help="sweep row: at most this many sweeps with --converge")
    ap.add_argument("--table-out", default=None, help="tune row: where to write the measured tile table (JSON)")
    ap.add_argument("--seed", type=int, default=None, help="sweep row: seeded random start of the warm-up")
    a = ap.parse_args()
    if a.steps is None:
        a.steps = 250 if a.row == "heff" else 10
    return a


def dist_setup(args):
    rank, world = 0, 1
    if "RANK" in os.environ and int(os.environ.get("WORLD_SIZE", "1")) > 1:
        import torch.distributed as dist

        rank = int(os.environ["RANK"])
        world = int(os.environ["WORLD_SIZE"])
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        import torch

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", rank)))
        dist.init_process_group("nccl")
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x, world):
    """The largest x over the ranks (replicas: each rank times its own copy of
    the workload; the job takes as long as the slowest)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_step, world, steps, seconds):
    """Whole-job rate: every rank processes units_per_step per step (weak
    scaling, replicas), over the max-over-ranks time."""
    return units_per_step * world * steps / seconds


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []
        self.mark = 0

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # nvidia-smi takes a moment to start: wait (at most 3 s) for its
            # first line, and count only the samples taken after it
            t_end = time.time() + 3.0
            while not self.lines and time.time() < t_end and self.proc.poll() is None:
                time.sleep(0.01)
            self.mark = len(self.lines)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self.lines[self.mark:] or self.lines[-1:]
        for ln in lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


MODES = {"f64": 0, "split": 1, "split-fast": 2}
SLICES = {"f64": 0, "split": 7, "split-fast": 6}


def bf16_peak():
    """Dense BF16 peak measured on this machine (MEASURED_PEAKS.json), else the
    documented fallback."""
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["bf16_tflops"]), "measured (MEASURED_PEAKS.json bf16_tflops, burst)"
    except (OSError, KeyError, ValueError):
        return 1900.0, "fallback 1.9 PFLOP/s"


def fp64_peak_tflops(torch):
    """Measured FP64 GEMM throughput (cuBLAS DGEMM 8192^3, best of 5): the
    denominator of the FP64 roofline, which MEASURED_PEAKS.json does not hold."""
    n = 8192
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    c = a @ b
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        torch.matmul(a, b, out=c)
        e.record()
        e.synchronize()
        best = min(best, s.elapsed_time(e) / 1e3)
    del a, b, c
    torch.cuda.empty_cache()
    return 2.0 * n**3 / best / 1e12


class CpuSample:
    """The oracle (CPU restatement of the reference hot path: C loops over
    the blocks, OpenBLAS dgemm, all host cores) applying the same synthetic
    H_eff as the GPU arm, full width.  The workload is built by the oracle
    itself (oracle.synthetic_heff draws the same numbers as the library's
    generator), so nothing of the GPU library is loaded on this path."""

    def __init__(self, D, nspin1):
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import oracle as o

        self.o = o
        o.build()
        self.cores = os.cpu_count() or 1
        o.set_blas_threads(self.cores)
        self.prob, self.psi = o.synthetic_heff(D=D, nspin1=nspin1, seed=1234)
        self.flops = o.heff_flops(self.prob)
        self.desc = (f"the full width-{nspin1 + 2} application ({nspin1} spin-1 terms + both spin-0 terms) "
                     f"at D={D} (oracle C restatement of the reference, OpenBLAS dgemm, {self.cores} threads)")

    def step(self):
        t0 = time.perf_counter()
        self.o.heff_apply(self.prob, self.psi)
        return time.perf_counter() - t0

    def measure(self, seconds=10.0, max_steps=30):
        self.step()  # warm
        ts = []
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < seconds and len(ts) < max_steps:
            ts.append(self.step())
        dt = float(np.median(ts))
        return {"value": self.flops / dt / 1e12, "unit": UNIT, "cores": self.cores, "kind": "port",
                "sample": f"{len(ts)} applications of {self.desc}; median time"}


def run_reference(args):
    """The reference arm: the CPU restatement of the reference's hot path
    (oracle/), on the GPU arm's workload and metric.  Only the oracle and
    numpy/SciPy are loaded; rank 0 alone runs under torchrun."""
    rank = int(os.environ.get("RANK", "0")) if args.gpus > 1 else 0
    if rank != 0:
        return 0
    cs = CpuSample(args.D, args.nspin1)
    for _ in range(args.warmup):
        cs.step()
    ts = [cs.step() for _ in range(args.steps)]
    total = float(np.sum(ts))
    v = cs.flops * args.steps / total / 1e12
    cb = {"value": v, "unit": UNIT, "cores": cs.cores, "kind": "port",
          "sample": f"each step = one application of {cs.desc}; {args.steps} steps"}
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"synthetic SU(2) two-site H_eff, D={args.D}, width {args.nspin1 + 2}",
                       "flops_per_step": cs.flops, "same_config": True},
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_su2g(args):
    import torch

    from su2dmrg_gb300 import capi
    from su2dmrg_gb300.su2 import HeffPlan
    from su2dmrg_gb300.workloads import synthetic_heff

    rank, world = dist_setup(args)
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", rank)) if world > 1 else 0)
    capi.lib()
    w = synthetic_heff(D=args.D, nspin1=args.nspin1, seed=1234)
    psi, terms, hl, hr = w.to_device()
    op_bytes = 8.0 * (sum(t[1].numel() + t[3].numel() for t in terms) + sum(h[1].numel() for h in (hl, hr) if h))
    plan = HeffPlan(w.psi, terms, hl, hr, mode=MODES[args.mode])
    info = plan.info()
    flops = info["flops"]
    y = torch.empty_like(psi)
    stream = torch.cuda.current_stream()

    for _ in range(args.warmup):
        plan.apply(psi, y, stream)
    torch.cuda.synchronize()

    # ---- device-resident timing ----
    barrier(world)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(torch.cuda.current_device()) as clk:
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for s, e in ev:
            s.record(stream)
            plan.apply(psi, y, stream)
            e.record(stream)
        t1.record(stream)
        torch.cuda.synchronize()
    barrier(world)
    total = t0.elapsed_time(t1) / 1e3
    total = max_over_ranks(total, world)
    ms_per_step = total / args.steps * 1e3
    value = job_throughput(flops, world, args.steps, total) / 1e12

    # ---- end to end through the C ABI with host buffers ----
    h_psi = torch.from_numpy(w.psi_data.copy()).pin_memory()
    h_y = torch.empty_like(h_psi).pin_memory()
    d_in = torch.empty_like(psi)
    for _ in range(2):
        d_in.copy_(h_psi, non_blocking=True)
        plan.apply(d_in, y, stream)
        h_y.copy_(y, non_blocking=True)
    torch.cuda.synchronize()
    barrier(world)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        d_in.copy_(h_psi, non_blocking=True)
        plan.apply(d_in, y, stream)
        h_y.copy_(y, non_blocking=True)
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_total = max_over_ranks(e0.elapsed_time(e1) / 1e3, world)
    e2e_value = job_throughput(flops, world, args.steps, e2e_total) / 1e12
    nbytes = psi.numel() * 8

    if rank != 0:
        return 0
    # parity spot check of the measured output against the host copy path
    assert torch.equal(h_y.cuda(), y), "e2e output differs from device-resident output"

    # per-launch times of one application (events between the launches)
    prof = [plan.apply_profile(psi, y, stream) for _ in range(3)]
    prof = [float(np.median([p[i] for p in prof])) for i in range(len(prof[0]))]
    S = SLICES[args.mode]
    if S == 0:
        peak = fp64_peak_tflops(torch)
        t_kernel = (prof[0] + prof[1]) / 1e3
        achieved = flops / t_kernel / 1e12
        roof = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "traffic": None, "kernel": "gemm_f64_tiles (FP64 DMMA m8n8k4), 2 launches per step",
                "launch_ms": prof,
                "peak_source": "measured cuBLAS DGEMM 8192^3 on this GPU (FP64 is not in MEASURED_PEAKS.json)"}
        accuracy = {"mode": "FP64", "rel_err_vs_fp64_path": 0.0}
        fp64 = {"value": value, "unit": UNIT, "ms_per_step": ms_per_step, "steps": args.steps,
                "path": "this line (mode f64)"}
    else:
        peak, src = bf16_peak()
        pairs = S * (S + 1) // 2
        t_kernel = (prof[1] + prof[3]) / 1e3
        achieved = pairs * flops / t_kernel / 1e12
        # DRAM bytes of the two GEMM launches, measured with ncu (dram__bytes_read.sum +
        # dram__bytes_write.sum) on this D=2000 width-20 workload: 1.828e9 (phase 1) +
        # 2.970e9 (phase 2) = 3.74 bytes per algorithmic byte of an application (FP64
        # operators + psi in/out); other sizes are scaled by their algorithmic bytes.
        alg_bytes = 8.0 * (sum(x.numel() for (_s1, x1, _s2, x2, _c) in terms for x in (x1, x2))
                           + sum(h[1].numel() for h in (hl, hr) if h is not None) + 2 * w.psi.size())
        captured = args.D == 2000 and args.nspin1 == 18 and S == 7
        traffic = 3.737 * alg_bytes / 2 if captured else None
        roof = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "traffic": traffic,
                "traffic_definition": "DRAM bytes per GEMM launch: ncu-measured 3.737 x algorithmic bytes per "
                                      "application (D=2000 width-20 capture: 1.828e9 + 2.970e9 B over the two "
                                      f"launches), this workload's algorithmic bytes {alg_bytes:.4g} B, halved "
                                      "over the two launches; the digit-pack launches are not included; "
                                      "null when the workload is not the captured one",
                "kernel": f"ozaki_gemm<{S}> (tcgen05 BF16, {pairs} digit-pair products per FP64 product), "
                          "2 launches per step",
                "achieved_definition": f"{pairs} x algorithmic FP64 FLOPs of the two GEMM launches / their time",
                "launch_ms": {"pack_psi": prof[0], "gemm_phase1": prof[1], "pack_intermediates": prof[2],
                              "gemm_phase2": prof[3], "sum_split_tiles": prof[4]},
                "peak_source": src}
        ref_plan = HeffPlan(w.psi, terms, hl, hr, mode=capi.MODE_F64)
        y64 = torch.empty_like(psi)
        ref_plan.apply(psi, y64, stream)
        plan.apply(psi, y, stream)
        torch.cuda.synchronize()
        rel = float((y - y64).norm() / y64.norm())
        # the plain FP64 GPU path on the same workload (the other half of the
        # split-vs-FP64 metric): a few applications, device time
        for _ in range(2):
            ref_plan.apply(psi, y64, stream)
        torch.cuda.synchronize()
        nf = max(3, min(args.steps, 10))
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(nf):
            ref_plan.apply(psi, y64, stream)
        f1.record(stream)
        torch.cuda.synchronize()
        f64_ms = f0.elapsed_time(f1) / nf
        fp64 = {"value": flops / (f64_ms / 1e3) / 1e12, "unit": UNIT, "ms_per_step": f64_ms, "steps": nf,
                "path": "gemm_f64_tiles (FP64 DMMA), same plan inputs, device-resident",
                "split_speedup": f64_ms / ms_per_step}
        ref_plan.close()
        accuracy = {"mode": f"BF16 x {S} slices", "rel_err_vs_fp64_path": rel,
                    "tolerance": 1e-12 if S == 7 else 1e-10}
        assert plan.status() == 0
    cb = None
    if not args.no_cpu_baseline:
        cb = CpuSample(args.D, args.nspin1).measure(seconds=10.0)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if S == 0 else f"f64 emulated by bf16 x{S} (fp32 accumulate)",
        "data": "synthetic",
        "config": {"workload": f"synthetic SU(2) two-site H_eff, D={args.D}, width {args.nspin1 + 2}",
                   "mode": args.mode, "psi_doubles": int(psi.numel()), "flops_per_step": flops,
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2": f"inputs (operators {op_bytes / 1e9:.1f} GB) larger than L2; no flush"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                "path": "su2g_heff_apply via ctypes, pinned host psi -> device -> host y; operators resident"},
        "gpu_launches": plan.launches() * args.steps,
        "roofline": roof,
        "accuracy": accuracy,
        "fp64": fp64,
        "cpu_baseline": cb,
        "clocks": clk.summary(),
    }
    print(json.dumps(line))
    return 0


def _time_calls(torch, fn, steps, warmup):
    """Device time of `steps` blocking calls, L2 flushed (256 MB written) before each."""
    buf = torch.zeros(32 << 20, dtype=torch.float64, device="cuda")
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    ts = []
    with ClockSampler(torch.cuda.current_device()) as clk:
        for _ in range(steps):
            buf.add_(1.0)
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            fn()
            e.record(stream)
            e.synchronize()
            ts.append(s.elapsed_time(e) / 1e3)
    return ts, clk.summary()


def _cpu_sample(fn, seconds=10.0, max_steps=10):
    fn()
    ts, t0 = [], time.perf_counter()
    while time.perf_counter() - t0 < seconds and len(ts) < max_steps:
        a = time.perf_counter()
        fn()
        ts.append(time.perf_counter() - a)
    return float(np.median(ts)), len(ts)


def _oracle():
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as o

    o.build()
    o.set_blas_threads(os.cpu_count() or 1)
    return o


def _oracle_struct(o, s):
    st = o.Struct([o.Bond(b.dir, list(b.angm), list(b.dim)) for b in s.bonds], s.locspin)
    st.flag = np.ascontiguousarray(s.flag, np.int32)
    return st


def _gemm_roofline(torch, flops, t, slices, what):
    if slices:
        pk, src = bf16_peak()
        pairs = slices * (slices + 1) // 2
        ach = pairs * flops / t / 1e12
        return {"bound": "tensor", "achieved": ach, "peak": pk, "unit": "TFLOP/s", "frac": ach / pk,
                "traffic": None, "peak_source": src,
                "achieved_definition": f"{pairs} BF16 products per FP64 product over the whole call ({what})"}
    pk = fp64_peak_tflops(torch)
    ach = flops / t / 1e12
    return {"bound": "tensor", "achieved": ach, "peak": pk, "unit": "TFLOP/s", "frac": ach / pk, "traffic": None,
            "peak_source": "measured cuBLAS DGEMM 8192^3 on this GPU",
            "achieved_definition": f"FP64 FLOPs over the whole call ({what})"}


def run_row(args):
    """One other operation of the site step (--row), single GPU."""
    import torch

    from su2dmrg_gb300 import capi
    from su2dmrg_gb300 import su2 as S
    from su2dmrg_gb300.workloads import synthetic_heff, synthetic_site_step

    capi.lib()
    torch.cuda.set_device(0)
    w = synthetic_site_step(D=args.D, nops=args.nspin1)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    mode = MODES[args.mode]
    slices = SLICES[args.mode]
    o = None if args.no_cpu_baseline else _oracle()
    cores = os.cpu_count() or 1
    cb = None
    extra = {}
    dtype = "f64" if not slices else f"f64 emulated by bf16 x{slices} (fp32 accumulate)"
    if args.row == "input_vector":
        (sl, xl), (sr, xr) = w.ul, w.ur
        dl, dr = dev(xl), dev(xr)
        vs = S.input_vector_layout(sl, sr)
        fl, fr = vs.bonds
        flops = 0.0
        for k, c in enumerate(sl.bonds[2].angm):
            if c in fl.angm and c in fr.angm:
                flops += 2.0 * fl.dim[fl.angm.index(c)] * fr.dim[fr.angm.index(c)] * sl.bonds[2].dim[k]
        keep = []
        tl, tr = S._tensor(sl, dl, keep), S._tensor(sr, dr, keep)
        yv = torch.empty(vs.size(), dtype=torch.float64, device="cuda")
        # the C-ABI call alone, its arguments prepared once (the structure is known to the caller)
        ts, clk = _time_calls(torch, lambda: capi.check(capi.lib().su2g_prepare_input_vector(
            tl, tr, capi.ptr(yv), mode, None)), args.steps, args.warmup)
        t = float(np.median(ts))
        metric, unit, hib = f"initial two-site vector TFLOP/s (FP64-equivalent), SU(2) D={args.D}", "TFLOP/s", True
        value = flops / t / 1e12
        roof = _gemm_roofline(torch, flops, t, slices, "transpose of ur, planning, pack and GEMM launches")
        _, yg = S.prepare_input_vector(sl, dl, sr, dr, mode=mode)
        if o is not None:
            osl, osr = _oracle_struct(o, sl), _oracle_struct(o, sr)
            ref = {}
            tc, n = _cpu_sample(lambda: ref.__setitem__("y", o.prepare_input_vector(osl, xl, osr, xr)[1]))
            cb = {"value": flops / tc / 1e12, "unit": unit, "cores": cores, "kind": "port",
                  "sample": f"the full call, oracle (numpy BLAS), median of {n}"}
            got = yg[: vs.size()].cpu().numpy()
            extra["rel_err_vs_oracle"] = float(np.linalg.norm(got - ref["y"]) / np.linalg.norm(ref["y"]))
        config = {"workload": f"synthetic SU(2) MPS pair, D={args.D}, spin-1/2 sites", "mode": args.mode,
                  "flops_per_step": flops, "vector_doubles": vs.size()}
    elif args.row == "vectran":
        su, xu = w.ul
        d = dev(xu)
        out = torch.empty_like(d)
        keep = []
        tu = S._tensor(su, d, keep)
        ts, clk = _time_calls(torch, lambda: capi.check(capi.lib().su2g_vectran(tu, 0, capi.ptr(out), None)),
                              args.steps, args.warmup)
        nbytes = 16.0 * su.size()
        t = float(np.median(ts))
        metric, unit, hib = f"vectran GB/s (right2left, read + write), SU(2) MPS tensor D={args.D}", "GB/s", True
        value = nbytes / t / 1e9
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            peak = float(json.load(f)["hbm_gbs"])
        roof = {"bound": "hbm", "achieved": value, "peak": peak, "unit": "GB/s", "frac": value / peak,
                "traffic": None, "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)",
                "achieved_definition": "16 bytes per element over the whole call (one transpose launch)"}
        dtype = "f64"
        if o is not None:
            osu = _oracle_struct(o, su)
            tc, n = _cpu_sample(lambda: o.vectran(osu, xu, 0))
            cb = {"value": nbytes / tc / 1e9, "unit": unit, "cores": 1, "kind": "port",
                  "sample": f"the full call, oracle (numpy), median of {n}"}
            extra["bit_exact_vs_oracle"] = bool(np.array_equal(out[: su.size()].cpu().numpy(),
                                                               o.vectran(osu, xu, 0)[1]))
        config = {"workload": f"synthetic SU(2) MPS tensor, D={args.D}", "elements": su.size()}
    elif args.row == "env":
        su, xu = w.uu
        du = dev(xu)
        jobs = [{"kind": "transform", "slot": i, "coef": 1.0, "x": (s_, dev(x_))} for i, (s_, x_) in enumerate(w.ops)]
        jobs.append({"kind": "overlap", "slot": len(w.ops), "coef": 1.0, "x": (w.hh[0], dev(w.hh[1]))})
        flops = S.env_validate(su, du, su, du, 0, jobs, mode=mode)["flops"]
        outs = [torch.empty(max(1, S.env_layout(su, du, su, du, 0, jobs, k).size()), dtype=torch.float64,
                            device="cuda") for k in range(len(jobs))]
        keep = []
        J = S._EnvJobs(jobs)
        tuu = S._tensor(su, du, keep)
        optr = (ctypes.c_void_p * len(outs))(*[capi.ptr(x) for x in outs])
        ts, clk = _time_calls(torch, lambda: capi.check(capi.lib().su2g_env_run(
            tuu, tuu, 0, J.n, J.ptr, len(outs), ctypes.addressof(optr), mode, None)), args.steps, args.warmup)
        t = float(np.median(ts))
        metric, unit, hib = (f"environment update TFLOP/s (FP64-equivalent), SU(2) D={args.D}, "
                             f"{len(w.ops)} spin-1 operators + block Hamiltonian"), "TFLOP/s", True
        value = flops / t / 1e12
        roof = _gemm_roofline(torch, flops, t, slices, "planning, pack and GEMM launches")
        if o is not None:
            # the oracle's operator_transformation costs minutes at full D: one operator at D/4
            ws = synthetic_site_step(D=args.D // 4, nops=1)
            su_s, xu_s = ws.uu
            s0, x0 = ws.ops[0]
            osu, os0 = _oracle_struct(o, su_s), _oracle_struct(o, s0)
            res = {}
            tc, n = _cpu_sample(lambda: res.__setitem__("y", o.env_transform(1, osu, xu_s, osu, xu_s, os0, x0, 0)[1]),
                                max_steps=3)
            du_s = dev(xu_s)
            job = [{"kind": "transform", "slot": 0, "coef": 1.0, "x": (s0, dev(x0))}]
            f1 = S.env_validate(su_s, du_s, su_s, du_s, 0, job, mode=0)["flops"]
            cb = {"value": f1 / tc / 1e12, "unit": unit, "cores": 1, "kind": "port",
                  "sample": f"one operator_transformation at D={args.D // 4}, oracle (C loops), median of {n}"}
            (_, ys), = S.env_batch(su_s, du_s, su_s, du_s, 0, job, mode=mode)
            got = ys[: len(res["y"])].cpu().numpy()
            extra["rel_err_vs_oracle_sample"] = float(np.linalg.norm(got - res["y"]) / np.linalg.norm(res["y"]))
        config = {"workload": f"synthetic SU(2) site update, D={args.D}, {len(w.ops)} spin-1 operators + "
                              "block Hamiltonian", "mode": args.mode, "flops_per_step": flops}
    else:  # svd
        h = synthetic_heff(D=args.D, nspin1=0, seed=1234, spin0=False)
        psi = dev(h.psi_data)
        tu = w.ul[0]
        ts, clk = _time_calls(torch, lambda: S.svd(h.psi, psi, tu, 1.0, tu, 0.0, args.D), args.steps, args.warmup)
        t = float(np.median(ts))
        metric, unit, hib = f"truncation ms per two-site vector, SU(2) D={args.D} -> {args.D} multiplets", "ms", False
        value = t * 1e3
        gram = 0.0
        for i in range(h.psi.nten):
            if h.psi.flag[i]:
                a, b = h.psi.block_shape(i)
                m, n = min(a, b), max(a, b)
                gram += 4.0 * m * m * n  # Gram matrix + the other factor
        roof = _gemm_roofline(torch, gram, t, 0, "Gram and second-factor products only; the eigendecompositions "
                                                 "and host sorting are not counted")
        dtype = "f64"
        if o is not None:
            ops_ = _oracle_struct(o, h.psi)
            tc, n = _cpu_sample(lambda: o.svd_truncate(ops_, h.psi_data, 1.0, 0.0, args.D), max_steps=3)
            cb = {"value": tc * 1e3, "unit": unit, "cores": cores, "kind": "port",
                  "sample": f"the same truncation, oracle (numpy LAPACK per sector + dsort2), median of {n}"}
        config = {"workload": f"synthetic SU(2) two-site vector, D={args.D}, spin-1/2 sites", "max_dcut": args.D}
    line = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": float(np.median(ts)) * 1e3, "higher_is_better": hib,
            "scaling": "weak", "vs_baseline": None, "dtype": dtype, "data": "synthetic",
            "config": {**config, "row": args.row, "l2": "flushed (256 MB write) before every call"},
            "roofline": roof, "cpu_baseline": cb, "clocks": clk, **extra}
    print(json.dumps(line))
    return 0


def _bond_dims(d):
    """Per site, the structure descriptor of its MPS tensor (its bonds'
    sectors and multiplet counts)."""
    return [d.uu[i][0].desc().tolist() for i in range(d.lat.ns)]


def _retained_compare(da, db, wa, wb):
    """Retained multiplets of two sweeps' MPS, bond by bond: identical sector
    by sector, or (where two runs settled on different truncations of the same
    quality) the same total with discarded weights within 1e-10."""
    def legs(desc):
        out, p = [], 2
        for _ in range(desc[0]):
            n = desc[p + 1]
            out.append((desc[p], desc[p + 2: p + 2 + n], desc[p + 2 + n: p + 2 + 2 * n]))
            p += 2 + 2 * n
        return out

    same, moved, bad = 0, 0, []
    for i, (a, b) in enumerate(zip(da, db)):
        if a == b:
            same += 1
            continue
        la, lb = legs(a), legs(b)
        ok = [x[:2] for x in la] == [x[:2] for x in lb]
        for x, y in zip(la, lb):
            if ok and x[2] != y[2]:
                ok = sum(x[2]) == sum(y[2]) and abs(wa.get(i, 0.0) - wb.get(i, 0.0)) <= 1e-10
        if ok:
            moved += 1
        else:
            bad.append(i)
    return {"sites_identical": same, "sites_same_totals_weights_within_1e-10": moved, "sites_differing": bad}


def _discarded_by_site(d, first):
    from su2dmrg_gb300.warmup import discarded_weight

    out = {}
    for il, ir, kept, w in d.truncations[first:]:
        out[il] = out[ir] = discarded_weight(kept, w)
    return out


def _svd_trace_summary(path, first_line):
    """Totals of the truncation trace lines written since first_line."""
    try:
        with open(path) as f:
            lines = f.readlines()[first_line:]
    except OSError:
        return None, first_line
    recs = [json.loads(x) for x in lines if x.strip()]
    lev = [len(s["levels"]) for r in recs for s in r["sectors"]]
    out = {"calls": len(recs), "seconds": sum(r["ms"] for r in recs) / 1e3,
           "calls_refining_everything": sum(1 for r in recs if r["lam_cut"] == 0.0),
           "max_levels": max(lev) if lev else 0, "mean_levels": float(np.mean(lev)) if lev else 0.0,
           "slowest_call_ms": max((r["ms"] for r in recs), default=0.0)}
    return out, first_line + len(lines)


def run_sweep(args):
    """DMRG sweeps (dmrg_su2::sweep) of an lx x ly J1-J2(-Q) cylinder at D
    multiplets, every tensor on the device.  The warm-up (do_idmrg), then
    split-precision sweeps: --sweeps-before of them, or with --converge until
    a sweep changes the energy by less than 1e-6 (main_omp's rule, at most
    --max-sweeps).  From that state the next sweep runs twice, with
    split-precision and with FP64 contractions (truncation, Lanczos scalars and
    the tridiagonal problem are FP64 in both), and the two are compared step
    by step (energies) and bond by bond (retained multiplets).  The first sweep
    after the warm-up is no comparison point: the warm-up's basis holds
    rounding-noise Schmidt directions and the engine's own first sweep passes
    through energies far below the ground state.  Wall-clock seconds with the
    device synchronised on both sides (every library call blocks); per-phase
    seconds of each timed sweep; the truncation's own trace (SU2G_SVD_TRACE)."""
    import torch

    from su2dmrg_gb300 import capi
    from su2dmrg_gb300.sweep import Dmrg
    from su2dmrg_gb300.warmup import Lattice

    trace = os.environ.get("SU2G_SVD_TRACE") or os.path.join(tempfile.gettempdir(), "su2g_svd_trace.jsonl")
    os.makedirs(os.path.dirname(trace), exist_ok=True)
    open(trace, "w").close()
    os.environ["SU2G_SVD_TRACE"] = trace
    tline = 0
    capi.lib()
    torch.cuda.set_device(0)
    lx, ly = (int(v) for v in args.lattice.lower().split("x"))
    lat = Lattice.cylinder(lx, ly, args.delta, args.qdelta, args.D)
    split = MODES["split"]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    d = Dmrg(lat, mode=split, seed=args.seed)
    d.offload = args.offload
    last = [0.0]
    if args.step_log:  # one stderr line per sweep step: a run cut short still shows its step times

        def log_step(il, ir, e):
            torch.cuda.synchronize()
            now = time.perf_counter()
            print(json.dumps({"progress": "step", "il": il, "ir": ir, "seconds": now - last[0],
                              "energy_per_site": e / lat.ns, "kept_multiplets": d.truncations[-1][2],
                              "torch_hbm_gb": torch.cuda.memory_allocated() / 1e9,
                              "host_resident_gb": getattr(d, "host_bytes", 0) / 1e9,
                              "phase_seconds": dict(d.phase_seconds)}), file=sys.stderr, flush=True)
            last[0] = now

        d.step_hook = log_step
    e_prev = d.run()
    torch.cuda.synchronize()
    warm_s = time.perf_counter() - t0
    last[0] = time.perf_counter()
    print(json.dumps({"progress": "warmup", "seconds": warm_s, "energy_per_site": e_prev / lat.ns}),
          file=sys.stderr, flush=True)
    e_warm = e_prev
    _, tline = _svd_trace_summary(trace, tline)
    before = []
    nmax = args.max_sweeps if args.converge else args.sweeps_before
    for k in range(nmax):
        d.phase_seconds.clear()
        t0 = time.perf_counter()
        e = d.sweep()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        tsum, tline = _svd_trace_summary(trace, tline)
        before.append({"seconds": dt, "energy_per_site": e / lat.ns, "delta_e": e - e_prev,
                       "phase_seconds": dict(d.phase_seconds), "truncation_trace": tsum,
                       "peak_hbm_gb": torch.cuda.max_memory_allocated() / 1e9})
        print(json.dumps({"progress": "sweep", **before[-1]}), file=sys.stderr, flush=True)
        converged = abs(e - e_prev) < 1e-6
        e_prev = e
        if args.converge and converged:
            break
    nwarm = len(d.energies)
    ntr = len(d.truncations)
    ref_state = None if args.skip_fp64 else d.clone(MODES["f64"])
    torch.cuda.synchronize()
    d.phase_seconds.clear()
    with ClockSampler(torch.cuda.current_device()) as clk:
        t0 = time.perf_counter()
        e_split = d.sweep()
        torch.cuda.synchronize()
        split_s = time.perf_counter() - t0
    tsum_split, tline = _svd_trace_summary(trace, tline)
    steps_split = np.array([e for _, _, e in d.energies[nwarm:]])
    line = {"metric": f"DMRG sweep seconds, {lx}x{ly} J1-J2 cylinder (delta {args.delta}, Q {args.qdelta}), "
                      f"D={args.D}, split-precision contractions",
            "value": split_s, "unit": "s", "n_gpus": 1, "steps": 1, "warmup": 0, "ms_per_step": split_s * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64 emulated by bf16 x7 (fp32 accumulate); FP64 truncation and Lanczos scalars",
            "data": "synthetic (lattice tables built here; " + (
                f"seeded random warm-up start, seed {args.seed})" if args.seed is not None
                else "the uniform warm-up start, as the engine)"),
            "config": {"workload": f"{lx}x{ly} cylinder, boundary 2, D={args.D}, sweep {len(before) + 1} "
                                   f"after the warm-up",
                       "row": "sweep", "two_site_steps": len(steps_split), "warmup_seconds": warm_s,
                       "block_tensors": "host-resident once passed" if args.offload else "device-resident",
                       "warmup_energy_per_site": e_warm / lat.ns, "earlier_sweeps": before,
                       "converged_before_timed_sweep": bool(before and abs(before[-1]["delta_e"]) < 1e-6),
                       "sweep_energy_per_site_split": e_split / lat.ns,
                       "phase_seconds_split": dict(d.phase_seconds), "truncation_trace_split": tsum_split},
            "clocks": clk.summary(), "cpu_baseline": None,
            "cpu_baseline_note": "the reference main_omp cannot run on the GPU host: its sources are not there"}
    if ref_state is not None:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e_f64 = ref_state.sweep()
        torch.cuda.synchronize()
        f64_s = time.perf_counter() - t0
        tsum_f64, tline = _svd_trace_summary(trace, tline)
        steps_f64 = np.array([e for _, _, e in ref_state.energies[nwarm:]])
        rel = np.abs(steps_split - steps_f64) / np.abs(steps_f64)
        line["config"].update({"fp64_sweep_seconds": f64_s, "split_speedup_vs_fp64": f64_s / split_s,
                               "phase_seconds_fp64": dict(ref_state.phase_seconds),
                               "truncation_trace_fp64": tsum_f64,
                               "sweep_energy_per_site_fp64": e_f64 / lat.ns,
                               "max_rel_step_energy_diff_split_vs_fp64": float(rel.max()),
                               "final_rel_energy_diff_split_vs_fp64": float(abs(e_split - e_f64) / abs(e_f64)),
                               "retained_multiplets_split_vs_fp64": _retained_compare(
                                   _bond_dims(d), _bond_dims(ref_state), _discarded_by_site(d, ntr),
                                   _discarded_by_site(ref_state, ntr))})
    line["config"]["peak_hbm_gb"] = torch.cuda.max_memory_allocated() / 1e9
    print(json.dumps(line))
    return 0


def run_serve(args):
    """The serving stream (su2dmrg_gb300.serve.request_stream: seeded Poisson
    arrivals at --rate; per request lx in {6, 8, 10, 12}, ly in {4, 6}, J2/J1 in
    U[0, 1], Q/J1 in U[0, 2], total spin 0 or 1, D in {128, 256, 512}; the
    warm-up and up to 4 sweeps in split mode) served with continuous batching
    (su2dmrg_gb300.serve.Server: --slots solves in flight, admission by
    device footprint, Lanczos solves in shared launches), then the first
    --seq-requests of the same requests one after another on the plain
    per-solve path.  Solves that converged (energy change below 1e-6) in both
    runs must agree to 1e-10 in energy; unconverged early sweeps amplify
    rounding differences between a solve that shared the GPU and one that ran
    alone, so they are reported but not compared.  Wall-clock seconds on the
    host, every library call blocking."""
    import copy

    import torch

    from su2dmrg_gb300 import capi
    from su2dmrg_gb300.serve import Server, request_stream

    capi.lib()
    torch.cuda.set_device(0)
    reqs = request_stream(args.requests, args.rate, seed=42)
    srv = Server(slots=args.slots, mode=MODES["split"], batch=not args.no_batch)
    torch.cuda.synchronize()
    with ClockSampler(0) as clk:
        res = srv.run(reqs)
        torch.cuda.synchronize()
    lat = np.array([r.latency for r in res])
    span = max(r.t_done for r in res) - min(r.t_arrive for r in res)
    recs = []
    for r in res:
        e = r.energies
        de = abs(e[-1] - e[-2]) if len(e) > 1 else None
        recs.append({**r.meta, "sweeps": len(e) - 1, "energy_per_site": e[-1] / reqs[r.rid].lattice.ns,
                     "last_delta_e": de, "converged": de is not None and de < 1e-6,
                     "arrive_s": r.t_arrive, "admit_s": r.t_admit, "done_s": r.t_done,
                     "service_s": r.service, "latency_s": r.latency, "footprint_gb": r.footprint / 1e9})
    seq = None
    k = min(args.seq_requests, len(reqs))
    if k > 0:
        sub = [copy.copy(r) for r in reqs[:k]]
        for r in sub:
            r.arrival = 0.0
        s1 = Server(slots=1, mode=MODES["split"], batch=False)
        t0 = time.perf_counter()
        res1 = s1.run(sub)
        torch.cuda.synchronize()
        total1 = time.perf_counter() - t0
        same = all(a.energies == b.energies and a.mps_desc == b.mps_desc for a, b in zip(res1, res[:k]))
        conv = lambda r: len(r.energies) > 1 and abs(r.energies[-1] - r.energies[-2]) < 1e-6
        pairs = [(a, b) for a, b in zip(res1, res[:k]) if conv(a) and conv(b)]
        close = all(abs(a.energies[-1] - b.energies[-1]) <= 1e-10 * abs(b.energies[-1]) for a, b in pairs)
        maxdiff = max([abs(a.energies[-1] - b.energies[-1]) / abs(b.energies[-1]) for a, b in pairs] or [0.0])
        seq = {"requests": k, "seconds": total1, "solves_per_s": k / total1,
               "mean_service_s": float(np.mean([r.service for r in res1])),
               "results_bit_identical_to_mix": bool(same),
               "converged_in_both": len(pairs),
               "converged_energies_within_1e-10": bool(close),
               "max_rel_converged_energy_diff_vs_mix": float(maxdiff)}
    line = {"metric": "DMRG solves per second (serving stream, one GPU, continuous batching)",
            "value": len(res) / span, "unit": "solves/s", "n_gpus": 1, "steps": len(res), "warmup": 0,
            "ms_per_step": 1e3 * span / len(res), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64 emulated by bf16 x7 (fp32 accumulate); FP64 truncation and Lanczos scalars",
            "data": "synthetic (seeded request stream, lattice tables built here)",
            "config": {"workload": f"serving stream of {len(res)} requests: random J1-J2-Q cylinders, "
                                   "D in {128, 256, 512}, up to 4 sweeps", "row": "serve",
                       "arrival_rate_per_s": args.rate, "seed": 42, "slots": args.slots,
                       "batching": "none (concurrent solves, own launches)" if args.no_batch
                       else "Lanczos solves of concurrent requests in shared launches",
                       "max_in_flight": srv.max_inflight, "max_reserved_gb": srv.max_reserved / 1e9,
                       "hbm_budget_gb": srv.budget / 1e9,
                       "lanczos_batches": len(srv.batch_sizes),
                       "mean_lanczos_batch": float(np.mean(srv.batch_sizes)) if srv.batch_sizes else 0.0,
                       "requests": recs},
            "throughput": {"arrival_span_per_s": len(res) / span,
                           "note": "requests / (last completion - first arrival); equals the arrival rate "
                                   "unless the server saturates",
                           "per_service_second": len(res) / float(sum(r.service for r in res)),
                           "per_service_second_note": "requests / the sum of their service times (each "
                                                      "solve's own start to finish; concurrent solves overlap)"},
            "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                          "max": float(lat.max()), "sample": len(res)},
            "sequential": seq, "clocks": clk.summary(), "cpu_baseline": None}
    print(json.dumps(line))
    return 0


def run_tune(args):
    """The block-size autotuner of the FP64 engine (su2dmrg_gb300.autotune):
    measures the four tile classes on every (M, N) size bucket, installs the
    fastest per bucket, writes the table to --table-out, and times FP64 H_eff
    applications with 64 x 64 tiles only and with the tuned table: synthetic
    two-site steps from small to large blocks (D = 100 .. 2000) and the centre
    step of a real J1-J2 8x4 warm-up at D = 256.  Results are bit-identical
    either way (the tile shape does not change any summation order)."""
    import torch

    from su2dmrg_gb300 import autotune as A
    from su2dmrg_gb300 import capi
    from su2dmrg_gb300 import su2 as S
    from su2dmrg_gb300.sweep import Dmrg
    from su2dmrg_gb300.warmup import Lattice
    from su2dmrg_gb300.workloads import synthetic_heff

    capi.lib()
    torch.cuda.set_device(0)
    A.reset()
    t0 = time.perf_counter()
    table = A.tune()
    tune_s = time.perf_counter() - t0
    if args.table_out:
        A.save(table, args.table_out)

    def time_plan(make, reps):
        out = {}
        for name, tab in (("64x64", None), ("tuned", table)):
            if tab is None:
                A.reset()
            else:
                A.install(tab)
            plan, psi = make()
            y = torch.empty_like(psi)
            for _ in range(2):
                plan.apply(psi, y)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                plan.apply(psi, y)
            e1.record()
            torch.cuda.synchronize()
            out[name] = (e0.elapsed_time(e1) / reps, y.clone(), plan.info()["flops"])
            plan.close()
        same = bool(torch.equal(out["64x64"][1], out["tuned"][1]))
        return {"ms_64x64": out["64x64"][0], "ms_tuned": out["tuned"][0],
                "speedup": out["64x64"][0] / out["tuned"][0], "bit_identical": same,
                "tflops_tuned": out["tuned"][2] / out["tuned"][0] / 1e9}

    rows = {}
    for D in (100, 200, 500, 2000):
        w = synthetic_heff(D=D, nspin1=18, seed=1234)
        dev = w.to_device()

        def make(w=w, dev=dev):
            psi, terms, hl, hr = dev
            return S.HeffPlan(w.psi, terms, hl, hr, mode=MODES["f64"]), psi
        rows[f"synthetic D={D}"] = time_plan(make, 3 if D == 2000 else 20)
    lat = Lattice.cylinder(8, 4, 2.0, 0.0, 256)
    d = Dmrg(lat, mode=MODES["f64"])
    d.run()
    il, ir = lat.ns // 2 - 1, lat.ns // 2
    vs, vx = S.prepare_input_vector(*d.uu[il], *d.uu[ir], mode=MODES["f64"])
    vx = vx[: vs.size()].clone()

    def make_real():
        return d.heff_plan(il, ir, vs), vx
    rows["8x4 J1-J2 D=256 warm-up, centre step"] = time_plan(make_real, 20)
    A.install(table)
    line = {"metric": "FP64 H_eff*psi speed-up of the tuned tile table over 64x64 tiles", "value":
            rows["synthetic D=200"]["speedup"], "unit": "x", "n_gpus": 1, "steps": 20, "warmup": 2,
            "ms_per_step": rows["synthetic D=200"]["ms_tuned"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "FP64 engine tile autotuning; H_eff steps from small to large blocks",
                       "row": "tune", "tune_seconds": tune_s, "table": {k: table[k] for k in
                                                                       ("m_edges", "n_edges", "cls")},
                       "steps": rows},
            "cpu_baseline": None}
    print(json.dumps(line))
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.row == "sweep":
        return run_sweep(args)
    if args.row == "serve":
        return run_serve(args)
    if args.row == "tune":
        return run_tune(args)
    if args.row != "heff":
        return run_row(args)
    return run_su2g(args)


if __name__ == "__main__":
    sys.exit(main())
