"""Builds libsu2g.so in-tree with nvcc/g++ for sm_103a (GB300 only).

Sources are compiled in parallel into su2dmrg_gb300/_build/ and linked into
su2dmrg_gb300/libsu2g.so.  Host C++ is compiled with -ffp-contract=off so the
recoupling-table arithmetic gives the same bits on x86 and Arm hosts.
"""
from __future__ import annotations

import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libsu2g.so")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["capi.cu", "devmem.cu", "heff_batch.cu", "kernels_f64.cu", "ozaki_pack.cu", "ozaki_gemm.cu", "noalloc.cu", "svd.cu", "combine.cu", "wavefunc.cu", "measure.cu"]
CXX_SOURCES = ["su2_meta.cpp", "heff_plan.cpp", "ozaki_plan.cpp", "env_plan.cpp", "checkpoint.cpp"]
LINK_LIBS = ["-lcudart", "-lcusolver", "-lpthread"]


def _headers():
    hs = [os.path.join(REPO, "include", "su2g.h")]
    for f in os.listdir(CSRC):
        if f.endswith((".hpp", ".cuh", ".h")):
            hs.append(os.path.join(CSRC, f))
    return hs


def _stale(obj, src, headers):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src, *headers])


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile (if needed) and return the path of libsu2g.so."""
    os.makedirs(BUILD, exist_ok=True)
    headers = _headers()
    inc = ["-I", os.path.join(REPO, "include"), "-I", CSRC]
    jobs, objs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, s, headers):
            cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                   "--expt-relaxed-constexpr", *inc, "-c", s, "-o", o]
            jobs.append((cmd, src))
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, s, headers):
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall",
                   "-I", os.path.join(CUDA_HOME, "include"), *inc, "-c", s, "-o", o]
            jobs.append((cmd, src))
    procs = [(subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT), src) for cmd, src in jobs]
    failed = []
    for p, src in procs:
        out, _ = p.communicate()
        if verbose or p.returncode != 0:
            sys.stderr.write(out.decode(errors="replace"))
        if p.returncode != 0:
            failed.append(src)
    if failed:
        raise RuntimeError(f"libsu2g build failed for: {', '.join(failed)}")
    if force or jobs or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-cudart", "shared",
               "-Xlinker", f"-rpath,{os.path.join(CUDA_HOME, 'lib64')}", *LINK_LIBS]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            sys.stderr.write(r.stdout.decode(errors="replace"))
            raise RuntimeError("libsu2g link failed")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
