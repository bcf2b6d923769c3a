"""The allocation-free H_eff entry point
(su2g_hamiltonian_vector_multiplication_noalloc), called through the C ABI.

It serves callers that may not allocate device memory when they apply a term
(engines that reserve all of HBM up front, many host threads calling per term
where cudaMalloc/cudaFree would synchronise the device, code inside another
library's callbacks).  Its output must match the allocating entry point,
su2g_hamiltonian_vector_multiplication, to the 1e-12 relative tolerance the
other H_eff tests use, on consecutive calls that reuse its fixed device
arrays, and terms larger than those arrays must be refused.  This file runs
last (pytest collects it last) and passes alone or after the other tests."""
import ctypes
import glob
import os
import warnings

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _pinned(struct):
    d = np.ascontiguousarray(struct.desc(), np.int32)
    f = np.ascontiguousarray(struct.flag, np.int32)
    return d, f


def _call(fn, vs, vx, s1, x1, s2, x2, y, stream):
    from su2dmrg_gb300 import capi

    vd, vf = _pinned(vs)
    d1, f1 = _pinned(s1)
    d2, f2 = _pinned(s2)
    t1 = capi.Tensor(d1.ctypes.data, f1.ctypes.data, capi.ptr(x1))
    t2 = capi.Tensor(d2.ctypes.data, f2.ctypes.data, capi.ptr(x2))
    return fn(vd.ctypes.data, vf.ctypes.data, capi.ptr(vx), t1, t2, capi.ptr(y), stream)


def _cases(torch, oracle):
    from su2dmrg_gb300.workloads import synthetic_heff

    out = []
    g = np.load(sorted(glob.glob(os.path.join(GOLDEN, "heff_term_*.npz")))[3])
    out.append((oracle.struct_from_desc(g["vdesc"], g["vflag"]), g["vx"], oracle.struct_from_desc(g["d1"], g["f1"]),
                g["x1"], oracle.struct_from_desc(g["d2"], g["f2"]), g["x2"]))
    w = synthetic_heff(D=400, nspin1=1, seed=21, spin0=False)
    s1, x1, s2, x2, _ = w.terms[0]
    out.append((w.psi, w.psi_data, s1, x1, s2, x2))
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float64)).cuda()
    return [(vs, dev(vx), a, dev(xa), b, dev(xb)) for (vs, vx, a, xa, b, xb) in out]


def test_noalloc_matches_allocating_entry_point(su2lib, oracle):
    import torch

    from su2dmrg_gb300 import capi

    L = capi.lib()
    stream = torch.cuda.current_stream().cuda_stream
    cases = _cases(torch, oracle)
    # two calls in a row on different terms, then the first again: the shared
    # device arrays carry the previous call's contents into the next call
    for (vs, vx, s1, x1, s2, x2) in cases + cases[:1]:
        y_ref = torch.zeros_like(vx)
        y_na = torch.full_like(vx, np.nan)
        capi.check(_call(L.su2g_hamiltonian_vector_multiplication, vs, vx, s1, x1, s2, x2, y_ref, stream))
        capi.check(_call(L.su2g_hamiltonian_vector_multiplication_noalloc, vs, vx, s1, x1, s2, x2, y_na, stream))
        torch.cuda.synchronize()
        ref = y_ref.cpu().numpy()
        got = y_na.cpu().numpy()
        assert np.all(np.isfinite(got))
        assert np.linalg.norm(ref) > 0
        assert np.linalg.norm(got - ref) <= TOL * np.linalg.norm(ref)


def test_noalloc_matches_reference_output(su2lib, oracle):
    """Against the reference's own tensor_su2::hamiltonian_vector_multiplication
    output stored with the fixture (rx), on two calls in a row."""
    import torch

    from su2dmrg_gb300 import capi

    L = capi.lib()
    stream = torch.cuda.current_stream().cuda_stream
    g = np.load(sorted(glob.glob(os.path.join(GOLDEN, "heff_term_*.npz")))[3])
    vs = oracle.struct_from_desc(g["vdesc"], g["vflag"])
    s1 = oracle.struct_from_desc(g["d1"], g["f1"])
    s2 = oracle.struct_from_desc(g["d2"], g["f2"])
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float64)).cuda()
    ref = oracle.to_layout(oracle.struct_from_desc(g["vdesc"], g["rflag"]), g["rx"], vs)
    vx, x1, x2 = dev(g["vx"]), dev(g["x1"]), dev(g["x2"])
    for _ in range(2):
        y = torch.full_like(vx, np.nan)
        capi.check(_call(L.su2g_hamiltonian_vector_multiplication_noalloc, vs, vx, s1, x1, s2, x2, y, stream))
        torch.cuda.synchronize()
        got = y.cpu().numpy()
        assert np.linalg.norm(got - ref) <= TOL * np.linalg.norm(ref)


def test_noalloc_threads_sharing_one_stream(su2lib, oracle):
    """Host threads that call the entry point on one shared stream (the
    reference's OpenMP loop over terms, each thread applying its own term)
    get their own results: every call queues its copies and launches as one
    group, so stream order keeps the shared arrays apart."""
    import threading

    import torch

    from su2dmrg_gb300 import capi

    L = capi.lib()
    stream = torch.cuda.Stream()
    sid = stream.cuda_stream
    cases = _cases(torch, oracle)
    torch.cuda.synchronize()
    refs = []
    for (vs, vx, s1, x1, s2, x2) in cases:
        y = torch.zeros_like(vx)
        capi.check(_call(L.su2g_hamiltonian_vector_multiplication, vs, vx, s1, x1, s2, x2, y, sid))
        refs.append(y)
    stream.synchronize()
    nthreads, rounds = 4, 6
    outs = [[torch.full_like(cases[t % len(cases)][1], np.nan) for _ in range(rounds)] for t in range(nthreads)]
    codes = [[None] * rounds for _ in range(nthreads)]
    go = threading.Barrier(nthreads)

    def work(t):
        vs, vx, s1, x1, s2, x2 = cases[t % len(cases)]
        go.wait()
        for r in range(rounds):
            codes[t][r] = _call(L.su2g_hamiltonian_vector_multiplication_noalloc, vs, vx, s1, x1, s2, x2,
                                outs[t][r], sid)

    th = [threading.Thread(target=work, args=(t,)) for t in range(nthreads)]
    for x in th:
        x.start()
    for x in th:
        x.join()
    stream.synchronize()
    for t in range(nthreads):
        ref = refs[t % len(cases)].cpu().numpy()
        for r in range(rounds):
            assert codes[t][r] == capi.SU2G_OK
            got = outs[t][r].cpu().numpy()
            assert np.linalg.norm(got - ref) <= TOL * np.linalg.norm(ref)


def test_noalloc_refuses_terms_beyond_its_arrays(su2lib):
    """A single D=2000 spin-1 term needs about 4.3M doubles of intermediate
    blocks, more than the fixed 4,194,304: refused before any device work."""
    import torch

    from su2dmrg_gb300 import capi
    from su2dmrg_gb300.workloads import synthetic_heff

    L = capi.lib()
    w = synthetic_heff(D=2000, nspin1=1, seed=3, spin0=False)
    s1, x1, s2, x2, _ = w.terms[0]
    y = np.zeros(1)
    rc = _call(L.su2g_hamiltonian_vector_multiplication_noalloc, w.psi, w.psi_data, s1, x1, s2, x2, y,
               torch.cuda.current_stream().cuda_stream)
    assert rc == capi.SU2G_EINVAL
    assert b"noalloc" in L.su2g_last_error()


def test_noalloc_refuses_stream_capture(su2lib, oracle):
    """The work list is copied from host memory that is freed on return, so a
    captured call could only replay from freed memory: on a capturing stream
    the entry point returns SU2G_EUNSUPPORTED and queues nothing."""
    import torch

    from su2dmrg_gb300 import capi

    L = capi.lib()
    vs, vx, s1, x1, s2, x2 = _cases(torch, oracle)[0]
    y = torch.zeros_like(vx)
    fn = L.su2g_hamiltonian_vector_multiplication_noalloc
    capi.check(_call(fn, vs, vx, s1, x1, s2, x2, y, torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    side = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    codes = []
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")  # the graph stays empty: nothing was queued
        with torch.cuda.graph(g, stream=side):
            codes.append(_call(fn, vs, vx, s1, x1, s2, x2, y, side.cuda_stream))
    assert codes == [capi.SU2G_EUNSUPPORTED]
    assert "captured" in L.su2g_last_error().decode()
