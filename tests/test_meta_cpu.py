"""libsu2g.so host entry points (no GPU needed): integer bookkeeping and the
recoupling tables must be bit-exact with the reference; the C ABI exports
every symbol include/su2g.h declares."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, REPO


def test_exports_match_header(su2lib):
    hdr = open(os.path.join(REPO, "include", "su2g.h")).read()
    declared = sorted(set(re.findall(r"\b(su2g_[a-z0-9_]+)\s*\(", hdr)))
    so = os.path.join(REPO, "su2dmrg_gb300", "libsu2g.so")
    out = subprocess.run(["nm", "-D", "--defined-only", so], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r" T (su2g_[a-z0-9_]+)$", out, re.M))
    missing = [d for d in declared if d not in exported]
    assert not missing, missing
    for d in declared:
        assert hasattr(su2lib, d)
    from su2dmrg_gb300 import capi

    assert sorted(capi.EXPORTED) == declared


def test_fac_table_bit_exact(su2lib):
    from su2dmrg_gb300.su2 import fac_hamilt_vec

    ref = np.load(os.path.join(GOLDEN, "fac_hamilt_vec.npy"))
    assert np.array_equal(fac_hamilt_vec(25), ref)


def test_cgc_bit_exact(su2lib):
    from su2dmrg_gb300.su2 import make_cgc

    g = np.load(os.path.join(GOLDEN, "cgc.npz"))
    for n, (j1, j2, j3) in enumerate(g["triples"]):
        assert np.array_equal(make_cgc(int(j1), int(j2), int(j3)), g["values"][g["idx"][n]: g["idx"][n + 1]])


def test_fuse_and_legality(su2lib):
    from su2dmrg_gb300.su2 import Su2Bond, Su2Struct

    g = np.load(os.path.join(GOLDEN, "meta.npz"))
    fin, idx = g["fuse_in"], g["fuse_in_idx"]
    for c in range(len(idx) - 1):
        v = fin[idx[c]: idx[c + 1]].tolist()
        n1 = v[0]
        a1, d1 = v[1: 1 + n1], v[1 + n1: 1 + 2 * n1]
        n2 = v[1 + 2 * n1]
        a2, d2 = v[2 + 2 * n1: 2 + 2 * n1 + n2], v[2 + 2 * n1 + n2:]
        f = Su2Bond(1, a1, d1).fuse(Su2Bond(1, a2, d2))
        assert f.angm == g["fuse_out_a"][g["fuse_out_idx"][c]: g["fuse_out_idx"][c + 1]].tolist()
        assert f.dim == g["fuse_out_d"][g["fuse_out_idx"][c]: g["fuse_out_idx"][c + 1]].tolist()
        assert f.dir == -1
    d, di, fl, fi = g["legal_desc"], g["legal_desc_idx"], g["legal_flag"], g["legal_flag_idx"]
    for c in range(len(di) - 1):
        desc = np.ascontiguousarray(d[di[c]: di[c + 1]], np.int32)
        out = np.zeros(fi[c + 1] - fi[c], np.int32)
        assert su2lib.su2g_struct_legal(desc.ctypes.data, out.ctypes.data) == len(out)
        assert out.tolist() == fl[fi[c]: fi[c + 1]].tolist()


def test_layout_offsets(su2lib):
    from su2dmrg_gb300.su2 import Su2Bond, Su2Struct

    s = Su2Struct([Su2Bond(-1, [0, 1, 2], [3, 4, 5]), Su2Bond(-1, [0, 1, 2], [2, 6, 7])], 0).with_legal_flags()
    assert s.flag.tolist() == [1, 0, 0, 0, 1, 0, 0, 0, 1]
    off, total = s.offsets()
    assert off.tolist() == [0, -1, -1, -1, 6, -1, -1, -1, 30]
    assert total == 6 + 24 + 35


def test_malformed_inputs_rejected(su2lib):
    bad = np.asarray([7, 0], np.int32)  # 7 legs
    assert su2lib.su2g_struct_nten(bad.ctypes.data) == -1
    unsorted = np.asarray([1, 0, -1, 2, 3, 1, 5, 5], np.int32)
    assert su2lib.su2g_struct_nten(unsorted.ctypes.data) == -1
    from su2dmrg_gb300 import capi

    out = np.zeros(8)
    assert su2lib.su2g_make_cgc(-1, 0, 0, out.ctypes.data) == capi.SU2G_EINVAL
    assert b"make_cgc" in su2lib.su2g_last_error()


def test_plan_validation_without_gpu(su2lib):
    """Structure mismatches are reported as SU2G_EINVAL before any device work."""
    from su2dmrg_gb300 import capi
    from su2dmrg_gb300.su2 import HeffPlan, Su2Bond, Su2Struct

    e = Su2Bond(-1, [0, 1, 2], [2, 3, 2])
    psi = Su2Struct([e, e], 0).with_legal_flags()
    other = Su2Bond(1, [0, 1, 2], [2, 9, 2])  # wrong dims
    op = Su2Struct([other, Su2Bond(1, [2], [1]), e], 0).with_legal_flags()
    x = np.zeros(op.size())
    with pytest.raises(capi.Su2gError) as ei:
        HeffPlan(psi, [(op, x, op, x, 1.0)])
    assert ei.value.code == capi.SU2G_EINVAL


@pytest.mark.parametrize("D,nspin1", [(60, 3), (2000, 18)])
def test_work_list_bounds_on_cpu(su2lib, D, nspin1):
    """Every element access of the H_eff kernels, at the benchmark shape,
    checked against the blocks it belongs to before anything runs on a GPU."""
    from su2dmrg_gb300.su2 import HeffPlan
    from su2dmrg_gb300.workloads import synthetic_heff

    w = synthetic_heff(D=D, nspin1=nspin1, seed=1234)
    r = HeffPlan.validate(w.psi, w.terms, w.hl, w.hr)
    assert r["flops"] > 0 and r["scratch_bytes"] > 0
    if D == 2000:
        # algorithmic FLOPs of the width-20 D=2000 step (18 spin-1 pairs + 2 spin-0)
        assert 1.0e11 < r["flops"] < 2.0e11


def test_golden_cases_build_valid_work_lists(su2lib, oracle):
    """The reference's golden H_eff inputs produce bounds-checked work lists
    (host dry run), with the oracle's structures passed straight through."""
    import glob

    from su2dmrg_gb300.su2 import HeffPlan

    for path in sorted(glob.glob(os.path.join(GOLDEN, "heff_term_*.npz"))):
        g = np.load(path)
        vs = oracle.struct_from_desc(g["vdesc"], g["vflag"])
        s1 = oracle.struct_from_desc(g["d1"], g["f1"])
        s2 = oracle.struct_from_desc(g["d2"], g["f2"])
        r = HeffPlan.validate(vs, [(s1, g["x1"], s2, g["x2"], 1.0)])
        prob = oracle.HeffProblem(vs, [(s1, g["x1"], s2, g["x2"], 1.0)])
        assert r["flops"] == oracle.heff_flops(prob)


@pytest.mark.parametrize("mode", [1, 2])
def test_split_work_lists_on_cpu(su2lib, mode):
    """Split-precision pack jobs and tiles at the benchmark shape, bounds
    checked on the host (no GPU)."""
    from su2dmrg_gb300.su2 import HeffPlan
    from su2dmrg_gb300.workloads import synthetic_heff

    w = synthetic_heff(D=2000, nspin1=18, seed=1234)
    r = HeffPlan.validate(w.psi, w.terms, w.hl, w.hr, mode=mode)
    assert r["scratch_bytes"] > 2e9  # packed operator slices + intermediates


def test_env_layouts_match_reference(su2lib, oracle):
    """Output structures of the transformations (which blocks exist), host only."""
    import glob

    from su2dmrg_gb300.su2 import operator_transformation_layout, overlap_transformation_layout

    for path in sorted(glob.glob(os.path.join(GOLDEN, "env_*.npz"))):
        g = np.load(path)
        su = oracle.struct_from_desc(g["du"], g["fu"])
        so = oracle.struct_from_desc(g["dop"], g["fop"])
        fn = overlap_transformation_layout if "env_ovl" in path else operator_transformation_layout
        out = fn(su, g["xu"], su, g["xv"], so, g["xop"], int(g["flag"]))
        assert out.flag.tolist() == g["rflag"].tolist(), path
        assert out.size() == g["rx"].size


def test_svd_argument_checks_without_gpu(su2lib):
    """su2g_svd rejects a psi whose legs are not the fused legs of tu / tv, and
    bad arguments, with SU2G_EINVAL before any device work."""
    import ctypes

    from su2dmrg_gb300 import capi

    g = np.load(os.path.join(GOLDEN, "svd_0.npz"))
    dvec, fvec, du, dv = (np.ascontiguousarray(g[k], np.int32) for k in ("dvec", "fvec", "du", "dv"))
    bond = np.zeros(256, np.int32)
    wout = np.zeros(4096)
    dout = ctypes.c_int()

    def call(d_u, d_v, dcut=10, wcap=4096):
        return su2lib.su2g_svd(dvec.ctypes.data, fvec.ctypes.data, 8, d_u.ctypes.data, 1.0, d_v.ctypes.data, 0.0,
                               dcut, bond.ctypes.data, len(bond), wout.ctypes.data, wcap, ctypes.addressof(dout),
                               None, 0, None, 0, None)

    bad = du.copy()
    bad[4 + bad[3]] += 1  # first multiplet dim of tu leg 0
    assert call(bad, dv) == capi.SU2G_EINVAL
    assert b"fused" in su2lib.su2g_last_error()
    assert call(du, dv, dcut=-1) == capi.SU2G_EINVAL
    two_leg = dvec.copy()
    assert call(two_leg, dv) == capi.SU2G_EINVAL


def test_fac_site_tables_match_reference(su2lib):
    """The library's onsite / pairup / permutation recoupling factors against
    the reference's own tables (1e-14 relative: the reference forms them with
    BLAS contractions, summation order unpinned)."""
    import ctypes

    g = np.load(os.path.join(GOLDEN, "fac_site.npz"))
    out = ctypes.c_double()
    for r, v in zip(g["idx"], g["val"]):
        assert su2lib.su2g_fac_table(*[int(x) for x in r], ctypes.addressof(out)) == 0
        assert abs(out.value - v) <= 1e-14 * abs(v), (r, out.value, v)
    assert su2lib.su2g_fac_table(3, 0, 0, 0, 0, 0, 0, ctypes.addressof(out)) != 0


def test_site_update_layouts_match_reference(su2lib, oracle):
    """Which blocks operator_initial / operator_pairup / permutation create
    (host only: the layout pass reads no device data)."""
    import glob

    from su2dmrg_gb300.su2 import env_layout

    for path in sorted(glob.glob(os.path.join(GOLDEN, "site_*.npz"))):
        g = np.load(path)
        su = oracle.struct_from_desc(g["du"], g["fu"])
        kind = str(g["kind"])
        kind = "init" if kind.startswith("init") else ("pair" if kind == "pair" else "perm")
        job = {"kind": kind}
        if "dx" in g.files:
            job["x"] = (oracle.struct_from_desc(g["dx"], g["fx"]), g["xx"])
        for i in range(2):
            if f"ds{i}" in g.files:
                job[f"site{i + 1}"] = (oracle.struct_from_desc(g[f"ds{i}"], g[f"fs{i}"]), g[f"xs{i}"])
        out = env_layout(su, g["xu"], su, g["xv"], int(g["flag"]), [job])
        assert out.desc().tolist() == g["rdesc"].tolist(), path
        assert out.flag.tolist() == g["rflag"].tolist(), path
        assert out.size() == g["rx"].size, path


@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("flag", [0, 1])
def test_site_step_work_lists_on_cpu(su2lib, oracle, flag, mode):
    """The batched site step of the GPU tests, built and bounds-checked on
    the host in every mode (the split planner's tile cuts included)."""
    from test_site_gpu import job_dicts, site_step_case

    from su2dmrg_gb300.su2 import env_validate

    su, xu, xv, jobs, _ = site_step_case(oracle, flag)
    r = env_validate(su, xu, su, xv, flag, job_dicts(jobs), mode=mode)
    assert r["flops"] > 1e7 and r["scratch_bytes"] > 0


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_idmrg_work_lists_on_cpu(su2lib, oracle, mode):
    """The engine's own two-site H_eff terms (plaquette and scalar pairs
    included) build and bounds-check as one plan in every mode (host only)."""
    import glob

    import idmrg_case

    from su2dmrg_gb300.su2 import HeffPlan

    for path in sorted(glob.glob(os.path.join(GOLDEN, "idmrg_*.npz"))):
        g = np.load(path)
        vs, vx, yref, _, T, terms, hl, hr = idmrg_case.load(oracle, g)
        tl = []
        for coef, left, right in terms:
            L, R = idmrg_case.combine_host(oracle, T, left), idmrg_case.combine_host(oracle, T, right)
            tl.append((L[0], L[1], R[0], R[1], coef))
        r = HeffPlan.validate(vs, tl, (hl[0], hl[1], 1.0), (hr[0], hr[1], 1.0), mode=mode)
        assert r["flops"] > 0


def _su2(oracle_struct_desc, flags):
    from su2dmrg_gb300.su2 import _parse_desc

    s = _parse_desc(oracle_struct_desc)
    s.flag = np.ascontiguousarray(flags, np.int32)
    return s


@pytest.mark.parametrize("ci", [0, 1, 2])
def test_input_vector_layout_matches_reference(su2lib, ci):
    """su2g_input_vector_layout gives the reference's vec structure: fused
    legs, every equal-spin block present (makeup_input_vector)."""
    from su2dmrg_gb300.su2 import input_vector_layout

    g = np.load(os.path.join(GOLDEN, f"inputvec_{ci}.npz"))
    s = input_vector_layout(_su2(g["dl"], g["fl"]), _su2(g["dr"], g["fr"]))
    assert s.desc().tolist() == g["rdesc"].tolist()
    assert s.flag.tolist() == g["rflag"].tolist()
    assert s.size() == len(g["rx"])


@pytest.mark.parametrize("ci", [0, 1, 2])
@pytest.mark.parametrize("direction", [0, 1])
def test_vectran_layout_matches_reference(su2lib, ci, direction):
    from su2dmrg_gb300.su2 import vectran_layout

    g = np.load(os.path.join(GOLDEN, f"vectran_{ci}_{direction}.npz"))
    s = vectran_layout(_su2(g["du"], g["fu"]), direction)
    assert s.desc().tolist() == g["rdesc"].tolist()
    assert s.flag.tolist() == g["rflag"].tolist()


def test_wavefunc_argument_checks_without_gpu(su2lib):
    """Structures the reference refuses (fuse of legs of different
    directions) and a bad vectran flag give SU2G_EINVAL before any device
    work; the vector's structure does not depend on the centre bonds (every
    block of equal spins, makeup_input_vector), so differing ones are refused
    only by the product (tests/test_wavefunc_gpu.py)."""
    from su2dmrg_gb300 import capi
    from su2dmrg_gb300.capi import Su2gError as CheckError
    from su2dmrg_gb300.su2 import input_vector_layout, vectran_layout

    g = np.load(os.path.join(GOLDEN, "inputvec_0.npz"))
    ul, ur = _su2(g["dl"], g["fl"]), _su2(g["dr"], g["fr"])
    bad = _su2(g["dl"], g["fl"])
    bad.bonds[1] = bad.bonds[1].inverted()
    with pytest.raises(CheckError, match="directions"):
        input_vector_layout(bad, ur)
    other = _su2(g["dr"], g["fr"])
    b2 = other.bonds[2]
    other.bonds[2] = type(b2)(b2.dir, list(b2.angm), [d + 1 for d in b2.dim])
    a, b = input_vector_layout(ul, other), input_vector_layout(ul, ur)
    assert a.desc().tolist() == b.desc().tolist() and np.array_equal(a.flag, b.flag)
    with pytest.raises(CheckError, match="flag"):
        vectran_layout(ul, 2)
    assert capi.SU2G_EINVAL == 1


def test_fuse_tensor_layout_matches_reference(su2lib):
    """tensor_su2::fuse(b1, b2): legs, every legal block present."""
    from su2dmrg_gb300 import su2 as S

    g = np.load(os.path.join(GOLDEN, "fuse_tensor.npz"))
    for i in range(2):
        b = S._parse_desc(g[f"bonds{i}"]).bonds
        s = S.fuse_tensor_layout(b[0], b[1])
        assert s.desc().tolist() == g[f"desc{i}"].tolist()
        assert s.flag.tolist() == g[f"flag{i}"].tolist()
        assert s.size() == len(g[f"x{i}"])


def test_cgc_orthonormal_up_to_the_fuse_cap(su2lib):
    """The recoupling coefficients extend past the engine's 2j < 25 tables to
    the fuse cap 2j = 38 (a large-D warm-up reaches such bonds): the
    Clebsch-Gordan tensors they are built from stay orthonormal there."""
    import ctypes

    def cgc(j1, j2, j3):
        out = np.zeros((j1 + 1) * (j2 + 1) * (j3 + 1))
        assert su2lib.su2g_make_cgc(j1, j2, j3, out.ctypes.data_as(ctypes.c_void_p)) == 0
        return out.reshape(j3 + 1, j2 + 1, j1 + 1)

    worst = 0.0
    for j1, j2 in [(24, 2), (31, 2), (38, 2), (37, 1), (34, 6), (20, 20)]:
        rows = {j3: cgc(j1, j2, j3) for j3 in range(abs(j1 - j2), min(j1 + j2, 38) + 1, 2)}
        for j3, C in rows.items():
            for m3 in range(-j3, j3 + 1, 2):
                a = C[(m3 + j3) // 2]
                worst = max(worst, abs(float(np.sum(a * a)) - 1.0))
                for j3b, Cb in rows.items():
                    if j3b > j3:
                        worst = max(worst, abs(float(np.sum(a * Cb[(m3 + j3b) // 2]))))
    assert worst < 1e-14


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    """No CPU fallback: without the built CUDA library every entry point
    raises instead of computing anything."""
    from su2dmrg_gb300 import capi

    monkeypatch.setattr(capi, "_lib", None)
    monkeypatch.setattr(capi, "LIB_PATH", str(tmp_path / "libsu2g.so"))
    with pytest.raises(RuntimeError, match="is not built"):
        capi.lib()
