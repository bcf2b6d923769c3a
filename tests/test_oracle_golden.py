"""The CPU oracle (oracle/su2_oracle.c) against fixtures produced by the
reference itself (tests/golden/gen_golden.py).  These pin the oracle before any
GPU result is compared with it."""
import glob
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from svd_checks import check_mps, check_truncation_values


def test_fac_hamilt_vec_bit_exact(oracle):
    ref = np.load(os.path.join(GOLDEN, "fac_hamilt_vec.npy"))
    got = oracle.fac_hamilt_vec(25)
    assert np.array_equal(got, ref), np.abs(got - ref).max()
    assert np.count_nonzero(ref) > 1000


def test_make_cgc_bit_exact(oracle):
    g = np.load(os.path.join(GOLDEN, "cgc.npz"))
    for n, (j1, j2, j3) in enumerate(g["triples"]):
        ref = g["values"][g["idx"][n]: g["idx"][n + 1]]
        got = oracle.make_cgc(int(j1), int(j2), int(j3))
        assert np.array_equal(got, ref), (j1, j2, j3)


def test_fuse_matches_reference(oracle):
    g = np.load(os.path.join(GOLDEN, "meta.npz"))
    fin, idx = g["fuse_in"], g["fuse_in_idx"]
    oa, od, oidx = g["fuse_out_a"], g["fuse_out_d"], g["fuse_out_idx"]
    for c in range(len(idx) - 1):
        v = fin[idx[c]: idx[c + 1]].tolist()
        n1 = v[0]
        a1, d1 = v[1: 1 + n1], v[1 + n1: 1 + 2 * n1]
        n2 = v[1 + 2 * n1]
        a2, d2 = v[2 + 2 * n1: 2 + 2 * n1 + n2], v[2 + 2 * n1 + n2:]
        f = oracle.fuse(oracle.Bond(1, a1, d1), oracle.Bond(1, a2, d2))
        assert f.angm == oa[oidx[c]: oidx[c + 1]].tolist()
        assert f.dim == od[oidx[c]: oidx[c + 1]].tolist()


def test_legality_matches_reference(oracle):
    g = np.load(os.path.join(GOLDEN, "meta.npz"))
    d, di, f, fi = g["legal_desc"], g["legal_desc_idx"], g["legal_flag"], g["legal_flag_idx"]
    for c in range(len(di) - 1):
        s = oracle.struct_from_desc(d[di[c]: di[c + 1]])
        assert s.legal().tolist() == f[fi[c]: fi[c + 1]].tolist()


def _singlet_cg_ok(oracle, s, rflag, rcg):
    """Every result block carries the canonical singlet CG (so comparing the
    reduced blocks alone is comparing the tensors)."""
    pos = 0
    for i in range(s.nten):
        if not rflag[i]:
            continue
        ja, jb = s.block_angm(i)
        n = (ja + 1) * (jb + 1)
        cg = rcg[pos: pos + n].reshape(ja + 1, jb + 1, order="F")
        pos += n
        sing = np.zeros((ja + 1, ja + 1))
        for r in range(ja + 1):
            m = 2 * r - ja
            sing[r, ja - r] = (1 if ((ja - m) // 2) % 2 == 0 else -1) / np.sqrt(ja + 1)
        assert ja == jb and np.allclose(cg, sing, atol=1e-14)


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "heff_term_*.npz"))))
def test_heff_term_matches_reference(oracle, path):
    g = np.load(path)
    vs = oracle.struct_from_desc(g["vdesc"], g["vflag"])
    s1 = oracle.struct_from_desc(g["d1"], g["f1"])
    s2 = oracle.struct_from_desc(g["d2"], g["f2"])
    y = np.zeros_like(g["vx"])
    oracle.heff_term(vs, g["vx"], s1, g["x1"], s2, g["x2"], vs, y)
    rs = oracle.struct_from_desc(g["vdesc"], g["rflag"])
    _singlet_cg_ok(oracle, rs, g["rflag"], g["rcg"])
    ref = oracle.to_layout(rs, g["rx"], vs)
    assert np.linalg.norm(ref) > 0
    assert np.linalg.norm(y - ref) <= 1e-13 * np.linalg.norm(ref)


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "spin0_*.npz"))))
def test_spin0_matches_reference(oracle, path):
    g = np.load(path)
    vs = oracle.struct_from_desc(g["vdesc"], g["vflag"])
    hs = oracle.struct_from_desc(g["hdesc"], g["hflag"])
    y = np.zeros_like(g["vx"])
    oracle.heff_spin0(int(g["side"]), hs, g["hx"], vs, g["vx"], vs, y)
    rs = oracle.struct_from_desc(g["vdesc"], g["rflag"])
    _singlet_cg_ok(oracle, rs, g["rflag"], g["rcg"])
    ref = oracle.to_layout(rs, g["rx"], vs)
    assert np.linalg.norm(y - ref) <= 1e-13 * np.linalg.norm(ref)


def test_dsort2_and_ran_restatement(oracle):
    """The C restatement of sort2.f / ran.f90 (oracle/fhelpers.c): ascending
    order with the companion array permuted alongside, and a deterministic
    LCG stream in (0,1)."""
    import ctypes

    L = oracle.lib()
    a = np.array([3.0, 1.0, 2.0, 1.0, 5.0, 0.5], np.float64)
    b = np.arange(6, dtype=np.int32)
    n = ctypes.c_int(6)
    L.dsort2_(ctypes.byref(n), a.ctypes.data_as(ctypes.c_void_p), b.ctypes.data_as(ctypes.c_void_p))
    assert a.tolist() == sorted([3.0, 1.0, 2.0, 1.0, 5.0, 0.5])
    assert sorted(b.tolist()) == list(range(6))
    assert all(np.array([3.0, 1.0, 2.0, 1.0, 5.0, 0.5])[b] == a)
    L.ran_.restype = ctypes.c_double
    seed = ctypes.c_int(12345)
    L.initran_(ctypes.byref(seed))
    xs = [L.ran_() for _ in range(1000)]
    L.initran_(ctypes.byref(seed))
    assert xs == [L.ran_() for _ in range(1000)]
    assert 0 < min(xs) and max(xs) < 1 and abs(np.mean(xs) - 0.5) < 0.05


def test_dmrg_energies_match_exact_diagonalisation():
    """The reference runs recorded in the fixtures converge to the exact lowest
    energies of the small lattices in their spin sector (E0 - 1000 is what
    the reference prints; the triplet value from exact diagonalisation with
    total spin measured)."""
    path = os.path.join(GOLDEN, "dmrg_energies.json")
    if not os.path.exists(path):
        pytest.skip("dmrg_energies.json not generated")
    runs = json.load(open(path))
    # (lx, ly, jcoup, qcoup, 2S): exact lowest energy of the spin-S sector
    exact = {(4, 2, 0.5, 0.0, 0): -3.296960690549784, (3, 4, 0.5, 0.0, 0): -6.762720424674632,
             (3, 4, 0.5, 1.0, 0): -10.228711857181608, (4, 2, 0.5, 0.0, 2): -2.7500783569326157}
    seen = 0
    for r in runs:
        key = (r["lx"], r["ly"], r["jcoup"], r["qcoup"], r["sec"])
        if key in exact:
            assert abs(r["energies_minus_1000"][-1] + 1000 - exact[key]) < 1e-8
            seen += 1
    assert seen == 4


def test_fac_operator_transformation_matches_reference(oracle):
    g = np.load(os.path.join(GOLDEN, "fac_optrans.npz"))
    for r, v in zip(g["idx"], g["val"]):
        got = oracle.fac_operator_transformation(*[int(x) for x in r])
        assert abs(got - v) <= 1e-14 * abs(v), (r, got, v)


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "env_*.npz"))))
def test_env_transform_matches_reference(oracle, path):
    g = np.load(path)
    kind = 0 if "env_ovl" in path else 1
    su = oracle.struct_from_desc(g["du"], g["fu"])
    so = oracle.struct_from_desc(g["dop"], g["fop"])
    out, y = oracle.env_transform(kind, su, g["xu"], su, g["xv"], so, g["xop"], int(g["flag"]))
    assert out.flag.tolist() == g["rflag"].tolist()  # the same blocks exist
    assert np.linalg.norm(y - g["rx"]) <= 1e-13 * np.linalg.norm(g["rx"])


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "svd_*.npz"))))
def test_truncation_matches_reference(oracle, path):
    """Kept multiplets per sector exactly; singular values as
    check_truncation_values states."""
    g = np.load(path)
    vs = oracle.struct_from_desc(g["dvec"], g["fvec"])
    dims, wout, uv = oracle.svd_truncate(vs, g["xvec"], float(g["p1"]), float(g["p2"]), int(g["dcut"]))
    kept = np.zeros(64, np.int32)
    for i, d in enumerate(dims):
        kept[vs.bonds[0].angm[i]] = d
    assert kept.tolist() == g["kept"].tolist()
    check_truncation_values(wout, g["wout"], int(g["kept"].sum()))


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "svd_*.npz"))))
def test_truncation_mps_matches_reference(oracle, path):
    """The new MPS tensors tu, tv: the oracle's row placement of the kept
    U, V columns against the reference's fuse + contract, gauge-free."""
    g = np.load(path)
    vs = oracle.struct_from_desc(g["dvec"], g["fvec"])
    dims, _, uv = oracle.svd_truncate(vs, g["xvec"], float(g["p1"]), float(g["p2"]), int(g["dcut"]))
    su, sv = oracle.struct_from_desc(g["du"]), oracle.struct_from_desc(g["dv"])
    tu, tv = oracle.svd_mps(vs, dims, uv, su.bonds[:2], sv.bonds[:2])
    rtu = (oracle.struct_from_desc(g["tu_desc"], g["tu_flag"]), g["tu_x"])
    rtv = (oracle.struct_from_desc(g["tv_desc"], g["tv_flag"]), g["tv_x"])
    check_mps(oracle, tu, tv, rtu, rtv)


def test_fac_site_tables_match_reference(oracle):
    g = np.load(os.path.join(GOLDEN, "fac_site.npz"))
    fns = (oracle.fac_operator_onsite, oracle.fac_operator_pairup, oracle.fac_permutation)
    for r, v in zip(g["idx"], g["val"]):
        got = fns[int(r[0])](*[int(x) for x in r[1:]])
        assert abs(got - v) <= 1e-14 * abs(v), (r, got, v)


def site_case(oracle, g):
    """(kind, flag, su, xu, xv, x, sites) of a site-update fixture."""
    su = oracle.struct_from_desc(g["du"], g["fu"])
    x = (oracle.struct_from_desc(g["dx"], g["fx"]), g["xx"]) if "dx" in g.files else None
    sites = [(oracle.struct_from_desc(g[f"ds{i}"], g[f"fs{i}"]), g[f"xs{i}"]) for i in range(2) if f"ds{i}" in g.files]
    kind = str(g["kind"])
    kind = "init" if kind.startswith("init") else ("pair" if kind == "pair" else "perm")
    return kind, int(g["flag"]), su, g["xu"], g["xv"], x, sites


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "site_*.npz"))))
def test_site_update_matches_reference(oracle, path):
    """operator_initial / operator_pairup / permutation: the same blocks, the
    same values to 1e-13 relative (Frobenius)."""
    g = np.load(path)
    kind, flag, su, xu, xv, x, sites = site_case(oracle, g)
    out, y = oracle.site_update(kind, flag, su, xu, su, xv, x, sites)
    assert out.desc().tolist() == g["rdesc"].tolist()
    assert out.flag.tolist() == g["rflag"].tolist()
    assert np.linalg.norm(y - g["rx"]) <= 1e-13 * np.linalg.norm(g["rx"])


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "idmrg_*.npz"))))
def test_idmrg_heff_matches_reference(oracle, path):
    """The engine's own H_eff psi at a real two-site step (J1-J2 and J-Q
    runs) rebuilt from its term decomposition: the combined partner
    operators, the spin-0 block Hamiltonians and the plaquette terms; 1e-12
    relative."""
    import idmrg_case

    g = np.load(path)
    vs, vx, yref, outside, T, terms, hl, hr = idmrg_case.load(oracle, g)
    assert outside <= 1e-24 * np.dot(yref, yref)
    tl = []
    for coef, left, right in terms:
        L = idmrg_case.combine_host(oracle, T, left)
        R = idmrg_case.combine_host(oracle, T, right)
        tl.append((L[0], L[1], R[0], R[1], coef))
    prob = oracle.HeffProblem(vs, tl, hl, hr)
    y = oracle.heff_apply(prob, vx)
    assert np.linalg.norm(y - yref) <= 1e-12 * np.linalg.norm(yref)


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "inputvec_*.npz"))))
def test_input_vector_matches_reference(oracle, path):
    g = np.load(path)
    sl, sr = oracle.struct_from_desc(g["dl"], g["fl"]), oracle.struct_from_desc(g["dr"], g["fr"])
    out, y = oracle.prepare_input_vector(sl, g["xl"], sr, g["xr"])
    assert out.desc().tolist() == g["rdesc"].tolist()
    assert out.flag.tolist() == g["rflag"].tolist()
    assert np.linalg.norm(y - g["rx"]) <= 1e-14 * np.linalg.norm(g["rx"])


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "vectran_*.npz"))))
def test_vectran_matches_reference(oracle, path):
    g = np.load(path)
    out, y = oracle.vectran(oracle.struct_from_desc(g["du"], g["fu"]), g["xu"], int(g["dir"]))
    assert out.desc().tolist() == g["rdesc"].tolist()
    assert out.flag.tolist() == g["rflag"].tolist()
    assert np.array_equal(y, g["rx"])


def _mea_tensor(oracle, g, i):
    d = g[f"d{i}"]
    if len(d) == 0:
        return None
    return oracle.struct_from_desc(d, g[f"f{i}"]), g[f"x{i}"]


def mea_case(oracle, g):
    """(hl, hr, ww, [(left, right, coef)]) of a mea_*.npz fixture (oracle structs, host data)."""
    ints, coefs = g["pairs"], g["coefs"]
    pairs = [(_mea_tensor(oracle, g, int(ints[1 + 2 * k])), _mea_tensor(oracle, g, int(ints[2 + 2 * k])), float(coefs[k]))
             for k in range(int(ints[0]))]
    return _mea_tensor(oracle, g, 0), _mea_tensor(oracle, g, 1), g["ww"], pairs


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "meaop_*.npz"))))
def test_measure_reductions_match_reference(oracle, path):
    g = np.load(path)
    sh = oracle.struct_from_desc(g["dh"], g["fh"])
    assert abs(oracle.take_trace(sh, g["xh"]) - g["trace"]) <= 1e-13 * max(1.0, abs(g["trace"]))
    for leg in (0, 1):
        assert np.allclose(oracle.multiply_singular_value(sh, g["xh"], leg, g["w"]), g[f"msv{leg}"], rtol=0, atol=1e-15)
    sa, sb = oracle.struct_from_desc(g["do"], g["fa"]), oracle.struct_from_desc(g["do"], g["fb"])
    assert abs(oracle.ss_inner_prod(sa, g["xa"], sb, g["xb"]) - g["inner"]) <= 1e-13 * max(1.0, abs(g["inner"]))


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "mea_*.npz"))))
def test_mea_enr_matches_reference(oracle, path):
    """The measurement variant's own mea_enr value, from its centre tensors."""
    g = np.load(path)
    hl, hr, ww, pairs = mea_case(oracle, g)
    e = oracle.mea_enr(hl, hr, ww, pairs)
    assert abs(e - g["parts"][4]) <= 1e-12 * abs(g["parts"][4])


def test_oracle_generator_matches_reference_draws(oracle):
    """ran() of the reference build (ran.f90 as linked there) for seed 1234:
    the oracle's seeded random vector draws the same numbers."""
    import json

    g = json.load(open(os.path.join(GOLDEN, "dmrg_seeded.json")))
    _, raw, _ = oracle.random_vector(1234, 16)
    assert np.array_equal(raw, np.array(g["ran_seed1234"]) * 2.0 - 1.0)
