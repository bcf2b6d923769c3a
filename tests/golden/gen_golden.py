"""Generates the golden fixtures of tests/golden/ from the reference itself.

Runs only where the reference sources exist (they are compiled by
oracle/ref/build_ref.sh into oracle/_ref/libsu2ref.so); the fixtures it writes
are committed and are what the tests read on every other machine.

    bash oracle/ref/build_ref.sh && python tests/golden/gen_golden.py

Fixtures:
  fac_hamilt_vec.npy   fac_hamilt_vec[25][25][25] (dmrg_su2.cpp:759-766)
  cgc.npz              tensor::make_cgc for a spread of (j1,j2,j3)
  meta.npz             su2bond::fuse and su2struct block legality cases
  heff_term_*.npz      tensor_su2::hamiltonian_vector_multiplication cases
  spin0_*.npz          tensor_su2::contract cases of the spin-0 terms
  env_op_*.npz         tensor_su2::operator_transformation cases (both flags)
  env_ovl_*.npz        tensor_su2::overlap_transformation cases (both flags)
  fac_optrans.npz      fac_operator_transformation_{left,rght} entries
  svd_*.npz            tensor_su2::svd truncation cases (singular values, kept
                       multiplets per sector)
  dmrg_energies.json   whole reference DMRG runs (E0 - 1000 per sweep)
  dmrg_seeded.json     whole runs from the seeded random start (-seed), and ran()
"""
from __future__ import annotations

import ctypes
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REFLIB = os.path.join(REPO, "oracle", "_ref", "libsu2ref.so")


def p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def desc_of(bonds, locspin=0):
    d = [len(bonds), locspin]
    for (dr, angm, dim) in bonds:
        d += [dr, len(angm)] + list(angm) + list(dim)
    return np.asarray(d, np.int32)


def nten_of(bonds):
    n = 1
    for b in bonds:
        n *= len(b[1])
    return n


def block_shape(bonds, idx):
    shp = []
    for (_, angm, dim) in bonds:
        shp.append(dim[idx % len(angm)])
        idx //= len(angm)
    return shp


def random_data(bonds, flag, rng):
    n = 0
    for i in range(nten_of(bonds)):
        if flag[i]:
            n += int(np.prod(block_shape(bonds, i)))
    return rng.standard_normal(n)


def legal_flags(L, desc):
    out = np.zeros(4096, np.int32)
    n = L.ref_legal(p(desc), p(out))
    return out[:n].copy()


def read_result(L):
    nten = ctypes.c_int()
    n1 = ctypes.c_int()
    n2 = ctypes.c_int()
    L.ref_result_sizes(ctypes.byref(nten), ctypes.byref(n1), ctypes.byref(n2))
    flag = np.zeros(nten.value, np.int32)
    x1 = np.zeros(max(1, n1.value))
    x2 = np.zeros(max(1, n2.value))
    L.ref_result_get(p(flag), p(x1), p(x2))
    return flag, x1[: n1.value], x2[: n2.value]


def heff_cases(L, rng):
    cases = []
    specs = [
        # (left sectors, right sectors, spin sectors(2j), spin dims, dropout)
        ([0, 1, 2, 3, 4], [0, 1, 2, 3, 4], [2], [1], 0.0),
        ([0, 2, 4], [0, 2, 4, 6], [2], [1], 0.0),
        ([1, 3, 5], [1, 3, 5], [2], [1], 0.25),
        ([0, 1, 2, 3, 4, 5, 6], [0, 1, 2, 3, 4, 5, 6], [0, 2], [2, 1], 0.2),
        ([0, 2, 4, 6, 8], [0, 2, 4, 6, 8], [2, 4], [1, 2], 0.1),
    ]
    for ci, (la, ra, sa, sd, drop) in enumerate(specs):
        common = sorted(set(la) & set(ra))
        ld = [int(rng.integers(1, 7)) for _ in la]
        rd = [int(rng.integers(1, 7)) for _ in ra]
        # psi/y legs must carry exactly the sectors the operators map onto
        EL = (-1, la, ld)
        ER = (-1, ra, rd)
        S = (1, sa, sd)
        vb = [EL, ER]
        o1b = [(1, la, ld), S, EL]
        o2b = [(1, ra, rd), S, ER]
        vdesc, d1, d2 = desc_of(vb), desc_of(o1b), desc_of(o2b)
        vflag = legal_flags(L, vdesc)
        f1 = legal_flags(L, d1) * (rng.random(nten_of(o1b)) >= drop)
        f2 = legal_flags(L, d2) * (rng.random(nten_of(o2b)) >= drop)
        f1 = f1.astype(np.int32)
        f2 = f2.astype(np.int32)
        vx = random_data(vb, vflag, rng)
        x1 = random_data(o1b, f1, rng)
        x2 = random_data(o2b, f2, rng)
        L.ref_heff_term(p(vdesc), p(vflag), p(vx), p(d1), p(f1), p(x1), p(d2), p(f2), p(x2))
        rflag, rx, rcg = read_result(L)
        cases.append(dict(name=f"heff_term_{ci}", vdesc=vdesc, vflag=vflag, vx=vx, d1=d1, f1=f1, x1=x1, d2=d2,
                          f2=f2, x2=x2, rflag=rflag, rx=rx, rcg=rcg, common=np.asarray(common, np.int32)))
    return cases


def spin0_cases(L, rng):
    cases = []
    for ci, (la, ra) in enumerate([([0, 1, 2, 3], [0, 1, 2, 3]), ([0, 2, 4, 6], [0, 2, 4, 6])]):
        ld = [int(rng.integers(1, 8)) for _ in la]
        rd = [int(rng.integers(1, 8)) for _ in ra]
        vb = [(-1, la, ld), (-1, ra, rd)]
        vdesc = desc_of(vb)
        vflag = legal_flags(L, vdesc)
        vx = random_data(vb, vflag, rng)
        for side in (0, 1):
            sec, dim = (la, ld) if side == 0 else (ra, rd)
            hb = [(1, sec, dim), (-1, sec, dim)]
            hdesc = desc_of(hb)
            hflag = legal_flags(L, hdesc)
            hx = random_data(hb, hflag, rng)
            if side == 0:  # contract(hh[il],0,vec1,0)
                L.ref_contract(p(hdesc), p(hflag), p(hx), 0, p(vdesc), p(vflag), p(vx), 0)
            else:  # contract(vec1,1,hh[ir],0)
                L.ref_contract(p(vdesc), p(vflag), p(vx), 1, p(hdesc), p(hflag), p(hx), 0)
            rflag, rx, rcg = read_result(L)
            cases.append(dict(name=f"spin0_{ci}_{side}", side=np.int32(side), vdesc=vdesc, vflag=vflag, vx=vx,
                              hdesc=hdesc, hflag=hflag, hx=hx, rflag=rflag, rx=rx, rcg=rcg))
    return cases


def env_cases(L, rng):
    """operator_transformation / overlap_transformation on random MPS tensors
    with a spin-1/2 physical leg and random operators."""
    cases = []
    specs = [([0, 1, 2, 3, 4], [0, 1, 2, 3, 4, 5], 0.0), ([0, 2, 4], [1, 3, 5], 0.2), ([1, 3, 5, 7], [0, 2, 4, 6, 8], 0.1)]
    for ci, (sa, sc, drop) in enumerate(specs):
        da = [int(rng.integers(1, 7)) for _ in sa]
        dc = [int(rng.integers(1, 7)) for _ in sc]
        for flag in (0, 1):
            phys = (-1, [1], [1])
            bond_a = (-1, sa, da)
            uub = [bond_a, phys, (1, sc, dc)] if flag == 0 else [phys, bond_a, (1, sc, dc)]
            du = desc_of(uub)
            fu = (legal_flags(L, du) * (rng.random(nten_of(uub)) >= drop)).astype(np.int32)
            xu = random_data(uub, fu, rng)
            xv = random_data(uub, fu, rng)
            for kind, spin in (("op", (1, [2], [1])), ("op", (1, [0, 2], [1, 1])), ("ovl", None)):
                if kind == "op":
                    ob = [(1, sa, da), spin, (-1, sa, da)]
                    fn = L.ref_operator_transformation
                else:
                    ob = [(1, sa, da), (-1, sa, da)]
                    fn = L.ref_overlap_transformation
                dop = desc_of(ob)
                fop = (legal_flags(L, dop) * (rng.random(nten_of(ob)) >= drop)).astype(np.int32)
                xop = random_data(ob, fop, rng)
                fn(p(du), p(fu), p(xu), p(du), p(fu), p(xv), p(dop), p(fop), p(xop), flag)
                rflag, rx, rcg = read_result(L)
                nten = ctypes.c_int()
                name = f"env_{kind}_{ci}_{flag}_{len(spin[1]) if spin else 0}"
                cases.append(dict(name=name, flag=np.int32(flag), du=du, fu=fu, xu=xu, xv=xv, dop=dop, fop=fop, xop=xop,
                                  rflag=rflag, rx=rx, rcg=rcg))
    return cases


def site_operator(L, kind, idx):
    """The engine's own site operator (sigma / qterm) as desc, flag, data."""
    L.ref_select_site(kind, idx)
    d = np.zeros(256, np.int32)
    n = L.ref_result_desc(p(d))
    f, x, _ = read_result(L)
    L.ref_select_result(0)
    return d[:n].copy(), f, x


def site_cases(L, rng):
    """operator_initial (with and without endt), operator_pairup and
    permutation on random MPS tensors and environment operators, with the
    engine's site operators, in the directions the engine uses them
    (dmrg_su2_omp.cpp:319-825)."""
    cases = []
    specs = [([0, 1, 2, 3, 4], [0, 1, 2, 3, 4, 5], 0.0), ([0, 2, 4, 6], [1, 3, 5, 7], 0.15),
             ([1, 3, 5], [0, 2, 4, 6], 0.1)]
    S, Q = 0, 1  # site operator kinds: sigma, qterm
    for ci, (sa, sc, drop) in enumerate(specs):
        da = [int(rng.integers(1, 7)) for _ in sa]
        dc = [int(rng.integers(1, 7)) for _ in sc]
        for flag in (0, 1):
            phys = (1, [1], [1])
            bond_a = (-1, sa, da)
            uub = [bond_a, phys, (1, sc, dc)] if flag == 0 else [phys, bond_a, (1, sc, dc)]
            du = desc_of(uub)
            fu = (legal_flags(L, du) * (rng.random(nten_of(uub)) >= drop)).astype(np.int32)
            xu = random_data(uub, fu, rng)
            xv = random_data(uub, fu, rng)

            def rand_op(bonds):
                d = desc_of(bonds)
                f = (legal_flags(L, d) * (rng.random(nten_of(bonds)) >= drop)).astype(np.int32)
                return d, f, random_data(bonds, f, rng)

            jobs = []
            sig = site_operator(L, S, 0 if flag == 0 else 1)
            jobs.append(("init", None, [sig], lambda x, s: L.ref_operator_initial(
                p(du), p(fu), p(xu), p(du), p(fu), p(xv), S, 0 if flag == 0 else 1, None, None, None, flag)))
            endt = rand_op([(1, sa, da), (-1, sa, da)])
            jobs.append(("initendt", endt, [sig], lambda x, s: L.ref_operator_initial(
                p(du), p(fu), p(xu), p(du), p(fu), p(xv), S, 0 if flag == 0 else 1, p(x[0]), p(x[1]), p(x[2]),
                flag)))
            op1 = rand_op([(1, sa, da), (-1, [2], [1]), (-1, sa, da)])
            sig2 = site_operator(L, S, 1 if flag == 0 else 0)
            jobs.append(("pair", op1, [sig2], lambda x, s: L.ref_operator_pairup(
                p(du), p(fu), p(xu), p(du), p(fu), p(xv), p(x[0]), p(x[1]), p(x[2]), S, 1 if flag == 0 else 0,
                flag)))
            # the two permutations of the plaquette chains (dmrg_su2_omp.cpp:430-434, 728-732)
            q1, q2 = (0, 1) if flag == 0 else (6, 7)
            q3, q4 = (2, 3) if flag == 0 else (4, 5)
            for tag, (a1, a2), spin in (("perm1", (q1, q2), (-1, [2], [1])), ("perm2", (q3, q4), (-1, [0, 2, 4], [1, 1, 1]))):
                vec = rand_op([(1, sa, da), spin, (-1, sa, da)])
                sites = [site_operator(L, Q, a1), site_operator(L, Q, a2)]
                jobs.append((tag, vec, sites, lambda x, s, a1=a1, a2=a2: L.ref_permutation(
                    p(du), p(fu), p(xu), p(du), p(fu), p(xv), p(x[0]), p(x[1]), p(x[2]), Q, a1, Q, a2, flag)))
            for tag, x, sites, fn in jobs:
                fn(x, sites)
                d = np.zeros(1024, np.int32)
                nd = L.ref_result_desc(p(d))
                rflag, rx, _ = read_result(L)
                c = dict(name=f"site_{tag}_{ci}_{flag}", kind=np.str_(tag), flag=np.int32(flag), du=du, fu=fu, xu=xu,
                         xv=xv, rdesc=d[:nd].copy(), rflag=rflag, rx=rx)
                if x is not None:
                    c.update(dx=x[0], fx=x[1], xx=x[2])
                for si, (sd, sf, sx) in enumerate(sites):
                    c.update({f"ds{si}": sd, f"fs{si}": sf, f"xs{si}": sx})
                cases.append(c)
    return cases


def fuse_bond(a, b):
    out = {}
    for x, dx in zip(a[1], a[2]):
        for y, dy in zip(b[1], b[2]):
            for k in range(abs(x - y), min(x + y, 38) + 1, 2):
                out[k] = out.get(k, 0) + dx * dy
    ks = sorted(out)
    return (-1, ks, [out[k] for k in ks])


def svd_cases(L, rng):
    L.ref_svd.restype = ctypes.c_int
    cases = []
    specs = [  # (left bond sectors, dims, right bond sectors, dims, p1, p2, max_dcut, scale decay)
        ([0, 1, 2, 3], [3, 5, 4, 2], [0, 1, 2, 3], [3, 5, 4, 2], 1.0, 0.0, 10, 0.0),
        ([0, 1, 2, 3], [3, 5, 4, 2], [0, 1, 2, 3], [2, 4, 6, 3], 0.0, 1.0, 12, 0.0),
        ([0, 2, 4, 6], [4, 8, 6, 3], [0, 2, 4], [6, 7, 4], 1.0, 0.0, 20, 1.0),
        ([1, 3, 5], [9, 7, 5], [1, 3, 5, 7], [5, 8, 8, 2], 0.0, 1.0, 1000, 0.3),
        ([0, 1, 2, 3, 4], [6, 10, 9, 6, 3], [0, 1, 2, 3, 4], [6, 10, 9, 6, 3], 1.0, 0.0, 30, 3.0),
    ]
    ph = (-1, [1], [1])
    for ci, (la, lda, ra, rda, p1, p2, dcut, decay) in enumerate(specs):
        Lb, Rb = (-1, la, lda), (-1, ra, rda)
        EL, ER = fuse_bond(Lb, ph), fuse_bond(Rb, ph)
        vb = [EL, ER]
        dvec = desc_of(vb)
        fvec = legal_flags(L, dvec)
        # blocks with decaying spectra: product of random orthogonal-ish factors
        xs = []
        for i in range(nten_of(vb)):
            if not fvec[i]:
                continue
            m, n = block_shape(vb, i)
            blk = rng.standard_normal((m, n))
            if decay > 0:
                u, sv, vt = np.linalg.svd(blk, full_matrices=False)
                sv = np.exp(-decay * np.arange(len(sv))) * (1 + rng.random(len(sv)))
                blk = (u * sv) @ vt
            xs.append(blk.ravel(order="F"))
        xvec = np.concatenate(xs)
        tub = [Lb, ph, (1, [0], [1])]
        tvb = [Rb, ph, (1, [0], [1])]
        du, dv = desc_of(tub), desc_of(tvb)
        fu, fv = legal_flags(L, du), legal_flags(L, dv)
        xu, xv = random_data(tub, fu, rng), random_data(tvb, fv, rng)
        w = np.zeros(4096)
        kept = np.zeros(64, np.int32)
        n = L.ref_svd(p(dvec), p(fvec), p(xvec), p(du), p(fu), p(xu), p(dv), p(fv), p(xv), ctypes.c_double(p1),
                      ctypes.c_double(p2), dcut, p(w), p(kept))
        out = {}
        for sel, nm in ((0, "tu"), (1, "tv")):  # the new MPS tensors tu, tv
            L.ref_select_result(sel)
            d = np.zeros(1024, np.int32)
            nd = L.ref_result_desc(p(d))
            f, x, _ = read_result(L)
            out.update({f"{nm}_desc": d[:nd].copy(), f"{nm}_flag": f, f"{nm}_x": x})
        L.ref_select_result(0)
        cases.append(dict(name=f"svd_{ci}", dvec=dvec, fvec=fvec, xvec=xvec, p1=np.float64(p1), p2=np.float64(p2),
                          dcut=np.int32(dcut), wout=w[:n].copy(), kept=kept, du=du, dv=dv, **out))
    return cases


def fac_site_tables(L):
    """Nonzero entries of fac_operator_onsite / fac_operator_pairup /
    fac_permutation (left and right) over the index ranges a spin-1/2 chain
    with 2j <= 12 bonds reaches."""
    L.ref_fac_table.restype = ctypes.c_double
    idx, val = [], []
    for table in range(3):
        for side in (0, 1):
            for a in range(13):
                for b in (range(7) if table == 0 else range(13)):
                    for c in range(13):
                        for d in (range(7) if table == 1 else range(13)):
                            for e in range(18 if table == 2 else 9):
                                v = L.ref_fac_table(table, side, a, b, c, d, e)
                                if v != 0.0:
                                    idx.append((table, side, a, b, c, d, e))
                                    val.append(v)
    return dict(idx=np.asarray(idx, np.int8), val=np.asarray(val))


def fac_optrans(L):
    L.ref_fac_operator_transformation.restype = ctypes.c_double
    idx, val = [], []
    for side in (0, 1):
        for j in range(11):
            for m in (0, 2, 4, 6):
                for l in range(11):
                    for i in range(11):
                        for k in range(11):
                            for pp in (0, 1, 2):
                                v = L.ref_fac_operator_transformation(side, j, m, l, i, k, pp)
                                if v != 0.0:
                                    idx.append((side, j, m, l, i, k, pp))
                                    val.append(v)
    return dict(idx=np.asarray(idx, np.int8), val=np.asarray(val))


def meta_cases(L, rng):
    fa, fd, fo_a, fo_d, fn = [], [], [], [], []
    for _ in range(40):
        n1 = int(rng.integers(1, 6))
        n2 = int(rng.integers(1, 4))
        a1 = sorted(rng.choice(np.arange(0, 30), n1, replace=False).tolist())
        a2 = sorted(rng.choice(np.arange(0, 12), n2, replace=False).tolist())
        d1 = rng.integers(1, 50, n1).tolist()
        d2 = rng.integers(1, 5, n2).tolist()
        ao = np.zeros(128, np.int32)
        do = np.zeros(128, np.int32)
        A1, D1, A2, D2 = (np.asarray(v, np.int32) for v in (a1, d1, a2, d2))
        n = L.ref_fuse(n1, p(A1), p(D1), n2, p(A2), p(D2), p(ao), p(do))
        fa.append(np.concatenate([[n1], a1, d1, [n2], a2, d2]).astype(np.int32))
        fo_a.append(ao[:n].copy())
        fo_d.append(do[:n].copy())
        fn.append(n)
    # legality of random 2-, 3- and 4-leg structures with several locspins
    ldesc, lflag = [], []
    for _ in range(30):
        nb = int(rng.integers(2, 5))
        bonds = []
        for _l in range(nb):
            k = int(rng.integers(1, 5))
            bonds.append((1, sorted(rng.choice(np.arange(0, 16), k, replace=False).tolist()), [1] * k))
        desc = desc_of(bonds, int(rng.integers(0, 5)))
        ldesc.append(desc)
        lflag.append(legal_flags(L, desc))
    pack = lambda arrs: (np.concatenate(arrs).astype(np.int32), np.cumsum([0] + [len(a) for a in arrs]))
    fin, fin_idx = pack(fa)
    foa, foa_idx = pack(fo_a)
    fod, _ = pack(fo_d)
    ld, ld_idx = pack(ldesc)
    lf, lf_idx = pack(lflag)
    return dict(fuse_in=fin, fuse_in_idx=fin_idx, fuse_out_a=foa, fuse_out_d=fod, fuse_out_idx=foa_idx,
                legal_desc=ld, legal_desc_idx=ld_idx, legal_flag=lf, legal_flag_idx=lf_idx)


def dmrg_runs(L):
    runs = [
        # (lx, ly, sec, D, niter, jcoup, qcoup, boundary)
        (4, 2, 0, 64, 4, 0.5, 0.0, 2),
        (3, 4, 0, 64, 4, 0.5, 0.0, 2),
        (3, 4, 0, 64, 4, 0.5, 1.0, 2),
        (6, 4, 0, 200, 4, 2.0, 0.0, 2),
        # total spin 1 (the engine's sector 2j = 2)
        (4, 2, 2, 64, 4, 0.5, 0.0, 2),
        (3, 4, 2, 64, 4, 0.5, 1.0, 2),
    ]
    out = []
    cwd = os.getcwd()
    for (lx, ly, sec, d, niter, jc, qc, bd) in runs:
        with tempfile.TemporaryDirectory() as tmp:
            os.chdir(tmp)
            e = np.zeros(64)
            n = L.ref_run_dmrg(lx, ly, sec, d, niter, ctypes.c_double(jc), ctypes.c_double(qc), bd, 1, p(e))
            os.chdir(cwd)
        # the structure of every MPS tensor at the end (kept multiplets per sector)
        descs = []
        for i in range(lx * ly):
            assert L.ref_select_mps(i) == 0
            dd = np.zeros(1024, np.int32)
            nd = L.ref_result_desc(p(dd))
            descs.append([int(v) for v in dd[:nd]])
        out.append(dict(lx=lx, ly=ly, sec=sec, d=d, niter=niter, jcoup=jc, qcoup=qc, boundary=bd,
                        energies_minus_1000=[float(v) for v in e[:n]], mps_desc=descs))
        print("dmrg", lx, ly, d, jc, qc, out[-1]["energies_minus_1000"], file=sys.stderr)
    return out


def seeded_runs(L):
    """Whole runs with the seeded random start (the -seed option of the parity
    runs, patch_ref.py): the warm-up's two-site steps start from
    random_initialize_tensor with the generator seeded once by initran.  The
    6x4 J1-J2 run at D = 200 is the benchmark's CPU-runnable configuration
    (4 sweeps from a seeded random MPS).  Also the first draws of ran() for
    seed 1234 (the generator of ran.f90 as the reference build links it)."""
    runs = [
        # (lx, ly, sec, D, niter, jcoup, qcoup, boundary, seed)
        (4, 2, 0, 64, 4, 0.5, 0.0, 2, 7),
        (3, 4, 0, 64, 4, 0.5, 1.0, 2, 99),
        (6, 4, 0, 200, 4, 2.0, 0.0, 2, 1234),
    ]
    out = {"runs": []}
    L.ran_.restype = ctypes.c_double
    seed = ctypes.c_int(1234)
    L.initran_(ctypes.byref(seed))
    out["ran_seed1234"] = [L.ran_() for _ in range(16)]
    cwd = os.getcwd()
    for (lx, ly, sec, d, niter, jc, qc, bd, sd) in runs:
        with tempfile.TemporaryDirectory() as tmp:
            os.chdir(tmp)
            e = np.zeros(64)
            L.su2ref_set_seed(sd)
            n = L.ref_run_dmrg(lx, ly, sec, d, niter, ctypes.c_double(jc), ctypes.c_double(qc), bd, 1, p(e))
            L.su2ref_clear_seed()
            os.chdir(cwd)
        descs = []
        for i in range(lx * ly):
            assert L.ref_select_mps(i) == 0
            dd = np.zeros(1024, np.int32)
            nd = L.ref_result_desc(p(dd))
            descs.append([int(v) for v in dd[:nd]])
        out["runs"].append(dict(lx=lx, ly=ly, sec=sec, d=d, niter=niter, jcoup=jc, qcoup=qc, boundary=bd, seed=sd,
                                energies_minus_1000=[float(v) for v in e[:n]], mps_desc=descs))
        print("seeded", lx, ly, d, sd, out["runs"][-1]["energies_minus_1000"], file=sys.stderr)
    return out


def input_vector_cases(L, rng):
    """prepare_input_vector (the initial two-site vector of a step) and the
    vectran permutations of wavefunc_transformation, on random MPS tensors."""
    cases = []
    specs = [([0, 1, 2, 3], [0, 1, 2, 3, 4], [0, 1, 2, 3], 0.0), ([0, 2, 4, 6], [1, 3, 5, 7], [0, 2, 4, 6], 0.1),
             ([1, 3, 5], [0, 2, 4, 6], [1, 3, 5], 0.0)]
    ph = (1, [1], [1])
    for ci, (sa, sc, sb, drop) in enumerate(specs):
        da = [int(rng.integers(1, 7)) for _ in sa]
        dc = [int(rng.integers(1, 7)) for _ in sc]
        db = [int(rng.integers(1, 7)) for _ in sb]
        ulb = [(1, sa, da), ph, (-1, sc, dc)]   # uu[il]: (bond, spin, centre bond)
        urb = [ph, (1, sb, db), (-1, sc, dc)]   # uu[ir]: (spin, bond, centre bond)
        dl, dr = desc_of(ulb), desc_of(urb)
        fl = (legal_flags(L, dl) * (rng.random(nten_of(ulb)) >= drop)).astype(np.int32)
        fr = (legal_flags(L, dr) * (rng.random(nten_of(urb)) >= drop)).astype(np.int32)
        xl, xr = random_data(ulb, fl, rng), random_data(urb, fr, rng)
        L.ref_prepare_input_vector(p(dl), p(fl), p(xl), p(dr), p(fr), p(xr))
        d = np.zeros(1024, np.int32)
        nd = L.ref_result_desc(p(d))
        rflag, rx, _ = read_result(L)
        cases.append(dict(name=f"inputvec_{ci}", dl=dl, fl=fl, xl=xl, dr=dr, fr=fr, xr=xr, rdesc=d[:nd].copy(),
                          rflag=rflag, rx=rx))
        for direction in (0, 1):
            L.ref_vectran(p(dl), p(fl), p(xl), direction)
            d = np.zeros(1024, np.int32)
            nd = L.ref_result_desc(p(d))
            rflag, rx, _ = read_result(L)
            cases.append(dict(name=f"vectran_{ci}_{direction}", du=dl, fu=fl, xu=xl, dir=np.int32(direction),
                              rdesc=d[:nd].copy(), rflag=rflag, rx=rx))
    return cases


def idmrg_cases(L):
    """The engine's own H_eff (hamiltonian_vector_multiplication_idmrg) at the
    last two-site step of short runs: real environments, the input vector the
    engine builds, its output, and the term decomposition it sums."""
    runs = [
        # (lx, ly, sec, D, niter, jcoup, qcoup, boundary)
        (6, 4, 0, 40, 1, 2.0, 0.0, 2),  # J1-J2
        (6, 4, 0, 30, 1, 1.0, 1.0, 2),  # J-Q: plaquette terms
    ]
    L.ref_idmrg_capture.restype = ctypes.c_int
    cases = []
    cwd = os.getcwd()
    for ci, (lx, ly, sec, d, niter, jc, qc, bd) in enumerate(runs):
        with tempfile.TemporaryDirectory() as tmp:
            os.chdir(tmp)
            e = np.zeros(64)
            nt = L.ref_idmrg_capture(lx, ly, sec, d, niter, ctypes.c_double(jc), ctypes.c_double(qc), bd, 1, p(e))
            os.chdir(cwd)
        c = dict(name=f"idmrg_{ci}", lx=lx, ly=ly, d=d, jcoup=jc, qcoup=qc, ntensors=np.int32(nt))
        for i in range(nt):
            L.ref_idmrg_select(i)
            dd = np.zeros(1024, np.int32)
            nd = L.ref_result_desc(p(dd))
            if dd[0] == 0:
                f, x = np.zeros(0, np.int32), np.zeros(0)
            else:
                f, x, _ = read_result(L)
            c.update({f"t{i}_desc": dd[:nd].copy(), f"t{i}_flag": f, f"t{i}_x": x})
        ti, td = np.zeros(100000, np.int32), np.zeros(100000)
        n = L.ref_idmrg_terms(p(ti), len(ti), p(td), len(td))
        ti = ti[:n].copy()
        nd, q = 0, 1
        for _ in range(ti[0]):  # per term: coef, then one coefficient per named operator
            nl = ti[q]
            nr = ti[q + 1 + nl]
            nd += 1 + nl + nr
            q += 2 + nl + nr
        c.update(term_i=ti, term_d=td[:nd].copy())
        L.ref_select_result(0)
        cases.append(c)
    return cases


def checkpoint_cases(L):
    """Checkpoint files written by the engine itself (save_mps2, save_enr,
    save_ww after do_idmrg and one sweep of a 4x2 J1 lattice at D=16), copied
    into tests/golden/ckpt/, with the engine's in-memory MPS tensors (reduced
    blocks and CG parts) and what its own readers return for the same files
    (read_mps, read_enr, read_ww)."""
    import shutil

    out = os.path.join(HERE, "ckpt")
    os.makedirs(out, exist_ok=True)
    tmp = tempfile.mkdtemp()
    L.ref_checkpoint_write.restype = ctypes.c_int
    L.ref_checkpoint_read.restype = ctypes.c_int
    e = ctypes.c_double()
    ns = L.ref_checkpoint_write(4, 2, 0, 16, 1, ctypes.c_double(1.0), ctypes.c_double(0.0), 2, 1,
                                tmp.encode(), ctypes.byref(e))
    assert ns > 0
    for f in sorted(os.listdir(tmp)):
        shutil.copy(os.path.join(tmp, f), out)
    case = dict(ns=np.int32(ns), enr_written=np.float64(e.value), files=np.array(sorted(os.listdir(tmp))))
    for i in range(ns):
        L.ref_idmrg_select(i)
        d = np.zeros(1024, np.int32)
        nd = L.ref_result_desc(p(d))
        flag, x1, x2 = read_result(L)
        case.update({f"desc{i}": d[:nd].copy(), f"flag{i}": flag, f"x{i}": x1, f"cg{i}": x2})
    e2 = ctypes.c_double()
    ww = np.zeros(64)
    r = L.ref_checkpoint_read(4, 2, 0, 16, tmp.encode(), ctypes.byref(e2), p(ww), 64)
    assert r == ns
    for i in range(ns):  # the engine reads back what it wrote
        L.ref_idmrg_select(i)
        flag, x1, x2 = read_result(L)
        assert np.array_equal(flag, case[f"flag{i}"]) and np.array_equal(x1, case[f"x{i}"])
    case.update(enr_read=np.float64(e2.value), ww_read=ww[:16].copy())
    shutil.rmtree(tmp)
    return case


def measure_op_cases(L, rng):
    """take_trace, ss_inner_prod and multiply_singular_value of the engine
    (tensor_su2.cpp:359-384, 687-742) on random block tensors."""
    L.ref_take_trace.restype = ctypes.c_double
    L.ref_ss_inner_prod.restype = ctypes.c_double
    cases = []
    specs = [([0, 2, 4], [5, 9, 3], [2], [1]), ([1, 3, 5, 7], [4, 6, 2, 7], [2], [1]), ([0, 1, 2, 3], [3, 4, 5, 2], [0, 2], [1, 2])]
    for ci, (sa, da, ss, ds) in enumerate(specs):
        h = [(1, sa, da), (-1, sa, da)]
        dh = desc_of(h)
        fh = legal_flags(L, dh)
        xh = random_data(h, fh, rng)
        tr = L.ref_take_trace(p(dh), p(fh), p(xh))
        w = rng.random(sum(da))
        out = {}
        for leg in (0, 1):
            L.ref_multiply_singular_value(p(dh), p(fh), p(xh), leg, p(w))
            _, y, _ = read_result(L)
            out[f"msv{leg}"] = y
        o = [(1, sa, da), (-1, ss, ds), (-1, sa, da)]
        do = desc_of(o)
        fb = legal_flags(L, do)
        fa = (fb * (rng.random(len(fb)) >= 0.3)).astype(np.int32)
        xa, xb = random_data(o, fa, rng), random_data(o, fb, rng)
        ip = L.ref_ss_inner_prod(p(do), p(fa), p(xa), p(do), p(fb), p(xb))
        cases.append(dict(name=f"meaop_{ci}", dh=dh, fh=fh, xh=xh, trace=np.float64(tr), w=w, do=do, fa=fa, xa=xa,
                          fb=fb, xb=xb, inner=np.float64(ip), **out))
    return cases


def mea_cases(L):
    """The centre-bond energy of the engine's measurement variant
    (prepare_sweep + mea_enr, dmrg_su2_omp_mea_enr.cpp:160-242, built into
    libsu2ref_mea.so) on checkpoint files the engine wrote after do_idmrg and
    one sweep: the centre tensors, the pair list, the weights, the parts and
    the energy mea_enr returned, next to the sweep's Lanczos energy."""
    M = ctypes.CDLL(REFLIB.replace("libsu2ref.so", "libsu2ref_mea.so"))
    M.ref_setup(1, 25)
    L.ref_checkpoint_write.restype = ctypes.c_int
    cases = []
    for ci, (lx, ly, d, jc, qc) in enumerate([(4, 2, 16, 1.0, 0.0), (4, 4, 24, 1.0, 1.0)]):
        tmp = tempfile.mkdtemp()
        e = ctypes.c_double()
        ns = L.ref_checkpoint_write(lx, ly, 0, d, 1, ctypes.c_double(jc), ctypes.c_double(qc), 2, 1, tmp.encode(),
                                    ctypes.byref(e))
        assert ns > 0
        parts = np.zeros(5)
        ww = np.zeros(4096)
        n = M.ref_mea_enr(lx, ly, 0, d, ctypes.c_double(jc), ctypes.c_double(qc), 2, 1, tmp.encode(), p(parts), p(ww),
                          len(ww))
        assert n > 0, n
        case = dict(name=f"mea_{ci}", lx=np.int32(lx), ly=np.int32(ly), d=np.int32(d), parts=parts, ww=ww[:d].copy(),
                    lanczos=np.float64(e.value + 1000.0), nexp=np.int32(n))
        for i in range(n):
            M.ref_idmrg_select(i)
            dd = np.zeros(1024, np.int32)
            nd = M.ref_result_desc(p(dd))
            if nd <= 2:  # an operator never built
                case[f"d{i}"] = dd[:0]
                continue
            flag, x1, _ = read_result(M)
            case.update({f"d{i}": dd[:nd].copy(), f"f{i}": flag, f"x{i}": x1})
        ints = np.zeros(1 << 16, np.int32)
        dbls = np.zeros(1 << 16)
        ni = M.ref_idmrg_terms(p(ints), len(ints), p(dbls), len(dbls))
        case.update(pairs=ints[:ni].copy(), coefs=dbls[: int(ints[0])].copy())
        cases.append(case)
        import shutil
        shutil.rmtree(tmp)
    return cases


def engine_tables(L, lx, ly, d, jc, qc, bd=2, sec=0):
    """The engine's lattice tables and one-site operators (sigma[0], sigma[1],
    qterm[0..8)) for one lattice, as the device warm-up and sweep take them."""
    L.ref_engine_tables.restype = ctypes.c_int
    ints = np.zeros(1 << 16, np.int32)
    dbls = np.zeros(4096)
    n = L.ref_engine_tables(lx, ly, sec, d, ctypes.c_double(jc), ctypes.c_double(qc), bd, p(ints), len(ints),
                            p(dbls), len(dbls))
    assert n > 0
    ns = int(ints[0])
    case = dict(lx=np.int32(lx), ly=np.int32(ly), d=np.int32(d), jcoup=np.float64(jc), qcoup=np.float64(qc),
                tables=ints[:n].copy(), coup=dbls[:ns].copy())
    for i in range(10):
        L.ref_idmrg_select(i)
        dd = np.zeros(1024, np.int32)
        nd = L.ref_result_desc(p(dd))
        flag, x1, _ = read_result(L)
        case.update({f"site{i}_desc": dd[:nd].copy(), f"site{i}_flag": flag, f"site{i}_x": x1})
    return case


def sweep_cases(L):
    """Lattice tables of the whole runs in dmrg_energies.json (their energies
    after the warm-up and after each sweep are the reference's, in that file)."""
    cases = []
    for ci, r in enumerate(json.load(open(os.path.join(HERE, "dmrg_energies.json")))):
        assert r["boundary"] == 2
        case = engine_tables(L, r["lx"], r["ly"], r["d"], r["jcoup"], r["qcoup"], sec=r["sec"])
        case["name"] = f"sweep_{ci}"
        cases.append(case)
    return cases


def warmup_cases(L):
    """do_idmrg alone on small lattices: the engine's lattice tables and
    one-site operators (inputs of the device warm-up), the eigenvalue of every
    two-site step and the singular values of the last truncation.  The J1 4x2
    warm-up runs as the engine has it (five Lanczos vectors per step); the
    J1-J2 6x2 and J-Q 4x4 warm-ups with mlanc Lanczos vectors (the
    su2ref_idmrg_mlanc hook of patch_ref.py): with five, their steps stop
    near an invariant subspace of the uniform start vector and the result
    follows rounding noise (the FP64 and split device engines already differ
    there at the second step)."""
    cases = []
    L.ref_engine_tables.restype = ctypes.c_int
    for ci, (lx, ly, d, jc, qc, mlanc) in enumerate([(4, 2, 16, 1.0, 0.0, 5), (6, 2, 24, 0.5, 0.0, 40),
                                                      (4, 4, 24, 1.0, 1.0, 40)]):
        ints = np.zeros(1 << 16, np.int32)
        dbls = np.zeros(4096)
        n = L.ref_engine_tables(lx, ly, 0, d, ctypes.c_double(jc), ctypes.c_double(qc), 2, p(ints), len(ints), p(dbls),
                                len(dbls))
        assert n > 0
        ns = int(ints[0])
        case = dict(name=f"warmup_{ci}", lx=np.int32(lx), ly=np.int32(ly), d=np.int32(d), jcoup=np.float64(jc),
                    qcoup=np.float64(qc), mlanc=np.int32(mlanc), tables=ints[:n].copy(), coup=dbls[:ns].copy())
        for i in range(10):  # sigma[0], sigma[1], qterm[0..8)
            L.ref_idmrg_select(i)
            dd = np.zeros(1024, np.int32)
            nd = L.ref_result_desc(p(dd))
            flag, x1, _ = read_result(L)
            case.update({f"site{i}_desc": dd[:nd].copy(), f"site{i}_flag": flag, f"site{i}_x": x1})
        # the warm-up in a child process: its per-step energies are only printed
        # ("lanczos <il> gs_enr[0]=<eigenvalue - 1000>", dmrg_su2.cpp:539; ref_warmup
        # prints them with 17 digits)
        code = (f"import ctypes, numpy as np; L = ctypes.CDLL({REFLIB!r}); L.ref_setup(1, 25); "
                f"L.su2ref_set_sign_convention(1); L.su2ref_set_idmrg_mlanc({mlanc}); "
                f"e = ctypes.c_double(); ww = np.zeros(4096); "
                f"L.ref_warmup({lx}, {ly}, 0, {d}, ctypes.c_double({jc}), ctypes.c_double({qc}), 2, 1, "
                f"ctypes.byref(e), ww.ctypes.data_as(ctypes.c_void_p), 4096); "
                f"print('RESULT', repr(float(e.value)), ' '.join(repr(float(v)) for v in ww[:{d}]))")
        out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, check=True).stdout
        steps = [float(ln.split("=")[-1]) + 1000.0 for ln in out.splitlines() if ln.startswith("lanczos")]
        res = [ln for ln in out.splitlines() if ln.startswith("RESULT")][0].split()[1:]
        case.update(energy=np.float64(float(res[0])), ww=np.array([float(v) for v in res[1:]]),
                    step_energies=np.array(steps))
        cases.append(case)
    fuse = []
    for bonds in ([(-1, [0, 2, 4], [3, 2, 1]), (-1, [1], [1])], [(1, [1], [1]), (1, [0, 1, 2, 3], [2, 4, 1, 3])]):
        bd = desc_of(bonds)
        L.ref_fuse_tensor(p(bd))
        dd = np.zeros(1024, np.int32)
        nd = L.ref_result_desc(p(dd))
        flag, x1, _ = read_result(L)
        fuse.append(dict(bonds=bd, desc=dd[:nd].copy(), flag=flag, x=x1))
    cases.append(dict(name="fuse_tensor", **{f"{k}{i}": v for i, c in enumerate(fuse) for k, v in c.items()}))
    return cases


def main():
    L = ctypes.CDLL(REFLIB)
    if "--only-dmrg" in sys.argv:
        L.ref_setup(1, 25)
        with open(os.path.join(HERE, "dmrg_energies.json"), "w") as f:
            json.dump(dmrg_runs(L), f, indent=1)
        return
    if "--only-seeded" in sys.argv:
        L.ref_setup(1, 25)
        with open(os.path.join(HERE, "dmrg_seeded.json"), "w") as f:
            json.dump(seeded_runs(L), f, indent=1)
        return
    if "--only-lattices" in sys.argv:
        # lattice tables of the other boundary conditions (0 square, 1 J1-J3,
        # 3 Shastry-Sutherland), with and without plaquettes
        L.ref_setup(1, 25)
        out = {}
        for ci, (lx, ly, bd, jc, qc) in enumerate([(4, 4, 0, 1.0, 0.0), (6, 4, 1, 0.5, 0.0), (4, 4, 3, 0.7, 0.0),
                                                  (6, 4, 0, 1.0, 0.5), (4, 6, 3, 1.0, 1.0), (5, 4, 1, 2.0, 0.3)]):
            c = engine_tables(L, lx, ly, 16, jc, qc, bd)
            for k in ("lx", "ly", "jcoup", "qcoup", "tables", "coup"):
                out[f"c{ci}_{k}"] = c[k]
            out[f"c{ci}_boundary"] = np.int32(bd)
        np.savez(os.path.join(HERE, "lattice_tables.npz"), **out)
        return
    if "--only-siteops" in sys.argv:
        # the engine's spin-1/2 one-site operators (initialize_local_operators,
        # dmrg_su2.cpp:427-520), packaged with the library for Lattice.cylinder
        L.ref_setup(1, 25)
        c = engine_tables(L, 4, 2, 16, 1.0, 1.0)
        np.savez(os.path.join(REPO, "su2dmrg_gb300", "site_ops_spin_half.npz"),
                 **{k: v for k, v in c.items() if k.startswith("site")})
        return
    if "--only-sweep" in sys.argv:
        L.ref_setup(1, 25)
        for c in sweep_cases(L):
            name = c.pop("name")
            np.savez(os.path.join(HERE, name + ".npz"), **c)
        return
    if "--only-warmup" in sys.argv:
        L.ref_setup(1, 25)
        for c in warmup_cases(L):
            name = c.pop("name")
            np.savez(os.path.join(HERE, name + ".npz"), **c)
        return
    if "--only-mea" in sys.argv:
        L.ref_setup(1, 25)
        rng = np.random.Generator(np.random.PCG64(777))
        for c in measure_op_cases(L, rng) + mea_cases(L):
            name = c.pop("name")
            np.savez(os.path.join(HERE, name + ".npz"), **c)
        return
    if "--only-ckpt" in sys.argv:
        L.ref_setup(1, 25)
        np.savez(os.path.join(HERE, "ckpt_engine.npz"), **checkpoint_cases(L))
        return
    L.ref_setup(1, 25)
    rng = np.random.Generator(np.random.PCG64(20241203))
    fac = np.zeros(25**3)
    L.ref_fac_hamilt_vec(25, p(fac))
    np.save(os.path.join(HERE, "fac_hamilt_vec.npy"), fac.reshape(25, 25, 25))
    trip, vals = [], []
    for (j1, j2, j3) in [(0, 0, 0), (1, 1, 0), (1, 1, 2), (2, 2, 2), (3, 2, 1), (4, 2, 6), (5, 3, 4), (6, 6, 0),
                         (7, 2, 9), (12, 2, 12), (13, 1, 12), (24, 2, 22), (24, 24, 24), (9, 8, 7)]:
        c = np.zeros((j1 + 1) * (j2 + 1) * (j3 + 1))
        L.ref_make_cgc(j1, j2, j3, p(c))
        trip.append((j1, j2, j3))
        vals.append(c)
    np.savez(os.path.join(HERE, "cgc.npz"), triples=np.asarray(trip, np.int32), values=np.concatenate(vals),
             idx=np.cumsum([0] + [len(v) for v in vals]))
    np.savez(os.path.join(HERE, "meta.npz"), **meta_cases(L, rng))
    np.savez_compressed(os.path.join(HERE, "fac_optrans.npz"), **fac_optrans(L))
    np.savez_compressed(os.path.join(HERE, "fac_site.npz"), **fac_site_tables(L))
    for c in (heff_cases(L, rng) + spin0_cases(L, rng) + env_cases(L, rng) + svd_cases(L, rng) + site_cases(L, rng)
              + input_vector_cases(L, rng)):
        name = c.pop("name")
        np.savez(os.path.join(HERE, name + ".npz"), **c)
    if "--no-idmrg" not in sys.argv:
        for c in idmrg_cases(L):
            name = c.pop("name")
            np.savez_compressed(os.path.join(HERE, name + ".npz"), **c)
    np.savez(os.path.join(HERE, "ckpt_engine.npz"), **checkpoint_cases(L))
    for c in measure_op_cases(L, np.random.Generator(np.random.PCG64(777))) + mea_cases(L) + warmup_cases(L):
        name = c.pop("name")
        np.savez(os.path.join(HERE, name + ".npz"), **c)
    if "--no-dmrg" not in sys.argv:
        with open(os.path.join(HERE, "dmrg_energies.json"), "w") as f:
            json.dump(dmrg_runs(L), f, indent=1)


if __name__ == "__main__":
    main()
