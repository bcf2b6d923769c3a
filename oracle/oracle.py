"""ORACLE / TEST INFRASTRUCTURE ONLY.

Python side of the CPU oracle: loads oracle/liboracle.so (the C restatement of
the reference hot path, su2_oracle.c) and offers numpy-level helpers.  Only
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
module; the GPU library never does.

Block tensors use the reference checkpoint layout (dmrg_su2_omp.cpp:864-941):
``desc`` = [nbond, locspin, {dir, n, angm..., dim...} per leg], ``flag`` = one
int per block (mixed radix, leg 0 fastest), ``data`` = present blocks packed in
block order, each column-major.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
MAX_ANGM = 25  # dmrg_su2.cpp:46

_lib = None


def build() -> str:
    """Compile liboracle.so (gcc, a second or two)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def _capsule_ptr(capsule) -> int:
    get_name = ctypes.pythonapi.PyCapsule_GetName
    get_name.restype = ctypes.c_char_p
    get_name.argtypes = [ctypes.py_object]
    get_ptr = ctypes.pythonapi.PyCapsule_GetPointer
    get_ptr.restype = ctypes.c_void_p
    get_ptr.argtypes = [ctypes.py_object, ctypes.c_char_p]
    return get_ptr(capsule, get_name(capsule))


def lib():
    """The loaded oracle library, with SciPy's BLAS dgemm installed."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        import scipy.linalg.cython_blas as cb

        L.or_set_dgemm(ctypes.c_void_p(_capsule_ptr(cb.__pyx_capi__["dgemm"])))
        L.or_factorial.restype = ctypes.c_double
        L.or_offsets.restype = ctypes.c_int64
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def set_blas_threads(n: int) -> None:
    """Best effort: pin SciPy's bundled OpenBLAS to n threads (the oracle
    parallelises above BLAS)."""
    try:
        import glob

        import scipy

        d = os.path.join(os.path.dirname(scipy.__file__), "..", "scipy.libs")
        for so in glob.glob(os.path.join(d, "libscipy_openblas*.so")):
            ob = ctypes.CDLL(so)
            for name in ("scipy_openblas_set_num_threads", "openblas_set_num_threads"):
                if hasattr(ob, name):
                    getattr(ob, name)(int(n))
                    return
    except OSError:
        pass


# --------------------------------------------------------------------------
# structures
# --------------------------------------------------------------------------
@dataclass
class Bond:
    """su2bond (su2bond.hpp:3-29): direction, 2j per sector, multiplet dims."""

    dir: int
    angm: list
    dim: list

    def inverted(self) -> "Bond":
        return Bond(-self.dir, list(self.angm), list(self.dim))


@dataclass
class Struct:
    """su2struct (su2struct.hpp:4-40) plus the block presence flags."""

    bonds: list
    locspin: int = 0
    flag: np.ndarray = field(default=None)

    def desc(self) -> np.ndarray:
        d = [len(self.bonds), self.locspin]
        for b in self.bonds:
            d += [b.dir, len(b.angm)] + list(b.angm) + list(b.dim)
        return np.asarray(d, dtype=np.int32)

    @property
    def nten(self) -> int:
        n = 1
        for b in self.bonds:
            n *= len(b.angm)
        return n

    def legal(self) -> np.ndarray:
        out = np.zeros(self.nten, dtype=np.int32)
        lib().or_legal_blocks(_p(self.desc()), _p(out))
        return out

    def with_legal_flags(self) -> "Struct":
        self.flag = self.legal()
        return self

    def offsets(self):
        off = np.zeros(self.nten, dtype=np.int64)
        total = lib().or_offsets(_p(self.desc()), _p(self.flag.astype(np.int32)), _p(off))
        return off, int(total)

    def block_shape(self, idx: int):
        shp = []
        for b in self.bonds:
            shp.append(b.dim[idx % len(b.angm)])
            idx //= len(b.angm)
        return tuple(shp)

    def block_angm(self, idx: int):
        out = []
        for b in self.bonds:
            out.append(b.angm[idx % len(b.angm)])
            idx //= len(b.angm)
        return tuple(out)


def fuse(b1: Bond, b2: Bond) -> Bond:
    """su2bond::fuse (su2bond.cpp:155-210): direction of the result is -b1.dir."""
    aout = np.zeros(128, np.int32)
    dout = np.zeros(128, np.int32)
    a1 = np.asarray(b1.angm, np.int32)
    d1 = np.asarray(b1.dim, np.int32)
    a2 = np.asarray(b2.angm, np.int32)
    d2 = np.asarray(b2.dim, np.int32)
    n = lib().or_fuse(len(a1), _p(a1), _p(d1), len(a2), _p(a2), _p(d2), _p(aout), _p(dout))
    return Bond(-b1.dir, aout[:n].tolist(), dout[:n].tolist())


# --------------------------------------------------------------------------
# tables
# --------------------------------------------------------------------------
def fac_hamilt_vec(max_angm: int = MAX_ANGM) -> np.ndarray:
    out = np.zeros(max_angm**3, dtype=np.float64)
    lib().or_fac_hamilt_vec(max_angm, _p(out))
    return out.reshape(max_angm, max_angm, max_angm)


def make_cgc(j1: int, j2: int, j3: int) -> np.ndarray:
    out = np.zeros((j1 + 1) * (j2 + 1) * (j3 + 1), dtype=np.float64)
    lib().or_make_cgc(j1, j2, j3, _p(out))
    return out


_FAC = None


def fac_table() -> np.ndarray:
    global _FAC
    if _FAC is None:
        _FAC = np.ascontiguousarray(fac_hamilt_vec(MAX_ANGM).ravel())
    return _FAC


# --------------------------------------------------------------------------
# H_eff pieces
# --------------------------------------------------------------------------
def heff_term(vs: Struct, vx, s1: Struct, x1, s2: Struct, x2, ys: Struct, y, coef=1.0) -> None:
    """y += coef * hamiltonian_vector_multiplication(vec, op1, op2)."""
    fac = fac_table()
    rc = lib().or_heff_term(
        _p(vs.desc()), _p(vs.flag.astype(np.int32)), _p(vx),
        _p(s1.desc()), _p(s1.flag.astype(np.int32)), _p(x1),
        _p(s2.desc()), _p(s2.flag.astype(np.int32)), _p(x2),
        _p(ys.desc()), _p(ys.flag.astype(np.int32)), _p(y),
        ctypes.c_double(coef), _p(fac), MAX_ANGM)
    if rc != 0:
        raise RuntimeError(f"or_heff_term failed: {rc}")


def heff_spin0(side: int, hs: Struct, hx, vs: Struct, vx, ys: Struct, y, coef=1.0) -> None:
    """y += coef * (H^T vec) for side 0, y += coef * (vec H) for side 1."""
    rc = lib().or_heff_spin0(
        side, _p(hs.desc()), _p(hs.flag.astype(np.int32)), _p(hx),
        _p(vs.desc()), _p(vs.flag.astype(np.int32)), _p(vx),
        _p(ys.desc()), _p(ys.flag.astype(np.int32)), _p(y), ctypes.c_double(coef))
    if rc != 0:
        raise RuntimeError(f"or_heff_spin0 failed: {rc}")


@dataclass
class HeffProblem:
    """One effective-Hamiltonian application: y = H_L^T psi + psi H_R
    + sum_t coef_t * [L_t psi R_t] (the orchestration of dmrg_su2.cpp:543-664
    with the complementary operators already combined)."""

    psi: Struct
    terms: list  # [(Struct op1, data1, Struct op2, data2, coef)]
    hl: tuple = None  # (Struct, data[, coef]) or None
    hr: tuple = None


def heff_apply(prob: HeffProblem, psi: np.ndarray) -> np.ndarray:
    y = np.zeros_like(psi)
    for side, h in ((0, prob.hl), (1, prob.hr)):
        if h is not None:
            coef = h[2] if len(h) > 2 else 1.0
            heff_spin0(side, h[0], h[1], prob.psi, psi, prob.psi, y, coef)
    for (s1, x1, s2, x2, c) in prob.terms:
        if len(s1.bonds) == 2 and len(s2.bonds) == 2:
            heff_scalar_pair(prob.psi, psi, s1, x1, s2, x2, prob.psi, y, c)
        else:
            heff_term(prob.psi, psi, s1, x1, s2, x2, prob.psi, y, c)
    return y


def heff_scalar_pair(vs: Struct, vx, s1: Struct, x1, s2: Struct, x2, ys: Struct, y, coef=1.0) -> None:
    """y += coef * hamiltonian_vector_multiplication(vec, op1, op2) for two
    2-leg scalar operators: contract(contract(op1, 0, vec, 0), 1, op2, 0)
    (tensor_su2_dmrg_src.cpp:902-906), i.e. (L^T psi) R per spin sector."""
    V, L, R = _blocks(vs, vx), _blocks(s1, x1), _blocks(s2, x2)
    yoff, _ = ys.offsets()
    for k, vb in V.items():
        ja, jb = vs.block_angm(k)
        for j, lb in L.items():
            if s1.block_angm(j)[0] != ja:
                continue
            jc = s1.block_angm(j)[1]
            t = lb.T @ vb
            for l, rb in R.items():
                if s2.block_angm(l)[0] != jb:
                    continue
                jd = s2.block_angm(l)[1]
                if jc != jd:
                    continue
                sec = (ys.bonds[0].angm.index(jc), ys.bonds[1].angm.index(jd))
                m = sec[0] + len(ys.bonds[0].angm) * sec[1]
                if not ys.flag[m]:
                    raise RuntimeError("scalar pair reaches a block the output layout does not store")
                blk = coef * (t @ rb)
                y[yoff[m]: yoff[m] + blk.size] += blk.ravel(order="F")


def heff_flops(prob: HeffProblem) -> float:
    """Algorithmic FLOPs of one application: 2*a*b*(m_s c) for step1 and
    2*c*(b m_s)*d for the second product, per contributing block pair, plus
    2*d^3-type products for the spin-0 terms."""
    fac = fac_table().reshape(MAX_ANGM, MAX_ANGM, MAX_ANGM)
    ps = prob.psi
    total = 0.0
    vblocks = [i for i in range(ps.nten) if ps.flag[i]]
    for (s1, _x1, s2, _x2, _c) in prob.terms:
        for k in vblocks:
            ja, jb = ps.block_angm(k)
            a, b = ps.block_shape(k)
            for j in range(s1.nten):
                if not s1.flag[j]:
                    continue
                a1 = s1.block_angm(j)
                if a1[0] != ja:
                    continue
                _, ms, c = s1.block_shape(j)
                used = False
                for l in range(s2.nten):
                    if not s2.flag[l]:
                        continue
                    a3 = s2.block_angm(l)
                    if a3[0] != jb or a3[1] != a1[1] or a3[2] != a1[2]:
                        continue
                    if abs(fac[a1[0], a1[1], a1[2]]) < 1e-12:
                        continue
                    d = s2.block_shape(l)[2]
                    total += 2.0 * c * (b * ms) * d
                    used = True
                if used:
                    total += 2.0 * a * b * ms * c
    for side, h in ((0, prob.hl), (1, prob.hr)):
        if h is None:
            continue
        for k in vblocks:
            a, b = ps.block_shape(k)
            total += 2.0 * a * b * (a if side == 0 else b)
    return total


# --------------------------------------------------------------------------
# Lanczos (lanczos_su2::lanczos1, lanczos_su2.cpp:125-195)
# --------------------------------------------------------------------------
def _tridiag(aal, nnl, m):
    from scipy.linalg import eigh_tridiagonal

    d = np.asarray(aal[:m], float)
    e = np.asarray(nnl[1:m], float)
    if m == 1:
        return d.copy(), np.ones((1, 1))
    return eigh_tridiagonal(d, e)


def lanczos1(matvec, psi: np.ndarray, mlanc: int = 5):
    """Restatement of lanczos_su2::lanczos1 with the start-vector
    normalisation of initialize_lanczos (lanczos_su2.cpp:36-47) and the mlanc
    clamp of dmrg_su2.cpp:532.  Returns (eigenvalue, eigenvector, nmatvec)."""
    n = psi.size
    if mlanc > n:
        mlanc = n + 1
    tol = 1.0e-6
    nmv = [0]

    def H(v):
        nmv[0] += 1
        return matvec(v)

    ff = [None] * (mlanc + 1)
    ff[0] = psi / np.sqrt(psi @ psi)
    aal = np.zeros(mlanc)
    nnl = np.zeros(mlanc + 1)

    def vout_of(z, m):
        v = ff[0] * z[0]
        for j in range(1, m):
            v = v + ff[j] * z[j]
        return v

    def check(v):
        v = v / np.sqrt(v @ v)
        hv = H(v)
        prod = np.sqrt(hv @ hv)
        return v, prod, abs((hv @ v) / prod)

    ff[1] = H(ff[0])
    aal[0] = ff[0] @ ff[1]
    ff[1] = ff[1] - aal[0] * ff[0]
    nnl[1] = np.sqrt(ff[1] @ ff[1])
    ff[1] = ff[1] / nnl[1]
    if mlanc == 2:
        if nnl[1] < tol:
            w, z = _tridiag(aal, nnl, 1)
            return w[0], vout_of(z[:, 0], 1), nmv[0]
        ff[2] = H(ff[1])
        aal[1] = ff[1] @ ff[2]
        w, z = _tridiag(aal, nnl, 2)
        return w[0], vout_of(z[:, 0], 2), nmv[0]
    for m in range(2, mlanc):
        ff[m] = H(ff[m - 1])
        aal[m - 1] = ff[m - 1] @ ff[m]
        ff[m] = ff[m] - aal[m - 1] * ff[m - 1]
        ff[m] = ff[m] - nnl[m - 1] * ff[m - 2]
        for j in range(m):
            q = ff[m] @ ff[j]
            ff[m] = ff[m] - q * ff[j]
        nnl[m] = np.sqrt(ff[m] @ ff[m])
        ff[m] = ff[m] / nnl[m]
        w, z = _tridiag(aal, nnl, m)
        if nnl[m] < tol:
            v, _, _ = check(vout_of(z[:, 0], m))
            return w[0], v, nmv[0]
        if m % 4 == 0:
            v, _, ov = check(vout_of(z[:, 0], m))
            if abs(ov - 1.0) < 1.0e-8:
                return w[0], v, nmv[0]
    ff[mlanc] = H(ff[mlanc - 1])
    aal[mlanc - 1] = ff[mlanc - 1] @ ff[mlanc]
    w, z = _tridiag(aal, nnl, mlanc)
    v, _, _ = check(vout_of(z[:, 0], mlanc))
    return w[0], v, nmv[0]


def struct_from_desc(desc, flag=None) -> Struct:
    """Struct from the int desc array ([nbond, locspin, {dir, n, angm, dim}...])."""
    d = [int(v) for v in desc]
    nb, loc, p = d[0], d[1], 2
    bonds = []
    for _ in range(nb):
        dr, n = d[p], d[p + 1]
        bonds.append(Bond(dr, d[p + 2: p + 2 + n], d[p + 2 + n: p + 2 + 2 * n]))
        p += 2 + 2 * n
    s = Struct(bonds, loc)
    s.flag = np.asarray(flag, np.int32) if flag is not None else s.legal()
    return s


def to_layout(src: Struct, x: np.ndarray, dst: Struct) -> np.ndarray:
    """Re-pack block data of src's layout into dst's layout (same block space);
    blocks absent from src become zeros, blocks absent from dst are dropped
    (they must be zero for the caller's comparison to be meaningful)."""
    so, _ = src.offsets()
    do, dt = dst.offsets()
    out = np.zeros(dt)
    for i in range(dst.nten):
        if dst.flag[i] and src.flag[i]:
            n = int(np.prod(dst.block_shape(i)))
            out[do[i]: do[i] + n] = x[so[i]: so[i] + n]
    return out


# --------------------------------------------------------------------------
# Environment updates (tensor_su2_dmrg_src.cpp:221-402, 531-688)
# --------------------------------------------------------------------------
def fac_operator_transformation(side, j, m, l, i, k, p):
    f = lib().or_fac_operator_transformation
    f.restype = ctypes.c_double
    return f(side, j, m, l, i, k, p)


def env_out_struct(kind: int, su: Struct, so: Struct, sv: Struct) -> Struct:
    """Output structure of the transformations: (uu leg 2[, op leg 1], vv leg 2 inverted)."""
    legs = [su.bonds[2]] + ([so.bonds[1]] if kind else []) + [sv.bonds[2].inverted()]
    return Struct(legs, 0)


def env_transform(kind: int, su: Struct, xu, sv: Struct, xv, so: Struct, xo, flag: int):
    """Returns (out Struct with the reference's presence flags, packed data)."""
    out = env_out_struct(kind, su, so, sv)
    fout = np.zeros(out.nten, np.int32)
    args = (kind, _p(su.desc()), _p(su.flag.astype(np.int32)), _p(np.ascontiguousarray(xu)),
            _p(sv.desc()), _p(sv.flag.astype(np.int32)), _p(np.ascontiguousarray(xv)),
            _p(so.desc()), _p(so.flag.astype(np.int32)), _p(np.ascontiguousarray(xo)), flag, _p(out.desc()), _p(fout))
    if lib().or_env_transform(*args, None) != 0:
        raise RuntimeError("or_env_transform failed (layout)")
    out.flag = fout
    _, total = out.offsets()
    y = np.zeros(total)
    if lib().or_env_transform(*args, _p(y)) != 0:
        raise RuntimeError("or_env_transform failed")
    return out, y


# --------------------------------------------------------------------------
# Truncation (tensor_su2::svd, tensor_su2.cpp:1619-1758; tensor::svd,
# tensor.cpp:1472-1700)
# --------------------------------------------------------------------------
def _eigh(a):
    """dsyev, eigenvalues ascending (obtain_symmetric_matrix_eigenvector, tensor.cpp:731-759)."""
    from scipy.linalg import eigh

    w, v = eigh(a, driver="ev")
    return w, v


def _refine(G, w, v, n):
    """Re-diagonalise the subspace of eigenvalues below 0.1 of the largest,
    repeatedly (tensor.cpp:1491-1527)."""
    tol1 = 1.0e-1
    np_ = 0
    for i in range(n - 1, -1, -1):
        if w[i] / w[n - 1] < tol1:
            np_ = i + 1
            break
    if np_ <= 1:
        return w, v
    ap = G.copy()
    vp = v.copy()
    npp = np_
    np_ = n
    w = w.copy()
    v = v.copy()
    while True:
        vsub = vp[:np_, :npp]
        vpp = vsub.T @ ap[:np_, :np_] @ vsub
        ap = vpp.copy()
        ww, vv = _eigh(vpp)
        w[:npp] = ww
        v[:, :npp] = v[:, :npp] @ vv
        vp = vv
        j = 0
        for i in range(npp - 1, -1, -1):
            if ww[i] / ww[npp - 1] < tol1:
                j = i + 1
                break
        np_ = npp
        npp = j
        if npp <= 1:
            break
    return w, v


def tensor_svd(blk, p1, p2, max_dcut):
    """One sector: returns (u (m x dcut), v (n x dcut), s ascending (dcut))."""
    m, n = blk.shape
    tol = 1.0e-100
    if m >= n:
        G = blk.T @ blk
        w, v = _eigh(G)
        w, v = _refine(G, w, v, n)
        u = blk @ v
        k = n
    else:
        G = blk @ blk.T
        w, u = _eigh(G)
        w, u = _refine(G, w, u, m)
        v = blk.T @ u
        k = m
    w = w.copy()
    num = w[k - 1]
    dcut = 0
    if num > tol:
        for i in range(k - 1, -1, -1):
            if w[i] / num > tol:
                w[i] = np.sqrt(w[i])
                dcut += 1
            else:
                w[i] = 0
    dcut = min(dcut, max_dcut, m if m >= n else n)
    for i in range(k - 1, k - dcut - 1, -1):
        if w[i] > 0:
            if m >= n:
                u[:, i] *= w[i] ** (p1 - 1.0)
                v[:, i] *= w[i] ** p2
            else:
                v[:, i] *= w[i] ** (p2 - 1.0)
                u[:, i] *= w[i] ** p1
        else:
            u[:, i] = 0
            v[:, i] = 0
    return u[:, k - dcut:], v[:, k - dcut:], w[k - dcut:k].copy()


def svd_truncate(vs: Struct, x, p1, p2, max_dcut):
    """Returns (kept per leg-0 sector, wout (kept, then discarded), [(u, v) per sector])."""
    off, _ = vs.offsets()
    n0, n1 = len(vs.bonds[0].angm), len(vs.bonds[1].angm)
    res = {}
    wsort, isort = [], []
    for i in range(n0):
        for j in range(n1):
            if vs.bonds[0].angm[i] != vs.bonds[1].angm[j]:
                continue
            b = i + j * n0
            if not vs.flag[b]:
                continue
            m, n = vs.bonds[0].dim[i], vs.bonds[1].dim[j]
            blk = np.asarray(x[off[b]: off[b] + m * n]).reshape(m, n, order="F")
            u, v, s = tensor_svd(blk, p1, p2, max_dcut)
            res[i] = (u, v, s)
            wsort += list(s)
            isort += [i] * len(s)
    n = len(wsort)
    ws = np.asarray(wsort, np.float64)
    iss = np.asarray(isort, np.int32)
    lib().dsort2_(ctypes.byref(ctypes.c_int(n)), _p(ws), _p(iss))
    dims = np.zeros(n0, np.int32)
    for i in range(n - 1, max(0, n - max_dcut) - 1, -1):
        dims[iss[i]] += 1
    kept_w, disc_w, uv = [], [], {}
    for i in range(n0):
        if i not in res:
            continue
        u, v, s = res[i]
        dc, d = len(s), dims[i]
        if d > 0:
            kept_w += list(s[dc - d:])
            disc_w += list(s[:dc - d])
            uv[i] = (u[:, dc - d:], v[:, dc - d:])
        else:
            disc_w += list(s)
    return dims, np.asarray(kept_w + disc_w), uv


def _fused_rows(b0: Bond, b1: Bond, c: int):
    """Row ranges of the (a, sigma) sub-blocks inside fused sector 2j = c, in the
    order tensor_su2::fuse places them (tensor_su2.cpp:878-900): sigma sectors
    outer, bond sectors inner, d_a * d_sigma rows each (a fastest)."""
    rows, pos = {}, 0
    for j1, s in enumerate(b1.angm):
        for j0, a in enumerate(b0.angm):
            if abs(a - s) <= c <= a + s and (a + s - c) % 2 == 0:
                rows[(j0, j1)] = (pos, b0.dim[j0] * b1.dim[j1])
                pos += b0.dim[j0] * b1.dim[j1]
    return rows


def svd_mps(vs: Struct, dims, uv, tu_bonds, tv_bonds):
    """The new MPS tensors of tensor_su2::svd (tensor_su2.cpp:1733-1745):
    tu = fuse(tu legs 0, 1) contracted with the kept U columns, tv likewise
    with V; new bond of direction -1 with the kept multiplets.  The fuse
    tensor is a row placement with canonical CG, so each block of tu is a row
    range of its sector's U.  Returns ((tu Struct, x), (tv Struct, x))."""
    n0 = len(vs.bonds[0].angm)
    kept = [i for i in range(n0) if dims[i] > 0]
    newb = Bond(-1, [vs.bonds[0].angm[i] for i in kept], [int(dims[i]) for i in kept])
    res = []
    for side, (b0, b1) in ((0, tu_bonds), (1, tv_bonds)):
        S = Struct([b0, b1, newb], 0).with_legal_flags()
        off, tot = S.offsets()
        x = np.zeros(tot)
        for bi in range(S.nten):
            if not S.flag[bi]:
                continue
            j0, j1, j2 = bi % len(b0.angm), (bi // len(b0.angm)) % len(b1.angm), bi // (len(b0.angm) * len(b1.angm))
            c = newb.angm[j2]
            r0, m = _fused_rows(b0, b1, c)[(j0, j1)]
            mat = uv[vs.bonds[0].angm.index(c)][side]
            x[off[bi]: off[bi] + m * newb.dim[j2]] = mat[r0: r0 + m, :].ravel(order="F")
        res.append((S, x))
    return tuple(res)


def mps_sector_matrices(S: Struct, x):
    """Inverse of the placement in svd_mps: {2j of leg 2: (fused rows x kept)}."""
    b0, b1, b2 = S.bonds
    off, _ = S.offsets()
    out = {}
    for j2, c in enumerate(b2.angm):
        rows = _fused_rows(b0, b1, c)
        nrow = sum(m for _, m in rows.values())
        mat = np.zeros((nrow, b2.dim[j2]))
        for (j0, j1), (r0, m) in rows.items():
            bi = j0 + len(b0.angm) * (j1 + len(b1.angm) * j2)
            if S.flag[bi]:
                mat[r0: r0 + m, :] = np.asarray(x[off[bi]: off[bi] + m * b2.dim[j2]]).reshape(m, -1, order="F")
        out[c] = mat
    return out


# --------------------------------------------------------------------------
# Site updates: operator_initial (tensor_su2_dmrg_src.cpp:27-218),
# operator_pairup (:691-890), permutation (tensor_su2_hamiltonian.cpp:871-1108)
# and their recoupling tables (dmrg_su2.cpp:776-1019)
# --------------------------------------------------------------------------
def _cg(a, b, c):
    return make_cgc(a, b, c).reshape((a + 1, b + 1, c + 1), order="F")


def make_singlet(j):
    """tensor::make_singlet (tensor.cpp:1331-1350): S[r, j - r] = (-1)^((j - m_r)/2) / sqrt(j + 1)."""
    s = np.zeros((j + 1, j + 1))
    for r in range(j + 1):
        m = 2 * r - j
        s[r, j - r] = (1 if ((j - m) // 2) % 2 == 0 else -1) / np.sqrt(j + 1.0)
    return s


def _ratio(t, ref):
    """tensor::is_proportional_to (tensor.cpp:1231-1269); None if not proportional."""
    tol = 1e-12
    tt, rr = t.ravel(order="F"), ref.ravel(order="F")
    if np.all(np.abs(tt) <= tol):
        return 0.0
    pos = int(np.argmax(np.abs(rr)))
    rat = tt[pos] / rr[pos]
    for a, b in zip(tt, rr):
        if abs(a) <= tol and abs(b) <= tol:
            continue
        if (abs(a) <= tol) != (abs(b) <= tol) or abs(a / b - rat) > tol:
            return None
    return rat


def _tri(a, b, c):
    return abs(a - b) <= c <= a + b


_SITE_CACHE = {}


def fac_operator_onsite(side, j, m, l, i, q):
    """fac_operator_onsite_{left,rght}[j][m][l][i][p0 + 3 p1] (dmrg_su2.cpp:804-833)."""
    p0, p1 = q % 3, q // 3
    if not (0 <= q < 9 and m in (0, 2, 4, 6) and _tri(i, p0, j) and _tri(i, p1, l) and _tri(j, m, l)
            and j % 2 == l % 2 and _tri(p0, m, p1)):
        return 0.0
    key = (0, side, j, m, l, i, q)
    if key not in _SITE_CACHE:
        if side == 0:
            t = np.einsum("iaj,amb,ibl->jml", _cg(i, p0, j), _cg(p0, m, p1), _cg(i, p1, l))
        else:
            t = np.einsum("aij,amb,bil->jml", _cg(p0, i, j), _cg(p0, m, p1), _cg(p1, i, l))
        r = _ratio(t, _cg(j, m, l))
        _SITE_CACHE[key] = 0.0 if r is None else float(r)
    return _SITE_CACHE[key]


def fac_operator_pairup(side, j, i, k, m, q):
    """fac_operator_pairup_{left,rght}[j][i][k][m][p0 + 3 p1] (dmrg_su2.cpp:920-943)."""
    p0, p1 = q % 3, q // 3
    if not (0 <= q < 9 and m in (0, 2, 4, 6) and _tri(i, p0, j) and _tri(k, p1, j) and _tri(i, m, k)
            and _tri(p0, m, p1)):
        return 0.0
    key = (1, side, j, i, k, m, q)
    if key not in _SITE_CACHE:
        w = np.sqrt(m + 1.0) * np.einsum("amb,nm->anb", _cg(p0, m, p1), make_singlet(m))
        if side == 0:
            t = np.einsum("iaj,imk,amb,kbl->jl", _cg(i, p0, j), _cg(i, m, k), w, _cg(k, p1, j))
        else:
            t = np.einsum("aij,imk,amb,bkl->jl", _cg(p0, i, j), _cg(i, m, k), w, _cg(p1, k, j))
        r = _ratio(t, np.eye(j + 1))
        _SITE_CACHE[key] = 0.0 if r is None else float(r)
    return _SITE_CACHE[key]


def fac_permutation(side, i, j, k, l, t):
    """fac_permutation_{left,rght}[i][j][k][l][t] for spin-1/2 sites (dmrg_su2.cpp:974-1017)."""
    P = 1
    if not (0 <= t < 18 and _tri(i, P, j) and _tri(k, P, l)):
        return 0.0
    a1, a2, a3 = (t % 3) * 2, ((t // 3) % 2) * 2 + 1, ((t // 6) % 3) * 2
    if not (_tri(a1, P, a2) and _tri(a2, P, a3)) or i % 2 != k % 2 or j % 2 != l % 2:
        return 0.0
    key = (2, side, i, j, k, l, t)
    if key not in _SITE_CACHE:
        r = None
        if side == 0 and _tri(a1, i, k) and _tri(a3, j, l):
            tt = np.einsum("iqj,qxy,iak,pay,kpl->jxl", _cg(i, P, j), _cg(P, a3, a2), _cg(i, a1, k), _cg(P, a1, a2),
                           _cg(k, P, l))
            r = _ratio(tt, _cg(j, a3, l))
        if side == 1 and _tri(a3, i, k) and _tri(a1, j, l):
            tt = np.einsum("qij,yqx,ixk,ypa,pkl->jal", _cg(P, i, j), _cg(a2, P, a3), _cg(i, a3, k), _cg(a2, P, a1),
                           _cg(P, k, l))
            r = _ratio(tt, _cg(j, a1, l))
        _SITE_CACHE[key] = 0.0 if r is None else float(r)
    return _SITE_CACHE[key]


def _blocks(S: Struct, x):
    """{block index: F-ordered array} of the present blocks."""
    off, _ = S.offsets()
    out = {}
    for b in range(S.nten):
        if S.flag[b]:
            shp = S.block_shape(b)
            out[b] = np.asarray(x[off[b]: off[b] + int(np.prod(shp))]).reshape(shp, order="F")
    return out


def site_update(kind: str, flag: int, su: Struct, xu, sv: Struct, xv, x=None, sites=()):
    """kind 'init' (x = endt or None), 'pair' (x = op1), 'perm' (x = vec); sites
    = [(Struct, host data), ...].  Returns (out Struct with the reference's
    presence flags, packed data).  Physical legs of multiplicity 1."""
    pl = 1 - flag
    U, V = _blocks(su, xu), _blocks(sv, xv)
    X = _blocks(*x) if x is not None else None
    XS = x[0] if x is not None else None
    site = [(_blocks(s, d), s) for s, d in sites]
    if kind == "pair":
        ybonds = [su.bonds[2], sv.bonds[2].inverted()]
    elif kind == "init":
        ybonds = [su.bonds[2], sites[0][0].bonds[1], sv.bonds[2].inverted()]
    else:
        mid = sites[1][0].bonds[1] if flag == 0 else sites[0][0].bonds[2]
        ybonds = [su.bonds[2], mid, sv.bonds[2].inverted()]
    Y = Struct(ybonds, 0)
    legal = Y.legal()
    acc = {}

    def umat(blk):  # (bond multiplets, c): the physical leg has multiplicity 1
        return blk.reshape(-1, blk.shape[2], order="F")

    def add(ang, mat):
        sec = [Y.bonds[q].angm.index(a) if a in Y.bonds[q].angm else -1 for q, a in enumerate(ang)]
        if min(sec) < 0:
            return False
        b = 0
        for q in range(len(sec) - 1, -1, -1):
            b = b * len(Y.bonds[q].angm) + sec[q]
        if not legal[b]:
            return False
        acc[b] = acc.get(b, 0) + mat
        return True

    ua = lambda k: su.block_angm(k)
    va = lambda l: sv.block_angm(l)
    if kind == "init":
        (sb, ss), = site
        for j, op in sb.items():
            sig, s, sigp = ss.block_angm(j)
            for k, ub in U.items():
                if ua(k)[pl] != sig:
                    continue
                a, c = ua(k)[flag], ua(k)[2]
                ends = [(None, a)] if X is None else [(e, XS.block_angm(e)[1]) for e in X if XS.block_angm(e)[0] == a]
                for e, ap in ends:
                    left = umat(ub) if e is None else X[e].T @ umat(ub)
                    for l, vb in V.items():
                        if va(l)[pl] != sigp or va(l)[flag] != ap:
                            continue
                        cp = va(l)[2]
                        fac = fac_operator_onsite(flag, c, s, cp, ap, sig + sigp * 3)
                        if abs(fac) < 1e-8:
                            continue
                        add((c, s, cp), (fac * op.ravel()[0] * (left.T @ umat(vb)))[:, None, :])
    elif kind == "pair":
        (sb, ss), = site
        for j, xb in X.items():
            a, s, ap = XS.block_angm(j)
            for k, ub in U.items():
                if ua(k)[flag] != a:
                    continue
                sig, c = ua(k)[pl], ua(k)[2]
                for l, vb in V.items():
                    if va(l)[flag] != ap:
                        continue
                    sigp, cp = va(l)[pl], va(l)[2]
                    for n, ob in sb.items():
                        if ss.block_angm(n) != (sig, s, sigp):
                            continue
                        fac = fac_operator_pairup(flag, c, a, ap, s, sig + sigp * 3)
                        if abs(fac) < 1e-8:
                            continue
                        tot = sum(ob.ravel()[g] * (umat(ub).T @ xb[:, g, :] @ umat(vb)) for g in range(xb.shape[1]))
                        add((c, cp), fac * tot)
    else:
        (b1, s1), (b2, s2) = site
        for j, ub in U.items():
            a, sig, c = ua(j)[flag], ua(j)[pl], ua(j)[2]
            for k, xb in X.items():
                if XS.block_angm(k)[0] != a:
                    continue
                s, ap = XS.block_angm(k)[1], XS.block_angm(k)[2]
                for l, vb in V.items():
                    if va(l)[flag] != ap:
                        continue
                    sigp, cp = va(l)[pl], va(l)[2]
                    core = umat(ub).T @ xb[:, 0, :] @ umat(vb)
                    for m, o1 in b1.items():
                        a4 = s1.block_angm(m)
                        for n, o2 in b2.items():
                            a5 = s2.block_angm(n)
                            if (flag == 0 and a4[2] != a5[2]) or (flag == 1 and a4[0] != a5[0]):
                                continue
                            if (flag == 0 and a4[1] != s) or (flag == 1 and a5[2] != s):
                                continue
                            if sig != a5[flag] or sigp != a4[flag]:
                                continue
                            so = a5[1] if flag == 0 else a4[2]
                            # C integer division, as the reference computes the index
                            cdiv = lambda x: int(x / 2)
                            t = (a4[1] // 2 + cdiv(a4[2] - 1) * 3 + (a5[1] // 2) * 6 if flag == 0
                                 else a4[2] // 2 + cdiv(a4[0] - 1) * 3 + (a5[2] // 2) * 6)
                            fac = fac_permutation(flag, a, c, ap, cp, t)
                            if abs(fac) < 1e-8:
                                continue
                            fac1 = float(np.dot(o1.ravel(order="F"), o2.ravel(order="F")))
                            add((c, so, cp), (fac * fac1 * core)[:, None, :])
    Y.flag = np.zeros(Y.nten, np.int32)
    for b in acc:
        Y.flag[b] = 1
    off, tot = Y.offsets()
    y = np.zeros(tot)
    for b, mat in acc.items():
        y[off[b]: off[b] + mat.size] = np.asarray(mat).ravel(order="F")
    return Y, y


# --------------------------------------------------------------------------
# Initial vector of a step and the vectran leg rotations
# (dmrg_su2::prepare_input_vector dmrg_su2_omp.cpp:229-254,
#  tensor_su2::right2left_vectran / left2right_vectran tensor_su2.cpp)
# --------------------------------------------------------------------------
def prepare_input_vector(sl: Struct, xl, sr: Struct, xr):
    """The two-site vector psi(F_L, F_R) of uu[il] (sl) and uu[ir] (sr): per
    spin sector c of their shared leg 2, psi_cc = U_L,c U_R,c^T with U the
    fused-row placements of the blocks (legs 0, 1 fused as tensor_su2::fuse
    orders them); every diagonal block present (makeup_input_vector, zeros
    where c is no sector of the shared leg).  Returns (Struct, data)."""
    fl = fuse(sl.bonds[0], sl.bonds[1])
    fr = fuse(sr.bonds[0], sr.bonds[1])
    V = Struct([Bond(sl.bonds[0].dir, fl.angm, fl.dim), Bond(sr.bonds[0].dir, fr.angm, fr.dim)], 0).with_legal_flags()
    UL, UR = mps_sector_matrices(sl, xl), mps_sector_matrices(sr, xr)
    off, tot = V.offsets()
    y = np.zeros(tot)
    for b in range(V.nten):
        if not V.flag[b]:
            continue
        c = V.block_angm(b)[0]
        if c in UL and c in UR:
            blk = UL[c] @ UR[c].T
            y[off[b]: off[b] + blk.size] = blk.ravel(order="F")
    return V, y


def vectran(s: Struct, x, direction: int):
    """right2left_vectran (direction 0: legs (0,1,2) -> (2,0,1)) or
    left2right_vectran (1: -> (1,2,0)): each block's legs rotated, the
    directions set to (+1, +1, -1), canonical CG kept."""
    shift = 1 if direction == 0 else 2  # new position of old leg q: (q + shift) % 3
    bonds = [None] * 3
    for q in range(3):
        bonds[(q + shift) % 3] = s.bonds[q]
    bonds = [Bond(d, list(b.angm), list(b.dim)) for d, b in zip((1, 1, -1), bonds)]
    out = Struct(bonds, s.locspin)
    out.flag = np.zeros(out.nten, np.int32)
    src = _blocks(s, x)
    dst = {}
    for b, blk in src.items():
        secs = []
        i = b
        for q in range(3):
            secs.append(i % len(s.bonds[q].angm))
            i //= len(s.bonds[q].angm)
        ns = [0] * 3
        for q in range(3):
            ns[(q + shift) % 3] = secs[q]
        nb = ns[0] + len(bonds[0].angm) * (ns[1] + len(bonds[1].angm) * ns[2])
        axes = [0] * 3  # new axis k takes old axis axes[k]
        for q in range(3):
            axes[(q + shift) % 3] = q
        dst[nb] = np.transpose(blk, axes)
        out.flag[nb] = 1
    off, tot = out.offsets()
    y = np.zeros(tot)
    for b, blk in dst.items():
        y[off[b]: off[b] + blk.size] = blk.ravel(order="F")
    return out, y


# --------------------------------------------------------------------------
# Centre-bond energy (dmrg_su2::mea_enr, dmrg_su2_omp_mea_enr.cpp:194-242)
# and its reductions (tensor_su2.cpp:359-384, 687-742)
# --------------------------------------------------------------------------
def take_trace(s: Struct, x) -> float:
    """Sum of the traces of the blocks of equal spins (no (2j+1) weight)."""
    t = 0.0
    for b, blk in _blocks(s, x).items():
        a = s.block_angm(b)
        if a[0] == a[1]:
            t += float(np.trace(blk))
    return t


def ss_inner_prod(sa: Struct, xa, sb: Struct, xb) -> float:
    """Block overlaps weighted by sqrt(2j_2+1)/sqrt(2j_0+1) (3 legs)."""
    B = _blocks(sb, xb)
    t = 0.0
    for b, blk in _blocks(sa, xa).items():
        a = sa.block_angm(b)
        w = np.sqrt(a[2] + 1) / np.sqrt(a[0] + 1) if len(sa.bonds) == 3 else 1.0
        t += float(np.sum(blk * B[b])) * w
    return t


def multiply_singular_value(s: Struct, x, leg: int, w):
    """Each multiplet of `leg` scaled by its weight (sector by sector)."""
    off = np.concatenate([[0], np.cumsum(s.bonds[leg].dim)])
    y = np.array(x, np.float64, copy=True)
    o, _ = s.offsets()
    for b, blk in _blocks(s, x).items():
        sec = (b // int(np.prod([len(q.angm) for q in s.bonds[:leg]], dtype=np.int64))) % len(s.bonds[leg].angm)
        shape = [1] * len(s.bonds)
        shape[leg] = blk.shape[leg]
        scaled = blk * np.asarray(w[off[sec]: off[sec] + blk.shape[leg]]).reshape(shape)
        y[o[b]: o[b] + blk.size] = scaled.ravel(order="F")
    return y


def mea_enr(hl, hr, ww, pairs):
    """[tr hl + tr(W hr W) + sum coef ss(L, R)] / sum ww^2, hl/hr = (Struct, x),
    pairs = [((Struct, x) | None, (Struct, x) | None, coef)]."""
    num = take_trace(*hl)
    s, x = hr
    y = multiply_singular_value(s, multiply_singular_value(s, x, 0, ww), 1, ww)
    num += take_trace(s, y)
    for l, r, c in pairs:
        if l is not None:
            num += c * ss_inner_prod(l[0], l[1], r[0], r[1])
    return num / float(np.sum(np.asarray(ww) ** 2))


# --------------------------------------------------------------------------
# the synthetic H_eff workload, built from the oracle alone
# --------------------------------------------------------------------------
def gaussian_sector_counts(total: int, max2j: int = 12, mean_j: float = 2.0, sd_j: float = 1.5):
    """Multiplet counts per 2j in 0..max2j from a discretised Gaussian in j,
    largest-remainder rounding to exactly `total`."""
    j = np.arange(max2j + 1) / 2.0
    w = np.exp(-0.5 * ((j - mean_j) / sd_j) ** 2)
    raw = w / w.sum() * total
    base = np.floor(raw).astype(int)
    order = np.argsort(-(raw - base), kind="stable")
    base[order[: total - base.sum()]] += 1
    return base.tolist()


def _symmetric_operator(st: Struct, rng, fac, ratio_side: bool) -> np.ndarray:
    """Operator blocks (ja, s, jc) drawn for ja <= jc (N(0,1)/sqrt(rows),
    diagonal blocks symmetrised); the mirror block (jc, s, ja) is the
    transpose, times fac[ja,s,jc]/fac[jc,s,ja] on the right-hand operator, so
    that the effective Hamiltonian is symmetric."""
    off, total = st.offsets()
    data = np.zeros(total)
    where = {st.block_angm(i): i for i in range(st.nten) if st.flag[i]}
    for (ja, s, jc), i in where.items():
        if ja > jc:
            continue
        a, _, c = st.block_shape(i)
        blk = rng.standard_normal((a, c)) / np.sqrt(a)
        if ja == jc:
            blk = 0.5 * (blk + blk.T)
        data[off[i]: off[i] + a * c] = blk.ravel(order="F")
        mirror = where.get((jc, s, ja))
        if ja != jc and mirror is not None:
            t = blk.T * (fac[ja, s, jc] / fac[jc, s, ja]) if ratio_side else blk.T
            data[off[mirror]: off[mirror] + a * c] = np.ascontiguousarray(t).ravel(order="F")
    return data


def synthetic_heff(D: int = 2000, nspin1: int = 18, seed: int = 1234, max2j: int = 12):
    """The seeded synthetic two-site H_eff of the D-multiplet benchmark shape
    (bond sectors 2j = 0..max2j with Gaussian counts, enlarged legs bond x
    spin-1/2, psi a normalised N(0,1) singlet, `nspin1` spin-1 operator pairs
    and the two spin-0 block Hamiltonians), drawn from numpy's PCG64 in the
    same order as the library's own generator, so both hold the same numbers.
    Built with the oracle's structures and recoupling table only.  Returns
    (HeffProblem, psi data)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    counts = gaussian_sector_counts(D, max2j)
    angm = [k for k in range(max2j + 1) if counts[k] > 0]
    bond = Bond(1, angm, [counts[k] for k in angm])
    enl = fuse(bond, Bond(1, [1], [1]))
    psi = Struct([enl, enl], 0).with_legal_flags()
    off, total = psi.offsets()
    x = np.zeros(total)
    for i in range(psi.nten):
        if psi.flag[i]:
            a, b = psi.block_shape(i)
            x[off[i]: off[i] + a * b] = rng.standard_normal(a * b)
    x /= np.linalg.norm(x)
    fac = fac_hamilt_vec(MAX_ANGM)
    spin = Bond(1, [2], [1])
    inb = enl.inverted()
    terms = []
    for _ in range(nspin1):
        s1 = Struct([inb, spin, enl], 0).with_legal_flags()
        s2 = Struct([inb, spin, enl], 0).with_legal_flags()
        x1 = _symmetric_operator(s1, rng, fac, ratio_side=False)
        x2 = _symmetric_operator(s2, rng, fac, ratio_side=True)
        terms.append((s1, x1, s2, x2, 1.0))
    hs = Struct([inb, enl], 0).with_legal_flags()
    hoff, htot = hs.offsets()
    hx = [np.zeros(htot), np.zeros(htot)]
    for side in range(2):
        for i in range(hs.nten):
            if hs.flag[i]:
                a, c = hs.block_shape(i)
                blk = rng.standard_normal((a, c)) / np.sqrt(a)
                hx[side][hoff[i]: hoff[i] + a * c] = (0.5 * (blk + blk.T)).ravel(order="F")
    return HeffProblem(psi, terms, (hs, hx[0], 1.0), (hs, hx[1], 1.0)), x


# --------------------------------------------------------------------------
# seeded random start vector
# --------------------------------------------------------------------------
def random_vector(state: int, n: int):
    """tensor_su2::random_initialize_tensor (tensor_su2.cpp:2375-2393) of an
    n-element packed vector followed by normalize_vector (tensor_su2.cpp:324-356)
    twice, the generator ran() of ran.f90:2-16 (fhelpers.c) continuing from
    `state`.  Returns (values, raw draws ran()*2-1, new state)."""
    L = lib()
    L.or_ran_state.restype = ctypes.c_int64
    L.or_set_ran_state.argtypes = [ctypes.c_int64]
    L.ran_.restype = ctypes.c_double
    L.or_set_ran_state(int(state))
    raw = np.array([L.ran_() * 2.0 - 1.0 for _ in range(n)])
    x = raw.copy()
    for _ in range(2):
        nor = 0.0
        for v in x:
            nor += v * v
        x = x / np.sqrt(nor)
    return x, raw, int(L.or_ran_state())
