"""Host-side mirror of the reference's SU(2) tensor interface for the hot path.

Names follow the reference so that callers read the same:
  Su2Bond    ~ su2bond   (su2bond.hpp:3-29)
  Su2Struct  ~ su2struct (su2struct.hpp:4-40) + the block presence flags
  HeffPlan   ~ dmrg_su2::hamiltonian_vector_multiplication_idmrg
               (dmrg_su2.cpp:543-664) with its term list fixed per two-site
               step; .lanczos() ~ lanczos_su2::lanczos1 (lanczos_su2.cpp:125-195)
  hamiltonian_vector_multiplication ~ tensor_su2::hamiltonian_vector_multiplication
               (tensor_su2_dmrg_src.cpp:893-1041)
All metadata work (legality, layout, fusion) is done by libsu2g.so's host
entry points; all arithmetic runs on the GPU through the C ABI.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field

import numpy as np

from . import capi
from .capi import check, lib, ptr, stream_handle


@dataclass
class Su2Bond:
    dir: int
    angm: list
    dim: list

    def inverted(self) -> "Su2Bond":
        return Su2Bond(-self.dir, list(self.angm), list(self.dim))

    def fuse(self, other: "Su2Bond") -> "Su2Bond":
        """su2bond::fuse: direction -self.dir, 2j capped at 38."""
        a1 = np.asarray(self.angm, np.int32)
        d1 = np.asarray(self.dim, np.int32)
        a2 = np.asarray(other.angm, np.int32)
        d2 = np.asarray(other.dim, np.int32)
        n = ctypes.c_int(0)
        ao = np.zeros(64, np.int32)
        do = np.zeros(64, np.int32)
        check(lib().su2g_bond_fuse(len(a1), ptr(a1), ptr(d1), len(a2), ptr(a2), ptr(d2), ctypes.addressof(n),
                                   ptr(ao), ptr(do)))
        return Su2Bond(-self.dir, ao[: n.value].tolist(), do[: n.value].tolist())


@dataclass
class Su2Struct:
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
        out = np.zeros(self.nten, np.int32)
        desc = self.desc()  # held: ptr() of a temporary could dangle during the call
        n = lib().su2g_struct_legal(ptr(desc), ptr(out))
        if n < 0:
            raise capi.Su2gError(capi.SU2G_EINVAL, "malformed structure")
        return out

    def with_legal_flags(self) -> "Su2Struct":
        self.flag = self.legal()
        return self

    def offsets(self):
        off = np.zeros(self.nten, np.int64)
        desc, flag = self.desc(), np.ascontiguousarray(self.flag, np.int32)
        total = lib().su2g_layout(ptr(desc), ptr(flag), ptr(off))
        if total < 0:
            raise capi.Su2gError(capi.SU2G_EINVAL, "malformed structure")
        return off, int(total)

    def size(self) -> int:
        return self.offsets()[1]

    def block_angm(self, idx: int):
        out = []
        for b in self.bonds:
            out.append(b.angm[idx % len(b.angm)])
            idx //= len(b.angm)
        return tuple(out)

    def block_shape(self, idx: int):
        out = []
        for b in self.bonds:
            out.append(b.dim[idx % len(b.angm)])
            idx //= len(b.angm)
        return tuple(out)

    def flag_array(self) -> np.ndarray:
        return np.ascontiguousarray(self.flag, np.int32)


def fac_hamilt_vec(max_angm: int = 25) -> np.ndarray:
    out = np.zeros(max_angm**3, np.float64)
    check(lib().su2g_fac_hamilt_vec(max_angm, ptr(out)))
    return out.reshape(max_angm, max_angm, max_angm)


def make_cgc(j1: int, j2: int, j3: int) -> np.ndarray:
    out = np.zeros((j1 + 1) * (j2 + 1) * (j3 + 1), np.float64)
    check(lib().su2g_make_cgc(j1, j2, j3, ptr(out)))
    return out


class _Pinned:
    """Keeps the host arrays a plan was built from alive (the library copies
    them, but the ctypes structures point at them during creation)."""

    def __init__(self, struct):
        self.desc = np.ascontiguousarray(struct.desc(), np.int32)
        self.flag = np.ascontiguousarray(struct.flag, np.int32)


def _tensor(struct: Su2Struct, data, keep: list) -> capi.Tensor:
    if getattr(data, "is_cuda", True) is False:  # a torch tensor in host memory
        raise ValueError("tensor data must be in device memory (numpy arrays for one-site operators)")
    p = _Pinned(struct)
    keep.append(p)
    return capi.Tensor(ptr(p.desc), ptr(p.flag), ptr(data))


class _PlanArgs:
    """Packs (psi, terms, hl, hr) into the C structures of su2g_heff_plan_*;
    the host arrays stay referenced while the call runs."""

    def __init__(self, psi, terms, hl, hr):
        self.keep = []
        self.tarr = (capi.Term * max(1, len(terms)))()
        for i, (s1, x1, s2, x2, c) in enumerate(terms):
            self.tarr[i] = capi.Term(_tensor(s1, x1, self.keep), _tensor(s2, x2, self.keep), float(c))
        self.h = []
        for h in (hl, hr):
            if h is None:
                self.h.append((None, 0.0))
            else:
                t = _tensor(h[0], h[1], self.keep)
                self.keep.append(t)
                self.h.append((ctypes.addressof(t), float(h[2])))
        self.pd = np.ascontiguousarray(psi.desc(), np.int32)
        self.pf = np.ascontiguousarray(psi.flag, np.int32)
        self.args = (ptr(self.pd), ptr(self.pf), len(terms), ctypes.addressof(self.tarr),
                     self.h[0][0], self.h[0][1], self.h[1][0], self.h[1][1])

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.keep.clear()


class HeffPlan:
    """Device work list of one effective Hamiltonian (see su2g_heff_plan_create).

    terms: list of (Su2Struct op1, device data1, Su2Struct op2, device data2, coef)
    hl, hr: (Su2Struct, device data, coef) or None.
    Device data are torch CUDA tensors (float64) or raw device addresses; they
    must outlive the plan (the plan holds references to torch tensors).
    """

    def __init__(self, psi: Su2Struct, terms, hl=None, hr=None, mode: int = capi.MODE_F64):
        self.psi = psi
        self._data_refs = [x for (_s1, x1, _s2, x2, _c) in terms for x in (x1, x2)]
        self._data_refs += [h[1] for h in (hl, hr) if h is not None]
        handle = ctypes.c_void_p()
        with _PlanArgs(psi, terms, hl, hr) as a:
            check(lib().su2g_heff_plan_create(*a.args, int(mode), ctypes.addressof(handle)))
        self._h = handle
        self.mode = mode

    @staticmethod
    def validate(psi: Su2Struct, terms, hl=None, hr=None, mode: int = capi.MODE_F64) -> dict:
        """Host-only dry run: builds the work lists of `mode` and bounds-checks
        every access (su2g_heff_plan_validate).  Data may be host arrays."""
        fl = ctypes.c_double()
        sb = ctypes.c_int64()
        with _PlanArgs(psi, terms, hl, hr) as a:
            check(lib().su2g_heff_plan_validate(*a.args, int(mode), ctypes.addressof(fl), ctypes.addressof(sb)))
        return {"flops": fl.value, "scratch_bytes": sb.value}

    @staticmethod
    def digest(psi: Su2Struct, terms, hl=None, hr=None, mode: int = capi.MODE_F64) -> int:
        """Host-only digest of every field of the work lists of `mode`
        (su2g_heff_plan_digest); operand addresses enter it."""
        dg = ctypes.c_uint64()
        with _PlanArgs(psi, terms, hl, hr) as a:
            check(lib().su2g_heff_plan_digest(*a.args, int(mode), ctypes.addressof(dg)))
        return dg.value

    def status(self) -> int:
        """Device error word (0 = no bounded wait gave up); raises on time-out."""
        code = ctypes.c_int()
        check(lib().su2g_heff_plan_status(self._h, ctypes.addressof(code)))
        return code.value

    @property
    def handle(self):
        return self._h

    def info(self) -> dict:
        fl = ctypes.c_double()
        n = ctypes.c_int64()
        sb = ctypes.c_int64()
        nt = ctypes.c_int()
        check(lib().su2g_heff_plan_info(self._h, ctypes.addressof(fl), ctypes.addressof(n), ctypes.addressof(sb),
                                        ctypes.addressof(nt)))
        return {"flops": fl.value, "psi_len": n.value, "scratch_bytes": sb.value, "ntiles": nt.value}

    def launches(self) -> int:
        """Kernels of this library one apply() launches."""
        n = ctypes.c_int()
        check(lib().su2g_heff_plan_launches(self._h, ctypes.addressof(n)))
        return n.value

    def apply(self, psi, y, stream=None) -> None:
        check(lib().su2g_heff_apply(self._h, ptr(psi), ptr(y), stream_handle(stream)))

    def apply_profile(self, psi, y, stream=None) -> list:
        """One application with per-launch device times in ms (see
        su2g_heff_apply_profile)."""
        ms = (ctypes.c_double * 8)()
        n = ctypes.c_int()
        check(lib().su2g_heff_apply_profile(self._h, ptr(psi), ptr(y), stream_handle(stream), ctypes.addressof(ms),
                                            ctypes.addressof(n)))
        return [ms[i] for i in range(n.value)]

    def add_projector(self, o, weight: float) -> None:
        """Excited-state penalty y -= weight (o . psi) o on every later
        application (o: device vector in psi's layout, kept alive here)."""
        self._data_refs.append(o)
        check(lib().su2g_heff_plan_add_projector(self._h, ptr(o), float(weight)))

    def lanczos(self, psi, mlanc: int = 5, stream=None):
        e = ctypes.c_double()
        nmv = ctypes.c_int()
        check(lib().su2g_lanczos(self._h, ptr(psi), int(mlanc), ctypes.addressof(e), ctypes.addressof(nmv),
                                 stream_handle(stream)))
        return e.value, nmv.value

    def close(self) -> None:
        if self._h:
            lib().su2g_heff_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class HeffBatch:
    """Several HeffPlans (one precision mode) applied in shared launches
    (su2g_heff_batch_*): plan i's vector lies at offsets()[i] of the batch
    vectors.  The plans must outlive the batch."""

    def __init__(self, plans):
        self.plans = list(plans)
        arr = (ctypes.c_void_p * len(self.plans))(*[p.handle.value for p in self.plans])
        h = ctypes.c_void_p()
        check(lib().su2g_heff_batch_create(ctypes.addressof(arr), len(self.plans), ctypes.addressof(h)))
        self._h = h
        tot = ctypes.c_int64()
        check(lib().su2g_heff_batch_info(self._h, ctypes.addressof(tot), None))
        self.total = tot.value
        lens = [p.info()["psi_len"] for p in self.plans]
        self._off = [int(x) for x in np.concatenate([[0], np.cumsum(lens)[:-1]])]

    def offsets(self):
        return list(self._off)

    def apply(self, x, y, stream=None) -> None:
        """y = H x for every plan on its slice of the batch vectors."""
        check(lib().su2g_heff_batch_apply(self._h, ptr(x), ptr(y), stream_handle(stream)))

    def status(self) -> None:
        check(lib().su2g_heff_batch_status(self._h))

    def lanczos(self, psis, mlanc: int = 5, stream=None):
        """Lockstep Lanczos of every plan (psis[i]: plan i's start vector,
        overwritten with its eigenvector); returns [(energy, nmatvec)]."""
        n = len(self.plans)
        arr = (ctypes.c_void_p * n)(*[ptr(v) for v in psis])
        e = (ctypes.c_double * n)()
        nm = (ctypes.c_int * n)()
        check(lib().su2g_heff_batch_lanczos(self._h, ctypes.addressof(arr), int(mlanc), ctypes.addressof(e),
                                            ctypes.addressof(nm), stream_handle(stream)))
        return [(e[i], nm[i]) for i in range(n)]

    def close(self) -> None:
        if self._h:
            lib().su2g_heff_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def hamiltonian_vector_multiplication(vec: Su2Struct, vec_data, op1: Su2Struct, x1, op2: Su2Struct, x2, y,
                                      stream=None) -> None:
    keep = []
    t1 = _tensor(op1, x1, keep)
    t2 = _tensor(op2, x2, keep)
    vd = np.ascontiguousarray(vec.desc(), np.int32)
    vf = np.ascontiguousarray(vec.flag, np.int32)
    check(lib().su2g_hamiltonian_vector_multiplication(ptr(vd), ptr(vf), ptr(vec_data), t1, t2, ptr(y),
                                                       stream_handle(stream)))


def _parse_desc(d):
    d = d.tolist() if isinstance(d, np.ndarray) else [int(v) for v in d]
    nb, loc, p = d[0], d[1], 2
    bonds = []
    for _ in range(nb):
        dr, n = d[p], d[p + 1]
        bonds.append(Su2Bond(dr, d[p + 2: p + 2 + n], d[p + 2 + n: p + 2 + 2 * n]))
        p += 2 + 2 * n
    return Su2Struct(bonds, loc)


def _env_layout(kind: int, uu, xu, vv, xv, op, xo, flag: int) -> Su2Struct:
    keep = []
    fn = lib().su2g_operator_transformation_layout if kind else lib().su2g_overlap_transformation_layout
    desc = np.zeros(4 + 3 * (2 + 2 * 64), np.int32)
    flags = np.zeros(64 ** 3, np.int32)
    n = ctypes.c_int64()
    check(fn(_tensor(uu, xu, keep), _tensor(vv, xv, keep), int(flag), _tensor(op, xo, keep), ptr(desc), len(desc),
             ptr(flags), len(flags), ctypes.addressof(n)))
    out = _parse_desc(desc)
    out.flag = flags[: out.nten].copy()
    return out


def operator_transformation_layout(uu, xu, vv, xv, op, xo, flag: int) -> Su2Struct:
    """Output structure of tensor_su2::operator_transformation (host only)."""
    return _env_layout(1, uu, xu, vv, xv, op, xo, flag)


def overlap_transformation_layout(uu, xu, vv, xv, hh, xh, flag: int) -> Su2Struct:
    """Output structure of tensor_su2::overlap_transformation (host only)."""
    return _env_layout(0, uu, xu, vv, xv, hh, xh, flag)


def _env_run(kind, uu, xu, vv, xv, ops, outs, flag, mode, stream):
    keep = []
    arr = (capi.Tensor * max(1, len(ops)))()
    for i, (s, x) in enumerate(ops):
        arr[i] = _tensor(s, x, keep)
    optr = (ctypes.c_void_p * max(1, len(outs)))(*[ptr(o) for o in outs])
    fn = lib().su2g_operator_transformation if kind else lib().su2g_overlap_transformation
    check(fn(_tensor(uu, xu, keep), _tensor(vv, xv, keep), int(flag), len(ops), ctypes.addressof(arr),
             ctypes.addressof(optr), int(mode), stream_handle(stream)))


def operator_transformation(uu, xu, vv, xv, ops, outs, flag: int, mode: int = capi.MODE_F64, stream=None) -> None:
    """Batch of tensor_su2::operator_transformation: ops = [(Su2Struct, device data)],
    outs = device buffers laid out by operator_transformation_layout."""
    _env_run(1, uu, xu, vv, xv, ops, outs, flag, mode, stream)


def overlap_transformation(uu, xu, vv, xv, hhs, outs, flag: int, mode: int = capi.MODE_F64, stream=None) -> None:
    """Batch of tensor_su2::overlap_transformation (2-leg scalar operators)."""
    _env_run(0, uu, xu, vv, xv, hhs, outs, flag, mode, stream)


def svd(vec: Su2Struct, vec_data, tu: Su2Struct, p1: float, tv: Su2Struct, p2: float, max_dcut: int, stream=None):
    """vec.svd(tu, p1, tv, p2, dout, wout) (tensor_su2.cpp:1619-1758) on the GPU.

    vec: the two-leg wave function (device data); tu, tv: the current MPS
    tensors' structures (legs 0, 1 are used).  Returns (tu_struct, tu_data,
    tv_struct, tv_data, wout): the new MPS tensors as device arrays (every
    legal block present) and the singular values, kept then discarded, as the
    reference writes them."""
    import torch

    vd = np.ascontiguousarray(vec.desc(), np.int32)
    vf = np.ascontiguousarray(vec.flag, np.int32)
    ud = np.ascontiguousarray(tu.desc(), np.int32)
    wd = np.ascontiguousarray(tv.desc(), np.int32)
    # capacity: every common sector keeps at most min(its two sizes, max_dcut) multiplets
    b0, b1 = vec.bonds
    ucap = vcap = nval = 0
    for a, m in zip(b0.angm, b0.dim):
        if a in b1.angm:
            n = b1.dim[b1.angm.index(a)]
            k = min(m, n, max_dcut)
            ucap += m * k
            vcap += n * k
            nval += min(m, n)
    bond = np.zeros(1 + 2 * len(b0.angm), np.int32)
    wout = np.zeros(max(1, nval))
    dout = ctypes.c_int(0)
    dev = vec_data.device if hasattr(vec_data, "device") else torch.device("cuda")
    xu = torch.empty(max(1, ucap), dtype=torch.float64, device=dev)
    xv = torch.empty(max(1, vcap), dtype=torch.float64, device=dev)
    check(lib().su2g_svd(ptr(vd), ptr(vf), ptr(vec_data), ptr(ud), float(p1), ptr(wd), float(p2), int(max_dcut),
                         ptr(bond), len(bond), ptr(wout), len(wout), ctypes.addressof(dout), ptr(xu), ucap, ptr(xv),
                         vcap, stream_handle(stream)))
    nb = int(bond[0])
    newb = Su2Bond(-1, bond[1: 1 + nb].tolist(), bond[1 + nb: 1 + 2 * nb].tolist())
    out = []
    for s, x in ((tu, xu), (tv, xv)):
        st = Su2Struct([s.bonds[0], s.bonds[1], newb], 0).with_legal_flags()
        out += [st, x[: st.size()]]
    return out[0], out[1], out[2], out[3], wout[: dout.value].copy()


_ENV_KINDS = {"overlap": capi.ENV_OVERLAP, "transform": capi.ENV_TRANSFORM, "init": capi.ENV_INITIAL,
              "pair": capi.ENV_PAIRUP, "perm": capi.ENV_PERMUTATION}


class _EnvJobs:
    """ctypes job array; keeps every desc/flag/data array alive for the call."""

    def __init__(self, jobs):
        self.keep = []
        self.arr = (capi.EnvJob * max(1, len(jobs)))()
        for i, jb in enumerate(jobs):
            kind, slot, coef = jb["kind"], jb.get("slot", 0), jb.get("coef", 1.0)
            e = self.arr[i]
            e.kind = _ENV_KINDS[kind] if isinstance(kind, str) else int(kind)
            e.slot = int(slot)
            e.coef = float(coef)
            if jb.get("x") is not None:
                e.x = _tensor(jb["x"][0], jb["x"][1], self.keep)
            for name in ("site1", "site2"):
                if jb.get(name) is not None:
                    s, d = jb[name]
                    d = np.ascontiguousarray(d, np.float64)  # site operators travel as host data
                    self.keep.append(d)
                    setattr(e, name, _tensor(s, d, self.keep))
        self.n = len(jobs)

    @property
    def ptr(self):
        return ctypes.addressof(self.arr)


def env_layout(uu, xu, vv, xv, flag: int, jobs, slot: int = 0) -> Su2Struct:
    """Structure of output slot `slot` of an env batch (host only)."""
    return env_layouts(uu, xu, vv, xv, flag, jobs, [slot])[0]


def env_layouts(uu, xu, vv, xv, flag: int, jobs, slots) -> list:
    """Structures of the output slots `slots` of an env batch (host only): the
    job array and the output buffers are built once for all of them."""
    keep = []
    J = _EnvJobs(jobs)
    tu, tv = _tensor(uu, xu, keep), _tensor(vv, xv, keep)
    desc = np.zeros(4 + 3 * (2 + 2 * 64), np.int32)
    flags = np.zeros(64 ** 3, np.int32)
    n = ctypes.c_int64()
    res = []
    for slot in slots:
        check(lib().su2g_env_layout(tu, tv, int(flag), J.n, J.ptr, int(slot), ptr(desc), len(desc), ptr(flags),
                                    len(flags), ctypes.addressof(n)))
        out = _parse_desc(desc)
        out.flag = flags[: out.nten].copy()
        res.append(out)
    return res


def env_run(uu, xu, vv, xv, flag: int, jobs, outs, mode: int = capi.MODE_F64, stream=None) -> None:
    """Runs an env batch: jobs = [{"kind": "overlap"|"transform"|"init"|"pair"|"perm",
    "slot": s, "coef": c, "x": (Su2Struct, device data) or None,
    "site1"/"site2": (Su2Struct, host data)}], outs[s] = device buffers laid out
    by env_layout(..., slot=s)."""
    keep = []
    J = _EnvJobs(jobs)
    optr = (ctypes.c_void_p * max(1, len(outs)))(*[ptr(o) for o in outs])
    check(lib().su2g_env_run(_tensor(uu, xu, keep), _tensor(vv, xv, keep), int(flag), J.n, J.ptr, len(outs),
                             ctypes.addressof(optr), int(mode), stream_handle(stream)))


def env_validate(uu, xu, vv, xv, flag: int, jobs, mode: int = capi.MODE_F64) -> dict:
    """Host-only dry run of env_run: {"flops": ..., "scratch_bytes": ...}."""
    keep = []
    J = _EnvJobs(jobs)
    nslots = 1 + max(int(j.get("slot", 0)) for j in jobs)
    flops = ctypes.c_double()
    scratch = ctypes.c_int64()
    check(lib().su2g_env_validate(_tensor(uu, xu, keep), _tensor(vv, xv, keep), int(flag), J.n, J.ptr, nslots,
                                  int(mode), ctypes.addressof(flops), ctypes.addressof(scratch)))
    return {"flops": flops.value, "scratch_bytes": scratch.value}


def env_digest(uu, xu, vv, xv, flag: int, jobs, outs, mode: int = capi.MODE_F64) -> int:
    """Host-only digest of the work lists of an env batch (su2g_env_digest);
    operand and output addresses enter it."""
    keep = []
    J = _EnvJobs(jobs)
    optr = (ctypes.c_void_p * max(1, len(outs)))(*[ptr(o) for o in outs])
    dg = ctypes.c_uint64()
    check(lib().su2g_env_digest(_tensor(uu, xu, keep), _tensor(vv, xv, keep), int(flag), J.n, J.ptr, len(outs),
                                ctypes.addressof(optr), int(mode), ctypes.addressof(dg)))
    return dg.value


def env_batch(uu, xu, vv, xv, flag: int, jobs, mode: int = capi.MODE_F64, stream=None):
    """env_layout + allocation + env_run: returns [(Su2Struct, device tensor)] per slot."""
    import torch

    nslots = 1 + max(int(j.get("slot", 0)) for j in jobs)
    dev = xu.device if hasattr(xu, "device") else torch.device("cuda")
    res = [(st, torch.empty(max(1, st.size()), dtype=torch.float64, device=dev))
           for st in env_layouts(uu, xu, vv, xv, flag, jobs, range(nslots))]
    env_run(uu, xu, vv, xv, flag, jobs, [r[1] for r in res], mode, stream)
    return res


def operator_initial(uu, xu, vv, xv, op, op_host, flag: int, endt=None, mode: int = capi.MODE_F64, stream=None):
    """tensor_su2::operator_initial(uu, vv, op[, endt], flag); op data on the host,
    endt = (Su2Struct, device data) or None.  Returns (Su2Struct, device tensor)."""
    return env_batch(uu, xu, vv, xv, flag, [{"kind": "init", "x": endt, "site1": (op, op_host)}], mode, stream)[0]


def operator_pairup(uu, xu, vv, xv, op1, x1, op2, op2_host, flag: int, mode: int = capi.MODE_F64, stream=None):
    """tensor_su2::operator_pairup(uu, vv, op1, op2, flag); op2 data on the host."""
    return env_batch(uu, xu, vv, xv, flag, [{"kind": "pair", "x": (op1, x1), "site1": (op2, op2_host)}], mode,
                     stream)[0]


def permutation(uu, xu, vv, xv, vec, xvec, op1, op1_host, op2, op2_host, flag: int, mode: int = capi.MODE_F64,
                stream=None):
    """tensor_su2::permutation(uu, vv, vec, op1, op2, flag); op1, op2 data on the host."""
    return env_batch(uu, xu, vv, xv, flag, [{"kind": "perm", "x": (vec, xvec), "site1": (op1, op1_host),
                                             "site2": (op2, op2_host)}], mode, stream)[0]


def operator_combine(ops, coefs, stream=None):
    """sum_i coefs[i] * ops[i] for ops = [(Su2Struct, device data)] of one
    structure: returns (Su2Struct with the union of blocks, device tensor)."""
    import torch

    keep = []
    arr = (capi.Tensor * len(ops))()
    for i, (s, x) in enumerate(ops):
        arr[i] = _tensor(s, x, keep)
    first = ops[0][0]
    flags = np.zeros(first.nten, np.int32)
    n = ctypes.c_int64()
    check(lib().su2g_operator_combine_layout(len(ops), ctypes.addressof(arr), ptr(flags), len(flags),
                                             ctypes.addressof(n)))
    out = Su2Struct(list(first.bonds), first.locspin)
    out.flag = flags
    c = np.ascontiguousarray(coefs, np.float64)
    dev = ops[0][1].device if hasattr(ops[0][1], "device") else torch.device("cuda")
    y = torch.empty(max(1, n.value), dtype=torch.float64, device=dev)
    check(lib().su2g_operator_combine(len(ops), ctypes.addressof(arr), ptr(c), ptr(y), stream_handle(stream)))
    return out, y


def _layout_out(fn, *args) -> Su2Struct:
    """Calls a *_layout entry point and returns its structure."""
    desc = np.zeros(4 + 3 * (2 + 2 * 64), np.int32)
    flags = np.zeros(64 ** 3, np.int32)
    n = ctypes.c_int64()
    check(fn(*args, ptr(desc), len(desc), ptr(flags), len(flags), ctypes.addressof(n)))
    out = _parse_desc(desc)
    out.flag = flags[: out.nten].copy()
    return out


def vectran_layout(u: Su2Struct, flag: int) -> Su2Struct:
    """Structure after right2left_vectran (flag 0) / left2right_vectran (1)."""
    keep = []
    return _layout_out(lib().su2g_vectran_layout, _tensor(u, None, keep), int(flag))


def vectran(u: Su2Struct, xu, flag: int, out=None, stream=None):
    """wavefunc_transformation of one MPS tensor (device data xu): returns
    (rotated Su2Struct, device tensor); out=xu rotates in place."""
    import torch

    keep = []
    s = vectran_layout(u, flag)
    y = out if out is not None else torch.empty(max(1, s.size()), dtype=torch.float64, device=xu.device)
    check(lib().su2g_vectran(_tensor(u, xu, keep), int(flag), ptr(y), stream_handle(stream)))
    return s, y


def input_vector_layout(ul: Su2Struct, ur: Su2Struct) -> Su2Struct:
    """Structure of prepare_input_vector's two-site vector."""
    keep = []
    return _layout_out(lib().su2g_input_vector_layout, _tensor(ul, None, keep), _tensor(ur, None, keep))


def prepare_input_vector(ul: Su2Struct, xl, ur: Su2Struct, xr, mode: int = capi.MODE_F64, stream=None):
    """dmrg_su2::prepare_input_vector from uu[il] = (ul, xl) and uu[ir] =
    (ur, xr) (device data): returns (Su2Struct, device tensor)."""
    import torch

    keep = []
    s = input_vector_layout(ul, ur)
    y = torch.empty(max(1, s.size()), dtype=torch.float64, device=xl.device)
    check(lib().su2g_prepare_input_vector(_tensor(ul, xl, keep), _tensor(ur, xr, keep), ptr(y), int(mode),
                                          stream_handle(stream)))
    return s, y



def fuse_tensor(b1: Su2Bond, b2: Su2Bond, device="cuda", stream=None):
    """tensor_su2::fuse(b1, b2): returns (Su2Struct, device tensor)."""
    import torch

    bd = Su2Struct([b1, b2], 0).desc()
    s = _layout_out(lib().su2g_fuse_tensor_layout, ptr(bd))
    y = torch.empty(max(1, s.size()), dtype=torch.float64, device=device)
    check(lib().su2g_fuse_tensor(ptr(bd), ptr(y), stream_handle(stream)))
    return s, y


def fuse_tensor_layout(b1: Su2Bond, b2: Su2Bond) -> Su2Struct:
    bd = Su2Struct([b1, b2], 0).desc()
    return _layout_out(lib().su2g_fuse_tensor_layout, ptr(bd))


def random_vector(x, state: int, stream=None) -> int:
    """Fills the device vector x with the seeded random start vector
    (su2g_random_vector); returns the generator's state after it."""
    st = ctypes.c_int64(int(state))
    check(lib().su2g_random_vector(ctypes.addressof(st), ptr(x), int(x.numel()), stream_handle(stream)))
    return st.value


def initial_vector(ul: Su2Struct, xl, ur: Su2Struct, xr, stream=None):
    """The warm-up's start vector on prepare_input_vector's structure."""
    import torch

    keep = []
    s = input_vector_layout(ul, ur)
    y = torch.empty(max(1, s.size()), dtype=torch.float64, device=xl.device)
    check(lib().su2g_initial_vector(_tensor(ul, xl, keep), _tensor(ur, xr, keep), ptr(y), stream_handle(stream)))
    return s, y


# ---------------------------------------------------------------- measurement
def _opt_tensor(t, keep):
    """(Su2Struct, data) or None (an operator never built) as a C tensor."""
    if t is None:
        return capi.Tensor(None, None, None)
    return _tensor(t[0], t[1], keep)


def take_trace(s: Su2Struct, x, stream=None) -> float:
    keep = []
    out = ctypes.c_double()
    check(lib().su2g_take_trace(_tensor(s, x, keep), ctypes.addressof(out), stream_handle(stream)))
    return out.value


def ss_inner_prod(a, b, stream=None) -> float:
    """a, b = (Su2Struct, device data) or None."""
    keep = []
    out = ctypes.c_double()
    check(lib().su2g_ss_inner_prod(_opt_tensor(a, keep), _opt_tensor(b, keep), ctypes.addressof(out),
                                   stream_handle(stream)))
    return out.value


def multiply_singular_value(s: Su2Struct, x, leg: int, w, stream=None) -> None:
    """In place on the device data x."""
    d = np.ascontiguousarray(s.desc(), np.int32)
    f = np.ascontiguousarray(s.flag, np.int32)
    wa = np.ascontiguousarray(w, np.float64)
    check(lib().su2g_multiply_singular_value(ptr(d), ptr(f), ptr(x), int(leg), ptr(wa), wa.size,
                                             stream_handle(stream)))


def mea_enr(hl, hr, ww, pairs, stream=None):
    """dmrg_su2::mea_enr: hl, hr = (Su2Struct, device data); pairs =
    [(left, right, coef)] with left/right (Su2Struct, device data) or None.
    Returns (energy, [tr hl, tr W hr W, pair sum, sum ww^2])."""
    keep = []
    n = len(pairs)
    L = (capi.Tensor * max(1, n))()
    R = (capi.Tensor * max(1, n))()
    c = np.zeros(max(1, n))
    for k, (l, r, cf) in enumerate(pairs):
        L[k] = _opt_tensor(l, keep)
        R[k] = _opt_tensor(r, keep)
        c[k] = cf
    wa = np.ascontiguousarray(ww, np.float64)
    e = ctypes.c_double()
    parts = np.zeros(4)
    check(lib().su2g_mea_enr(_tensor(hl[0], hl[1], keep), _tensor(hr[0], hr[1], keep), ptr(wa), wa.size, n,
                             ctypes.addressof(L), ctypes.addressof(R), ptr(c), ctypes.addressof(e), ptr(parts),
                             stream_handle(stream)))
    return e.value, parts


# ---------------------------------------------------------------- checkpoints
CKPT_MPS_DAT, CKPT_MPS_BIN, CKPT_ENR, CKPT_WW = 0, 1, 2, 3


def checkpoint_name(kind: int, ns: int, dcut: int, totspin: int = 0, ky: int = 0, exc: int = 0, pos: int = 0) -> str:
    """A checkpoint file name as the engine builds it (kind CKPT_*)."""
    buf = ctypes.create_string_buffer(256)
    check(lib().su2g_checkpoint_name(int(kind), int(ns), int(dcut), int(totspin), int(ky), int(exc), int(pos),
                                     buf, len(buf)))
    return buf.value.decode()


def _path(p) -> bytes:
    return os.fsencode(p)


def mps_save(dat_path, bin_path, s: Su2Struct, data, stream=None) -> None:
    """One site's MPS tensor (device data) to its .dat / .bin files."""
    keep = []
    check(lib().su2g_mps_save(_path(dat_path), _path(bin_path), _tensor(s, data, keep), stream_handle(stream)))


def mps_load_layout(dat_path, bin_path) -> Su2Struct:
    return _layout_out(lib().su2g_mps_load_layout, _path(dat_path), _path(bin_path))


def mps_load(dat_path, bin_path, device="cuda", stream=None):
    """read_mps for one site: returns (Su2Struct, device tensor)."""
    import torch

    s = mps_load_layout(dat_path, bin_path)
    y = torch.empty(max(1, s.size()), dtype=torch.float64, device=device)
    check(lib().su2g_mps_load(_path(dat_path), _path(bin_path), ptr(y), y.numel(), stream_handle(stream)))
    return s, y


def enr_append(path, value: float) -> None:
    check(lib().su2g_enr_append(_path(path), float(value)))


def enr_read(path) -> np.ndarray:
    """Every value of an energy file, in order."""
    n = ctypes.c_int()
    out = np.zeros(4096)
    rc = lib().su2g_enr_read(_path(path), ptr(out), len(out), ctypes.addressof(n))
    if rc == capi.SU2G_EINVAL and n.value > len(out):
        out = np.zeros(n.value)
        rc = lib().su2g_enr_read(_path(path), ptr(out), len(out), ctypes.addressof(n))
    check(rc)
    return out[: n.value].copy()


def ww_save(path, ww) -> None:
    a = np.ascontiguousarray(ww, np.float64)
    check(lib().su2g_ww_save(_path(path), ptr(a), a.size))


def ww_load(path, n: int) -> np.ndarray:
    out = np.zeros(max(1, n))
    got = ctypes.c_int64()
    check(lib().su2g_ww_load(_path(path), ptr(out), int(n), ctypes.addressof(got)))
    return out[: got.value].copy()
