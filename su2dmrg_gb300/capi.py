"""ctypes binding of libsu2g.so (include/su2g.h).

The library is the product; this module only loads it and forwards calls.
There is no CPU fallback: if libsu2g.so is missing, or a GPU entry point runs
without a CUDA device, the call raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libsu2g.so")

SU2G_OK = 0
SU2G_EINVAL = 1
SU2G_ENOMEM = 2
SU2G_ECUDA = 3
SU2G_ETIMEOUT = 4
SU2G_EUNSUPPORTED = 5
SU2G_EIO = 6

MODE_F64 = 0
MODE_SPLIT_BF16 = 1
MODE_SPLIT_BF16_FAST = 2


class Su2gError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"su2g error {code}: {msg}")
        self.code = code


class Tensor(ctypes.Structure):
    _fields_ = [("desc", ctypes.c_void_p), ("flag", ctypes.c_void_p), ("data", ctypes.c_void_p)]


class Term(ctypes.Structure):
    _fields_ = [("op1", Tensor), ("op2", Tensor), ("coef", ctypes.c_double)]


class EnvJob(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("slot", ctypes.c_int), ("coef", ctypes.c_double), ("x", Tensor),
                ("site1", Tensor), ("site2", Tensor)]


ENV_OVERLAP = 0
ENV_TRANSFORM = 1
ENV_INITIAL = 2
ENV_PAIRUP = 3
ENV_PERMUTATION = 4

_lib = None

_vp = ctypes.c_void_p
_i = ctypes.c_int
_i64 = ctypes.c_int64
_d = ctypes.c_double

_PROTOS = {
    "su2g_version": (_i, []),
    "su2g_last_error": (ctypes.c_char_p, []),
    "su2g_struct_nten": (_i, [_vp]),
    "su2g_struct_legal": (_i, [_vp, _vp]),
    "su2g_layout": (_i64, [_vp, _vp, _vp]),
    "su2g_bond_fuse": (_i, [_i, _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp]),
    "su2g_make_cgc": (_i, [_i, _i, _i, _vp]),
    "su2g_fac_hamilt_vec": (_i, [_i, _vp]),
    "su2g_fac_operator_transformation": (_i, [_i, _i, _i, _i, _i, _i, _i, _vp]),
    "su2g_heff_plan_create": (_i, [_vp, _vp, _i, _vp, _vp, _d, _vp, _d, _i, _vp]),
    "su2g_heff_plan_validate": (_i, [_vp, _vp, _i, _vp, _vp, _d, _vp, _d, _i, _vp, _vp]),
    "su2g_heff_plan_digest": (_i, [_vp, _vp, _i, _vp, _vp, _d, _vp, _d, _i, _vp]),
    "su2g_heff_plan_status": (_i, [_vp, _vp]),
    "su2g_heff_plan_mark_failed": (_i, [_vp, _i]),
    "su2g_f64_tile_table": (_i, [_vp, _i, _vp, _i, _vp]),
    "su2g_f64_tile_bench": (_i, [_i, _i, _i, _i, _i, _i, _vp, _vp]),
    "su2g_heff_batch_create": (_i, [_vp, _i, _vp]),
    "su2g_heff_batch_destroy": (_i, [_vp]),
    "su2g_heff_batch_info": (_i, [_vp, _vp, _vp]),
    "su2g_heff_batch_apply": (_i, [_vp, _vp, _vp, _vp]),
    "su2g_heff_batch_status": (_i, [_vp]),
    "su2g_heff_batch_lanczos": (_i, [_vp, _vp, _i, _vp, _vp, _vp]),
    "su2g_selftest_bounded_wait": (_i, [ctypes.c_longlong, _vp]),
    "su2g_heff_plan_info": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "su2g_heff_apply": (_i, [_vp, _vp, _vp, _vp]),
    "su2g_heff_plan_launches": (_i, [_vp, _vp]),
    "su2g_heff_apply_profile": (_i, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "su2g_heff_plan_destroy": (_i, [_vp]),
    "su2g_heff_plan_add_projector": (_i, [_vp, _vp, _d]),
    "su2g_operator_combine_layout": (_i, [_i, _vp, _vp, _i, _vp]),
    "su2g_operator_combine": (_i, [_i, _vp, _vp, _vp, _vp]),
    "su2g_hamiltonian_vector_multiplication": (_i, [_vp, _vp, _vp, Tensor, Tensor, _vp, _vp]),
    "su2g_hamiltonian_vector_multiplication_noalloc": (_i, [_vp, _vp, _vp, Tensor, Tensor, _vp, _vp]),
    "su2g_lanczos": (_i, [_vp, _vp, _i, _vp, _vp, _vp]),
    "su2g_operator_transformation_layout": (_i, [Tensor, Tensor, _i, Tensor, _vp, _i, _vp, _i, _vp]),
    "su2g_operator_transformation": (_i, [Tensor, Tensor, _i, _i, _vp, _vp, _i, _vp]),
    "su2g_overlap_transformation_layout": (_i, [Tensor, Tensor, _i, Tensor, _vp, _i, _vp, _i, _vp]),
    "su2g_overlap_transformation": (_i, [Tensor, Tensor, _i, _i, _vp, _vp, _i, _vp]),
    "su2g_env_layout": (_i, [Tensor, Tensor, _i, _i, _vp, _i, _vp, _i, _vp, _i, _vp]),
    "su2g_env_run": (_i, [Tensor, Tensor, _i, _i, _vp, _i, _vp, _i, _vp]),
    "su2g_env_validate": (_i, [Tensor, Tensor, _i, _i, _vp, _i, _i, _vp, _vp]),
    "su2g_env_digest": (_i, [Tensor, Tensor, _i, _i, _vp, _i, _vp, _i, _vp]),
    "su2g_fac_table": (_i, [_i, _i, _i, _i, _i, _i, _i, _vp]),
    "su2g_svd": (_i, [_vp, _vp, _vp, _vp, _d, _vp, _d, _i, _vp, _i, _vp, _i, _vp, _vp, _i64, _vp, _i64, _vp]),
    "su2g_vectran_layout": (_i, [Tensor, _i, _vp, _i, _vp, _i, _vp]),
    "su2g_vectran": (_i, [Tensor, _i, _vp, _vp]),
    "su2g_input_vector_layout": (_i, [Tensor, Tensor, _vp, _i, _vp, _i, _vp]),
    "su2g_fuse_tensor_layout": (_i, [_vp, _vp, _i, _vp, _i, _vp]),
    "su2g_fuse_tensor": (_i, [_vp, _vp, _vp]),
    "su2g_initial_vector": (_i, [Tensor, Tensor, _vp, _vp]),
    "su2g_random_vector": (_i, [_vp, _vp, ctypes.c_int64, _vp]),
    "su2g_prepare_input_vector": (_i, [Tensor, Tensor, _vp, _i, _vp]),
    "su2g_take_trace": (_i, [Tensor, _vp, _vp]),
    "su2g_ss_inner_prod": (_i, [Tensor, Tensor, _vp, _vp]),
    "su2g_multiply_singular_value": (_i, [_vp, _vp, _vp, _i, _vp, _i64, _vp]),
    "su2g_mea_enr": (_i, [Tensor, Tensor, _vp, _i64, _i, _vp, _vp, _vp, _vp, _vp, _vp]),
    "su2g_checkpoint_name": (_i, [_i, _i, _i, _i, _i, _i, _i, _vp, _i]),
    "su2g_mps_save": (_i, [_vp, _vp, Tensor, _vp]),
    "su2g_mps_load_layout": (_i, [_vp, _vp, _vp, _i, _vp, _i, _vp]),
    "su2g_mps_load": (_i, [_vp, _vp, _vp, _i64, _vp]),
    "su2g_enr_append": (_i, [_vp, _d]),
    "su2g_enr_read": (_i, [_vp, _vp, _i, _vp]),
    "su2g_ww_save": (_i, [_vp, _vp, _i64]),
    "su2g_ww_load": (_i, [_vp, _vp, _i64, _vp]),
    "su2g_vec_dot": (_i, [_vp, _vp, _i64, _vp, _vp]),
    "su2g_vec_axpy": (_i, [_d, _vp, _vp, _i64, _vp]),
    "su2g_vec_scale": (_i, [_d, _vp, _i64, _vp]),
}

# every symbol include/su2g.h declares (checked by the CPU test suite)
EXPORTED = sorted(_PROTOS)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is not built: run `python -c 'import __graft_entry__ as g; g.build()'`")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _PROTOS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
        from . import autotune

        autotune.load()  # the FP64 engine's tile table measured on GB300 (shipped with the package)
    return _lib


def check(rc: int) -> None:
    if rc != SU2G_OK:
        raise Su2gError(rc, lib().su2g_last_error().decode(errors="replace"))


def ptr(a) -> int:
    """Address of a numpy array or torch tensor."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()


def stream_handle(stream=None):
    if stream is None:
        import torch

        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream
